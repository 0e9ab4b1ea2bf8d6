"""Non-negative CP (multiplicative updates) and the NNDSVD initialisation on
the GPU against the reference runs (tests/golden) and the NumPy oracle.

Tolerances: f64 runs match the reference to 1e-9 relative (factors, error
list, same number of iterations); f32 runs to 1e-3 on the factors and 1e-4 on
the errors (multiplicative updates) or 1e-2 and 1e-3 (HALS)."""

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu

NN_CASES = ["nn_mu_random", "nn_mu_svd", "nn_mu_4way_fixed", "nn_mu_stop", "nn_mu_f32"]


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("case", NN_CASES)
def test_non_negative_parafac_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = gb300.non_negative_parafac(torch.as_tensor(x, device="cuda"), rank,
                                              return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-4 if f32 else 1e-9,
                               atol=1e-6 if f32 else 1e-12)
    np.testing.assert_allclose(host(w), run["weights"])
    for a, b in zip(f, run["factors"]):
        a = host(a)
        assert (a >= 0).all()
        tol = 1e-3 if f32 else 1e-9
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_nndsvda_unfolding_matches_oracle(gb300, mode):
    from tensorly_gb300.svd import svd_interface_unfolding
    rs = np.random.RandomState(3 + mode)
    x = rs.rand(11, 9, 13) + 0.1 * rs.randn(11, 9, 13)
    W, S = svd_interface_unfolding(torch.as_tensor(x, device="cuda"), mode, 4,
                                   non_negative=True)
    Wo, So, _ = oracle.svd_interface(oracle.unfold(x, mode), n_eigenvecs=4, non_negative=True)
    np.testing.assert_allclose(host(S), So, rtol=1e-10)
    np.testing.assert_allclose(host(W), Wo, rtol=1e-9, atol=1e-12)


def test_cp_nn_estimator_and_host_inputs(gb300, golden):
    run = golden["runs"]["nn_mu_random"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    est = gb300.CP_NN(rank, **kw)
    cp = est.fit_transform(x)                      # NumPy in, NumPy out
    assert isinstance(cp.factors[0], np.ndarray)
    np.testing.assert_allclose(est.errors_, run["errors"], rtol=1e-9, atol=1e-12)
    for a, b in zip(cp.factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())


def test_non_negative_parafac_unsupported_options_raise(gb300):
    x = torch.rand(5, 6, 7, device="cuda", dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        gb300.non_negative_parafac(x, 2, normalize_factors=True)
    with pytest.raises(NotImplementedError):
        gb300.non_negative_parafac(x, 2, mask=torch.ones_like(x))
    with pytest.raises(TypeError):
        gb300.non_negative_parafac(x, 2, cvg_criterion="nope")


HALS_CASES = ["nn_hals_random", "nn_hals_svd", "nn_hals_stop", "nn_hals_f32", "nn_hals_rank1",
              "nn_hals_exact"]


@pytest.mark.parametrize("case", HALS_CASES)
def test_non_negative_parafac_hals_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = gb300.non_negative_parafac_hals(torch.as_tensor(x, device="cuda"), rank,
                                                   return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    # f32: rounding in the Gauss-Seidel inner sweeps compounds along a run that
    # is still descending, so the f32 tolerance is 1e-3 on the error list
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-9,
                               atol=1e-6 if f32 else 1e-12)
    for a, b in zip(f, run["factors"]):
        a = host(a)
        assert (a >= 0).all()
        tol = 1e-2 if f32 else 1e-8
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


def test_hals_sparsity_and_fixed_mode_match_reference(gb300, golden):
    run = golden["runs"]["nn_hals_sparse_fixed"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    with pytest.warns(UserWarning):
        (w, f), errs = gb300.non_negative_parafac_hals(torch.as_tensor(x, device="cuda"), rank,
                                                       return_errors=True, **kw)
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-9, atol=1e-12)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(host(a), b, rtol=1e-8, atol=1e-8 * np.abs(b).max())


def test_hals_estimator_and_unsupported_options(gb300, golden):
    run = golden["runs"]["nn_hals_random"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    est = gb300.CP_NN_HALS(rank, **kw)
    cp = est.fit_transform(x)
    np.testing.assert_allclose(est.errors_, run["errors"], rtol=1e-9, atol=1e-12)
    assert isinstance(cp.factors[0], np.ndarray)
    xt = torch.as_tensor(x, device="cuda")
    with pytest.raises(NotImplementedError):
        gb300.non_negative_parafac_hals(xt, 2, fixed_modes=[2])


@pytest.mark.parametrize("case", ["nn_hals_modes_02", "nn_hals_normalize"])
def test_hals_nn_modes_subset_and_normalize_match_reference(gb300, golden, case):
    """A mode outside nn_modes takes the least-squares update
    (tensorly/decomposition/_nn_cp.py:337-341); normalize_factors renormalises
    after every updated mode but the last and after every iteration, with the
    weights in the normal equations (:316-320, :342-343, :373-374).  f64,
    against the reference's runs."""
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = gb300.non_negative_parafac_hals(torch.as_tensor(x, device="cuda"), rank,
                                                   return_errors=True, **kw)
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(host(w), run["weights"], rtol=1e-8, atol=1e-10)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(host(a), b, rtol=1e-8, atol=1e-8 * np.abs(b).max())


@pytest.mark.parametrize("dtype,rank", [(np.float64, 130), (np.float64, 100),
                                        (np.float32, 100), (np.float64, 33)])
def test_hals_wide_ranks_match_oracle(gb300, dtype, rank):
    """Ranks that fill 2 to 5 register slots per lane; f64 rank 130 reads the
    Gram product from global memory (it does not fit shared memory)."""
    rs = np.random.RandomState(rank)
    x = rs.rand(14, 12, 10).astype(dtype)
    kw = dict(init="random", random_state=3, n_iter_max=2, tol=1e-12)
    (_, fo), eo = oracle.non_negative_parafac_hals(x, rank, return_errors=True, **kw)
    (_, fg), eg = gb300.non_negative_parafac_hals(torch.as_tensor(x, device="cuda"), rank,
                                                  return_errors=True, **kw)
    f32 = dtype == np.float32
    np.testing.assert_allclose(eg, eo, rtol=1e-4 if f32 else 1e-9)
    for a, b in zip(fg, fo):
        tol = 1e-2 if f32 else 1e-8
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("algo", ["mu", "hals", "admm"])
def test_f32_split_tensor_core_mttkrp_in_nn_loops(gb300, algo):
    """f32 tensors whose modes suit the tensor-core plans run the MTTKRP of
    the multiplicative-update, HALS and AO-ADMM loops as the exact
    three-plane bf16 split on the tensor cores.  Against the same loops on
    the SIMT f32 MTTKRP (split_simt knob): the error lists to 1e-4 and the
    factors to 1e-3 (the tensor cores' f32 accumulation rounds toward zero,
    about -2e-7 of |M|), and both against the f64 oracle to 1e-3; the
    workspace grows by the three tensor planes, so the split path is the one
    that ran."""
    import ctypes
    from tensorly_gb300 import _lib
    rs = np.random.RandomState(21)
    fs = [rs.rand(s, 6) for s in (48, 40, 32)]
    x64 = np.einsum("ir,jr,kr->ijk", *fs) + 0.01 * rs.rand(48, 40, 32)
    x = torch.as_tensor(x64, dtype=torch.float32, device="cuda")
    kw = dict(init="random", random_state=5, n_iter_max=6, tol=1e-12)
    lib = _lib.lib()

    def run():
        if algo == "mu":
            return gb300.non_negative_parafac(x, 6, return_errors=True, **kw)
        if algo == "hals":
            return gb300.non_negative_parafac_hals(x, 6, return_errors=True, **kw)
        np.random.seed(5)     # its 'random' start draws from NumPy's global generator
        return gb300.constrained_parafac(x, 6, non_negative=True, return_errors=True,
                                         init="random", random_state=5, n_iter_max=6,
                                         tol_outer=1e-12)

    def ws_bytes():
        nb = ctypes.c_size_t(0)
        sh = _lib.i64_array(x.shape)
        _lib.check(lib.tlgb_cp_nn_mu_workspace_size(_lib.TLGB_F32, 3, sh, 6, 6, ctypes.byref(nb)))
        return nb.value

    try:
        tc_bytes = ws_bytes()
        (w1, f1), e1 = run()
        _lib.check(lib.tlgb_set_tuning(b"split_simt", 1))
        simt_bytes = ws_bytes()
        (w2, f2), e2 = run()
    finally:
        _lib.check(lib.tlgb_set_tuning(b"split_simt", 0))
    assert tc_bytes >= simt_bytes + 3 * 2 * x.numel()
    assert len(e1) == len(e2)
    np.testing.assert_allclose(e1, e2, rtol=1e-4)
    for a, b in zip(f1, f2):
        np.testing.assert_allclose(host(a), host(b), rtol=1e-3, atol=1e-3 * host(b).max())
    if algo == "mu":
        (_, fo), eo = oracle.non_negative_parafac(x64, 6, return_errors=True, **kw)
    elif algo == "hals":
        (_, fo), eo = oracle.non_negative_parafac_hals(x64, 6, return_errors=True, **kw)
    else:
        np.random.seed(5)
        (_, fo), eo = oracle.constrained_parafac(x64, 6, non_negative=True, return_errors=True,
                                                 init="random", random_state=5, n_iter_max=6,
                                                 tol_outer=1e-12)
    np.testing.assert_allclose(e1, eo, rtol=1e-3)
