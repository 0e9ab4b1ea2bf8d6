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
