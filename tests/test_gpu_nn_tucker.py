"""Non-negative Tucker (multiplicative updates) on the GPU
(tensorly/decomposition/_tucker.py:348-454) against the reference runs
(tests/golden) and the NumPy oracle, and the small operations it is built
from (tlgb_gemm, tlgb_mu_update, tlgb_dot).

Tolerances: f64 1e-8 on the error list, 1e-7 (of the largest entry) on core
and factors: the products come from the TTM chain instead of the
reference's explicit B, and the error from the norm expansion; f32 1e-3 and
1e-2."""

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("case", ["nnt_svd", "nnt_random", "nnt_stop", "nnt_f32",
                                  "nnt_normalize"])
def test_non_negative_tucker_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (core, factors), errs = gb300.non_negative_tucker(torch.as_tensor(x, device="cuda"), rank,
                                                      return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-8)
    tol = 1e-2 if f32 else 1e-7
    c = host(core)
    assert (c >= 0).all()
    np.testing.assert_allclose(c, run["core"], rtol=tol, atol=tol * np.abs(run["core"]).max())
    for a, b in zip(factors, run["factors"]):
        a = host(a)
        assert (a >= 0).all()
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


def test_non_negative_tucker_host_input_and_options(gb300, golden):
    run = golden["runs"]["nnt_svd"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    tt = gb300.non_negative_tucker(x, rank, **kw)
    assert isinstance(tt.core, np.ndarray)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_small_ops_match_numpy(gb300, dtype):
    from tensorly_gb300 import decomposition as d
    rs = np.random.RandomState(0)
    a = rs.randn(37, 19).astype(dtype)
    b = rs.randn(23, 19).astype(dtype)
    c = rs.randn(19, 41).astype(dtype)
    ta, tb, tc = (torch.as_tensor(v, device="cuda") for v in (a, b, c))
    tol = 1e-12 if dtype == np.float64 else 1e-5
    np.testing.assert_allclose(host(d._mat_nt(ta, tb)), a @ b.T, rtol=tol, atol=tol * 10)
    np.testing.assert_allclose(host(d._mat_nn(ta, tc)), a @ c, rtol=tol, atol=tol * 10)
    np.testing.assert_allclose(host(d._mat_tn(ta, ta)), a.T @ a, rtol=tol, atol=tol * 10)
    num = np.abs(rs.randn(37, 19)).astype(dtype)
    den = np.abs(rs.randn(37, 19)).astype(dtype)
    num[0, 0] = 0.0
    t = torch.as_tensor(a.copy(), device="cuda")
    d._mu_update(t, torch.as_tensor(num, device="cuda"), torch.as_tensor(den, device="cuda"),
                 1e-3)
    np.testing.assert_allclose(host(t), a * np.maximum(num, 1e-3) / np.maximum(den, 1e-3),
                               rtol=tol)
    np.testing.assert_allclose(d._dot(ta, ta).item(), float((a.astype(np.float64) ** 2).sum()),
                               rtol=1e-12 if dtype == np.float64 else 1e-6)


@pytest.mark.parametrize("case", ["nnth_svd", "nnth_random", "nnth_sparse", "nnth_f32",
                                  "nnth_normalize", "nnth_active_set", "nnth_active_set_4way",
                                  "nnth_active_set_normalize", "nnth_active_set_f32",
                                  "nnth_active_set_stop"])
def test_non_negative_tucker_hals_matches_reference(gb300, golden, case):
    """HALS factor updates with the FISTA or the active-set core update,
    with and without normalize_factors; f64 1e-8 on the error list and 1e-6
    on core and factors (the HALS rows move P A incrementally, the passive
    systems are solved by the library's LU), f32 1e-3 and 1e-2."""
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (core, factors), errs = gb300.non_negative_tucker_hals(torch.as_tensor(x, device="cuda"),
                                                           rank, return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-8)
    tol = 1e-2 if f32 else 1e-6
    np.testing.assert_allclose(host(core), run["core"], rtol=tol,
                               atol=tol * np.abs(run["core"]).max())
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("exact", [False, True])
def test_hals_nnls_matches_oracle(gb300, exact):
    rs = np.random.RandomState(5)
    U = np.abs(rs.randn(40, 6))
    M = np.abs(rs.randn(40, 30))
    UtM, UtU = U.T @ M, U.T @ U
    V0 = np.abs(rs.randn(6, 30))
    ref = oracle.hals_nnls(UtM, UtU, V0.copy(), n_iter_max=200, sparsity_coefficient=0.01,
                           exact=exact)
    out = gb300.hals_nnls(UtM, UtU, V0.copy(), n_iter_max=200, sparsity_coefficient=0.01,
                          exact=exact)
    assert isinstance(out, np.ndarray) and out.shape == (6, 30)
    np.testing.assert_allclose(out, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    with pytest.raises(NotImplementedError):
        gb300.hals_nnls(UtM, UtU)
    x = torch.rand(8, 7, 6, device="cuda", dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        gb300.non_negative_tucker_hals(x, [2, 2, 2], algorithm="lbfgs")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_tucker_kats_match_reference(gb300, golden, dtype):
    """tucker_normalize, kronecker and active_set_nnls on the GPU against the
    reference's outputs on the recorded inputs (f64 1e-12, or 1e-9 for the
    active set's LU solves; f32 1e-5 relative)."""
    from tensorly_gb300.cp_tensor import tucker_normalize
    from tensorly_gb300.decomposition import active_set_nnls
    from tensorly_gb300.tenalg import kronecker
    f64 = dtype == np.float64
    for k in golden["tucker_kats"]:
        if k["op"] == "tucker_normalize":
            core = torch.as_tensor(k["core"].astype(dtype), device="cuda")
            fs = [torch.as_tensor(f.astype(dtype), device="cuda") for f in k["factors"]]
            c, f = tucker_normalize((core, fs))
            tol = 1e-12 if f64 else 1e-5
            np.testing.assert_allclose(host(c), k["out_core"], rtol=tol,
                                       atol=tol * np.abs(k["out_core"]).max())
            for a, b in zip(f, k["out_factors"]):
                np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol)
            assert (host(f[0])[:, 0] == 0).all()       # the zero column stays zero
        elif k["op"] == "kronecker":
            ms = [torch.as_tensor(m.astype(dtype), device="cuda") for m in k["matrices"]]
            out = host(kronecker(ms))
            if f64:
                np.testing.assert_array_equal(out, k["out"])
            else:
                np.testing.assert_allclose(out, k["out"], rtol=1e-5, atol=1e-6)
            out2 = host(kronecker(ms, skip_matrix=1, reverse=True))
            np.testing.assert_allclose(out2, k["out_skip1_rev"], rtol=1e-5 if not f64 else 0)
        elif k["op"] == "active_set_nnls" and f64:
            x0 = None if k["x0"] is None else torch.as_tensor(k["x0"], device="cuda")
            out = host(active_set_nnls(torch.as_tensor(k["Utm"], device="cuda"),
                                       torch.as_tensor(k["UtU"], device="cuda"), x=x0,
                                       n_iter_max=100))
            assert (out >= 0).all()
            np.testing.assert_allclose(out, k["out"], rtol=1e-9,
                                       atol=1e-9 * np.abs(k["out"]).max())
    # the one-CTA solve holds up to 128 unknowns
    big = torch.eye(129, dtype=torch.float64, device="cuda")
    with pytest.raises(NotImplementedError):
        active_set_nnls(torch.ones(129, dtype=torch.float64, device="cuda"), big)


def test_active_set_nnls_host_arrays_and_oracle(gb300):
    """NumPy in, NumPy out; a random well-posed system against the oracle."""
    from tensorly_gb300.decomposition import active_set_nnls
    rs = np.random.RandomState(3)
    a = rs.randn(80, 40)
    b = a @ (np.abs(rs.randn(40)) * (rs.rand(40) > 0.5)) + 0.1 * rs.randn(80)
    out = active_set_nnls(a.T @ b, a.T @ a, n_iter_max=200)
    assert isinstance(out, np.ndarray) and out.shape == (40,)
    ref = oracle.active_set_nnls(a.T @ b, a.T @ a, n_iter_max=200)
    np.testing.assert_allclose(out, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


def test_fixed_modes_raise_the_reference_error(gb300, golden):
    """With fixed modes the reference's loop fails on its first misaligned
    mode_dot; the same ValueError and message come back, before any work."""
    for e in golden["fixed_mode_errors"]:
        x = torch.rand(*e["shape"], dtype=torch.float64, device="cuda")
        with pytest.raises(ValueError) as info:
            gb300.non_negative_tucker_hals(x, e["rank"], n_iter_max=2, init=e["init"],
                                           random_state=0, fixed_modes=list(e["fixed"]))
        assert str(info.value) == e["message"]
