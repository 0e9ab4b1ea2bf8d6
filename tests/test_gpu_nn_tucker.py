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


@pytest.mark.parametrize("case", ["nnt_svd", "nnt_random", "nnt_stop", "nnt_f32"])
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
    with pytest.raises(NotImplementedError):
        gb300.non_negative_tucker(x, rank, normalize_factors=True)


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


@pytest.mark.parametrize("case", ["nnth_svd", "nnth_random", "nnth_sparse", "nnth_f32"])
def test_non_negative_tucker_hals_matches_reference(gb300, golden, case):
    """HALS factor updates and the FISTA core update; f64 1e-8 on the error
    list and 1e-6 on core and factors (the HALS rows move P A incrementally),
    f32 1e-3 and 1e-2."""
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
        gb300.non_negative_tucker_hals(x, [2, 2, 2], algorithm="active_set")
