"""GPU parity of the SVD / eigensolver / Tucker-HOOI path against the NumPy
oracle and the reference's recorded runs (tests/golden)."""

import ctypes

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu


def cuda(a, dtype=torch.float64):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device="cuda")


def host(t):
    return t.detach().cpu().numpy()


def _eig(gb300, a, k, flip=True):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    code = _lib.TLGB_F64 if a.dtype == torch.float64 else _lib.TLGB_F32
    n = a.shape[0]
    nb = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_sym_eig_workspace_size(code, n, k, ctypes.byref(nb)))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    U = torch.empty((n, k), dtype=a.dtype, device="cuda")
    lam = torch.empty((k,), dtype=a.dtype, device="cuda")
    _lib.check(lib.tlgb_sym_eig(code, a.data_ptr(), n, k, U.data_ptr(), lam.data_ptr(),
                                1 if flip else 0, ws.data_ptr(), ws.numel(),
                                torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return host(U), host(lam)


def _check_flip(U):
    for c in range(U.shape[1]):
        i = int(np.argmax(np.abs(U[:, c])))
        assert U[i, c] > 0


@pytest.mark.parametrize("n,k", [(1, 1), (2, 1), (3, 3), (7, 4), (33, 5), (64, 64), (128, 16),
                                 (160, 10)])
@pytest.mark.parametrize("psd", [True, False])
def test_sym_eig_f64_matches_numpy(gb300, n, k, psd):
    rs = np.random.RandomState(n * 10 + k + psd)
    b = rs.randn(n, n + 3)
    a = b @ b.T if psd else (b[:, :n] + b[:, :n].T)
    U, lam = _eig(gb300, cuda(a), k)
    w, v = np.linalg.eigh(a)
    w, v = w[::-1][:k], v[:, ::-1][:, :k]
    scale = np.abs(w).max() if n > 0 else 1.0
    np.testing.assert_allclose(lam, w, rtol=0, atol=1e-12 * scale * max(1, n / 8))
    # vectors up to sign, then the svd_flip rule
    gaps = np.abs(np.diff(np.concatenate([[np.inf], w, [-np.inf]])))
    for c in range(k):
        gap = min(gaps[c], gaps[c + 1]) / scale
        if gap < 1e-6:
            continue
        d = abs(float(U[:, c] @ v[:, c]))
        assert d >= 1 - 1e-10 / gap - 1e-14, (c, d, gap)
    _check_flip(U)
    np.testing.assert_allclose(U.T @ U, np.eye(k), atol=1e-10)


@pytest.mark.parametrize("n,k", [(5, 2), (100, 12), (224, 8)])
def test_sym_eig_f32(gb300, n, k):
    rs = np.random.RandomState(n + k)
    b = rs.randn(n, 2 * n).astype(np.float32)
    a = (b @ b.T).astype(np.float32)
    U, lam = _eig(gb300, cuda(a, torch.float32), k)
    w, v = np.linalg.eigh(a.astype(np.float64))
    w, v = w[::-1][:k], v[:, ::-1][:, :k]
    np.testing.assert_allclose(lam, w, rtol=2e-5 * max(1, n / 32))
    for c in range(k):
        assert abs(float(U[:, c].astype(np.float64) @ v[:, c])) > 1 - 1e-3
    _check_flip(U)


def test_sym_eig_clustered_eigenvalues_orthonormal(gb300):
    # a repeated eigenvalue: the returned vectors must stay orthonormal
    rs = np.random.RandomState(5)
    q, _ = np.linalg.qr(rs.randn(20, 20))
    w = np.array([5.0, 3.0, 3.0, 3.0] + list(np.linspace(1.0, 0.1, 16)))
    a = (q * w) @ q.T
    U, lam = _eig(gb300, cuda(a), 6)
    np.testing.assert_allclose(lam, w[:6], atol=1e-12)
    np.testing.assert_allclose(U.T @ U, np.eye(6), atol=1e-9)
    # the span of the cluster is the right one
    P = q[:, 1:4]
    for c in (1, 2, 3):
        assert np.linalg.norm(P.T @ U[:, c]) > 1 - 1e-9


@pytest.mark.parametrize("shape,mode,k", [((12, 10, 9), 0, 3), ((12, 10, 9), 1, 4),
                                          ((12, 10, 9), 2, 9), ((4, 10, 9), 0, 4),
                                          ((30, 3, 2), 0, 5), ((6, 7, 5, 8), 3, 3),
                                          ((25, 6), 0, 3), ((7, 30), 0, 4)])
def test_svd_unfolding_matches_oracle(gb300, shape, mode, k):
    from tensorly_gb300.svd import svd_interface_unfolding
    rs = np.random.RandomState(sum(shape) + mode + k)
    x = rs.randn(*shape)
    U, S = svd_interface_unfolding(cuda(x), mode, n_eigenvecs=k)
    Uo, So, _ = oracle.svd_interface(oracle.unfold(x, mode), n_eigenvecs=k)
    np.testing.assert_allclose(host(S), So, rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(host(U), Uo, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("case", ["svd_wide", "svd_tall"])
def test_svd_interface_matches_reference(gb300, golden, case):
    from tensorly_gb300.svd import svd_interface
    run = golden["runs"][case]
    m = regenerate(run)
    U, S, V = svd_interface(cuda(m), n_eigenvecs=run["kwargs"]["n_eigenvecs"])
    np.testing.assert_allclose(host(U), run["U"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(host(S), run["S"], rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(host(V), run["V"], rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("case", ["tucker_svd", "tucker_random", "tucker_4way"])
def test_tucker_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    tt, errs = gb300.tucker(cuda(x), return_errors=True, **run["kwargs"])
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(host(tt.core), run["core"], rtol=1e-9, atol=1e-10)
    for a, b in zip(tt.factors, run["factors"]):
        np.testing.assert_allclose(host(a), b, rtol=1e-9, atol=1e-10)


def test_tucker_host_inputs_come_back_on_host(gb300, golden):
    run = golden["runs"]["tucker_svd"]
    x = regenerate(run)
    tt = gb300.tucker(x, **run["kwargs"])
    assert isinstance(tt.core, np.ndarray)
    np.testing.assert_allclose(tt.core, run["core"], rtol=1e-9, atol=1e-10)


def test_partial_tucker_unsorted_modes_raise_like_the_reference(gb300):
    x = np.random.RandomState(8).randn(9, 8, 10)
    with pytest.raises(ValueError):
        oracle.partial_tucker(x, [3, 2], modes=[2, 0], n_iter_max=3, tol=0)
    with pytest.raises(ValueError):
        gb300.partial_tucker(cuda(x), [3, 2], modes=[2, 0], n_iter_max=3, tol=0)


@pytest.mark.parametrize("modes", [[0, 2], [1, 2], [1]])
def test_partial_tucker_matches_oracle(gb300, modes):
    rs = np.random.RandomState(7 + len(modes))
    x = rs.randn(9, 8, 10)
    rank = [3, 2][: len(modes)]
    (core, factors), errs = gb300.partial_tucker(cuda(x), rank, modes=modes, n_iter_max=12,
                                                 tol=0)
    (co, fo), eo = oracle.partial_tucker(x, rank, modes=modes, n_iter_max=12, tol=0)
    np.testing.assert_allclose(errs, eo, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(host(core), co, rtol=1e-9, atol=1e-10)
    for a, b in zip(factors, fo):
        np.testing.assert_allclose(host(a), b, rtol=1e-9, atol=1e-10)


def test_tucker_fixed_factors_matches_oracle(gb300):
    rs = np.random.RandomState(11)
    x = rs.randn(8, 7, 6)
    # uniform ranks: the reference indexes `rank` by position among the free
    # modes on this path, so only equal ranks give a well-formed problem
    core0 = rs.randn(3, 3, 3)
    f0 = [np.linalg.qr(rs.randn(s, r))[0] for s, r in zip(x.shape, core0.shape)]
    tt = gb300.tucker(cuda(x), rank=[3, 3, 3], fixed_factors=[1],
                      init=(cuda(core0), [cuda(f) for f in f0]), n_iter_max=8, tol=0)
    co, fo = oracle.tucker(x, rank=[3, 3, 3], fixed_factors=[1], init=(core0, f0), n_iter_max=8,
                           tol=0)
    np.testing.assert_allclose(host(tt.core), co, rtol=1e-9, atol=1e-10)
    for a, b in zip(tt.factors, fo):
        np.testing.assert_allclose(host(a), b, rtol=1e-9, atol=1e-10)


def test_tucker_f32_close_to_f64(gb300):
    rs = np.random.RandomState(3)
    core = rs.randn(4, 4, 4)
    fs = [np.linalg.qr(rs.randn(s, 4))[0] for s in (40, 32, 48)]
    x = oracle.multi_mode_dot(core, fs) + 0.01 * rs.randn(40, 32, 48)
    tt, errs = gb300.tucker(cuda(x, torch.float32), rank=[4, 4, 4], return_errors=True,
                            n_iter_max=10, tol=0)
    (co, fo), eo = oracle.partial_tucker(x, [4, 4, 4], n_iter_max=10, tol=0)
    np.testing.assert_allclose(errs, eo, rtol=1e-4)
    for a, b in zip(tt.factors, fo):
        np.testing.assert_allclose(host(a), b, atol=1e-4)


@pytest.mark.parametrize("case", ["svd_init", "svd_init_short_mode"])
def test_parafac_svd_init_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    cp, errs = gb300.parafac(cuda(x), rank, return_errors=True, **kw)
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(host(cp.weights), run["weights"], rtol=1e-9, atol=1e-10)
    for a, b in zip(cp.factors, run["factors"]):
        np.testing.assert_allclose(host(a), b, rtol=1e-8, atol=1e-9 * np.abs(b).max())


def test_tucker_estimator(gb300, golden):
    run = golden["runs"]["tucker_4way"]
    x = regenerate(run)
    est = gb300.Tucker(**run["kwargs"])
    tt = est.fit_transform(cuda(x))
    np.testing.assert_allclose(host(tt.core), run["core"], rtol=1e-9, atol=1e-10)
    assert repr(est).startswith("Rank-")


@pytest.mark.parametrize("shape,rank", [((40, 6, 5, 7), [3, 2, 3, 2]),
                                        ((12, 14, 16, 10), [4, 5, 3, 4])])
def test_tucker_4way_uneven_matches_oracle(gb300, shape, rank):
    """Four modes: every chain has two products on the second stream and the
    factor updated last applied last; (40, 6, 5, 7) makes mode 0's unfolding
    tall after the chain (the SVD's input is read again after the eigensolver)."""
    rs = np.random.RandomState(sum(shape))
    x = rs.randn(*shape)
    (core, factors), errs = gb300.partial_tucker(cuda(x), rank, modes=[0, 1, 2, 3],
                                                 n_iter_max=6, tol=0)
    (co, fo), eo = oracle.partial_tucker(x, rank, modes=[0, 1, 2, 3], n_iter_max=6, tol=0)
    np.testing.assert_allclose(errs, eo, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(host(core), co, rtol=1e-9, atol=1e-10)
    for a, b in zip(factors, fo):
        np.testing.assert_allclose(host(a), b, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("shape,mode,side", [((70, 33, 50), 0, 0), ((70, 33, 50), 1, 0),
                                             ((70, 33, 50), 2, 0), ((9, 200, 7), 0, 1),
                                             ((20, 30, 3), 2, 1), ((130, 64, 3), 2, 0),
                                             ((64, 64, 64), 1, 0)])
def test_gram_unfolding_f32_matches_f64(gb300, shape, mode, side):
    """Gram of an f32 unfolding (M M^T, or M^T M for side 1) against f64 NumPy."""
    import ctypes
    from tensorly_gb300 import _lib
    from tensorly_gb300._tensor import workspace
    rs = np.random.RandomState(sum(shape) + mode)
    x = rs.randn(*shape).astype(np.float32)
    M = np.moveaxis(x.astype(np.float64), mode, 0).reshape(shape[mode], -1)
    want = M @ M.T if side == 0 else M.T @ M
    xt = cuda(x, torch.float32)
    n = want.shape[0]
    G = torch.empty((n, n), dtype=torch.float32, device="cuda")
    shp = (ctypes.c_int64 * 3)(*shape)
    nb = ctypes.c_size_t(0)
    lib = _lib.lib()
    _lib.check(lib.tlgb_gram_unfolding_workspace_size(3, shp, mode, side, ctypes.byref(nb)))
    ws = workspace(nb.value, xt.device)
    _lib.check(lib.tlgb_gram_unfolding(_lib.TLGB_F32, xt.data_ptr(), 3, shp, mode, side,
                                       G.data_ptr(), ws.data_ptr(), ws.numel(),
                                       torch.cuda.current_stream().cuda_stream))
    got = G.cpu().numpy().astype(np.float64)
    scale = np.sqrt(np.outer(np.diag(want), np.diag(want)))
    assert np.abs(got - want).max() / scale.max() < 2e-6
    np.testing.assert_array_equal(got, got.T)
