"""bf16 tensor-core MTTKRP (tcgen05 + TMA) against an f64 evaluation of the
same contraction on the bf16-rounded tensor and the bf16 hi+lo split of the
inner factor (outer factors stay f32, as in the kernel's epilogue).
Tolerance: 2e-5 of the output's max-abs, the f32-accumulation error of a
bf16 product sum."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def bf16_round(a):
    return torch.as_tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()


def split_t(f):
    """(2, R, rows) bf16 planes: hi = bf16(f^T), lo = bf16(f^T - hi)."""
    ft = f.t().contiguous()
    hi = ft.to(torch.bfloat16)
    lo = (ft - hi.float()).to(torch.bfloat16)
    return torch.stack([hi, lo]).contiguous()


def split_value(f):
    """f64 value the kernel contracts with: hi + lo."""
    hi = bf16_round(f)
    return hi + bf16_round(f.astype(np.float64) - hi)


def reference(x, factors, weights, mode):
    """M = unfold(x, mode) . KR(weights; factors != mode), in f64."""
    n = x.ndim
    rank = factors[(mode + 1) % n].shape[1]
    others = [k for k in range(n) if k != mode]
    kr = np.ones((1, rank))
    for k in others:
        kr = (kr[:, None, :] * factors[k][None, :, :]).reshape(-1, rank)
    if weights is not None:
        kr = kr * weights
    unf = np.moveaxis(x, mode, 0).reshape(x.shape[mode], -1)
    return unf @ kr


def run_bf16(gb300, x_np, factors_np, weights_np, mode):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    n = x_np.ndim
    rank = factors_np[0].shape[1]
    xb = torch.as_tensor(x_np, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    fs = [torch.as_tensor(f, dtype=torch.float32, device="cuda").contiguous() for f in factors_np]
    fbt = [split_t(f) for f in fs]
    w = None if weights_np is None else torch.as_tensor(weights_np, dtype=torch.float32,
                                                         device="cuda")
    shape = _lib.i64_array(x_np.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_mttkrp_bf16_workspace_size(n, shape, rank, mode, ctypes.byref(nbytes)))
    ws = torch.zeros(nbytes.value, dtype=torch.uint8, device="cuda")
    out = torch.empty((x_np.shape[mode], rank), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.tlgb_mttkrp_bf16(xb.data_ptr(), n, shape,
                                    _lib.ptr_array([f.data_ptr() for f in fs]),
                                    _lib.ptr_array([f.data_ptr() for f in fbt]),
                                    None if w is None else w.data_ptr(), rank, mode,
                                    out.data_ptr(), ws.data_ptr(), ws.numel(), st))
    status = ctypes.c_int(-1)
    _lib.check(lib.tlgb_workspace_status(ws.data_ptr(), st, ctypes.byref(status)))
    assert status.value == 0, "tensor-core pipeline reported a timeout"
    return out.cpu().numpy().astype(np.float64)


CASES = [((16, 16, 64), 8), ((64, 40, 128), 16), ((130, 24, 72), 20), ((128, 64, 128), 32),
         ((24, 16, 32, 40), 16), ((96, 72, 200), 64), ((40, 136, 48), 100), ((8, 8, 8, 8, 8), 5)]


@pytest.mark.parametrize("shape,rank", CASES)
def test_mttkrp_bf16_matches_f64(gb300, shape, rank):
    rs = np.random.RandomState(sum(shape) + rank)
    x = rs.randn(*shape).astype(np.float32)
    factors = [rs.randn(s, rank).astype(np.float32) for s in shape]
    weights = (rs.rand(rank) + 0.5).astype(np.float32)
    xr = bf16_round(x)
    n = len(shape)
    for mode in range(n):
        inner = n - 1 if mode != n - 1 else n - 2
        fr = [f.astype(np.float64) for f in factors]
        fr[inner] = split_value(factors[inner])
        ref = reference(xr, fr, weights.astype(np.float64), mode)
        got = run_bf16(gb300, x, factors, weights, mode)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 2e-5, (mode, err)


def test_mttkrp_bf16_deterministic(gb300):
    rs = np.random.RandomState(3)
    x = rs.randn(64, 48, 96).astype(np.float32)
    factors = [rs.randn(s, 24).astype(np.float32) for s in x.shape]
    for mode in range(3):
        a = run_bf16(gb300, x, factors, None, mode)
        b = run_bf16(gb300, x, factors, None, mode)
        assert np.array_equal(a, b)


def test_mttkrp_bf16_rejects_unsupported_shapes(gb300):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    nbytes = ctypes.c_size_t(0)
    # inner mode not a multiple of 8
    rc = lib.tlgb_mttkrp_bf16_workspace_size(3, _lib.i64_array([16, 16, 20]), 8, 0,
                                             ctypes.byref(nbytes))
    assert rc == _lib.TLGB_EUNSUPPORTED
    # rank above 128
    rc = lib.tlgb_mttkrp_bf16_workspace_size(3, _lib.i64_array([16, 16, 64]), 129, 0,
                                             ctypes.byref(nbytes))
    assert rc == _lib.TLGB_EUNSUPPORTED


def test_parafac_bf16_reaches_f64_fit(gb300):
    """Mixed precision CP-ALS: bf16 tensor-core sweeps then 3 f32 sweeps reach
    the f64 oracle's final relative error within 1e-4 (relative)."""
    import oracle
    from tensorly_gb300 import workloads
    x, _ = workloads.dense_cp_large(size=96, rank=8, seed=1)
    init = oracle.random_cp(x.shape, 8, random_state=0, dtype=np.float32)[1]
    (_, _), oerr = oracle.parafac(x.astype(np.float64), 8,
                                  init=(None, [f.astype(np.float64) for f in init]),
                                  n_iter_max=25, tol=0, return_errors=True)
    xt = torch.as_tensor(x, device="cuda")
    cp, errs = gb300.parafac(xt, 8, init=gb300.CPTensor((None, [torch.as_tensor(f, device="cuda")
                                                               for f in init])),
                             n_iter_max=25, tol=0, return_errors=True, precision="bf16",
                             refine_sweeps=3)
    assert len(errs) == 25
    assert abs(errs[-1] - oerr[-1]) <= 1e-4 * oerr[-1], (errs[-1], oerr[-1])


@pytest.mark.parametrize("planes", [3, 2])
@pytest.mark.parametrize("shape,rank", [((64, 48, 40), 24), ((40, 24, 16, 32), 8),
                                        ((128, 96, 80), 64), ((32, 40, 48), 5)])
def test_f32_split_sweep_matches_simt_f32(gb300, shape, rank, planes):
    """A closing sweep whose MTTKRPs run on the tensor cores with the bf16
    split of the f32 tensor and factor.  With three tensor planes
    (x0 . (f0+f1+f2) + x1 . (f0+f1) + x2 . f0, tuning key closing_planes = 3)
    it matches the same sweep with the SIMT f32 MTTKRP to f32 accuracy, and
    both match the f64 oracle sweep on the same f32 bytes.  With the default
    two (x2 dropped: the tensor enters with 16 significant bits) the factors
    stay within 2e-4 of the f64 sweep's largest entry on this incoherent
    random data and the error within 1e-4 (it is computed on the f32 tensor)."""
    import oracle
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    rs = np.random.RandomState(sum(shape) + rank)
    x = rs.randn(*shape).astype(np.float32)
    init = [rs.randn(s, rank).astype(np.float32) for s in shape]
    xt = torch.as_tensor(x, device="cuda")

    def one_sweep(refine_simt):
        lib.tlgb_set_tuning(b"refine_simt", refine_simt)
        try:
            # n_iter_max == refine_sweeps: the only sweep is the f32 refinement sweep
            cp, errs = gb300.parafac(
                xt, rank, init=gb300.CPTensor((None, [torch.as_tensor(f, device="cuda")
                                                      for f in init])),
                n_iter_max=1, tol=0, return_errors=True, precision="bf16", refine_sweeps=1)
        finally:
            lib.tlgb_set_tuning(b"refine_simt", 0)
        return [f.double().cpu().numpy() for f in cp.factors], errs[-1]

    try:
        lib.tlgb_set_tuning(b"closing_planes", planes)
        f_tc, e_tc = one_sweep(0)
    finally:
        lib.tlgb_set_tuning(b"closing_planes", 0)
    f_simt, e_simt = one_sweep(1)
    _, f_o, e_list = oracle.parafac_sweeps(x.astype(np.float64), np.ones(rank),
                                           [f.astype(np.float64) for f in init], 1)
    e_o = e_list[-1]
    for a, b, c in zip(f_tc, f_simt, f_o):
        scale = np.abs(c).max()
        assert np.abs(a - c).max() <= 2e-4 * scale
        assert np.abs(b - c).max() <= 2e-4 * scale
        if planes == 3:
            # the split path is at least as close to f64 as the SIMT f32 path (x4 slack)
            assert np.abs(a - c).max() <= 4 * np.abs(b - c).max() + 1e-6 * scale
    assert abs(e_simt - e_o) <= 1e-5 * e_o
    assert abs(e_tc - e_o) <= (1e-5 if planes == 3 else 1e-4) * e_o


def test_parafac_reports_mttkrp_times(gb300):
    """The per-sweep-kind MTTKRP durations come back for every kind that ran."""
    rs = np.random.RandomState(3)
    x = torch.as_tensor(rs.randn(64, 48, 40).astype(np.float32), device="cuda")
    init = [torch.as_tensor(rs.randn(s, 8).astype(np.float32), device="cuda") for s in x.shape]
    times = {}
    gb300.parafac(x, 8, init=gb300.CPTensor((None, init)), n_iter_max=6, tol=0,
                  precision="bf16", refine_sweeps=3, mttkrp_times=times)
    assert set(times) == {"bf16", "f32_split", "closing"}
    for name, row in times.items():
        assert len(row) == 3 and all(0 < v < 1000 for v in row), (name, row)
    native = {}
    gb300.parafac(x, 8, init=gb300.CPTensor((None, init)), n_iter_max=2, tol=0,
                  mttkrp_times=native, use_graph=False)
    assert set(native) == {"native"} and all(v > 0 for v in native["native"])


def test_dense_autotuner_picks_valid_tiles_and_keeps_results(gb300):
    """autotune.tune_dense searches the inner-mode group, ring depth and wave
    count on the caller's tensor; every choice is one of the searched values,
    it is cached, and bf16 parafac under it reaches the same fit as under the
    defaults (1e-5 relative: only the summation order of the split-K partial
    tiles changes)."""
    from tensorly_gb300 import autotune
    rs = np.random.RandomState(4)
    fs = [rs.rand(s, 16) for s in (96, 80, 72)]
    x = torch.as_tensor(np.einsum("ir,jr,kr->ijk", *fs), dtype=torch.float32, device="cuda")
    init = [torch.as_tensor(rs.rand(s, 16), dtype=torch.float32, device="cuda")
            for s in x.shape]
    kw = dict(n_iter_max=12, tol=0, precision="bf16", refine_sweeps=2, return_errors=True)
    try:
        autotune.reset_dense()
        _, e0 = gb300.parafac(x, 16, init=gb300.CPTensor((None, [f.clone() for f in init])), **kw)
        choice = autotune.tune_dense(x, 16, sweeps=4, refine_sweeps=1, reps=1)
        space = dict(autotune.DENSE_SPACE)
        assert set(choice) == set(space)
        for k, v in choice.items():
            assert v in space[k]
        assert autotune.tune_dense(x, 16, sweeps=4, refine_sweeps=1) == choice   # cached
        _, e1 = gb300.parafac(x, 16, init=gb300.CPTensor((None, [f.clone() for f in init])), **kw)
        np.testing.assert_allclose(e1, e0, rtol=1e-5, atol=1e-7)
    finally:
        autotune.reset_dense()
