"""tlgb_mttkrp_noalloc (fixed in-library scratch, no workspace) against
tlgb_mttkrp with a caller workspace, through the C ABI.

The file name sorts last so that the test also runs after every other GPU
test in the same process (the scratch set-up must not depend on call order).
"""

import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

NOALLOC_SCRATCH_BYTES = 16 << 20

CASES = [
    ((17, 9, 23), 3, torch.float64),
    ((64, 64, 64), 8, torch.float32),
    ((4, 5, 3, 6, 4), 2, torch.float64),
    ((40, 50, 36), 70, torch.float32),
    ((5, 130), 70, torch.float64),
    ((512, 512, 512), 64, torch.float32),
]


def _dtype_code(dtype):
    from tensorly_gb300 import _lib
    return _lib.TLGB_F32 if dtype == torch.float32 else _lib.TLGB_F64


def _call_pair(lib, _lib, x, fs, w, rank, mode):
    """Two tlgb_mttkrp_noalloc calls and one tlgb_mttkrp call on one stream."""
    code = _dtype_code(x.dtype)
    shape = _lib.i64_array(x.shape)
    fp = _lib.ptr_array([f.data_ptr() for f in fs])
    st = torch.cuda.current_stream().cuda_stream
    # two-way tensors: the reference ignores the weights (callers pass none)
    wp = None if x.dim() == 2 else w.data_ptr()
    nb = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_mttkrp_workspace_size(code, x.dim(), shape, rank, mode, ctypes.byref(nb)))
    ws = torch.empty(max(1, nb.value), dtype=torch.uint8, device="cuda")
    ref = torch.empty(x.shape[mode], rank, dtype=x.dtype, device="cuda")
    outs = [torch.full_like(ref, float("nan")) for _ in range(2)]
    for out in outs:
        _lib.check(lib.tlgb_mttkrp_noalloc(code, x.data_ptr(), x.dim(), shape, fp,
                                           wp, rank, mode, out.data_ptr(), st))
    _lib.check(lib.tlgb_mttkrp(code, x.data_ptr(), x.dim(), shape, fp, wp, rank, mode,
                               ref.data_ptr(), ws.data_ptr(), ws.numel(), st))
    torch.cuda.synchronize()
    return ref, outs, nb.value


@pytest.mark.parametrize("shape,rank,dtype", CASES)
def test_noalloc_matches_workspace_entry_point(gb300, shape, rank, dtype):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    g = torch.Generator(device="cuda").manual_seed(sum(shape) + rank)
    x = torch.randn(*shape, generator=g, device="cuda", dtype=dtype)
    fs = [torch.randn(s, rank, generator=g, device="cuda", dtype=dtype) for s in shape]
    w = torch.rand(rank, generator=g, device="cuda", dtype=dtype) + 0.5
    modes = range(len(shape)) if x.numel() < 1 << 20 else (1,)
    for mode in modes:
        ref, outs, need = _call_pair(lib, _lib, x, fs, w, rank, mode)
        assert need <= NOALLOC_SCRATCH_BYTES
        for out in outs:
            assert torch.equal(out, ref), f"mode {mode}: noalloc result differs from tlgb_mttkrp"
        if x.numel() < 1 << 20:
            xn = x.double().cpu().numpy()
            fn = [f.double().cpu().numpy() for f in fs]
            want = oracle.unfolding_dot_khatri_rao(
                xn, (w.double().cpu().numpy() if len(shape) > 2 else None, fn), mode)
            scale = np.abs(want).max()
            tol = 1e-12 if dtype == torch.float64 else 1e-5
            assert np.abs(ref.double().cpu().numpy() - want).max() <= tol * scale * 10


def test_noalloc_rejects_oversized_plan(gb300):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    # one split's partial tile alone is 20000 x 128 x 8 B = 20.5 MB, so the
    # plan exceeds the scratch whatever split count the device's SM count gives
    shape, rank, mode = (20000, 8, 8), 128, 0
    code = _lib.TLGB_F64
    sh = _lib.i64_array(shape)
    nb = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_mttkrp_workspace_size(code, 3, sh, rank, mode, ctypes.byref(nb)))
    assert nb.value > NOALLOC_SCRATCH_BYTES
    x = torch.zeros(shape, dtype=torch.float64, device="cuda")
    fs = [torch.zeros(s, rank, dtype=torch.float64, device="cuda") for s in shape]
    out = torch.zeros(shape[mode], rank, dtype=torch.float64, device="cuda")
    rc = lib.tlgb_mttkrp_noalloc(code, x.data_ptr(), 3, sh, _lib.ptr_array([f.data_ptr() for f in fs]),
                                 None, rank, mode, out.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TLGB_EWORKSPACE
    assert b"16 MiB" in lib.tlgb_last_error()
