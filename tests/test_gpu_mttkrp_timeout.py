"""The bounded pipeline waits of the tensor-core MTTKRP, driven to expiry
without faulting anything.

With the "tc_test_starve" tuning key the producer issues no copies, so the
MMA and epilogue waits (given a 1 ms limit in that mode) expire: the kernel
records TLGB_ETIMEOUT in the workspace status, frees its tensor memory and
returns.  Nothing is in flight when it exits (no copy was issued).  The
device must stay usable: the next normal call on the same device is
correct, and a CP-ALS run that meets the timeout reports it as an error.
"""

import ctypes

import numpy as np
import pytest
import torch

from test_gpu_mttkrp_bf16 import reference, split_t, split_value

pytestmark = pytest.mark.gpu


def _call(lib, _lib, xb, fs, fbt, rank, mode, out, ws):
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.tlgb_mttkrp_bf16(xb.data_ptr(), xb.dim(), _lib.i64_array(xb.shape),
                                    _lib.ptr_array([f.data_ptr() for f in fs]),
                                    _lib.ptr_array([f.data_ptr() for f in fbt]), None, rank, mode,
                                    out.data_ptr(), ws.data_ptr(), ws.numel(), st))
    status = ctypes.c_int(-1)
    _lib.check(lib.tlgb_workspace_status(ws.data_ptr(), st, ctypes.byref(status)))
    return status.value


def test_starved_pipeline_times_out_and_the_device_stays_usable(gb300):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    rs = np.random.RandomState(5)
    shape, rank, mode = (64, 40, 128), 16, 0
    x = rs.randn(*shape).astype(np.float32)
    f_np = [rs.randn(s, rank).astype(np.float32) for s in shape]
    xb = torch.as_tensor(x, device="cuda").to(torch.bfloat16).contiguous()
    fs = [torch.as_tensor(f, device="cuda") for f in f_np]
    fbt = [split_t(f) for f in fs]
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_mttkrp_bf16_workspace_size(3, _lib.i64_array(shape), rank, mode,
                                                   ctypes.byref(nbytes)))
    ws = torch.zeros(nbytes.value, dtype=torch.uint8, device="cuda")
    out = torch.empty((shape[mode], rank), dtype=torch.float32, device="cuda")
    lib.tlgb_set_tuning(b"tc_test_starve", 1)
    try:
        status = _call(lib, _lib, xb, fs, fbt, rank, mode, out, ws)
    finally:
        lib.tlgb_set_tuning(b"tc_test_starve", 0)
    assert status == _lib.TLGB_ETIMEOUT
    # the same device, a normal call: the pipeline runs and the result is right
    assert _call(lib, _lib, xb, fs, fbt, rank, mode, out, ws) == 0
    xr = torch.as_tensor(x).to(torch.bfloat16).to(torch.float64).numpy()
    f_used = [f.astype(np.float64) for f in f_np]
    f_used[2] = split_value(f_np[2])           # the inner factor enters as bf16 hi + lo
    want = reference(xr, f_used, None, mode)
    got = out.cpu().numpy().astype(np.float64)
    assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max()


def test_cp_als_reports_the_timeout_then_runs(gb300):
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    rs = np.random.RandomState(6)
    x = torch.as_tensor(rs.rand(64, 48, 40).astype(np.float32), device="cuda")
    init = [torch.as_tensor(rs.rand(s, 4).astype(np.float32), device="cuda") for s in x.shape]
    kw = dict(init=gb300.CPTensor((None, init)), n_iter_max=3, tol=0, precision="bf16",
              refine_sweeps=0, return_errors=True)
    lib.tlgb_set_tuning(b"tc_test_starve", 1)
    try:
        with pytest.raises(RuntimeError, match="timed out"):
            gb300.parafac(x, 4, **kw)
    finally:
        lib.tlgb_set_tuning(b"tc_test_starve", 0)
    _, errs = gb300.parafac(x, 4, **kw)
    assert len(errs) == 3 and all(np.isfinite(errs)) and errs[-1] < 1.0
