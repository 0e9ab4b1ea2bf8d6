"""Tensor plumbing: device placement, dtype codes, raw pointers and streams.

PyTorch is used only for device memory and streams; every computation goes
through the CUDA library.
"""

import numpy as np
import torch

from . import _lib

MAX_MODES = 8


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError(
            "tensorly_gb300 needs a CUDA GPU (sm_103a); there is no CPU fallback")


def dtype_code(t):
    if t.dtype == torch.float32:
        return _lib.TLGB_F32
    if t.dtype == torch.float64:
        return _lib.TLGB_F64
    raise TypeError(f"tensorly_gb300 supports float32 and float64 tensors, got {t.dtype}")


class Placement:
    """Remembers where an input came from so results go back the same way."""

    def __init__(self, kind, device=None, dtype=None):
        self.kind = kind      # 'cuda', 'torch_cpu' or 'numpy'
        self.device = device
        self.dtype = dtype

    def back(self, t):
        if t is None:
            return None
        if self.kind == "cuda":
            return t
        if self.kind == "torch_cpu":
            return t.cpu()
        return t.cpu().numpy()


def to_device(x, device=None, dtype=None):
    """Return (cuda tensor, Placement).  Host inputs are copied to the GPU."""
    require_cuda()
    if isinstance(x, torch.Tensor):
        if x.is_complex():
            raise NotImplementedError("complex tensors are not supported by tensorly_gb300")
        if x.is_cuda:
            t = x
            pl = Placement("cuda", x.device, x.dtype)
        else:
            pl = Placement("torch_cpu", None, x.dtype)
            t = x.to(device or "cuda", non_blocking=False)
    else:
        arr = np.asarray(x)
        if np.iscomplexobj(arr):
            raise NotImplementedError("complex tensors are not supported by tensorly_gb300")
        if arr.dtype not in (np.float32, np.float64):
            arr = arr.astype(np.float64)
        pl = Placement("numpy", None, arr.dtype)
        t = torch.from_numpy(np.ascontiguousarray(arr)).to(device or "cuda")
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if t.dtype not in (torch.float32, torch.float64):
        t = t.to(torch.float64)
    return t.contiguous(), pl


def like(x, ref):
    """Move/cast `x` (tensor or array) to ref's device and dtype, contiguous."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if t.is_complex():
        raise NotImplementedError("complex tensors are not supported by tensorly_gb300")
    return t.to(device=ref.device, dtype=ref.dtype).contiguous()


def ptr(t):
    return t.data_ptr() if t is not None else None


def stream_of(t):
    return ctypes_stream(torch.cuda.current_stream(t.device))


def ctypes_stream(s):
    return s.cuda_stream


def workspace(nbytes, device):
    """A device scratch buffer from the caching allocator (>= 1 byte)."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
