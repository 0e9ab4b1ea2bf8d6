"""Unfolding and folding (tensorly/base.py:5-79) on the GPU.

``unfold`` and ``fold`` move data with the library's ``tlgb_unfold`` /
``tlgb_fold`` kernels; ``tensor_to_vec`` and ``vec_to_tensor`` are views of a
C-contiguous tensor, as in the reference (a reshape).
"""

import torch

from . import _lib
from ._tensor import dtype_code, ptr, stream_of


def _cuda(tensor, what):
    if not isinstance(tensor, torch.Tensor) or not tensor.is_cuda:
        raise TypeError(f"{what} takes CUDA tensors")
    return tensor.contiguous()


def unfold(tensor, mode):
    """Mode-``mode`` unfolding, shape ``(tensor.shape[mode], -1)``, columns in the
    C order of the other modes (tensorly/base.py:39-53)."""
    x = _cuda(tensor, "unfold")
    mode = int(mode)
    if not 0 <= mode < x.ndim:
        raise ValueError(f"mode {mode} out of range for a {x.ndim}-way tensor")
    out = torch.empty((x.shape[mode], x.numel() // max(x.shape[mode], 1)), dtype=x.dtype,
                      device=x.device)
    _lib.check(_lib.lib().tlgb_unfold(dtype_code(x), ptr(x), x.ndim,
                                      _lib.i64_array(x.shape), mode, ptr(out), stream_of(x)))
    return out


def fold(unfolded_tensor, mode, shape):
    """Inverse of ``unfold``: the tensor of ``shape`` (tensorly/base.py:56-79)."""
    u = _cuda(unfolded_tensor, "fold")
    shape = tuple(int(s) for s in shape)
    mode = int(mode)
    if not 0 <= mode < len(shape):
        raise ValueError(f"mode {mode} out of range for a {len(shape)}-way tensor")
    n = 1
    for s in shape:
        n *= s
    if u.numel() != n or u.shape[0] != shape[mode]:
        raise ValueError(f"cannot fold a {tuple(u.shape)} unfolding into {shape} along mode {mode}")
    out = torch.empty(shape, dtype=u.dtype, device=u.device)
    _lib.check(_lib.lib().tlgb_fold(dtype_code(u), ptr(u), len(shape), _lib.i64_array(shape),
                                    mode, ptr(out), stream_of(u)))
    return out


def tensor_to_vec(tensor):
    """tensorly/base.py:5-18: the C-order vectorisation."""
    return tensor.reshape(-1)


def vec_to_tensor(vec, shape):
    """tensorly/base.py:21-36."""
    return vec.reshape(shape)
