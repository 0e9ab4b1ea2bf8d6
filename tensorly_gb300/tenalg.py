"""GB300 tensor-algebra primitives with the signatures of ``tensorly.tenalg``.

khatri_rao               tensorly/tenalg/core_tenalg/_khatri_rao.py:9-109
unfolding_dot_khatri_rao tensorly/tenalg/core_tenalg/mttkrp.py:9-50
mode_dot                 tensorly/tenalg/core_tenalg/n_mode_product.py:5-76
multi_mode_dot           tensorly/tenalg/core_tenalg/n_mode_product.py:79-135

Inputs are CUDA float32/float64 tensors (host tensors and arrays are copied
to the GPU and results returned the same way).  Validation errors mirror the
reference's ``ValueError`` messages.
"""

import warnings

import numpy as np
import torch

from . import _lib
from ._tensor import (MAX_MODES, dtype_code, like, ptr, stream_of, to_device, workspace)


def _khatri_rao_raw(matrices, weights=None, mask=None):
    """Library Khatri-Rao of CUDA matrices (no single-matrix shortcut)."""
    ref = matrices[0]
    rank = int(ref.shape[1])
    rows = [int(m.shape[0]) for m in matrices]
    total = int(np.prod(rows))
    out = torch.empty((total, rank), dtype=ref.dtype, device=ref.device)
    w = None if weights is None else like(weights, ref)
    mk = None if mask is None else like(mask, ref).reshape(-1)
    if mk is not None and mk.numel() != total:
        raise ValueError(f"mask has {mk.numel()} entries, expected {total}")
    mats = [m.contiguous() for m in matrices]
    _lib.check(_lib.lib().tlgb_khatri_rao(
        dtype_code(ref), len(mats), _lib.ptr_array([ptr(m) for m in mats]), _lib.i64_array(rows),
        rank, ptr(w), ptr(mk), ptr(out), stream_of(ref)))
    return out


def khatri_rao(matrices, weights=None, skip_matrix=None, mask=None):
    """Khatri-Rao product, first matrix slowest (reference ``:64-109``).

    A single remaining matrix is returned as is, weights ignored (``:71-73``).
    """
    if skip_matrix is not None:
        matrices = [matrices[i] for i in range(len(matrices)) if i != skip_matrix]
    if len(matrices) == 1:
        return matrices[0]
    placed = []
    first, pl = to_device(matrices[0])
    for m in matrices:
        t = like(m, first) if not (isinstance(m, torch.Tensor) and m.is_cuda) else m
        placed.append(t)
    matrices = placed
    if matrices[0].ndim == 2:
        n_columns = matrices[0].shape[1]
    else:
        n_columns = 1
        matrices = [m.reshape(-1, 1) for m in matrices]
        warnings.warn("Khatri-rao of a series of vectors instead of matrices. "
                      "Considering each as a matrix with 1 column.")
    for i, matrix in enumerate(matrices):
        if matrix.ndim != 2:
            raise ValueError("All the matrices must have exactly 2 dimensions!"
                             f"Matrix {i} has dimension {matrix.ndim} != 2.")
        if matrix.shape[1] != n_columns:
            raise ValueError("All matrices must have same number of columns!"
                             f"Matrix {i} has {matrix.shape[1]} columns != {n_columns}.")
    if len(matrices) > MAX_MODES:
        raise NotImplementedError(f"khatri_rao of more than {MAX_MODES} matrices")
    matrices = [m.to(matrices[0].dtype).contiguous() for m in matrices]
    return pl.back(_khatri_rao_raw(matrices, weights, mask))


def unfolding_dot_khatri_rao(tensor, cp_tensor, mode):
    """MTTKRP ``unfold(tensor, mode) . KR(weights; factors, skip=mode)``
    without forming either operand (reference mttkrp.py:9-50).

    For a 2-way tensor the reference's Khatri-Rao of the single remaining
    factor ignores the weights (_khatri_rao.py:71-73); that is kept.
    """
    weights, factors = cp_tensor
    x, pl = to_device(tensor)
    n = x.ndim
    if n < 2:
        raise ValueError("unfolding_dot_khatri_rao needs a tensor of order >= 2")
    if n > MAX_MODES:
        raise NotImplementedError(f"tensors of order > {MAX_MODES} are not supported")
    if len(factors) != n:
        raise ValueError(f"expected {n} factors, got {len(factors)}")
    mode = mode % n
    fs = [like(f, x) for f in factors]
    rank = int(fs[(mode + 1) % n].shape[1])
    for k, f in enumerate(fs):
        if k != mode and (f.ndim != 2 or f.shape[0] != x.shape[k] or f.shape[1] != rank):
            raise ValueError(f"factor {k} has shape {tuple(f.shape)}, expected "
                             f"({x.shape[k]}, {rank})")
    w = None if (weights is None or n == 2) else like(weights, x)
    lib = _lib.lib()
    shape = _lib.i64_array(x.shape)
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.tlgb_mttkrp_workspace_size(dtype_code(x), n, shape, rank, mode,
                                              _lib.ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    out = torch.empty((x.shape[mode], rank), dtype=x.dtype, device=x.device)
    _lib.check(lib.tlgb_mttkrp(dtype_code(x), ptr(x), n, shape,
                               _lib.ptr_array([ptr(f) if k != mode else None
                                               for k, f in enumerate(fs)]),
                               ptr(w), rank, mode, ptr(out), ptr(ws), ws.numel(), stream_of(x)))
    return pl.back(out)


def _mode_dot_cuda(x, u, mode, transpose):
    """x: CUDA tensor, u: CUDA matrix; returns x x_mode u (or u^T)."""
    J = int(u.shape[1] if transpose else u.shape[0])
    new_shape = list(x.shape)
    new_shape[mode] = J
    out = torch.empty(new_shape, dtype=x.dtype, device=x.device)
    if out.numel() == 0:
        return out
    _lib.check(_lib.lib().tlgb_mode_dot(dtype_code(x), ptr(x), x.ndim, _lib.i64_array(x.shape),
                                        ptr(u.contiguous()), J, 1 if transpose else 0, mode,
                                        ptr(out), stream_of(x)))
    return out


def mode_dot(tensor, matrix_or_vector, mode, transpose=False):
    """n-mode product (reference n_mode_product.py:5-76)."""
    x, pl = to_device(tensor)
    if x.ndim > MAX_MODES:
        raise NotImplementedError(f"tensors of order > {MAX_MODES} are not supported")
    m = like(matrix_or_vector, x)
    new_shape = list(x.shape)
    if m.ndim == 2:
        dim = 0 if transpose else 1
        if m.shape[dim] != x.shape[mode]:
            raise ValueError(
                f"shapes {tuple(x.shape)} and {tuple(m.shape)} not aligned in mode-{mode} "
                f"multiplication: {x.shape[mode]} (mode {mode}) != {m.shape[dim]} "
                f"(dim 1 of matrix)")
        return pl.back(_mode_dot_cuda(x, m, mode, transpose))
    if m.ndim == 1:
        if m.shape[0] != x.shape[mode]:
            raise ValueError(
                f"shapes {tuple(x.shape)} and {tuple(m.shape)} not aligned for mode-{mode} "
                f"multiplication: {x.shape[mode]} (mode {mode}) != {m.shape[0]} (vector size)")
        res = _mode_dot_cuda(x, m.reshape(1, -1), mode, False)
        if len(new_shape) > 1:
            new_shape.pop(mode)
        else:
            new_shape = []
        return pl.back(res.reshape(new_shape))
    raise ValueError("Can only take n_mode_product with a vector or a matrix."
                     f"Provided array of dimension {m.ndim} not in [1, 2].")


def multi_mode_dot(tensor, matrix_or_vec_list, modes=None, skip=None, transpose=False):
    """Chain of mode_dot in sorted mode order (reference :79-135)."""
    x, pl = to_device(tensor)
    if modes is None:
        modes = range(len(matrix_or_vec_list))
    decrement = 0
    res = x
    factors_modes = sorted(zip(matrix_or_vec_list, modes), key=lambda t: t[1])
    for i, (m, mode) in enumerate(factors_modes):
        if skip is not None and i == skip:
            continue
        m = like(m, x)
        if transpose and m.ndim == 2:
            md = mode - decrement
            if m.shape[0] != res.shape[md]:   # the reference reports the transposed matrix
                raise ValueError(
                    f"shapes {tuple(res.shape)} and {(int(m.shape[1]), int(m.shape[0]))} not "
                    f"aligned in mode-{md} multiplication: {res.shape[md]} (mode {md}) != "
                    f"{m.shape[0]} (dim 1 of matrix)")
            res = mode_dot(res, m, md, transpose=True)
        else:
            res = mode_dot(res, m, mode - decrement)
        if m.ndim == 1:
            decrement += 1
    return pl.back(res)


def kronecker(matrices, skip_matrix=None, reverse=False):
    """Kronecker product of a list of matrices, the first varying slowest
    (tensorly/tenalg/core_tenalg/_kronecker.py:8-57), by ``tlgb_kronecker``."""
    if skip_matrix is not None:
        matrices = [matrices[i] for i in range(len(matrices)) if i != skip_matrix]
    if reverse:
        matrices = matrices[::-1]
    x, pl = to_device(matrices[0])
    ms = [like(m, x).contiguous() for m in matrices]
    if len(ms) > MAX_MODES:
        raise NotImplementedError(f"kronecker of more than {MAX_MODES} matrices is not supported")
    for m in ms:
        if m.ndim != 2:
            raise ValueError("kronecker takes matrices")
    rows = [int(m.shape[0]) for m in ms]
    cols = [int(m.shape[1]) for m in ms]
    out = torch.empty((int(np.prod(rows)), int(np.prod(cols))), dtype=x.dtype, device=x.device)
    if out.numel() == 0:
        return pl.back(out)
    _lib.check(_lib.lib().tlgb_kronecker(dtype_code(x), len(ms),
                                         _lib.ptr_array([ptr(m) for m in ms]),
                                         _lib.i64_array(rows), _lib.i64_array(cols), ptr(out),
                                         stream_of(x)))
    return pl.back(out)
