"""CP and Tucker containers and helpers (tensorly/cp_tensor.py, tensorly/tucker_tensor.py).

The containers behave like the reference's: a CPTensor unpacks as
``weights, factors = cp``; a TuckerTensor as ``core, factors = tt``.
"""

import warnings

import numpy as np
import torch

from . import _lib
from ._tensor import dtype_code, ptr, stream_of, workspace


def _shape_of(x):
    return tuple(int(v) for v in x.shape)


def _validate_cp_tensor(cp_tensor):
    """(shape, rank) of a (weights, factors) pair, with the reference's
    ValueErrors for malformed input (tensorly/cp_tensor.py:163-214)."""
    if isinstance(cp_tensor, CPTensor):
        return cp_tensor.shape, cp_tensor.rank
    if isinstance(cp_tensor, (float, int)):
        return 0, 0
    weights, factors = cp_tensor
    f0 = _shape_of(factors[0])
    if len(f0) == 2:
        rank = f0[1]
    elif len(f0) == 1:
        rank = 1
    else:
        raise ValueError("Got a factor with 3 dimensions but CP factors should be at most 2D, "
                         "of shape (size, rank).")
    shape = []
    for i, factor in enumerate(factors):
        s = _shape_of(factor)
        if len(s) == 2:
            size, current_rank = s
        else:
            size, current_rank = s[0], 1
        if current_rank != rank:
            # s[1] is read as the reference reads it (an IndexError for a 1-D factor)
            raise ValueError("All the factors of a CP tensor should have the same number of "
                             f"column.However, factors[0].shape[1]={rank} but "
                             f"factors[{i}].shape[1]={s[1]}.")
        shape.append(size)
    if weights is not None and _shape_of(weights) != (rank,):
        raise ValueError(f"Given factors for a rank-{rank} CP tensor but "
                         f"len(weights)={_shape_of(weights)}.")
    return tuple(shape), rank


def _validate_tucker_tensor(tucker_tensor):
    """(shape, rank) of a (core, factors) pair, with the reference's
    ValueErrors for malformed input (tensorly/tucker_tensor.py:19-47)."""
    core, factors = tucker_tensor
    if len(factors) < 2:
        raise ValueError("A Tucker tensor should be composed of at least two factors and a "
                         f"core.However, {len(factors)} factor was given.")
    core_shape = _shape_of(core)
    if len(factors) != len(core_shape):
        raise ValueError("Tucker decompositions should have one factor per more of the core "
                         f"tensor.However, core has {len(core_shape)} modes but {len(factors)} "
                         "factors have been provided")
    shape, rank = [], []
    for i, factor in enumerate(factors):
        current_shape, current_rank = _shape_of(factor)
        if current_rank != core_shape[i]:
            raise ValueError("Factor `n` of Tucker decomposition should verify:\n"
                             "factors[n].shape[1] = core.shape[n]."
                             f"However, factors[{i}].shape[1]={current_rank} but "
                             f"core.shape[{i}]={core_shape[i]}.")
        shape.append(current_shape)
        rank.append(current_rank)
    return tuple(shape), tuple(rank)


class CPTensor:
    """(weights, factors) pair; tensorly/cp_tensor.py:17-160.

    Validated on construction as the reference does (``_validate_cp_tensor``);
    ``weights`` default to ones (``:25-26``).
    """

    def __init__(self, cp_tensor):
        shape, rank = _validate_cp_tensor(cp_tensor)
        weights, factors = cp_tensor
        factors = list(factors)
        if weights is None:
            f0 = factors[0]
            if isinstance(f0, torch.Tensor):
                weights = torch.ones(rank, dtype=f0.dtype, device=f0.device)
            else:
                weights = np.ones(rank, dtype=np.asarray(f0).dtype)
        self.weights = weights
        self.factors = factors
        self.shape = tuple(shape)
        self.rank = int(rank)

    def __getitem__(self, i):
        if i == 0:
            return self.weights
        if i == 1:
            return self.factors
        raise IndexError(f"CPTensor index {i} out of range (0: weights, 1: factors)")

    def __setitem__(self, i, value):
        if i == 0:
            self.weights = value
        elif i == 1:
            self.factors = list(value)
        else:
            raise IndexError(f"CPTensor index {i} out of range")

    def __iter__(self):
        yield self.weights
        yield self.factors

    def __len__(self):
        return 2

    def __repr__(self):
        return f"(weights, factors) : rank-{self.rank} CPTensor of shape {self.shape}"

    def to_tensor(self):
        return cp_to_tensor(self)

    def norm(self):
        return cp_norm(self)

    def normalize(self, inplace=True):
        w, f = cp_normalize(self)
        if inplace:
            self.weights, self.factors = w, f
            return self
        return CPTensor((w, f))


class TuckerTensor:
    """(core, factors) pair; tensorly/tucker_tensor.py:227-320."""

    def __init__(self, tucker_tensor):
        shape, rank = _validate_tucker_tensor(tucker_tensor)
        core, factors = tucker_tensor
        self.core = core
        self.factors = list(factors)
        self.shape = shape
        self.rank = rank

    def __getitem__(self, i):
        if i == 0:
            return self.core
        if i == 1:
            return self.factors
        raise IndexError(f"TuckerTensor index {i} out of range (0: core, 1: factors)")

    def __iter__(self):
        yield self.core
        yield self.factors

    def __len__(self):
        return 2

    def __repr__(self):
        return f"Decomposed Tucker tensor of shape {self.shape} with rank {self.rank}"

    def to_tensor(self):
        return tucker_to_tensor(self)


def validate_cp_rank(tensor_shape, rank="same", rounding="round"):
    """tensorly/cp_tensor.py:240-275."""
    fun = {"ceil": np.ceil, "floor": np.floor, "round": np.round}.get(rounding)
    if fun is None:
        raise ValueError(f"Rounding should be of round, floor or ceil, but got {rounding}")
    if rank == "same":
        rank = float(1)
    if isinstance(rank, float):
        rank = int(fun(np.prod(tensor_shape) * rank / np.sum(tensor_shape)))
    return rank


def validate_tucker_rank(tensor_shape, rank="same", rounding="round", fixed_modes=None):
    """tensorly/tucker_tensor.py:344-447: a list of per-mode ranks.  'same'
    and fractional ranks keep that fraction of the tensor's parameter count
    (core plus factors), an int is used for every free mode, a sequence is
    returned as given."""
    fun_r = {"ceil": np.ceil, "floor": np.floor, "round": np.round}.get(rounding)
    if fun_r is None:
        raise ValueError(f"Rounding should be round, floor or ceil, but got {rounding}")
    if rank == "same":
        rank = float(1)
    if isinstance(rank, float):
        from scipy.optimize import brentq
        n_modes = len(tensor_shape)
        n_param = np.prod(tensor_shape)
        shape = list(tensor_shape)
        n_fixed = 0
        fixed = None
        if fixed_modes is not None:
            fixed = [(m, shape.pop(m)) for m in sorted(fixed_modes, reverse=True)][::-1]
            n_fixed = np.sum([s ** 2 for _, s in fixed])
            n_modes -= len(fixed)
        sq = np.sum([s ** 2 for s in shape])
        f = lambda x: n_param * x ** n_modes + sq * x + n_fixed * x - rank * n_param  # noqa: E731
        frac = brentq(f, 0.0, max(rank, 1.0))
        out = [max(int(fun_r(s * frac)), 1) for s in shape]
        if fixed is not None:
            for m, s in fixed:
                out.insert(m, s)
        return out
    if isinstance(rank, int):
        warnings.warn(
            f"Given only one int for 'rank' for decomposition a tensor of order "
            f"{len(tensor_shape)}. Using this rank for all modes.", RuntimeWarning)
        if fixed_modes is None:
            return [rank] * len(tensor_shape)
        return [rank if i not in fixed_modes else s for i, s in enumerate(tensor_shape)]
    return rank


def _factors_cuda(cp_tensor):
    weights, factors = cp_tensor
    ref = factors[0]
    if not isinstance(ref, torch.Tensor) or not ref.is_cuda:
        raise TypeError("tensorly_gb300 CP helpers take CUDA tensors")
    return weights, factors


def cp_normalize(cp_tensor):
    """Unit-norm factor columns, norms into the weights
    (tensorly/cp_tensor.py:278-321), by the library's normalisation kernel."""
    weights, factors = _factors_cuda(cp_tensor)
    factors = [f.contiguous().clone() for f in factors]
    rank = factors[0].shape[1]
    if weights is None:
        weights = torch.ones(rank, dtype=factors[0].dtype, device=factors[0].device)
    else:
        weights = weights.to(factors[0].dtype).contiguous().clone()
    lib = _lib.lib()
    rows = _lib.i64_array([f.shape[0] for f in factors])
    _lib.check(lib.tlgb_cp_normalize(dtype_code(factors[0]), len(factors), rows, rank,
                                     _lib.ptr_array([ptr(f) for f in factors]), ptr(weights),
                                     stream_of(factors[0])))
    return CPTensor((weights, factors))


def cp_norm(cp_tensor):
    """||[[w; A]]||_F from the Hadamard product of the factor Grams
    (tensorly/cp_tensor.py:614-644); f64 accumulation on the GPU."""
    weights, factors = _factors_cuda(cp_tensor)
    factors = [f.contiguous() for f in factors]
    rank = factors[0].shape[1]
    lib = _lib.lib()
    out = torch.empty(1, dtype=torch.float64, device=factors[0].device)
    rows = _lib.i64_array([f.shape[0] for f in factors])
    w = None if weights is None else weights.to(factors[0].dtype).contiguous()
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_norm_workspace_size(len(factors), rows, rank, _lib.ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, factors[0].device)
    _lib.check(lib.tlgb_cp_norm(dtype_code(factors[0]), len(factors), rows, rank,
                                _lib.ptr_array([ptr(f) for f in factors]), ptr(w), ptr(out),
                                ptr(ws), ws.numel(), stream_of(factors[0])))
    return out[0].to(factors[0].dtype)


def cp_to_tensor(cp_tensor, mask=None):
    """Full tensor of a CP model (tensorly/cp_tensor.py:433-485): the mode-0
    unfolding ``(A_0 * w) . KR(A_1..A_{N-1})^T`` by ``tlgb_cp_to_tensor``, which
    forms the Khatri-Rao entries in shared memory instead of in HBM.  A mask
    (broadcastable to the full shape) multiplies the result.  A 1-way model
    gives ``sum_r w_r A_0[:, r]``."""
    weights, factors = _factors_cuda(cp_tensor)
    factors = [f.contiguous() for f in factors]
    f0 = factors[0]
    rank = int(f0.shape[1])
    shape = tuple(int(f.shape[0]) for f in factors)
    for f in factors:
        if f.ndim != 2 or int(f.shape[1]) != rank or f.dtype != f0.dtype or f.device != f0.device:
            raise ValueError("cp_to_tensor: factors must be matrices with the same rank, "
                             "dtype and device")
    if weights is None and len(shape) == 1:
        # the reference multiplies None by the factor here (cp_tensor.py:470-471)
        raise TypeError("cp_to_tensor of a 1-way model needs weights")
    w = None
    if weights is not None:
        w = torch.as_tensor(weights).to(device=f0.device, dtype=f0.dtype).reshape(-1).contiguous()
        if w.numel() != rank:
            raise ValueError(f"cp_to_tensor: {w.numel()} weights for rank {rank}")
    m = None
    if mask is not None and len(shape) > 1:
        m = torch.as_tensor(mask).to(device=f0.device, dtype=f0.dtype).expand(shape).contiguous()
    out = torch.empty(shape, dtype=f0.dtype, device=f0.device)
    lib = _lib.lib()
    dims = _lib.i64_array(shape)
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_to_tensor_workspace_size(dtype_code(f0), len(shape), dims, rank,
                                                    _lib.ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, f0.device)
    _lib.check(lib.tlgb_cp_to_tensor(dtype_code(f0), len(shape), dims, rank,
                                     _lib.ptr_array([ptr(f) for f in factors]), ptr(w), ptr(m),
                                     ptr(out), ptr(ws), ws.numel(), stream_of(f0)))
    return out


def cp_to_unfolded(cp_tensor, mode):
    """Mode-``mode`` unfolding of the full tensor (tensorly/cp_tensor.py:488-521):
    ``(A_mode * w) . KR(others)^T``, i.e. ``cp_to_tensor`` of the factors with
    ``A_mode`` moved first, read as a matrix."""
    weights, factors = _factors_cuda(cp_tensor)
    mode = int(mode)
    order = [mode] + [k for k in range(len(factors)) if k != mode]
    full = cp_to_tensor((weights, [factors[k] for k in order]))
    return full.reshape(int(factors[mode].shape[0]), -1)


def cp_to_vec(cp_tensor):
    """C-order vectorisation of the full tensor (tensorly/cp_tensor.py:524-546)."""
    return cp_to_tensor(cp_tensor).reshape(-1)


def tucker_normalize(tucker_tensor):
    """Unit-norm factor columns with the norms multiplied into the core
    (tensorly/tucker_tensor.py:78-102), by ``tlgb_tucker_normalize``.
    Returns a new TuckerTensor of CUDA tensors."""
    core, factors = tucker_tensor
    if not isinstance(core, torch.Tensor) or not core.is_cuda:
        raise TypeError("tensorly_gb300 Tucker helpers take CUDA tensors")
    core = core.contiguous().clone()
    factors = [f.to(core.dtype).contiguous().clone() for f in factors]
    n = len(factors)
    ranks = _lib.i64_array([int(f.shape[1]) for f in factors])
    rows = _lib.i64_array([int(f.shape[0]) for f in factors])
    if tuple(core.shape) != tuple(int(f.shape[1]) for f in factors):
        raise ValueError("tucker_normalize: the core shape must match the factor ranks")
    lib = _lib.lib()
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.tlgb_tucker_normalize_workspace_size(n, ranks, _lib.ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, core.device)
    _lib.check(lib.tlgb_tucker_normalize(dtype_code(core), n, rows, ranks,
                                         _lib.ptr_array([ptr(f) for f in factors]), ptr(core),
                                         ptr(ws), ws.numel(), stream_of(core)))
    return TuckerTensor((core, factors))


def tucker_to_tensor(tucker_tensor, skip_factor=None, transpose_factors=False, modes=None):
    """tensorly/tucker_tensor.py:50-75: multi_mode_dot of the core."""
    from .tenalg import multi_mode_dot
    core, factors = tucker_tensor
    return multi_mode_dot(core, factors, skip=skip_factor, transpose=transpose_factors, modes=modes)


def tucker_to_unfolded(tucker_tensor, mode=0, skip_factor=None, transpose_factors=False):
    """tensorly/tucker_tensor.py:106-131: unfold of ``tucker_to_tensor``."""
    from .base import unfold
    return unfold(tucker_to_tensor(tucker_tensor, skip_factor=skip_factor,
                                   transpose_factors=transpose_factors), mode)


def tucker_to_vec(tucker_tensor, skip_factor=None, transpose_factors=False):
    """tensorly/tucker_tensor.py:134-162: vectorised ``tucker_to_tensor``."""
    return tucker_to_tensor(tucker_tensor, skip_factor=skip_factor,
                            transpose_factors=transpose_factors).reshape(-1)
