"""Partial SVDs on the GPU (tensorly/tenalg/svd.py).

``svd_interface`` / ``truncated_svd`` of a matrix or of a tensor unfolding
run in ``libtensorly_gb300.so``: the Gram matrix of the (never formed)
unfolding, then the leading eigenpairs of that small symmetric matrix
(Householder tridiagonalisation, multisection, inverse iteration; f64 for f64
tensors, f32 for f32 tensors), then the svd_flip sign rule.  The singular
triplets equal LAPACK's (up to that sign) wherever the k-th singular value is
separated from the next one.
"""

import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from ._tensor import dtype_code, ptr, stream_of, to_device, workspace

SVD_FUNS = ["truncated_svd", "symeig_svd"]


def _svd_unfolding_raw(x, mode, k, flip=True):
    """U (shape[mode] x k) and S (k) of unfold(x, mode); x a CUDA tensor."""
    lib = _lib.lib()
    shape = _lib.i64_array(x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_svd_unfolding_workspace_size(dtype_code(x), x.ndim, shape, int(mode),
                                                     int(k), ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    U = torch.empty((x.shape[mode], k), dtype=x.dtype, device=x.device)
    S = torch.empty((k,), dtype=x.dtype, device=x.device)
    _lib.check(lib.tlgb_svd_unfolding(dtype_code(x), ptr(x), x.ndim, shape, int(mode), int(k),
                                      ptr(U), ptr(S), 1 if flip else 0, ptr(ws), ws.numel(),
                                      stream_of(x)))
    return U, S


def _n_eigenvecs(rows, cols, n_eigenvecs):
    """Column count of U after tensorly/tenalg/svd.py:182-208 (svd_checks)
    and truncated_svd's slicing."""
    min_dim, max_dim = min(rows, cols), max(rows, cols)
    if n_eigenvecs is None:
        n_eigenvecs = max_dim
    if n_eigenvecs > max_dim:
        warnings.warn(f"Trying to compute SVD with n_eigenvecs={n_eigenvecs}, which is larger "
                      f"than max(matrix.shape)={max_dim}. Setting n_eigenvecs to {max_dim}.")
        n_eigenvecs = max_dim
    if n_eigenvecs > min_dim:
        # full_matrices=True: U is rows x rows, V cols x cols, S min_dim
        if rows > cols:
            raise NotImplementedError("svd with n_eigenvecs above the number of columns of a "
                                      "tall matrix (full_matrices) is not supported")
        return rows, min_dim
    return n_eigenvecs, n_eigenvecs


def svd_interface_unfolding(tensor, mode, n_eigenvecs, method="truncated_svd",
                            non_negative=False, flip_sign=True):
    """(U, S) of ``svd_interface(unfold(tensor, mode), n_eigenvecs, method,
    non_negative=non_negative)`` (tensorly/tenalg/svd.py:366-447) without
    forming the unfolding; ``non_negative`` (True = 'nndsvda', or 'nndsvd')
    replaces U by the NNDSVD factor W (``:443-444``, ``:68-134``)."""
    if non_negative not in (None, False, True, "nndsvd", "nndsvda"):
        raise ValueError(f'Invalid nntype parameter: got {non_negative} instead of one of '
                         '("nndsvd", "nndsvda")')
    if not (method in SVD_FUNS):
        if callable(method) or method == "randomized_svd":
            raise NotImplementedError(f"svd method {method!r} is not supported by tensorly_gb300")
        raise ValueError(f"Got svd={method}. However, the possible choices are {SVD_FUNS} or to "
                         "pass a callable.")
    x, _ = to_device(tensor)
    x = x.contiguous()
    rows = x.shape[mode]
    cols = x.numel() // max(1, rows)
    ucols, scount = _n_eigenvecs(rows, cols, n_eigenvecs)
    U, S = _svd_unfolding_raw(x, mode, ucols, flip=flip_sign)
    S = S[:scount]
    if non_negative not in (None, False):
        U = _nndsvd_unfolding(x, mode, U, S, "nndsvda" if non_negative is True else non_negative)
    return U, S


def _nndsvd_unfolding(x, mode, U, S, nntype):
    """W of NNDSVD (tensorly/tenalg/svd.py:68-134) for the mode-`mode`
    unfolding M of x from its (U, S).  V's rows enter through U^T M = S V,
    which is the mode-n product of x with U^T; the norms of their positive
    and negative parts, the column choice and the fill run in the library."""
    from .tenalg import mode_dot
    lib = _lib.lib()
    k = min(int(U.shape[1]), int(S.shape[0]))
    Uk = U[:, :k].contiguous()
    Y = mode_dot(x, Uk.t().contiguous(), mode)
    L = int(np.prod(x.shape[:mode])) if mode > 0 else 1
    Tt = int(np.prod(x.shape[mode + 1:])) if mode + 1 < x.ndim else 1
    code = dtype_code(x)
    ws = torch.empty(max(256, 2 * k) * 8, dtype=torch.uint8, device=x.device)
    total = torch.zeros(1, dtype=torch.float64, device=x.device)
    st = stream_of(x)
    _lib.check(lib.tlgb_sum(code, x.data_ptr(), x.numel(), total.data_ptr(), ws.data_ptr(),
                            ws.numel(), st))
    fill = 1 if nntype == "nndsvda" else 0
    avg = float(total.item()) / x.numel() if fill else 0.0
    W = torch.empty_like(Uk)
    _lib.check(lib.tlgb_nndsvd_columns(code, Uk.data_ptr(), S.contiguous().data_ptr(),
                                       Y.contiguous().data_ptr(), int(Uk.shape[0]), k, L, Tt,
                                       fill, avg, W.data_ptr(), ws.data_ptr(), ws.numel(), st))
    if U.shape[1] > k:   # columns past the singular values stay zero before the fill
        extra = torch.full((U.shape[0], U.shape[1] - k), avg if fill else 0.0,
                           dtype=U.dtype, device=U.device)
        W = torch.cat([W, extra], dim=1)
    return W


def svd_flip(U, V, u_based_decision=True):
    """tensorly/tenalg/svd.py:13-65 for real matrices on the device."""
    Ut, pl = to_device(U)
    Vt, _ = to_device(V, device=Ut.device)
    if u_based_decision:
        idx = torch.argmax(torch.abs(Ut), dim=0)
        signs = torch.sign(Ut[idx, torch.arange(Ut.shape[1], device=Ut.device)])
    else:
        idx = torch.argmax(torch.abs(Vt), dim=1)
        signs = torch.sign(Vt[torch.arange(Vt.shape[0], device=Vt.device), idx])
    if u_based_decision:
        Ut = Ut * signs
        extra = Vt.shape[0] - Ut.shape[1]
        if extra > 0:
            signs = torch.cat([signs, torch.ones(extra, dtype=signs.dtype, device=signs.device)])
        Vt = Vt * signs[: Vt.shape[0]][:, None]
    else:
        Vt = Vt * signs[:, None]
        extra = Ut.shape[1] - Vt.shape[0]
        if extra > 0:
            signs = torch.cat([signs, torch.ones(extra, dtype=signs.dtype, device=signs.device)])
        Ut = Ut * signs[: Ut.shape[1]]
    return pl.back(Ut), pl.back(Vt)


def truncated_svd(matrix, n_eigenvecs=None, **kwargs):
    """tensorly/tenalg/svd.py:211-235 for a 2-D matrix: (U, S, V) with U's
    columns sign-fixed (svd_flip is applied by svd_interface in the
    reference; the GPU path fixes the signs while forming U, which svd_flip
    then leaves unchanged)."""
    m, pl = to_device(matrix)
    if m.ndim != 2:
        raise ValueError("truncated_svd expects a matrix")
    m = m.contiguous()
    rows, cols = m.shape
    ucols, scount = _n_eigenvecs(rows, cols, n_eigenvecs)
    U, S = _svd_unfolding_raw(m, 0, ucols, flip=True)
    S = S[:scount]
    # V = S^-1 U^T M for the non-zero singular values (rows of V)
    from .tenalg import _khatri_rao_raw, mode_dot
    s_host = S.double().cpu().numpy()
    inv = np.where(s_host > 0, 1.0 / np.where(s_host > 0, s_host, 1.0), 0.0)
    Us = _khatri_rao_raw([U[:, :scount].contiguous()],
                         weights=torch.as_tensor(inv, dtype=m.dtype, device=m.device))
    V = mode_dot(m, Us, 0, transpose=True)
    return pl.back(U), pl.back(S), pl.back(V)


def svd_interface(matrix, method="truncated_svd", n_eigenvecs=None, flip_sign=True,
                  u_based_flip_sign=True, non_negative=None, mask=None,
                  n_iter_mask_imputation=5, **kwargs):
    """tensorly/tenalg/svd.py:366-447 for method 'truncated_svd' / 'symeig_svd'."""
    if mask is not None:
        raise NotImplementedError("svd with missing-value imputation is not supported")
    if non_negative not in (None, False):
        raise NotImplementedError("non-negative SVD is not supported")
    if method not in SVD_FUNS:
        if callable(method) or method == "randomized_svd":
            raise NotImplementedError(f"svd method {method!r} is not supported by tensorly_gb300")
        raise ValueError(f"Got svd={method}. However, the possible choices are {SVD_FUNS} or to "
                         "pass a callable.")
    U, S, V = truncated_svd(matrix, n_eigenvecs=n_eigenvecs)
    if flip_sign and not u_based_flip_sign:
        U, V = svd_flip(U, V, u_based_decision=False)
    return U, S, V
