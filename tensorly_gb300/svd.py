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

SVD_FUNS = ["truncated_svd", "symeig_svd", "randomized_svd"]


def _check_method(method):
    if method in SVD_FUNS:
        return
    if callable(method):
        raise NotImplementedError("a callable svd method is not supported by tensorly_gb300")
    raise ValueError(f"Got svd={method}. However, the possible choices are {SVD_FUNS} or to "
                     "pass a callable.")


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
                            non_negative=False, flip_sign=True, mask=None,
                            n_iter_mask_imputation=5, random_state=None):
    """(U, S) of ``svd_interface(unfold(tensor, mode), n_eigenvecs, method,
    non_negative=non_negative, mask=unfold(mask, mode), ...)``
    (tensorly/tenalg/svd.py:366-447).  The Gram methods never form the
    unfolding.  ``non_negative`` (True = 'nndsvda', or 'nndsvd') replaces U by
    the NNDSVD factor W (``:443-444``, ``:68-134``).  With a mask the missing
    entries are refilled ``n_iter_mask_imputation`` times from the rank
    ``n_eigenvecs`` reconstruction U U^T M (``:431-439``); the tensor is not
    changed.  'randomized_svd' works on the explicit unfolding
    (``randomized_svd``)."""
    if non_negative not in (None, False, True, "nndsvd", "nndsvda"):
        raise ValueError(f'Invalid nntype parameter: got {non_negative} instead of one of '
                         '("nndsvd", "nndsvda")')
    _check_method(method)
    x, _ = to_device(tensor)
    x = x.contiguous()
    if mask is not None and n_eigenvecs is not None:
        m = torch.as_tensor(mask).to(device=x.device, dtype=x.dtype).expand(x.shape).contiguous()
        x = x.clone()
        U, S, V = _svd_any(x, mode, n_eigenvecs, method, random_state, flip=False)
        for _ in range(int(n_iter_mask_imputation)):
            _refill(x, m, mode, U, S, V)
            U, S, V = _svd_any(x, mode, n_eigenvecs, method, random_state, flip=False)
        if flip_sign:
            U = _flip_columns(U)
    else:
        U, S, _ = _svd_any(x, mode, n_eigenvecs, method, random_state, flip=flip_sign)
    if non_negative not in (None, False):
        U = _nndsvd_unfolding(x, mode, U, S, "nndsvda" if non_negative is True else non_negative)
    return U, S


def _svd_any(x, mode, n_eigenvecs, method, random_state, flip):
    """(U, S, V) of unfold(x, mode) by the randomised range finder, or (U, S,
    None) by the Gram eigensolver (whose V is never needed: U diag(S) V is
    U U^T M there)."""
    rows = x.shape[mode]
    cols = x.numel() // max(1, rows)
    if method == "randomized_svd":
        from .base import unfold
        U, S, V = randomized_svd(x if x.ndim == 2 and mode == 0 else unfold(x, mode),
                                 n_eigenvecs=n_eigenvecs, random_state=random_state)
        if flip:
            U, V = svd_flip(U, V)
        return U, S, V
    ucols, scount = _n_eigenvecs(rows, cols, n_eigenvecs)
    U, S = _svd_unfolding_raw(x, mode, ucols, flip=flip)
    return U, S[:scount], None


def _refill(x, mask, mode, U, S, V):
    """x = x * mask + R * (1 - mask) in place (``tlgb_mask_impute``), R the
    rank-k reconstruction U diag(S) V of the mode-`mode` unfolding M of x
    (tensorly/tenalg/svd.py:431-439).  With the Gram eigensolver's exact
    singular vectors R = U U^T M, two mode products; the randomised SVD's V
    is only approximately M's, so there R is formed from U, S and V and
    folded back."""
    from .tenalg import _mode_dot_cuda
    k = int(S.shape[0])
    Uk = U[:, :k].contiguous()
    if V is None:
        rec = _mode_dot_cuda(_mode_dot_cuda(x, Uk, mode, True), Uk, mode, False)
    else:
        from .base import fold
        from .decomposition import _mat_nn, _scale_columns
        rec_m = _mat_nn(_scale_columns(Uk, S.contiguous()), V[:k].contiguous())
        rec = rec_m if (x.ndim == 2 and mode == 0) else fold(rec_m, mode, tuple(x.shape))
    lib = _lib.lib()
    ws = workspace(int(lib.tlgb_mask_impute_workspace_bytes()), x.device)
    norms = torch.empty(2, dtype=torch.float64, device=x.device)
    _lib.check(lib.tlgb_mask_impute(dtype_code(x), ptr(x), ptr(mask), ptr(rec.contiguous()),
                                    x.numel(), ptr(norms), ptr(ws), ws.numel(), stream_of(x)))


def _flip_columns(U):
    """svd_flip's U-based sign rule (tensorly/tenalg/svd.py:13-65) on U alone."""
    Ut, _ = svd_flip(U, U[:0].t().contiguous())
    return Ut


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


def randomized_svd(matrix, n_eigenvecs=None, n_oversamples=5, n_iter=2, random_state=None,
                   **kwargs):
    """Truncated randomised SVD (tensorly/tenalg/svd.py:288-357, Halko et al.
    2009, algorithms 4.4 and 5.1): the reference's Gaussian test matrix drawn
    from ``random_state`` on the host, then on the GPU the range finder's
    products (``tlgb_gemm``) and Householder QRs (``tlgb_qr``, NumPy's column
    signs), and the truncated SVD of the reduced matrix.  The reference's
    choice of transposing a wide matrix is kept.  The QR'd blocks must be
    tall and at most 256 columns wide."""
    from .decomposition import _mat_nn, _mat_tn, _mat_nt
    from .parafac2 import _qr
    from .random import check_random_state
    m, pl = to_device(matrix)
    if m.ndim != 2:
        raise ValueError("randomized_svd expects a matrix")
    m = m.contiguous()
    dim_1, dim_2 = int(m.shape[0]), int(m.shape[1])
    min_dim, max_dim = min(dim_1, dim_2), max(dim_1, dim_2)
    if n_eigenvecs is None:
        n_eigenvecs = max_dim
    if n_eigenvecs > max_dim:
        warnings.warn(f"Trying to compute SVD with n_eigenvecs={n_eigenvecs}, which is larger "
                      f"than max(matrix.shape)={max_dim}. Setting n_eigenvecs to {max_dim}.")
        n_eigenvecs = max_dim
    n_dims = min(n_eigenvecs + n_oversamples, max_dim)
    transpose = ((dim_1 > dim_2 and n_eigenvecs > min(min_dim, n_dims))
                 or (dim_1 < dim_2 and n_eigenvecs < min(min_dim, n_dims)))
    a = m.t().contiguous() if transpose else m          # the matrix whose range is found
    ra, ca = int(a.shape[0]), int(a.shape[1])
    if n_dims > min(ra, ca) or n_dims > 256:
        raise NotImplementedError("randomized_svd: the range finder's blocks must be tall and at "
                                  "most 256 columns wide")
    rng = check_random_state(random_state)
    g = torch.from_numpy(rng.normal(size=(ca, n_dims))).to(device=m.device, dtype=m.dtype)
    q = _qr(_mat_nn(a, g))
    for _ in range(int(n_iter)):
        q = _qr(_mat_tn(a, q))
        q = _qr(_mat_nn(a, q))
    if transpose:
        # matrix_reduced = (Q^H A)^T = M Q (dim_1 x n_dims); V = V_r Q^T
        U, S, V = truncated_svd(_mat_nn(m, q), n_eigenvecs=n_eigenvecs)
        V = _mat_nt(V, q)
    else:
        U, S, V = truncated_svd(_mat_tn(q, m), n_eigenvecs=n_eigenvecs)
        U = _mat_nn(q, U)
    return pl.back(U), pl.back(S), pl.back(V)


def svd_interface(matrix, method="truncated_svd", n_eigenvecs=None, flip_sign=True,
                  u_based_flip_sign=True, non_negative=None, mask=None,
                  n_iter_mask_imputation=5, **kwargs):
    """tensorly/tenalg/svd.py:366-447: 'truncated_svd' / 'symeig_svd' (Gram
    eigensolver) or 'randomized_svd', the mask refill loop (``:431-439``) and
    svd_flip.  The non-negative post-processing is not supported here
    (``svd_interface_unfolding`` provides it for tensor unfoldings)."""
    if non_negative not in (None, False):
        raise NotImplementedError("non-negative SVD of a matrix is not supported")
    _check_method(method)
    m, pl = to_device(matrix)
    if m.ndim != 2:
        raise ValueError("svd_interface expects a matrix")

    def svd_fun(a):
        if method == "randomized_svd":
            return randomized_svd(a, n_eigenvecs=n_eigenvecs, **kwargs)
        return truncated_svd(a, n_eigenvecs=n_eigenvecs)

    if mask is not None and n_eigenvecs is not None:
        m = m.contiguous().clone()
        mk = torch.as_tensor(mask).to(device=m.device, dtype=m.dtype).expand(m.shape).contiguous()
        U, S, V = svd_fun(m)
        for _ in range(int(n_iter_mask_imputation)):
            _refill(m, mk, 0, U, S, V)
            U, S, V = svd_fun(m)
    else:
        U, S, V = svd_fun(m.contiguous())
    if flip_sign:
        U, V = svd_flip(U, V, u_based_decision=u_based_flip_sign)
    return pl.back(U), pl.back(S), pl.back(V)
