"""PARAFAC2 (tensorly/decomposition/_parafac2.py, tensorly/parafac2_tensor.py).

The reference's algorithm, composed of the library's kernels:

* the projections P_k = (U Vh)^T of M_k = B (A_k * C)^T X_k^T are the polar
  factor M_k^T (M_k M_k^T)^(-1/2), from the R x R eigenproblem of M_k M_k^T
  (``tlgb_sym_eig``) and ``tlgb_gemm`` products; for a full-rank M_k this is
  the reference's U Vh (the polar factor is unique);
* the projected slices P_k^T X_k feed ``parafac`` (the GPU CP-ALS) for
  ``n_iter_parafac`` sweeps from the current factors;
* the line search (``_BroThesisLineSearch``) extrapolates with ``tlgb_lerp``;
* the error is the reference's expansion (:300-362) on the GPU;
* ``nn_modes``: the projected slices feed ``non_negative_parafac_hals``
  (HALS on the constrained modes, least squares on the others) and the line
  search clips the non-negative modes (``tlgb_clip_min``);
* masks: missing entries start at their slice's observed mean (or the given
  model) and are refilled from the model after every iteration
  (``tlgb_mask_where``); the error is then the masked residual
  (``tlgb_masked_sq_diff``);
* the random start draws as the reference (uniform blocks, then random_cp)
  and orthonormalises with ``tlgb_qr`` (LAPACK's Householder conventions,
  so the signs are NumPy's).
"""

import ctypes
import math

import torch

from . import _lib
from ._tensor import dtype_code, like, ptr, stream_of, to_device, workspace
from .random import check_random_state


class Parafac2Tensor:
    """(weights, factors, projections) triple; tensorly/parafac2_tensor.py:12-92."""

    def __init__(self, parafac2_tensor):
        weights, factors, projections = parafac2_tensor
        self.weights = weights
        self.factors = list(factors)
        self.projections = list(projections)
        self.rank = int(self.factors[0].shape[1])

    def __getitem__(self, i):
        return (self.weights, self.factors, self.projections)[i]

    def __iter__(self):
        return iter((self.weights, self.factors, self.projections))

    def __len__(self):
        return 3

    def to_slices(self):
        return parafac2_to_slices(self)

    def to_tensor(self):
        return parafac2_to_tensor(self)


def _mm(M, N, K, A, sam, sak, B, sbk, sbn, out=None):
    C = out if out is not None else torch.empty((M, N), dtype=A.dtype, device=A.device)
    _lib.check(_lib.lib().tlgb_gemm(dtype_code(A), M, N, K, A.data_ptr(), sam, sak, B.data_ptr(),
                                    sbk, sbn, C.data_ptr(), stream_of(A)))
    return C


def _nn(A, B, out=None):      # A B
    A, B = A.contiguous(), B.contiguous()
    return _mm(A.shape[0], B.shape[1], A.shape[1], A, A.shape[1], 1, B, B.shape[1], 1, out)


def _nt(A, B, out=None):      # A B^T
    A, B = A.contiguous(), B.contiguous()
    return _mm(A.shape[0], B.shape[0], A.shape[1], A, A.shape[1], 1, B, 1, B.shape[1], out)


def _tn(A, B, out=None):      # A^T B
    A, B = A.contiguous(), B.contiguous()
    return _mm(A.shape[1], B.shape[1], A.shape[0], A, 1, A.shape[1], B, B.shape[1], 1, out)


def _scale_cols(m, s):
    from .tenalg import _khatri_rao_raw
    return _khatri_rao_raw([m.contiguous()], weights=s.contiguous())


def _dot(a, b):
    lib = _lib.lib()
    ws = workspace(lib.tlgb_dot_workspace_bytes(), a.device)
    out = torch.empty(1, dtype=torch.float64, device=a.device)
    a, b = a.contiguous(), b.contiguous()
    _lib.check(lib.tlgb_dot(dtype_code(a), a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(),
                            ptr(ws), ws.numel(), stream_of(a)))
    return float(out.item())


def _lerp(x, y, s):
    out = torch.empty_like(x)
    _lib.check(_lib.lib().tlgb_lerp(dtype_code(x), x.contiguous().data_ptr(),
                                    y.contiguous().data_ptr(), x.numel(), float(s),
                                    out.data_ptr(), stream_of(x)))
    return out


def _inv_sqrt(x):
    out = torch.empty_like(x)
    _lib.check(_lib.lib().tlgb_inv_sqrt(dtype_code(x), x.contiguous().data_ptr(), x.numel(),
                                        out.data_ptr(), stream_of(x)))
    return out


def _qr(a):
    lib = _lib.lib()
    m, n = int(a.shape[0]), int(a.shape[1])
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_qr_workspace_size(dtype_code(a), m, n, ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, a.device)
    q = torch.empty((m, n), dtype=a.dtype, device=a.device)
    _lib.check(lib.tlgb_qr(dtype_code(a), a.contiguous().data_ptr(), m, n, q.data_ptr(), ptr(ws),
                           ws.numel(), stream_of(a)))
    return q


def _transpose(m):
    from .base import unfold
    return unfold(m, 1)


def _eig(g):
    """All eigenpairs of a symmetric R x R matrix, largest first."""
    lib = _lib.lib()
    n = int(g.shape[0])
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_sym_eig_workspace_size(dtype_code(g), n, n, ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, g.device)
    u = torch.empty((n, n), dtype=g.dtype, device=g.device)
    ev = torch.empty(n, dtype=g.dtype, device=g.device)
    _lib.check(lib.tlgb_sym_eig(dtype_code(g), g.contiguous().data_ptr(), n, n, u.data_ptr(),
                                ev.data_ptr(), 0, ptr(ws), ws.numel(), stream_of(g)))
    return u, ev


def _compute_projections(slices, factors):
    """tensorly/decomposition/_parafac2.py:158-171 as polar factors."""
    A, B, C = factors
    out = []
    for k, x in enumerate(slices):
        lhs = _nt(B, _scale_cols(C, A[k]))                 # B (A_k * C)^T   (R x J)
        m = _nt(lhs, x)                                    # lhs X_k^T        (R x I_k)
        u, ev = _eig(_nt(m, m))
        w = _nt(_scale_cols(u, _inv_sqrt(ev)), u)          # (M M^T)^(-1/2)
        out.append(_tn(m, w))                              # M^T W            (I_k x R)
    return out


def _project(slices, projections):
    """tensorly/decomposition/_parafac2.py:174-178."""
    R, J = int(projections[0].shape[1]), int(slices[0].shape[1])
    y = torch.empty((len(slices), R, J), dtype=slices[0].dtype, device=slices[0].device)
    for k, (x, p) in enumerate(zip(slices, projections)):
        _tn(p, x, out=y[k])
    return y


def _sum(x):
    lib = _lib.lib()
    ws = workspace(256 * 8, x.device)
    total = torch.zeros(1, dtype=torch.float64, device=x.device)
    _lib.check(lib.tlgb_sum(dtype_code(x), x.data_ptr(), x.numel(), total.data_ptr(), ptr(ws),
                            ws.numel(), stream_of(x)))
    return float(total.item())


def _where(x, mask, rec=None, fill=0.0):
    """x = where(mask == 0, rec or fill, x), in place."""
    _lib.check(_lib.lib().tlgb_mask_where(dtype_code(x), x.data_ptr(), mask.data_ptr(), ptr(rec),
                                          float(fill), x.numel(), stream_of(x)))


def _masked_sq(x, mask, rec):
    """sum((mask * x - mask * rec)^2)."""
    lib = _lib.lib()
    ws = workspace(int(lib.tlgb_dot_workspace_bytes()), x.device)
    out = torch.empty(1, dtype=torch.float64, device=x.device)
    _lib.check(lib.tlgb_masked_sq_diff(dtype_code(x), x.data_ptr(), mask.data_ptr(),
                                       rec.contiguous().data_ptr(), x.numel(), out.data_ptr(),
                                       ptr(ws), ws.numel(), stream_of(x)))
    return float(out.item())


def _clip_min0(x):
    x = x.contiguous().clone()
    _lib.check(_lib.lib().tlgb_clip_min(dtype_code(x), x.data_ptr(), x.numel(), 0.0,
                                        stream_of(x)))
    return x


def _update_imputed(slices, masks, decomposition, method):
    """tensorly/decomposition/_parafac2.py:21-65, in place: 'mode-2' fills the
    missing entries of each slice with the mean of its observed entries,
    'factors' with the model's reconstruction."""
    if method == "mode-2":
        for x, m in zip(slices, masks):
            _where(x, m, fill=_dot(x, m) / _sum(m))
    else:
        for x, m, r in zip(slices, masks, parafac2_to_slices(decomposition)):
            _where(x, m, r.contiguous())


def _reconstruction_error(slices, decomposition, norm_x, projected=None, masks=None):
    """tensorly/decomposition/_parafac2.py:321-396."""
    if masks is not None:
        total = sum(_masked_sq(x, m, r) for x, m, r in
                    zip(slices, masks, parafac2_to_slices(decomposition)))
        return math.sqrt(total)
    weights, (A, B, C), projections = decomposition
    if weights is not None:
        A = _scale_cols(A, weights)
    norm_cmf_sq = 0.0
    inner = 0.0
    ctc = _tn(C, C)
    ct = _transpose(C)
    for i, x in enumerate(slices):
        b_i = _scale_cols(_nn(projections[i], B), A[i])
        if projected is None:
            tmp = _tn(b_i, x)
        else:
            tmp = _tn(_scale_cols(B, A[i]), projected[i])
        inner += _dot(tmp, ct)
        norm_cmf_sq += _dot(_tn(b_i, b_i), ctc)
    return math.sqrt(max(norm_x ** 2 - 2 * inner + norm_cmf_sq, 0.0))


def random_parafac2(shapes, rank, random_state=None, dtype=torch.float64, device="cuda"):
    """tensorly/random/base.py:18-61 (full=False, not normalised): the
    reference's draws on the host, the orthonormalisation by ``tlgb_qr``."""
    rns = check_random_state(random_state)
    if not all(shape[1] == shapes[0][1] for shape in shapes):
        raise ValueError("All matrices must have equal number of columns.")
    projections = [_qr(torch.from_numpy(rns.random_sample((shape[0], rank))).to(device, dtype))
                   for shape in shapes]
    factors = [torch.from_numpy(rns.random_sample((s, rank))).to(device, dtype)
               for s in (len(shapes), rank, shapes[0][1])]
    weights = torch.ones(rank, dtype=dtype, device=device)
    return Parafac2Tensor((weights, factors, projections))


def _initialize(slices, rank, init, svd, random_state):
    """tensorly/decomposition/_parafac2.py:69-155."""
    from .svd import svd_interface
    shapes = [tuple(m.shape) for m in slices]
    dev, dt = slices[0].device, slices[0].dtype
    if isinstance(init, str) and init == "random":
        return random_parafac2(shapes, rank, random_state=random_state, dtype=dt, device=dev)
    if isinstance(init, str) and init == "svd":
        if shapes[0][1] < rank:
            raise ValueError(f"Cannot perform SVD init if rank ({rank}) is greater than the "
                             f"number of columns in each tensor slice ({shapes[0][1]})")
        A = torch.ones((len(slices), rank), dtype=dt, device=dev)
        if sum(s[0] for s in shapes) > shapes[0][1]:
            cat = torch.cat(list(slices), dim=0)             # sum_k X_k^T X_k in one product
            unf = _tn(cat, cat)
        else:
            unf = _transpose(torch.cat(list(slices), dim=0))
        C = svd_interface(unf, n_eigenvecs=rank, method=svd)[0]
        B = torch.eye(rank, dtype=dt, device=dev)
        projections = _compute_projections(slices, (A, B, C))
        return Parafac2Tensor((None, [A, B, C], projections))
    if isinstance(init, str):
        raise ValueError(f'Initialization method "{init}" not recognized')
    w, f, p = init
    return Parafac2Tensor((w, [to_device(x)[0] for x in f], [to_device(x)[0] for x in p]))


class _LineSearch:
    """tensorly/decomposition/_parafac2.py:183-318."""

    def __init__(self, norm_tensor, acc_pow=2.0, max_fail=4, verbose=False, nn_modes=None,
                 masks=None):
        self.norm_tensor = norm_tensor
        self.nn_modes = nn_modes
        self.masks = masks
        self.acc_pow = acc_pow
        self.max_fail = max_fail
        self.acc_fail = 0
        self.verbose = verbose

    def line_step(self, iteration, slices, factors_last, weights, factors, projections,
                  rec_error):
        jump = iteration ** (1.0 / self.acc_pow)
        factors_ls = [_lerp(factors_last[ii], factors[ii], jump) for ii in range(len(factors))]
        if self.nn_modes:
            # `0 in nn_modes` as the reference writes it (a TypeError for 'all')
            if 0 in self.nn_modes:
                factors_ls[0] = _clip_min0(factors_ls[0])
            if 2 in self.nn_modes:
                factors_ls[2] = _clip_min0(factors_ls[2])
        projections_ls = _compute_projections(slices, factors_ls)
        ls_rec_error = _reconstruction_error(slices, (weights, factors_ls, projections_ls),
                                             self.norm_tensor,
                                             masks=self.masks) / self.norm_tensor
        if ls_rec_error < rec_error:
            self.acc_fail = 0
            if self.verbose:
                print(f"Accepted line search jump of {jump}.")
            return factors_ls, projections_ls, ls_rec_error
        self.acc_fail += 1
        if self.verbose:
            print(f"Line search failed for jump of {jump}.")
        if self.acc_fail == self.max_fail:
            self.acc_pow += 1.0
            self.acc_fail = 0
        return factors, projections, rec_error


def parafac2(tensor_slices, rank, n_iter_max=2000, init="random", svd="truncated_svd",
             normalize_factors=False, tol=1.0e-8, nn_modes=None, random_state=None,
             verbose=False, return_errors=False, n_iter_parafac=5, linesearch=True, mask=None):
    """PARAFAC2 by ALS (tensorly/decomposition/_parafac2.py:399-707), same
    signature and returns, with non-negative modes and masks.  f32 slices are
    computed in f64 and the results returned in f32; the caller's slices are
    not modified (the masked refill works on copies)."""
    from warnings import warn
    from .cp_tensor import cp_normalize
    from .decomposition import non_negative_parafac_hals, parafac
    placement = to_device(tensor_slices[0])[1]
    slices = [to_device(t)[0].contiguous() for t in tensor_slices]
    # f32 slices run the f64 path (the R x R eigenproblems of the projections
    # are ill-conditioned in f32) and come back in f32
    out_dtype = slices[0].dtype
    if out_dtype == torch.float32:
        slices = [t.double() for t in slices]
    assert rank <= slices[0].shape[1], (
        f"PARAFAC2 rank ({rank}) cannot be greater than the number of columns in each tensor "
        f"slice ({slices[0].shape[1]}).")
    for ii in range(1, len(slices)):
        assert slices[0].shape[1] == slices[ii].shape[1], \
            "All tensor slices must have the same number of columns."
    dt, dev = slices[0].dtype, slices[0].device
    masks = None if mask is None else [like(m, slices[0]) for m in mask]
    weights, factors, projections = _initialize(slices, rank, init, svd, random_state)
    factors = [f.to(dt).contiguous() for f in factors]
    if masks is not None:
        slices = [t.clone() for t in slices]
        if isinstance(init, str) and init in ("random", "svd"):
            _update_imputed(slices, masks, None, "mode-2")
        else:
            _update_imputed(slices, masks, (weights, factors, projections), "factors")
    if weights is None:
        weights = torch.ones(rank, dtype=dt, device=dev)
    if masks is not None:
        norm_x = math.sqrt(sum(_masked_sq(t, m, torch.zeros_like(t))
                               for t, m in zip(slices, masks)))
    else:
        norm_x = math.sqrt(sum(_dot(t, t) for t in slices))
    ls = (_LineSearch(norm_x, verbose=verbose, nn_modes=nn_modes, masks=masks)
          if linesearch else None)
    if nn_modes is not None and (nn_modes == "all" or 1 in nn_modes):
        warn("Mode `1` of PARAFAC2 fitted with ALS cannot be constrained to be truly "
             "non-negative. See the documentation for more info.")
    rec_errors = []
    for iteration in range(n_iter_max):
        factors[1] = _scale_cols(factors[1], weights.to(dt))
        weights = torch.ones(rank, dtype=dt, device=dev)
        line_iter = bool(ls is not None and iteration % 2 == 0 and iteration > 5)
        if line_iter:
            factors_last = [f.clone() for f in factors]
        projections = _compute_projections(slices, factors)
        projected = _project(slices, projections)
        if nn_modes is None:
            cp = parafac(projected, rank, n_iter_max=n_iter_parafac, init=(weights, factors),
                         svd=svd, normalize_factors=False, tol=1e-100)
        else:
            cp = non_negative_parafac_hals(projected, rank, n_iter_max=n_iter_parafac,
                                           init=(weights, factors), svd=svd, nn_modes=nn_modes,
                                           tol=1e-100)
        factors = [f.contiguous() for f in cp.factors]
        if line_iter:
            factors, projections, rec_errors[-1] = ls.line_step(
                iteration, slices, factors_last, weights, factors, projections, rec_errors[-1])
        if masks is not None:
            _update_imputed(slices, masks, (weights, factors, projections), "factors")
        if normalize_factors:
            weights, factors = cp_normalize((weights, factors))
            factors = list(factors)
        if tol and not line_iter:
            rec_error = _reconstruction_error(slices, (weights, factors, projections), norm_x,
                                              projected, masks)
            rec_errors.append(rec_error / norm_x)
        if tol and iteration >= 1:
            if verbose:
                print(f"PARAFAC2 reconstruction error={rec_errors[-1]}, "
                      f"variation={rec_errors[-2] - rec_errors[-1]}.")
            if abs(rec_errors[-2] - rec_errors[-1]) < tol:
                if verbose:
                    print(f"converged in {iteration} iterations.")
                break
    back = lambda t: placement.back(t.to(out_dtype))
    out = Parafac2Tensor((back(weights), [back(f) for f in factors],
                          [back(p) for p in projections]))
    if return_errors:
        return out, rec_errors
    return out


def parafac2_to_slices(parafac2_tensor):
    """tensorly/parafac2_tensor.py:310-372: slice k = P_k B diag(w * A_k) C^T."""
    weights, (A, B, C), projections = parafac2_tensor
    out = []
    for k, p in enumerate(projections):
        a_k = A[k] if weights is None else _scale_cols(A[k:k + 1], weights)[0]
        bk = _scale_cols(_nn(p, B), a_k)
        out.append(_nt(bk, C))
    return out


def parafac2_to_tensor(parafac2_tensor):
    """tensorly/parafac2_tensor.py:375-429: the slices stacked (zero padded to
    the longest)."""
    slices = parafac2_to_slices(parafac2_tensor)
    rows = max(int(s.shape[0]) for s in slices)
    out = torch.zeros((len(slices), rows, int(slices[0].shape[1])), dtype=slices[0].dtype,
                      device=slices[0].device)
    for k, s in enumerate(slices):
        out[k, :s.shape[0]].copy_(s)
    return out


class Parafac2:
    """sklearn-style wrapper of ``parafac2`` (tensorly/decomposition/_parafac2.py:710-)."""

    def __init__(self, rank, n_iter_max=2000, init="random", svd="truncated_svd",
                 normalize_factors=False, tol=1e-8, nn_modes=None, random_state=None,
                 verbose=False, return_errors=False, n_iter_parafac=5, linesearch=True):
        self.rank = rank
        self.n_iter_max = n_iter_max
        self.init = init
        self.svd = svd
        self.normalize_factors = normalize_factors
        self.tol = tol
        self.nn_modes = nn_modes
        self.random_state = random_state
        self.verbose = verbose
        self.return_errors = return_errors
        self.n_iter_parafac = n_iter_parafac
        self.linesearch = linesearch

    def fit_transform(self, tensor):
        self.decomposition_, self.errors_ = parafac2(
            tensor, self.rank, n_iter_max=self.n_iter_max, init=self.init, svd=self.svd,
            normalize_factors=self.normalize_factors, tol=self.tol, nn_modes=self.nn_modes,
            random_state=self.random_state, verbose=self.verbose, return_errors=True,
            n_iter_parafac=self.n_iter_parafac, linesearch=self.linesearch)
        return self.decomposition_

    def fit(self, tensor):
        self.fit_transform(tensor)
        return self
