"""Drop-in ``parafac`` / ``CP`` (tensorly/decomposition/_cp.py) and
``tucker`` / ``partial_tucker`` / ``Tucker`` (tensorly/decomposition/_tucker.py)
running on the GB300 library.

The whole ALS sweep loop runs in the library (``tlgb_cp_als``); Python only
prepares the initial factors, the options and the workspace.  Unsupported
options raise ``NotImplementedError``; there is no CPU fallback.
"""

import ctypes
import math
import warnings

import numpy as np
import torch

from . import _lib
from ._tensor import MAX_MODES, dtype_code, like, ptr, stream_of, to_device, workspace
from .cp_tensor import (CPTensor, TuckerTensor, cp_normalize, validate_cp_rank,
                        validate_tucker_rank)
from .random import check_random_state


class DecompositionMixin:
    """tensorly/decomposition/_base_decomposition.py:5-13."""

    def fit(self, tensor, **kwargs):
        _ = self.fit_transform(tensor, **kwargs)
        return self

    def __repr__(self):
        return f"{self.__class__.__name__} decomposition of rank {self.rank}."


# ----------------------------------------------------------------------------
# CP
# ----------------------------------------------------------------------------
def initialize_cp(tensor, rank, init="svd", svd="truncated_svd", non_negative=False,
                  random_state=None, normalize_factors=False, mask=None, svd_mask_repeats=5):
    """Initial CP tensor (tensorly/decomposition/_cp.py:26-137) on the tensor's device.

    ``'random'``: the reference's host draws (random/base.py:104), copied once.
    ``'svd'``: leading left singular vectors of each unfolding from the
    library's f64 Gram eigensolver, sign-fixed like svd_flip; mode 0 scaled
    by the singular values; random columns appended when a mode is shorter
    than the rank (``:90-96``).
    A CPTensor / (weights, factors): weights folded in as their geometric
    mean (``:102-126``).
    """
    x, _ = to_device(tensor)
    rng = check_random_state(random_state)
    if isinstance(init, str) and init == "random":
        factors = [torch.from_numpy(rng.random_sample((int(s), int(rank)))).to(x.device, x.dtype)
                   for s in x.shape]
        kt = CPTensor((None, factors))
    elif isinstance(init, str) and init == "svd":
        from .svd import svd_interface_unfolding
        factors = []
        for mode in range(x.ndim):
            # the reference passes no random_state here: a randomised SVD draws
            # from NumPy's global generator
            U, S = svd_interface_unfolding(x, mode, n_eigenvecs=rank, method=svd,
                                           non_negative=non_negative, mask=mask,
                                           n_iter_mask_imputation=svd_mask_repeats)
            if mode == 0:
                idx = min(rank, S.shape[0])
                U = U.clone()
                U[:, :idx] = _scale_columns(U[:, :idx], S[:idx])
            if x.shape[mode] < rank:
                rp = torch.from_numpy(rng.random_sample((U.shape[0], rank - x.shape[mode])))
                U = torch.cat([U, rp.to(x.device, x.dtype)], dim=1)
            factors.append(U[:, :rank].contiguous())
        kt = CPTensor((None, factors))
    elif isinstance(init, (tuple, list, CPTensor)):
        try:
            if normalize_factors is True:
                warnings.warn("It is not recommended to initialize a tensor with normalizing. "
                              "Consider normalizing the tensor before using this function")
            weights, factors = init
            factors = [like(f, x) for f in factors]
            if weights is None:
                return CPTensor((None, factors))
            w = like(weights, x)
            if bool((w == 1).all()):
                return CPTensor((None, factors))
            avg = float(torch.prod(w.double()) ** (1.0 / w.shape[0]))
            return CPTensor((None, [_scale_all(f, avg) for f in factors]))
        except ValueError:
            raise ValueError("If initialization method is a mapping, then it must "
                             "be possible to convert it to a CPTensor instance")
    else:
        raise ValueError(f'Initialization method "{init}" not recognized')
    if non_negative:
        kt.factors = [f.abs() for f in kt.factors]
    if normalize_factors:
        kt = cp_normalize(kt)
    return kt


def _scale_columns(m, s):
    from .tenalg import _khatri_rao_raw
    return _khatri_rao_raw([m.contiguous()], weights=s)


def _scale_all(m, scalar):
    from .tenalg import _khatri_rao_raw
    w = torch.full((m.shape[1],), scalar, dtype=m.dtype, device=m.device)
    return _khatri_rao_raw([m.contiguous()], weights=w)


_PRECISIONS = {"native": _lib.TLGB_PREC_NATIVE, "bf16": _lib.TLGB_PREC_BF16}


def parafac(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
            normalize_factors=False, orthogonalise=False, tol=1e-8, random_state=None,
            verbose=0, return_errors=False, sparsity=None, l2_reg=0, mask=None,
            cvg_criterion="abs_rec_error", fixed_modes=None, svd_mask_repeats=5,
            linesearch=False, callback=None, *, precision="native", refine_sweeps=1,
            check_every=8, use_graph=False, mttkrp_times=None):
    """CP decomposition by ALS (tensorly/decomposition/_cp.py:230-543).

    Same signature, return types and stopping rule as the reference.  The
    keyword-only arguments select the GB300 execution: ``precision='bf16'``
    stores an f32 tensor in bf16 and runs the tensor-core MTTKRP for all but
    the last ``refine_sweeps`` sweeps, which run in f32; ``check_every`` is the
    number of sweeps between host reads of the device-side stop flag (the
    sweeps are launched a group ahead of those reads); ``use_graph`` replays
    groups of captured sweeps as CUDA graphs instead.  If
    ``mttkrp_times`` is a dict, it receives, per sweep kind that ran
    (``'native'``, ``'bf16'``, ``'f32_split'``, ``'closing'``), the list of
    per-mode MTTKRP durations (ms, CUDA events inside the sweep) of the last
    sweep of that kind.
    """
    if sparsity and callback is not None:
        raise NotImplementedError("parafac with both sparsity and a callback is not supported "
                                  "by tensorly_gb300")
    if (linesearch or orthogonalise or mask is not None or sparsity) and precision != "native":
        raise NotImplementedError("parafac line search, orthogonalise, masks and sparsity run "
                                  "at native precision")
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
    x, pl = to_device(tensor)
    if x.ndim < 2 or x.ndim > MAX_MODES:
        raise NotImplementedError(f"parafac supports tensors of order 2..{MAX_MODES}")
    rank = validate_cp_rank(tuple(x.shape), rank=rank)
    if tol and cvg_criterion not in ("abs_rec_error", "rec_error"):
        raise TypeError("Unknown convergence criterion")

    weights, factors = initialize_cp(x, rank, init=init, svd=svd, random_state=random_state,
                                     normalize_factors=normalize_factors, mask=mask,
                                     svd_mask_repeats=svd_mask_repeats)
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    if weights is None:
        weights = torch.ones(rank, dtype=x.dtype, device=x.device)
    else:
        weights = weights.to(x.dtype).contiguous().clone()

    fixed = [] if fixed_modes is None else list(fixed_modes)
    if fixed == list(range(x.ndim)):
        return _place_cp(weights, factors, pl)
    if x.ndim - 1 in fixed:
        warnings.warn("You asked for fixing the last mode, which is not supported.\n The last "
                      "mode will not be fixed. Consider using tl.moveaxis()")
        fixed.remove(x.ndim - 1)
    fixed_mask = 0
    for m in fixed:
        fixed_mask |= 1 << int(m)

    if linesearch or orthogonalise or mask is not None or sparsity:
        return _parafac_host_loop(x, pl, rank, weights, factors, n_iter_max=n_iter_max,
                                  orthogonalise=orthogonalise, tol=tol, verbose=verbose,
                                  return_errors=return_errors, l2_reg=l2_reg,
                                  cvg_criterion=cvg_criterion, fixed_mask=fixed_mask,
                                  normalize_factors=normalize_factors, linesearch=linesearch,
                                  callback=callback, mask=mask, sparsity=sparsity)

    lib = _lib.lib()
    opts = _lib.CpAlsOptions()
    lib.tlgb_cp_als_default_options(ctypes.byref(opts))
    opts.n_iter_max = int(n_iter_max)
    opts.tol = float(tol) if tol else 0.0
    opts.l2_reg = float(l2_reg) if l2_reg else 0.0
    opts.cvg_criterion = 1 if cvg_criterion == "rec_error" else 0
    opts.normalize_factors = 1 if normalize_factors else 0
    opts.fixed_modes = fixed_mask
    opts.precision = _PRECISIONS[precision]
    opts.refine_sweeps = int(refine_sweeps)
    opts.check_every = int(check_every)
    opts.use_graph = 1 if use_graph else 0
    times = None
    if mttkrp_times is not None:
        times = (ctypes.c_double * (_lib.CP_ALS_SWEEP_KINDS * MAX_MODES))()
        opts.mttkrp_ms = ctypes.cast(times, ctypes.POINTER(ctypes.c_double))

    failure = []
    if callback is not None:
        def _cb(_user, iteration, rec_error):
            try:
                cp = _place_cp(weights.clone(), [f.clone() for f in factors], pl)
                ret = callback(cp, float(rec_error))
                return 1 if (iteration >= 0 and ret is True) else 0
            except BaseException as e:  # re-raised after the library returns
                failure.append(e)
                return 1
        c_cb = _lib.SWEEP_CALLBACK(_cb)
        opts.callback = c_cb
    shape = _lib.i64_array(x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_als_workspace_size(dtype_code(x), x.ndim, shape, rank,
                                              ctypes.byref(opts), ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    errs = (ctypes.c_double * max(1, int(n_iter_max)))()
    n_err = ctypes.c_int(0)
    rc = lib.tlgb_cp_als(dtype_code(x), ptr(x), x.ndim, shape, rank,
                         _lib.ptr_array([ptr(f) for f in factors]), ptr(weights),
                         ctypes.byref(opts), errs, ctypes.byref(n_err), ptr(ws), ws.numel(),
                         stream_of(x))
    if failure:
        raise failure[0]
    _lib.check(rc)
    if times is not None:
        for kind, name in enumerate(_lib.SWEEP_KIND_NAMES):
            row = [float(times[kind * MAX_MODES + m]) for m in range(x.ndim)]
            if any(v != 0.0 for v in row):
                mttkrp_times[name] = row
    rec_errors = [float(errs[i]) for i in range(n_err.value)]
    if verbose:
        for i, e in enumerate(rec_errors):
            print(f"iteration {i}, reconstruction error: {e}")
    cp = _place_cp(weights, factors, pl)
    if return_errors:
        return cp, rec_errors
    return cp


def _parafac_host_loop(x, pl, rank, weights, factors, *, n_iter_max, orthogonalise, tol,
                       verbose, return_errors, l2_reg, cvg_criterion, fixed_mask,
                       normalize_factors, linesearch, callback, mask=None, sparsity=None):
    """parafac with orthogonalisation, the line search, a mask and / or a
    sparse component (tensorly/decomposition/_cp.py:392-401, :430-478,
    :194-215, :441-446, :372-377, :532-538): the reference's iteration loop
    on the host around single-sweep ``tlgb_cp_als`` calls.

    With ``sparsity`` (a fraction of the entries, or a count) every error is
    the norm of R - sparsify(R) for the residual R = X - [[w; A]], the model
    formed by ``tlgb_cp_to_tensor`` and the card-th largest |R| found by the
    radix select of ``tlgb_sparse_residual``; the sweeps themselves are the
    plain ones, as in the reference, and the sparse component of the final
    model is returned beside it.

    With a mask the sweeps run on a working copy of the tensor whose missing
    entries are refilled from the model after every sweep
    (x = x * mask + cp_to_tensor(model) * (1 - mask), ``tlgb_cp_to_tensor`` and
    ``tlgb_mask_impute``); the error is then the norm of the explicit residual
    over the refilled tensor's norm, as the reference's error_calc computes it.

    Per iteration: QR of each factor while ``iteration <= orthogonalise``
    (``tlgb_qr``, LAPACK's sign convention); one ALS sweep in the library,
    which also returns the error from the last mode's MTTKRP; on every even
    iteration after the fifth, the extrapolated model
    ``last + (current - last) * iteration ** (1 / acc_pow)`` (``tlgb_lerp``)
    is scored by the explicit residual (``tlgb_cp_residual_norm``) and kept if
    it lowers the error.  Line-search iterations record no error, as in the
    reference.  The stop test and the normalisation follow ``:505-530``."""
    from .parafac2 import _lerp, _qr
    if orthogonalise and not isinstance(orthogonalise, int):
        orthogonalise = n_iter_max
    lib = _lib.lib()
    opts = _lib.CpAlsOptions()
    lib.tlgb_cp_als_default_options(ctypes.byref(opts))
    opts.n_iter_max = 1
    opts.tol = 0.0
    opts.l2_reg = float(l2_reg) if l2_reg else 0.0
    opts.cvg_criterion = 0
    opts.normalize_factors = 0
    opts.fixed_modes = fixed_mask
    opts.precision = _lib.TLGB_PREC_NATIVE
    opts.use_graph = 0
    shape = _lib.i64_array(x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_als_workspace_size(dtype_code(x), x.ndim, shape, rank,
                                              ctypes.byref(opts), ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    errs = (ctypes.c_double * 1)()
    n_err = ctypes.c_int(0)

    def sweep():
        # `x` is read at call time: with a mask it is the refilled working tensor
        _lib.check(lib.tlgb_cp_als(dtype_code(x), ptr(x), x.ndim, shape, rank,
                                   _lib.ptr_array([ptr(f) for f in factors]), ptr(weights),
                                   ctypes.byref(opts), errs, ctypes.byref(n_err), ptr(ws),
                                   ws.numel(), stream_of(x)))
        return float(errs[0])

    norm_tensor = _norm_on_device(x)
    n_entries = x.numel()
    card = None
    if sparsity:
        card = int(sparsity * n_entries) if isinstance(sparsity, float) else int(sparsity)
        # sparsify_tensor's bound is sort(|R|)[-card]: the card-th largest for
        # card >= 1, position -card from the smallest otherwise
        if card >= n_entries:
            sel_k = n_entries + 1                      # keeps the whole residual
        elif card >= 1:
            sel_k = card
        elif -card < n_entries:
            sel_k = n_entries + card
        else:
            raise IndexError(f"index {-card} is out of bounds for axis 0 with size {n_entries}")
        sel_ws = workspace(int(lib.tlgb_sparse_residual_workspace_bytes()), x.device)
        sel_out = torch.empty(1, dtype=torch.float64, device=x.device)
    if mask is not None or sparsity:
        rec = torch.empty_like(x)
        dims = _lib.i64_array(x.shape)
        rec_bytes = ctypes.c_size_t(0)
        _lib.check(lib.tlgb_cp_to_tensor_workspace_size(dtype_code(x), x.ndim, dims, rank,
                                                        ctypes.byref(rec_bytes)))
        rec_ws = workspace(rec_bytes.value, x.device)
    if mask is not None:
        mask_t = like(mask, x).expand(x.shape).contiguous()
        x = x.clone()   # the refilled working tensor; the caller's tensor is not modified
        imp_ws = workspace(int(lib.tlgb_mask_impute_workspace_bytes()), x.device)
        imp_out = torch.empty(2, dtype=torch.float64, device=x.device)

    def model(w, fs):
        _lib.check(lib.tlgb_cp_to_tensor(dtype_code(x), x.ndim, dims, rank,
                                         _lib.ptr_array([ptr(f) for f in fs]), ptr(w), None,
                                         ptr(rec), ptr(rec_ws), rec_ws.numel(), stream_of(x)))

    def sparse_error(target, sparse_out=None):
        """||R - sparsify(R)|| for R = target - rec (the model already in rec)."""
        _lib.check(lib.tlgb_sparse_residual(dtype_code(x), ptr(target), ptr(rec), n_entries,
                                            sel_k, ptr(sel_out), ptr(sparse_out), ptr(sel_ws),
                                            sel_ws.numel(), stream_of(x)))
        return float(sel_out.item())

    def refill(target, w, fs):
        """target = target * mask + [[w; fs]] * (1 - mask); (||target||, the
        error of [[w; fs]] against it: ||target - [[w; fs]]||, or with a sparse
        component ||R - sparsify(R)||)."""
        model(w, fs)
        _lib.check(lib.tlgb_mask_impute(dtype_code(x), ptr(target), ptr(mask_t), ptr(rec),
                                        target.numel(), ptr(imp_out), ptr(imp_ws),
                                        imp_ws.numel(), stream_of(x)))
        v = imp_out.cpu()
        if sparsity:
            return float(v[0]), sparse_error(target)
        return float(v[0]), float(v[1])

    def explicit_error(w, fs):
        """The unmasked error of [[w; fs]]: explicit residual, sparse if asked."""
        if sparsity:
            model(w, fs)
            return sparse_error(x)
        return _residual_norm(x, fs, w)

    if callback is not None:
        if mask is not None:
            # the reference refills a copy for this first error and keeps its norm
            norm_tensor, unnorm0 = refill(x.clone(), weights, factors)
        else:
            unnorm0 = _residual_norm(x, factors, weights)
        callback(_place_cp(weights.clone(), [f.clone() for f in factors], pl),
                 unnorm0 / norm_tensor)
    acc_pow, acc_fail, max_fail = 2.0, 0, 4
    rec_errors = []
    rec_error = None
    for iteration in range(n_iter_max):
        if orthogonalise and iteration <= orthogonalise:
            factors = [_qr(f) if min(f.shape) >= rank else f for f in factors]
        if linesearch and iteration % 2 == 0:
            factors_last = [f.clone() for f in factors]
            weights_last = weights.clone()
        fast_error = sweep()
        line_iter = bool(linesearch and iteration % 2 == 0 and iteration > 5)
        if not line_iter:
            if mask is not None:
                norm_tensor, unnorm = refill(x, weights, factors)
            elif sparsity:
                unnorm = explicit_error(weights, factors)
            else:
                unnorm = fast_error * norm_tensor
        else:
            if mask is not None:
                refill(x, weights, factors)
            jump = iteration ** (1.0 / acc_pow)
            new_weights = _lerp(weights_last, weights, jump)
            new_factors = [_lerp(a, b, jump) for a, b in zip(factors_last, factors)]
            if mask is not None:
                x_new = x.clone()
                new_norm, new_error = refill(x_new, new_weights, new_factors)
            else:
                new_norm, new_error = norm_tensor, explicit_error(new_weights, new_factors)
            if new_error / new_norm < rec_errors[-1]:
                factors, weights = new_factors, new_weights
                if mask is not None:
                    x = x_new
                norm_tensor = new_norm
                unnorm = new_error
                acc_fail = 0
                if verbose:
                    print(f"Accepted line search jump of {jump}.")
            else:
                if mask is not None:
                    norm_tensor, unnorm = refill(x, weights, factors)
                elif sparsity:
                    unnorm = explicit_error(weights, factors)
                else:
                    unnorm = fast_error * norm_tensor
                acc_fail += 1
                if verbose:
                    print(f"Line search failed for jump of {jump}.")
                if acc_fail == max_fail:
                    acc_pow += 1.0
                    acc_fail = 0
        if not line_iter:
            rec_error = unnorm / norm_tensor
            rec_errors.append(rec_error)
        if callback is not None:
            ret = callback(_place_cp(weights.clone(), [f.clone() for f in factors], pl),
                           rec_error)
            if ret is True:
                break
        if tol and iteration >= 1:
            dec = rec_errors[-2] - rec_errors[-1]
            if verbose:
                print(f"iteration {iteration}, reconstruction error: {rec_error}, "
                      f"decrease = {dec}")
            stop = abs(dec) < tol if cvg_criterion == "abs_rec_error" else dec < tol
            if stop:
                break
        if normalize_factors:
            weights, factors = cp_normalize((weights, factors))
            factors = list(factors)
    cp = _place_cp(weights, factors, pl)
    if sparsity:
        # the sparse component of the final model against the (refilled) tensor
        model(weights, factors)
        sparse = torch.empty_like(x)
        sparse_error(x, sparse)
        cp = (cp, pl.back(sparse))
    if return_errors:
        return cp, rec_errors
    return cp


def _place_cp(weights, factors, pl):
    return CPTensor((pl.back(weights), [pl.back(f) for f in factors]))


class CP(DecompositionMixin):
    """Estimator wrapper of :func:`parafac` (tensorly/decomposition/_cp.py:765-916)."""

    def __init__(self, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                 normalize_factors=False, orthogonalise=False, tol=1e-8, random_state=None,
                 verbose=0, sparsity=None, l2_reg=0, mask=None, cvg_criterion="abs_rec_error",
                 fixed_modes=None, svd_mask_repeats=5, linesearch=False, callback=None):
        self.rank = rank
        self.n_iter_max = n_iter_max
        self.init = init
        self.svd = svd
        self.normalize_factors = normalize_factors
        self.orthogonalise = orthogonalise
        self.tol = tol
        self.random_state = random_state
        self.verbose = verbose
        self.sparsity = sparsity
        self.l2_reg = l2_reg
        self.mask = mask
        self.cvg_criterion = cvg_criterion
        self.fixed_modes = fixed_modes
        self.svd_mask_repeats = svd_mask_repeats
        self.linesearch = linesearch
        self.callback = callback

    def fit_transform(self, tensor):
        cp_tensor, errors = parafac(
            tensor, rank=self.rank, n_iter_max=self.n_iter_max, init=self.init, svd=self.svd,
            normalize_factors=self.normalize_factors, orthogonalise=self.orthogonalise,
            tol=self.tol, random_state=self.random_state, verbose=self.verbose,
            return_errors=True, sparsity=self.sparsity, l2_reg=self.l2_reg, mask=self.mask,
            cvg_criterion=self.cvg_criterion, fixed_modes=self.fixed_modes,
            svd_mask_repeats=self.svd_mask_repeats, linesearch=self.linesearch,
            callback=self.callback)
        self.decomposition_ = cp_tensor
        self.errors_ = errors
        return self.decomposition_


# ----------------------------------------------------------------------------
# Tucker
# ----------------------------------------------------------------------------
def initialize_tucker(tensor, rank, modes, random_state, init="svd", svd="truncated_svd",
                      non_negative=False, mask=None, svd_mask_repeats=5):
    """Initial core and factors (tensorly/decomposition/_tucker.py:25-102).

    ``'svd'``: the leading left singular vectors of each unfolding from the
    library (Gram eigensolver, svd_flip signs), core = X x_n U_n^T.
    ``'random'``: the reference's host draws (core + 0.01), copied once.
    A (core, factors) pair is used as given.  With a mask, each unfolding's
    SVD refills the missing entries ``svd_mask_repeats`` times; the core is
    taken from the tensor as given, as in the reference.
    """
    x, _ = to_device(tensor)
    if isinstance(init, str) and init == "svd":
        from .svd import svd_interface_unfolding
        from .tenalg import multi_mode_dot
        factors = []
        for index, mode in enumerate(modes):
            U, _ = svd_interface_unfolding(x, mode, n_eigenvecs=rank[index], method=svd,
                                           non_negative=non_negative, mask=mask,
                                           n_iter_mask_imputation=svd_mask_repeats,
                                           random_state=random_state)
            factors.append(U)
        core = multi_mode_dot(x, factors, modes=modes, transpose=True)
    elif isinstance(init, str) and init == "random":
        rng = check_random_state(random_state)
        core = torch.from_numpy(rng.random_sample([rank[i] for i in range(len(modes))]) + 0.01)
        core = core.to(x.device, x.dtype)
        factors = [torch.from_numpy(rng.random_sample((x.shape[mode], rank[i]))).to(x.device,
                                                                                    x.dtype)
                   for i, mode in enumerate(modes)]
    else:
        core, factors = init
        core = like(core, x)
        factors = [like(f, x) for f in factors]
    if non_negative is True:
        factors = [f.abs() for f in factors]
        core = core.abs()
    return core, list(factors)


def _hooi(x, rank, modes, factors, n_iter_max, tol, init_svd):
    """Runs tlgb_tucker_hooi; returns (core, factors, errors)."""
    lib = _lib.lib()
    n_modes = len(modes)
    for i, (m, f) in enumerate(zip(modes, factors)):
        if f is not None and tuple(f.shape) != (x.shape[m], int(rank[i])):
            raise ValueError(f"initial factor {i} has shape {tuple(f.shape)}, expected "
                             f"{(x.shape[m], int(rank[i]))} (mode {m}, rank {rank[i]})")
    factors = [f.to(x.dtype).contiguous().clone() if f is not None else
               torch.empty((x.shape[m], rank[i]), dtype=x.dtype, device=x.device)
               for i, (m, f) in enumerate(zip(modes, factors))]
    core_shape = list(x.shape)
    for i, m in enumerate(modes):
        core_shape[m] = int(rank[i])
    core = torch.empty(core_shape, dtype=x.dtype, device=x.device)
    shape = _lib.i64_array(x.shape)
    cmodes = (ctypes.c_int * n_modes)(*[int(m) for m in modes])
    cranks = _lib.i64_array(rank)
    opts = _lib.TuckerOptions()
    lib.tlgb_tucker_default_options(ctypes.byref(opts))
    opts.n_iter_max = int(n_iter_max)
    opts.tol = float(tol) if tol else 0.0
    opts.init_svd = 1 if init_svd else 0
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_tucker_workspace_size(dtype_code(x), x.ndim, shape, n_modes, cmodes,
                                              cranks, ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    errs = (ctypes.c_double * max(1, int(n_iter_max)))()
    n_err = ctypes.c_int(0)
    _lib.check(lib.tlgb_tucker_hooi(dtype_code(x), ptr(x), x.ndim, shape, n_modes, cmodes,
                                    cranks, _lib.ptr_array([ptr(f) for f in factors]), ptr(core),
                                    ctypes.byref(opts), errs, ctypes.byref(n_err), ptr(ws),
                                    ws.numel(), stream_of(x)))
    return core, factors, [float(errs[i]) for i in range(n_err.value)]


def _masked_hooi(x, mask, rank, modes, core, factors, n_iter_max, tol):
    """The masked iteration of tensorly/decomposition/_tucker.py:184-221:
    refill, then one HOOI iteration of the library on the refilled tensor."""
    from .tenalg import multi_mode_dot
    lib = _lib.lib()
    m = torch.as_tensor(mask).to(device=x.device, dtype=x.dtype).expand(x.shape).contiguous()
    norm2 = float(_dot(x, x).item())
    norm_tensor = math.sqrt(norm2)
    cur = x.clone()      # the reference refills its working copy in place every iteration
    ws = workspace(int(lib.tlgb_mask_impute_workspace_bytes()), x.device)
    norms = torch.empty(2, dtype=torch.float64, device=x.device)
    rec_errors = []
    for iteration in range(int(n_iter_max)):
        rec = multi_mode_dot(core, factors, modes=modes).contiguous()
        _lib.check(lib.tlgb_mask_impute(dtype_code(x), ptr(cur), ptr(m), ptr(rec), x.numel(),
                                        ptr(norms), ptr(ws), ws.numel(), stream_of(x)))
        core, factors, _ = _hooi(cur, rank, modes, factors, 1, 0.0, False)
        c2 = float(_dot(core, core).item())
        rec_errors.append(math.sqrt(abs(norm2 - c2)) / norm_tensor)
        if iteration > 1 and tol and abs(rec_errors[-2] - rec_errors[-1]) < tol:
            break
    return core, factors, rec_errors


def partial_tucker(tensor, rank, modes=None, n_iter_max=100, init="svd", tol=10e-5,
                   svd="truncated_svd", random_state=None, verbose=False, mask=None,
                   svd_mask_repeats=5):
    """Partial Tucker decomposition by HOOI (tensorly/decomposition/_tucker.py:105-221).

    Same signature and return value, ``((core, factors), rec_errors)``; the
    iteration runs in the library (``tlgb_tucker_hooi``).  With a mask every
    iteration first refills the missing entries from the current model
    (``tensor * mask + [[core; factors]] * (1 - mask)``, ``tlgb_mask_impute``)
    and runs one library iteration on the refilled tensor; the error uses the
    norm of the tensor as given, as the reference does.
    """
    x, pl = to_device(tensor)
    x = x.contiguous()
    if modes is None:
        modes = list(range(x.ndim))
    if rank is None:
        warnings.warn("No value given for 'rank'. The decomposition will preserve the original "
                      "size.", Warning)
        rank = [x.shape[mode] for mode in modes]
    elif isinstance(rank, int):
        warnings.warn(f"Given only one int for 'rank' instead of a list of {len(modes)} modes. "
                      "Using this rank for all modes.", Warning)
        rank = tuple(rank for _ in modes)
    else:
        rank = tuple(rank)
    modes = [int(m) for m in modes]
    if modes != sorted(modes):
        # the reference applies `skip=index` as a position in the mode-sorted
        # factor list (core_tenalg/n_mode_product.py:117-124), so unsorted
        # modes feed it mismatched factors and end in a shape error
        raise ValueError(f"partial_tucker: modes {modes} are not in ascending order")
    if (isinstance(init, str) and init == "svd" and svd in ("truncated_svd", "symeig_svd")
            and mask is None):
        init_factors = [None] * len(modes)
        core0 = None
        init_svd = True
    else:
        core0, init_factors = initialize_tucker(x, rank, modes, random_state, init=init, svd=svd,
                                                mask=mask, svd_mask_repeats=svd_mask_repeats)
        init_svd = False
    if int(n_iter_max) <= 0:
        if init_svd:
            core0, init_factors = initialize_tucker(x, rank, modes, random_state, init=init,
                                                    svd=svd)
        return (pl.back(core0), [pl.back(f) for f in init_factors]), []
    if mask is not None:
        core, factors, rec_errors = _masked_hooi(x, mask, rank, modes, core0, init_factors,
                                                 n_iter_max, tol)
    else:
        core, factors, rec_errors = _hooi(x, rank, modes, init_factors, n_iter_max, tol,
                                          init_svd)
    if verbose:
        for i in range(2, len(rec_errors)):
            print(f"reconstruction error={rec_errors[i]}, "
                  f"variation={rec_errors[i - 1] - rec_errors[i]}.")
    return (pl.back(core), [pl.back(f) for f in factors]), rec_errors


def tucker(tensor, rank, fixed_factors=None, n_iter_max=100, init="svd", return_errors=False,
           svd="truncated_svd", tol=10e-5, random_state=None, mask=None, verbose=False):
    """Tucker decomposition by HOOI (tensorly/decomposition/_tucker.py:224-345).

    Same signature and return types: a ``TuckerTensor``, or
    ``(TuckerTensor, rec_errors)`` with ``return_errors`` (without
    ``fixed_factors``, as in the reference).
    """
    from .tenalg import multi_mode_dot
    if fixed_factors:
        try:
            (core, factors) = init
        except Exception:
            raise ValueError(f"Got fixed_factor={fixed_factors} but no appropriate Tucker tensor "
                             'was passed for "init".')
        x, pl = to_device(tensor)
        core = like(core, x)
        factors = [like(f, x) for f in factors]
        fixed_factors = sorted(fixed_factors)
        modes_fixed, factors_fixed = zip(*[(i, f) for (i, f) in enumerate(factors)
                                           if i in fixed_factors])
        core = multi_mode_dot(core, list(factors_fixed), modes=list(modes_fixed))
        modes, factors = zip(*[(i, f) for (i, f) in enumerate(factors)
                               if i not in fixed_factors])
        init = (core, list(factors))
        (core, new_factors), rec_errors = partial_tucker(
            x, rank=rank, modes=list(modes), n_iter_max=n_iter_max, init=init, svd=svd, tol=tol,
            random_state=random_state, mask=mask, verbose=verbose)
        factors = list(new_factors)
        for i, e in enumerate(fixed_factors):
            factors.insert(e, factors_fixed[i])
        core = multi_mode_dot(core, list(factors_fixed), modes=list(modes_fixed),
                              transpose=True)
        return TuckerTensor((pl.back(core), [pl.back(f) for f in factors]))
    x, pl = to_device(tensor)
    modes = list(range(x.ndim))
    rank = validate_tucker_rank(tuple(x.shape), rank=rank)
    (core, factors), rec_errors = partial_tucker(
        x, rank=rank, modes=modes, n_iter_max=n_iter_max, init=init, svd=svd, tol=tol,
        random_state=random_state, mask=mask, verbose=verbose)
    tt = TuckerTensor((pl.back(core), [pl.back(f) for f in factors]))
    if return_errors:
        return tt, rec_errors
    return tt


class Tucker(DecompositionMixin):
    """Estimator wrapper of :func:`tucker` (tensorly/decomposition/_tucker.py:697-797)."""

    def __init__(self, rank=None, n_iter_max=100, init="svd", return_errors=False,
                 svd="truncated_svd", tol=10e-5, fixed_factors=None, random_state=None,
                 mask=None, verbose=False):
        self.rank = rank
        self.fixed_factors = fixed_factors
        self.n_iter_max = n_iter_max
        self.init = init
        self.return_errors = return_errors
        self.svd = svd
        self.tol = tol
        self.random_state = random_state
        self.mask = mask
        self.verbose = verbose

    def fit_transform(self, tensor):
        tucker_tensor = tucker(
            tensor, rank=self.rank, fixed_factors=self.fixed_factors, n_iter_max=self.n_iter_max,
            init=self.init, return_errors=self.return_errors, svd=self.svd, tol=self.tol,
            random_state=self.random_state, mask=self.mask, verbose=self.verbose)
        self.decomposition_ = tucker_tensor
        return self.decomposition_

    def __repr__(self):
        return f"Rank-{self.rank} Tucker decomposition via HOOI."


# ----------------------------------------------------------------------------
# Batched CP-ALS
# ----------------------------------------------------------------------------
def non_negative_parafac(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                         tol=10e-7, random_state=None, verbose=0, normalize_factors=False,
                         return_errors=False, mask=None, cvg_criterion="abs_rec_error",
                         fixed_modes=None):
    """Non-negative CP by multiplicative updates
    (tensorly/decomposition/_nn_cp.py:26-183), same signature and returns.

    The initial factors are ``initialize_cp(..., non_negative=True)``: for
    ``init='svd'`` the NNDSVDA form of each unfolding's SVD, then absolute
    values.  The loop runs in ``tlgb_cp_nn_mu``: per free mode, the Hadamard
    product of the other Grams, the MTTKRP and the update
    ``A * clip(M, eps) / clip(A accum, eps)``; with ``tol`` the error of every
    iteration and the reference's stop test.  ``normalize_factors`` and masks
    are not supported.
    """
    if mask is not None:
        raise NotImplementedError("masked non_negative_parafac is not supported by tensorly_gb300")
    if normalize_factors:
        raise NotImplementedError("non_negative_parafac with normalize_factors=True is not "
                                  "supported by tensorly_gb300")
    if tol and n_iter_max > 1 and cvg_criterion not in ("abs_rec_error", "rec_error"):
        raise TypeError("Unknown convergence criterion")   # _nn_cp.py:166-167
    x, placement = to_device(tensor)
    code = dtype_code(x)
    x = x.contiguous()
    rank = validate_cp_rank(tuple(x.shape), rank=rank)
    if x.ndim < 2:
        raise NotImplementedError("non_negative_parafac needs at least two modes")
    _, factors = initialize_cp(x, rank, init=init, svd=svd, non_negative=True,
                               random_state=random_state, normalize_factors=False)
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    fixed = [] if fixed_modes is None else list(fixed_modes)
    if x.ndim - 1 in fixed:
        warnings.warn("You asked for fixing the last mode, which is not supported while tol "
                      "is fixed.\n The last mode will not be fixed. Consider using tl.moveaxis()")
        fixed.remove(x.ndim - 1)
    free = [m for m in range(x.ndim) if m not in fixed]
    lib = _lib.lib()
    shape = (ctypes.c_int64 * x.ndim)(*x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_nn_mu_workspace_size(code, x.ndim, shape, rank, int(n_iter_max),
                                                ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    fptrs = (ctypes.c_void_p * x.ndim)(*[f.data_ptr() for f in factors])
    free_arr = (ctypes.c_int * len(free))(*free)
    errs = (ctypes.c_double * max(1, int(n_iter_max)))()
    n_err = ctypes.c_int(0)
    _lib.check(lib.tlgb_cp_nn_mu(code, x.data_ptr(), x.ndim, shape, fptrs, rank, free_arr,
                                 len(free), int(n_iter_max), float(tol) if tol else 0.0,
                                 0 if cvg_criterion == "abs_rec_error" else 1, errs,
                                 ctypes.byref(n_err), ptr(ws), ws.numel(), stream_of(x)))
    weights = torch.ones(rank, dtype=x.dtype, device=x.device)
    cp = CPTensor((placement.back(weights), [placement.back(f) for f in factors]))
    if return_errors:
        return cp, [float(errs[i]) for i in range(n_err.value)]
    return cp


def non_negative_parafac_hals(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                              tol=10e-8, random_state=None, sparsity_coefficients=None,
                              fixed_modes=None, nn_modes="all", exact=False,
                              normalize_factors=False, verbose=False, return_errors=False,
                              cvg_criterion="abs_rec_error"):
    """Non-negative CP by HALS (tensorly/decomposition/_nn_cp.py:186-377),
    same signature and returns.  The loop runs in ``tlgb_cp_nn_hals``: per
    free mode the Hadamard of the other Grams, the MTTKRP and the
    ``hals_nnls`` row updates (tensorly/solvers/nnls.py:5-150) with their own
    stop test, or, for a mode outside ``nn_modes``, the least-squares update
    of CP-ALS; with ``normalize_factors`` the model is renormalised after
    every updated mode but the last and after every iteration, and the
    weights enter the normal equations and the MTTKRP; with ``tol`` the error
    of every iteration and the outer test.  A fixed last mode is not
    supported."""
    if tol and n_iter_max > 1 and cvg_criterion not in ("abs_rec_error", "rec_error"):
        raise TypeError("Unknown convergence criterion")   # _nn_cp.py:363-364
    x, placement = to_device(tensor)
    code = dtype_code(x)
    x = x.contiguous()
    if x.ndim < 2:
        raise NotImplementedError("non_negative_parafac_hals needs at least two modes")
    n_modes = x.ndim
    if nn_modes == "all":
        nn_set = set(range(n_modes))
    elif nn_modes is None:
        nn_set = set()
    else:
        nn_set = set(int(m) for m in nn_modes)
    nn_mask = 0
    for m in nn_set:
        if 0 <= m < n_modes:
            nn_mask |= 1 << m
    weights, factors = initialize_cp(x, rank, init=init, svd=svd, non_negative=True,
                                     random_state=random_state,
                                     normalize_factors=normalize_factors)
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    if weights is None:
        weights = torch.ones(int(rank), dtype=x.dtype, device=x.device)
    weights = weights.to(x.dtype).contiguous().clone()
    if sparsity_coefficients is None or isinstance(sparsity_coefficients, float):
        sparsity_coefficients = [sparsity_coefficients] * n_modes
    sparsity_coefficients = list(sparsity_coefficients)
    fixed = [] if fixed_modes is None else list(fixed_modes)
    for m in fixed:
        sparsity_coefficients[m] = None
    for m in range(n_modes):
        if sparsity_coefficients[m] is not None:
            warnings.warn("Sparsity coefficient is ignored in unconstrained modes.")
    free = [m for m in range(n_modes) if m not in fixed]
    if not free or free[-1] != n_modes - 1:
        raise NotImplementedError("non_negative_parafac_hals with a fixed last mode is not "
                                  "supported by tensorly_gb300")
    lib = _lib.lib()
    shape = (ctypes.c_int64 * n_modes)(*x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_nn_mu_workspace_size(code, n_modes, shape, int(rank), int(n_iter_max),
                                                ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    fptrs = (ctypes.c_void_p * n_modes)(*[f.data_ptr() for f in factors])
    free_arr = (ctypes.c_int * len(free))(*free)
    sp = (ctypes.c_double * n_modes)(*[float("nan") if c is None else float(c)
                                       for c in sparsity_coefficients])
    errs = (ctypes.c_double * max(1, int(n_iter_max)))()
    n_err = ctypes.c_int(0)
    _lib.check(lib.tlgb_cp_nn_hals(code, x.data_ptr(), n_modes, shape, fptrs, weights.data_ptr(),
                                   int(rank), free_arr, len(free), nn_mask,
                                   1 if normalize_factors else 0, int(n_iter_max),
                                   float(tol) if tol else 0.0,
                                   0 if cvg_criterion == "abs_rec_error" else 1, sp,
                                   1 if exact else 0, errs, ctypes.byref(n_err), ptr(ws),
                                   ws.numel(), stream_of(x)))
    cp = CPTensor((placement.back(weights), [placement.back(f) for f in factors]))
    if return_errors:
        return cp, [float(errs[i]) for i in range(n_err.value)]
    return cp


class CP_NN_HALS:
    """sklearn-style wrapper of ``non_negative_parafac_hals``
    (tensorly/decomposition/_nn_cp.py:517-656): every keyword is passed
    through; ``decomposition_`` and ``errors_`` hold the last fit."""

    def __init__(self, rank, n_iter_max=100, init="svd", svd="truncated_svd", tol=10e-8,
                 sparsity_coefficients=None, fixed_modes=None, nn_modes="all", exact=False,
                 verbose=False, normalize_factors=False, cvg_criterion="abs_rec_error",
                 random_state=None):
        self.rank = rank
        self.random_state = random_state
        self.n_iter_max = n_iter_max
        self.init = init
        self.svd = svd
        self.tol = tol
        self.sparsity_coefficients = sparsity_coefficients
        self.fixed_modes = fixed_modes
        self.nn_modes = nn_modes
        self.exact = exact
        self.verbose = verbose
        self.normalize_factors = normalize_factors
        self.cvg_criterion = cvg_criterion

    def fit_transform(self, tensor):
        cp, errors = non_negative_parafac_hals(
            tensor, rank=self.rank, n_iter_max=self.n_iter_max, init=self.init, svd=self.svd,
            tol=self.tol, random_state=self.random_state,
            sparsity_coefficients=self.sparsity_coefficients,
            fixed_modes=self.fixed_modes, nn_modes=self.nn_modes, exact=self.exact,
            verbose=self.verbose, normalize_factors=self.normalize_factors,
            cvg_criterion=self.cvg_criterion, return_errors=True)
        self.decomposition_ = cp
        self.errors_ = errors
        return self.decomposition_

    def fit(self, tensor):
        self.fit_transform(tensor)
        return self

    def __repr__(self):
        return f"Rank-{self.rank} Non-Negative CP decomposition."


class CP_NN:
    """sklearn-style wrapper of ``non_negative_parafac``
    (tensorly/decomposition/_nn_cp.py:382-514): every keyword is passed
    through; ``decomposition_`` and ``errors_`` hold the last fit."""

    def __init__(self, rank, n_iter_max=100, init="svd", svd="truncated_svd", tol=10e-7,
                 random_state=None, verbose=0, normalize_factors=False, mask=None,
                 cvg_criterion="abs_rec_error", fixed_modes=None):
        self.rank = rank
        self.n_iter_max = n_iter_max
        self.init = init
        self.svd = svd
        self.tol = tol
        self.random_state = random_state
        self.verbose = verbose
        self.normalize_factors = normalize_factors
        self.mask = mask
        self.cvg_criterion = cvg_criterion
        self.fixed_modes = fixed_modes

    def fit_transform(self, tensor):
        cp, errors = non_negative_parafac(
            tensor, rank=self.rank, n_iter_max=self.n_iter_max, init=self.init, svd=self.svd,
            tol=self.tol, random_state=self.random_state, verbose=self.verbose,
            normalize_factors=self.normalize_factors, mask=self.mask,
            cvg_criterion=self.cvg_criterion, fixed_modes=self.fixed_modes, return_errors=True)
        self.decomposition_ = cp
        self.errors_ = errors
        return self.decomposition_

    def fit(self, tensor):
        self.fit_transform(tensor)
        return self

    def __repr__(self):
        return f"Rank-{self.rank} Non-Negative CP decomposition."


def sample_khatri_rao(matrices, n_samples, skip_matrix=None, indices_list=None,
                      return_sampled_rows=False, random_state=None):
    """Rows of the Khatri-Rao product at random positions
    (tensorly/decomposition/_cp.py:546-630), same signature and returns.

    The row indices are drawn on the host with NumPy's RandomState exactly as
    the reference draws them (one ``randint`` per matrix, in order); the
    product of the sampled rows is formed by ``tlgb_sample_khatri_rao``."""
    if skip_matrix is not None:
        matrices = [matrices[i] for i in range(len(matrices)) if i != skip_matrix]
    if indices_list is None:
        if random_state is None or not isinstance(random_state, np.random.RandomState):
            rng = check_random_state(random_state)
            warnings.warn(
                "You are creating a new random number generator at each call.\n"
                "If you are calling sample_khatri_rao inside a loop this will be slow:"
                " best to create a rng outside and pass it as argument (random_state=rng).")
        else:
            rng = random_state
        indices_list = [rng.randint(0, m.shape[0], size=n_samples, dtype=int) for m in matrices]
    mats = [to_device(m)[0].contiguous() for m in matrices]
    pl = to_device(matrices[0])[1]
    m0 = mats[0]
    rank = int(m0.shape[1])
    sizes = [int(m.shape[0]) for m in mats]
    idx = np.stack([np.asarray(i, dtype=np.int64).reshape(-1) for i in indices_list])
    if idx.shape[1] != n_samples:
        raise ValueError(f"{idx.shape[1]} indices for {n_samples} samples")
    for size, i in zip(sizes, idx):
        if i.size and (i.min() < 0 or i.max() >= size):
            raise IndexError("sample_khatri_rao: index out of range")
    out = torch.empty((n_samples, rank), dtype=m0.dtype, device=m0.device)
    d_idx = torch.from_numpy(np.ascontiguousarray(idx)).to(m0.device)
    _lib.check(_lib.lib().tlgb_sample_khatri_rao(
        dtype_code(m0), len(mats), _lib.ptr_array([m.data_ptr() for m in mats]),
        (ctypes.c_int64 * len(sizes))(*sizes), rank, int(n_samples), d_idx.data_ptr(),
        out.data_ptr(), stream_of(m0)))
    sampled_kr = pl.back(out)
    if return_sampled_rows:
        indices_kr = np.zeros((n_samples), dtype=int)
        for size, indices in zip(sizes, indices_list):
            indices_kr = indices_kr * size + indices
        return sampled_kr, indices_list, indices_kr
    return sampled_kr, indices_list


def _norm_on_device(x):
    """||X||_F by the residual kernel against a zero rank-1 model."""
    zeros = [torch.zeros((s, 1), dtype=x.dtype, device=x.device) for s in x.shape]
    return _residual_norm(x, zeros)


def _residual_norm(x, factors, weights=None):
    lib = _lib.lib()
    shape = (ctypes.c_int64 * x.ndim)(*x.shape)
    rank = int(factors[0].shape[1])
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_to_tensor_workspace_size(dtype_code(x), x.ndim, shape, rank,
                                                    ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    out = torch.empty(1, dtype=torch.float64, device=x.device)
    _lib.check(lib.tlgb_cp_residual_norm(dtype_code(x), x.data_ptr(), x.ndim, shape, rank,
                                         _lib.ptr_array([f.data_ptr() for f in factors]),
                                         ptr(weights), out.data_ptr(), ptr(ws), ws.numel(),
                                         stream_of(x)))
    return float(out.item())


def randomised_parafac(tensor, rank, n_samples, n_iter_max=100, init="random",
                       svd="truncated_svd", tol=10e-9, max_stagnation=20, return_errors=False,
                       random_state=None, verbose=0, callback=None):
    """Randomised CP-ALS (tensorly/decomposition/_cp.py:633-762), same
    signature, stop rules and returns.

    Per iteration the host draws every mode's sample indices with NumPy's
    RandomState in the reference's order; ``tlgb_cp_randomised_launch``
    then enqueues the mode updates (sampled Khatri-Rao rows, sampled
    unfolding, the normal equations of the sampled least-squares problem)
    and the reconstruction error ||X - [[A]]|| without forming the full
    tensor.  While the GPU runs them, the next iteration's indices are drawn
    from a copy of the generator; ``tlgb_cp_randomised_finish`` returns the
    error, and the copy's state becomes the generator's only if the loop
    goes on, so the draws are the reference's whatever iteration stops."""
    x, placement = to_device(tensor)
    code = dtype_code(x)
    x = x.contiguous()
    rank = validate_cp_rank(tuple(x.shape), rank=rank)
    rng = check_random_state(random_state)
    _, factors = initialize_cp(x, rank, init=init, svd=svd, random_state=random_state)
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    n_dims = x.ndim
    norm_tensor = _norm_on_device(x)
    weights = torch.ones(rank, dtype=x.dtype, device=x.device)

    def cp_now():
        return CPTensor((placement.back(weights), [placement.back(f) for f in factors]))

    rec_errors = []
    min_error = 0
    stagnation = 0
    if callback is not None:
        callback(cp_now())
    lib = _lib.lib()
    shape = (ctypes.c_int64 * n_dims)(*x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_randomised_workspace_size(code, n_dims, shape, rank, int(n_samples),
                                                     ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    fptrs = (ctypes.c_void_p * n_dims)(*[f.data_ptr() for f in factors])
    rec = ctypes.c_double(0.0)

    def draw(gen):
        idx = np.empty((n_dims, n_dims - 1, n_samples), dtype=np.int64)
        for mode in range(n_dims):
            others = [k for k in range(n_dims) if k != mode]
            for q, k in enumerate(others):          # sample_khatri_rao(..., random_state=rng)
                idx[mode, q] = gen.randint(0, x.shape[k], size=n_samples, dtype=int)
        return idx

    def fork(gen):
        twin = np.random.RandomState()
        twin.set_state(gen.get_state())
        return twin

    idx_host = torch.empty((n_dims, n_dims - 1, n_samples), dtype=torch.int64).pin_memory()
    d_idx = torch.empty(idx_host.shape, dtype=torch.int64, device=x.device)
    ahead, ahead_idx = None, None
    for iteration in range(n_iter_max):
        if ahead is not None:                        # the loop goes on: keep the early draws
            rng.set_state(ahead.get_state())
            idx = ahead_idx
        else:
            idx = draw(rng)
        idx_host.copy_(torch.from_numpy(idx))
        d_idx.copy_(idx_host, non_blocking=True)
        _lib.check(lib.tlgb_cp_randomised_launch(code, x.data_ptr(), n_dims, shape, rank, fptrs,
                                                 int(n_samples), d_idx.data_ptr(), ptr(ws),
                                                 ws.numel(), stream_of(x)))
        ahead = fork(rng) if iteration + 1 < n_iter_max else None
        ahead_idx = draw(ahead) if ahead is not None else None
        _lib.check(lib.tlgb_cp_randomised_finish(code, n_dims, shape, rank, int(n_samples),
                                                 ptr(ws), ws.numel(), ctypes.byref(rec),
                                                 stream_of(x)))
        rec_error = rec.value / norm_tensor
        if callback is not None:
            if callback(cp_now(), rec_error) is True:
                if verbose:
                    print("Received True from callback function. Exiting.")
                break
        if max_stagnation or tol:                    # _cp.py:731-755
            if not min_error or rec_error < min_error:
                min_error = rec_error
                stagnation = -1
            stagnation += 1
            rec_errors.append(rec_error)
            if iteration > 1:
                if verbose:
                    print(f"reconstruction error={rec_errors[-1]}, "
                          f"variation={rec_errors[-2] - rec_errors[-1]}.")
                if (tol and abs(rec_errors[-2] - rec_errors[-1]) < tol) or \
                        (stagnation and (stagnation > max_stagnation)):
                    if verbose:
                        print(f"converged in {iteration} iterations.")
                    break
    if return_errors:
        return cp_now(), rec_errors
    return cp_now()


class RandomizedCP:
    """sklearn-style wrapper of ``randomised_parafac``
    (tensorly/decomposition/_cp.py:919-1004); ``decomposition_`` and
    ``errors_`` hold the last fit."""

    def __init__(self, rank, n_samples, n_iter_max=100, init="random", svd="truncated_svd",
                 tol=10e-9, max_stagnation=20, return_errors=False, random_state=None,
                 verbose=0, callback=None):
        self.rank = rank
        self.n_samples = n_samples
        self.n_iter_max = n_iter_max
        self.init = init
        self.svd = svd
        self.tol = tol
        self.max_stagnation = max_stagnation
        self.return_errors = return_errors
        self.random_state = random_state
        self.verbose = verbose
        self.callback = callback

    def fit_transform(self, tensor):
        self.decomposition_, self.errors_ = randomised_parafac(
            tensor, rank=self.rank, n_samples=self.n_samples, n_iter_max=self.n_iter_max,
            init=self.init, svd=self.svd, tol=self.tol, return_errors=True,
            max_stagnation=self.max_stagnation, random_state=self.random_state,
            verbose=self.verbose, callback=self.callback)
        return self.decomposition_

    def fit(self, tensor):
        self.fit_transform(tensor)
        return self

    def __repr__(self):
        return f"Rank-{self.rank} Randomized CP decomposition."


_CONSTRAINT_NAMES = ("non_negative", "l1_reg", "l2_reg", "l2_square_reg", "unimodality",
                     "normalize", "simplex", "normalized_sparsity", "soft_sparsity",
                     "smoothness", "monotonicity", "hard_sparsity")
# library kinds of the proximal operators (TLGB_CONS_*): whole-matrix 1-5,
# column-wise and rank-based 6-12
_CONSTRAINT_KIND = {None: 0, "non_negative": 1, "l1_reg": 2, "l2_reg": 3, "l2_square_reg": 4,
                    "normalize": 5, "unimodality": 6, "simplex": 7, "normalized_sparsity": 8,
                    "soft_sparsity": 9, "smoothness": 10, "monotonicity": 11,
                    "hard_sparsity": 12}
_PARAMETRIC = ("l1_reg", "l2_reg", "l2_square_reg", "simplex", "normalized_sparsity",
               "soft_sparsity", "smoothness", "hard_sparsity")


def validate_constraints(non_negative=None, l1_reg=None, l2_reg=None, l2_square_reg=None,
                         unimodality=None, normalize=None, simplex=None, normalized_sparsity=None,
                         soft_sparsity=None, smoothness=None, monotonicity=None,
                         hard_sparsity=None, n_const=1, order=0):
    """(constraint, parameter) of mode ``order`` (tensorly/tenalg/proximal.py:4-145):
    a scalar applies to every mode; a list gives every mode the constraint with
    its own entry; a dict constrains the listed modes; a mode constrained twice
    raises ValueError."""
    values = [non_negative, l1_reg, l2_reg, l2_square_reg, unimodality, normalize, simplex,
              normalized_sparsity, soft_sparsity, smoothness, monotonicity, hard_sparsity]
    constraints = [None] * n_const
    parameters = [None] * n_const
    seen = set()
    twice = "You selected two constraints for the same mode. Consider to check your input"
    for v in values:
        if not v:
            continue
        if isinstance(v, dict):
            for mode in v:
                if mode in seen:
                    raise ValueError(twice)
                seen.add(mode)
        elif isinstance(v, list):
            for mode in range(len(v)):
                if v[mode]:
                    if mode in seen:
                        raise ValueError(twice)
                    seen.add(mode)
        else:
            if len(seen) > 0:
                raise ValueError(twice)
            seen.update(range(n_const))
    for v, name in zip(values, _CONSTRAINT_NAMES):
        if not v:
            continue
        if isinstance(v, dict):
            for mode in v:
                constraints[mode] = name
                parameters[mode] = v[mode]
        else:
            for i in range(n_const):
                constraints[i] = name
                parameters[i] = v[i] if isinstance(v, list) else v
    return constraints[order], parameters[order]


def _constraint_kind(constraint, parameter):
    if constraint not in _CONSTRAINT_KIND:
        raise RuntimeError("Invalid constraint name")        # tensorly/tenalg/proximal.py:267
    if constraint in _PARAMETRIC and parameter is None:
        raise TypeError(f"{constraint} needs a numeric parameter for every constrained mode")
    return _CONSTRAINT_KIND[constraint], float(parameter) if constraint in _PARAMETRIC else 0.0


def proximal_operator(tensor, n_const=1, order=0, **constraints):
    """The proximal operator of mode ``order``'s constraint
    (tensorly/tenalg/proximal.py:148-267) by ``tlgb_proximal_matrix``: the
    whole-matrix operators entry by entry, the column-wise ones (unimodality,
    simplex, soft_sparsity, smoothness, monotonicity) per column of a matrix
    (a vector is one column), the rank-based ones (hard_sparsity,
    normalized_sparsity) over all entries."""
    x, pl = to_device(tensor)
    if n_const is None:
        return pl.back(x)
    constraint, parameter = validate_constraints(n_const=n_const, order=order, **constraints)
    if constraint is None:
        return pl.back(x)
    kind, param = _constraint_kind(constraint, parameter)
    x = x.contiguous()
    if constraint in ("unimodality", "monotonicity") and x.ndim > 2:
        raise ValueError(f"{constraint.capitalize()} prox doesn't support an input which has "
                         "more than 2 dimensions.")
    rows = int(x.shape[0]) if x.ndim >= 1 else 1
    cols = x.numel() // max(rows, 1) if x.ndim >= 2 else 1
    if constraint in ("hard_sparsity", "normalized_sparsity") or kind <= 5:
        rows, cols = x.numel(), 1                     # the entries in any layout
    out = torch.empty_like(x)
    lib = _lib.lib()
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_proximal_matrix_workspace_size(dtype_code(x), rows, cols, kind,
                                                       ctypes.byref(nbytes)))
    ws = workspace(max(nbytes.value, 256), x.device)
    _lib.check(lib.tlgb_proximal_matrix(dtype_code(x), x.data_ptr(), rows, cols, kind, param,
                                        out.data_ptr(), ptr(ws), ws.numel(), stream_of(x)))
    return pl.back(out)


def initialize_constrained_parafac(tensor, rank, init="svd", svd="truncated_svd",
                                   random_state=None, **constraints):
    """tensorly/decomposition/_constrained_cp.py:22-163: the 'svd' start of
    ``initialize_cp``, or for 'random' factors drawn from NumPy's global
    generator as the reference's random_cp without a seed does; then every
    factor passes through its mode's proximal operator.  A CPTensor start is
    returned with its weights folded into the factors, without the operator."""
    x, pl = to_device(tensor)
    n_modes = x.ndim
    if init == "random":
        rns = check_random_state(None)
        factors = [torch.from_numpy(rns.random_sample((s, rank))).to(x.device, x.dtype)
                   for s in x.shape]
    elif init == "svd":
        _, factors = initialize_cp(x, rank, init="svd", svd=svd, random_state=random_state)
        factors = [f.to(x.dtype) for f in factors]
    elif isinstance(init, (tuple, list, CPTensor)):
        weights, factors = init
        factors = [to_device(f)[0].to(x.dtype) for f in factors]
        w = to_device(weights)[0] if weights is not None else None
        if w is not None and not bool((w == 1).all()):
            weights_avg = float(torch.prod(w.double()) ** (1.0 / w.shape[0]))
            factors = [_scale_all(f, weights_avg) for f in factors]
        return CPTensor((None, [pl.back(f) for f in factors]))
    else:
        raise ValueError(f'Initialization method "{init}" not recognized')
    factors = [to_device(proximal_operator(f, n_const=n_modes, order=i, **constraints))[0]
               for i, f in enumerate(factors)]
    return CPTensor((None, [pl.back(f) for f in factors]))


def constrained_parafac(tensor, rank, n_iter_max=100, n_iter_max_inner=10, init="svd",
                        svd="truncated_svd", tol_outer=1e-8, tol_inner=1e-6, random_state=None,
                        verbose=0, return_errors=False, cvg_criterion="abs_rec_error",
                        fixed_modes=None, non_negative=None, l1_reg=None, l2_reg=None,
                        l2_square_reg=None, unimodality=None, normalize=None, simplex=None,
                        normalized_sparsity=None, soft_sparsity=None, smoothness=None,
                        monotonicity=None, hard_sparsity=None):
    """Constrained CP by AO-ADMM (tensorly/decomposition/_constrained_cp.py:166-435),
    same signature and returns.

    The outer and inner (ADMM) loops run in ``tlgb_cp_constrained``: per free
    mode the factorisation of (Hadamard of Grams) + rho I, the MTTKRP, and
    ADMM iterations (solve, proximal operator, dual update, stop test) with no
    host round trip; one synchronisation per outer iteration for the error
    and the stop tests.  Every proximal operator of the reference is
    supported: entry-wise (non_negative, l1_reg, l2_reg, l2_square_reg,
    normalize), per column (unimodality, simplex, soft_sparsity, smoothness,
    monotonicity) and rank-based (hard_sparsity, normalized_sparsity)."""
    cons = dict(non_negative=non_negative, l1_reg=l1_reg, l2_reg=l2_reg,
                l2_square_reg=l2_square_reg, unimodality=unimodality, normalize=normalize,
                simplex=simplex, normalized_sparsity=normalized_sparsity,
                soft_sparsity=soft_sparsity, smoothness=smoothness, monotonicity=monotonicity,
                hard_sparsity=hard_sparsity)
    x, placement = to_device(tensor)
    code = dtype_code(x)
    x = x.contiguous()
    n_modes = x.ndim
    if n_modes < 2:
        raise NotImplementedError("constrained_parafac needs at least two modes")
    rank = validate_cp_rank(tuple(x.shape), rank=rank)
    kinds, params = [], []
    for mode in range(n_modes):
        k, p = _constraint_kind(*validate_constraints(n_const=n_modes, order=mode, **cons))
        kinds.append(k)
        params.append(p)
    if cvg_criterion not in ("abs_rec_error", "rec_error") and tol_outer and n_iter_max > 1:
        raise TypeError("Unknown convergence criterion")
    _, factors = initialize_constrained_parafac(x, rank, init=init, svd=svd,
                                                random_state=random_state, **cons)
    factors = [to_device(f)[0].to(x.dtype).contiguous().clone() for f in factors]
    fixed = [] if fixed_modes is None else list(fixed_modes)
    if n_modes - 1 in fixed:
        warnings.warn("You asked for fixing the last mode, which is not supported.\n "
                      "The last mode will not be fixed. Consider using tl.moveaxis()")
        fixed.remove(n_modes - 1)
    free = [m for m in range(n_modes) if m not in fixed]
    lib = _lib.lib()
    shape = (ctypes.c_int64 * n_modes)(*x.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_cp_constrained_workspace_size(code, n_modes, shape, rank,
                                                      ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, x.device)
    fptrs = (ctypes.c_void_p * n_modes)(*[f.data_ptr() for f in factors])
    errs = (ctypes.c_double * max(1, int(n_iter_max)))()
    n_err = ctypes.c_int(0)
    _lib.check(lib.tlgb_cp_constrained(
        code, x.data_ptr(), n_modes, shape, fptrs, rank, (ctypes.c_int * len(free))(*free),
        len(free), (ctypes.c_int * n_modes)(*kinds), (ctypes.c_double * n_modes)(*params),
        int(n_iter_max), int(n_iter_max_inner), float(tol_outer or 0.0), float(tol_inner),
        0 if cvg_criterion == "abs_rec_error" else 1, errs, ctypes.byref(n_err), ptr(ws),
        ws.numel(), stream_of(x)))
    weights = torch.ones(rank, dtype=x.dtype, device=x.device)
    cp = CPTensor((placement.back(weights), [placement.back(f) for f in factors]))
    if return_errors:
        return cp, [float(errs[i]) for i in range(n_err.value)]
    return cp


class ConstrainedCP(DecompositionMixin):
    """sklearn-style wrapper of ``constrained_parafac``
    (tensorly/decomposition/_constrained_cp.py:426-612)."""

    def __init__(self, rank, n_iter_max=100, n_iter_max_inner=10, init="svd",
                 svd="truncated_svd", tol_outer=1e-8, tol_inner=1e-6, random_state=None,
                 verbose=0, return_errors=False, cvg_criterion="abs_rec_error", fixed_modes=None,
                 non_negative=None, l1_reg=None, l2_reg=None, l2_square_reg=None,
                 unimodality=None, normalize=None, simplex=None, normalized_sparsity=None,
                 soft_sparsity=None, smoothness=None, monotonicity=None, hard_sparsity=None):
        self.rank = rank
        self.n_iter_max = n_iter_max
        self.n_iter_max_inner = n_iter_max_inner
        self.init = init
        self.svd = svd
        self.tol_outer = tol_outer
        self.tol_inner = tol_inner
        self.random_state = random_state
        self.verbose = verbose
        self.return_errors = return_errors
        self.cvg_criterion = cvg_criterion
        self.fixed_modes = fixed_modes
        self.non_negative = non_negative
        self.l1_reg = l1_reg
        self.l2_reg = l2_reg
        self.l2_square_reg = l2_square_reg
        self.unimodality = unimodality
        self.normalize = normalize
        self.simplex = simplex
        self.normalized_sparsity = normalized_sparsity
        self.soft_sparsity = soft_sparsity
        self.smoothness = smoothness
        self.monotonicity = monotonicity
        self.hard_sparsity = hard_sparsity

    def fit_transform(self, tensor):
        cp, errors = constrained_parafac(
            tensor, rank=self.rank, n_iter_max=self.n_iter_max,
            n_iter_max_inner=self.n_iter_max_inner, init=self.init, svd=self.svd,
            tol_outer=self.tol_outer, tol_inner=self.tol_inner, random_state=self.random_state,
            verbose=self.verbose, cvg_criterion=self.cvg_criterion,
            fixed_modes=self.fixed_modes, non_negative=self.non_negative, l1_reg=self.l1_reg,
            l2_reg=self.l2_reg, l2_square_reg=self.l2_square_reg, unimodality=self.unimodality,
            normalize=self.normalize, simplex=self.simplex,
            normalized_sparsity=self.normalized_sparsity, soft_sparsity=self.soft_sparsity,
            smoothness=self.smoothness, monotonicity=self.monotonicity,
            hard_sparsity=self.hard_sparsity, return_errors=True)
        self.decomposition_ = cp
        self.errors_ = errors
        return self.decomposition_


def _gemm(M, N, K, A, sam, sak, B, sbk, sbn):
    """C (M x N) = sum_k A[m*sam + k*sak] B[k*sbk + n*sbn] by ``tlgb_gemm``."""
    C = torch.empty((M, N), dtype=A.dtype, device=A.device)
    _lib.check(_lib.lib().tlgb_gemm(dtype_code(A), M, N, K, A.data_ptr(), sam, sak, B.data_ptr(),
                                    sbk, sbn, C.data_ptr(), stream_of(A)))
    return C


def _mat_nt(A, B):      # A B^T, A: M x K, B: N x K (row-major)
    A, B = A.contiguous(), B.contiguous()
    return _gemm(A.shape[0], B.shape[0], A.shape[1], A, A.shape[1], 1, B, 1, B.shape[1])


def _mat_tn(A, B):      # A^T B, A: K x M, B: K x N
    A, B = A.contiguous(), B.contiguous()
    return _gemm(A.shape[1], B.shape[1], A.shape[0], A, 1, A.shape[1], B, B.shape[1], 1)


def _mat_nn(A, B):      # A B, A: M x K, B: K x N
    A, B = A.contiguous(), B.contiguous()
    return _gemm(A.shape[0], B.shape[1], A.shape[1], A, A.shape[1], 1, B, B.shape[1], 1)


def _mu_update(A, num, den, eps):
    _lib.check(_lib.lib().tlgb_mu_update(dtype_code(A), A.data_ptr(), num.contiguous().data_ptr(),
                                         den.contiguous().data_ptr(), A.numel(), float(eps),
                                         stream_of(A)))


def _dot(a, b):
    lib = _lib.lib()
    ws = workspace(lib.tlgb_dot_workspace_bytes(), a.device)
    out = torch.empty(1, dtype=torch.float64, device=a.device)
    a, b = a.contiguous(), b.contiguous()
    _lib.check(lib.tlgb_dot(dtype_code(a), a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(),
                            ptr(ws), ws.numel(), stream_of(a)))
    return out


def non_negative_tucker(tensor, rank, n_iter_max=10, init="svd", tol=10e-5, random_state=None,
                        verbose=False, return_errors=False, normalize_factors=False):
    """Non-negative Tucker by multiplicative updates
    (tensorly/decomposition/_tucker.py:348-454), same signature and returns.

    The reference forms B = unfold(tucker_to_tensor(core, factors, skip=mode))^T
    (prod(I_k) x R_mode); here the same products come from the TTM chain:
    X_(n) B = [X x_{k!=n} U_k^T]_(n) G_(n)^T and B^T B = [G x_{k!=n} U_k^T U_k]_(n)
    G_(n)^T, so nothing of the size of the tensor is formed besides the chain.
    The error ||X - [[G; U]]|| comes from ||X||^2 - 2 <X x_k U_k^T, G> + <G,
    G x_k U_k^T U_k>.  normalize_factors applies ``tucker_normalize`` after
    every iteration that does not stop, as the reference does."""
    from .base import unfold
    from .cp_tensor import tucker_normalize, validate_tucker_rank
    from .tenalg import multi_mode_dot
    x, placement = to_device(tensor)
    x = x.contiguous()
    n_modes = x.ndim
    rank = validate_tucker_rank(tuple(x.shape), rank=rank)
    epsilon = 10e-12
    core, factors = initialize_tucker(x, rank, range(n_modes), init=init,
                                      random_state=random_state, non_negative=True)
    core = core.to(x.dtype).contiguous().clone()
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    norm_x2 = float(_dot(x, x).item())
    rec_errors = []
    for iteration in range(n_iter_max):
        for mode in range(n_modes):
            grams = [_mat_tn(f, f) for f in factors]
            y = multi_mode_dot(x, factors, skip=mode, transpose=True)
            num = _mat_nt(unfold(y, mode), unfold(core, mode))
            w = multi_mode_dot(core, grams, skip=mode)
            btb = _mat_nt(unfold(w, mode), unfold(core, mode))
            den = _mat_nn(factors[mode], btb)
            _mu_update(factors[mode], num, den, epsilon)
        grams = [_mat_tn(f, f) for f in factors]
        num_c = multi_mode_dot(x, factors, transpose=True).contiguous()
        den_c = multi_mode_dot(core, grams).contiguous()
        _mu_update(core, num_c, den_c, epsilon)
        t2 = float(_dot(core, multi_mode_dot(core, grams)).item())
        xt = float(_dot(num_c, core).item())
        rec_error = math.sqrt(max(norm_x2 - 2.0 * xt + t2, 0.0) / norm_x2)
        rec_errors.append(rec_error)
        if iteration > 1 and verbose:
            print(f"reconstruction error={rec_errors[-1]}, "
                  f"variation={rec_errors[-2] - rec_errors[-1]}.")
        if iteration > 1 and abs(rec_errors[-2] - rec_errors[-1]) < tol:
            if verbose:
                print(f"converged in {iteration} iterations.")
            break
        if normalize_factors:
            core, factors = tucker_normalize((core, factors))
    out = TuckerTensor((placement.back(core), [placement.back(f) for f in factors]))
    if return_errors:
        return out, rec_errors
    return out


def hals_nnls(UtM, UtU, V=None, n_iter_max=500, tol=1e-8, sparsity_coefficient=None,
              ridge_coefficient=None, nonzero_rows=False, exact=False, epsilon=0.0,
              callback=None):
    """HALS non-negative least squares (tensorly/solvers/nnls.py:5-175), same
    signature and return (V, R x n), by ``tlgb_hals_nnls``: one warp per
    column of V, the reference's stop test applied after each chunk of
    iterations.  A starting V is required; ridge, nonzero_rows, epsilon and
    callback are not supported."""
    from .base import unfold
    if V is None:
        raise NotImplementedError("hals_nnls without a starting V is not supported by "
                                  "tensorly_gb300")
    if ridge_coefficient is not None or nonzero_rows or epsilon != 0.0 or callback is not None:
        raise NotImplementedError("hals_nnls with ridge_coefficient, nonzero_rows, epsilon or "
                                  "callback is not supported by tensorly_gb300")
    utm, pl = to_device(UtM)
    utu = to_device(UtU)[0].to(utm.dtype).contiguous()
    v = to_device(V)[0].to(utm.dtype)
    if exact:
        n_iter_max, tol = 50000, 1e-16
    rank, n = int(utm.shape[0]), int(utm.shape[1])
    mtu = unfold(utm, 1)                      # n x rank: the transposed layout
    vt = unfold(v, 1).contiguous()
    _hals_nnls_t(mtu, utu, vt, int(n_iter_max), float(tol), sparsity_coefficient)
    return pl.back(unfold(vt, 1))


def _hals_nnls_t(mtu, utu, vt, n_iter_max, tol, sparsity):
    lib = _lib.lib()
    n, rank = int(vt.shape[0]), int(vt.shape[1])
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_hals_nnls_workspace_size(dtype_code(vt), n, rank, ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, vt.device)
    sp = float("nan") if sparsity is None else float(sparsity)
    _lib.check(lib.tlgb_hals_nnls(dtype_code(vt), mtu.contiguous().data_ptr(),
                                  utu.contiguous().data_ptr(), vt.data_ptr(), n, rank,
                                  int(n_iter_max), float(tol), sp, ptr(ws), ws.numel(),
                                  stream_of(vt)))


def active_set_nnls(Utm, UtU, x=None, n_iter_max=100, tol=10e-8):
    """Active-set non-negative least squares (tensorly/solvers/nnls.py:279-426,
    Bro and De Jong), same signature and return (the solution vector), by
    ``tlgb_active_set_nnls`` (one CTA, up to 128 unknowns).  Where the
    reference's np.linalg.solve would raise on an exactly singular passive
    system, SingularMatrixError is raised."""
    utu, pl = to_device(UtU)
    utu = utu.contiguous()
    n = int(utu.shape[1])
    utm = like(Utm, utu).reshape(-1).contiguous()
    xv = (torch.zeros(n, dtype=utu.dtype, device=utu.device) if x is None
          else like(x, utu).reshape(-1).clone())
    _active_set_t(utm, utu, xv, int(n_iter_max), float(tol))
    return pl.back(xv)


def _active_set_t(utm, utu, xv, n_iter_max, tol):
    n = int(xv.numel())
    status = torch.zeros(1, dtype=torch.int32, device=xv.device)
    _lib.check(_lib.lib().tlgb_active_set_nnls(dtype_code(xv), ptr(utu), ptr(utm), ptr(xv), n,
                                               n_iter_max, tol, ptr(status), stream_of(xv)))
    rc = int(status.item())
    if rc != _lib.TLGB_OK:
        raise _lib.SingularMatrixError(rc, "active_set_nnls: singular passive-set system")


def _tucker_fixed_modes_error(shape, rank, fixed, init="svd"):
    """The ValueError the reference's non_negative_tucker_hals raises with
    fixed modes, or None where this walk does not find it.  Its
    initialize_tucker then gives the j-th free mode the rank rank[j] and keeps
    only the free modes' factors, while the first mode loop indexes that list
    by mode number; the first misaligned mode_dot of that loop raises
    (tensorly/decomposition/_tucker.py:591-630, _tucker.py:22-110).  Only the
    shapes are walked, nothing is computed."""
    n = len(shape)
    modes = [m for m in range(n) if m not in fixed]
    if init == "svd":
        core = list(shape)
        for j, m in enumerate(modes):
            core[m] = rank[j]
    elif init == "random":
        core = [rank[j] for j in range(len(modes))]
    else:
        return None
    mode = modes[0]

    def misaligned(dims, mat, i):
        return ValueError(f"shapes {tuple(dims)} and {mat} not aligned in mode-{i} "
                          f"multiplication: {dims[i]} (mode {i}) != {mat[1]} (dim 1 of matrix)")

    # multi_mode_dot(core, grams, skip=mode): list entry i, the Gram of the
    # factor of free mode modes[i] (rank[i] x rank[i]), acts on core mode i
    for i in range(len(modes)):
        if i == mode:
            continue
        if i >= len(core):
            return None
        if core[i] != rank[i]:
            return misaligned(core, (rank[i], rank[i]), i)
    if mode >= len(core):
        return None
    # multi_mode_dot(tensor, factors, skip=mode, transpose=True): entry i is
    # the transposed factor of free mode modes[i], rank[i] x shape[modes[i]]
    dims = list(shape)
    for i in range(len(modes)):
        if i == mode:
            continue
        if dims[i] != shape[modes[i]]:
            return misaligned(dims, (rank[i], shape[modes[i]]), i)
        dims[i] = rank[i]
    return None


def _largest_eig(a):
    """Largest eigenvalue of a symmetric matrix (the first singular value of a
    Gram, tl.truncated_svd(MtM)[1][0]) by the library's eigensolver."""
    lib = _lib.lib()
    n = int(a.shape[0])
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_sym_eig_workspace_size(dtype_code(a), n, 1, ctypes.byref(nbytes)))
    ws = workspace(nbytes.value, a.device)
    u = torch.empty((n, 1), dtype=a.dtype, device=a.device)
    ev = torch.empty(1, dtype=a.dtype, device=a.device)
    _lib.check(lib.tlgb_sym_eig(dtype_code(a), a.contiguous().data_ptr(), n, 1, u.data_ptr(),
                                ev.data_ptr(), 0, ptr(ws), ws.numel(), stream_of(a)))
    return float(ev.item())


def non_negative_tucker_hals(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                             tol=1e-8, sparsity_coefficients=None, core_sparsity_coefficient=None,
                             fixed_modes=None, random_state=None, verbose=False,
                             normalize_factors=False, return_errors=False, exact=False,
                             algorithm="fista"):
    """Non-negative Tucker by HALS (tensorly/decomposition/_tucker.py:457-691),
    same signature and returns, for algorithm='fista'.

    Per mode the factor update is the reference's hals_nnls call on
    UtU = [G x_{k!=n} U_k^T U_k]_(n) G_(n)^T and MtU = [X x_{k!=n} U_k^T]_(n) G_(n)^T
    (``tlgb_hals_nnls``); the core update is the reference's FISTA with the
    step prod_k 1 / lambda_max(U_k^T U_k) (``tlgb_fista_tucker_core``, the
    eigenvalues from the library's eigensolver).  With algorithm='active_set'
    the core is the reference's active_set_nnls on the Kronecker product of
    the factor Grams and vec(X x_k U_k^T) (``tlgb_kronecker``,
    ``tlgb_active_set_nnls``; up to 128 core entries).  normalize_factors
    applies ``tucker_normalize`` after every iteration that does not stop, as
    the reference does.  The error comes from the norm expansion.  With fixed
    modes the reference's own loop fails on its first mode_dot; the same
    ValueError is raised here before any work."""
    from collections.abc import Iterable
    from .base import unfold
    from .cp_tensor import tucker_normalize, validate_tucker_rank
    from .tenalg import kronecker, multi_mode_dot
    if algorithm not in ("fista", "active_set"):
        raise NotImplementedError("non_negative_tucker_hals supports algorithm='fista' or "
                                  "'active_set'")
    x, placement = to_device(tensor)
    x = x.contiguous()
    n_modes = x.ndim
    rank = validate_tucker_rank(tuple(x.shape), rank=rank)
    if sparsity_coefficients is None or not isinstance(sparsity_coefficients, Iterable):
        sparsity_coefficients = [sparsity_coefficients] * n_modes
    fixed = [] if fixed_modes is None else list(fixed_modes)
    if n_modes - 1 in fixed:
        warnings.warn("You asked for fixing the last mode, which is not supported. The last mode "
                      "will not be fixed. Consider using tl.moveaxis() to permute it to another "
                      "position and keep it fixed there.")
        fixed.remove(n_modes - 1)
    if fixed:
        err = (_tucker_fixed_modes_error(tuple(x.shape), rank, fixed, init)
               if n_iter_max > 0 and isinstance(init, str) else None)
        if err is not None:
            raise err
        raise NotImplementedError("non_negative_tucker_hals with these fixed modes is not "
                                  "supported by tensorly_gb300")
    n_inner, tol_inner = (50000, 1e-16) if exact else (100, 1e-8)
    core, factors = initialize_tucker(x, rank, range(n_modes), init=init, svd=svd,
                                      random_state=random_state, non_negative=True)
    core = core.to(x.dtype).contiguous().clone()
    factors = [f.to(x.dtype).contiguous().clone() for f in factors]
    norm_x2 = float(_dot(x, x).item())
    lib = _lib.lib()
    cshape = (ctypes.c_int64 * n_modes)(*core.shape)
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.tlgb_fista_tucker_core_workspace_size(dtype_code(x), n_modes, cshape,
                                                         ctypes.byref(nbytes)))
    fws = workspace(nbytes.value, x.device)
    csp = 0.0 if core_sparsity_coefficient is None else float(core_sparsity_coefficient)
    if algorithm == "active_set" and core.numel() > 128:
        raise NotImplementedError("non_negative_tucker_hals(algorithm='active_set') supports "
                                  "cores of up to 128 entries")
    rec_errors = []
    for iteration in range(n_iter_max):
        for mode in range(n_modes):
            grams = [_mat_tn(f, f) for f in factors]
            core_cross = multi_mode_dot(core, grams, skip=mode)
            utu = _mat_nt(unfold(core_cross, mode), unfold(core, mode))
            y = multi_mode_dot(x, factors, skip=mode, transpose=True)
            mtu = _mat_nt(unfold(y, mode), unfold(core, mode))
            _hals_nnls_t(mtu, utu, factors[mode], n_inner, tol_inner,
                         sparsity_coefficients[mode])
        grams = [_mat_tn(f, f).contiguous() for f in factors]
        core_est = multi_mode_dot(x, factors, transpose=True).contiguous()
        if algorithm == "fista":
            lr = 1.0
            for g in grams:
                lr *= 1.0 / _largest_eig(g)
            _lib.check(lib.tlgb_fista_tucker_core(
                dtype_code(x), core_est.data_ptr(), n_modes, cshape,
                _lib.ptr_array([g.data_ptr() for g in grams]), core.data_ptr(), int(n_iter_max),
                csp, lr, 1e-8, 1e-8, ptr(fws), fws.numel(), stream_of(x)))
        else:
            cvec = core.reshape(-1)
            _active_set_t(core_est.reshape(-1), kronecker(grams).contiguous(), cvec,
                          int(n_iter_max), 10e-8)
        t2 = float(_dot(core, multi_mode_dot(core, grams)).item())
        xt = float(_dot(core_est, core).item())
        rec_error = math.sqrt(max(norm_x2 - 2.0 * xt + t2, 0.0) / norm_x2)
        rec_errors.append(rec_error)
        if iteration > 1:
            if verbose:
                print(f"reconstruction error={rec_errors[-1]}, "
                      f"variation={rec_errors[-2] - rec_errors[-1]}.")
            if tol and abs(rec_errors[-2] - rec_errors[-1]) < tol:
                if verbose:
                    print(f"converged in {iteration} iterations.")
                break
        if normalize_factors:
            core, factors = tucker_normalize((core, factors))
    out = TuckerTensor((placement.back(core), [placement.back(f) for f in factors]))
    if return_errors:
        return out, rec_errors
    return out


class BatchedProblem:
    """Many small 3-way f32 tensors packed for ``tlgb_cp_als_batched``.

    The tensors go into one device buffer and the initial factors into
    another (``init='random'``: the reference's per-tensor draws,
    random/base.py:104, with ``random_state`` None, one int, or one seed per
    tensor; or a list of factor lists / CPTensors).  ``run`` restarts from
    the initial factors every time, so it can be timed repeatedly.
    """

    def __init__(self, tensors, ranks, init="random", random_state=None):
        stacked = isinstance(tensors, torch.Tensor) and tensors.ndim == 4
        if stacked:   # one tensor of shape (n, I0, I1, I2): used in place when on the GPU
            x4, x4_placement = to_device(tensors)
            tensors = list(x4)
        else:
            tensors = list(tensors)
        n = len(tensors)
        if isinstance(ranks, int):
            ranks = [ranks] * n
        self.ranks = [int(r) for r in ranks]
        if len(self.ranks) != n:
            raise ValueError("one rank per tensor is needed")
        if n == 0:
            raise ValueError("empty batch")
        if stacked:
            self.placement = x4_placement
            dev = x4.device
            self.shapes = [tuple(int(d) for d in x4.shape[1:])] * n
            self.xbuf = x4.to(torch.float32).contiguous().reshape(-1)
            xoff = np.arange(n + 1, dtype=np.int64) * int(np.prod(self.shapes[0]))
        else:
            placed = [to_device(t) for t in tensors]
            self.placement = placed[0][1]
            dev = placed[0][0].device
            xs = []
            for x, _ in placed:
                if x.ndim != 3:
                    raise NotImplementedError("parafac_batched takes 3-way tensors")
                xs.append(x.to(dev, torch.float32).contiguous().reshape(-1))
            self.shapes = [tuple(int(s) for s in x.shape) for x, _ in placed]
            xoff = np.cumsum([0] + [int(x.numel()) for x in xs])
            self.xbuf = torch.cat(xs) if n > 1 else xs[0].clone()
        self.device = dev
        foff = [0]
        for sh, r in zip(self.shapes, self.ranks):
            for d in sh:
                foff.append(foff[-1] + d * r)
        self.foff = foff
        self.finit = torch.empty(foff[-1], dtype=torch.float32, device=dev)
        if isinstance(init, str) and init == "random":
            if random_state is None or isinstance(random_state, (int, np.integer)):
                seeds = [random_state] * n
            else:
                seeds = list(random_state)
            host = np.empty(foff[-1], dtype=np.float32)
            q = 0
            for t, (sh, r) in enumerate(zip(self.shapes, self.ranks)):
                s = seeds[t]
                rng = check_random_state(int(s) if isinstance(s, np.integer) else s)
                for d in sh:
                    host[foff[q]:foff[q + 1]] = rng.random_sample((d, r)).astype(np.float32).ravel()
                    q += 1
            self.finit.copy_(torch.from_numpy(host))
        elif isinstance(init, torch.Tensor):   # packed: (n, ...) in the layout of self.finit
            f = like(init, self.xbuf).to(torch.float32).reshape(-1)
            if f.numel() != foff[-1]:
                raise ValueError("packed initial factors have the wrong size")
            self.finit.copy_(f)
        elif isinstance(init, (list, tuple)):
            q = 0
            for t, (sh, r) in enumerate(zip(self.shapes, self.ranks)):
                f_init = init[t].factors if isinstance(init[t], CPTensor) else init[t]
                for k, d in enumerate(sh):
                    f = like(f_init[k], self.xbuf).to(torch.float32).reshape(-1)
                    if f.numel() != d * r:
                        raise ValueError(f"initial factor {k} of tensor {t} has the wrong size")
                    self.finit[foff[q]:foff[q + 1]].copy_(f)
                    q += 1
        else:
            raise ValueError(f'Initialization method "{init}" not recognized')
        self.fbuf = torch.empty_like(self.finit)
        self.items = (_lib.BatchItem * n)()
        q = 0
        for t, (sh, r) in enumerate(zip(self.shapes, self.ranks)):
            self.items[t].X = self.xbuf.data_ptr() + 4 * int(xoff[t])
            for k in range(3):
                self.items[t].factors[k] = self.fbuf.data_ptr() + 4 * foff[q]
                self.items[t].dims[k] = sh[k]
                q += 1
            self.items[t].rank = r
        self.final = torch.empty(n, dtype=torch.float64, device=dev)
        self.n_sweeps = torch.zeros(n, dtype=torch.int32, device=dev)
        nbytes = ctypes.c_size_t(0)
        _lib.check(_lib.lib().tlgb_cp_als_batched_workspace_size(n, ctypes.byref(nbytes)))
        self.ws = workspace(nbytes.value, dev)
        self.sweeps = None

    def __len__(self):
        return len(self.ranks)

    def run(self, n_iter_max, sweeps_per_launch=0, sweep_errors=False, exact_sweep_errors=False,
            tol=0.0):
        """Restart from the initial factors and run ``n_iter_max`` sweeps, or
        with ``tol`` > 0 stop each tensor at the reference's 'abs_rec_error'
        test; ``exact_sweep_errors`` computes the per-sweep errors from the
        residual (always so with ``tol``).  ``n_sweeps`` holds the sweeps
        each tensor ran; per-sweep errors past a tensor's stop are NaN."""
        n = len(self)
        self.fbuf.copy_(self.finit)
        self.sweeps = (torch.full((n, max(1, int(n_iter_max))), float("nan"), dtype=torch.float64,
                                  device=self.device) if sweep_errors else None)
        _lib.check(_lib.lib().tlgb_cp_als_batched(
            n, self.items, int(n_iter_max), int(sweeps_per_launch),
            1 if exact_sweep_errors else 0, float(tol), ptr(self.final),
            ptr(self.sweeps) if self.sweeps is not None else None, ptr(self.n_sweeps),
            ptr(self.ws), self.ws.numel(), stream_of(self.xbuf)))
        return self

    def results(self):
        out = []
        q = 0
        for sh, r in zip(self.shapes, self.ranks):
            fs = []
            for k in range(3):
                fs.append(self.placement.back(self.fbuf[self.foff[q]:self.foff[q + 1]]
                                              .view(sh[k], r).clone()))
                q += 1
            w = self.placement.back(torch.ones(r, dtype=torch.float32, device=self.device))
            out.append(CPTensor((w, fs)))
        return out


def parafac_batched(tensors, ranks, n_iter_max=100, init="random", random_state=None,
                    return_errors=False, sweep_errors=False, sweeps_per_launch=0, tol=0.0):
    """CP-ALS of many small 3-way f32 tensors at once (one persistent kernel
    per size class of tensors).

    Per tensor this is ``parafac(tensor, rank, n_iter_max=n_iter_max, tol=tol,
    init=..., normalize_factors=False)`` (tensorly/decomposition/_cp.py:230-543),
    weights all one: exactly ``n_iter_max`` sweeps with ``tol=0``, else each
    tensor stops at the reference's 'abs_rec_error' test on its relative
    error (computed from the residual).  ``init``: ``'random'``
    (``random_state``: None, an int applied to every tensor, or one seed per
    tensor; the reference's draws, random/base.py:104) or a list of factor
    lists, or one packed tensor of all initial factors (tensor-major, then
    mode, each ``I_k x rank`` row-major).  ``tensors`` may be a list or one
    ``(n, I0, I1, I2)`` tensor.  Mode sizes 1..64, ranks 1..16.

    Returns the list of ``CPTensor``; with ``return_errors`` also the final
    relative errors (from the residual, as a NumPy array), and with
    ``sweep_errors`` the per-sweep errors (n_tensors x n_iter_max).
    """
    if not (isinstance(tensors, torch.Tensor) and tensors.ndim == 4):
        tensors = list(tensors)   # a (n, I0, I1, I2) tensor is packed as it is
    if len(tensors) == 0:
        return ([], np.zeros(0)) if return_errors else []
    prob = BatchedProblem(tensors, ranks, init=init, random_state=random_state)
    prob.run(n_iter_max, sweeps_per_launch=sweeps_per_launch, sweep_errors=sweep_errors, tol=tol)
    out = prob.results()
    res = [out]
    if return_errors:
        res.append(prob.final.cpu().numpy())
    if sweep_errors:
        res.append(prob.sweeps[:, : int(n_iter_max)].cpu().numpy())
    return out if len(res) == 1 else tuple(res)
