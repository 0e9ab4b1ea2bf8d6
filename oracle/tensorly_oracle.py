"""NumPy restatement of TensorLy 0.9.0's CP-ALS / Tucker-HOOI hot path.

TEST INFRASTRUCTURE: this module is the oracle the CUDA library is checked
against.  It is imported only by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py``; the shipped package never calls it.

Every function names the reference file:line whose behaviour it restates
(paths are relative to the TensorLy source tree, ``tensorly/...``).  The
arithmetic that TensorLy delegates to NumPy/LAPACK (``np.dot``,
``np.linalg.solve`` = LAPACK gesv, ``np.linalg.svd`` = LAPACK gesdd) is called
the same way here, so on identical inputs this module reproduces the
reference's NumPy backend to rounding (pinned by ``tests/golden``).

Only the dense, real, unmasked, non-sparse branches are restated: those are
the branches the GB300 library implements.  Other branches raise
``NotImplementedError``.
"""

import math
import warnings

import numpy as np

__all__ = [
    "check_random_state", "unfold", "fold", "khatri_rao",
    "unfolding_dot_khatri_rao", "mode_dot", "multi_mode_dot", "svd_flip",
    "truncated_svd", "svd_interface", "random_cp", "cp_to_tensor", "cp_norm",
    "cp_normalize", "validate_cp_rank", "initialize_cp", "error_calc",
    "parafac", "initialize_tucker", "partial_tucker", "tucker", "non_negative_parafac",
    "make_svd_non_negative", "hals_nnls", "non_negative_parafac_hals",
    "tucker_to_tensor", "validate_tucker_rank", "parafac_sweeps", "cp_to_unfolded",
    "cp_to_vec", "tucker_to_unfolded", "tucker_to_vec", "sample_khatri_rao",
    "randomised_parafac", "sparsify_tensor", "error_calc_ext", "validate_constraints", "proximal_operator", "admm",
    "initialize_constrained_parafac", "constrained_parafac", "non_negative_tucker", "fista",
    "non_negative_tucker_hals", "active_set_nnls", "kronecker", "tucker_normalize",
    "randomized_svd", "randomized_range_finder",
]


# --------------------------------------------------------------------------
# random state, norm, unfolding
# --------------------------------------------------------------------------
def norm(tensor, axis=None):
    """tensorly/backend/core.py:714-739 (order 2): sqrt(sum(|x|**2))."""
    return np.sqrt(np.sum(np.abs(tensor) ** 2, axis=axis))


def check_random_state(seed):
    """tensorly/backend/core.py:163-188: None -> global RandomState,
    int -> RandomState(seed), RandomState -> itself."""
    if seed is None:
        return np.random.mtrand._rand
    if isinstance(seed, (int, np.integer)):
        return np.random.RandomState(int(seed))
    if isinstance(seed, np.random.RandomState):
        return seed
    raise ValueError("Seed should be None, int or np.random.RandomState")


def unfold(tensor, mode):
    """tensorly/base.py:39-53: moveaxis(mode -> 0) then C-order reshape."""
    return np.reshape(np.moveaxis(tensor, mode, 0), (tensor.shape[mode], -1))


def fold(unfolded, mode, shape):
    """tensorly/base.py:56-79: inverse of :func:`unfold`."""
    full_shape = list(shape)
    mode_dim = full_shape.pop(mode)
    full_shape.insert(0, mode_dim)
    return np.moveaxis(np.reshape(unfolded, full_shape), 0, mode)


# --------------------------------------------------------------------------
# tenalg primitives
# --------------------------------------------------------------------------
def khatri_rao(matrices, weights=None, skip_matrix=None, mask=None):
    """tensorly/tenalg/core_tenalg/_khatri_rao.py:64-109.

    Column-wise Kronecker product; the first matrix varies slowest.  Weights
    multiply the first matrix (``:96-99``) before the pairwise products
    (``:101-105``); the optional mask multiplies the rows (``:107-109``).
    """
    if skip_matrix is not None:
        matrices = [matrices[i] for i in range(len(matrices)) if i != skip_matrix]
    if len(matrices) == 1:
        return matrices[0]
    if np.ndim(matrices[0]) == 2:
        n_columns = matrices[0].shape[1]
    else:
        n_columns = 1
        matrices = [np.reshape(m, (-1, 1)) for m in matrices]
    for i, matrix in enumerate(matrices):
        if np.ndim(matrix) != 2:
            raise ValueError(
                "All the matrices must have exactly 2 dimensions!"
                f"Matrix {i} has dimension {np.ndim(matrix)} != 2.")
        if matrix.shape[1] != n_columns:
            raise ValueError(
                "All matrices must have same number of columns!"
                f"Matrix {i} has {matrix.shape[1]} columns != {n_columns}.")
    res = None
    for i, e in enumerate(matrices[1:]):
        if not i:
            res = matrices[0] if weights is None else matrices[0] * np.reshape(weights, (1, -1))
        s1, s2 = res.shape
        s3, s4 = e.shape
        res = np.reshape(np.reshape(res, (s1, 1, s2)) * np.reshape(e, (1, s3, s4)),
                         (-1, n_columns))
    m = np.reshape(mask, (-1, 1)) if mask is not None else 1
    return res * m


def unfolding_dot_khatri_rao(tensor, cp_tensor, mode):
    """tensorly/tenalg/core_tenalg/mttkrp.py:9-50: explicit KR, then
    ``dot(unfold(tensor, mode), conj(KR))``."""
    weights, factors = cp_tensor
    kr = khatri_rao(factors, weights=weights, skip_matrix=mode)
    return np.dot(unfold(tensor, mode), np.conj(kr))


def mode_dot(tensor, matrix_or_vector, mode, transpose=False):
    """tensorly/tenalg/core_tenalg/n_mode_product.py:5-76."""
    fold_mode = mode
    new_shape = list(tensor.shape)
    if np.ndim(matrix_or_vector) == 2:
        dim = 0 if transpose else 1
        if matrix_or_vector.shape[dim] != tensor.shape[mode]:
            raise ValueError(
                f"shapes {tensor.shape} and {matrix_or_vector.shape} not aligned in "
                f"mode-{mode} multiplication: {tensor.shape[mode]} (mode {mode}) != "
                f"{matrix_or_vector.shape[dim]} (dim 1 of matrix)")
        if transpose:
            matrix_or_vector = np.conj(np.transpose(matrix_or_vector))
        new_shape[mode] = matrix_or_vector.shape[0]
        vec = False
    elif np.ndim(matrix_or_vector) == 1:
        if matrix_or_vector.shape[0] != tensor.shape[mode]:
            raise ValueError(
                f"shapes {tensor.shape} and {matrix_or_vector.shape} not aligned for "
                f"mode-{mode} multiplication: {tensor.shape[mode]} (mode {mode}) != "
                f"{matrix_or_vector.shape[0]} (vector size)")
        if len(new_shape) > 1:
            new_shape.pop(mode)
        else:
            new_shape = ()
        vec = True
    else:
        raise ValueError(
            "Can only take n_mode_product with a vector or a matrix."
            f"Provided array of dimension {np.ndim(matrix_or_vector)} not in [1, 2].")
    res = np.dot(matrix_or_vector, unfold(tensor, mode))
    if vec:
        return np.reshape(res, new_shape)
    return fold(res, fold_mode, new_shape)


def multi_mode_dot(tensor, matrix_or_vec_list, modes=None, skip=None, transpose=False):
    """tensorly/tenalg/core_tenalg/n_mode_product.py:79-135: modes applied in
    sorted order, ``skip`` indexes the sorted list, vectors drop a mode."""
    if modes is None:
        modes = range(len(matrix_or_vec_list))
    decrement = 0
    res = tensor
    factors_modes = sorted(zip(matrix_or_vec_list, modes), key=lambda x: x[1])
    for i, (m, mode) in enumerate(factors_modes):
        if skip is not None and i == skip:
            continue
        if transpose:
            res = mode_dot(res, np.conj(np.transpose(m)), mode - decrement)
        else:
            res = mode_dot(res, m, mode - decrement)
        if np.ndim(m) == 1:
            decrement += 1
    return res


# --------------------------------------------------------------------------
# SVD
# --------------------------------------------------------------------------
def svd_flip(U, V, u_based_decision=True):
    """tensorly/tenalg/svd.py:13-65: make the max-|.| entry of each U column
    positive (U-based rule) and flip the matching V rows."""
    if u_based_decision:
        max_abs_cols = np.argmax(np.abs(U), axis=0)
        signs = np.sign(U[max_abs_cols, np.arange(U.shape[1])])
        U = U * np.conj(signs)
        if V.shape[0] > U.shape[1]:
            signs = np.concatenate((signs, np.ones(V.shape[0] - U.shape[1])))
        V = V * signs[: V.shape[0]][:, None]
    else:
        max_abs_rows = np.argmax(np.abs(V), axis=1)
        signs = np.sign(V[np.arange(V.shape[0]), max_abs_rows])
        V = V * np.conj(signs[:, None])
        if U.shape[1] > V.shape[0]:
            signs = np.concatenate((signs, np.ones(U.shape[1] - V.shape[0])))
        U = U * signs[: U.shape[1]]
    return U, V


def _svd_checks(matrix, n_eigenvecs=None):
    """tensorly/tenalg/svd.py:172-208 (shape checks of the SVD helpers)."""
    if np.ndim(matrix) != 2:
        raise ValueError(f"matrix be a matrix. matrix.ndim is {np.ndim(matrix)} != 2")
    dim_1, dim_2 = matrix.shape
    min_dim, max_dim = (dim_1, dim_2) if dim_1 <= dim_2 else (dim_2, dim_1)
    if n_eigenvecs is None:
        n_eigenvecs = max_dim
    if n_eigenvecs > max_dim:
        warnings.warn(
            f"Trying to compute SVD with n_eigenvecs={n_eigenvecs}, which is larger "
            f"than max(matrix.shape)={max_dim}. Setting n_eigenvecs to {max_dim}.")
        n_eigenvecs = max_dim
    return n_eigenvecs, min_dim, max_dim


def truncated_svd(matrix, n_eigenvecs=None, **kwargs):
    """tensorly/tenalg/svd.py:211-235: full ``np.linalg.svd`` then truncate."""
    n_eigenvecs, min_dim, _ = _svd_checks(matrix, n_eigenvecs)
    full_matrices = n_eigenvecs > min_dim
    U, S, V = np.linalg.svd(matrix, full_matrices=full_matrices)
    return U[:, :n_eigenvecs], S[:n_eigenvecs], V[:n_eigenvecs, :]


def randomized_range_finder(A, n_dims, n_iter=2, random_state=None):
    """tensorly/tenalg/svd.py:138-170 (Halko et al. 2009, algorithm 4.4)."""
    rng = check_random_state(random_state)
    dim_1, dim_2 = A.shape
    Q = rng.normal(size=(dim_2, n_dims)).astype(A.dtype)
    Q, _ = np.linalg.qr(np.dot(A, Q))
    A_H = np.conj(np.transpose(A))
    for _ in range(n_iter):
        Q, _ = np.linalg.qr(np.dot(A_H, Q))
        Q, _ = np.linalg.qr(np.dot(A, Q))
    return Q


def randomized_svd(matrix, n_eigenvecs=None, n_oversamples=5, n_iter=2, random_state=None,
                   **kwargs):
    """tensorly/tenalg/svd.py:288-357 (Halko et al. 2009, algorithm 5.1),
    transposing as the reference does to keep the reduced matrix small."""
    n_eigenvecs, min_dim, max_dim = _svd_checks(matrix, n_eigenvecs=n_eigenvecs)
    dim_1, dim_2 = matrix.shape
    n_dims = min(n_eigenvecs + n_oversamples, max_dim)
    if ((dim_1 > dim_2 and n_eigenvecs > min(min_dim, n_dims))
            or (dim_1 < dim_2 and n_eigenvecs < min(min_dim, n_dims))):
        matrix_T = np.transpose(matrix)
        Q = randomized_range_finder(matrix_T, n_dims=n_dims, n_iter=n_iter,
                                    random_state=random_state)
        matrix_reduced = np.transpose(np.dot(np.conj(np.transpose(Q)), matrix_T))
        U, S, V = truncated_svd(matrix_reduced, n_eigenvecs=n_eigenvecs)
        V = np.dot(V, np.transpose(Q))
    else:
        Q = randomized_range_finder(matrix, n_dims=n_dims, n_iter=n_iter,
                                    random_state=random_state)
        matrix_reduced = np.dot(np.conj(np.transpose(Q)), matrix)
        U, S, V = truncated_svd(matrix_reduced, n_eigenvecs=n_eigenvecs)
        U = np.dot(Q, U)
    return U, S, V


def svd_interface(matrix, method="truncated_svd", n_eigenvecs=None, flip_sign=True,
                  u_based_flip_sign=True, non_negative=None, mask=None,
                  n_iter_mask_imputation=5, **kwargs):
    """tensorly/tenalg/svd.py:366-447 ('truncated_svd' or 'randomized_svd');
    the mask refill loop (``:431-439``) and the non-negative branch
    (``:443-444``, ``make_svd_non_negative``)."""
    if method == "truncated_svd":
        svd_fun = truncated_svd
    elif method == "randomized_svd":
        svd_fun = randomized_svd
    else:
        raise NotImplementedError("oracle restates 'truncated_svd' and 'randomized_svd'")
    U, S, V = svd_fun(matrix, n_eigenvecs=n_eigenvecs, **kwargs)
    if mask is not None and n_eigenvecs is not None:
        for _ in range(n_iter_mask_imputation):
            St = np.eye(U.shape[1], V.shape[0], dtype=matrix.dtype)
            for i in range(S.shape[0]):
                St[i, i] = S[i]
            matrix = matrix * mask + (U @ St @ V) * (1 - mask)
            U, S, V = svd_fun(matrix, n_eigenvecs=n_eigenvecs, **kwargs)
    if flip_sign:
        U, V = svd_flip(U, V, u_based_decision=u_based_flip_sign)
    if non_negative is not False and non_negative is not None:
        U, V = make_svd_non_negative(matrix, U, S, V, non_negative)
    return U, S, V


def make_svd_non_negative(tensor, U, S, V, nntype=True):
    """tensorly/tenalg/svd.py:68-134: NNDSVD (Boutsidis & Gallopoulos 2008).
    Column 0 is sqrt(S_0) |U_0|; column j >= 1 takes the positive or the
    negative parts of (U_j, V_j), whichever has the larger product of norms,
    scaled by sqrt(S_j * that product).  'nndsvda' (the default for True)
    then replaces entries below eps by the tensor's mean."""
    if nntype is True:
        nntype = "nndsvda"
    W = np.zeros_like(U)
    H = np.zeros_like(V)
    W[:, 0] = np.sqrt(S[0]) * np.abs(U[:, 0])
    H[0, :] = np.sqrt(S[0]) * np.abs(V[0, :])
    for j in range(1, min(U.shape[1], V.shape[0])):
        x, y = U[:, j], V[j, :]
        x_p, y_p = np.clip(x, 0.0, None), np.clip(y, 0.0, None)
        x_n, y_n = np.abs(np.clip(x, None, 0.0)), np.abs(np.clip(y, None, 0.0))
        x_p_nrm, y_p_nrm = np.linalg.norm(x_p), np.linalg.norm(y_p)
        x_n_nrm, y_n_nrm = np.linalg.norm(x_n), np.linalg.norm(y_n)
        m_p, m_n = x_p_nrm * y_p_nrm, x_n_nrm * y_n_nrm
        if m_p > m_n:
            u, v, sigma = x_p / x_p_nrm, y_p / y_p_nrm, m_p
        else:
            u, v, sigma = x_n / x_n_nrm, y_n / y_n_nrm, m_n
        lbd = np.sqrt(S[j] * sigma)
        W[:, j] = lbd * u
        H[j, :] = lbd * v
    eps = np.finfo(np.asarray(tensor).dtype).eps
    if nntype == "nndsvd":
        W = np.where(W > eps, W - eps, np.where(W < -eps, W + eps, 0.0))
        H = np.where(H > eps, H - eps, np.where(H < -eps, H + eps, 0.0))
    elif nntype == "nndsvda":
        avg = np.mean(tensor)
        W = np.where(W < eps, np.ones(W.shape, dtype=W.dtype) * avg, W)
        H = np.where(H < eps, np.ones(H.shape, dtype=H.dtype) * avg, H)
    else:
        raise ValueError(f'Invalid nntype parameter: got {nntype} instead of one of '
                         '("nndsvd", "nndsvda")')
    return W, H


# --------------------------------------------------------------------------
# CP tensors
# --------------------------------------------------------------------------
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


def random_cp(shape, rank, random_state=None, dtype=np.float64):
    """tensorly/random/base.py:64-114 with ``normalise_factors=False``:
    one ``random_sample((s, rank))`` draw per mode, in mode order (``:104``),
    float64 cast to the tensor dtype; weights are ones (``:105``)."""
    rns = check_random_state(random_state)
    factors = [rns.random_sample((s, rank)).astype(dtype) for s in shape]
    return np.ones(rank, dtype=dtype), factors


def cp_to_tensor(cp_tensor, mask=None):
    """tensorly/cp_tensor.py:433-485: mode-0 unfolding
    ``dot(factors[0]*weights, KR(factors[1:]).T)`` folded back; with a mask,
    the sum over r of the masked Khatri-Rao product of all factors."""
    weights, factors = cp_tensor
    shape = tuple(f.shape[0] for f in factors)
    if len(shape) == 1:
        return np.sum(weights * factors[0], axis=1)
    w = 1 if weights is None else weights
    if mask is None:
        full = np.dot(factors[0] * w, np.transpose(khatri_rao(factors, skip_matrix=0)))
    else:
        full = np.sum(khatri_rao([factors[0] * w] + list(factors[1:]), mask=mask), axis=1)
    return fold(full, 0, shape)


def cp_to_unfolded(cp_tensor, mode):
    """tensorly/cp_tensor.py:488-521."""
    weights, factors = cp_tensor
    a = factors[mode] if weights is None else factors[mode] * weights
    return np.dot(a, np.transpose(khatri_rao(factors, skip_matrix=mode)))


def cp_to_vec(cp_tensor):
    """tensorly/cp_tensor.py:524-546."""
    return np.reshape(cp_to_tensor(cp_tensor), (-1,))


def cp_norm(cp_tensor):
    """tensorly/cp_tensor.py:614-644: sqrt(sum(Hadamard of Grams * w w^T))."""
    weights, factors = cp_tensor
    r = factors[0].shape[1]
    norm = np.ones((r, r), dtype=factors[0].dtype)
    for f in factors:
        norm = norm * np.dot(np.transpose(f), np.conj(f))
    if weights is not None:
        norm = norm * (np.reshape(weights, (-1, 1)) * np.reshape(weights, (1, -1)))
    return np.sqrt(np.sum(norm))


def cp_normalize(cp_tensor):
    """tensorly/cp_tensor.py:278-321: unit-norm columns, norms into weights
    (weights are first folded into factor 0)."""
    weights, factors = cp_tensor
    rank = factors[0].shape[1]
    if weights is None:
        weights = np.ones(rank, dtype=factors[0].dtype)
    out = []
    for i, factor in enumerate(factors):
        if i == 0:
            factor = factor * weights
            weights = np.ones(rank, dtype=factor.dtype)
        scales = norm(factor, axis=0)
        scales_nz = np.where(scales == 0, np.ones(scales.shape, dtype=factor.dtype), scales)
        weights = weights * scales
        out.append(factor / np.reshape(scales_nz, (1, -1)))
    return weights, out


def initialize_cp(tensor, rank, init="svd", svd="truncated_svd", random_state=None,
                  normalize_factors=False, non_negative=False, mask=None, svd_mask_repeats=5):
    """tensorly/decomposition/_cp.py:26-137; ``non_negative`` makes the SVD
    non-negative (NNDSVDA) and takes absolute values (``:129-131``); a mask
    refills each unfolding inside svd_interface."""
    rng = check_random_state(random_state)
    if isinstance(init, str) and init == "random":
        weights, factors = random_cp(tensor.shape, rank, random_state=rng, dtype=tensor.dtype)
    elif isinstance(init, str) and init == "svd":
        factors = []
        for mode in range(tensor.ndim):
            mask_unfold = None if mask is None else unfold(mask, mode)
            U, S, _ = svd_interface(unfold(tensor, mode), n_eigenvecs=rank, method=svd,
                                    non_negative=non_negative, mask=mask_unfold,
                                    n_iter_mask_imputation=svd_mask_repeats)
            if mode == 0:
                idx = min(rank, S.shape[0])
                U = U.copy()
                U[:, :idx] = U[:, :idx] * S[:idx]
            if tensor.shape[mode] < rank:
                random_part = rng.random_sample((U.shape[0], rank - tensor.shape[mode]))
                U = np.concatenate([U, random_part.astype(tensor.dtype)], axis=1)
            factors.append(U[:, :rank])
        weights = None
    elif isinstance(init, (tuple, list)):
        weights, factors = init
        factors = list(factors)
        if weights is None or np.all(weights == 1):
            return None, factors
        avg = np.prod(weights) ** (1.0 / weights.shape[0])
        return None, [f * avg for f in factors]
    else:
        raise ValueError(f'Initialization method "{init}" not recognized')
    if non_negative:
        factors = [np.abs(f) for f in factors]
    if normalize_factors:
        weights, factors = cp_normalize((weights, factors))
    return weights, factors


def non_negative_parafac(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                         tol=10e-7, random_state=None, verbose=0, normalize_factors=False,
                         return_errors=False, mask=None, cvg_criterion="abs_rec_error",
                         fixed_modes=None):
    """tensorly/decomposition/_nn_cp.py:26-183: non-negative CP by the
    multiplicative updates of Shashua & Hazan (ICML 2005).  Per mode
    (``:116-138``): accum = Hadamard of the other Grams scaled by w w^T;
    A <- A * clip(MTTKRP, eps) / clip(A accum, eps).  The error (``:140-152``,
    only when ``tol``) uses the last mode's MTTKRP; stop on the 'abs_rec_error'
    or 'rec_error' test from the second iteration on."""
    if mask is not None:
        raise NotImplementedError("oracle restates the unmasked branch only")
    tensor = np.asarray(tensor)
    epsilon = np.finfo(tensor.dtype).eps
    rank = validate_cp_rank(tensor.shape, rank=rank)
    weights, factors = initialize_cp(tensor, rank, init=init, svd=svd,
                                     random_state=random_state,
                                     normalize_factors=normalize_factors, non_negative=True)
    if weights is None:
        weights = np.ones(rank, dtype=tensor.dtype)
    factors = list(factors)
    rec_errors = []
    norm_tensor = norm(tensor)
    fixed_modes = [] if fixed_modes is None else list(fixed_modes)
    if tensor.ndim - 1 in fixed_modes:
        warnings.warn("You asked for fixing the last mode, which is not supported while tol "
                      "is fixed.\n The last mode will not be fixed. Consider using tl.moveaxis()")
        fixed_modes.remove(tensor.ndim - 1)
    modes_list = [m for m in range(tensor.ndim) if m not in fixed_modes]
    mttkrp = None
    for iteration in range(n_iter_max):
        for mode in modes_list:
            accum = None
            for i, e in enumerate([k for k in range(len(factors)) if k != mode]):
                g = factors[e].T @ factors[e]
                accum = g if i == 0 else accum * g
            accum = weights.reshape(-1, 1) * accum * weights.reshape(1, -1)
            mttkrp = unfolding_dot_khatri_rao(tensor, (weights, factors), mode)
            numerator = np.clip(mttkrp, epsilon, None)
            denominator = np.clip(factors[mode] @ accum, epsilon, None)
            factors[mode] = factors[mode] * numerator / denominator
            if normalize_factors and mode != modes_list[-1]:
                weights, factors = cp_normalize((weights, factors))
        if tol:
            rec_error = error_calc(tensor, norm_tensor, weights, factors, mttkrp) / norm_tensor
            rec_errors.append(rec_error)
            if iteration >= 1:
                dec = rec_errors[-2] - rec_errors[-1]
                if cvg_criterion == "abs_rec_error":
                    stop = abs(dec) < tol
                elif cvg_criterion == "rec_error":
                    stop = dec < tol
                else:
                    raise TypeError("Unknown convergence criterion")
                if stop:
                    break
        if normalize_factors:
            weights, factors = cp_normalize((weights, factors))
    cp = (weights, factors)
    return (cp, rec_errors) if return_errors else cp


def hals_nnls(UtM, UtU, V=None, n_iter_max=500, tol=1e-8, sparsity_coefficient=None,
              ridge_coefficient=None, nonzero_rows=False, exact=False, epsilon=0.0):
    """tensorly/solvers/nnls.py:5-150: row-wise (Gauss-Seidel) HALS for
    min_{V >= epsilon} ||M - U V||.  The inner stop test compares the sum,
    over the rows k updated in an iteration, of ||V - newV||^2 with newV
    broadcast against every row of V (the reference's expression), to tol
    times the first iteration's sum."""
    rank = UtM.shape[0]
    if V is None:
        V = np.linalg.solve(UtU, UtM)
        V = np.clip(V, 0, None)
        scale = np.sum(UtM * V) / np.sum(UtU * (V @ V.T))
        V = V * scale
    V = np.array(V, copy=True)
    if exact:
        n_iter_max = 50000
        tol = 1e-16
    rec_error0 = None
    for iteration in range(n_iter_max):
        rec_error = 0
        for k in range(rank):
            if UtU[k, k]:
                num = UtM[k, :] - UtU[k, :] @ V + UtU[k, k] * V[k, :]
                den = UtU[k, k]
                if sparsity_coefficient is not None:
                    num = num - sparsity_coefficient
                if ridge_coefficient is not None:
                    den = den + 2 * ridge_coefficient
                newV = np.clip(num / den, epsilon, None)
                rec_error += np.linalg.norm(V - newV) ** 2
                V[k, :] = newV
                if nonzero_rows and np.all(V[k, :] == 0):
                    V[k, :] = np.finfo(V.dtype).eps * np.max(V)
            elif nonzero_rows:
                raise ValueError("Column " + str(k) + " of U is zero with nonzero condition")
        if iteration == 0:
            rec_error0 = rec_error
        if rec_error < tol * rec_error0:
            break
    return V


def non_negative_parafac_hals(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                              tol=10e-8, random_state=None, sparsity_coefficients=None,
                              fixed_modes=None, nn_modes="all", exact=False,
                              normalize_factors=False, verbose=False, return_errors=False,
                              cvg_criterion="abs_rec_error"):
    """tensorly/decomposition/_nn_cp.py:186-377: non-negative CP by HALS
    (Gillis & Glineur 2012).  Per free mode: the Hadamard of the other Grams,
    the MTTKRP, then ``hals_nnls(M^T, pinv, A^T, n_iter_max=100)`` (or the
    unconstrained solve for modes outside ``nn_modes``); the error from the
    last MTTKRP when ``tol``."""
    tensor = np.asarray(tensor)
    weights, factors = initialize_cp(tensor, rank, init=init, svd=svd, random_state=random_state,
                                     normalize_factors=normalize_factors, non_negative=True)
    if weights is None:
        weights = np.ones(rank, dtype=tensor.dtype)
    factors = list(factors)
    norm_tensor = norm(tensor)
    n_modes = tensor.ndim
    if sparsity_coefficients is None or isinstance(sparsity_coefficients, float):
        sparsity_coefficients = [sparsity_coefficients] * n_modes
    sparsity_coefficients = list(sparsity_coefficients)
    fixed_modes = [] if fixed_modes is None else list(fixed_modes)
    if nn_modes == "all":
        nn_modes = set(range(n_modes))
    elif nn_modes is None:
        nn_modes = set()
    for fixed_value in fixed_modes:
        sparsity_coefficients[fixed_value] = None
    for mode in range(n_modes):
        if sparsity_coefficients[mode] is not None:
            warnings.warn("Sparsity coefficient is ignored in unconstrained modes.")
    modes = [m for m in range(n_modes) if m not in fixed_modes]
    rec_errors = []
    mttkrp = None
    for iteration in range(n_iter_max):
        for mode in modes:
            pseudo_inverse = np.ones((rank, rank), dtype=tensor.dtype)
            for i, factor in enumerate(factors):
                if i != mode:
                    pseudo_inverse = pseudo_inverse * (factor.T @ factor)
            pseudo_inverse = weights.reshape(-1, 1) * pseudo_inverse * weights.reshape(1, -1)
            mttkrp = unfolding_dot_khatri_rao(tensor, (weights, factors), mode)
            if mode in nn_modes:
                nn_factor = hals_nnls(mttkrp.T, pseudo_inverse, factors[mode].T, n_iter_max=100,
                                      sparsity_coefficient=sparsity_coefficients[mode],
                                      exact=exact)
                factors[mode] = nn_factor.T
            else:
                factors[mode] = np.linalg.solve(pseudo_inverse.T, mttkrp.T).T
            if normalize_factors and mode != modes[-1]:
                weights, factors = cp_normalize((weights, factors))
        if tol:
            factors_norm = cp_norm((weights, factors))
            iprod = np.sum(np.sum(mttkrp * factors[-1], axis=0))
            rec_error = np.sqrt(np.abs(norm_tensor ** 2 + factors_norm ** 2 - 2 * iprod)) \
                / norm_tensor
            rec_errors.append(rec_error)
            if iteration >= 1:
                dec = rec_errors[-2] - rec_errors[-1]
                if cvg_criterion == "abs_rec_error":
                    stop = abs(dec) < tol
                elif cvg_criterion == "rec_error":
                    stop = dec < tol
                else:
                    raise TypeError("Unknown convergence criterion")
                if stop:
                    break
        if normalize_factors:
            weights, factors = cp_normalize((weights, factors))
    cp = (weights, factors)
    return (cp, rec_errors) if return_errors else cp


def sample_khatri_rao(matrices, n_samples, skip_matrix=None, indices_list=None,
                      return_sampled_rows=False, random_state=None):
    """tensorly/decomposition/_cp.py:546-630 (no warning text)."""
    if skip_matrix is not None:
        matrices = [matrices[i] for i in range(len(matrices)) if i != skip_matrix]
    if indices_list is None:
        rng = random_state if isinstance(random_state, np.random.RandomState) \
            else check_random_state(random_state)
        indices_list = [rng.randint(0, m.shape[0], size=n_samples, dtype=int) for m in matrices]
    rank = matrices[0].shape[1]
    sizes = [m.shape[0] for m in matrices]
    if return_sampled_rows:
        indices_kr = np.zeros((n_samples), dtype=int)
        for size, indices in zip(sizes, indices_list):
            indices_kr = indices_kr * size + indices
    sampled_kr = np.ones((n_samples, rank), dtype=matrices[0].dtype)
    for indices, matrix in zip(indices_list, matrices):
        sampled_kr = sampled_kr * matrix[indices, :]
    if return_sampled_rows:
        return sampled_kr, indices_list, indices_kr
    return sampled_kr, indices_list


def randomised_parafac(tensor, rank, n_samples, n_iter_max=100, init="random",
                       svd="truncated_svd", tol=10e-9, max_stagnation=20, return_errors=False,
                       random_state=None):
    """tensorly/decomposition/_cp.py:633-762 (no callback, not verbose):
    per mode the least-squares update from sampled Khatri-Rao rows, the error
    ||X - [[A]]|| / ||X|| after each iteration, the tol and stagnation stops."""
    rank = validate_cp_rank(tensor.shape, rank=rank)
    rng = check_random_state(random_state)
    _, factors = initialize_cp(tensor, rank, init=init, svd=svd, random_state=random_state)
    factors = list(factors)
    rec_errors = []
    n_dims = tensor.ndim
    norm_tensor = norm(tensor)
    min_error = 0
    weights = np.ones(rank, dtype=tensor.dtype)
    for iteration in range(n_iter_max):
        for mode in range(n_dims):
            kr_prod, indices_list = sample_khatri_rao(factors, n_samples, skip_matrix=mode,
                                                      random_state=rng)
            indices_list = [i.tolist() for i in indices_list]
            indices_list.insert(mode, slice(None, None, None))
            indices_list = tuple(indices_list)
            if mode:
                sampled_unfolding = tensor[indices_list]
            else:
                sampled_unfolding = np.transpose(tensor[indices_list])
            pseudo_inverse = np.dot(np.transpose(kr_prod), kr_prod)
            factor = np.dot(np.transpose(kr_prod), sampled_unfolding)
            factor = np.transpose(np.linalg.solve(pseudo_inverse, factor))
            factors[mode] = factor
        if max_stagnation or tol:
            rec_error = norm(tensor - cp_to_tensor((weights, factors))) / norm_tensor
            if not min_error or rec_error < min_error:
                min_error = rec_error
                stagnation = -1
            stagnation += 1
            rec_errors.append(rec_error)
            if iteration > 1:
                if (tol and abs(rec_errors[-2] - rec_errors[-1]) < tol) or (
                        stagnation and (stagnation > max_stagnation)):
                    break
    if return_errors:
        return (weights, factors), rec_errors
    return weights, factors


_CONSTRAINT_NAMES = ("non_negative", "l1_reg", "l2_reg", "l2_square_reg", "unimodality",
                     "normalize", "simplex", "normalized_sparsity", "soft_sparsity",
                     "smoothness", "monotonicity", "hard_sparsity")


def validate_constraints(n_const=1, order=0, **given):
    """tensorly/tenalg/proximal.py:4-145: (constraint name, parameter) of mode
    ``order``.  A scalar applies to every mode; a list gives every mode the
    constraint with its own entry; a dict constrains the listed modes."""
    constraints = [None] * n_const
    parameters = [None] * n_const
    values = [given.get(n) for n in _CONSTRAINT_NAMES]
    seen = set()
    for v in values:
        if v:
            if isinstance(v, dict):
                for mode in v:
                    if mode in seen:
                        raise ValueError("You selected two constraints for the same mode. "
                                         "Consider to check your input")
                    seen.add(mode)
            elif isinstance(v, list):
                for mode in range(len(v)):
                    if v[mode]:
                        if mode in seen:
                            raise ValueError("You selected two constraints for the same "
                                             "mode. Consider to check your input")
                        seen.add(mode)
            else:
                if len(seen) > 0:
                    raise ValueError("You selected two constraints for the same mode. "
                                     "Consider to check your input")
                for i in range(n_const):
                    seen.add(i)
    for v, name in zip(values, _CONSTRAINT_NAMES):
        if v:
            if isinstance(v, dict):
                for mode in v:
                    constraints[mode] = name
                    parameters[mode] = v[mode]
            else:
                for i in range(n_const):
                    constraints[i] = name
                    parameters[i] = v[i] if isinstance(v, list) else v
    return constraints[order], parameters[order]


def proximal_operator(tensor, n_const=1, order=0, **given):
    """tensorly/tenalg/proximal.py:148-267: the whole-matrix operators here,
    the column-wise and sparsity ones from proximal_oracle (:270-628)."""
    if n_const is None:
        return tensor
    constraint, parameter = validate_constraints(n_const=n_const, order=order, **given)
    if constraint is None:
        return tensor
    if constraint == "non_negative":
        return np.clip(tensor, 0, np.max(tensor))
    if constraint == "l1_reg":                      # soft_thresholding, :631-671
        return np.sign(tensor) * np.clip(np.abs(tensor) - parameter, a_min=0, a_max=None)
    if constraint == "l2_reg":                      # l2_prox, :466-493
        nrm = norm(tensor)
        bigger = nrm if nrm > parameter else parameter
        return tensor - (tensor * parameter / bigger)
    if constraint == "l2_square_reg":               # l2_square_prox, :444-463
        return tensor / (1 + 2 * parameter)
    if constraint == "normalize":
        return tensor / np.max(np.abs(tensor))
    from . import proximal_oracle as po             # the column-wise and sparsity operators
    if constraint == "unimodality":
        return po.unimodality_prox(tensor)
    if constraint == "simplex":
        return po.simplex_prox(tensor, parameter)
    if constraint == "normalized_sparsity":
        return po.normalized_sparsity_prox(tensor, parameter)
    if constraint == "soft_sparsity":
        return po.soft_sparsity_prox(tensor, parameter)
    if constraint == "smoothness":
        return po.smoothness_prox(tensor, parameter)
    if constraint == "monotonicity":
        return po.monotonicity_prox(tensor)
    if constraint == "hard_sparsity":
        return po.hard_thresholding(tensor, parameter)
    raise NotImplementedError(f"oracle restates no {constraint} proximal operator")


def admm(UtM, UtU, x, dual_var, n_iter_max=100, n_const=None, order=None, tol=1e-4, **given):
    """tensorly/solvers/admm.py:5-135."""
    rho = np.trace(UtU) / x.shape[1]
    x_split = None
    for _ in range(n_iter_max):
        x_old = np.copy(x)
        x_split = np.linalg.solve(np.transpose(UtU + rho * np.eye(UtU.shape[1])),
                                  np.transpose(UtM + rho * (x + dual_var)))
        x = proximal_operator(np.transpose(x_split) - dual_var, n_const=n_const, order=order,
                              **given)
        if n_const is None:
            x = np.transpose(np.linalg.solve(np.transpose(UtU), np.transpose(UtM)))
            return x, x_split, dual_var
        dual_var = dual_var + x - np.transpose(x_split)
        dual_residual = x - np.transpose(x_split)
        primal_residual = x - x_old
        if norm(dual_residual) < tol * norm(x) and norm(primal_residual) < tol * norm(dual_var):
            break
    return x, x_split, dual_var


def fista(UtM, UtU, x=None, n_iter_max=100, non_negative=True, sparsity_coef=0, ridge_coef=0,
          lr=None, tol=1e-8, epsilon=1e-8):
    """tensorly/solvers/nnls.py:177-272."""
    if sparsity_coef is None:
        sparsity_coef = 0
    if x is None:
        x = np.zeros(UtM.shape, dtype=UtM.dtype)
    if lr is None:
        lr = 1 / (truncated_svd(UtU)[1][0] + 2 * ridge_coef)
    momentum_old = 1.0
    norm_0 = 0.0
    x_update = np.copy(x)
    for iteration in range(n_iter_max):
        if isinstance(UtU, list):
            x_gradient = (-UtM + multi_mode_dot(x_update, UtU, transpose=False) + sparsity_coef
                          + 2 * ridge_coef * x_update)
        else:
            x_gradient = -UtM + np.dot(UtU, x_update) + sparsity_coef + 2 * ridge_coef * x_update
        x_new = x_update - lr * x_gradient
        if non_negative:
            x_new = np.where(x_new < epsilon, epsilon, x_new)
        momentum = (1 + math.sqrt(1 + 4 * momentum_old ** 2)) / 2
        x_update = x_new + ((momentum_old - 1) / momentum) * (x_new - x)
        momentum_old = momentum
        nrm = abs(np.sum(x - x_new))
        x = np.copy(x_new)
        if iteration == 0:
            norm_0 = nrm
        if nrm < tol * norm_0:
            break
    return x


def tucker_normalize(tucker_tensor):
    """tensorly/tucker_tensor.py:78-102: unit-norm factor columns, the norms
    multiplied into the core along each mode in mode order."""
    core, factors = tucker_tensor
    out = []
    for i, factor in enumerate(factors):
        scales = np.linalg.norm(factor, axis=0)
        nz = np.where(scales == 0, np.ones(scales.shape, dtype=factor.dtype), scales)
        core = core * np.reshape(scales, (1,) * i + (-1,) + (1,) * (core.ndim - i - 1))
        out.append(factor / np.reshape(nz, (1, -1)))
    return core, out


def kronecker(matrices):
    """tensorly/tenalg/core_tenalg/_kronecker.py: left-to-right Kronecker product."""
    res = matrices[0]
    for m in matrices[1:]:
        res = np.kron(res, m)
    return res


def _active_solve(UtU, Utm, passive_set, support_vec):
    """Solve on the passive set and scatter into the support vector."""
    passive_solution = np.linalg.solve(UtU[passive_set, :][:, passive_set], Utm[passive_set])
    support_vec = np.zeros(support_vec.shape, dtype=support_vec.dtype)
    support_vec[passive_set] = passive_solution
    return support_vec


def active_set_nnls(Utm, UtU, x=None, n_iter_max=100, tol=10e-8):
    """tensorly/solvers/nnls.py:275-406: Lawson-Hanson style active set."""
    x_vec = np.zeros(UtU.shape[1], dtype=UtU.dtype) if x is None else np.reshape(x, (-1,))
    x_gradient = Utm - np.dot(UtU, x_vec)
    passive_set = x_vec > 0
    active_set = x_vec <= 0
    support_vec = np.zeros(x_vec.shape, dtype=x_vec.dtype)
    for iteration in range(n_iter_max):
        if iteration > 0 or np.all(x_vec == 0):
            indice = np.argmax(x_gradient)
            passive_set = passive_set.copy()
            active_set = active_set.copy()
            passive_set[indice] = True
            active_set[indice] = False
        try:
            support_vec = _active_solve(UtU, Utm, passive_set, support_vec)
        except Exception:
            x_vec = np.zeros(UtU.shape[1])
            support_vec = np.zeros(x_vec.shape, dtype=x_vec.dtype)
            passive_set = x_vec > 0
            active_set = x_vec <= 0
            if np.any(active_set):
                indice = np.argmax(x_gradient)
                passive_set[indice] = True
                active_set[indice] = False
            support_vec = _active_solve(UtU, Utm, passive_set, support_vec)
        if np.min(support_vec[passive_set]) <= 0:
            for _ in range(len(passive_set)):
                sel = support_vec[passive_set] <= 0
                alpha = np.min(x_vec[passive_set][sel]
                               / (x_vec[passive_set][sel] - support_vec[passive_set][sel]))
                x_vec = x_vec + alpha * (support_vec - x_vec)
                passive_set = x_vec > 0
                active_set = x_vec <= 0
                support_vec = _active_solve(UtU, Utm, passive_set, support_vec)
                if np.any(passive_set) != True or np.min(support_vec[passive_set]) > 0:
                    break
        x_vec = np.clip(support_vec, 0, np.max(support_vec))
        x_gradient = Utm - np.dot(UtU, x_vec)
        if np.any(active_set) != True or np.max(x_gradient[active_set]) <= tol:
            break
    return x_vec


def non_negative_tucker_hals(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
                             tol=1e-8, sparsity_coefficients=None, core_sparsity_coefficient=None,
                             random_state=None, return_errors=False, exact=False,
                             algorithm="fista", normalize_factors=False):
    """tensorly/decomposition/_tucker.py:457-691 (no fixed modes; algorithm
    'fista' or 'active_set')."""
    rank = validate_tucker_rank(tensor.shape, rank=rank)
    n_modes = tensor.ndim
    if sparsity_coefficients is None or not isinstance(sparsity_coefficients, (list, tuple)):
        sparsity_coefficients = [sparsity_coefficients] * n_modes
    modes = list(range(n_modes))
    nn_core, nn_factors = initialize_tucker(tensor, rank, modes, init=init, svd=svd,
                                            random_state=random_state, non_negative=True)
    nn_factors = list(nn_factors)
    norm_tensor = norm(tensor)
    rec_errors = []
    for iteration in range(n_iter_max):
        for mode in modes:
            pseudo_inverse = list(nn_factors)
            for i, factor in enumerate(nn_factors):
                if i != mode:
                    pseudo_inverse[i] = np.dot(np.conj(np.transpose(factor)), factor)
            core_cross = multi_mode_dot(nn_core, pseudo_inverse, skip=mode)
            UtU = np.dot(unfold(core_cross, mode), np.transpose(unfold(nn_core, mode)))
            tensor_cross = multi_mode_dot(tensor, nn_factors, skip=mode, transpose=True)
            MtU = np.dot(unfold(tensor_cross, mode), np.transpose(unfold(nn_core, mode)))
            UtM = np.transpose(MtU)
            nn_factor = hals_nnls(UtM, UtU, np.transpose(nn_factors[mode]), n_iter_max=100,
                                  sparsity_coefficient=sparsity_coefficients[mode], exact=exact)
            nn_factors[mode] = np.transpose(nn_factor)
        pseudo_inverse[-1] = np.dot(np.transpose(nn_factors[-1]), nn_factors[-1])
        if algorithm == "fista":
            core_estimation = multi_mode_dot(tensor, nn_factors, transpose=True)
            learning_rate = 1
            for MtM in pseudo_inverse:
                learning_rate *= 1 / (truncated_svd(MtM)[1][0])
            nn_core = fista(core_estimation, pseudo_inverse, x=nn_core, n_iter_max=n_iter_max,
                            sparsity_coef=core_sparsity_coefficient, lr=learning_rate)
        elif algorithm == "active_set":
            core_estimation_vec = np.reshape(
                mode_dot(tensor_cross, np.transpose(nn_factors[modes[-1]]), modes[-1]), (-1,))
            vectorcore = active_set_nnls(core_estimation_vec, kronecker(pseudo_inverse),
                                         x=nn_core, n_iter_max=n_iter_max)
            nn_core = np.reshape(vectorcore, nn_core.shape)
        rec_error = norm(tensor - tucker_to_tensor((nn_core, nn_factors))) / norm_tensor
        rec_errors.append(rec_error)
        if iteration > 1:
            if tol and abs(rec_errors[-2] - rec_errors[-1]) < tol:
                break
        if normalize_factors:
            nn_core, nn_factors = tucker_normalize((nn_core, nn_factors))
    if return_errors:
        return (nn_core, nn_factors), rec_errors
    return nn_core, nn_factors


def initialize_constrained_parafac(tensor, rank, init="svd", svd="truncated_svd",
                                   random_state=None, **given):
    """tensorly/decomposition/_constrained_cp.py:22-163 ('random': the global
    NumPy generator, as the reference's random_cp without a seed)."""
    n_modes = tensor.ndim
    rng = check_random_state(random_state)
    if init == "random":
        rns = check_random_state(None)
        factors = [rns.random_sample((s, rank)).astype(tensor.dtype) for s in tensor.shape]
    elif init == "svd":
        factors = []
        for mode in range(n_modes):
            U, S, _ = svd_interface(unfold(tensor, mode), n_eigenvecs=rank, method=svd)
            if mode == 0:
                idx = min(rank, S.shape[0])
                U = U.copy()
                U[:, :idx] = U[:, :idx] * S[:idx]
            if tensor.shape[mode] < rank:
                random_part = rng.random_sample((U.shape[0], rank - tensor.shape[mode]))
                U = np.concatenate([U, random_part.astype(U.dtype)], axis=1)
            factors.append(U[:, :rank])
    else:
        weights, factors = init
        factors = list(factors)
        if not np.all(weights == 1):
            weights_avg = np.prod(weights) ** (1.0 / weights.shape[0])
            factors = [f * weights_avg for f in factors]
        return None, factors
    for i in range(n_modes):
        factors[i] = proximal_operator(factors[i], n_const=n_modes, order=i, **given)
    return None, factors


def constrained_parafac(tensor, rank, n_iter_max=100, n_iter_max_inner=10, init="svd",
                        svd="truncated_svd", tol_outer=1e-8, tol_inner=1e-6, random_state=None,
                        return_errors=False, cvg_criterion="abs_rec_error", fixed_modes=None,
                        **given):
    """tensorly/decomposition/_constrained_cp.py:166-435 (AO-ADMM)."""
    rank = validate_cp_rank(tensor.shape, rank=rank)
    _, factors = initialize_constrained_parafac(tensor, rank, init=init, svd=svd,
                                                random_state=random_state, **given)
    weights = np.ones(rank, dtype=tensor.dtype)
    rec_errors = []
    norm_tensor = norm(tensor)
    fixed_modes = [] if fixed_modes is None else list(fixed_modes)
    if tensor.ndim - 1 in fixed_modes:
        warnings.warn("You asked for fixing the last mode, which is not supported.\n "
                      "The last mode will not be fixed. Consider using tl.moveaxis()")
        fixed_modes.remove(tensor.ndim - 1)
    modes_list = [m for m in range(tensor.ndim) if m not in fixed_modes]
    dual_variables = [np.zeros(f.shape) for f in factors]
    factors_aux = [np.transpose(np.zeros(f.shape)) for f in factors]
    mttkrp = None
    for iteration in range(n_iter_max):
        for mode in modes_list:
            pseudo_inverse = np.ones((rank, rank), dtype=tensor.dtype)
            for i, factor in enumerate(factors):
                if i != mode:
                    pseudo_inverse = pseudo_inverse * np.dot(np.transpose(factor), factor)
            mttkrp = unfolding_dot_khatri_rao(tensor, (None, factors), mode)
            factors[mode], factors_aux[mode], dual_variables[mode] = admm(
                mttkrp, pseudo_inverse, factors[mode], dual_variables[mode],
                n_iter_max=n_iter_max_inner, n_const=tensor.ndim, order=mode, tol=tol_inner,
                **given)
        factors_norm = cp_norm((weights, factors))
        iprod = np.sum(np.sum(mttkrp * factors[-1], axis=0) * weights)
        rec_error = np.sqrt(np.abs(norm_tensor ** 2 + factors_norm ** 2 - 2 * iprod)) / norm_tensor
        rec_errors.append(rec_error)
        constraint_error = 0
        for mode in modes_list:
            constraint_error += norm(factors[mode] - np.transpose(factors_aux[mode])) / \
                norm(factors[mode])
        if tol_outer:
            if iteration >= 1:
                dec = rec_errors[-2] - rec_errors[-1]
                if constraint_error < tol_outer:
                    break
                if cvg_criterion == "abs_rec_error":
                    stop_flag = abs(dec) < tol_outer
                elif cvg_criterion == "rec_error":
                    stop_flag = dec < tol_outer
                else:
                    raise TypeError("Unknown convergence criterion")
                if stop_flag:
                    break
    if return_errors:
        return (weights, factors), rec_errors
    return weights, factors


def error_calc(tensor, norm_tensor, weights, factors, mttkrp):
    """tensorly/decomposition/_cp.py:162-227, fast branch ``:217-225``:
    ||X - rec||^2 = ||X||^2 + ||rec||^2 - 2 <X, rec>, with <X, rec> taken from
    the last mode's MTTKRP."""
    factors_norm = cp_norm((weights, factors))
    iprod = np.sum(np.sum(mttkrp * np.conj(factors[-1]), axis=0))
    return np.sqrt(np.abs(norm_tensor ** 2 + factors_norm ** 2 - 2 * iprod))


def sparsify_tensor(tensor, card):
    """tensorly/decomposition/_cp.py:140-159: keep the ``card`` entries of
    largest magnitude."""
    if card >= np.prod(tensor.shape):
        return tensor
    bound = np.sort(np.abs(tensor), axis=None)[-card]
    return np.where(np.abs(tensor) < bound, np.zeros(tensor.shape, dtype=tensor.dtype), tensor)


def error_calc_ext(tensor, norm_tensor, weights, factors, sparsity, mask, mttkrp=None):
    """tensorly/decomposition/_cp.py:162-227 (all branches): returns
    (unnormalised error, tensor, norm_tensor); with a mask the tensor's
    missing entries are refilled from the model."""
    if (mask is not None) or (mttkrp is None):
        low_rank_component = cp_to_tensor((weights, factors))
        if mask is not None:
            tensor = tensor * mask + low_rank_component * (1 - mask)
            norm_tensor = norm(tensor)
        if sparsity:
            sparse_component = sparsify_tensor(tensor - low_rank_component, sparsity)
        else:
            sparse_component = 0.0
        unnorm = norm(tensor - low_rank_component - sparse_component)
    else:
        if sparsity:
            low_rank_component = cp_to_tensor((weights, factors))
            sparse_component = sparsify_tensor(tensor - low_rank_component, sparsity)
            unnorm = norm(tensor - low_rank_component - sparse_component)
        else:
            unnorm = error_calc(tensor, norm_tensor, weights, factors, mttkrp)
    return unnorm, tensor, norm_tensor


def parafac(tensor, rank, n_iter_max=100, init="svd", svd="truncated_svd",
            normalize_factors=False, orthogonalise=False, tol=1e-8, random_state=None,
            verbose=0, return_errors=False, sparsity=None, l2_reg=0, mask=None,
            cvg_criterion="abs_rec_error", fixed_modes=None, svd_mask_repeats=5,
            linesearch=False, callback=None):
    """tensorly/decomposition/_cp.py:230-543.

    Per sweep and mode (``:407-428``): Hadamard of the other factors' Grams
    plus ``l2_reg*I``, scaled by ``w w^T``; MTTKRP; ``solve(V^H, M^T)^T``
    (LAPACK gesv).  Error from the last mode's MTTKRP (``:437-440``), stop on
    ``|e[-2]-e[-1]| < tol`` (``:505-524``), then optional normalisation
    (``:529-530``).  Also the orthogonalisation (QR of the factors in the
    first sweeps, ``:392-397``), the line search (``:398-401``, ``:430-478``),
    the sparse component (``:366-370``, ``:532-536``) and the mask (missing
    entries refilled from the model, ``:441-446``; a masked 'svd' start
    refills each unfolding inside svd_interface).  Returns
    ``((weights, factors), errors)`` or ``(weights, factors)``; with sparsity
    ``((weights, factors), sparse)`` in place of the CP pair.
    """
    if callback is not None and sparsity:
        raise NotImplementedError("oracle restates callbacks without sparsity")
    rank = validate_cp_rank(tensor.shape, rank=rank)
    if orthogonalise and not isinstance(orthogonalise, int):
        orthogonalise = n_iter_max
    acc_pow, acc_fail, max_fail = 2.0, 0, 4
    weights, factors = initialize_cp(tensor, rank, init=init, svd=svd,
                                     random_state=random_state,
                                     normalize_factors=normalize_factors, mask=mask,
                                     svd_mask_repeats=svd_mask_repeats)
    factors = [np.array(f, copy=True) for f in factors]
    if weights is None:
        weights = np.ones(rank, dtype=tensor.dtype)
    rec_errors = []
    norm_tensor = norm(tensor)
    Id = np.eye(rank, dtype=tensor.dtype) * l2_reg if l2_reg else 0
    fixed_modes = [] if fixed_modes is None else list(fixed_modes)
    if fixed_modes == list(range(tensor.ndim)):
        return (weights, factors)
    if tensor.ndim - 1 in fixed_modes:
        warnings.warn("You asked for fixing the last mode, which is not supported.")
        fixed_modes.remove(tensor.ndim - 1)
    modes_list = [m for m in range(tensor.ndim) if m not in fixed_modes]
    if sparsity:
        if isinstance(sparsity, float):
            sparsity = int(sparsity * np.prod(tensor.shape))
        else:
            sparsity = int(sparsity)
    if callback is not None:
        unnorm = error_calc_full(tensor, weights, factors)
        callback((weights, factors), unnorm / norm_tensor)
    mttkrp = None
    unnorm = None
    for iteration in range(n_iter_max):
        if orthogonalise and iteration <= orthogonalise:
            factors = [np.linalg.qr(f)[0] if min(f.shape) >= rank else f for f in factors]
        if linesearch and iteration % 2 == 0:
            factors_last = [np.copy(f) for f in factors]
            weights_last = np.copy(weights)
        for mode in modes_list:
            V = np.ones((rank, rank), dtype=tensor.dtype)
            for i, f in enumerate(factors):
                if i != mode:
                    V = V * np.dot(np.conj(np.transpose(f)), f)
            V = V + Id
            V = np.reshape(weights, (-1, 1)) * V * np.reshape(weights, (1, -1))
            mttkrp = unfolding_dot_khatri_rao(tensor, (weights, factors), mode)
            factors[mode] = np.transpose(
                np.linalg.solve(np.conj(np.transpose(V)), np.transpose(mttkrp)))
        line_iter = bool(linesearch and iteration % 2 == 0 and iteration > 5)
        if (tol or return_errors) and not line_iter:
            unnorm, tensor, norm_tensor = error_calc_ext(tensor, norm_tensor, weights, factors,
                                                         sparsity, mask, mttkrp)
        elif mask is not None:
            tensor = tensor * mask + cp_to_tensor((weights, factors), mask=1 - mask)
        if line_iter:
            jump = iteration ** (1.0 / acc_pow)
            new_weights = weights_last + (weights - weights_last) * jump
            new_factors = [factors_last[ii] + (factors[ii] - factors_last[ii]) * jump
                           for ii in range(tensor.ndim)]
            new_err, new_tensor, new_norm = error_calc_ext(tensor, norm_tensor, new_weights,
                                                           new_factors, sparsity, mask)
            if (new_err / new_norm) < rec_errors[-1]:
                factors, weights = new_factors, new_weights
                tensor, norm_tensor = new_tensor, new_norm
                unnorm = new_err
                acc_fail = 0
            else:
                unnorm, tensor, norm_tensor = error_calc_ext(tensor, norm_tensor, weights,
                                                             factors, sparsity, mask, mttkrp)
                acc_fail += 1
                if acc_fail == max_fail:
                    acc_pow += 1.0
                    acc_fail = 0
        if (tol or return_errors) and not line_iter:
            rec_errors.append(unnorm / norm_tensor)
        if callback is not None:
            if callback((weights, factors), rec_errors[-1]) is True:
                break
        if tol and iteration >= 1:
            dec = rec_errors[-2] - rec_errors[-1]
            if cvg_criterion == "abs_rec_error":
                stop = abs(dec) < tol
            elif cvg_criterion == "rec_error":
                stop = dec < tol
            else:
                raise TypeError("Unknown convergence criterion")
            if stop:
                break
        if normalize_factors:
            weights, factors = cp_normalize((weights, factors))
            factors = list(factors)
    cp = (weights, factors)
    if sparsity:
        cp = (cp, sparsify_tensor(tensor - cp_to_tensor(cp), sparsity))
    if return_errors:
        return cp, rec_errors
    return cp


def error_calc_full(tensor, weights, factors):
    """tensorly/decomposition/_cp.py:194-207 (``mttkrp=None`` branch, no mask):
    norm of the explicit residual."""
    return norm(tensor - cp_to_tensor((weights, factors)))


def parafac_sweeps(tensor, weights, factors, n_sweeps, l2_reg=0.0, norm_tensor=None):
    """A bounded number of ALS sweeps from given factors (the body of
    tensorly/decomposition/_cp.py:394-440), used to time a CPU sample of a
    long run.  ``norm_tensor``: ||X|| when the caller already has it (parafac
    computes it once per run, tensorly/decomposition/_cp.py:350), so that
    consecutive samples of one run do not recompute it.  Returns (weights,
    factors, errors)."""
    rank = factors[0].shape[1]
    factors = [np.array(f, copy=True) for f in factors]
    if norm_tensor is None:
        norm_tensor = norm(tensor)
    Id = np.eye(rank, dtype=tensor.dtype) * l2_reg if l2_reg else 0
    errors = []
    for _ in range(n_sweeps):
        for mode in range(tensor.ndim):
            V = np.ones((rank, rank), dtype=tensor.dtype)
            for i, f in enumerate(factors):
                if i != mode:
                    V = V * np.dot(np.conj(np.transpose(f)), f)
            V = V + Id
            V = np.reshape(weights, (-1, 1)) * V * np.reshape(weights, (1, -1))
            mttkrp = unfolding_dot_khatri_rao(tensor, (weights, factors), mode)
            factors[mode] = np.transpose(
                np.linalg.solve(np.conj(np.transpose(V)), np.transpose(mttkrp)))
        errors.append(error_calc(tensor, norm_tensor, weights, factors, mttkrp) / norm_tensor)
    return weights, factors, errors


# --------------------------------------------------------------------------
# Tucker
# --------------------------------------------------------------------------
def validate_tucker_rank(tensor_shape, rank="same"):
    """tensorly/tucker_tensor.py:344-447 (int and sequence ranks)."""
    if isinstance(rank, int):
        warnings.warn("Given only one int for 'rank'. Using this rank for all modes.")
        return tuple([rank] * len(tensor_shape))
    if rank == "same" or isinstance(rank, float):
        raise NotImplementedError("oracle restates int / sequence ranks only")
    return tuple(rank)


def tucker_to_tensor(tucker_tensor, skip_factor=None, transpose_factors=False, modes=None):
    """tensorly/tucker_tensor.py:50-75."""
    core, factors = tucker_tensor
    return multi_mode_dot(core, factors, skip=skip_factor,
                          transpose=transpose_factors, modes=modes)


def tucker_to_unfolded(tucker_tensor, mode=0, skip_factor=None, transpose_factors=False):
    """tensorly/tucker_tensor.py:105-131."""
    return unfold(tucker_to_tensor(tucker_tensor, skip_factor=skip_factor,
                                   transpose_factors=transpose_factors), mode)


def tucker_to_vec(tucker_tensor, skip_factor=None, transpose_factors=False):
    """tensorly/tucker_tensor.py:134-162."""
    return np.reshape(tucker_to_tensor(tucker_tensor, skip_factor=skip_factor,
                                       transpose_factors=transpose_factors), (-1,))


def initialize_tucker(tensor, rank, modes, random_state, init="svd", svd="truncated_svd",
                      non_negative=False, mask=None, svd_mask_repeats=5):
    """tensorly/decomposition/_tucker.py:25-102."""
    if isinstance(init, str) and init == "svd":
        factors = []
        for index, mode in enumerate(modes):
            mask_unfold = None if mask is None else unfold(mask, mode)
            U, _, _ = svd_interface(unfold(tensor, mode), n_eigenvecs=rank[index], method=svd,
                                    non_negative=non_negative, mask=mask_unfold,
                                    n_iter_mask_imputation=svd_mask_repeats,
                                    random_state=random_state)
            factors.append(U)
        core = multi_mode_dot(tensor, factors, modes=modes, transpose=True)
    elif isinstance(init, str) and init == "random":
        rng = check_random_state(random_state)
        core = (rng.random_sample([rank[i] for i in range(len(modes))]) + 0.01).astype(tensor.dtype)
        factors = [rng.random_sample((tensor.shape[mode], rank[index])).astype(tensor.dtype)
                   for index, mode in enumerate(modes)]
    else:
        core, factors = init
    if non_negative is True:
        factors = [np.abs(f) for f in factors]
        core = np.abs(core)
    return core, list(factors)


def non_negative_tucker(tensor, rank, n_iter_max=10, init="svd", tol=10e-5, random_state=None,
                        return_errors=False, normalize_factors=False):
    """tensorly/decomposition/_tucker.py:348-454 (multiplicative updates, not
    verbose), with the reference's explicit B."""
    rank = validate_tucker_rank(tensor.shape, rank=rank)
    epsilon = 10e-12
    nn_core, nn_factors = initialize_tucker(tensor, rank, range(tensor.ndim), init=init,
                                            random_state=random_state, non_negative=True)
    nn_factors = list(nn_factors)
    norm_tensor = norm(tensor)
    rec_errors = []
    for iteration in range(n_iter_max):
        for mode in range(tensor.ndim):
            B = tucker_to_tensor((nn_core, nn_factors), skip_factor=mode)
            B = np.transpose(unfold(B, mode))
            numerator = np.dot(unfold(tensor, mode), B)
            numerator = np.clip(numerator, a_min=epsilon, a_max=None)
            denominator = np.dot(nn_factors[mode], np.dot(np.transpose(B), B))
            denominator = np.clip(denominator, a_min=epsilon, a_max=None)
            nn_factors[mode] = nn_factors[mode] * (numerator / denominator)
        numerator = tucker_to_tensor((tensor, nn_factors), transpose_factors=True)
        numerator = np.clip(numerator, a_min=epsilon, a_max=None)
        for i, f in enumerate(nn_factors):
            if i:
                denominator = mode_dot(denominator, np.dot(np.transpose(f), f), i)
            else:
                denominator = mode_dot(nn_core, np.dot(np.transpose(f), f), i)
        denominator = np.clip(denominator, a_min=epsilon, a_max=None)
        nn_core = nn_core * (numerator / denominator)
        rec_error = norm(tensor - tucker_to_tensor((nn_core, nn_factors))) / norm_tensor
        rec_errors.append(rec_error)
        if iteration > 1 and abs(rec_errors[-2] - rec_errors[-1]) < tol:
            break
        if normalize_factors:
            nn_core, nn_factors = tucker_normalize((nn_core, nn_factors))
    if return_errors:
        return (nn_core, nn_factors), rec_errors
    return nn_core, nn_factors


def partial_tucker(tensor, rank, modes=None, n_iter_max=100, init="svd", tol=10e-5,
                   svd="truncated_svd", random_state=None, verbose=False, mask=None,
                   svd_mask_repeats=5):
    """tensorly/decomposition/_tucker.py:105-221 (HOOI); with a mask the
    missing entries are refilled from the model at each iteration
    (``:194-197``), and a masked 'svd' start refills inside svd_interface."""
    if modes is None:
        modes = list(range(tensor.ndim))
    if rank is None:
        rank = [tensor.shape[m] for m in modes]
    elif isinstance(rank, int):
        rank = tuple(rank for _ in modes)
    else:
        rank = tuple(rank)
    core, factors = initialize_tucker(tensor, rank, modes, init=init, svd=svd,
                                      random_state=random_state, mask=mask,
                                      svd_mask_repeats=svd_mask_repeats)
    rec_errors = []
    norm_tensor = norm(tensor)
    for iteration in range(n_iter_max):
        if mask is not None:
            tensor = tensor * mask + multi_mode_dot(core, factors, modes=modes,
                                                    transpose=False) * (1 - mask)
        for index, mode in enumerate(modes):
            core_approximation = multi_mode_dot(tensor, factors, modes=modes, skip=index,
                                                transpose=True)
            eigenvecs, _, _ = svd_interface(unfold(core_approximation, mode),
                                            n_eigenvecs=rank[index])
            factors[index] = eigenvecs
        core = multi_mode_dot(tensor, factors, modes=modes, transpose=True)
        rec_error = math.sqrt(abs(norm_tensor ** 2 - norm(core) ** 2)) / norm_tensor
        rec_errors.append(rec_error)
        if iteration > 1:
            if tol and abs(rec_errors[-2] - rec_errors[-1]) < tol:
                break
    return (core, factors), rec_errors


def tucker(tensor, rank, fixed_factors=None, n_iter_max=100, init="svd",
           return_errors=False, svd="truncated_svd", tol=10e-5, random_state=None,
           mask=None, verbose=False):
    """tensorly/decomposition/_tucker.py:224-345 (all modes; fixed_factors path
    ``:288-322`` included)."""
    if fixed_factors:
        core, factors = init
        fixed_factors = sorted(fixed_factors)
        modes_fixed, factors_fixed = zip(*[(i, f) for i, f in enumerate(factors)
                                           if i in fixed_factors])
        core = multi_mode_dot(core, factors_fixed, modes=modes_fixed)
        modes, factors = zip(*[(i, f) for i, f in enumerate(factors) if i not in fixed_factors])
        (core, new_factors), rec_errors = partial_tucker(
            tensor, rank=rank, modes=modes, n_iter_max=n_iter_max, init=(core, list(factors)),
            svd=svd, tol=tol, random_state=random_state, mask=mask)
        factors = list(new_factors)
        for i, e in enumerate(fixed_factors):
            factors.insert(e, factors_fixed[i])
        core = multi_mode_dot(core, factors_fixed, modes=modes_fixed, transpose=True)
        return (core, factors)
    modes = list(range(tensor.ndim))
    rank = validate_tucker_rank(tensor.shape, rank=rank)
    (core, factors), rec_errors = partial_tucker(
        tensor, rank=rank, modes=modes, n_iter_max=n_iter_max, init=init, svd=svd, tol=tol,
        random_state=random_state, mask=mask)
    if return_errors:
        return (core, factors), rec_errors
    return (core, factors)
