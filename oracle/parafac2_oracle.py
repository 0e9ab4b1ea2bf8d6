"""NumPy restatement of PARAFAC2 (TEST INFRASTRUCTURE ONLY).

Follows tensorly/decomposition/_parafac2.py:21-707, with non-negative modes
(nn_modes, through non_negative_parafac_hals) and masks (missing entries
imputed, :21-66), with the reference's line search
(_BroThesisLineSearch, :183-318), projections (:158-171), projected slices
(:174-178) and error expansion (:321-396), and the random start of
tensorly/random/base.py:18-61 (QR of uniform draws, then random_cp).  Only
``tests/`` import it; it is pinned by the reference runs in tests/golden.
"""

import numpy as np

from . import tensorly_oracle as tlo


def random_parafac2(shapes, rank, random_state=None, dtype=np.float64):
    """tensorly/random/base.py:18-61 (full=False, not normalised)."""
    rns = tlo.check_random_state(random_state)
    if not all(shape[1] == shapes[0][1] for shape in shapes):
        raise ValueError("All matrices must have equal number of columns.")
    projections = [np.linalg.qr(rns.random_sample((shape[0], rank)).astype(dtype))[0]
                   for shape in shapes]
    weights, factors = tlo.random_cp([len(shapes), rank, shapes[0][1]], rank,
                                     random_state=rns, dtype=dtype)
    return weights, list(factors), projections


def compute_projections(tensor_slices, factors, svd="truncated_svd"):
    """tensorly/decomposition/_parafac2.py:158-171."""
    n_eig = factors[0].shape[1]
    out = []
    for A, tensor_slice in zip(factors[0], tensor_slices):
        lhs = np.dot(factors[1], np.transpose(A * factors[2]))
        rhs = np.transpose(tensor_slice)
        U, _, Vh = tlo.svd_interface(np.dot(lhs, rhs), n_eigenvecs=n_eig, method=svd,
                                     flip_sign=False)
        out.append(np.transpose(np.dot(U, Vh)))
    return out


def project_tensor_slices(tensor_slices, projections):
    """tensorly/decomposition/_parafac2.py:174-178."""
    return np.stack([np.dot(np.transpose(p), t) for t, p in zip(tensor_slices, projections)])


def initialize_decomposition(tensor_slices, rank, init="random", svd="truncated_svd",
                             random_state=None):
    """tensorly/decomposition/_parafac2.py:69-155 (random / svd / tuple)."""
    shapes = [m.shape for m in tensor_slices]
    concat_shape = sum(shape[0] for shape in shapes)
    dtype = tensor_slices[0].dtype
    if init == "random":
        return random_parafac2(shapes, rank, random_state=random_state, dtype=dtype)
    if init == "svd":
        if shapes[0][1] < rank:
            raise ValueError("Cannot perform SVD init if rank is greater than the number of "
                             "columns in each tensor slice")
        A = np.ones((len(tensor_slices), rank), dtype=dtype)
        if concat_shape > shapes[0][1]:
            unfolded_mode_2 = np.transpose(tensor_slices[0]) @ tensor_slices[0]
            for s in tensor_slices[1:]:
                unfolded_mode_2 = unfolded_mode_2 + np.matmul(np.transpose(s), s)
        else:
            unfolded_mode_2 = np.transpose(np.concatenate(list(tensor_slices), axis=0))
        C = tlo.svd_interface(unfolded_mode_2, n_eigenvecs=rank, method=svd)[0]
        B = np.eye(rank, dtype=dtype)
        projections = compute_projections(tensor_slices, (A, B, C), svd)
        return None, [A, B, C], projections
    weights, factors, projections = init
    return weights, list(factors), list(projections)


def parafac2_to_slices(decomposition):
    """tensorly/parafac2_tensor.py:310-372: slice i = (P_i B) (A_i w) C^T."""
    weights, (A, B, C), projections = decomposition
    out = []
    for i, p in enumerate(projections):
        a = A[i] if weights is None else A[i] * weights
        out.append(np.dot(np.dot(p, B) * a, np.transpose(C)))
    return out


def update_imputed(tensor_slices, mask, decomposition, method):
    """tensorly/decomposition/_parafac2.py:21-66: the missing entries become
    the slice's observed mean ('mode-2') or the model's value ('factors')."""
    if method == "mode-2":
        out = []
        for s, m in zip(tensor_slices, mask):
            mean = np.sum(s * m) / np.sum(m)
            out.append(np.where(m == 0, mean, s))
        return out
    rec = parafac2_to_slices(decomposition)
    return [np.where(m == 0, r, s) for s, r, m in zip(tensor_slices, rec, mask)]


def reconstruction_error(tensor_slices, decomposition, norm_matrices=None,
                         projected_tensor=None, mask=None):
    """tensorly/decomposition/_parafac2.py:321-396."""
    if mask is not None:
        rec = parafac2_to_slices(decomposition)
        total = 0.0
        for s, r, m in zip(tensor_slices, rec, mask):
            total += tlo.norm(m * s - m * r) ** 2
        return np.sqrt(total)
    if norm_matrices is None:
        norm_X_sq = sum(tlo.norm(t) ** 2 for t in tensor_slices)
    else:
        norm_X_sq = norm_matrices ** 2
    weights, (A, B, C), projections = decomposition
    if weights is not None:
        A = A * weights
    norm_cmf_sq = 0
    inner_product = 0
    CtC = np.dot(np.transpose(C), C)
    for i, t_slice in enumerate(tensor_slices):
        B_i = (projections[i] @ B) * A[i]
        if projected_tensor is None:
            tmp = np.dot(np.transpose(B_i), t_slice)
        else:
            tmp = np.reshape(A[i], (-1, 1)) * np.transpose(B) @ projected_tensor[i]
        inner_product += np.trace(np.dot(tmp, C))
        norm_cmf_sq += np.sum((np.transpose(B_i) @ B_i) * CtC)
    return np.sqrt(norm_X_sq - 2 * inner_product + norm_cmf_sq)


class LineSearch:
    """tensorly/decomposition/_parafac2.py:183-318 (_BroThesisLineSearch), clipping
    the non-negative modes 0 and 2 of the extrapolated step."""

    def __init__(self, norm_tensor, svd, nn_modes=None, mask=None, acc_pow=2.0, max_fail=4):
        self.norm_tensor = norm_tensor
        self.svd = svd
        self.nn_modes = nn_modes
        self.mask = mask
        self.acc_pow = acc_pow
        self.max_fail = max_fail
        self.acc_fail = 0

    def line_step(self, iteration, tensor_slices, factors_last, weights, factors, projections,
                  rec_error):
        jump = iteration ** (1.0 / self.acc_pow)
        factors_ls = [factors_last[ii] + (factors[ii] - factors_last[ii]) * jump
                      for ii, _ in enumerate(factors)]
        if self.nn_modes:
            if 0 in self.nn_modes:
                factors_ls[0] = np.clip(factors_ls[0], 0, None)
            if 2 in self.nn_modes:
                factors_ls[2] = np.clip(factors_ls[2], 0, None)
        projections_ls = compute_projections(tensor_slices, factors_ls, self.svd)
        ls_rec_error = reconstruction_error(tensor_slices, (weights, factors_ls, projections_ls),
                                            norm_matrices=self.norm_tensor, mask=self.mask)
        ls_rec_error /= self.norm_tensor
        if ls_rec_error < rec_error:
            self.acc_fail = 0
            return factors_ls, projections_ls, ls_rec_error
        self.acc_fail += 1
        if self.acc_fail == self.max_fail:
            self.acc_pow += 1.0
            self.acc_fail = 0
        return factors, projections, rec_error


def parafac2(tensor_slices, rank, n_iter_max=2000, init="random", svd="truncated_svd",
             normalize_factors=False, tol=1.0e-8, nn_modes=None, random_state=None,
             return_errors=False, n_iter_parafac=5, linesearch=True, mask=None):
    """tensorly/decomposition/_parafac2.py:399-707."""
    weights, factors, projections = initialize_decomposition(tensor_slices, rank, init=init,
                                                             svd=svd, random_state=random_state)
    factors = list(factors)
    if mask is not None:
        if init in ("random", "svd"):
            tensor_slices = update_imputed(list(tensor_slices), mask, None, "mode-2")
        else:
            tensor_slices = update_imputed(tensor_slices, mask,
                                           (weights, factors, projections), "factors")
    rec_errors = []
    if mask is not None:
        norm_tensor = np.sqrt(sum(tlo.norm(t * m) ** 2 for t, m in zip(tensor_slices, mask)))
    else:
        norm_tensor = np.sqrt(sum(tlo.norm(t) ** 2 for t in tensor_slices))
    ls = LineSearch(norm_tensor, svd, nn_modes=nn_modes, mask=mask) if linesearch else None
    if weights is None:
        weights = np.ones(rank, dtype=tensor_slices[0].dtype)
    for iteration in range(n_iter_max):
        factors[1] = factors[1] * np.reshape(weights, (1, -1))
        weights = np.ones(weights.shape, dtype=tensor_slices[0].dtype)
        if ls is not None and iteration % 2 == 0 and iteration > 5:
            line_iter = True
            factors_last = [np.copy(f) for f in factors]
        else:
            line_iter = False
        projections = compute_projections(tensor_slices, factors, svd)
        projected_tensor = project_tensor_slices(tensor_slices, projections)
        if nn_modes is None:
            (_, factors) = tlo.parafac(projected_tensor, rank, n_iter_max=n_iter_parafac,
                                       init=(weights, factors), svd=svd, normalize_factors=False,
                                       random_state=random_state, tol=1e-100)
        else:
            (_, factors) = tlo.non_negative_parafac_hals(
                projected_tensor, rank, n_iter_max=n_iter_parafac, init=(weights, factors),
                svd=svd, nn_modes=nn_modes, tol=1e-100)
        factors = list(factors)
        if line_iter:
            factors, projections, rec_errors[-1] = ls.line_step(
                iteration, tensor_slices, factors_last, weights, factors, projections,
                rec_errors[-1])
        if mask is not None:
            tensor_slices = update_imputed(tensor_slices, mask,
                                           (weights, factors, projections), "factors")
        if normalize_factors:
            weights, factors = tlo.cp_normalize((weights, factors))
            factors = list(factors)
        if tol and not line_iter:
            rec_error = reconstruction_error(tensor_slices, (weights, factors, projections),
                                             norm_tensor, projected_tensor, mask)
            rec_errors.append(rec_error / norm_tensor)
        if tol:
            if iteration >= 1:
                if abs(rec_errors[-2] - rec_errors[-1]) < tol:
                    break
    out = (weights, factors, projections)
    if return_errors:
        return out, rec_errors
    return out
