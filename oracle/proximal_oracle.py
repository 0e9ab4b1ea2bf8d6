"""NumPy restatement of the proximal operators (TEST INFRASTRUCTURE ONLY).

Follows tensorly/tenalg/proximal.py:270-701: the operators constrained_parafac
applies per factor matrix, including the column-wise ones the GPU path does
not provide yet (unimodality, simplex, normalized_sparsity, soft_sparsity,
smoothness, monotonicity, hard_sparsity), and svd_thresholding / procrustes.
Pinned by tests/golden/proximal_kats.pkl, the calls of the reference's own
tests (tensorly/tenalg/tests/test_proximal.py).  Only ``tests/`` import it.
"""

import numpy as np

from .tensorly_oracle import truncated_svd


def soft_thresholding(tensor, threshold):
    """:631-671."""
    return np.sign(tensor) * np.clip(np.abs(tensor) - threshold, a_min=0, a_max=None)


def l2_square_prox(tensor, regularizer):
    """:444-463."""
    return tensor / (1 + 2 * regularizer)


def l2_prox(tensor, regularizer):
    """:466-493: shrink the whole matrix towards 0 by ``regularizer`` in norm."""
    nrm = np.sqrt(np.sum(np.abs(tensor) ** 2))
    bigger = nrm if nrm > regularizer else regularizer
    return tensor - (tensor * regularizer / bigger)


def smoothness_prox(tensor, regularizer):
    """:270-289: solve (I (1 + 2 r) - r (sub + super diagonal)) x = tensor."""
    n = tensor.shape[0]
    m = (np.diag(2 * regularizer * np.ones(n) + 1)
         + np.diag(-regularizer * np.ones(n - 1), k=-1)
         + np.diag(-regularizer * np.ones(n - 1), k=1)).astype(tensor.dtype)
    return np.linalg.solve(m, tensor)


def monotonicity_prox(tensor, decreasing=False):
    """:292-356: per column, the running maxima of the trailing means of the
    cumulative sums, then a backward pass that removes decreases."""
    if tensor.ndim == 1:
        tensor = np.reshape(tensor, [tensor.shape[0], 1])
    elif tensor.ndim > 2:
        raise ValueError("Monotonicity prox doesn't support an input which has more than "
                         "2 dimensions.")
    mon = np.copy(tensor)
    if decreasing:
        mon = np.flip(mon, axis=0)
    row, column = mon.shape
    cum = np.cumsum(mon, axis=0)
    for j in range(column):
        assisted = np.zeros([row, row])
        for i in range(row):
            counts = (np.arange(row - i) + 1).astype(tensor.dtype)
            if i == 0:
                assisted[i, i:] = cum[i:, j] / counts
            else:
                assisted[i, i:] = (cum[i:, j] - cum[i - 1, j]) / counts
        mon[:, j] = np.max(assisted, axis=0)
        for i in reversed(range(row - 1)):
            if mon[i, j] > mon[i + 1, j]:
                mon[i, j] = mon[i + 1, j]
    if decreasing:
        mon = np.flip(mon, axis=0)
    return mon


def unimodality_prox(tensor):
    """:359-441: per column, the increasing fit up to the mode and the
    decreasing fit after it, the mode the index of least total deviation."""
    if tensor.ndim == 1:
        tensor = np.reshape(tensor, [tensor.shape[0], 1])
    elif tensor.ndim > 2:
        raise ValueError("Unimodality prox doesn't support an input which has more than "
                         "2 dimensions.")
    out = np.copy(tensor)
    inc = monotonicity_prox(tensor)
    dec = monotonicity_prox(tensor, decreasing=True)
    values = (tensor - dec >= 0) * (tensor - inc >= 0)
    sum_inc = np.where(values == 1, np.cumsum(np.abs(tensor - inc), axis=0), 0)
    sum_inc = np.where(values == 1, sum_inc - np.abs(tensor - inc), 0)
    fv = np.flip(values, axis=0)
    ft, fd = np.flip(tensor, axis=0), np.flip(dec, axis=0)
    sum_dec = np.where(fv == 1, np.cumsum(np.abs(ft - fd), axis=0), 0)
    sum_dec = np.where(fv == 1, sum_dec - np.abs(ft - fd), 0)
    total = sum_inc + np.flip(sum_dec, axis=0)
    difference = np.where(values == 1, total, np.max(total))
    min_indice = np.argmin(difference, axis=0)
    for i in range(len(min_indice)):
        k = int(min_indice[i])
        out[:k, i] = inc[:k, i]
        out[k + 1:, i] = dec[k + 1:, i]
    return out


def hard_thresholding(tensor, number_of_non_zero):
    """:602-628: keep the ``number_of_non_zero`` entries of largest magnitude
    (ranks from a double argsort, as the reference computes them)."""
    vec = np.copy(np.reshape(tensor, (-1,)))
    ranks = np.argsort(np.flip(np.argsort(np.abs(vec), axis=0), axis=0), axis=0)
    return np.reshape(np.where(ranks < number_of_non_zero, vec, 0), tensor.shape)


def normalized_sparsity_prox(tensor, threshold):
    """:496-526."""
    hard = hard_thresholding(tensor, threshold)
    return hard / np.sqrt(np.sum(np.abs(hard) ** 2))


def simplex_prox(tensor, parameter):
    """:558-599: per column, the projection onto {x >= 0, sum x = parameter}
    by the sorted cumulative-sum threshold."""
    if tensor.ndim > 1:
        row, col = tensor.shape
    else:
        row, col = tensor.shape[0], 1
        tensor = np.reshape(tensor, [row, col])
    srt = np.flip(np.sort(tensor, axis=0), axis=0)
    thr = (np.cumsum(srt, axis=0) - parameter) / np.cumsum(np.ones([row, 1]), axis=0)
    to_change = np.sum(np.where(srt > thr, 1, 0), axis=0) - 1
    difference = np.zeros(col)
    for i in range(col):
        difference[i] = thr[to_change[i], i]
    out = np.clip(tensor - difference, a_min=0, a_max=None)
    return out if col > 1 else np.reshape(out, (-1,))


def soft_sparsity_prox(tensor, threshold):
    """:529-555."""
    return simplex_prox(np.abs(tensor), threshold) * np.sign(tensor)


def svd_thresholding(matrix, threshold):
    """:674-692."""
    U, s, V = truncated_svd(matrix, n_eigenvecs=min(matrix.shape))
    return np.dot(U, np.reshape(soft_thresholding(s, threshold), (-1, 1)) * V)


def procrustes(matrix):
    """:695-701."""
    U, _, V = truncated_svd(matrix, n_eigenvecs=min(matrix.shape))
    return np.dot(U, V)
