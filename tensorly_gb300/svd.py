"""Partial SVD of unfoldings (tensorly/tenalg/svd.py:366-447, truncated_svd + svd_flip)."""


def svd_interface_unfolding(tensor, mode, n_eigenvecs, method="truncated_svd", non_negative=False):
    raise NotImplementedError("SVD initialisation is not built yet")
