"""Random CP initialisation with the reference's exact draw order.

tensorly/random/base.py:64-114 (random_cp) draws ``random_sample((s, rank))``
for every mode in order from NumPy's RandomState, in float64, then casts to
the tensor dtype; tensorly/backend/core.py:163-188 (check_random_state)
resolves the seed.  The draws stay on the host (they are the reference's
definition of the initial factors) and are copied to the GPU once.
"""

import numpy as np
import torch


def check_random_state(seed):
    """None -> NumPy's global RandomState, int -> RandomState(seed), RandomState
    -> itself, anything else ValueError.  As in the reference, a Python int
    (bool included) is a seed and a NumPy integer is not."""
    if seed is None:
        return np.random.mtrand._rand
    if isinstance(seed, int):
        return np.random.RandomState(seed)
    if isinstance(seed, np.random.RandomState):
        return seed
    raise ValueError("Seed should be None, int or np.random.RandomState")


def random_cp(shape, rank, random_state=None, dtype=torch.float32, device="cuda",
              normalise_factors=False):
    """Random CP tensor (weights, factors) on `device` (reference random_cp,
    ``full=False``, ``orthogonal=False``)."""
    from .cp_tensor import CPTensor, cp_normalize
    rns = check_random_state(random_state)
    factors = [torch.from_numpy(rns.random_sample((int(s), int(rank)))).to(device=device, dtype=dtype)
               for s in shape]
    weights = torch.ones(int(rank), dtype=dtype, device=device)
    cp = CPTensor((weights, factors))
    if normalise_factors:
        return cp_normalize(cp)
    return cp
