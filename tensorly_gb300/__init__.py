"""tensorly_gb300: TensorLy's CP-ALS / Tucker-HOOI hot path on GB300 (sm_103a).

Public API mirrors ``tensorly.decomposition`` and ``tensorly.tenalg``:

    parafac, CP, initialize_cp, tucker, partial_tucker, Tucker,
    non_negative_parafac, CP_NN, non_negative_parafac_hals, CP_NN_HALS
    khatri_rao, unfolding_dot_khatri_rao, mode_dot, multi_mode_dot
    CPTensor, TuckerTensor, cp_norm, cp_normalize, cp_to_tensor, tucker_to_tensor

All computation runs in ``libtensorly_gb300.so`` (CUDA, sm_103a) through its
C ABI (``include/tensorly_gb300.h``); tensors are PyTorch CUDA tensors.
``plugin.register()`` installs the primitives as a TensorLy tenalg backend.
"""

from ._lib import GB300Error, SingularMatrixError, build, lib
from .base import fold, tensor_to_vec, unfold, vec_to_tensor
from .cp_tensor import (CPTensor, TuckerTensor, cp_norm, cp_normalize, cp_to_tensor,
                        cp_to_unfolded, cp_to_vec, tucker_normalize, tucker_to_tensor,
                        tucker_to_unfolded, tucker_to_vec, validate_cp_rank,
                        validate_tucker_rank)
from .decomposition import (CP, CP_NN, CP_NN_HALS, ConstrainedCP, RandomizedCP, Tucker,
                            active_set_nnls, constrained_parafac, initialize_constrained_parafac, initialize_cp,
                            initialize_tucker, non_negative_parafac, non_negative_parafac_hals,
                            non_negative_tucker, non_negative_tucker_hals, hals_nnls,
                            parafac, parafac_batched, partial_tucker, proximal_operator,
                            randomised_parafac, sample_khatri_rao, tucker, validate_constraints)
from .svd import randomized_svd, svd_flip, svd_interface, truncated_svd
from .parafac2 import (Parafac2, Parafac2Tensor, parafac2, parafac2_to_slices,
                       parafac2_to_tensor, random_parafac2)
from .random import check_random_state, random_cp
from .tenalg import khatri_rao, kronecker, mode_dot, multi_mode_dot, unfolding_dot_khatri_rao

__version__ = "0.1.0"
