"""ctypes binding of libtensorly_gb300.so (the C ABI declared in include/tensorly_gb300.h).

The library is required: every public function of this package calls into
it, and there is no CPU fallback.  ``lib()`` raises if the shared object is
missing or fails to load; ``build()`` compiles it with nvcc.
"""

import ctypes
import os
import threading

from . import _build

TLGB_OK = 0
TLGB_EINVAL = 1
TLGB_ECUDA = 2
TLGB_ESINGULAR = 3
TLGB_EUNSUPPORTED = 4
TLGB_ETIMEOUT = 5
TLGB_EWORKSPACE = 6

TLGB_F32 = 0
TLGB_F64 = 1
TLGB_BF16 = 2

TLGB_PREC_NATIVE = 0
TLGB_PREC_BF16 = 1

_c_i64p = ctypes.POINTER(ctypes.c_int64)
_c_vpp = ctypes.POINTER(ctypes.c_void_p)

SWEEP_CALLBACK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double)


class CpAlsOptions(ctypes.Structure):
    """Mirror of ``tlgb_cp_als_options``."""
    _fields_ = [
        ("n_iter_max", ctypes.c_int),
        ("tol", ctypes.c_double),
        ("l2_reg", ctypes.c_double),
        ("cvg_criterion", ctypes.c_int),
        ("normalize_factors", ctypes.c_int),
        ("fixed_modes", ctypes.c_uint32),
        ("precision", ctypes.c_int),
        ("refine_sweeps", ctypes.c_int),
        ("check_every", ctypes.c_int),
        ("use_graph", ctypes.c_int),
        ("callback", SWEEP_CALLBACK),
        ("callback_user", ctypes.c_void_p),
        ("mttkrp_ms", ctypes.POINTER(ctypes.c_double)),
    ]


class TuckerOptions(ctypes.Structure):
    """Mirror of ``tlgb_tucker_options``."""
    _fields_ = [
        ("n_iter_max", ctypes.c_int),
        ("tol", ctypes.c_double),
        ("init_svd", ctypes.c_int),
    ]


class BatchItem(ctypes.Structure):
    """Mirror of ``tlgb_batch_item``."""
    _fields_ = [
        ("X", ctypes.c_void_p),
        ("factors", ctypes.c_void_p * 3),
        ("dims", ctypes.c_int64 * 3),
        ("rank", ctypes.c_int64),
    ]


CP_ALS_SWEEP_KINDS = 4
SWEEP_KIND_NAMES = ("native", "bf16", "f32_split", "closing")


# (name, restype, argtypes) for every entry point of include/tensorly_gb300.h
SIGNATURES = [
    ("tlgb_version", ctypes.c_int, []),
    ("tlgb_last_error", ctypes.c_char_p, []),
    ("tlgb_khatri_rao", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_vpp, _c_i64p, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_mttkrp_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.c_int,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_mttkrp", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_void_p,
      ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("tlgb_mttkrp_noalloc", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_void_p,
      ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_mttkrp_bf16_workspace_size", ctypes.c_int,
     [ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_mttkrp_bf16", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, _c_vpp, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_set_tuning", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    ("tlgb_workspace_status", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    ("tlgb_mode_dot", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_sym_eig_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_sym_eig", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_gram_unfolding_workspace_size", ctypes.c_int,
     [ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_gram_unfolding", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_int,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_svd_unfolding_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_int64,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_svd_unfolding", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("tlgb_tucker_default_options", None, [ctypes.POINTER(TuckerOptions)]),
    ("tlgb_tucker_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _c_i64p,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_tucker_hooi", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int,
      ctypes.POINTER(ctypes.c_int), _c_i64p, _c_vpp, ctypes.c_void_p,
      ctypes.POINTER(TuckerOptions), ctypes.POINTER(ctypes.c_double),
      ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_als_batched_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_als_batched", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_nn_mu_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.c_int,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_nn_mu", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_int64,
      ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_nn_hals", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_void_p,
      ctypes.c_int64, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_uint, ctypes.c_int,
      ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
      ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_sum", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_nndsvd_columns", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_ws_omega", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_ws_generate", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_ws_sketch", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_void_p]),
    ("tlgb_ws_gemm", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_ws_colsum", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_void_p]),
    ("tlgb_ws_cp_loss", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_ws_sketch_skip", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_ws_lift", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
      ctypes.c_void_p]),
    ("tlgb_ws_adam", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int,
      ctypes.c_void_p]),
    ("tlgb_ws_svd_init_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_ws_svd_init", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("tlgb_cp_als_default_options", None, [ctypes.POINTER(CpAlsOptions)]),
    ("tlgb_cp_als_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.POINTER(CpAlsOptions),
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_als", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp,
      ctypes.c_void_p, ctypes.POINTER(CpAlsOptions), ctypes.POINTER(ctypes.c_double),
      ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_normalize", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp, ctypes.c_void_p,
      ctypes.c_void_p]),
    ("tlgb_cp_norm_workspace_size", ctypes.c_int,
     [ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_norm", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_to_tensor_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_to_tensor", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_residual_norm", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_randomised_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.c_int64,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_randomised_iteration", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp,
      ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_sample_khatri_rao", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_vpp, _c_i64p, ctypes.c_int64, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_cp_constrained_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_cp_constrained", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_int64,
      ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
      ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
      ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_proximal_workspace_bytes", ctypes.c_size_t, []),
    ("tlgb_proximal", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_proximal_matrix_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
      ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_proximal_matrix", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
      ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_gemm", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_mu_update", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_double, ctypes.c_void_p]),
    ("tlgb_dot_workspace_bytes", ctypes.c_size_t, []),
    ("tlgb_dot", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_hals_nnls_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_hals_nnls", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_fista_tucker_core_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_fista_tucker_core", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, _c_vpp, ctypes.c_void_p,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_inv_sqrt", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_cp_randomised_launch", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int64, _c_vpp,
      ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_cp_randomised_finish", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_size_t, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    ("tlgb_ws_gemm_tc_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_ws_gemm_tc", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("tlgb_sparse_residual_workspace_bytes", ctypes.c_size_t, []),
    ("tlgb_sparse_residual", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_kronecker", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_vpp, _c_i64p, _c_i64p, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_active_set_nnls", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_tucker_normalize_workspace_size", ctypes.c_int,
     [ctypes.c_int, _c_i64p, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_tucker_normalize", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int, _c_i64p, _c_i64p, _c_vpp, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_mask_where", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
      ctypes.c_int64, ctypes.c_void_p]),
    ("tlgb_masked_sq_diff", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_clip_min", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p]),
    ("tlgb_mask_impute_workspace_bytes", ctypes.c_size_t, []),
    ("tlgb_mask_impute", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_lerp", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("tlgb_qr_workspace_size", ctypes.c_int,
     [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    ("tlgb_qr", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("tlgb_unfold", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_void_p,
      ctypes.c_void_p]),
    ("tlgb_fold", ctypes.c_int,
     [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _c_i64p, ctypes.c_int, ctypes.c_void_p,
      ctypes.c_void_p]),
]

_lock = threading.Lock()
_lib = None


class GB300Error(RuntimeError):
    """Error status returned by the CUDA library."""

    def __init__(self, code, message):
        super().__init__(f"tensorly_gb300 error {code}: {message}")
        self.code = code


class SingularMatrixError(GB300Error):
    """The normal equations of an ALS step are exactly singular."""


def library_path():
    return _build.LIB_PATH


def build(verbose=False):
    """Compile the CUDA library (sm_103a) and load it."""
    global _lib
    with _lock:
        _build.build(verbose=verbose)
        _lib = None
    return lib()


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"{path} is missing: build it with tensorly_gb300.build() (nvcc, sm_103a). "
                    "There is no CPU fallback.")
            handle = ctypes.CDLL(path)
            for name, res, args in SIGNATURES:
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(rc):
    """Raise the matching exception for a non-zero status."""
    if rc == TLGB_OK:
        return
    msg = lib().tlgb_last_error().decode(errors="replace")
    if rc == TLGB_ESINGULAR:
        raise SingularMatrixError(rc, msg)
    if rc == TLGB_EUNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == TLGB_EINVAL:
        raise ValueError(msg)
    raise GB300Error(rc, msg)


def i64_array(values):
    values = [int(v) for v in values]
    return (ctypes.c_int64 * max(1, len(values)))(*values)


def ptr_array(ptrs):
    return (ctypes.c_void_p * max(1, len(ptrs)))(*[ctypes.c_void_p(p) if p else None for p in ptrs])
