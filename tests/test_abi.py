"""The C ABI library builds, loads without a GPU and exports every entry
point that include/tensorly_gb300.h declares (no compute calls here)."""

import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "tensorly_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(tlgb_[a-z0-9_]+)\s*\(", text))
    names.discard("tlgb_sweep_callback")
    return sorted(names)


@pytest.fixture(scope="module")
def library():
    from tensorly_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("tlgb_mttkrp", "tlgb_khatri_rao", "tlgb_mode_dot", "tlgb_cp_als",
              "tlgb_cp_als_workspace_size", "tlgb_last_error"):
        assert s in syms


def test_every_declared_symbol_is_exported(library):
    missing = [s for s in declared_symbols() if not hasattr(library, s)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header():
    from tensorly_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_header_has_no_torch_types():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for bad in ("torch", "at::", "Tensor", "c10", "cudaStream_t"):
        assert bad not in text


def test_version_and_error_string(library):
    library.tlgb_version.restype = ctypes.c_int
    assert library.tlgb_version() >= 100
    library.tlgb_last_error.restype = ctypes.c_char_p
    assert isinstance(library.tlgb_last_error(), bytes)


def test_argument_validation_without_gpu(library):
    """Host-side checks reject bad arguments before any CUDA call."""
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    nbytes = ctypes.c_size_t(0)
    shape = _lib.i64_array([4, 5, 6])
    assert lib.tlgb_mttkrp_workspace_size(_lib.TLGB_F32, 3, shape, 2, 3,
                                          ctypes.byref(nbytes)) == _lib.TLGB_EINVAL
    assert b"mode" in lib.tlgb_last_error()
    assert lib.tlgb_mttkrp_workspace_size(7, 3, shape, 2, 0, ctypes.byref(nbytes)) == _lib.TLGB_EINVAL
    assert lib.tlgb_mttkrp_workspace_size(_lib.TLGB_F64, 9, shape, 2, 0,
                                          ctypes.byref(nbytes)) == _lib.TLGB_EINVAL
    opts = _lib.CpAlsOptions()
    lib.tlgb_cp_als_default_options(ctypes.byref(opts))
    assert opts.n_iter_max == 100 and abs(opts.tol - 1e-8) < 1e-20 and opts.use_graph == 0
    opts.precision = _lib.TLGB_PREC_BF16
    rc = lib.tlgb_cp_als_workspace_size(_lib.TLGB_F64, 3, shape, 2, ctypes.byref(opts),
                                        ctypes.byref(nbytes))
    assert rc == _lib.TLGB_EUNSUPPORTED
    opts.precision = _lib.TLGB_PREC_NATIVE
    rc = lib.tlgb_cp_als_workspace_size(_lib.TLGB_F64, 3, shape, 500, ctypes.byref(opts),
                                        ctypes.byref(nbytes))
    assert rc == _lib.TLGB_EUNSUPPORTED


def test_new_entry_points_validate_without_gpu(library):
    """The reconstruction, randomised, constrained, non-negative Tucker and
    PARAFAC2 entry points reject bad arguments before any CUDA call."""
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    F32, F64, EINVAL = _lib.TLGB_F32, _lib.TLGB_F64, _lib.TLGB_EINVAL
    nbytes = ctypes.c_size_t(0)
    shape = _lib.i64_array([4, 5, 6])
    fake = ctypes.c_void_p(16)                      # never dereferenced on the host
    fptrs = (ctypes.c_void_p * 3)(16, 16, 16)
    assert lib.tlgb_cp_to_tensor_workspace_size(7, 3, shape, 2, ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_cp_to_tensor_workspace_size(F32, 9, shape, 2, ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_cp_residual_norm(F32, None, 3, shape, 2, fptrs, None, None, None, 0,
                                     None) == EINVAL
    assert lib.tlgb_cp_randomised_workspace_size(F32, 3, shape, 2, 0,
                                                 ctypes.byref(nbytes)) == EINVAL
    assert b"n_samples" in lib.tlgb_last_error()
    assert lib.tlgb_cp_randomised_workspace_size(F64, 3, shape, 500, 10,
                                                 ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_sample_khatri_rao(F32, 0, fptrs, shape, 2, 4, fake, fake, None) == EINVAL
    assert lib.tlgb_cp_constrained_workspace_size(F64, 3, shape, 500,
                                                  ctypes.byref(nbytes)) == EINVAL
    free = (ctypes.c_int * 3)(0, 1, 2)
    kinds = (ctypes.c_int * 3)(1, 13, 0)   # 13: no such constraint kind
    params = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    errs = (ctypes.c_double * 4)()
    n_err = ctypes.c_int(0)
    assert lib.tlgb_cp_constrained(F64, fake, 3, shape, fptrs, 2, free, 3, kinds, params, 4, 10,
                                   1e-8, 1e-6, 0, errs, ctypes.byref(n_err), None, 0,
                                   None) == EINVAL
    assert b"constraint kind" in lib.tlgb_last_error()
    free2 = (ctypes.c_int * 2)(0, 1)                # the last mode must be free
    kinds0 = (ctypes.c_int * 3)(0, 0, 0)
    assert lib.tlgb_cp_constrained(F64, fake, 3, shape, fptrs, 2, free2, 2, kinds0, params, 4,
                                   10, 1e-8, 1e-6, 0, errs, ctypes.byref(n_err), None, 0,
                                   None) == EINVAL
    assert lib.tlgb_proximal(F32, fake, 4, 9, 0.0, fake, None, 0, None) == EINVAL
    assert lib.tlgb_hals_nnls_workspace_size(F32, 10, 200, ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_fista_tucker_core_workspace_size(F32, 0, shape, ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_gemm(F64, -1, 2, 2, fake, 2, 1, fake, 2, 1, fake, None) == EINVAL
    assert lib.tlgb_mu_update(7, fake, fake, fake, 4, 1e-12, None) == EINVAL
    assert lib.tlgb_dot(F32, fake, fake, 4, fake, None, 0, None) == _lib.TLGB_EWORKSPACE
    assert lib.tlgb_qr_workspace_size(F64, 3, 5, ctypes.byref(nbytes)) == EINVAL
    assert lib.tlgb_lerp(F32, None, fake, 4, 0.5, fake, None) == EINVAL
    assert lib.tlgb_inv_sqrt(7, fake, 4, fake, None) == EINVAL
    assert lib.tlgb_unfold(F32, fake, 3, shape, 5, fake, None) == EINVAL
