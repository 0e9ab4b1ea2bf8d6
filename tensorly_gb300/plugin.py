"""TensorLy tenalg backend "gb300" (the reference's own plugin interface).

TensorLy dispatches its tensor-algebra primitives through
``tensorly.tenalg.TenalgBackendManager`` (tensorly/tenalg/__init__.py:15-92):
a backend is a subclass of ``TenalgBackend`` (tensorly/tenalg/base_tenalg.py:4-33)
created with ``backend_name=...``, which registers itself on class creation,
and whose methods are attached with ``register_method``.  ``register()``
builds that subclass with the GB300 implementations of the hot-path
primitives (``unfolding_dot_khatri_rao``, ``khatri_rao``, ``mode_dot``,
``multi_mode_dot``), takes the remaining primitives (kronecker, inner, outer,
...) from the reference's ``core`` backend unchanged, adds "gb300" to the
manager's known names and, by default, selects it.  Calls made through
``tensorly.tenalg`` (including the ones inside ``tensorly.decomposition``'s
``parafac`` and ``tucker``, which resolve the name per call) then run on the
GPU.  The functions take and return whatever the active TensorLy backend
uses: CUDA tensors stay on the device, NumPy arrays go to the GPU and back.
"""

from . import tenalg as _gb

BACKEND_NAME = "gb300"

# the names this package implements; every other name keeps the core version
HOT_PATH = {
    "unfolding_dot_khatri_rao": _gb.unfolding_dot_khatri_rao,
    "khatri_rao": _gb.khatri_rao,
    "mode_dot": _gb.mode_dot,
    "multi_mode_dot": _gb.multi_mode_dot,
}


def register(tenalg=None, activate=True):
    """Register (and by default select) the "gb300" tenalg backend.

    ``tenalg`` is the ``tensorly.tenalg`` module (imported when None).
    Returns the backend class.  Registering twice reuses the first class.
    """
    if tenalg is None:
        import tensorly.tenalg as tenalg
    base = tenalg.TenalgBackend
    manager = tenalg.TenalgBackendManager
    known = base._available_tenalg_backends
    cls = known.get(BACKEND_NAME)
    if cls is None:
        cls = type("GB300TenalgBackend", (base,), {}, backend_name=BACKEND_NAME)
        core = manager.load_backend("core")
        for name in manager._functions:
            if name not in HOT_PATH and hasattr(core, name):
                cls.register_method(name, getattr(core, name))
        for name, fn in HOT_PATH.items():
            cls.register_method(name, fn)
    if BACKEND_NAME not in manager.available_backend_names:
        manager.available_backend_names.append(BACKEND_NAME)
    if activate:
        tenalg.set_backend(BACKEND_NAME)
    return cls


def unregister(tenalg=None):
    """Select the "core" tenalg backend again (the class stays registered)."""
    if tenalg is None:
        import tensorly.tenalg as tenalg
    tenalg.set_backend("core")
