"""The tenalg plugin registration against a stand-in of TensorLy's backend
registry (the same class protocol as tensorly/tenalg/base_tenalg.py:4-33 and
tensorly/tenalg/__init__.py:15-92); runs without a GPU and without TensorLy."""

import types

import pytest


def _fake_tenalg():
    class TenalgBackend:
        _available_tenalg_backends = {}

        def __init_subclass__(cls, backend_name, **kwargs):
            super().__init_subclass__(**kwargs)
            cls._available_tenalg_backends[backend_name.lower()] = cls
            cls.backend_name = backend_name

        @classmethod
        def register_method(cls, name, func):
            setattr(cls, name, staticmethod(func))

    class Core(TenalgBackend, backend_name="core"):
        pass

    for name in ("mode_dot", "multi_mode_dot", "kronecker", "khatri_rao", "inner", "outer",
                 "batched_outer", "higher_order_moment", "_tt_matrix_to_tensor",
                 "unfolding_dot_khatri_rao", "tensordot"):
        Core.register_method(name, (lambda n: (lambda *a, **k: ("core", n)))(name))

    class Manager:
        _functions = ["mode_dot", "multi_mode_dot", "kronecker", "khatri_rao", "inner", "outer",
                      "batched_outer", "higher_order_moment", "_tt_matrix_to_tensor",
                      "unfolding_dot_khatri_rao", "tensordot"]
        available_backend_names = ["core", "einsum"]
        _loaded = {}
        current = "core"

        @classmethod
        def load_backend(cls, name):
            if name not in cls.available_backend_names:
                raise ValueError(name)
            return TenalgBackend._available_tenalg_backends[name]()

    mod = types.SimpleNamespace(TenalgBackend=TenalgBackend, TenalgBackendManager=Manager)

    def set_backend(name):
        if name not in Manager.available_backend_names:
            raise ValueError(name)
        Manager.current = name

    mod.set_backend = set_backend
    return mod


def test_register_builds_gb300_backend():
    from tensorly_gb300 import plugin, tenalg
    fake = _fake_tenalg()
    cls = plugin.register(fake)
    assert fake.TenalgBackend._available_tenalg_backends["gb300"] is cls
    assert "gb300" in fake.TenalgBackendManager.available_backend_names
    assert fake.TenalgBackendManager.current == "gb300"
    backend = cls()
    # the hot-path names are this package's functions ...
    assert backend.unfolding_dot_khatri_rao is tenalg.unfolding_dot_khatri_rao
    assert backend.khatri_rao is tenalg.khatri_rao
    assert backend.mode_dot is tenalg.mode_dot
    assert backend.multi_mode_dot is tenalg.multi_mode_dot
    # ... every other name keeps the core implementation
    assert backend.kronecker() == ("core", "kronecker")
    assert backend.tensordot() == ("core", "tensordot")
    for name in fake.TenalgBackendManager._functions:
        assert hasattr(backend, name)


def test_register_is_idempotent_and_unregister_restores_core():
    from tensorly_gb300 import plugin
    fake = _fake_tenalg()
    a = plugin.register(fake)
    b = plugin.register(fake, activate=False)
    assert a is b
    assert fake.TenalgBackendManager.available_backend_names.count("gb300") == 1
    plugin.unregister(fake)
    assert fake.TenalgBackendManager.current == "core"


def test_register_with_real_tensorly_if_installed():
    tl = _real_tensorly()
    from tensorly_gb300 import plugin
    cls = plugin.register(tl.tenalg, activate=False)
    assert tl.tenalg.TenalgBackend._available_tenalg_backends["gb300"] is cls


def _real_tensorly():
    """TensorLy itself, from an installed package or from the source tree
    named by TENSORLY_REFERENCE; skips when neither is there."""
    import os
    import sys
    ref = os.environ.get("TENSORLY_REFERENCE")
    if ref and os.path.isdir(os.path.join(ref, "tensorly")) and ref not in sys.path:
        sys.path.insert(0, ref)
    return pytest.importorskip("tensorly")


def test_real_tensorly_decompositions_dispatch_to_gb300():
    """With the real registry, tensorly.decomposition.parafac and tucker
    resolve their tenalg calls to the "gb300" backend.  Without a GPU the
    backend's hot-path entries are replaced by recording wrappers around the
    core functions, so what is checked is the dispatch, and that the
    decompositions still give the core backend's results through it."""
    tl = _real_tensorly()
    import numpy as np
    from tensorly.decomposition import parafac, tucker
    from tensorly_gb300 import plugin
    tl.set_backend("numpy")
    cls = plugin.register(tl.tenalg, activate=False)
    core = tl.tenalg.TenalgBackendManager.load_backend("core")
    calls = {}
    saved = {name: getattr(cls, name) for name in plugin.HOT_PATH}

    def recorder(name):
        fn = getattr(core, name)

        def wrapped(*args, **kwargs):
            calls[name] = calls.get(name, 0) + 1
            return fn(*args, **kwargs)
        return wrapped

    try:
        for name in plugin.HOT_PATH:
            cls.register_method(name, recorder(name))
        x = np.random.RandomState(0).rand(6, 5, 4)
        ref_cp = parafac(x, 3, n_iter_max=4, init="random", random_state=1, tol=0)
        ref_tk = tucker(x, [2, 2, 2], n_iter_max=3, init="random", random_state=1, tol=0)
        assert not calls
        tl.tenalg.set_backend("gb300")
        cp = parafac(x, 3, n_iter_max=4, init="random", random_state=1, tol=0)
        assert calls.get("unfolding_dot_khatri_rao", 0) == 4 * 3
        tk = tucker(x, [2, 2, 2], n_iter_max=3, init="random", random_state=1, tol=0)
        assert calls.get("multi_mode_dot", 0) > 0
        for a, b in zip(cp.factors, ref_cp.factors):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(tk.core, ref_tk.core)
    finally:
        for name, fn in saved.items():
            cls.register_method(name, fn)
        plugin.unregister(tl.tenalg)
