"""Generate the golden fixtures of the CP-ALS / Tucker path by running TensorLy.

Run where the reference source tree is available (it is pure Python):

    TENSORLY_REFERENCE=<path of the TensorLy source tree> python tests/golden/make_golden.py

The path comes from the environment only; the script stops with a message
when it is unset.

Outputs (committed, small, platform independent):

* ``tenalg_kats.pkl``: every call of khatri_rao / mode_dot / multi_mode_dot /
  unfolding_dot_khatri_rao made by the reference's own unit tests
  (tensorly/tenalg/tests/test_khatri_rao.py, test_n_mode_product.py,
  test_unfolding_dot_khatri_rao.py), recorded with its inputs, its output or
  the exception it raised.  The tests run unmodified against the NumPy
  backend with ``np.random.seed(0)``; the recorders wrap the functions the
  test modules call and the ``assert_*`` helpers they use (which additionally
  records the known answers the tests compare against).
* ``reconstruction_kats.pkl``: the same for cp_to_tensor / cp_to_unfolded /
  cp_to_vec / tucker_to_tensor / tucker_to_unfolded / tucker_to_vec, recorded
  from their tests in tensorly/tests/test_cp_tensor.py and
  test_tucker_tensor.py (CP and Tucker arguments stored as plain tuples).
* ``proximal_kats.pkl``: the same for the proximal operators called by
  tensorly/tenalg/tests/test_proximal.py.
* ``reference_runs.pkl``: reference ``parafac`` / ``non_negative_parafac`` /
  ``tucker`` / ``svd_interface``
  outputs on seeded inputs (the tensors are regenerated from their seeds by
  ``tensorly_gb300.workloads`` or by the case's own RandomState; each record
  stores a checksum of the input so a regeneration mismatch is caught).

Versions of numpy/scipy/tensorly used are stored in both files.
"""

import copy
import importlib
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("TENSORLY_REFERENCE")


def _versions():
    import scipy
    import tensorly
    return {"numpy": np.__version__, "scipy": scipy.__version__,
            "tensorly": getattr(tensorly, "__version__", "?")}


def _np(x):
    return np.array(x, copy=True) if isinstance(x, np.ndarray) else copy.deepcopy(x)


def record_kats():
    import tensorly as tl
    tl.set_backend("numpy")
    records = []

    def wrap(name, fn):
        def recorder(*args, **kwargs):
            rec = {"fn": name, "args": _np(list(args)), "kwargs": _np(dict(kwargs))}
            try:
                out = fn(*args, **kwargs)
            except Exception as e:  # the reference's expected failures
                rec["raises"] = type(e).__name__
                records.append(rec)
                raise
            rec["result"] = _np(out)
            records.append(rec)
            return out
        return recorder

    def wrap_assert(name, fn):
        def recorder(*args, **kwargs):
            records.append({"fn": name, "args": _np(list(args)), "kwargs": _np(dict(kwargs))})
            return fn(*args, **kwargs)
        return recorder

    mods = ["tensorly.tenalg.tests.test_khatri_rao",
            "tensorly.tenalg.tests.test_n_mode_product",
            "tensorly.tenalg.tests.test_unfolding_dot_khatri_rao"]
    for mname in mods:
        mod = importlib.import_module(mname)
        for fname in ("khatri_rao", "mode_dot", "multi_mode_dot", "unfolding_dot_khatri_rao"):
            if hasattr(mod, fname):
                setattr(mod, fname, wrap(fname, getattr(mod, fname)))
        for aname in ("assert_array_equal", "assert_array_almost_equal"):
            if hasattr(mod, aname):
                setattr(mod, aname, wrap_assert(aname, getattr(mod, aname)))
        for tname in sorted(n for n in dir(mod) if n.startswith("test_")):
            np.random.seed(0)
            records.append({"fn": "__test__", "name": f"{mname}.{tname}"})
            getattr(mod, tname)()
    return records


def _plain(x):
    """CPTensor / TuckerTensor arguments as plain (weights|core, [factors]) tuples,
    so the fixture loads without TensorLy."""
    if hasattr(x, "factors") and hasattr(x, "weights"):
        return (_np(x.weights), [_np(f) for f in x.factors])
    if hasattr(x, "factors") and hasattr(x, "core"):
        return (_np(x.core), [_np(f) for f in x.factors])
    if isinstance(x, tuple):
        return tuple(_plain(v) for v in x)
    if isinstance(x, list):
        return [_plain(v) for v in x]
    return _np(x)


def record_reconstruction():
    """Calls of cp_to_tensor / cp_to_unfolded / cp_to_vec / tucker_to_tensor /
    tucker_to_unfolded / tucker_to_vec (and the assertions with their known
    answers) made by the reference's tests of them
    (tensorly/tests/test_cp_tensor.py, tensorly/tests/test_tucker_tensor.py)."""
    import tensorly as tl
    tl.set_backend("numpy")
    records = []

    def wrap(name, fn):
        def recorder(*args, **kwargs):
            rec = {"fn": name, "args": _plain(list(args)), "kwargs": _plain(dict(kwargs))}
            out = fn(*args, **kwargs)
            rec["result"] = _np(out)
            records.append(rec)
            return out
        return recorder

    def wrap_assert(name, fn):
        def recorder(*args, **kwargs):
            records.append({"fn": name, "args": _plain(list(args)), "kwargs": _np(dict(kwargs))})
            return fn(*args, **kwargs)
        return recorder

    plan = {"tensorly.tests.test_cp_tensor":
            (("cp_to_tensor", "cp_to_unfolded", "cp_to_vec"),
             ("test_cp_to_tensor", "test_cp_to_tensor_with_weights", "test_cp_to_unfolded",
              "test_cp_to_vec")),
            "tensorly.tests.test_tucker_tensor":
            (("tucker_to_tensor", "tucker_to_unfolded", "tucker_to_vec"),
             ("test_tucker_to_tensor", "test_tucker_to_tensor_with_partial_modes",
              "test_tucker_to_unfolded", "test_tucker_to_vec"))}
    for mname, (fns, tests) in plan.items():
        mod = importlib.import_module(mname)
        for fname in fns:
            setattr(mod, fname, wrap(fname, getattr(mod, fname)))
        for aname in ("assert_array_equal", "assert_array_almost_equal"):
            if hasattr(mod, aname):
                setattr(mod, aname, wrap_assert(aname, getattr(mod, aname)))
        for tname in tests:
            np.random.seed(0)
            records.append({"fn": "__test__", "name": f"{mname}.{tname}"})
            getattr(mod, tname)()
    return records


def record_proximal():
    """Every proximal-operator call of the reference's tests
    (tensorly/tenalg/tests/test_proximal.py), with its output, and the
    assertions with their known answers."""
    import tensorly as tl
    tl.set_backend("numpy")
    records = []
    names = ("svd_thresholding", "smoothness_prox", "soft_thresholding", "procrustes",
             "hard_thresholding", "soft_sparsity_prox", "simplex_prox",
             "normalized_sparsity_prox", "monotonicity_prox", "unimodality_prox", "l2_prox",
             "l2_square_prox")

    def wrap(name, fn):
        def recorder(*args, **kwargs):
            rec = {"fn": name, "args": _np(list(args)), "kwargs": _np(dict(kwargs))}
            out = fn(*args, **kwargs)
            rec["result"] = _np(out)
            records.append(rec)
            return out
        return recorder

    def wrap_assert(name, fn):
        def recorder(*args, **kwargs):
            records.append({"fn": name, "args": _np(list(args)), "kwargs": _np(dict(kwargs))})
            return fn(*args, **kwargs)
        return recorder

    mod = importlib.import_module("tensorly.tenalg.tests.test_proximal")
    for fname in names:
        setattr(mod, fname, wrap(fname, getattr(mod, fname)))
    for aname in ("assert_array_equal", "assert_array_almost_equal"):
        if hasattr(mod, aname):
            setattr(mod, aname, wrap_assert(aname, getattr(mod, aname)))
    for tname in sorted(n for n in dir(mod) if n.startswith("test_")):
        np.random.seed(0)
        records.append({"fn": "__test__", "name": f"tensorly.tenalg.tests.test_proximal.{tname}"})
        getattr(mod, tname)()
    return records


def record_host_validators():
    """The reference's host-side helpers on a grid of arguments
    (tensorly/cp_tensor.py:240-275 validate_cp_rank,
    tensorly/tucker_tensor.py:344-447 validate_tucker_rank,
    tensorly/backend/core.py:163-188 check_random_state): the value, or the
    exception type, and the warning category raised."""
    import warnings
    import tensorly as tl
    from tensorly.cp_tensor import validate_cp_rank
    from tensorly.tucker_tensor import validate_tucker_rank
    records = []

    def call(fn, name, *args, **kwargs):
        rec = {"fn": name, "args": args, "kwargs": kwargs}
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            try:
                out = fn(*args, **kwargs)
                rec["out"] = [int(v) for v in out] if isinstance(out, list) else out
                rec["type"] = type(out).__name__
            except Exception as e:      # noqa: BLE001 (the exception type is the record)
                rec["raises"] = type(e).__name__
        rec["warns"] = sorted({type(x.message).__name__ for x in w})
        records.append(rec)

    shapes = [(3, 4, 5), (10, 10, 10), (7, 2, 9, 4), (100, 3), (30, 5, 12)]
    for shape in shapes:
        for rank in ("same", 0.5, 0.25, 1.7, 4):
            for rounding in ("round", "floor", "ceil"):
                call(validate_cp_rank, "validate_cp_rank", shape, rank=rank, rounding=rounding)
        call(validate_cp_rank, "validate_cp_rank", shape, rank=2, rounding="bad")
        for rank in ("same", 0.5, 0.1, 2.0, 3, [2] * len(shape)):
            for rounding in ("round", "floor", "ceil"):
                call(validate_tucker_rank, "validate_tucker_rank", shape, rank=rank,
                     rounding=rounding)
            for fixed in ([0], [1, len(shape) - 1]):
                call(validate_tucker_rank, "validate_tucker_rank", shape, rank=rank,
                     fixed_modes=fixed)
        call(validate_tucker_rank, "validate_tucker_rank", shape, rank=0.5, rounding="bad")
    crs = tl.check_random_state
    for seed in (0, 5, 123456, True):
        rec = {"fn": "check_random_state", "args": (seed,), "kwargs": {},
               "out": crs(seed).random_sample(4), "warns": []}
        records.append(rec)
    for seed in (np.int64(5), 1.5, "seed"):
        call(crs, "check_random_state", seed)
    return records


def reference_runs():
    import tensorly as tl
    from tensorly.decomposition import parafac, tucker
    from tensorly.decomposition._cp import initialize_cp
    from tensorly.tenalg.svd import svd_interface
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from tensorly_gb300 import workloads
    from golden_inputs import slice_masks
    tl.set_backend("numpy")
    runs = []

    def cs(x):
        x = np.asarray(x, dtype=np.float64)
        return [float(x.sum()), float(np.linalg.norm(x))]

    # dense 64^3 f64 rank-8 parity case (init 'random', seed 0, tol 1e-8)
    x, _ = workloads.dense_cp_small()
    init = initialize_cp(x, 8, init="random", random_state=0)
    cp, errs = parafac(x, 8, init="random", random_state=0, n_iter_max=100, tol=1e-8,
                       return_errors=True)
    runs.append({"case": "dense_cp_small", "gen": {"fn": "dense_cp_small"}, "checksum": cs(x),
                 "kwargs": {"rank": 8, "init": "random", "random_state": 0, "n_iter_max": 100,
                            "tol": 1e-8},
                 "init_factors": [np.array(f) for f in init.factors],
                 "weights": np.array(cp.weights), "factors": [np.array(f) for f in cp.factors],
                 "errors": [float(e) for e in errs]})

    def small(seed, shape, rank, dtype=np.float64, noise=0.01):
        rs = np.random.RandomState(seed)
        fs = [rs.uniform(size=(s, rank)) for s in shape]
        t = tl.cp_to_tensor((None, fs))
        n = rs.randn(*shape)
        t = t + noise * np.linalg.norm(t) * n / np.linalg.norm(n)
        return t.astype(dtype)

    variants = [
        ("normalize", dict(shape=(9, 8, 7), rank=3, seed=11),
         dict(init="random", random_state=3, n_iter_max=30, tol=1e-10, normalize_factors=True)),
        ("l2_reg", dict(shape=(9, 8, 7), rank=3, seed=12),
         dict(init="random", random_state=4, n_iter_max=25, tol=0, l2_reg=0.05)),
        ("fixed_mode0", dict(shape=(10, 6, 5), rank=2, seed=13),
         dict(init="random", random_state=5, n_iter_max=20, tol=0, fixed_modes=[0])),
        ("rec_error_crit", dict(shape=(7, 9, 8), rank=4, seed=14),
         dict(init="random", random_state=6, n_iter_max=200, tol=1e-7,
              cvg_criterion="rec_error")),
        ("svd_init", dict(shape=(12, 10, 9), rank=3, seed=15),
         dict(init="svd", n_iter_max=30, tol=1e-9)),
        ("svd_init_short_mode", dict(shape=(4, 10, 9), rank=6, seed=16),
         dict(init="svd", random_state=7, n_iter_max=15, tol=0)),
        ("fourway", dict(shape=(6, 5, 7, 4), rank=3, seed=17),
         dict(init="random", random_state=8, n_iter_max=40, tol=1e-9)),
        ("twoway", dict(shape=(11, 9), rank=3, seed=18),
         dict(init="random", random_state=9, n_iter_max=20, tol=0)),
        ("fiveway", dict(shape=(4, 5, 3, 6, 4), rank=2, seed=19),
         dict(init="random", random_state=10, n_iter_max=12, tol=0)),
        ("rank1", dict(shape=(6, 8, 7), rank=1, seed=20),
         dict(init="random", random_state=11, n_iter_max=20, tol=1e-10)),
        ("f32_small", dict(shape=(16, 12, 10), rank=4, seed=21, dtype=np.float32),
         dict(init="random", random_state=12, n_iter_max=30, tol=0)),
    ]
    for name, g, kw in variants:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        try:
            cp, errs = parafac(x, g["rank"], return_errors=True, **copy.deepcopy(kw))
        except Exception as e:
            raise RuntimeError(f"reference parafac failed on case {name}") from e
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
                     "kwargs": {"rank": g["rank"], **kw},
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})

    # non-negative CP by multiplicative updates (tensorly/decomposition/_nn_cp.py)
    from tensorly.decomposition import non_negative_parafac
    nn_variants = [
        ("nn_mu_random", dict(shape=(9, 8, 7), rank=3, seed=51),
         dict(init="random", random_state=13, n_iter_max=60, tol=1e-12)),
        ("nn_mu_svd", dict(shape=(12, 10, 9), rank=3, seed=52),
         dict(init="svd", n_iter_max=40, tol=1e-12)),
        ("nn_mu_4way_fixed", dict(shape=(6, 5, 7, 4), rank=2, seed=53),
         dict(init="random", random_state=14, n_iter_max=30, tol=1e-12, fixed_modes=[1])),
        ("nn_mu_stop", dict(shape=(10, 9, 8), rank=2, seed=54),
         dict(init="svd", n_iter_max=500, tol=1e-7)),
        ("nn_mu_f32", dict(shape=(16, 12, 10), rank=4, seed=55, dtype=np.float32),
         dict(init="random", random_state=15, n_iter_max=30, tol=1e-12)),
    ]
    for name, g, kw in nn_variants:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        cp, errs = non_negative_parafac(x, g["rank"], return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
                     "kwargs": {"rank": g["rank"], **kw},
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})

    # non-negative CP by HALS (tensorly/decomposition/_nn_cp.py:186-377)
    from tensorly.decomposition import non_negative_parafac_hals
    hals_variants = [
        ("nn_hals_random", dict(shape=(9, 8, 7), rank=3, seed=61),
         dict(init="random", random_state=16, n_iter_max=25, tol=1e-12)),
        ("nn_hals_svd", dict(shape=(12, 10, 9), rank=3, seed=62),
         dict(init="svd", n_iter_max=20, tol=1e-12)),
        ("nn_hals_sparse_fixed", dict(shape=(8, 7, 6, 5), rank=2, seed=63),
         dict(init="random", random_state=17, n_iter_max=15, tol=1e-12,
              sparsity_coefficients=[0.01, None, 0.02, None], fixed_modes=[1])),
        ("nn_hals_stop", dict(shape=(10, 9, 8), rank=2, seed=64),
         dict(init="svd", n_iter_max=300, tol=1e-9)),
        ("nn_hals_f32", dict(shape=(16, 12, 10), rank=4, seed=65, dtype=np.float32),
         dict(init="random", random_state=18, n_iter_max=15, tol=1e-12)),
        # rank 1: the inner stop test ends each hals_nnls call after 2 iterations
        ("nn_hals_rank1", dict(shape=(9, 8, 7), rank=1, seed=66),
         dict(init="random", random_state=19, n_iter_max=6, tol=1e-12)),
        # exact=True: 50000 inner iterations per call, no early stop at rank 2
        ("nn_hals_exact", dict(shape=(8, 7, 6), rank=2, seed=67),
         dict(init="svd", n_iter_max=2, tol=1e-12, exact=True)),
        # unconstrained mode 1 (solved by the normal equations), normalised factors
        ("nn_hals_modes_02", dict(shape=(10, 9, 8), rank=3, seed=68),
         dict(init="svd", n_iter_max=12, tol=1e-12, nn_modes=[0, 2])),
        ("nn_hals_normalize", dict(shape=(9, 8, 7), rank=3, seed=69),
         dict(init="random", random_state=20, n_iter_max=10, tol=1e-12,
              normalize_factors=True)),
    ]
    for name, g, kw in hals_variants:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        cp, errs = non_negative_parafac_hals(x, g["rank"], return_errors=True,
                                             **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
                     "kwargs": {"rank": g["rank"], **kw},
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})

    # randomised CP-ALS (tensorly/decomposition/_cp.py:546-762)
    from tensorly.decomposition import randomised_parafac
    from tensorly.decomposition._cp import sample_khatri_rao
    rand_variants = [
        ("rand_random", dict(shape=(10, 10, 10), rank=4, seed=71),
         dict(n_samples=100, n_iter_max=30, tol=0, init="random", random_state=5)),
        ("rand_svd_tol", dict(shape=(12, 11, 10), rank=3, seed=72),
         dict(n_samples=50, n_iter_max=40, tol=1e-6, init="svd", random_state=6)),
        ("rand_4way", dict(shape=(6, 5, 7, 4), rank=3, seed=73),
         dict(n_samples=40, n_iter_max=15, tol=0, init="random", random_state=7)),
        ("rand_f32", dict(shape=(14, 12, 10), rank=4, seed=74, dtype=np.float32),
         dict(n_samples=80, n_iter_max=20, tol=0, init="random", random_state=8)),
    ]
    for name, g, kw in rand_variants:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        cp, errs = randomised_parafac(x, g["rank"], return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
                     "kwargs": {"rank": g["rank"], **kw},
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})
    rs = np.random.RandomState(9)
    fs = [rs.random_sample((s, 3)) for s in (8, 9, 10)]
    skr, ind, ind_kr = sample_khatri_rao(fs, 6, skip_matrix=1, return_sampled_rows=True,
                                         random_state=np.random.RandomState(11))
    runs.append({"case": "sample_kr", "gen": {"fn": "factors", "seed": 9},
                 "checksum": cs(np.concatenate([f.ravel() for f in fs])),
                 "kwargs": {"n_samples": 6, "skip_matrix": 1, "random_state": 11},
                 "factors_in": fs, "sampled_kr": np.array(skr),
                 "indices_list": [np.array(i) for i in ind], "indices_kr": np.array(ind_kr)})

    # constrained CP by AO-ADMM (tensorly/decomposition/_constrained_cp.py:166-435);
    # init='random' draws from NumPy's global generator, seeded per case
    from tensorly.decomposition import constrained_parafac
    cons_variants = [
        ("cons_nonneg_svd", dict(shape=(10, 9, 8), rank=3, seed=81),
         dict(non_negative=True, init="svd", n_iter_max=20, tol_outer=1e-10), None),
        ("cons_l1_random", dict(shape=(9, 8, 7), rank=3, seed=82),
         dict(l1_reg=0.05, init="random", n_iter_max=15, tol_outer=1e-10), 5),
        ("cons_l2sq_list", dict(shape=(8, 7, 6), rank=2, seed=83),
         dict(l2_square_reg=[0.1, 0.2, 0.3], init="svd", n_iter_max=15, tol_outer=1e-10), None),
        ("cons_l2_dict_fixed", dict(shape=(8, 7, 6, 5), rank=2, seed=84),
         dict(l2_reg={0: 0.01, 2: 0.02}, fixed_modes=[1], init="svd", n_iter_max=10,
              tol_outer=1e-10, cvg_criterion="rec_error"), None),
        ("cons_normalize_mixed", dict(shape=(9, 8, 7), rank=3, seed=85),
         dict(normalize={1: True}, non_negative={0: True, 2: True}, init="svd", n_iter_max=12,
              tol_outer=1e-10), None),
        ("cons_inner", dict(shape=(10, 9, 8), rank=2, seed=86),
         dict(non_negative=True, init="svd", n_iter_max=8, n_iter_max_inner=30,
              tol_inner=1e-10, tol_outer=1e-10), None),
        ("cons_stop", dict(shape=(10, 9, 8), rank=2, seed=87),
         dict(l2_square_reg=0.01, init="svd", n_iter_max=200, tol_outer=1e-7), None),
        ("cons_f32", dict(shape=(12, 10, 9), rank=3, seed=88, dtype=np.float32),
         dict(non_negative=True, init="svd", n_iter_max=10, tol_outer=1e-10), None),
    ]
    for name, g, kw, gseed in cons_variants:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        if gseed is not None:
            np.random.seed(gseed)
        cp, errs = constrained_parafac(x, g["rank"], return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
                     "kwargs": {"rank": g["rank"], **kw}, "global_seed": gseed,
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})

    # non-negative Tucker by multiplicative updates (tensorly/decomposition/_tucker.py:348-454)
    from tensorly.decomposition import non_negative_tucker
    nnt_variants = [
        ("nnt_svd", dict(shape=(10, 9, 8), rank=3, seed=91),
         dict(rank=[3, 4, 2], n_iter_max=15, init="svd", tol=1e-12)),
        ("nnt_random", dict(shape=(9, 8, 7, 6), rank=2, seed=92),
         dict(rank=[2, 3, 2, 3], n_iter_max=12, init="random", random_state=3, tol=1e-12)),
        ("nnt_stop", dict(shape=(12, 10, 9), rank=2, seed=93),
         dict(rank=[2, 2, 2], n_iter_max=100, init="svd", tol=1e-6)),
        ("nnt_f32", dict(shape=(14, 12, 10), rank=3, seed=94, dtype=np.float32),
         dict(rank=[3, 3, 3], n_iter_max=10, init="svd", tol=1e-12)),
    ]
    for name, g, kw in nnt_variants:
        x = np.abs(small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64)))
        tt, errs = non_negative_tucker(x, return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", "abs": True, **g}, "checksum": cs(x),
                     "kwargs": kw, "core": np.array(tt.core),
                     "factors": [np.array(f) for f in tt.factors],
                     "errors": [float(e) for e in errs]})

    # non-negative Tucker by HALS + FISTA (tensorly/decomposition/_tucker.py:457-691)
    from tensorly.decomposition import non_negative_tucker_hals
    nnth_variants = [
        ("nnth_svd", dict(shape=(10, 9, 8), rank=3, seed=95),
         dict(rank=[3, 4, 2], n_iter_max=10, init="svd", tol=1e-12)),
        ("nnth_random", dict(shape=(9, 8, 7, 6), rank=2, seed=96),
         dict(rank=[2, 3, 2, 3], n_iter_max=8, init="random", random_state=4, tol=1e-12)),
        ("nnth_sparse", dict(shape=(10, 9, 8), rank=3, seed=97),
         dict(rank=[3, 3, 3], n_iter_max=8, init="svd", tol=1e-12,
              sparsity_coefficients=[0.01, None, 0.02], core_sparsity_coefficient=0.001)),
        ("nnth_f32", dict(shape=(12, 10, 9), rank=3, seed=98, dtype=np.float32),
         dict(rank=[3, 3, 3], n_iter_max=8, init="svd", tol=1e-12)),
        ("nnth_active_set", dict(shape=(9, 8, 7), rank=2, seed=99),
         dict(rank=[2, 3, 2], n_iter_max=6, init="svd", tol=1e-12, algorithm="active_set")),
        ("nnth_active_set_4way", dict(shape=(7, 6, 5, 6), rank=2, seed=100),
         dict(rank=[2, 2, 2, 2], n_iter_max=5, init="random", random_state=7, tol=1e-12,
              algorithm="active_set")),
    ]
    for name, g, kw in nnth_variants:
        x = np.abs(small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64)))
        tt, errs = non_negative_tucker_hals(x, return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", "abs": True, **g}, "checksum": cs(x),
                     "kwargs": kw, "core": np.array(tt.core),
                     "factors": [np.array(f) for f in tt.factors],
                     "errors": [float(e) for e in errs]})

    # PARAFAC2 (tensorly/decomposition/_parafac2.py:399-707), ragged slices
    from tensorly.decomposition import parafac2
    p2_variants = [
        ("p2_random", dict(seed=101, rows=[8, 9, 10, 11, 12], cols=6),
         dict(rank=3, n_iter_max=12, random_state=1)),
        ("p2_svd", dict(seed=102, rows=[7, 9, 8, 10], cols=5),
         dict(rank=2, n_iter_max=10, init="svd")),
        ("p2_nols", dict(seed=103, rows=[9, 9, 10, 8, 11, 12], cols=7),
         dict(rank=3, n_iter_max=15, random_state=2, linesearch=False)),
        ("p2_normalize", dict(seed=104, rows=[8, 10, 9], cols=6),
         dict(rank=2, n_iter_max=8, random_state=3, normalize_factors=True)),
        ("p2_f32", dict(seed=105, rows=[10, 11, 12, 9], cols=6, dtype=np.float32),
         dict(rank=3, n_iter_max=10, random_state=4)),
    ]
    # non-negative modes (HALS inner solve) and masked slices (imputation);
    # nn_modes="all" only without line search: the reference's line search
    # tests ``0 in nn_modes``, a TypeError on the string
    p2_variants += [
        ("p2_nn_all", dict(seed=106, rows=[8, 9, 10, 11], cols=6),
         dict(rank=3, n_iter_max=10, random_state=5, nn_modes="all", linesearch=False)),
        ("p2_nn_02", dict(seed=107, rows=[9, 8, 10, 12, 11], cols=7),
         dict(rank=3, n_iter_max=12, random_state=6, nn_modes=[0, 2])),
        ("p2_mask", dict(seed=108, rows=[8, 10, 9, 11], cols=6, mask_keep=0.8),
         dict(rank=2, n_iter_max=12, random_state=7)),
        ("p2_mask_svd", dict(seed=109, rows=[7, 9, 8], cols=5, mask_keep=0.7),
         dict(rank=2, n_iter_max=8, init="svd", linesearch=False)),
    ]
    for name, g, kw in p2_variants:
        rsl = np.random.RandomState(g["seed"])
        xs = [rsl.rand(r, g["cols"]).astype(g.get("dtype", np.float64)) for r in g["rows"]]
        ck = [float(sum(np.asarray(t, np.float64).sum() for t in xs)),
              float(np.sqrt(sum((np.asarray(t, np.float64) ** 2).sum() for t in xs)))]
        kw_call = copy.deepcopy(kw)
        if "mask_keep" in g:
            kw_call["mask"] = slice_masks(g)
        out, errs = parafac2(xs, return_errors=True, **kw_call)
        w, fs, ps = out
        runs.append({"case": name, "gen": {"fn": "slices", **g}, "checksum": ck, "kwargs": kw,
                     "weights": np.array(w), "factors": [np.array(f) for f in fs],
                     "projections": [np.array(p) for p in ps],
                     "errors": [float(e) for e in errs]})

    # parafac branches the GPU path does not take yet: line search,
    # orthogonalisation, sparse component, mask (tensorly/decomposition/_cp.py:230-543)
    cp_branches = [
        ("cp_linesearch", dict(shape=(12, 11, 10), rank=3, seed=111),
         dict(init="random", random_state=11, linesearch=True, n_iter_max=30, tol=1e-10), None),
        ("cp_orth", dict(shape=(10, 9, 8), rank=3, seed=112),
         dict(init="svd", orthogonalise=5, n_iter_max=15, tol=1e-10), None),
        ("cp_sparsity", dict(shape=(10, 9, 8), rank=3, seed=113),
         dict(init="svd", sparsity=0.05, n_iter_max=10, tol=1e-10), None),
        ("cp_mask", dict(shape=(10, 9, 8), rank=3, seed=114),
         dict(init="random", random_state=12, n_iter_max=10, tol=1e-10), 0.8),
        ("cp_mask_linesearch", dict(shape=(10, 9, 8), rank=2, seed=115),
         dict(init="random", random_state=13, n_iter_max=12, tol=1e-10, linesearch=True), 0.7),
    ]
    for name, g, kw, keep in cp_branches:
        x = small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        kwr = copy.deepcopy(kw)
        mask = None
        if keep is not None:
            mask = (np.random.RandomState(g["seed"] + 1000).rand(*g["shape"]) < keep).astype(
                x.dtype)
            kwr["mask"] = mask
        out, errs = parafac(x, g["rank"], return_errors=True, **kwr)
        rec = {"case": name, "gen": {"fn": "small", **g}, "checksum": cs(x),
               "kwargs": {"rank": g["rank"], **kw}, "mask_keep": keep,
               "errors": [float(e) for e in errs]}
        if kw.get("sparsity"):
            (w, f), sparse = out
            rec["sparse"] = np.array(sparse)
        else:
            w, f = out
        rec["weights"] = np.array(w)
        rec["factors"] = [np.array(m) for m in f]
        runs.append(rec)

    # Tucker (HOOI) small cases
    tcases = [
        ("tucker_svd", dict(shape=(12, 10, 8), seed=31), dict(rank=[3, 4, 2], init="svd",
                                                             n_iter_max=20, tol=1e-9)),
        ("tucker_random", dict(shape=(9, 8, 10), seed=32), dict(rank=[2, 3, 3], init="random",
                                                               random_state=1, n_iter_max=15,
                                                               tol=0)),
        ("tucker_4way", dict(shape=(6, 7, 5, 8), seed=33), dict(rank=[2, 3, 2, 3], init="svd",
                                                               n_iter_max=10, tol=1e-10)),
    ]
    for name, g, kw in tcases:
        rs = np.random.RandomState(g["seed"])
        x = rs.randn(*g["shape"])
        tt, errs = tucker(x, return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "randn", **g}, "checksum": cs(x),
                     "kwargs": kw, "core": np.array(tt.core),
                     "factors": [np.array(f) for f in tt.factors],
                     "errors": [float(e) for e in errs]})

    # masked Tucker (missing entries refilled from the model each iteration)
    for name, g, kw, keep in (
            ("tucker_mask", dict(shape=(10, 9, 8), seed=34),
             dict(rank=[3, 3, 2], init="random", random_state=5, n_iter_max=12, tol=1e-9), 0.8),
            ("tucker_mask_4way", dict(shape=(6, 7, 5, 6), seed=35),
             dict(rank=[2, 3, 2, 2], init="random", random_state=6, n_iter_max=8, tol=0), 0.7)):
        rs = np.random.RandomState(g["seed"])
        x = rs.randn(*g["shape"])
        mask = (np.random.RandomState(g["seed"] + 1000).rand(*g["shape"]) < keep).astype(x.dtype)
        tt, errs = tucker(x, return_errors=True, mask=mask, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "randn", **g}, "checksum": cs(x),
                     "kwargs": kw, "mask_keep": keep, "core": np.array(tt.core),
                     "factors": [np.array(f) for f in tt.factors],
                     "errors": [float(e) for e in errs]})

    # svd_interface of a tall and a wide matrix
    for name, shape, k in (("svd_wide", (7, 30), 4), ("svd_tall", (25, 6), 3)):
        rs = np.random.RandomState(40 + shape[0])
        m = rs.randn(*shape)
        U, S, V = svd_interface(m, n_eigenvecs=k)
        runs.append({"case": name, "gen": {"fn": "randn", "shape": shape, "seed": 40 + shape[0]},
                     "checksum": cs(m), "kwargs": {"n_eigenvecs": k},
                     "U": np.array(U), "S": np.array(S), "V": np.array(V)})
    return runs


def record_container_validation():
    """CPTensor and TuckerTensor construction on well-formed and malformed
    inputs (tensorly/cp_tensor.py:17-29 with _validate_cp_tensor :163-214;
    tensorly/tucker_tensor.py:227-236 with _validate_tucker_tensor :19-47):
    the shape and rank, or the exception type and message."""
    from tensorly.cp_tensor import CPTensor
    from tensorly.tucker_tensor import TuckerTensor
    rs = np.random.RandomState(7)
    records = []

    def call(kind, value):
        rec = {"kind": kind, "value": value}
        try:
            obj = (CPTensor if kind == "cp" else TuckerTensor)(value)
            rec["shape"] = tuple(int(v) for v in obj.shape)
            rec["rank"] = (int(obj.rank) if kind == "cp" else tuple(int(v) for v in obj.rank))
        except Exception as e:      # noqa: BLE001 (the exception is the record)
            rec["raises"] = type(e).__name__
            rec["message"] = str(e)
        records.append(rec)

    m = lambda *s: rs.random_sample(s)   # noqa: E731
    call("cp", (None, [m(4, 3), m(5, 3), m(6, 3)]))
    call("cp", (np.ones(3), [m(4, 3), m(5, 3), m(6, 3)]))
    call("cp", (np.ones(2), [m(4, 3), m(5, 3), m(6, 3)]))
    call("cp", (np.ones((3, 1)), [m(4, 3), m(5, 3)]))
    call("cp", (None, [m(4, 3), m(5, 2), m(6, 3)]))
    call("cp", (None, [m(4, 3), m(5, 3), m(6, 4)]))
    call("cp", (None, [m(4), m(5), m(6)]))
    call("cp", (np.ones(1), [m(4), m(5, 1)]))
    call("cp", (None, [m(4), m(5, 2)]))
    call("cp", (None, [m(4, 3, 2), m(5, 3)]))
    call("cp", (None, [m(7, 1)]))
    call("cp", (np.ones(5), [m(3, 5), m(2, 5), m(4, 5), m(1, 5)]))
    call("tucker", (m(2, 3, 4), [m(5, 2), m(6, 3), m(7, 4)]))
    call("tucker", (m(2, 3), [m(5, 2), m(6, 3)]))
    call("tucker", (m(2, 3, 4), [m(5, 2), m(6, 3)]))
    call("tucker", (m(2, 3), [m(5, 2), m(6, 3), m(7, 4)]))
    call("tucker", (m(2, 3, 4), [m(5, 2), m(6, 4), m(7, 4)]))
    call("tucker", (m(2,), [m(5, 2)]))
    call("tucker", (m(3, 3, 3, 3), [m(4, 3)] * 4))
    call("tucker", (m(3, 3, 3, 3), [m(4, 3)] * 3 + [m(4, 2)]))
    return records


def record_cons_columns():
    """constrained_parafac (tensorly/decomposition/_constrained_cp.py:166-435)
    with the column-wise proximal operators and the whole-matrix sparsity
    ones of tensorly/tenalg/proximal.py:270-628: unimodality, monotonicity,
    simplex, soft_sparsity, normalized_sparsity, smoothness, hard_sparsity,
    and a mix of three on different modes."""
    import copy
    from golden_inputs import small_cp
    from tensorly.decomposition import constrained_parafac
    cases = [
        ("cons_unimodality", dict(unimodality=True)),
        ("cons_monotonicity", dict(monotonicity=True)),
        ("cons_simplex", dict(simplex=3.0)),
        ("cons_soft_sparsity", dict(soft_sparsity=3.0)),
        ("cons_normalized_sparsity", dict(normalized_sparsity=12)),
        ("cons_smoothness", dict(smoothness=0.1)),
        ("cons_hard_sparsity", dict(hard_sparsity=15)),
        ("cons_columns_mixed", dict(monotonicity={0: True}, smoothness={1: 0.2},
                                    simplex={2: 2.0})),
    ]
    runs = []
    for i, (name, cons) in enumerate(cases):
        g = dict(shape=(10, 9, 8), rank=3, seed=101 + i)
        x = small_cp(g["seed"], g["shape"], g["rank"])
        kw = dict(cons, init="svd", n_iter_max=8, tol_outer=1e-10)
        cp, errs = constrained_parafac(x, g["rank"], return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "gen": {"fn": "small", **g}, "checksum":
                     [float(np.asarray(x, np.float64).sum()), float(np.linalg.norm(x))],
                     "kwargs": {"rank": g["rank"], **kw}, "global_seed": None,
                     "weights": np.array(cp.weights),
                     "factors": [np.array(f) for f in cp.factors],
                     "errors": [float(e) for e in errs]})
    return runs


def record_tucker_extras():
    """Non-negative Tucker with normalize_factors (MU and HALS, both core
    updates), the reference's tucker_normalize, kronecker and active_set_nnls
    on fixed inputs (tensorly/solvers/tests/test_nnls.py:45-60 is the shape of
    the last), and the ValueError non_negative_tucker_hals raises with fixed
    modes (tensorly/decomposition/_tucker.py:457-691)."""
    import copy
    from golden_inputs import small_cp as small
    import tensorly as tl
    from tensorly.decomposition import non_negative_tucker, non_negative_tucker_hals
    from tensorly.solvers.nnls import active_set_nnls
    from tensorly.tenalg import kronecker
    from tensorly.tucker_tensor import tucker_normalize
    runs = []
    variants = [
        ("nnt_normalize", non_negative_tucker, dict(shape=(10, 9, 8), rank=3, seed=131),
         dict(rank=[3, 2, 3], n_iter_max=8, init="svd", tol=1e-12, normalize_factors=True)),
        ("nnth_normalize", non_negative_tucker_hals, dict(shape=(9, 8, 7), rank=2, seed=132),
         dict(rank=[2, 3, 2], n_iter_max=6, init="svd", tol=1e-12, normalize_factors=True)),
        ("nnth_active_set_normalize", non_negative_tucker_hals,
         dict(shape=(8, 7, 6), rank=2, seed=133),
         dict(rank=[2, 2, 3], n_iter_max=5, init="random", random_state=11, tol=1e-12,
              algorithm="active_set", normalize_factors=True)),
        ("nnth_active_set_f32", non_negative_tucker_hals,
         dict(shape=(9, 8, 7), rank=2, seed=134, dtype=np.float32),
         dict(rank=[2, 2, 2], n_iter_max=5, init="svd", tol=1e-12, algorithm="active_set")),
        ("nnth_active_set_stop", non_negative_tucker_hals, dict(shape=(8, 8, 8), rank=2, seed=135),
         dict(rank=[2, 2, 2], n_iter_max=60, init="svd", tol=1e-6, algorithm="active_set")),
    ]
    for name, fn, g, kw in variants:
        x = np.abs(small(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64)))
        tt, errs = fn(x, return_errors=True, **copy.deepcopy(kw))
        runs.append({"case": name, "fn": fn.__name__,
                     "gen": {"fn": "small", "abs": True, **g},
                     "checksum": [float(np.asarray(x, np.float64).sum()),
                                  float(np.linalg.norm(np.asarray(x, np.float64)))],
                     "kwargs": kw, "core": np.array(tt.core),
                     "factors": [np.array(f) for f in tt.factors],
                     "errors": [float(e) for e in errs]})
    kats = []
    rs = np.random.RandomState(136)
    for shape, rank in (((3, 4, 5), (3, 2, 4)), ((6, 5, 4, 3), (2, 3, 2, 2)), ((5, 6), (4, 1))):
        core = rs.randn(*rank)
        factors = [rs.randn(s, r) for s, r in zip(shape, rank)]
        factors[0][:, 0] = 0.0                      # a zero column keeps its zeros
        c2, f2 = tucker_normalize((core.copy(), [f.copy() for f in factors]))
        kats.append({"op": "tucker_normalize", "core": core, "factors": factors,
                     "out_core": np.array(c2), "out_factors": [np.array(f) for f in f2]})
    for dims in (((2, 3), (4, 2)), ((3, 3), (2, 2), (2, 4)), ((1, 5), (3, 1), (2, 2), (2, 3))):
        ms = [rs.randn(*d) for d in dims]
        kats.append({"op": "kronecker", "matrices": ms, "out": np.array(kronecker(ms)),
                     "out_skip1_rev": np.array(kronecker(ms, skip_matrix=1, reverse=True))})
    for n, m, seed in ((10, 30, 137), (24, 60, 138), (64, 128, 139)):
        r = np.random.RandomState(seed)
        a = r.randn(m, n)
        xtrue = np.abs(r.randn(n)) * (r.rand(n) > 0.4)
        b = a @ xtrue + 0.01 * r.randn(m)
        ata, atb = a.T @ a, a.T @ b
        x0 = None if seed != 138 else np.abs(r.randn(n))
        out = active_set_nnls(tl.tensor(atb), tl.tensor(ata), x=x0, n_iter_max=100)
        kats.append({"op": "active_set_nnls", "UtU": ata, "Utm": atb, "x0": x0,
                     "out": np.array(out)})
    errors = []
    for shape, rank, fixed in (((6, 5, 4), [2, 2, 2], [0]), ((6, 5, 4), [2, 2, 2], [1]),
                               ((7, 6, 5, 4), [2, 3, 2, 2], [0, 2]),
                               ((7, 6, 5, 4), [3, 2, 4, 2], [1])):
        for init in ("svd", "random"):
            x = np.abs(np.random.RandomState(140).randn(*shape))
            try:
                non_negative_tucker_hals(x, rank, n_iter_max=2, init=init, random_state=0,
                                         fixed_modes=list(fixed))
                msg = None
            except ValueError as e:
                msg = str(e)
            errors.append({"shape": shape, "rank": rank, "fixed": fixed, "init": init,
                           "message": msg})
    return {"runs": runs, "kats": kats, "fixed_mode_errors": errors}


def record_svd_extras():
    """svd_interface with a mask and with 'randomized_svd'
    (tensorly/tenalg/svd.py:138-170, :288-357, :431-439), and the callers
    that reach them: masked tucker (tensorly/decomposition/_tucker.py:25-221)
    from 'svd' and 'random' starts, tucker and parafac with
    svd='randomized_svd', and parafac with a mask from an 'svd' start
    (tensorly/decomposition/_cp.py:26-137).  Randomised runs without a
    random_state draw from NumPy's global generator, seeded here and in the
    tests by ``np_seed``."""
    import copy
    from golden_inputs import small_cp
    import tensorly as tl
    from tensorly.decomposition import parafac, tucker
    from tensorly.tenalg.svd import randomized_svd, svd_interface
    rs = np.random.RandomState(150)
    kats = []
    for (r, c), k, method, keep in (((30, 20), 4, "truncated_svd", 0.8),
                                    ((20, 45), 3, "truncated_svd", 0.7),
                                    ((40, 25), 5, "randomized_svd", 0.85),
                                    ((18, 60), 4, "randomized_svd", 0.8),
                                    ((50, 12), 3, "truncated_svd", None),
                                    ((12, 70), 5, "randomized_svd", None),
                                    ((64, 30), 6, "randomized_svd", None)):
        lr = rs.randn(r, k + 1) @ rs.randn(k + 1, c) + 0.05 * rs.randn(r, c)
        mask = None if keep is None else (rs.rand(r, c) < keep).astype(np.float64)
        kw = dict(n_eigenvecs=k, method=method)
        if method == "randomized_svd":
            kw["random_state"] = 7
        U, S, V = svd_interface(tl.tensor(lr), mask=None if mask is None else tl.tensor(mask),
                                n_iter_mask_imputation=4, **kw)
        kats.append({"op": "svd_interface", "matrix": lr, "mask": mask, "kwargs": kw,
                     "n_iter_mask_imputation": 4,
                     "U": np.array(U), "S": np.array(S), "V": np.array(V)})
    for (r, c), k in (((40, 15), 4), ((15, 40), 4), ((30, 30), 6)):
        m = rs.randn(r, c)
        U, S, V = randomized_svd(tl.tensor(m), n_eigenvecs=k, n_iter=3, random_state=11)
        kats.append({"op": "randomized_svd", "matrix": m, "kwargs": dict(n_eigenvecs=k, n_iter=3),
                     "random_state": 11, "U": np.array(U), "S": np.array(S), "V": np.array(V)})
    runs = []
    variants = [
        ("tucker_mask_svd", "tucker", dict(shape=(10, 9, 8), rank=3, seed=151, mask_keep=0.85),
         dict(rank=[3, 3, 2], n_iter_max=6, init="svd", tol=0), None),
        ("tucker_mask_random", "tucker", dict(shape=(9, 8, 7, 6), rank=2, seed=152,
                                              mask_keep=0.8),
         dict(rank=[2, 2, 2, 2], n_iter_max=5, init="random", random_state=3, tol=0), None),
        ("tucker_randomized", "tucker", dict(shape=(12, 10, 9), rank=3, seed=153),
         dict(rank=[3, 3, 3], n_iter_max=4, init="svd", svd="randomized_svd", random_state=5,
              tol=0), None),
        ("cp_randomized", "parafac", dict(shape=(11, 10, 9), rank=3, seed=154),
         dict(rank=3, n_iter_max=6, init="svd", svd="randomized_svd", tol=0), 21),
        ("cp_mask_svd", "parafac", dict(shape=(10, 9, 8), rank=3, seed=155, mask_keep=0.85),
         dict(rank=3, n_iter_max=8, init="svd", tol=0, svd_mask_repeats=3), None),
    ]
    for name, fn, g, kw, np_seed in variants:
        x = small_cp(g["seed"], g["shape"], g["rank"])
        kwc = copy.deepcopy(kw)
        if "mask_keep" in g:
            kwc["mask"] = tl.tensor((np.random.RandomState(g["seed"] + 1000)
                                     .rand(*g["shape"]) < g["mask_keep"]).astype(np.float64))
        rank = kwc.pop("rank")
        if np_seed is not None:
            np.random.seed(np_seed)
        if fn == "tucker":
            tt, errs = tucker(tl.tensor(x), rank, return_errors=True, **kwc)
            rec = {"core": np.array(tt.core), "factors": [np.array(f) for f in tt.factors]}
        else:
            cp, errs = parafac(tl.tensor(x), rank, return_errors=True, **kwc)
            rec = {"weights": np.array(cp.weights), "factors": [np.array(f) for f in cp.factors]}
        runs.append({"case": name, "fn": fn, "gen": {"fn": "small", **g}, "np_seed": np_seed,
                     "checksum": [float(x.sum()), float(np.linalg.norm(x))], "kwargs": kw,
                     "errors": [float(e) for e in errs], **rec})
    return {"runs": runs, "kats": kats}


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "tensorly")):
        sys.exit("make_golden: set TENSORLY_REFERENCE to the TensorLy source tree "
                 "(the directory that holds the tensorly package)")
    sys.path.insert(0, REF)
    import tensorly  # noqa: F401  (the reference)
    cont = record_container_validation()
    with open(os.path.join(HERE, "container_kats.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "records": cont}, f, protocol=4)
    if "containers" in sys.argv[1:]:
        print(f"{len(cont)} container records")
        return
    sys.path.insert(0, os.path.dirname(HERE))    # tests/: golden_inputs
    sys.path.insert(0, REPO)                     # the oracle golden_inputs imports
    cols = record_cons_columns()
    with open(os.path.join(HERE, "cons_column_runs.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "runs": cols}, f, protocol=4)
    if "cons_columns" in sys.argv[1:]:
        print(f"{len(cols)} constrained runs with column-wise operators")
        return
    extras = record_tucker_extras()
    with open(os.path.join(HERE, "tucker_extra_runs.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), **extras}, f, protocol=4)
    if "tucker_extras" in sys.argv[1:]:
        print(f"{len(extras['runs'])} Tucker runs, {len(extras['kats'])} records")
        return
    svdx = record_svd_extras()
    with open(os.path.join(HERE, "svd_extra_runs.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), **svdx}, f, protocol=4)
    if "svd_extras" in sys.argv[1:]:
        print(f"{len(svdx['runs'])} runs, {len(svdx['kats'])} records")
        return
    kats = record_kats()
    with open(os.path.join(HERE, "tenalg_kats.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "records": kats}, f, protocol=4)
    runs = reference_runs()
    with open(os.path.join(HERE, "reference_runs.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "runs": runs}, f, protocol=4)
    recon = record_reconstruction()
    with open(os.path.join(HERE, "reconstruction_kats.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "records": recon}, f, protocol=4)
    prox = record_proximal()
    with open(os.path.join(HERE, "proximal_kats.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "records": prox}, f, protocol=4)
    host = record_host_validators()
    with open(os.path.join(HERE, "host_kats.pkl"), "wb") as f:
        pickle.dump({"versions": _versions(), "records": host}, f, protocol=4)
    print(f"{len(kats)} tenalg records, {len(runs)} reference runs, "
          f"{len(recon)} reconstruction records, {len(prox)} proximal records, "
          f"{len(host)} host-helper records")


if __name__ == "__main__":
    main()
