"""Pins the NumPy oracle to the reference: replays the reference's own
tenalg unit-test calls and its parafac / tucker / svd runs (tests/golden)."""

import warnings

import numpy as np
import pytest

import oracle
from golden_inputs import regenerate, slice_masks

FN = {"khatri_rao": oracle.khatri_rao, "mode_dot": oracle.mode_dot,
      "multi_mode_dot": oracle.multi_mode_dot,
      "unfolding_dot_khatri_rao": oracle.unfolding_dot_khatri_rao}


def test_kat_records_present(golden):
    names = {r["fn"] for r in golden["kats"]}
    assert {"khatri_rao", "mode_dot", "multi_mode_dot", "unfolding_dot_khatri_rao"} <= names
    assert sum(1 for r in golden["kats"] if r["fn"] == "__test__") >= 4


def test_oracle_replays_reference_tenalg_calls(golden):
    n = 0
    for rec in golden["kats"]:
        fn = FN.get(rec["fn"])
        if fn is None:
            continue
        args = [np.asarray(a) if isinstance(a, np.ndarray) else a for a in rec["args"]]
        if "raises" in rec:
            with pytest.raises(ValueError if rec["raises"] == "ValueError" else Exception):
                fn(*args, **rec["kwargs"])
            continue
        out = fn(*args, **rec["kwargs"])
        np.testing.assert_array_equal(np.asarray(out), np.asarray(rec["result"]))
        n += 1
    assert n >= 30


RFN = {"cp_to_tensor": oracle.cp_to_tensor, "cp_to_unfolded": oracle.cp_to_unfolded,
       "cp_to_vec": oracle.cp_to_vec, "tucker_to_tensor": oracle.tucker_to_tensor,
       "tucker_to_unfolded": oracle.tucker_to_unfolded, "tucker_to_vec": oracle.tucker_to_vec}


def test_oracle_replays_reference_reconstruction_calls(golden):
    """Every cp_to_* / tucker_to_* call of the reference's own tests
    (tensorly/tests/test_cp_tensor.py, test_tucker_tensor.py) gives the
    reference's output bit for bit."""
    n = 0
    for rec in golden["recon"]:
        fn = RFN.get(rec["fn"])
        if fn is None:
            continue
        out = fn(*rec["args"], **rec["kwargs"])
        np.testing.assert_array_equal(np.asarray(out), np.asarray(rec["result"]))
        n += 1
    assert n >= 20
    assert sum(1 for r in golden["recon"] if r["fn"] == "__test__") == 8


def test_known_answers_hold_for_oracle(golden):
    """The reference tests' hard-coded answers (assert_array_equal operands
    that are constants) agree with the oracle's outputs recorded above."""
    checked = 0
    recs = golden["kats"]
    for i, rec in enumerate(recs):
        if rec["fn"] != "assert_array_equal":
            continue
        a, b = (np.asarray(v) for v in rec["args"][:2])
        if a.shape == b.shape and a.size:
            np.testing.assert_array_equal(a, b)
            checked += 1
    assert checked >= 5


@pytest.mark.parametrize("case", [
    "dense_cp_small", "normalize", "l2_reg", "fixed_mode0", "rec_error_crit", "svd_init",
    "svd_init_short_mode", "fourway", "twoway", "fiveway", "rank1", "f32_small"])
def test_oracle_parafac_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = oracle.parafac(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-12
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    np.testing.assert_allclose(w, run["weights"], rtol=tol, atol=tol)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["nn_mu_random", "nn_mu_svd", "nn_mu_4way_fixed",
                                  "nn_mu_stop", "nn_mu_f32"])
def test_oracle_non_negative_parafac_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = oracle.non_negative_parafac(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-11
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    np.testing.assert_allclose(w, run["weights"], rtol=tol, atol=tol)
    for a, b in zip(f, run["factors"]):
        assert (a >= 0).all()
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["nn_hals_random", "nn_hals_svd", "nn_hals_sparse_fixed",
                                  "nn_hals_stop", "nn_hals_f32", "nn_hals_rank1",
                                  "nn_hals_exact", "nn_hals_modes_02", "nn_hals_normalize"])
def test_oracle_non_negative_parafac_hals_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        (w, f), errs = oracle.non_negative_parafac_hals(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-10
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    nn_modes = kw.get("nn_modes", "all")
    for mode, (a, b) in enumerate(zip(f, run["factors"])):
        if nn_modes == "all" or mode in nn_modes:
            assert (a >= 0).all()
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["rand_random", "rand_svd_tol", "rand_4way", "rand_f32"])
def test_oracle_randomised_parafac_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = oracle.randomised_parafac(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-12
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


def test_oracle_sample_khatri_rao_matches_reference(golden):
    run = golden["runs"]["sample_kr"]
    kw = run["kwargs"]
    kr, ind, ind_kr = oracle.sample_khatri_rao(
        run["factors_in"], kw["n_samples"], skip_matrix=kw["skip_matrix"],
        return_sampled_rows=True, random_state=np.random.RandomState(kw["random_state"]))
    np.testing.assert_array_equal(kr, run["sampled_kr"])
    np.testing.assert_array_equal(ind_kr, run["indices_kr"])
    for a, b in zip(ind, run["indices_list"]):
        np.testing.assert_array_equal(a, b)


CONS_CASES = ["cons_nonneg_svd", "cons_l1_random", "cons_l2sq_list", "cons_l2_dict_fixed",
              "cons_normalize_mixed", "cons_inner", "cons_stop", "cons_f32",
              # the column-wise and sparsity operators (tests/golden/cons_column_runs.pkl)
              "cons_unimodality", "cons_monotonicity", "cons_simplex", "cons_soft_sparsity",
              "cons_normalized_sparsity", "cons_smoothness", "cons_hard_sparsity",
              "cons_columns_mixed"]


@pytest.mark.parametrize("case", CONS_CASES)
def test_oracle_constrained_parafac_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if run["global_seed"] is not None:
        np.random.seed(run["global_seed"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        (w, f), errs = oracle.constrained_parafac(x, rank, return_errors=True, **kw)
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())


@pytest.mark.parametrize("case", ["nnt_svd", "nnt_random", "nnt_stop", "nnt_f32",
                                  "nnt_normalize"])
def test_oracle_non_negative_tucker_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (core, factors), errs = oracle.non_negative_tucker(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-10
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    np.testing.assert_allclose(core, run["core"], rtol=tol, atol=tol * np.abs(run["core"]).max())
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["nnth_svd", "nnth_random", "nnth_sparse", "nnth_f32",
                                  "nnth_active_set", "nnth_active_set_4way", "nnth_normalize",
                                  "nnth_active_set_normalize", "nnth_active_set_f32",
                                  "nnth_active_set_stop"])
def test_oracle_non_negative_tucker_hals_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (core, factors), errs = oracle.non_negative_tucker_hals(x, rank, return_errors=True, **kw)
    tol = 1e-5 if x.dtype == np.float32 else 1e-10
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    np.testing.assert_allclose(core, run["core"], rtol=tol, atol=tol * np.abs(run["core"]).max())
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["p2_random", "p2_svd", "p2_nols", "p2_normalize", "p2_f32",
                                  "p2_nn_all", "p2_nn_02", "p2_mask", "p2_mask_svd"])
def test_oracle_parafac2_matches_reference(golden, case):
    from oracle import parafac2_oracle
    run = golden["runs"][case]
    xs = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if "mask_keep" in run["gen"]:
        kw["mask"] = slice_masks(run["gen"])
    (w, f, p), errs = parafac2_oracle.parafac2(xs, rank, return_errors=True, **kw)
    tol = 1e-4 if xs[0].dtype == np.float32 else 1e-9
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=tol, atol=tol * 1e-2)
    np.testing.assert_allclose(w, run["weights"], rtol=tol, atol=tol)
    for a, b in zip(list(f) + list(p), run["factors"] + run["projections"]):
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("case", ["cp_linesearch", "cp_orth", "cp_sparsity", "cp_mask",
                                  "cp_mask_linesearch"])
def test_oracle_parafac_branches_match_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if run["mask_keep"] is not None:
        shape = run["gen"]["shape"]
        kw["mask"] = (np.random.RandomState(run["gen"]["seed"] + 1000).rand(*shape)
                      < run["mask_keep"]).astype(x.dtype)
    out, errs = oracle.parafac(x, rank, return_errors=True, **kw)
    if "sparse" in run:
        (w, f), sparse = out
        np.testing.assert_allclose(sparse, run["sparse"], rtol=1e-10, atol=1e-12)
    else:
        w, f = out
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(w, run["weights"], rtol=1e-10, atol=1e-12)
    for a, b in zip(f, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())


@pytest.mark.parametrize("case", ["tucker_svd", "tucker_random", "tucker_4way"])
def test_oracle_tucker_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    (core, factors), errs = oracle.tucker(x, return_errors=True, **run["kwargs"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(core, run["core"], rtol=1e-9, atol=1e-10)
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("case", ["tucker_mask", "tucker_mask_4way"])
def test_oracle_masked_tucker_matches_reference(golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    g = run["gen"]
    mask = (np.random.RandomState(g["seed"] + 1000).rand(*g["shape"])
            < run["mask_keep"]).astype(x.dtype)
    (core, factors), errs = oracle.tucker(x, return_errors=True, mask=mask, **run["kwargs"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(core, run["core"], rtol=1e-9, atol=1e-10)
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("case", ["svd_wide", "svd_tall"])
def test_oracle_svd_interface_matches_reference(golden, case):
    run = golden["runs"][case]
    m = regenerate(run)
    U, S, V = oracle.svd_interface(m, n_eigenvecs=run["kwargs"]["n_eigenvecs"])
    np.testing.assert_allclose(U, run["U"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(S, run["S"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(V, run["V"], rtol=1e-12, atol=1e-12)


def test_oracle_cp_helpers():
    rs = np.random.RandomState(0)
    fs = [rs.randn(s, 3) for s in (4, 5, 6)]
    w = rs.rand(3) + 0.5
    full = oracle.cp_to_tensor((w, fs))
    assert np.isclose(oracle.cp_norm((w, fs)), np.linalg.norm(full))
    w2, f2 = oracle.cp_normalize((w, fs))
    np.testing.assert_allclose(oracle.cp_to_tensor((w2, f2)), full, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose([np.linalg.norm(f, axis=0) for f in f2], 1.0)


def test_oracle_tucker_kats_match_reference(golden):
    """tucker_normalize, kronecker and active_set_nnls of the oracle against
    the reference's outputs on the recorded inputs."""
    seen = set()
    for k in golden["tucker_kats"]:
        seen.add(k["op"])
        if k["op"] == "tucker_normalize":
            c, f = oracle.tucker_normalize((k["core"], k["factors"]))
            np.testing.assert_allclose(c, k["out_core"], rtol=1e-13, atol=1e-13)
            for a, b in zip(f, k["out_factors"]):
                np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13)
        elif k["op"] == "kronecker":
            np.testing.assert_array_equal(oracle.kronecker(k["matrices"]), k["out"])
            ms = [m for i, m in enumerate(k["matrices"]) if i != 1][::-1]
            np.testing.assert_array_equal(oracle.kronecker(ms), k["out_skip1_rev"])
        elif k["op"] == "active_set_nnls":
            x0 = None if k["x0"] is None else k["x0"].copy()
            out = oracle.active_set_nnls(k["Utm"], k["UtU"], x=x0, n_iter_max=100)
            np.testing.assert_allclose(out, k["out"], rtol=1e-10,
                                       atol=1e-10 * np.abs(k["out"]).max())
    assert seen == {"tucker_normalize", "kronecker", "active_set_nnls"}


def test_fixed_modes_error_matches_reference(golden):
    """non_negative_tucker_hals with fixed modes: the reference's first
    misaligned mode_dot, reproduced by walking the shapes on the host."""
    from tensorly_gb300.decomposition import _tucker_fixed_modes_error
    assert golden["fixed_mode_errors"]
    for e in golden["fixed_mode_errors"]:
        err = _tucker_fixed_modes_error(e["shape"], e["rank"], e["fixed"], e["init"])
        assert e["message"] is not None
        assert isinstance(err, ValueError) and str(err) == e["message"]


def test_oracle_svd_kats_match_reference(golden):
    """svd_interface with a mask and with 'randomized_svd', and
    randomized_svd itself, against the reference on the recorded inputs."""
    for k in golden["svd_kats"]:
        if k["op"] == "svd_interface":
            U, S, V = oracle.svd_interface(k["matrix"], mask=k["mask"],
                                           n_iter_mask_imputation=k["n_iter_mask_imputation"],
                                           **k["kwargs"])
        else:
            U, S, V = oracle.randomized_svd(k["matrix"], random_state=k["random_state"],
                                            **k["kwargs"])
        np.testing.assert_allclose(S, k["S"], rtol=1e-11)
        np.testing.assert_allclose(U, k["U"], rtol=1e-9, atol=1e-10)
        np.testing.assert_allclose(V, k["V"], rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("case", ["tucker_mask_svd", "tucker_mask_random", "tucker_randomized",
                                  "cp_randomized", "cp_mask_svd"])
def test_oracle_svd_callers_match_reference(golden, case):
    from golden_inputs import dense_mask
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if "mask_keep" in run["gen"]:
        kw["mask"] = dense_mask(run["gen"])
    if run["np_seed"] is not None:
        np.random.seed(run["np_seed"])
    if run["fn"] == "tucker":
        (core, factors), errs = oracle.tucker(x, rank, return_errors=True, **kw)
        np.testing.assert_allclose(core, run["core"], rtol=1e-9,
                                   atol=1e-9 * np.abs(run["core"]).max())
    else:
        (w, factors), errs = oracle.parafac(x, rank, return_errors=True, **kw)
        np.testing.assert_allclose(w, run["weights"], rtol=1e-9)
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-13)
    for a, b in zip(factors, run["factors"]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())
