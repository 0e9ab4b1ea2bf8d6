"""GPU CP-ALS parity against the reference runs (tests/golden) and the oracle.

Tolerances: the f64 path must match the reference NumPy backend to 1e-10
relative (factors, weights, error list) with the same number of sweeps; f32
inputs are compared with 1e-4 relative on the errors and factors.
"""

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu

F64_CASES = ["dense_cp_small", "normalize", "l2_reg", "fixed_mode0", "rec_error_crit",
             "fourway", "twoway", "fiveway", "rank1"]


def host(t):
    return t.detach().cpu().numpy()


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300)


def run_case(gb300, run, **extra):
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    xt = torch.as_tensor(x, device="cuda")
    return gb300.parafac(xt, rank, return_errors=True, **kw, **extra)


@pytest.mark.parametrize("case", F64_CASES)
def test_parafac_f64_parity(gb300, golden, case):
    run = golden["runs"][case]
    (w, f), errs = run_case(gb300, run)
    assert len(errs) == len(run["errors"]), "different number of sweeps"
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-13)
    assert rel(host(w), run["weights"]) < 1e-10
    for a, b in zip(f, run["factors"]):
        assert rel(host(a), b) < 1e-10


def test_parafac_f32_against_f64_oracle(gb300, golden):
    """f32 tensor: the library keeps Grams, solves and the fit in f64, so it is
    compared with the f64 oracle run on the same f32 bytes and the same
    (f32-rounded) initial factors: errors within 2e-6 absolute, factors 1e-4.
    The reference's own f32 error list carries f32 cancellation noise in
    ||X||^2 + ||rec||^2 - 2<X, rec> (about 1e-3 relative here), so it is
    checked only to 2e-3."""
    run = golden["runs"]["f32_small"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = gb300.parafac(torch.as_tensor(x, device="cuda"), rank, return_errors=True, **kw)
    _, init = oracle.random_cp(x.shape, rank, random_state=kw["random_state"], dtype=np.float32)
    (ow, of), oerrs = oracle.parafac(x.astype(np.float64), rank, init=(None, [
        i.astype(np.float64) for i in init]), n_iter_max=kw["n_iter_max"], tol=0,
        return_errors=True)
    assert len(errs) == len(oerrs) == len(run["errors"])
    np.testing.assert_allclose(errs, oerrs, rtol=0, atol=2e-6)
    for a, b in zip(f, of):
        assert rel(host(a), b) < 1e-4
    np.testing.assert_allclose(errs, run["errors"], rtol=2e-3)


def test_graph_and_check_every_do_not_change_results(gb300, golden):
    run = golden["runs"]["dense_cp_small"]
    (w0, f0), e0 = run_case(gb300, run, use_graph=True, check_every=8)
    (w1, f1), e1 = run_case(gb300, run, use_graph=False, check_every=1)
    (w2, f2), e2 = run_case(gb300, run, use_graph=True, check_every=3)
    assert e0 == e1 == e2
    for a, b, c in zip(f0, f1, f2):
        assert torch.equal(a, b) and torch.equal(a, c)


@pytest.mark.parametrize("precision", ["native", "bf16"])
def test_deferred_fit_and_lookahead_stop_like_one_sweep_at_a_time(gb300, precision):
    """A converging run (tol > 0) launched a group ahead of the host, with the
    last mode's fit deferred to the side stream (the defaults), stops at the
    same sweep and returns the same bits as sweeps run one at a time with the
    fit in line, and as graph replay; with small and large groups."""
    from tensorly_gb300 import _lib
    lib = _lib.lib()
    rs = np.random.RandomState(11)
    fs = [rs.rand(d, 6) for d in (48, 40, 32)]
    x = torch.as_tensor(np.einsum("ir,jr,kr->ijk", *fs) + 0.01 * rs.randn(48, 40, 32),
                        dtype=torch.float32, device="cuda")
    # a start near the generating factors: the error change falls below tol
    # after about 14 sweeps (f64 oracle)
    init = [torch.as_tensor(f * (1 + 0.3 * rs.randn(*f.shape)), dtype=torch.float32,
                            device="cuda") for f in fs]
    kw = dict(n_iter_max=60, tol=1e-5, precision=precision, return_errors=True)

    def run(**extra):
        (w, f), e = gb300.parafac(x, 6, init=gb300.CPTensor((None, [a.clone() for a in init])),
                                  **kw, **extra)
        return w, f, e

    try:
        lib.tlgb_set_tuning(b"cp_inline_fit", 1)
        w0, f0, e0 = run(use_graph=False, check_every=1)
    finally:
        lib.tlgb_set_tuning(b"cp_inline_fit", 0)
    assert len(e0) < 60, "the case must converge before n_iter_max"
    for extra in (dict(), dict(check_every=3), dict(check_every=64),
                  dict(use_graph=True, check_every=8)):
        w1, f1, e1 = run(**extra)
        assert e1 == e0, extra
        assert torch.equal(w1, w0)
        for a, b in zip(f1, f0):
            assert torch.equal(a, b), extra


def test_callback_semantics(gb300, golden):
    run = golden["runs"]["dense_cp_small"]
    seen = []

    def cb(cp, err):
        seen.append(err)
        assert len(cp.factors) == 3
        return len(seen) == 4  # initial call + 3 sweeps, then stop

    (w, f), errs = run_case(gb300, run, callback=cb)
    assert len(errs) == 3
    np.testing.assert_allclose(seen[1:], errs, rtol=0, atol=0)
    np.testing.assert_allclose(errs, run["errors"][:3], rtol=1e-10)
    x = regenerate(run)
    init = run["init_factors"]
    e0 = np.linalg.norm(x - oracle.cp_to_tensor((None, init))) / np.linalg.norm(x)
    assert abs(seen[0] - e0) < 1e-10


def test_callback_exception_propagates(gb300, golden):
    run = golden["runs"]["dense_cp_small"]

    def cb(cp, err):
        raise KeyError("boom")

    with pytest.raises(KeyError):
        run_case(gb300, run, callback=cb)


def test_all_modes_fixed_returns_init(gb300, golden):
    run = golden["runs"]["dense_cp_small"]
    x = torch.as_tensor(regenerate(run), device="cuda")
    cp = gb300.parafac(x, 8, init="random", random_state=0, fixed_modes=[0, 1, 2])
    for a, b in zip(cp.factors, run["init_factors"]):
        np.testing.assert_array_equal(host(a), b)


def test_host_input_returns_host_output(gb300, golden):
    run = golden["runs"]["dense_cp_small"]
    x = regenerate(run)
    cp, errs = gb300.parafac(x, 8, init="random", random_state=0, tol=1e-8, return_errors=True)
    assert isinstance(cp.factors[0], np.ndarray)
    assert rel(cp.factors[0], run["factors"][0]) < 1e-10


def test_cp_estimator(gb300, golden):
    run = golden["runs"]["dense_cp_small"]
    x = torch.as_tensor(regenerate(run), device="cuda")
    est = gb300.CP(8, init="random", random_state=0, tol=1e-8)
    cp = est.fit_transform(x)
    assert len(est.errors_) == len(run["errors"])
    assert rel(host(cp.factors[2]), run["factors"][2]) < 1e-10
    assert repr(est) == "CP decomposition of rank 8."


@pytest.mark.parametrize("case", ["cp_linesearch", "cp_orth"])
def test_parafac_linesearch_and_orthogonalise_match_reference(gb300, golden, case):
    """The line search (tensorly/decomposition/_cp.py:398-401, :447-478) and the
    QR orthogonalisation of the first sweeps (:392-397), f64, against the
    reference's runs: same error list (line-search iterations record none),
    weights and factors to 1e-10."""
    run = golden["runs"][case]
    (w, f), errs = run_case(gb300, run)
    assert len(errs) == len(run["errors"]), "different number of recorded errors"
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-13)
    assert rel(host(w), run["weights"]) < 1e-10
    for a, b in zip(f, run["factors"]):
        assert rel(host(a), b) < 1e-10


@pytest.mark.parametrize("case", ["cp_mask", "cp_mask_linesearch"])
def test_masked_parafac_matches_reference(gb300, golden, case):
    """Missing entries refilled from the model after every sweep
    (tensorly/decomposition/_cp.py:194-207, :441-446), with and without the
    line search, f64, against the reference's runs to 1e-10."""
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    shape = run["gen"]["shape"]
    mask = (np.random.RandomState(run["gen"]["seed"] + 1000).rand(*shape)
            < run["mask_keep"]).astype(x.dtype)
    xt = torch.as_tensor(x, device="cuda")
    (w, f), errs = gb300.parafac(xt, rank, mask=torch.as_tensor(mask, device="cuda"),
                                 return_errors=True, **kw)
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-13)
    assert rel(host(w), run["weights"]) < 1e-10
    for a, b in zip(f, run["factors"]):
        assert rel(host(a), b) < 1e-10
    assert torch.equal(xt, torch.as_tensor(x, device="cuda")), "the input tensor was modified"


def test_parafac_sparse_component_matches_reference(gb300, golden):
    """The sparse component (tensorly/decomposition/_cp.py:140-159, :202-215,
    :532-538): every error is that of the residual minus its largest entries
    (radix select on the device), and the final sparse component comes back
    beside the model; f64 against the reference's run to 1e-10."""
    run = golden["runs"]["cp_sparsity"]
    (cp, sparse), errs = run_case(gb300, run)
    w, f = cp
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-10, atol=1e-13)
    assert rel(host(w), run["weights"]) < 1e-10
    for a, b in zip(f, run["factors"]):
        assert rel(host(a), b) < 1e-10
    s = host(sparse)
    assert (s != 0).sum() == (run["sparse"] != 0).sum()
    np.testing.assert_allclose(s, run["sparse"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sparse_residual_selects_like_sort(gb300, dtype):
    """tlgb_sparse_residual against NumPy's sort on ties, a count above the
    size and the negative counts sparsify_tensor's indexing allows."""
    from tensorly_gb300 import _lib
    from tensorly_gb300._tensor import dtype_code, workspace
    rs = np.random.RandomState(9)
    x = rs.randn(3000)
    x[::7] = 0.5                    # ties at one magnitude
    x[5::11] = -0.5
    lm = rs.randn(3000) * 0.01
    xt = torch.as_tensor(x, device="cuda", dtype=dtype)
    lt = torch.as_tensor(lm, device="cuda", dtype=dtype)
    r = (xt - lt).cpu().numpy().astype(np.float64)
    lib = _lib.lib()
    ws = workspace(int(lib.tlgb_sparse_residual_workspace_bytes()), xt.device)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for k in (1, 17, 429, 1500, 2999, 3000, 3001):
        sp = torch.empty_like(xt)
        _lib.check(lib.tlgb_sparse_residual(dtype_code(xt), xt.data_ptr(), lt.data_ptr(), 3000, k,
                                            out.data_ptr(), sp.data_ptr(), ws.data_ptr(),
                                            ws.numel(), None))
        torch.cuda.synchronize()
        if k > 3000:
            want = r
        else:
            bound = np.sort(np.abs(r))[-k]
            want = np.where(np.abs(r) < bound, 0.0, r)
        np.testing.assert_array_equal(host(sp).astype(np.float64), want)
        ref = np.linalg.norm(r - want)
        assert abs(out.item() - ref) <= 1e-12 * max(ref, 1.0)


def test_unsupported_options_raise(gb300):
    x = torch.rand(4, 5, 6, device="cuda", dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        gb300.parafac(x, 2, init="random", sparsity=0.1, callback=lambda *a: None)
    for kw in ({"linesearch": True}, {"orthogonalise": True}, {"mask": torch.ones_like(x)},
               {"sparsity": 0.1}):
        with pytest.raises(NotImplementedError):
            gb300.parafac(x.float(), 2, init="random", precision="bf16", **kw)
    with pytest.raises(ValueError):
        gb300.parafac(x, 2, init="bogus")
    with pytest.raises(TypeError):
        gb300.parafac(x, 2, init="random", cvg_criterion="nope")


def test_cp_norm_and_normalize(gb300):
    rs = np.random.RandomState(5)
    fs = [rs.randn(s, 4) for s in (6, 7, 8)]
    w = rs.rand(4) + 0.5
    cp = gb300.CPTensor((torch.as_tensor(w, device="cuda"),
                         [torch.as_tensor(f, device="cuda") for f in fs]))
    assert abs(float(gb300.cp_norm(cp)) - oracle.cp_norm((w, fs))) < 1e-12 * oracle.cp_norm((w, fs))
    w2, f2 = gb300.cp_normalize(cp)
    ow, of = oracle.cp_normalize((w, fs))
    np.testing.assert_allclose(host(w2), ow, rtol=1e-13)
    for a, b in zip(f2, of):
        np.testing.assert_allclose(host(a), b, rtol=1e-13, atol=1e-15)
    full = gb300.cp_to_tensor(cp)
    np.testing.assert_allclose(host(full), oracle.cp_to_tensor((w, fs)), rtol=1e-12, atol=1e-12)


def test_parafac_deterministic(gb300):
    rs = np.random.RandomState(7)
    x = torch.as_tensor(rs.randn(40, 36, 44).astype(np.float32), device="cuda")
    a, ea = gb300.parafac(x, 6, init="random", random_state=1, n_iter_max=10, tol=0,
                          return_errors=True)
    b, eb = gb300.parafac(x, 6, init="random", random_state=1, n_iter_max=10, tol=0,
                          return_errors=True)
    assert ea == eb
    for u, v in zip(a.factors, b.factors):
        assert torch.equal(u, v)


def test_ill_conditioned_normal_equations_use_f64_fallback(gb300):
    """Nearly collinear initial components make V ill-conditioned (pivot
    spread > 1e5): the library factorises in f64 (Cholesky, LU if needed)
    instead of refining from an f32 inverse; the first sweeps still match the
    NumPy reference (LAPACK gesv) to the accuracy the conditioning allows."""
    rs = np.random.RandomState(11)
    shape, rank = (20, 18, 16), 4
    fs = [rs.uniform(size=(s, rank)) for s in shape]
    x = oracle.cp_to_tensor((None, fs)) + 0.01 * rs.randn(*shape)
    init = [rs.uniform(size=(s, rank)) for s in shape]
    for f in init:
        f[:, 1] = f[:, 0] * (1 + 1e-4 * rs.randn(f.shape[0]))
    (ow, of), oe = oracle.parafac(x, rank, init=(None, [f.copy() for f in init]), n_iter_max=3,
                                  tol=0, return_errors=True)
    xt = torch.as_tensor(x, device="cuda")
    cp, errs = gb300.parafac(xt, rank, init=gb300.CPTensor((None, [torch.as_tensor(f, device="cuda")
                                                                  for f in init])),
                             n_iter_max=3, tol=0, return_errors=True)
    np.testing.assert_allclose(errs, oe, rtol=1e-6)
    for a, b in zip(cp.factors, of):
        assert rel(host(a), b) < 1e-4


@pytest.mark.parametrize("shape,rank,precision", [
    ((53, 59, 22), 9, "native"), ((12, 45, 43), 5, "native"), ((30, 31, 29), 7, "native"),
    ((40, 33, 35), 1, "native"), ((48, 40, 36), 11, "bf16"), ((64, 48, 40), 3, "bf16")])
def test_parafac_f32_odd_ranks_match_f64_oracle(gb300, shape, rank, precision):
    """Odd ranks (R * R odd) through the f32 normal-equation solve: same final
    error as the f64 oracle from the same random initial factors."""
    rs = np.random.RandomState(rank)
    A = [rs.rand(d, rank) for d in shape]
    x = (oracle.cp_to_tensor((None, A)) + 0.01 * rs.randn(*shape)).astype(np.float32)
    init = oracle.random_cp(shape, rank, random_state=7, dtype=np.float64)[1]
    # bf16 sweeps take a different path to the optimum: compare once converged
    n_iter = 25 if precision == "native" else 120
    (_, f), errs = gb300.parafac(torch.as_tensor(x, device="cuda"), rank, n_iter_max=n_iter,
                                 init=(None, [torch.as_tensor(a.astype(np.float32), device="cuda")
                                              for a in init]),
                                 tol=0, return_errors=True, precision=precision)
    x64 = x.astype(np.float64)
    _, f64, _ = oracle.parafac_sweeps(x64, np.ones(rank), init, n_iter)
    e64 = np.linalg.norm(x64 - oracle.cp_to_tensor((None, f64))) / np.linalg.norm(x64)
    e = np.linalg.norm(x64 - oracle.cp_to_tensor((None, [host(t).astype(np.float64) for t in f]))) \
        / np.linalg.norm(x64)
    assert abs(e - e64) / e64 < 1e-3, (e, e64)


@pytest.mark.parametrize("dtype,rank", [
    (np.float64, 130), (np.float64, 100), (np.float64, 70), (np.float64, 40),
    (np.float32, 90), (np.float32, 120), (np.float32, 50), (np.float32, 20)])
def test_parafac_wide_ranks_match_oracle(gb300, dtype, rank):
    """Every padded order of the blocked Gauss-Jordan inverse (32, 64, 96 and
    160) and both builds of V (double-float from the Grams' f32 planes for
    f32 factors up to rank 96, f64 otherwise), three sweeps from the same
    initial factors as the f64 oracle: f64 errors to 1e-9 and factors to
    1e-7, f32 errors to 2e-6 absolute and factors to 1e-3."""
    rs = np.random.RandomState(rank)
    shape = (24, 22, 20)
    x = rs.rand(*shape).astype(dtype)
    init = [rs.rand(d, rank).astype(dtype) for d in shape]
    (_, f), errs = gb300.parafac(torch.as_tensor(x, device="cuda"), rank, n_iter_max=3, tol=0,
                                 init=(None, [torch.as_tensor(a, device="cuda") for a in init]),
                                 return_errors=True)
    x64 = x.astype(np.float64)
    _, of, oerrs = oracle.parafac_sweeps(x64, np.ones(rank), [a.astype(np.float64) for a in init],
                                         3)
    if dtype == np.float64:
        np.testing.assert_allclose(errs, oerrs, rtol=1e-9)
        for a, b in zip(f, of):
            assert rel(host(a), b) < 1e-7
    else:
        np.testing.assert_allclose(errs, oerrs, rtol=0, atol=2e-6)
        for a, b in zip(f, of):
            assert rel(host(a), b) < 1e-3
