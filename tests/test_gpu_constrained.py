"""Constrained CP by AO-ADMM on the GPU
(tensorly/decomposition/_constrained_cp.py:166-612, tensorly/solvers/admm.py,
tensorly/tenalg/proximal.py) against the reference runs (tests/golden) and the
NumPy oracle.

Tolerances: f64 runs 1e-8 on the error list and 1e-6 (of the largest entry)
on the factors; the f32 run 1e-3 and 1e-2 (the reference's dual variables are
float64, so its f32 run is promoted to f64 after the first update while the
GPU stays in f32); proximal operators 1e-12 (f64) / 1e-6 (f32)."""

import warnings

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu

CASES = ["cons_nonneg_svd", "cons_l1_random", "cons_l2sq_list", "cons_l2_dict_fixed",
         "cons_normalize_mixed", "cons_inner", "cons_stop", "cons_f32"]


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("case", CASES)
def test_constrained_parafac_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if run["global_seed"] is not None:
        np.random.seed(run["global_seed"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        (w, f), errs = gb300.constrained_parafac(torch.as_tensor(x, device="cuda"), rank,
                                                 return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-8)
    for a, b in zip(f, run["factors"]):
        tol = 1e-2 if f32 else 1e-6
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cons", [dict(non_negative=True), dict(l1_reg=0.3), dict(l2_reg=2.0),
                                  dict(l2_reg=1e6), dict(l2_square_reg=0.25),
                                  dict(normalize=True)])
def test_proximal_operators_match_oracle(gb300, dtype, cons):
    rs = np.random.RandomState(3)
    y = rs.randn(37, 5).astype(dtype)
    out = host(gb300.proximal_operator(torch.as_tensor(y, device="cuda"), n_const=1, order=0,
                                       **cons))
    ref = oracle.proximal_operator(y, n_const=1, order=0, **cons)
    tol = 1e-12 if dtype == np.float64 else 1e-6
    np.testing.assert_allclose(out, ref, rtol=tol, atol=tol * max(np.abs(ref).max(), 1e-30))


def test_proximal_edge_cases_and_constraint_parsing(gb300):
    # the reference clips to [0, max]: an all-negative matrix becomes its max
    y = -np.abs(np.random.RandomState(1).randn(6, 3)) - 0.1
    out = host(gb300.proximal_operator(y, non_negative=True))
    np.testing.assert_array_equal(out, oracle.proximal_operator(y, non_negative=True))
    assert isinstance(out, np.ndarray)
    # a dict constrains only its modes; a list gives every mode the constraint
    assert gb300.validate_constraints(l1_reg={1: 0.2}, n_const=3, order=0) == (None, None)
    assert gb300.validate_constraints(l1_reg={1: 0.2}, n_const=3, order=1) == ("l1_reg", 0.2)
    assert gb300.validate_constraints(non_negative=[True, False, True], n_const=3, order=1) \
        == ("non_negative", False)
    with pytest.raises(ValueError):
        gb300.validate_constraints(non_negative=True, l1_reg={0: 0.1}, n_const=2, order=0)
    x = torch.rand(6, 5, 4, device="cuda", dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        gb300.constrained_parafac(x, 2, simplex=1.0)
    with pytest.raises(NotImplementedError):
        gb300.constrained_parafac(x, 2, monotonicity=True)


def test_constrained_wrapper_and_host_input(gb300, golden):
    run = golden["runs"]["cons_nonneg_svd"]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    est = gb300.ConstrainedCP(rank, **kw)
    cp = est.fit_transform(x)
    assert isinstance(cp.factors[0], np.ndarray)
    np.testing.assert_allclose(est.errors_, run["errors"], rtol=1e-8)
    assert all((f >= 0).all() for f in cp.factors)
