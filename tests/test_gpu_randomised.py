"""Randomised CP-ALS and sample_khatri_rao on the GPU
(tensorly/decomposition/_cp.py:546-1004) against the reference runs
(tests/golden) and the NumPy oracle.

The sample indices are drawn on the host with NumPy's RandomState, exactly as
the reference draws them, so a run follows the reference's iterations.
Tolerances: f64 1e-8 on the error list and 1e-6 (of the largest entry) on the
factors, where the sampled normal equations are solved by another method than
LAPACK's gesv; f32 1e-3 and 1e-2; sampled Khatri-Rao rows bit-exact (same
products in the same order)."""

import numpy as np
import pytest
import torch

import oracle
from golden_inputs import regenerate

pytestmark = pytest.mark.gpu


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("case", ["rand_random", "rand_svd_tol", "rand_4way", "rand_f32"])
def test_randomised_parafac_matches_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    (w, f), errs = gb300.randomised_parafac(torch.as_tensor(x, device="cuda"), rank,
                                            return_errors=True, **kw)
    f32 = x.dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-8)
    np.testing.assert_allclose(host(w), run["weights"])
    for a, b in zip(f, run["factors"]):
        tol = 1e-2 if f32 else 1e-6
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


def test_sample_khatri_rao_matches_reference(gb300, golden):
    run = golden["runs"]["sample_kr"]
    kw = run["kwargs"]
    fs = [torch.as_tensor(m, device="cuda") for m in run["factors_in"]]
    kr, ind, ind_kr = gb300.sample_khatri_rao(
        fs, kw["n_samples"], skip_matrix=kw["skip_matrix"], return_sampled_rows=True,
        random_state=np.random.RandomState(kw["random_state"]))
    np.testing.assert_array_equal(host(kr), run["sampled_kr"])
    np.testing.assert_array_equal(ind_kr, run["indices_kr"])
    # host inputs come back on the host; explicit indices; the reference's warning
    kr2, _ = gb300.sample_khatri_rao(run["factors_in"], kw["n_samples"],
                                     skip_matrix=kw["skip_matrix"], indices_list=ind)
    assert isinstance(kr2, np.ndarray)
    np.testing.assert_array_equal(kr2, run["sampled_kr"])
    with pytest.warns(UserWarning):
        gb300.sample_khatri_rao(fs, 3, random_state=0)
    with pytest.raises(IndexError):
        gb300.sample_khatri_rao(fs, 2, indices_list=[np.array([0, 99]), np.array([0, 1]),
                                                     np.array([0, 1])])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_randomised_parafac_matches_oracle_larger(gb300, dtype):
    rs = np.random.RandomState(21)
    shape, rank = (40, 33, 29), 6
    fs = [rs.rand(s, rank) for s in shape]
    x = (oracle.cp_to_tensor((None, fs)) + 0.01 * rs.randn(*shape)).astype(dtype)
    kw = dict(n_samples=200, n_iter_max=12, tol=0, init="random", random_state=4)
    (_, fo), eo = oracle.randomised_parafac(x, rank, return_errors=True, **kw)
    (_, fg), eg = gb300.randomised_parafac(torch.as_tensor(x, device="cuda"), rank,
                                           return_errors=True, **kw)
    f32 = dtype == np.float32
    np.testing.assert_allclose(eg, eo, rtol=1e-3 if f32 else 1e-8)
    for a, b in zip(fg, fo):
        tol = 1e-2 if f32 else 1e-6
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


def test_randomised_parafac_reconstructs_and_wrapper(gb300):
    """The reference's own check (tensorly/decomposition/tests/test_cp.py:482-511):
    a rank-4 10^3 CP tensor, 100 samples, 60 iterations, error below 5 %."""
    rng = np.random.RandomState(1234)
    rng.random_sample((10, 10, 10))
    fs = [rng.random_sample((10, 4)) for _ in range(3)]
    tensor = oracle.cp_to_tensor((None, fs))
    cp = gb300.randomised_parafac(tensor, rank=4, n_samples=100, max_stagnation=20,
                                  n_iter_max=60, tol=0, verbose=0, random_state=rng)
    for i, f in enumerate(cp[1]):
        assert f.shape == (10, 4)
    rec = oracle.cp_to_tensor((None, [host(f) for f in cp.factors]))
    assert np.linalg.norm(rec - tensor) / np.linalg.norm(tensor) < 0.05
    est = gb300.RandomizedCP(rank=3, n_samples=100, n_iter_max=5, random_state=0)
    out = est.fit_transform(tensor)
    assert len(est.errors_) == 5 and out.factors[0].shape == (10, 3)
    seen = []
    gb300.randomised_parafac(tensor, 3, 50, n_iter_max=3, random_state=0,
                             callback=lambda cp, *e: seen.append(len(e)))
    assert seen == [0, 1, 1, 1]
