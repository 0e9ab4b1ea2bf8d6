"""Parity at the sizes the throughput figures are quoted on.

The other GPU tests tie every function to the oracle and the reference runs on
small shapes.  These tie the library to the oracle on the full workloads:

* 512^3 rank 64 (the headline): two f64 sweeps against the NumPy restatement
  of parafac on the same f64 bytes and initial factors (1e-10 relative), and
  the 50-sweep bf16 run with its 3 closing f32 sweeps against the f64 GPU run
  (final relative error within 1e-4 relative, factor congruence stated);
* 128^4 four-way: two sweeps of rank-32 CP and two HOOI iterations of
  tucker(rank=[16]*4, init='random') in f64 against the oracle (1e-10);
* the 4096-tensor uneven batch: the batched kernel's final errors against
  per-tensor f64 oracle runs from the same initial factors on a sample spread
  over the whole batch.

Tolerances: f64 paths 1e-10 relative (factors, weights, error lists), as in
tensorly/decomposition/tests; bf16 and f32 paths the +-1e-4 relative final
error gate of the mixed-precision metric.
"""

import numpy as np
import pytest
import torch

import oracle
from tensorly_gb300 import workloads

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def congruence(fa, fb):
    """Mean factor congruence after matching components (Hungarian
    assignment on the product over modes of |cosine|)."""
    from scipy.optimize import linear_sum_assignment
    r = fa[0].shape[1]
    c = np.ones((r, r))
    for a, b in zip(fa, fb):
        an = a / np.maximum(np.linalg.norm(a, axis=0), 1e-300)
        bn = b / np.maximum(np.linalg.norm(b, axis=0), 1e-300)
        c *= np.abs(an.T @ bn)
    ri, ci = linear_sum_assignment(-c)
    return float(c[ri, ci].mean())


@pytest.fixture(scope="module")
def c2():
    """The 512^3 rank-64 headline tensor (f32) and the initial factors the
    benchmark uses: RandomState(0).random_sample((512, 64)) per mode."""
    x, _ = workloads.dense_cp_large(size=512, rank=64)
    rs = np.random.RandomState(0)
    init = [rs.random_sample((512, 64)).astype(np.float32) for _ in range(3)]
    return x, init


def test_c2_f64_two_sweeps_match_oracle(gb300, c2):
    x, init = c2
    x64 = x.astype(np.float64)
    init64 = [f.astype(np.float64) for f in init]
    _, f_ref, e_ref = oracle.parafac_sweeps(x64, np.ones(64), init64, 2)
    xt = torch.from_numpy(x64).cuda()
    (w, f), errs = gb300.parafac(xt, 64, init=gb300.CPTensor((None, [torch.from_numpy(a).cuda()
                                                                    for a in init64])),
                                 n_iter_max=2, tol=0, return_errors=True)
    del xt
    assert len(errs) == 2
    np.testing.assert_allclose(errs, e_ref, rtol=1e-10, atol=0)
    assert rel(w.cpu().numpy(), np.ones(64)) < 1e-12
    for a, b in zip(f, f_ref):
        assert rel(a.cpu().numpy(), b) < 1e-10


def test_c2_bf16_50_sweeps_reach_f64_fit(gb300, c2):
    """The 512^3 rank-64 workload, 50 sweeps from the same start: bf16 sweeps
    with one closing f32 sweep (the default) and with three reach the f64
    run's final error and factors."""
    x, init = c2
    xt = torch.from_numpy(x).cuda()
    it = [torch.from_numpy(a).cuda() for a in init]
    runs = {}
    for refine in (1, 3):
        runs[refine] = gb300.parafac(xt, 64, init=gb300.CPTensor((None, [a.clone() for a in it])),
                                     n_iter_max=50, tol=0, precision="bf16",
                                     refine_sweeps=refine, return_errors=True)
    x64 = xt.double()
    del xt
    (w64, f64), errs64 = gb300.parafac(x64, 64, init=gb300.CPTensor((None, [a.double() for a in it])),
                                       n_iter_max=50, tol=0, return_errors=True)
    del x64
    for refine, ((w, f), errs) in runs.items():
        assert len(errs) == len(errs64) == 50
        d = abs(errs[-1] - errs64[-1]) / errs64[-1]
        cong = congruence([a.double().cpu().numpy() for a in f], [a.cpu().numpy() for a in f64])
        print(f"512^3 R64 bf16 + {refine} f32 closing sweep(s): final error {errs[-1]:.10f}, f64 "
              f"{errs64[-1]:.10f}, relative difference {d:.2e}, congruence {cong:.7f}")
        assert d < 1e-4
        assert cong > 0.999


@pytest.fixture(scope="module")
def c3():
    """The 128^4 four-way tensor (CP rank 32 + Tucker 16^4 + 1 % noise) in f64."""
    return workloads.cp_tucker_4way().astype(np.float64)


def test_c3_cp_rank32_two_sweeps_match_oracle(gb300, c3):
    x = c3
    _, init = oracle.random_cp(x.shape, 32, random_state=0, dtype=np.float64)
    _, f_ref, e_ref = oracle.parafac_sweeps(x, np.ones(32), init, 2)
    xt = torch.from_numpy(x).cuda()
    (w, f), errs = gb300.parafac(xt, 32, init="random", random_state=0, n_iter_max=2, tol=0,
                                 return_errors=True)
    del xt
    np.testing.assert_allclose(errs, e_ref, rtol=1e-10, atol=0)
    for a, b in zip(f, f_ref):
        assert rel(a.cpu().numpy(), b) < 1e-10


def test_c3_tucker_two_hooi_iterations_match_oracle(gb300, c3):
    x = c3
    (core_ref, f_ref), e_ref = oracle.tucker(x, rank=[16] * 4, n_iter_max=2, init="random",
                                             tol=0, random_state=0, return_errors=True)
    xt = torch.from_numpy(x).cuda()
    (core, f), errs = gb300.tucker(xt, rank=[16] * 4, n_iter_max=2, init="random", tol=0,
                                   random_state=0, return_errors=True)
    del xt
    assert len(errs) == len(e_ref)
    np.testing.assert_allclose(errs, e_ref, rtol=1e-10, atol=0)
    assert rel(core.cpu().numpy(), core_ref) < 1e-10
    for a, b in zip(f, f_ref):
        assert rel(a.cpu().numpy(), b) < 1e-10


def test_c4_full_batch_matches_f64_oracle_on_a_sample(gb300):
    """All 4096 tensors in the persistent kernel, 100 sweeps; 48 of them,
    spread over the batch, against per-tensor f64 oracle runs."""
    batch = workloads.batched_uneven(count=4096, seed=0)
    xs = [b[0] for b in batch]
    ranks = [b[1] for b in batch]
    seeds = [b[2] for b in batch]
    cps, final = gb300.parafac_batched(xs, ranks, n_iter_max=100, random_state=seeds,
                                       return_errors=True)
    assert len(cps) == 4096 and final.shape == (4096,)
    assert np.isfinite(final).all()
    rel_diff = []
    for t in np.linspace(0, 4095, 48).astype(int):
        x64 = xs[t].astype(np.float64)
        init = oracle.random_cp(x64.shape, ranks[t], random_state=seeds[t], dtype=np.float64)[1]
        _, f64, _ = oracle.parafac_sweeps(x64, np.ones(ranks[t]), init, 100)
        e64 = np.linalg.norm(x64 - oracle.cp_to_tensor((None, f64))) / np.linalg.norm(x64)
        rel_diff.append(abs(final[t] - e64) / e64)
    rel_diff = np.array(rel_diff)
    print(f"4096-tensor batch, 48-tensor sample: final error vs f64 oracle, median "
          f"{np.median(rel_diff):.2e}, max {rel_diff.max():.2e}")
    assert np.median(rel_diff) < 1e-5
    assert (rel_diff < 1e-4).mean() >= 0.9, rel_diff
