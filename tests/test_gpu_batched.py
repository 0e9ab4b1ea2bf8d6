"""Batched CP-ALS (one persistent kernel for many small uneven tensors)
against per-tensor f64 oracle runs from the same initial factors."""

import numpy as np
import pytest
import torch

import oracle
from tensorly_gb300 import workloads

pytestmark = pytest.mark.gpu


def _oracle_run(x, rank, seed, n_iter):
    init = oracle.random_cp(x.shape, rank, random_state=seed, dtype=np.float64)[1]
    x64 = x.astype(np.float64)
    w, f, errs = oracle.parafac_sweeps(x64, np.ones(rank), init, n_iter)
    rec = oracle.cp_to_tensor((None, f))
    final = np.linalg.norm(x64 - rec) / np.linalg.norm(x64)
    return f, errs, final


def test_batched_matches_f64_oracle(gb300):
    batch = workloads.batched_uneven(count=24, seed=3)
    xs = [b[0] for b in batch]
    ranks = [b[1] for b in batch]
    seeds = [b[2] for b in batch]
    cps, final, sweeps = gb300.parafac_batched(xs, ranks, n_iter_max=30, random_state=seeds,
                                               return_errors=True, sweep_errors=True)
    assert len(cps) == 24 and final.shape == (24,) and sweeps.shape == (24, 30)
    rel = []
    for t, (x, r, s) in enumerate(batch):
        f64, errs64, final64 = _oracle_run(x, r, s, 30)
        rel.append(abs(final[t] - final64) / final64)
        # the per-sweep expansion in f64 from f32 pieces tracks the oracle's errors
        np.testing.assert_allclose(sweeps[t], errs64, rtol=5e-2, atol=1e-4)
    rel = np.array(rel)
    assert np.median(rel) < 1e-4, rel
    assert (rel < 1e-2).all(), rel


def test_batched_global_path_and_launch_split(gb300):
    # 64^3 tensors do not fit in shared memory (global-memory path); a run
    # split into launches of 7 sweeps equals the single-launch run bitwise
    rs = np.random.RandomState(4)
    xs, ranks = [], []
    for dims, r in (((64, 64, 64), 16), ((40, 20, 64), 5), ((8, 9, 10), 4), ((64, 8, 64), 11)):
        fs = [rs.randn(d, r) for d in dims]
        x = oracle.cp_to_tensor((None, fs))
        x = (x + 0.01 * np.linalg.norm(x) * rs.randn(*dims) / np.sqrt(x.size)).astype(np.float32)
        xs.append(x)
        ranks.append(r)
    a, fa = gb300.parafac_batched(xs, ranks, n_iter_max=20, random_state=[1, 2, 3, 4],
                                  return_errors=True)
    b, fb = gb300.parafac_batched(xs, ranks, n_iter_max=20, random_state=[1, 2, 3, 4],
                                  return_errors=True, sweeps_per_launch=7)
    np.testing.assert_array_equal(fa, fb)
    for ca, cb in zip(a, b):
        for u, v in zip(ca.factors, cb.factors):
            np.testing.assert_array_equal(u, v)
    for t, (x, r) in enumerate(zip(xs, ranks)):
        _, _, final64 = _oracle_run(x, r, t + 1, 20)
        assert abs(fa[t] - final64) / final64 < 1e-2


def test_batched_deterministic_and_cuda_inputs(gb300):
    batch = workloads.batched_uneven(count=10, seed=5)
    xs = [torch.as_tensor(b[0], device="cuda") for b in batch]
    ranks = [b[1] for b in batch]
    r1 = gb300.parafac_batched(xs, ranks, n_iter_max=15, random_state=0)
    r2 = gb300.parafac_batched(xs, ranks, n_iter_max=15, random_state=0)
    for c1, c2 in zip(r1, r2):
        assert c1.factors[0].is_cuda
        for u, v in zip(c1.factors, c2.factors):
            assert torch.equal(u, v)


def test_batched_rejects_out_of_range(gb300):
    x = np.zeros((65, 4, 4), dtype=np.float32)
    with pytest.raises(NotImplementedError):
        gb300.parafac_batched([x], [3], n_iter_max=2)
    y = np.zeros((8, 8, 8), dtype=np.float32)
    with pytest.raises(NotImplementedError):
        gb300.parafac_batched([y], [17], n_iter_max=2)


def test_autotuner_picks_a_variant_and_variants_agree(gb300):
    from tensorly_gb300 import autotune
    from tensorly_gb300.decomposition import BatchedProblem
    batch = workloads.batched_uneven(count=40, seed=9)
    prob = BatchedProblem([b[0] for b in batch], [b[1] for b in batch],
                          random_state=[b[2] for b in batch])
    finals = []
    try:
        for nt in autotune.VARIANTS:
            for cls in autotune.CLASSES:
                autotune._set(cls, nt)
            finals.append(prob.run(12).final.cpu().numpy())
        for cls in autotune.CLASSES:
            autotune._set(cls, 256)
        for ot in autotune.OUTER_TILES[1:]:      # the MTTKRP's outer-slice tiles
            for cls in autotune.CLASSES:
                autotune._set_tile(cls, ot)
            finals.append(prob.run(12).final.cpu().numpy())
        choice, tiles = autotune.tune_batched(prob, sweeps=2, reps=1)
        assert set(choice) == set(autotune.CLASSES) == set(tiles)
        assert all(v in autotune.VARIANTS for v in choice.values())
        assert all(v in autotune.OUTER_TILES for v in tiles.values())
        assert autotune.tune_batched(prob) == (choice, tiles)      # cached
    finally:
        autotune.reset_batched()
    for f in finals[1:]:
        # f32 rounding differs between variants; unconverged trajectories drift a little
        np.testing.assert_allclose(f, finals[0], rtol=2e-3)
