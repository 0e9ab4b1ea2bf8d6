"""Regenerates the inputs of the golden reference runs from their seeds."""

import numpy as np

from oracle import cp_to_tensor
from tensorly_gb300 import workloads


def small_cp(seed, shape, rank, dtype=np.float64, noise=0.01):
    rs = np.random.RandomState(seed)
    fs = [rs.uniform(size=(s, rank)) for s in shape]
    t = cp_to_tensor((None, fs))
    n = rs.randn(*shape)
    t = t + noise * np.linalg.norm(t) * n / np.linalg.norm(n)
    return t.astype(dtype)


def slice_masks(g):
    """0/1 masks of PARAFAC2 slices, keeping each entry with probability
    ``g["mask_keep"]`` (seeded by ``g["seed"] + 1000``)."""
    rs = np.random.RandomState(g["seed"] + 1000)
    dtype = g.get("dtype", np.float64)
    return [(rs.rand(r, g["cols"]) < g["mask_keep"]).astype(dtype) for r in g["rows"]]


def regenerate(run):
    g = run["gen"]
    if g["fn"] == "dense_cp_small":
        x, _ = workloads.dense_cp_small()
    elif g["fn"] == "small":
        x = small_cp(g["seed"], g["shape"], g["rank"], g.get("dtype", np.float64))
        if g.get("abs"):
            x = np.abs(x)
    elif g["fn"] == "randn":
        x = np.random.RandomState(g["seed"]).randn(*g["shape"])
    elif g["fn"] == "slices":             # PARAFAC2 input: uniform slices of ragged height
        rs = np.random.RandomState(g["seed"])
        xs = [rs.rand(r, g["cols"]).astype(g.get("dtype", np.float64)) for r in g["rows"]]
        cs = [float(sum(np.asarray(t, np.float64).sum() for t in xs)),
              float(np.sqrt(sum((np.asarray(t, np.float64) ** 2).sum() for t in xs)))]
        np.testing.assert_allclose(cs, run["checksum"], rtol=1e-12, atol=1e-12)
        return xs
    else:
        raise KeyError(g["fn"])
    cs = [float(np.asarray(x, np.float64).sum()), float(np.linalg.norm(np.asarray(x, np.float64)))]
    np.testing.assert_allclose(cs, run["checksum"], rtol=1e-12, atol=1e-12)
    return x


def dense_mask(g):
    """0/1 mask of a dense tensor, keeping each entry with probability
    ``g["mask_keep"]`` (seeded by ``g["seed"] + 1000``)."""
    return (np.random.RandomState(g["seed"] + 1000).rand(*g["shape"])
            < g["mask_keep"]).astype(np.float64)
