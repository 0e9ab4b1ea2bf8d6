"""GPU parity of the tenalg primitives against the NumPy oracle and the
reference's own recorded unit-test calls."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def cuda(a, dtype=torch.float64):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device="cuda")


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_khatri_rao_bit_exact(gb300, dtype):
    rs = np.random.RandomState(0)
    npd = np.float32 if dtype == torch.float32 else np.float64
    mats = [rs.randn(s, 5).astype(npd) for s in (3, 7, 4)]
    w = rs.rand(5).astype(npd)
    mask = (rs.rand(3 * 7 * 4) > 0.3).astype(npd)
    for kw in ({}, {"weights": w}, {"skip_matrix": 1}, {"weights": w, "mask": mask}):
        ref = oracle.khatri_rao(mats, **kw)
        got = gb300.khatri_rao([cuda(m, dtype) for m in mats],
                               **{k: (cuda(v, dtype) if isinstance(v, np.ndarray) else v)
                                  for k, v in kw.items()})
        np.testing.assert_array_equal(host(got), ref)


MTTKRP_CASES = [
    ((10, 10, 10, 4), 5), ((17, 9, 23), 3), ((64, 64, 64), 8), ((5, 130), 70),
    ((33, 1, 7), 2), ((4, 5, 3, 6, 4), 2), ((3, 4, 2, 3, 2, 2, 3), 4), ((40, 50, 36), 70),
    ((128, 8, 24), 1), ((7, 6, 5), 33),
]


@pytest.mark.parametrize("shape,rank", MTTKRP_CASES)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_mttkrp_matches_oracle(gb300, shape, rank, dtype):
    rs = np.random.RandomState(sum(shape) + rank)
    x = rs.randn(*shape)
    fs = [rs.randn(s, rank) for s in shape]
    w = rs.rand(rank) + 0.5
    xt = cuda(x, dtype)
    ft = [cuda(f, dtype) for f in fs]
    for mode in range(len(shape)):
        ref = oracle.unfolding_dot_khatri_rao(x, (w if len(shape) > 2 else None, fs), mode)
        got = host(gb300.unfolding_dot_khatri_rao(xt, (cuda(w, dtype), ft), mode)).astype(np.float64)
        scale = np.abs(ref).max() + 1e-30
        tol = 1e-12 if dtype == torch.float64 else 2e-5
        assert np.abs(got - ref).max() <= tol * scale * max(1.0, np.sqrt(np.prod(shape) / shape[mode]) / 8)


def test_mttkrp_deterministic(gb300):
    rs = np.random.RandomState(1)
    x = cuda(rs.randn(48, 40, 56), torch.float32)
    fs = [cuda(rs.randn(s, 16), torch.float32) for s in (48, 40, 56)]
    for mode in range(3):
        a = gb300.unfolding_dot_khatri_rao(x, (None, fs), mode)
        b = gb300.unfolding_dot_khatri_rao(x, (None, fs), mode)
        assert torch.equal(a, b)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_mode_dot_matches_oracle(gb300, dtype):
    rs = np.random.RandomState(2)
    x = rs.randn(6, 7, 5, 9)
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    for mode in range(4):
        for J in (1, 3, 17, 70):
            u = rs.randn(J, x.shape[mode])
            ref = oracle.mode_dot(x, u, mode)
            got = host(gb300.mode_dot(cuda(x, dtype), cuda(u, dtype), mode))
            np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
            ut = rs.randn(x.shape[mode], J)
            ref = oracle.mode_dot(x, ut, mode, transpose=True)
            got = host(gb300.mode_dot(cuda(x, dtype), cuda(ut, dtype), mode, transpose=True))
            np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
        v = rs.randn(x.shape[mode])
        ref = oracle.mode_dot(x, v, mode)
        got = host(gb300.mode_dot(cuda(x, dtype), cuda(v, dtype), mode))
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())


def test_multi_mode_dot_matches_oracle(gb300):
    rs = np.random.RandomState(3)
    x = rs.randn(5, 6, 7, 4)
    us = [rs.randn(3, s) for s in x.shape]
    for skip in (None, 0, 2):
        ref = oracle.multi_mode_dot(x, us, skip=skip)
        got = host(gb300.multi_mode_dot(cuda(x), [cuda(u) for u in us], skip=skip))
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    ut = [rs.randn(s, 2) for s in x.shape]
    ref = oracle.multi_mode_dot(x, ut, transpose=True)
    got = host(gb300.multi_mode_dot(cuda(x), [cuda(u) for u in ut], transpose=True))
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    vs = [np.ones(s) / s for s in x.shape]
    got = gb300.multi_mode_dot(cuda(np.ones(x.shape)), [cuda(v) for v in vs])
    assert tuple(got.shape) == () and abs(float(got) - 1.0) < 1e-12


def test_replays_reference_unit_test_calls(gb300, golden):
    """Every recorded call of the reference's tenalg tests, on float64 CUDA
    tensors: same results (or the same ValueError)."""
    fn = {"khatri_rao": gb300.khatri_rao, "mode_dot": gb300.mode_dot,
          "multi_mode_dot": gb300.multi_mode_dot,
          "unfolding_dot_khatri_rao": gb300.unfolding_dot_khatri_rao}

    def conv(a):
        if isinstance(a, np.ndarray):
            return cuda(a)
        if isinstance(a, (list, tuple)) and a and any(isinstance(v, np.ndarray) for v in a):
            return type(a)(conv(v) for v in a)
        return a

    n = 0
    for rec in golden["kats"]:
        f = fn.get(rec["fn"])
        if f is None:
            continue
        args = [conv(a) for a in rec["args"]]
        kwargs = {k: conv(v) for k, v in rec["kwargs"].items()}
        if "raises" in rec:
            with pytest.raises(ValueError):
                f(*args, **kwargs)
            continue
        out = f(*args, **kwargs)
        ref = np.asarray(rec["result"], dtype=np.float64)
        got = host(out) if isinstance(out, torch.Tensor) else np.asarray(out)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * (np.abs(ref).max() + 1))
        n += 1
    assert n >= 30
