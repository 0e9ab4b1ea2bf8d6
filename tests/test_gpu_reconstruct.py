"""Reconstruction on the GPU (tensorly/cp_tensor.py:433-546,
tensorly/tucker_tensor.py:50-162, tensorly/base.py:39-79) against the
reference's own test calls (tests/golden/reconstruction_kats.pkl) and the
NumPy oracle.

Tolerances: f64 1e-12 relative to the largest entry (the sum over the rank
runs in another order than NumPy's dot); the reference tests' integer-valued
known answers exactly; f32 1e-5 relative to the largest entry; unfold / fold
bit-exact (pure data movement)."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def host(t):
    return t.detach().cpu().numpy()


def dev(x):
    if isinstance(x, np.ndarray):
        return torch.as_tensor(x, device="cuda")
    if isinstance(x, tuple):
        return tuple(dev(v) for v in x)
    if isinstance(x, list):
        return [dev(v) for v in x]
    return x


def close(a, b, rel):
    b = np.asarray(b)
    np.testing.assert_allclose(a, b, rtol=rel, atol=rel * max(np.abs(b).max(), 1e-300))


def test_replays_reference_reconstruction_calls(gb300, golden):
    fns = {"cp_to_tensor": gb300.cp_to_tensor, "cp_to_unfolded": gb300.cp_to_unfolded,
           "cp_to_vec": gb300.cp_to_vec, "tucker_to_tensor": gb300.tucker_to_tensor,
           "tucker_to_unfolded": gb300.tucker_to_unfolded, "tucker_to_vec": gb300.tucker_to_vec}
    n = 0
    for rec in golden["recon"]:
        fn = fns.get(rec["fn"])
        if fn is None:
            continue
        out = host(fn(*dev(rec["args"]), **dev(rec["kwargs"])))
        ref = np.asarray(rec["result"])
        assert out.shape == ref.shape
        if np.array_equal(ref, np.round(ref)) and np.abs(ref).max() < 2 ** 40:
            np.testing.assert_array_equal(out, ref)     # integer-valued known answers
        else:
            close(out, ref, 1e-12)
        n += 1
    assert n >= 20


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape,rank", [((70, 29, 23), 17), ((9, 7, 5, 11), 6), ((130, 300), 70),
                                        ((33,), 5), ((3, 4, 2, 3, 2), 40), ((65, 1, 257), 3)])
def test_cp_to_tensor_matches_oracle(gb300, dtype, shape, rank):
    rs = np.random.RandomState(rank + len(shape))
    fs = [rs.randn(s, rank).astype(dtype) for s in shape]
    w = rs.rand(rank).astype(dtype) + 0.5
    ref = oracle.cp_to_tensor((w, fs))
    out = host(gb300.cp_to_tensor((dev(w), dev(fs))))
    close(out, ref, 1e-12 if dtype == np.float64 else 1e-5)
    if len(shape) > 1:
        close(host(gb300.cp_to_tensor((None, dev(fs)))), oracle.cp_to_tensor((None, fs)),
              1e-12 if dtype == np.float64 else 1e-5)
    else:                       # as the reference: None * factor
        with pytest.raises(TypeError):
            oracle.cp_to_tensor((None, fs))
        with pytest.raises(TypeError):
            gb300.cp_to_tensor((None, dev(fs)))
    close(host(gb300.cp_to_vec((dev(w), dev(fs)))), oracle.cp_to_vec((w, fs)),
          1e-12 if dtype == np.float64 else 1e-5)
    for mode in range(len(shape) if len(shape) > 1 else 0):
        close(host(gb300.cp_to_unfolded((dev(w), dev(fs)), mode)),
              oracle.cp_to_unfolded((w, fs), mode), 1e-12 if dtype == np.float64 else 1e-5)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_cp_to_tensor_with_mask(gb300, dtype):
    rs = np.random.RandomState(5)
    shape, rank = (21, 18, 16), 7
    fs = [rs.randn(s, rank).astype(dtype) for s in shape]
    w = rs.rand(rank).astype(dtype)
    mask = (rs.rand(*shape) > 0.3).astype(dtype)
    ref = oracle.cp_to_tensor((w, fs), mask=mask)
    out = host(gb300.cp_to_tensor((dev(w), dev(fs)), mask=dev(mask)))
    close(out, ref, 1e-12 if dtype == np.float64 else 1e-5)
    assert (out[mask == 0] == 0).all()
    # a mask broadcast along the first mode
    m2 = (rs.rand(*shape[1:]) > 0.5).astype(dtype)
    close(host(gb300.cp_to_tensor((dev(w), dev(fs)), mask=dev(m2))),
          oracle.cp_to_tensor((w, fs), mask=np.broadcast_to(m2, shape)),
          1e-12 if dtype == np.float64 else 1e-5)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_unfold_fold_round_trip(gb300, dtype):
    rs = np.random.RandomState(11)
    for shape in [(5, 6, 7), (3, 1, 4, 2), (40, 33), (17,), (2, 3, 2, 3, 2)]:
        x = rs.randn(*shape).astype(dtype)
        xt = dev(x)
        for mode in range(len(shape)):
            u = gb300.unfold(xt, mode)
            np.testing.assert_array_equal(host(u), oracle.unfold(x, mode))
            np.testing.assert_array_equal(host(gb300.fold(u, mode, shape)), x)
    with pytest.raises(ValueError):
        gb300.unfold(xt, 5)


def test_tucker_unfolded_and_vec_match_oracle(gb300):
    rs = np.random.RandomState(3)
    core = rs.rand(4, 3, 5, 2)
    fs = [rs.rand(r, s) for r, s in zip((2, 2, 3, 4), core.shape)]
    for mode in range(4):
        close(host(gb300.tucker_to_unfolded((dev(core), dev(fs)), mode)),
              oracle.tucker_to_unfolded((core, fs), mode), 1e-12)
    close(host(gb300.tucker_to_vec((dev(core), dev(fs)))), oracle.tucker_to_vec((core, fs)), 1e-12)


def test_cp_to_tensor_full_size_sampled(gb300):
    """512^3 f32 rank 64 (the headline model size): 4096 sampled entries
    against an f64 evaluation of the same factors."""
    g = torch.Generator(device="cuda").manual_seed(0)
    fs = [torch.randn(512, 64, device="cuda", generator=g) for _ in range(3)]
    w = torch.rand(64, device="cuda", generator=g) + 0.5
    full = gb300.cp_to_tensor((w, fs))
    assert full.shape == (512, 512, 512)
    rs = np.random.RandomState(0)
    idx = rs.randint(0, 512, size=(4096, 3))
    f64 = [host(f).astype(np.float64) for f in fs]
    w64 = host(w).astype(np.float64)
    ref = np.einsum("r,nr,nr,nr->n", w64, f64[0][idx[:, 0]], f64[1][idx[:, 1]], f64[2][idx[:, 2]])
    got = host(full)[idx[:, 0], idx[:, 1], idx[:, 2]].astype(np.float64)
    scale = np.abs(host(full)).max()
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6 * scale)
