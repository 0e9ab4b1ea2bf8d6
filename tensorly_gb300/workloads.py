"""Seeded synthetic workloads (host NumPy arrays).

No public dataset is involved: every input is generated from NumPy
RandomState seeds, so the GPU path, the CPU oracle and the reference see the
same bytes on any machine.

dense_cp_small   64^3 f64 rank-8 CP, U(0,1) factors, 1 % Gaussian noise
dense_cp_large   512^3 f32 rank-64 CP, N(0,1) unit-norm columns, 20 dB SNR
cp_tucker_4way   128^4 f32 rank-32 CP + 16^4 Tucker (orthonormal factors), 1 % noise
batched_uneven   4096 3-way f32 tensors, modes U{8..64}, rank U{4..16}, 1 % noise
"""

import numpy as np


def _cp_full(factors, weights=None):
    """Full tensor of a CP model: mode-0 unfolding A0 . KR(A1..)^T, folded."""
    shape = tuple(f.shape[0] for f in factors)
    rank = factors[0].shape[1]
    kr = factors[-1]
    for f in reversed(factors[1:-1]):
        kr = (f[:, None, :] * kr[None, :, :]).reshape(-1, rank)
    a0 = factors[0] if weights is None else factors[0] * weights
    return (a0 @ kr.T).reshape(shape)


def _add_noise(x, rs, level):
    """x + level * ||x|| * N / ||N|| with N ~ N(0, 1) from `rs`."""
    n = rs.randn(*x.shape)
    return x + level * np.linalg.norm(x) * n / np.linalg.norm(n)


def dense_cp_small(size=64, rank=8, seed=0):
    """64^3 float64 tensor from a rank-8 CP model with U(0,1) factors plus
    Gaussian noise at 1 % of the Frobenius norm."""
    rs = np.random.RandomState(seed)
    factors = [rs.uniform(size=(size, rank)) for _ in range(3)]
    x = _cp_full(factors)
    return _add_noise(x, rs, 0.01), factors


def dense_cp_large(size=512, rank=64, seed=0, dtype=np.float32):
    """float32 size^3 tensor from a rank-64 CP model with N(0,1) factor entries
    and unit-normalised columns, plus Gaussian noise at 20 dB SNR (noise norm
    = 10 % of the signal norm)."""
    rs = np.random.RandomState(seed)
    factors = []
    for _ in range(3):
        f = rs.randn(size, rank)
        f /= np.linalg.norm(f, axis=0, keepdims=True)
        factors.append(f.astype(dtype))
    x = _cp_full(factors).astype(dtype)
    nrm = float(np.linalg.norm(x.astype(np.float64)))
    noise = rs.randn(*x.shape).astype(dtype)
    noise *= dtype(0.1 * nrm / float(np.linalg.norm(noise.astype(np.float64))))
    x += noise
    return x, factors


def cp_tucker_4way(size=128, cp_rank=32, tucker_rank=16, seed=0, dtype=np.float32):
    """float32 size^4 tensor: a rank-32 CP model (N(0,1) factors) plus a
    Tucker model (N(0,1) 16^4 core, orthonormal factors), each scaled to unit
    Frobenius norm, plus Gaussian noise at 1 % of the signal norm."""
    rs = np.random.RandomState(seed)
    cpf = [rs.randn(size, cp_rank) for _ in range(4)]
    core = rs.randn(*([tucker_rank] * 4))
    tf = [np.linalg.qr(rs.randn(size, tucker_rank))[0] for _ in range(4)]
    cp = _cp_full(cpf).astype(dtype)
    cp /= dtype(np.linalg.norm(cp.astype(np.float64)))
    tk = core
    for k, f in enumerate(tf):
        tk = np.moveaxis(np.tensordot(f, np.moveaxis(tk, k, 0), axes=(1, 0)), 0, k)
    tk = tk.astype(dtype)
    tk /= dtype(np.linalg.norm(tk.astype(np.float64)))
    x = cp + tk
    nrm = float(np.linalg.norm(x.astype(np.float64)))
    noise = rs.randn(*x.shape).astype(dtype)
    noise *= dtype(0.01 * nrm / float(np.linalg.norm(noise.astype(np.float64))))
    x += noise
    return x


def batched_uneven(count=4096, seed=0, dtype=np.float32, lo=8, hi=64, rlo=4, rhi=16):
    """`count` independent 3-way tensors; mode sizes U{lo..hi}, rank U{rlo..rhi},
    N(0,1) factors, 1 % noise.  Returns a list of (tensor, rank, init_seed)."""
    master = np.random.RandomState(seed)
    out = []
    for t in range(count):
        rs = np.random.RandomState(master.randint(2 ** 31))
        dims = [int(rs.randint(lo, hi + 1)) for _ in range(3)]
        rank = int(rs.randint(rlo, rhi + 1))
        factors = [rs.randn(d, rank) for d in dims]
        x = _add_noise(_cp_full(factors), rs, 0.01).astype(dtype)
        out.append((x, rank, t))
    return out
