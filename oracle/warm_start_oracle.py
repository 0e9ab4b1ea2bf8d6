"""NumPy restatement of the learned warm start's kernels (TEST INFRASTRUCTURE ONLY).

The learned warm start has no counterpart in TensorLy; its fallback is the
reference's ``init='svd'`` (tensorly/decomposition/_cp.py:70-96, restated in
``tensorly_oracle.initialize_cp``).  This module restates, in float64 NumPy,
what the CUDA kernels of ``tensorly_gb300/csrc/learned.cu`` compute, so the
tests can check the generator, the sketches, the network's forward and
backward passes, the CP reconstruction loss and its gradient, and Adam
against it.  Its own gradients are checked by finite differences in
``tests/test_warm_start_oracle.py``.  Only ``tests/``, ``smoke()`` and the
CPU legs of ``bench.py`` import it.

Random numbers follow the kernels exactly: z = SplitMix64((stream << 40) ^ i)
(Steele, Lea and Flood, OOPSLA 2014), a uniform is ((z >> 40) + 1/2) / 2^24
rounded as float32, a Gaussian is Box-Muller on the uniforms of indices 2i
and 2i + 1 (evaluated here in float64, on the GPU in float32).
"""

import numpy as np

from . import tensorly_oracle as tlo

I, R, S = 32, 8, 16
N3 = I * I * I
FEAT = 3 * I * S
OUT = 3 * I * R
SIZES = (FEAT, 1024, 512, OUT)

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(stream, idx):
    """float32 uniforms in (0, 1) of counter indices ``idx`` of ``stream``."""
    key = (np.uint64(stream) << np.uint64(40)) ^ np.asarray(idx, dtype=np.uint64)
    hi = (splitmix64(key) >> np.uint64(40)).astype(np.float32)
    return (hi + np.float32(0.5)) * np.float32(1.0 / 16777216.0)


def gauss(stream, idx):
    idx = np.asarray(idx, dtype=np.uint64)
    u1 = uniform(stream, 2 * idx).astype(np.float64)
    u2 = uniform(stream, 2 * idx + 1).astype(np.float64)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def omega():
    """The fixed sketch matrices Omega_n (3 x 1024 x 16)."""
    return np.stack([gauss((1 << 23) + n, np.arange(I * I * S)).reshape(I * I, S)
                     for n in range(3)])


def factors_of(seed):
    """The three 32 x 8 factors of tensor ``seed``: Gram-Schmidt of a Gaussian
    matrix times L^T, L = chol((1 - c) I + c 1 1^T), c = 0.9 U."""
    t = int(seed)
    out = []
    for n in range(3):
        g = gauss(8 * t + n, np.arange(I * R)).reshape(I, R)
        q = g.copy()
        for r in range(R):                      # modified Gram-Schmidt
            for s in range(r):
                q[:, r] -= (q[:, s] @ q[:, r]) * q[:, s]
            q[:, r] /= np.linalg.norm(q[:, r])
        c = 0.9 * float(uniform(8 * t + 3 + n, 0))
        C = (1.0 - c) * np.eye(R) + c * np.ones((R, R))
        L = np.linalg.cholesky(C)
        out.append(q @ L.T)
    return out


def sketch(X, om):
    """(features batch x 1536, norms) of tensors X (batch x 32768)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, I, I, I)
    nrm = np.sqrt((X.reshape(len(X), -1) ** 2).sum(axis=1))
    feats = []
    for n in range(3):
        U = np.moveaxis(X, n + 1, 1).reshape(len(X), I, I * I)   # C-order unfolding
        feats.append((U @ om[n]).reshape(len(X), -1))
    return np.concatenate(feats, axis=1) / nrm[:, None], nrm


def generate(seeds, om):
    """Tensors (batch x 32768), features and norms, as the generator kernel."""
    Xs = []
    for t in seeds:
        A = factors_of(t)
        X = np.einsum("ir,jr,kr->ijk", *A).reshape(-1)
        z = gauss(8 * int(t) + 6, np.arange(N3))
        X = X + 0.01 * np.linalg.norm(X) / np.linalg.norm(z) * z
        Xs.append(X)
    X = np.stack(Xs)
    feats, nrm = sketch(X, om)
    return X, feats, nrm


# ---- network ------------------------------------------------------------------

def unflatten(params):
    """[W1, b1, W2, b2, W3, b3] (W: fan_out x fan_in) from the flat buffer."""
    out, o = [], 0
    for fin, fout in zip(SIZES[:-1], SIZES[1:]):
        out.append(np.asarray(params[o:o + fin * fout], dtype=np.float64).reshape(fout, fin))
        o += fin * fout
        out.append(np.asarray(params[o:o + fout], dtype=np.float64))
        o += fout
    return out


def flatten(ps):
    return np.concatenate([p.ravel() for p in ps])


def sketch_skip(feats):
    """The first R columns of each 32 x 16 sketch block, as (batch x 768)."""
    f = np.asarray(feats, dtype=np.float64).reshape(-1, 3, I, S)
    return f[:, :, :, :R].reshape(len(f), OUT)


def forward(ps, feats):
    """Activations [H1, H2, out]: ReLU after the first two layers, the fixed
    sketch skip added to the output."""
    x = np.asarray(feats, dtype=np.float64)
    acts = []
    n_layers = len(ps) // 2
    for li in range(n_layers):
        y = x @ ps[2 * li].T + ps[2 * li + 1]
        if li < n_layers - 1:
            y = np.maximum(y, 0.0)
        acts.append(y)
        x = y
    acts[-1] = acts[-1] + sketch_skip(feats)
    return acts


def backward(ps, feats, acts, dout):
    """Gradients [dW1, db1, ...] from d loss / d out."""
    xs = [np.asarray(feats, dtype=np.float64)] + acts[:-1]
    grads = [None] * len(ps)
    dy = dout
    for li in reversed(range(len(ps) // 2)):
        grads[2 * li] = dy.T @ xs[li]
        grads[2 * li + 1] = dy.sum(axis=0)
        if li > 0:
            dy = (dy @ ps[2 * li]) * (xs[li] > 0)
    return grads


def cp_loss(X, out, xnorm, batch=None):
    """Scale-free loss of A_n = out_n ||X_b||^(1/3): with p = <X, [[A]]> and
    q = ||[[A]]||^2, loss_b = 1 - p^2 / (||X||^2 q) = min_a ||X - a [[A]]||^2 /
    ||X||^2, d (sum_b loss_b / batch) / d out_n = ||X||^(1/3) (2 p / (||X||^2 q))
    ((p / q) A_n V_n - M_n) / batch, and the best scale alpha = p / q."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, I, I, I)
    out = np.asarray(out, dtype=np.float64).reshape(-1, 3, I, R)
    nx = np.asarray(xnorm, dtype=np.float64)
    b = len(X)
    batch = b if batch is None else batch
    sc = np.cbrt(nx)
    A = out * sc[:, None, None, None]
    rec = np.einsum("bir,bjr,bkr->bijk", A[:, 0], A[:, 1], A[:, 2])
    p = (X * rec).sum(axis=(1, 2, 3))
    q = (rec * rec).sum(axis=(1, 2, 3))
    loss = 1.0 - p * p / (nx ** 2 * q)
    G = np.einsum("bnir,bnis->bnrs", A, A)
    M = [np.einsum("bijk,bjr,bkr->bir", X, A[:, 1], A[:, 2]),
         np.einsum("bijk,bir,bkr->bjr", X, A[:, 0], A[:, 2]),
         np.einsum("bijk,bir,bjr->bkr", X, A[:, 0], A[:, 1])]
    dout = np.empty_like(out)
    for n in range(3):
        V = np.prod([G[:, k] for k in range(3) if k != n], axis=0)
        coef = (2.0 * p / (nx ** 2 * q))[:, None, None]
        dA = coef * ((p / q)[:, None, None] * (A[:, n] @ V) - M[n])
        dout[:, n] = dA * sc[:, None, None] / batch
    return loss, dout.reshape(b, OUT), p / q


def lift(out, xnorm, alpha):
    """Initial factors out * (||X|| alpha)^(1/3) (batch x 3 x 32 x 8)."""
    out = np.asarray(out, dtype=np.float64).reshape(-1, 3, I, R)
    return out * np.cbrt(np.asarray(xnorm) * np.asarray(alpha))[:, None, None, None]


def adam(p, g, m, v, lr, beta1, beta2, eps, step):
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    c1, c2 = 1 - beta1 ** step, 1 - beta2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def svd_init(X):
    """The reference's init='svd' factors (batch x 3 x 32 x 8)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, I, I, I)
    return np.stack([np.stack(tlo.initialize_cp(x, R, init="svd")[1]) for x in X])
