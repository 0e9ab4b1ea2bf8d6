"""CPU checks of the learned warm start's oracle: the random-number generator
against SplitMix64's published outputs, the generated factors' structure,
and the oracle's analytic gradients (CP loss, network backward pass, Adam)
against finite differences."""

import numpy as np

from oracle import warm_start_oracle as wo


def test_splitmix64_known_outputs():
    # the first three outputs of SplitMix64 seeded with 0 (Steele, Lea and
    # Flood, OOPSLA 2014; the seeding generator of xoshiro/xorshift)
    gamma = 0x9E3779B97F4A7C15
    z = np.array([0, gamma, (2 * gamma) % 2 ** 64], dtype=np.uint64)
    got = [int(v) for v in wo.splitmix64(z)]
    assert got == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_range_and_gauss_moments():
    u = wo.uniform(5, np.arange(200_000))
    assert u.dtype == np.float32 and u.min() > 0 and u.max() < 1
    assert abs(u.mean() - 0.5) < 5e-3
    g = wo.gauss(7, np.arange(100_000))
    assert abs(g.mean()) < 2e-2 and abs(g.std() - 1) < 2e-2


def test_factors_have_requested_congruence():
    for seed in (0, 11, 123456):
        for n, A in enumerate(wo.factors_of(seed)):
            c = 0.9 * float(wo.uniform(8 * seed + 3 + n, 0))
            G = A.T @ A
            want = (1 - c) * np.eye(wo.R) + c * np.ones((wo.R, wo.R))
            np.testing.assert_allclose(G, want, atol=1e-12)


def test_generate_noise_level_and_sketch():
    om = wo.omega()
    X, feats, nrm = wo.generate([3, 4], om)
    for b, t in enumerate([3, 4]):
        clean = np.einsum("ir,jr,kr->ijk", *wo.factors_of(t)).ravel()
        noise = np.linalg.norm(X[b] - clean) / np.linalg.norm(clean)
        np.testing.assert_allclose(noise, 0.01, rtol=1e-10)
    np.testing.assert_allclose(nrm, np.linalg.norm(X, axis=1))
    f2, n2 = wo.sketch(X, om)
    np.testing.assert_array_equal(f2, feats)
    # mode-1 sketch block by an explicit unfolding
    U1 = X[0].reshape(32, 32, 32).transpose(1, 0, 2).reshape(32, 1024)
    np.testing.assert_allclose(feats[0, 512:1024].reshape(32, 16), U1 @ om[1] / nrm[0])


def _small_problem(seed=0, b=2):
    rs = np.random.RandomState(seed)
    X = rs.randn(b, wo.N3)
    nx = np.linalg.norm(X, axis=1)
    out = rs.randn(b, wo.OUT) * 0.3
    return X, nx, out


def test_cp_loss_gradient_finite_differences():
    X, nx, out = _small_problem()
    loss, dout, _ = wo.cp_loss(X, out, nx)
    rs = np.random.RandomState(1)
    h = 1e-6
    for _ in range(12):
        b, e = rs.randint(2), rs.randint(wo.OUT)
        op, om_ = out.copy(), out.copy()
        op[b, e] += h
        om_[b, e] -= h
        fd = (wo.cp_loss(X, op, nx)[0].sum() - wo.cp_loss(X, om_, nx)[0].sum()) / (2 * h) / 2
        np.testing.assert_allclose(dout[b, e], fd, rtol=1e-5, atol=1e-10)


def test_cp_loss_is_error_at_best_scale():
    X, nx, out = _small_problem(3)
    loss, _, alpha = wo.cp_loss(X, out, nx)
    A = out.reshape(-1, 3, 32, 8) * np.cbrt(nx)[:, None, None, None]
    for b in range(len(X)):
        rec = np.einsum("ir,jr,kr->ijk", *A[b]).ravel()
        best = min(np.sum((X[b] - a * rec) ** 2) for a in alpha[b] * (1 + np.linspace(-1e-3, 1e-3, 5)))
        np.testing.assert_allclose(loss[b], np.sum((X[b] - alpha[b] * rec) ** 2) / nx[b] ** 2,
                                   rtol=1e-10)
        assert loss[b] * nx[b] ** 2 <= best * (1 + 1e-12)
    # and the lifted factors reproduce the best-scaled model
    F = wo.lift(out, nx, alpha)
    rec = np.einsum("ir,jr,kr->ijk", *F[0]).ravel()
    np.testing.assert_allclose(np.sum((X[0] - rec) ** 2) / nx[0] ** 2, loss[0], rtol=1e-10)


def test_network_backward_finite_differences():
    rs = np.random.RandomState(2)
    ps = []
    for fin, fout in zip(wo.SIZES[:-1], wo.SIZES[1:]):
        ps += [rs.randn(fout, fin) * np.sqrt(2.0 / fin), rs.randn(fout) * 0.1]
    feats = rs.randn(3, wo.FEAT)
    X, nx, _ = _small_problem(4, 3)

    def total_loss(ps_):
        acts = wo.forward(ps_, feats)
        return wo.cp_loss(X, acts[-1], nx)[0].mean()

    acts = wo.forward(ps, feats)
    _, dout, _ = wo.cp_loss(X, acts[-1], nx)
    grads = wo.backward(ps, feats, acts, dout)
    h = 1e-6
    for k in range(len(ps)):
        for _ in range(3):
            idx = tuple(rs.randint(s) for s in ps[k].shape)
            pp = [p.copy() for p in ps]
            pm = [p.copy() for p in ps]
            pp[k][idx] += h
            pm[k][idx] -= h
            fd = (total_loss(pp) - total_loss(pm)) / (2 * h)
            np.testing.assert_allclose(grads[k][idx], fd, rtol=2e-4, atol=1e-9)


def test_flatten_roundtrip():
    n = sum(fi * fo + fo for fi, fo in zip(wo.SIZES[:-1], wo.SIZES[1:]))
    flat = np.arange(n, dtype=np.float64)
    np.testing.assert_array_equal(wo.flatten(wo.unflatten(flat)), flat)


def test_adam_first_step_is_signed_lr():
    g = np.array([0.5, -2.0, 1e-3])
    p, m, v = wo.adam(np.zeros(3), g, np.zeros(3), np.zeros(3), 0.01, 0.9, 0.999, 1e-8, 1)
    np.testing.assert_allclose(p, -0.01 * g / (np.abs(g) + 1e-8), rtol=1e-12)
