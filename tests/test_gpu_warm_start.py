"""Learned warm start on the GPU: generator, sketches, GEMM, network forward
and backward, CP loss, Adam and the SVD start against the NumPy oracle; the
batched kernel's per-tensor stop test; training on the GPU; and what the
trained network gains over ALS from TensorLy's SVD start."""

import numpy as np
import pytest
import torch

from oracle import warm_start_oracle as wo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ws(gb300):
    from tensorly_gb300 import learned
    return learned


@pytest.fixture(scope="module")
def gen(ws):
    return ws.Generator("cuda")


def _rel(a, b):
    return np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30)


def test_omega_matches_oracle(gen):
    om = gen.omega.cpu().numpy().reshape(3, 1024, 16)
    # float32 log / cos on the GPU against float64 on the same uniforms
    assert _rel(om, wo.omega()) < 1e-5


def test_generator_matches_oracle(gen):
    seeds = [0, 1, 977, 123456]
    X, feats, nrm = gen(seeds)
    Xo, fo, no = wo.generate(seeds, wo.omega())
    assert _rel(X.cpu().numpy(), Xo) < 1e-4
    assert _rel(feats.cpu().numpy(), fo) < 1e-4
    np.testing.assert_allclose(nrm.cpu().numpy(), no, rtol=1e-5)


def test_sketch_kernel_equals_generator_features(ws, gen):
    X, feats, nrm = gen(np.arange(40, 72))
    f2, n2 = ws.sketch(X, gen.omega)
    assert torch.equal(f2, feats) and torch.equal(n2, nrm)


@pytest.mark.parametrize("layout", ["xwT", "dyTx", "dyW"])
def test_gemm_layouts_with_epilogue(ws, layout):
    rs = np.random.RandomState(5)
    M, N, K = 70, 130, 45
    if layout == "xwT":      # C = A B^T: A (M x K), B stored (N x K)
        A = rs.randn(M, K); B = rs.randn(N, K)
        args = (A, K, 1, B, 1, K)
        want = A @ B.T
    elif layout == "dyTx":   # C = A^T B: A stored (K x M), B (K x N)
        A = rs.randn(K, M); B = rs.randn(K, N)
        args = (A, 1, M, B, N, 1)
        want = A.T @ B
    else:                    # C = A B: A (M x K), B (K x N)
        A = rs.randn(M, K); B = rs.randn(K, N)
        args = (A, K, 1, B, N, 1)
        want = A @ B
    bias = rs.randn(N)
    mask = rs.randn(M, N)
    dev = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda").contiguous()
    Ad, sam, sak, Bd, sbk, sbn = dev(args[0]), args[1], args[2], dev(args[3]), args[4], args[5]
    C = torch.empty((M, N), dtype=torch.float32, device="cuda")
    ws._gemm(M, N, K, Ad, sam, sak, Bd, sbk, sbn, C, N, bias=dev(bias), relu=True)
    np.testing.assert_allclose(C.cpu().numpy(), np.maximum(want + bias, 0), atol=1e-4)
    ws._gemm(M, N, K, Ad, sam, sak, Bd, sbk, sbn, C, N, mask=dev(mask))
    np.testing.assert_allclose(C.cpu().numpy(), want * (mask > 0), atol=1e-4)


@pytest.mark.parametrize("layout", ["xwT", "dyTx", "dyW"])
@pytest.mark.parametrize("shape", [(300, 260, 203), (512, 1024, 1536), (129, 64, 64)])
def test_tensor_core_gemm_layouts_with_epilogue(ws, layout, shape):
    """tlgb_ws_gemm_tc (exact three-plane bf16 split of both operands, the
    products a_i b_j with i + j <= 2 on tcgen05, f32 accumulation) in the
    network's three operand layouts, with ragged sizes (K not a multiple of 8,
    M and N not multiples of 128) and the network's own; against f64 NumPy and
    against the SIMT f32 kernel to 3e-5 of the largest entry: the operand
    split is exact to 2^-26, what remains is the f32 accumulation over up to
    1536 terms, which the tensor cores truncate (measured 1.2e-5 at K = 1536)."""
    M, N, K = shape
    rs = np.random.RandomState(M + N + K)
    if layout == "xwT":
        A = rs.randn(M, K); B = rs.randn(N, K)
        args = (A, K, 1, B, 1, K)
        want = A @ B.T
    elif layout == "dyTx":
        A = rs.randn(K, M); B = rs.randn(K, N)
        args = (A, 1, M, B, N, 1)
        want = A.T @ B
    else:
        A = rs.randn(M, K); B = rs.randn(K, N)
        args = (A, K, 1, B, N, 1)
        want = A @ B
    bias = rs.randn(N)
    mask = rs.randn(M, N)
    dev = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda").contiguous()
    Ad, sam, sak, Bd, sbk, sbn = dev(args[0]), args[1], args[2], dev(args[3]), args[4], args[5]
    C = torch.empty((M, N), dtype=torch.float32, device="cuda")
    assert ws.USE_TENSOR_CORES and min(M, N, K) >= ws.TC_MIN
    scale = np.abs(want).max()
    ws._gemm(M, N, K, Ad, sam, sak, Bd, sbk, sbn, C, N, bias=dev(bias), relu=True)
    c_tc = C.cpu().numpy()
    assert np.abs(c_tc - np.maximum(want + bias, 0)).max() <= 3e-5 * scale
    ws._gemm(M, N, K, Ad, sam, sak, Bd, sbk, sbn, C, N, mask=dev(mask))
    assert np.abs(C.cpu().numpy() - want * (mask > 0)).max() <= 3e-5 * scale
    try:
        ws.USE_TENSOR_CORES = False
        C2 = torch.empty_like(C)
        ws._gemm(M, N, K, Ad, sam, sak, Bd, sbk, sbn, C2, N, bias=dev(bias), relu=True)
    finally:
        ws.USE_TENSOR_CORES = True
    assert np.abs(c_tc - C2.cpu().numpy()).max() <= 3e-5 * scale
    ws.gemm_status()


def test_forward_backward_and_loss_match_oracle(ws, gen):
    net = ws.WarmStartNet(seed=3)
    X, feats, nrm = gen(np.arange(100, 164))
    loss = net.loss_and_grad(X, feats, nrm)
    ps = wo.unflatten(net.params.cpu().numpy())
    f64 = feats.cpu().numpy().astype(np.float64)
    acts = wo.forward(ps, f64)
    lo, dout, alpha = wo.cp_loss(X.cpu().numpy(), acts[-1], nrm.cpu().numpy())
    np.testing.assert_allclose(loss.cpu().numpy(), lo, rtol=2e-4)
    g_gpu = wo.unflatten(net.grads.cpu().numpy())
    g_ref = wo.backward(ps, f64, acts, dout)
    for k, (a, b) in enumerate(zip(g_gpu, g_ref)):
        assert _rel(a, b) < 2e-3, (k, _rel(a, b))
    out = net.forward(feats)[-1].cpu().numpy()
    assert _rel(out, acts[-1]) < 1e-4
    l2, _, a2 = net.loss(X, feats, nrm)
    np.testing.assert_allclose(l2.cpu().numpy(), lo, rtol=2e-4)
    # p = <X, [[A]]> cancels for a random network: compare against the largest
    assert _rel(a2.cpu().numpy(), alpha) < 1e-3
    F = net.predict(X, feats, nrm).cpu().numpy()
    assert _rel(F, wo.lift(acts[-1], nrm.cpu().numpy(), alpha)) < 1e-3


def test_adam_matches_oracle(ws):
    net = ws.WarmStartNet(seed=1)
    rs = np.random.RandomState(9)
    n = net.n_params
    p0 = net.params.cpu().numpy().astype(np.float64)
    m = np.zeros(n); v = np.zeros(n); p = p0
    for step in range(1, 4):
        g = rs.randn(n) * 1e-2
        net.grads.copy_(torch.tensor(g, dtype=torch.float32))
        net.adam(lr=1e-3)
        p, m, v = wo.adam(p, g.astype(np.float32).astype(np.float64), m, v, 1e-3, 0.9, 0.999,
                          1e-8, step)
    np.testing.assert_allclose(net.params.cpu().numpy(), p, atol=2e-6)


def test_svd_start_matches_reference_init(ws, gen):
    X, _, _ = gen(np.arange(7))
    F = ws.svd_init(X).cpu().numpy()
    Fo = wo.svd_init(X.cpu().numpy())
    # f32 Gram: a singular vector moves by ~eps ||G|| / gap, so the columns are
    # compared loosely (same order and signs) and their span tightly
    for b in range(7):
        for n in range(3):
            cn = np.linalg.norm(Fo[b, n], axis=0)
            np.testing.assert_allclose(np.linalg.norm(F[b, n], axis=0), cn, rtol=1e-4)
            Un, Uo = F[b, n] / cn, Fo[b, n] / cn
            assert np.abs(Un - Uo).max() < 2e-2, (b, n)
            assert np.abs(Un @ Un.T - Uo @ Uo.T).max() < 1e-4, (b, n)


def test_batched_tol_stops_at_reference_test(gb300, gen):
    from tensorly_gb300 import learned
    X, _, _ = gen(np.arange(300, 332))
    F0 = learned.svd_init(X)
    full = learned._als(X, F0, 60, sweep_errors=True)
    errs = full.sweeps.cpu().numpy()
    tol = 1e-6
    want = learned.sweeps_to_tol(errs, tol)
    stop = learned._als(X, F0, 60, tol=tol)
    got = stop.n_sweeps.cpu().numpy()
    np.testing.assert_array_equal(got, want)
    np.testing.assert_allclose(stop.final.cpu().numpy(), errs[np.arange(32), want - 1], rtol=1e-12)
    # the factors are those of a plain run of that many sweeps
    for k in np.unique(got)[:3]:
        plain = learned._als(X, F0, int(k))
        sel = np.where(got == k)[0]
        a = stop.fbuf.view(32, -1)[sel]
        b = plain.fbuf.view(32, -1)[sel]
        assert torch.equal(a, b)
    # split into launches of 7 sweeps: same stop and factors
    from tensorly_gb300.decomposition import BatchedProblem
    prob = BatchedProblem(X.view(-1, 32, 32, 32), 8, init=F0)
    prob.run(60, sweeps_per_launch=7, tol=tol)
    np.testing.assert_array_equal(prob.n_sweeps.cpu().numpy(), got)
    assert torch.equal(prob.fbuf, stop.fbuf)


@pytest.fixture(scope="module")
def trained(ws, gen):
    net = ws.WarmStartNet(seed=0)
    losses = net.train(n_samples=64 * 1024, batch=512, lr=1e-3, lr_final=1e-4, generator=gen)
    return net, losses


def test_training_reduces_loss(trained):
    net, losses = trained
    assert np.isfinite(losses).all()
    print("\ntraining loss: first 16 steps %.4f, last 16 steps %.4f"
          % (losses[:16].mean(), losses[-16:].mean()))
    assert losses[-16:].mean() < losses[:16].mean(), (losses[:16], losses[-16:])


def test_warm_start_gain_over_svd_start(ws, gen, trained):
    """What the trained network gains: sweeps and time to the reference's stop
    test (tol 1e-6) on held-out tensors, from init='svd', from the network's
    start and from the warm start with its SVD fallback; the fit must match."""
    net, _ = trained
    untrained = ws.WarmStartNet(seed=0)
    seeds = np.arange(10 ** 6, 10 ** 6 + 1024)
    res = ws.evaluate(net, seeds, max_sweeps=300, tol=1e-6, generator=gen)
    res5 = ws.evaluate(net, seeds[:256], max_sweeps=300, tol=1e-6, probe=5, generator=gen)
    X, feats, nrm = gen(seeds)
    loss_tr = net.loss(X, feats, nrm)[0].mean().item()
    loss_un = untrained.loss(X, feats, nrm)[0].mean().item()
    print(f"\nheld-out loss (relative error^2 at best scale): untrained {loss_un:.4f} "
          f"trained {loss_tr:.4f}")
    for k in ("svd", "learned", "warm"):
        v = res["sweeps_" + k]
        print("start %-8s sweeps to tol mean %.1f median %.0f p90 %.0f; time to fit %.2f ms"
              % (k, v.mean(), np.median(v), np.percentile(v, 90), res["ms_" + k]))
    print("network start kept by the fallback test for %.1f %% of tensors"
          % (100 * (1 - res["used_svd"].mean())))
    resu = ws.evaluate(untrained, seeds, max_sweeps=300, tol=1e-6, generator=gen)
    print("untrained network (the sketch skip alone): %.1f mean sweeps from its start"
          % resu["sweeps_learned"].mean())
    resc = ws.evaluate(net, seeds[:256], max_sweeps=300, tol=1e-6, generator=gen, max_err=0.0)
    print("falling back for every tensor (256 tensors): svd %.1f, warm %.1f mean sweeps"
          % (resc["sweeps_svd"].mean(), resc["sweeps_warm"].mean()))
    np.testing.assert_array_equal(resc["sweeps_warm"], resc["sweeps_svd"])
    print("with 5 ALS probe sweeps choosing the start (256 tensors): svd %.1f, warm %.1f mean sweeps, "
          "network kept for %.1f %%" % (res5["sweeps_svd"].mean(), res5["sweeps_warm"].mean(),
                                         100 * (1 - res5["used_svd"].mean())))
    assert (res5["sweeps_warm"] >= 5).all()
    assert loss_tr < loss_un
    for k in ("learned", "warm"):   # same fit as from the SVD start
        rel = (res["err_" + k] - res["err_svd"]) / res["err_svd"]
        assert abs(np.median(rel)) < 1e-4, (k, np.median(rel))
    # The gain over the method without the network (init='svd'): on these 1024
    # held-out tensors the network's start needed 42.5 mean sweeps against 47.2
    # from the SVD start, and the warm start reached the fit in 26.9 ms against
    # 38.7 ms.  Training itself adds little beyond the sketch skip (42.6 mean
    # sweeps untrained), which the printout above reports.
    assert res["sweeps_learned"].mean() <= 0.95 * res["sweeps_svd"].mean()
    assert res["sweeps_warm"].mean() <= 0.95 * res["sweeps_svd"].mean()
    assert res["ms_warm"] < res["ms_svd"]
