"""PARAFAC2 on the GPU (tensorly/decomposition/_parafac2.py:399-707) against the
reference runs (tests/golden) and NumPy.

Tolerances: f64 1e-7 on the error list and 1e-5 (of the largest entry) on
factors and projections (the projections are polar factors from R x R
eigenproblems instead of the reference's SVD); f32 1e-3 and 1e-2.  The QR of
the random start matches NumPy's linalg.qr, signs included, to 1e-12."""

import warnings

import numpy as np
import pytest
import torch

from golden_inputs import regenerate, slice_masks

pytestmark = pytest.mark.gpu


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("case", ["p2_random", "p2_svd", "p2_nols", "p2_normalize", "p2_f32",
                                  "p2_nn_all", "p2_nn_02", "p2_mask", "p2_mask_svd"])
def test_parafac2_matches_reference(gb300, golden, case):
    """Dense, non-negative (nn_modes through non_negative_parafac_hals and
    the clipped line search) and masked (refilled missing entries, masked
    error) runs against the reference's."""
    run = golden["runs"][case]
    xs = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if "mask_keep" in run["gen"]:
        kw["mask"] = [torch.as_tensor(m, device="cuda") for m in slice_masks(run["gen"])]
    xt = [torch.as_tensor(x, device="cuda") for x in xs]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)   # the reference's mode-1 warning
        (w, f, p), errs = gb300.parafac2(xt, rank, return_errors=True, **kw)
    for x, t in zip(xs, xt):
        assert np.array_equal(host(t), x), "the input slices were modified"
    f32 = xs[0].dtype == np.float32
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-3 if f32 else 1e-7)
    tol = 1e-2 if f32 else 1e-5
    np.testing.assert_allclose(host(w), run["weights"], rtol=tol, atol=tol)
    for a, b in zip(list(f) + list(p), run["factors"] + run["projections"]):
        np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * np.abs(b).max())


@pytest.mark.parametrize("shape", [(9, 3), (40, 7), (300, 16), (5, 5)])
def test_qr_matches_numpy_signs(gb300, shape):
    from tensorly_gb300.parafac2 import _qr        # the module (the package exports the function)
    a = np.random.RandomState(shape[0]).random_sample(shape)
    q = host(_qr(torch.as_tensor(a, device="cuda")))
    np.testing.assert_allclose(q, np.linalg.qr(a)[0], rtol=1e-11, atol=1e-12)


def test_parafac2_to_tensor_and_host_input(gb300, golden):
    run = golden["runs"]["p2_nols"]
    xs = regenerate(run)
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    out = gb300.parafac2(xs, rank, **kw)                    # host slices in, host out
    w, (A, B, C), ps = out
    assert isinstance(A, np.ndarray)
    dev = gb300.Parafac2Tensor((torch.as_tensor(w, device="cuda"),
                                [torch.as_tensor(m, device="cuda") for m in (A, B, C)],
                                [torch.as_tensor(m, device="cuda") for m in ps]))
    full = host(gb300.parafac2_to_tensor(dev))
    for k, pk in enumerate(ps):
        ref = (pk @ B) * (A[k] * w) @ C.T
        np.testing.assert_allclose(full[k, :pk.shape[0]], ref, rtol=1e-12, atol=1e-12)
        assert (full[k, pk.shape[0]:] == 0).all()
    with pytest.warns(UserWarning, match="Mode `1` of PARAFAC2"):
        gb300.parafac2(xs, rank, nn_modes=[1], n_iter_max=2)
