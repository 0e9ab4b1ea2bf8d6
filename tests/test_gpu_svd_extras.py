"""svd_interface with a mask and with 'randomized_svd' on the GPU
(tensorly/tenalg/svd.py:138-170, :288-357, :431-439), and the decompositions
that reach them: masked tucker from 'svd' and 'random' starts
(tensorly/decomposition/_tucker.py:25-221), tucker and parafac with
svd='randomized_svd', parafac with a mask from an 'svd' start
(tensorly/decomposition/_cp.py:26-137), all against runs of the reference.

Tolerances (f64): singular values 1e-10 relative; U, V, factors and cores
1e-8 of the largest entry (the Gram eigensolver's vectors, and the
refill loops that repeat it); error lists 1e-9 relative.  A bare
randomized_svd call is compared up to the sign of each singular pair, which
the reference leaves to LAPACK."""

import numpy as np
import pytest
import torch

from golden_inputs import dense_mask, regenerate

pytestmark = pytest.mark.gpu


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def close(a, b, tol):
    np.testing.assert_allclose(host(a), b, rtol=tol, atol=tol * max(np.abs(b).max(), 1e-300))


def test_svd_kats_match_reference(gb300, golden):
    from tensorly_gb300.svd import randomized_svd, svd_interface
    seen = set()
    for k in golden["svd_kats"]:
        m = torch.as_tensor(k["matrix"], device="cuda")
        if k["op"] == "svd_interface":
            mask = None if k["mask"] is None else torch.as_tensor(k["mask"], device="cuda")
            U, S, V = svd_interface(m, mask=mask,
                                    n_iter_mask_imputation=k["n_iter_mask_imputation"],
                                    **k["kwargs"])
            seen.add((k["kwargs"]["method"], mask is not None))
        else:
            U, S, V = randomized_svd(m, random_state=k["random_state"], **k["kwargs"])
            seen.add(("randomized_svd()", False))
            # randomized_svd alone leaves each singular pair's sign to LAPACK
            # (svd_interface then applies svd_flip); match the signs first
            sg = np.sign((host(U) * k["U"]).sum(axis=0))
            U = host(U) * sg
            V = host(V) * sg[:, None]
        np.testing.assert_allclose(host(S), k["S"], rtol=1e-10)
        close(U, k["U"], 1e-8)
        close(V, k["V"], 1e-8)
    assert len(seen) == 5


def test_svd_interface_host_arrays_and_errors(gb300, golden):
    from tensorly_gb300.svd import svd_interface
    k = golden["svd_kats"][0]
    U, S, V = svd_interface(k["matrix"], mask=k["mask"],
                            n_iter_mask_imputation=k["n_iter_mask_imputation"], **k["kwargs"])
    assert isinstance(U, np.ndarray)
    close(U, k["U"], 1e-8)
    with pytest.raises(ValueError):
        svd_interface(k["matrix"], method="no_such_svd", n_eigenvecs=2)


@pytest.mark.parametrize("case", ["tucker_mask_svd", "tucker_mask_random", "tucker_randomized",
                                  "cp_randomized", "cp_mask_svd"])
def test_svd_callers_match_reference(gb300, golden, case):
    run = golden["runs"][case]
    x = torch.as_tensor(regenerate(run), device="cuda")
    kw = dict(run["kwargs"])
    rank = kw.pop("rank")
    if "mask_keep" in run["gen"]:
        kw["mask"] = torch.as_tensor(dense_mask(run["gen"]), device="cuda")
    if run["np_seed"] is not None:
        np.random.seed(run["np_seed"])
    if run["fn"] == "tucker":
        (core, factors), errs = gb300.tucker(x, rank, return_errors=True, **kw)
        close(core, run["core"], 1e-8)
    else:
        (w, factors), errs = gb300.parafac(x, rank, return_errors=True, **kw)
        np.testing.assert_allclose(host(w), run["weights"], rtol=1e-8)
    assert len(errs) == len(run["errors"])
    np.testing.assert_allclose(errs, run["errors"], rtol=1e-9, atol=1e-12)
    for a, b in zip(factors, run["factors"]):
        close(a, b, 1e-8)
