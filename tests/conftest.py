import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gb300():
    """The built and loaded library (builds it on first use)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import tensorly_gb300 as tg
    tg.build()
    return tg


@pytest.fixture(scope="session")
def golden():
    import pickle
    here = os.path.join(REPO, "tests", "golden")
    with open(os.path.join(here, "tenalg_kats.pkl"), "rb") as f:
        kats = pickle.load(f)
    with open(os.path.join(here, "reference_runs.pkl"), "rb") as f:
        runs = pickle.load(f)
    with open(os.path.join(here, "reconstruction_kats.pkl"), "rb") as f:
        recon = pickle.load(f)
    with open(os.path.join(here, "cons_column_runs.pkl"), "rb") as f:
        cons_cols = pickle.load(f)
    with open(os.path.join(here, "tucker_extra_runs.pkl"), "rb") as f:
        tucker_extra = pickle.load(f)
    with open(os.path.join(here, "svd_extra_runs.pkl"), "rb") as f:
        svd_extra = pickle.load(f)
    return {"kats": kats["records"],
            "runs": {r["case"]: r for r in runs["runs"] + cons_cols["runs"]
                     + tucker_extra["runs"] + svd_extra["runs"]},
            "svd_kats": svd_extra["kats"],
            "recon": recon["records"], "versions": runs["versions"],
            "tucker_kats": tucker_extra["kats"],
            "fixed_mode_errors": tucker_extra["fixed_mode_errors"]}
