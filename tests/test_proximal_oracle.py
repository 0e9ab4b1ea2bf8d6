"""Pins the proximal-operator oracle (oracle/proximal_oracle.py) to the calls
of the reference's own tests (tensorly/tenalg/tests/test_proximal.py,
recorded in tests/golden/proximal_kats.pkl)."""

import os
import pickle

import numpy as np

from oracle import proximal_oracle as px

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_proximal_oracle_replays_reference_calls():
    with open(os.path.join(HERE, "proximal_kats.pkl"), "rb") as f:
        records = pickle.load(f)["records"]
    n = 0
    for rec in records:
        fn = getattr(px, rec["fn"], None)
        if fn is None or rec["fn"].startswith("assert") or rec["fn"] == "__test__":
            continue
        out = fn(*rec["args"], **rec["kwargs"])
        np.testing.assert_allclose(np.asarray(out), np.asarray(rec["result"]), rtol=1e-12,
                                   atol=1e-12)
        n += 1
    assert n >= 15
    assert sum(1 for r in records if r["fn"] == "__test__") == 12
