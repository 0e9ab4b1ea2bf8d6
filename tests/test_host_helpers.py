"""Host-side helpers against the reference's answers (tests/golden/host_kats.pkl):
validate_cp_rank (tensorly/cp_tensor.py:240-275), validate_tucker_rank
(tensorly/tucker_tensor.py:344-447) and check_random_state
(tensorly/backend/core.py:163-188) give the same value and type, raise the
same exception and warn with the same category on every recorded call."""

import os
import pickle
import warnings

import numpy as np
import pytest

from tensorly_gb300.cp_tensor import validate_cp_rank, validate_tucker_rank
from tensorly_gb300.random import check_random_state

HERE = os.path.dirname(os.path.abspath(__file__))
RECORDS = pickle.load(open(os.path.join(HERE, "golden", "host_kats.pkl"), "rb"))["records"]
FUNCS = {"validate_cp_rank": validate_cp_rank, "validate_tucker_rank": validate_tucker_rank,
         "check_random_state": check_random_state}


def test_record_count():
    assert len(RECORDS) >= 200


@pytest.mark.parametrize("i", range(len(RECORDS)))
def test_host_helper_matches_reference(i):
    rec = RECORDS[i]
    fn = FUNCS[rec["fn"]]
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        if "raises" in rec:
            with pytest.raises(Exception) as exc:
                fn(*rec["args"], **rec["kwargs"])
            assert type(exc.value).__name__ == rec["raises"]
            return
        out = fn(*rec["args"], **rec["kwargs"])
    assert sorted({type(x.message).__name__ for x in w}) == rec["warns"]
    if rec["fn"] == "check_random_state":
        np.testing.assert_array_equal(out.random_sample(4), rec["out"])
    else:
        assert type(out).__name__ == rec["type"]
        assert (list(out) if isinstance(out, list) else out) == rec["out"]


def test_global_random_state_is_numpys():
    assert check_random_state(None) is np.random.mtrand._rand
    rs = np.random.RandomState(3)
    assert check_random_state(rs) is rs
