"""CPTensor and TuckerTensor validate their input on construction as the
reference's containers do (tensorly/cp_tensor.py:163-214,
tensorly/tucker_tensor.py:19-47): the recorded shape and rank of every
well-formed call of tests/golden/container_kats.pkl, and the same exception
type and message for every malformed one."""

import os
import pickle

import numpy as np
import pytest
import torch

from tensorly_gb300.cp_tensor import CPTensor, TuckerTensor

HERE = os.path.dirname(os.path.abspath(__file__))
RECORDS = pickle.load(open(os.path.join(HERE, "golden", "container_kats.pkl"), "rb"))["records"]


def _build(rec, as_torch):
    conv = (lambda a: None if a is None else torch.from_numpy(np.asarray(a))) if as_torch \
        else (lambda a: a)
    first, factors = rec["value"]
    value = (conv(first), [conv(f) for f in factors])
    return (CPTensor if rec["kind"] == "cp" else TuckerTensor), value


@pytest.mark.parametrize("as_torch", [False, True])
@pytest.mark.parametrize("i", range(len(RECORDS)))
def test_container_matches_reference(i, as_torch):
    rec = RECORDS[i]
    cls, value = _build(rec, as_torch)
    if "raises" in rec:
        with pytest.raises(Exception) as exc:
            cls(value)
        assert type(exc.value).__name__ == rec["raises"]
        assert str(exc.value) == rec["message"]
        return
    obj = cls(value)
    assert tuple(obj.shape) == rec["shape"]
    assert obj.rank == rec["rank"]


def test_cp_default_weights_follow_the_factors():
    f = [torch.ones(4, 3, dtype=torch.float64), torch.ones(5, 3, dtype=torch.float64)]
    cp = CPTensor((None, f))
    assert cp.weights.dtype == torch.float64 and tuple(cp.weights.shape) == (3,)
    assert CPTensor(cp).shape == (4, 5)
