"""Host logic of constrained_parafac: the constraint parsing of
tensorly/tenalg/proximal.py:4-145 (mirrored in decomposition.validate_constraints)
against the oracle's restatement, pinned by the constrained reference runs."""

import itertools

import pytest

import oracle
from tensorly_gb300.decomposition import validate_constraints

SPECS = [
    dict(non_negative=True),
    dict(l1_reg=0.1),
    dict(l1_reg=[0.1, 0.2, 0.3]),
    dict(l2_square_reg=[0.1, None, 0.3]),
    dict(l2_reg={0: 0.5, 2: 1.0}),
    dict(normalize={1: True}, non_negative={0: True, 2: True}),
    dict(non_negative=[True, False, True]),
    dict(simplex={2: 1.0}, l1_reg={0: 0.1}),
    dict(),
]


@pytest.mark.parametrize("spec", SPECS)
def test_validate_constraints_matches_oracle(spec):
    for order in range(3):
        assert validate_constraints(n_const=3, order=order, **spec) == \
            oracle.validate_constraints(n_const=3, order=order, **spec)


@pytest.mark.parametrize("a,b", list(itertools.combinations(
    [dict(non_negative=True), dict(l1_reg={0: 0.1}), dict(l2_reg=[0.1, 0.2, 0.3])], 2)))
def test_two_constraints_on_one_mode_raise(a, b):
    spec = {**a, **b}
    with pytest.raises(ValueError):
        validate_constraints(n_const=3, order=0, **spec)
    with pytest.raises(ValueError):
        oracle.validate_constraints(n_const=3, order=0, **spec)
