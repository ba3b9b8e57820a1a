"""The oracle and the workload generator against the frozen fixtures of tests/golden (made by
tests/golden/make_golden.py): the same seeded inputs, and the same results bit for bit."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

FIXTURES = [c[0] for c in G.cases()]


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_inputs_are_the_generators(name):
    f = load(name)
    e = {c[0]: c[1] for c in G.cases()}[name]
    for k in ("t0", "tf", "y0", "params", "rtol", "atol", "family"):
        assert np.array_equal(f[k], getattr(e, k)), k


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(name):
    f = load(name)
    _, e, method, te = next(c for c in G.cases() if c[0] == name)
    o = G.solve(e, method, te)
    for k in ("status", "accepted", "rejected", "fevals", "y_final", "t_final"):
        assert np.array_equal(o[k], f[k]), k
    if te is not None:
        assert np.array_equal(o["dense"], f["dense"], equal_nan=True)
