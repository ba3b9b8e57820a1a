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
    """The generator still draws these inputs.  The normal draws go through numpy's log and cos,
    whose last bit differs between platforms (the fixtures come from an x86 host), so y0 is
    compared to 1e-15; everything else bit for bit."""
    f = load(name)
    e = {c[0]: c[1] for c in G.cases()}[name]
    for k in ("t0", "tf", "params", "rtol", "atol", "family"):
        assert np.array_equal(f[k], getattr(e, k)), k
    assert np.allclose(f["y0"], e.y0, rtol=1e-15, atol=0.0)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(name):
    """The oracle on the fixture's own inputs gives the fixture's results bit for bit."""
    f = load(name)
    _, e, method, te = next(c for c in G.cases() if c[0] == name)
    for k in ("t0", "tf", "y0", "params", "rtol", "atol", "family"):
        setattr(e, k, f[k])
    o = G.solve(e, method, te)
    for k in ("status", "accepted", "rejected", "fevals", "y_final", "t_final"):
        assert np.array_equal(o[k], f[k]), k
    if te is not None:
        assert np.array_equal(o["dense"], f["dense"], equal_nan=True)
