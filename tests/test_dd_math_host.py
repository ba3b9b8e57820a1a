"""The parity path's correctly rounded pow/sin/cos (dd_math.cuh), compiled for the host, against
the oracle's binary128 evaluations: identical results on random inputs across the ranges an
integrator produces.  Also records how often the host libm differs (the unpinned boundary)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O

CSRC = os.path.join(O.REPO, "differential-equations_gb300", "csrc")
SO = os.path.join(CSRC, "libddmath_host.so")


@pytest.fixture(scope="module")
def H():
    src = os.path.join(CSRC, "dd_math_host.cpp")
    deps = [src, os.path.join(CSRC, "dd_math.cuh"), os.path.join(CSRC, "dd_tables.inc")]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", SO, src], check=True)
    h = C.CDLL(SO)
    h.degpu_host_pow_ctrl.argtypes = [O.DP, C.c_double, O.DP, C.c_int64]
    h.degpu_host_sincos_cr.argtypes = [O.DP, O.DP, O.DP, C.c_int64]
    return h


@pytest.mark.parametrize("y", [0.2, -0.2, 0.125, -0.125])
def test_pow_ctrl_correctly_rounded(H, y):
    rng = np.random.default_rng(11)
    n = 200_000
    x = np.exp(rng.uniform(np.log(1e-300), np.log(1e300), n))
    x[: n // 2] = np.exp(rng.uniform(-12, 12, n // 2))  # the controller's typical range
    out = np.empty(n)
    H.degpu_host_pow_ctrl(O.p(x), y, O.p(out), n)
    ref = np.empty(n)
    yy = np.full(n, y)
    O.lib().oracle_cr_pow_batch(O.p(x), O.p(yy), O.p(ref), n)
    assert np.array_equal(out, ref)


def test_pow_ctrl_special_values(H):
    x = np.array([0.0, np.inf, 1.0, np.nan, 5e-324, 1.7976931348623157e308])
    for y in (0.2, -0.2, 0.125, -0.125):
        out = np.empty(len(x))
        H.degpu_host_pow_ctrl(O.p(x), y, O.p(out), len(x))
        ref = np.array([O.lib().oracle_cr_pow(v, y) for v in x])
        assert np.array_equal(out, ref, equal_nan=True), (y, out, ref)


@pytest.mark.parametrize("lo,hi", [(-10, 10), (-2e4, 2e4), (-1e-6, 1e-6), (-1e6, 1e6)])
def test_sincos_correctly_rounded(H, lo, hi):
    rng = np.random.default_rng(12)
    n = 200_000
    x = rng.uniform(lo, hi, n)
    s, c = np.empty(n), np.empty(n)
    H.degpu_host_sincos_cr(O.p(x), O.p(s), O.p(c), n)
    rs, rc = np.empty(n), np.empty(n)
    O.lib().oracle_cr_sincos_batch(O.p(x), O.p(rs), O.p(rc), n)
    assert np.array_equal(s, rs) and np.array_equal(c, rc)


def test_host_libm_is_not_correctly_rounded_everywhere():
    """The crate's pow goes to the platform libm, which misrounds a small fraction of inputs:
    the reason the parity path fixes pow to the correctly rounded value."""
    rng = np.random.default_rng(13)
    n = 200_000
    x = np.exp(rng.uniform(-12, 12, n))
    yy = np.full(n, -0.2)
    a, b = np.empty(n), np.empty(n)
    O.lib().oracle_cr_pow_batch(O.p(x), O.p(yy), O.p(a), n)
    O.lib().oracle_libm_pow_batch(O.p(x), O.p(yy), O.p(b), n)
    frac = np.mean(a != b)
    assert frac < 0.01
