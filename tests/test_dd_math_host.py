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
    deps = [src, os.path.join(CSRC, "dd_math.cuh"), os.path.join(CSRC, "dd_tables.inc"),
            os.path.join(CSRC, "f32_math.cuh")]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", SO, src], check=True)
    h = C.CDLL(SO)
    h.degpu_host_pow_ctrl.argtypes = [O.DP, C.c_double, O.DP, C.c_int64]
    h.degpu_host_pow_ctrl_neg.argtypes = [O.DP, C.c_double, O.DP, C.c_int64]
    h.degpu_host_pow_residual.argtypes = [O.DP, O.DP, C.c_int, O.DP, C.c_int64]
    h.degpu_host_sincos_cr.argtypes = [O.DP, O.DP, O.DP, C.c_int64]
    FP = C.POINTER(C.c_float)
    h.degpu_host_sincos_f32.argtypes = [FP, FP, FP, C.c_int64]
    return h


@pytest.mark.parametrize("y", [0.2, -0.2, 0.125, -0.125, 1 / 6, -1 / 6, 1 / 7, -1 / 7, 1 / 9, -1 / 9])
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


@pytest.mark.parametrize("y", [-0.2, -0.125])
def test_pow_ctrl_neg_correctly_rounded(H, y):
    """The plain path's controller power (FP32 start from the bit pattern, FP32 logarithm in the
    binary64-exponent factor, Ziv's test with an FP64 logarithm fallback) equals the correctly
    rounded value, on random inputs, near powers of two and near 1."""
    rng = np.random.default_rng(21)
    n = 400_000
    x = np.exp(rng.uniform(np.log(1e-240), np.log(1e240), n))
    x[: n // 2] = np.exp(rng.uniform(-12, 12, n // 2))
    x[:1000] = 2.0 ** rng.integers(-700, 700, 1000)            # results that are powers of two
    x[1000:2000] = 1.0 + rng.uniform(-1e-12, 1e-12, 1000)      # ln x near 0
    x[2000:3000] = np.nextafter(2.0 ** (5 * rng.integers(-100, 100, 1000)), 0.0)
    out = np.empty(n)
    H.degpu_host_pow_ctrl_neg(O.p(x), y, O.p(out), n)
    ref = np.empty(n)
    O.lib().oracle_cr_pow_batch(O.p(x), O.p(np.full(n, y)), O.p(ref), n)
    assert np.array_equal(out, ref)
    # outside the direct range it defers to pow_ctrl
    x2 = np.array([1e-300, 1e300, 0.0, np.inf, np.nan])
    out2 = np.empty(5)
    H.degpu_host_pow_ctrl_neg(O.p(x2), y, O.p(out2), 5)
    ref2 = np.array([O.lib().oracle_cr_pow(v, y) for v in x2])
    assert np.array_equal(out2, ref2, equal_nan=True)


@pytest.mark.parametrize("q", [5, 8])
def test_pow_residual_fixed_point_exact(H, q):
    """The controller power's residual e = 1 - x s^q, formed in 128-bit fixed point on the
    integer pipe, against exact rational arithmetic: e is the exact residual rounded toward zero to
    53 bits (the fixed-point truncation, below 2^-120, never shows), on starting values s within
    2^-19 of x^(-1/q) and exactly on x^(-1/q) rounded, across the exponent range."""
    from fractions import Fraction
    H.degpu_host_pow_residual.argtypes = [O.DP, O.DP, C.c_int, O.DP, C.c_int64]
    rng = np.random.default_rng(5 + q)
    n = 3000
    x = np.exp(rng.uniform(np.log(2.0 ** -800), np.log(2.0 ** 800), n))
    x[:200] = 2.0 ** rng.integers(-790, 790, 200)
    s = x ** (-1.0 / q)
    s[n // 2:] *= 1.0 + rng.uniform(-2.0 ** -19, 2.0 ** -19, n - n // 2)
    e = np.empty(n)
    H.degpu_host_pow_residual(O.p(x), O.p(s), q, O.p(e), n)
    for xi, si, ei in zip(x, s, e):
        exact = 1 - Fraction(xi) * Fraction(si) ** q
        if exact == 0:
            assert ei == 0.0
            continue
        assert np.isfinite(ei) and Fraction(ei) * exact >= 0           # same sign
        assert abs(Fraction(ei)) <= abs(exact)                          # toward zero
        assert abs(exact - Fraction(ei)) < abs(exact) * Fraction(1, 2 ** 52)  # within 53 bits
    # outside [1/2, 2) the residual is refused
    bad = np.array([1.0, 2.0 ** 10]), np.array([2.0, 1.0])
    out = np.empty(2)
    H.degpu_host_pow_residual(O.p(bad[0]), O.p(bad[1]), q, O.p(out), 2)
    assert np.all(np.isnan(out))


def test_pow_ctrl_special_values(H):
    x = np.array([0.0, np.inf, 1.0, np.nan, 5e-324, 1.7976931348623157e308])
    for y in (0.2, -0.2, 0.125, -0.125, 1 / 6, -1 / 6, 1 / 7, -1 / 7, 1 / 9, -1 / 9):
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


@pytest.mark.parametrize("lo,hi", [(-1e-3, 1e-3), (-3.2, 3.2), (-200, 200), (-99999, 99999)])
def test_sincos_f32_mixed_form(H, lo, hi):
    """The mixed form's FP32 sin/cos (f32_math.cuh): within 2 units of the FP32 spacing of the
    exact value (a correctly rounded FP32 result measures 1.4 the same way)."""
    rng = np.random.default_rng(13)
    n = 400_000
    x = rng.uniform(lo, hi, n).astype(np.float32)
    s, c = np.empty_like(x), np.empty_like(x)
    FP = C.POINTER(C.c_float)
    H.degpu_host_sincos_f32(x.ctypes.data_as(FP), s.ctypes.data_as(FP), c.ctypes.data_as(FP), n)
    xd = x.astype(np.float64)
    for got, ref in ((s, np.sin(xd)), (c, np.cos(xd))):
        spacing = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
        assert np.max(np.abs(got.astype(np.float64) - ref) / spacing) <= 2.0


def test_sincos_f32_falls_back_beyond_its_range(H):
    x = np.array([1.0e5, -3.0e7, np.inf, np.nan, 0.0, -0.0], dtype=np.float32)
    s, c = np.empty_like(x), np.empty_like(x)
    FP = C.POINTER(C.c_float)
    H.degpu_host_sincos_f32(x.ctypes.data_as(FP), s.ctypes.data_as(FP), c.ctypes.data_as(FP), len(x))
    assert np.allclose(s[:2], np.sin(x[:2].astype(np.float64)), atol=1e-6)
    assert np.isnan(s[2]) and np.isnan(s[3]) and np.isnan(c[2]) and np.isnan(c[3])
    # sin(+-0) is a zero (its sign is not kept); cos(+-0) is 1 within one unit in the last place
    assert s[4] == 0.0 and s[5] == 0.0
    assert abs(float(c[4]) - 1.0) <= 2.0 ** -24 and c[5] == c[4]
