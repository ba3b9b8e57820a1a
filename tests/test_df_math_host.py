"""The double-float (FP32 pair) arithmetic of the mixed form's tight-tolerance stages
(df_math.cuh), compiled for the host: products, sums and sin/cos against exact references.
A pair carries about 48 bits; sin and cos are within 1e-12 + 2^-47 |x| of the correctly rounded
value (absolute), far below any tolerance the stages serve."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O

CSRC = os.path.join(O.REPO, "differential-equations_gb300", "csrc")
SO = os.path.join(CSRC, "libdfmath_host.so")
FP = C.POINTER(C.c_float)


@pytest.fixture(scope="module")
def H():
    src = os.path.join(CSRC, "df_math_host.cpp")
    deps = [src] + [os.path.join(CSRC, f) for f in ("df_math.cuh", "f64_tab_math.cuh", "df_tables.inc")]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", SO, src], check=True)
    h = C.CDLL(SO)
    h.degpu_host_df_sincos.argtypes = [FP, FP, O.DP, O.DP, C.c_int64]
    h.degpu_host_df_ops.argtypes = [FP, FP, FP, FP, FP, FP, O.DP, O.DP, C.c_int64]
    h.degpu_host_f64t_sincos.argtypes = [O.DP, O.DP, O.DP, C.c_int64]
    h.degpu_host_df_stage_sum.argtypes = [FP, FP, FP, FP, FP, FP, C.c_int32, C.c_int32, O.DP, C.c_int64]
    return h


def pairs(x):
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo, hi.astype(np.float64) + lo.astype(np.float64)


def fp(a):
    return a.ctypes.data_as(FP)


def test_pair_products_and_sums(H):
    rng = np.random.default_rng(3)
    n = 200_000
    a, b, c = (rng.uniform(-4, 4, n) * 10.0 ** rng.integers(-3, 3, n) for _ in range(3))
    (ah, al, av), (bh, bl, bv), (ch, cl, cv) = pairs(a), pairs(b), pairs(c)
    f, s = np.empty(n), np.empty(n)
    H.degpu_host_df_ops(fp(ah), fp(al), fp(bh), fp(bl), fp(ch), fp(cl), O.p(f), O.p(s), n)
    ref_f = (np.longdouble(av) * np.longdouble(bv) + np.longdouble(cv)).astype(np.float64)
    scale = np.abs(av * bv) + np.abs(cv)
    assert np.max(np.abs(f - ref_f) / scale) < 2.0 ** -44
    ref_s = av - bv
    assert np.max(np.abs(s - ref_s) / (np.abs(av) + np.abs(bv))) < 2.0 ** -46


@pytest.mark.parametrize("last_f32", [0, 1])
def test_pair_stage_sums(H, last_f32):
    """The stage sums' accumulator: y + sum of six products, the state's magnitude against
    increments that range from comparable to 1e-6 of it, and sums that cancel to near zero."""
    rng = np.random.default_rng(5 + last_f32)
    n, m = 100_000, 6
    y = rng.uniform(-4, 4, n) * 10.0 ** rng.integers(-2, 2, n)
    a = rng.uniform(-3, 3, (m, n)) * 10.0 ** rng.integers(-6, 0, (m, n))
    k = rng.uniform(-4, 4, (m, n)) * 10.0 ** rng.integers(-2, 2, (m, n))
    yh, yl, yv = pairs(y)
    ah, al, av = pairs(a)
    kh, kl, kv = pairs(k)
    if last_f32:
        al[-1] = 0.0
        av[-1] = ah[-1].astype(np.float64)
    # a third of the rows cancel: y = -(sum of the terms), rounded to a pair
    cancel = np.arange(n) % 3 == 0
    tot = np.sum(np.longdouble(av) * np.longdouble(kv), axis=0)
    y2 = np.where(cancel, -(tot.astype(np.float64)), y)
    yh, yl, yv = pairs(y2)
    out = np.empty(n)
    H.degpu_host_df_stage_sum(fp(yh), fp(yl), fp(np.ascontiguousarray(ah)), fp(np.ascontiguousarray(al)),
                              fp(np.ascontiguousarray(kh)), fp(np.ascontiguousarray(kl)), m, last_f32, O.p(out), n)
    ref = np.longdouble(yv) + np.sum(np.longdouble(av) * np.longdouble(kv), axis=0)
    scale = np.abs(yv) + np.sum(np.abs(av * kv), axis=0)
    err = np.abs(out - ref.astype(np.float64)) / scale
    assert np.max(err) < 2.0 ** -44


@pytest.mark.parametrize("lo_,hi_", [(-4.0, 4.0), (-60.0, 60.0), (-1e3, 1e3), (-1e-3, 1e-3)])
def test_pair_sin_cos(H, lo_, hi_):
    rng = np.random.default_rng(4)
    n = 100_000
    x = rng.uniform(lo_, hi_, n)
    xh, xl, xv = pairs(x)
    s, c = np.empty(n), np.empty(n)
    H.degpu_host_df_sincos(fp(xh), fp(xl), O.p(s), O.p(c), n)
    rs, rc = np.empty(n), np.empty(n)
    O.lib().oracle_cr_sincos_batch(O.p(xv), O.p(rs), O.p(rc), n)
    # the FP32 parts of the small-angle series bound the error near 1e-12; the reduction's FP32
    # tail adds 2^-47 |x|
    bound = 1e-12 + 2.0 ** -47 * max(abs(lo_), abs(hi_))
    assert np.max(np.abs(s - rs)) < bound
    assert np.max(np.abs(c - rc)) < bound
    small = np.abs(xv) < 1e-2  # near zero sin keeps its relative accuracy
    if small.any():
        assert np.max(np.abs(s[small] - rs[small]) / np.abs(rs[small])) < 5e-12


@pytest.mark.parametrize("lo_,hi_", [(-4.0, 4.0), (-60.0, 60.0), (-1e6, 1e6), (-1e-3, 1e-3)])
def test_f64_table_sin_cos(H, lo_, hi_):
    """The plain FP64 form's table-driven sin and cos: within one unit in the last place of the
    correctly rounded value, and equal to it on at least 97 % of arguments."""
    rng = np.random.default_rng(8)
    n = 200_000
    x = rng.uniform(lo_, hi_, n)
    s, c = np.empty(n), np.empty(n)
    H.degpu_host_f64t_sincos(O.p(x), O.p(s), O.p(c), n)
    rs, rc = np.empty(n), np.empty(n)
    O.lib().oracle_cr_sincos_batch(O.p(x), O.p(rs), O.p(rc), n)
    for got, ref in ((s, rs), (c, rc)):
        assert np.all(np.abs(got - ref) <= np.spacing(np.abs(ref)))
        assert np.mean(got == ref) >= 0.97
