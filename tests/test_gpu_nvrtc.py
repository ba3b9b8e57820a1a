"""Run-time right-hand sides (degpu_register_rhs_nvrtc): a system written as CUDA source solves
exactly like the built-in twin of the same equations."""
import ctypes as C

import numpy as np
import pytest

import degpu
from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu

LORENZ_SRC = r"""
template <class R>
__device__ void my_lorenz(R t, const R* y, R* dydt, const double* p) {
    R sigma = (R)p[0], rho = (R)p[1], beta = (R)p[2];
    R x = y[0], yv = y[1], z = y[2];
    dydt[0] = sigma * (yv - x);
    dydt[1] = x * (rho - z) - yv;
    dydt[2] = x * yv - beta * z;
}
"""


def register(src, name, dim, n_params):
    lib = abi.load()
    rid = C.c_int32(0)
    log = C.create_string_buffer(1 << 16)
    rc = lib.degpu_register_rhs_nvrtc(src.encode(), name.encode(), dim, n_params, C.byref(rid), log, len(log))
    assert rc == abi.OK, log.value.decode()
    return rid.value


@pytest.mark.parametrize("precision,kernel", [(abi.FP64_PARITY, abi.KERNEL_THREAD),
                                              (abi.FP64_PARITY, abi.KERNEL_PERSISTENT),
                                              (abi.MIXED, abi.KERNEL_PERSISTENT)])
def test_nvrtc_lorenz_matches_builtin(precision, kernel):
    rid = register(LORENZ_SRC, "my_lorenz", 3, 3)
    assert rid >= abi.RHS_NVRTC_BASE
    e = W.config0(n=1024)
    m = degpu.ExplicitRungeKutta(abi.DOPRI5)
    m.cfg.precision, m.cfg.kernel, m.cfg.max_steps = precision, kernel, 10_000_000
    a = degpu.solve_ensemble(rid, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m)
    b = degpu.solve_ensemble(abi.RHS["LORENZ"], 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m)
    assert np.array_equal(a.status, b.status)
    assert np.array_equal(a.accepted, b.accepted) and np.array_equal(a.rejected, b.rejected)
    assert np.array_equal(a.y_final, b.y_final)
    d, p = C.c_int32(), C.c_int32()
    assert abi.load().degpu_rhs_info(rid, C.byref(d), C.byref(p)) == abi.OK and (d.value, p.value) == (3, 3)


def test_nvrtc_compile_error_reported():
    lib = abi.load()
    rid = C.c_int32(0)
    log = C.create_string_buffer(1 << 16)
    rc = lib.degpu_register_rhs_nvrtc(b"this is not cuda", b"f", 2, 0, C.byref(rid), log, len(log))
    assert rc == abi.BAD_INPUT
    assert len(log.value) > 0


PENDULUM_SRC = r"""
template <class R>
__device__ void my_pendulum(R t, const R* y, R* dydt, const double* p) {
    R gamma = (R)p[0], A = (R)p[1], W = (R)p[2];
    dydt[0] = y[1];
    dydt[1] = -gamma * y[1] - sin(y[0]) + A * cos(W * t);
}
"""

DECAY_SRC = r"""
template <class R>
__device__ void my_decay(R t, const R* y, R* dydt, const double* p) {
    dydt[0] = -(R)p[0] * y[0] * exp(-t);
}
"""


def register_with_log(src, name, dim, n_params):
    lib = abi.load()
    rid = C.c_int32(0)
    log = C.create_string_buffer(1 << 16)
    rc = lib.degpu_register_rhs_nvrtc(src.encode(), name.encode(), dim, n_params, C.byref(rid), log, len(log))
    assert rc == abi.OK, log.value.decode()
    return rid.value, log.value.decode()


def test_nvrtc_pair_build_tight_class_tracks_fp64():
    """A source with sin/cos builds for FP32 pairs too: the tight class of a MIXED DOPRI5 solve
    (rtol below the bound) follows the FP64 result at the same tolerances."""
    rid, log = register_with_log(PENDULUM_SRC, "my_pendulum", 2, 3)
    assert "no FP32-pair build" not in log
    e = W.config1(n=3 * 600, first=4242)
    e = e.subset(np.nonzero(e.family == abi.RHS["PENDULUM"])[0])
    e.tf = np.minimum(e.tf, 20.0)
    e.rtol = W.logU(13, np.arange(e.n), 1, 1e-10, 1e-7)
    e.atol = 1e-2 * e.rtol
    out = {}
    for prec in (abi.MIXED, abi.FP64_FAST):
        m = degpu.ExplicitRungeKutta(abi.DOPRI5)
        m.cfg.precision, m.cfg.kernel, m.cfg.max_steps = prec, abi.KERNEL_THREAD, 10_000_000
        out[prec] = degpu.solve_ensemble(rid, 2, e.t0, e.tf, e.y0[:2], e.params, e.rtol, e.atol, m)
    a, b = out[abi.MIXED], out[abi.FP64_FAST]
    ok = (a.status == abi.COMPLETE) & (b.status == abi.COMPLETE)
    assert ok.mean() > 0.99
    rel = np.max(np.abs(a.y_final[:, ok] - b.y_final[:, ok]), axis=0) / \
        np.maximum(np.max(np.abs(b.y_final[:, ok]), axis=0), 1e-300)
    assert np.median(rel) < 1e-8


def test_nvrtc_source_without_pair_overloads_still_solves_mixed():
    """A source that calls a function with no pair overload (exp) registers without its pair
    build; its tight class runs in FP64 fast arithmetic, equal to an FP64_FAST solve."""
    rid, log = register_with_log(DECAY_SRC, "my_decay", 1, 1)
    assert "no FP32-pair build" in log
    n = 256
    t0, tf = np.zeros(n), np.full(n, 3.0)
    y0 = np.ones((1, n))
    p = np.linspace(0.5, 2.0, n).reshape(1, n)
    rtol = np.full(n, 1e-9)
    atol = 1e-2 * rtol
    res = {}
    for prec in (abi.MIXED, abi.FP64_FAST):
        m = degpu.ExplicitRungeKutta(abi.DOPRI5)
        m.cfg.precision, m.cfg.kernel = prec, abi.KERNEL_THREAD
        res[prec] = degpu.solve_ensemble(rid, 1, t0, tf, y0, p, rtol, atol, m)
    assert np.array_equal(res[abi.MIXED].y_final, res[abi.FP64_FAST].y_final)
    assert np.array_equal(res[abi.MIXED].accepted, res[abi.FP64_FAST].accepted)
    exact = np.exp(-p[0] * (1.0 - np.exp(-3.0)))
    assert np.max(np.abs(res[abi.FP64_FAST].y_final[0] - exact)) < 1e-7
