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
