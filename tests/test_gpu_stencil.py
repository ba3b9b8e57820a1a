"""Gray–Scott method-of-lines path on the GPU against the CPU oracle's restatement of the
crate's SemiDiscretePde::diff (with the periodic extension) and fixed RK4 step."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu


def gs_struct(nx, ny, dx):
    p = W.GRAY_SCOTT
    return abi.GrayScott(nx=nx, ny=ny, dx=dx, Du=p["Du"], Dv=p["Dv"], F=p["F"], k=p["k"])


def small_state(nx, ny, seed=3):
    rng = np.random.default_rng(seed)
    u = 1.0 - 0.5 * rng.random((ny, nx)) * (rng.random((ny, nx)) < 0.1)
    v = 0.25 * rng.random((ny, nx)) * (rng.random((ny, nx)) < 0.1)
    return np.ascontiguousarray(u), np.ascontiguousarray(v)


def gpu_rk4(gs, prec, dt, steps, u, v):
    torch = pytest.importorskip("torch")
    dt_ = torch.float32 if prec == abi.MIXED else torch.float64
    tu = torch.as_tensor(u, dtype=dt_, device="cuda")
    tv = torch.as_tensor(v, dtype=dt_, device="cuda")
    rc = abi.load().degpu_gray_scott_rk4(C.byref(gs), prec, 0.0, dt, steps, C.c_void_p(tu.data_ptr()),
                                         C.c_void_p(tv.data_ptr()), None)
    assert rc == abi.OK
    torch.cuda.synchronize()
    return tu.double().cpu().numpy(), tv.double().cpu().numpy()


# (64, 48): one node per thread; (256, 128): the register-blocked 4 x 4 kernel (nx % 128, ny % 16)
@pytest.mark.parametrize("shape", [(64, 48), (256, 128)])
@pytest.mark.parametrize("dx", [1.0 / 64, 0.013])  # power of two (exact reciprocal) and not
def test_gray_scott_rhs_parity(dx, shape):
    torch = pytest.importorskip("torch")
    nx, ny = shape
    gs = gs_struct(nx, ny, dx)
    u, v = small_state(nx, ny)
    du, dv = np.zeros_like(u), np.zeros_like(v)
    O.lib().oracle_gray_scott_rhs(C.byref(gs), O.p(u), O.p(v), O.p(du), O.p(dv), 1)
    tu, tv = torch.as_tensor(u, device="cuda"), torch.as_tensor(v, device="cuda")
    gu, gv = torch.empty_like(tu), torch.empty_like(tv)
    rc = abi.load().degpu_gray_scott_rhs(C.byref(gs), abi.ptr(tu), abi.ptr(tv), abi.ptr(gu), abi.ptr(gv), None)
    assert rc == abi.OK
    torch.cuda.synchronize()
    assert np.array_equal(gu.cpu().numpy(), du) and np.array_equal(gv.cpu().numpy(), dv)


@pytest.mark.parametrize("shape", [(64, 64), (256, 128)])
@pytest.mark.parametrize("steps", [1, 2, 5])
def test_gray_scott_rk4_parity(steps, shape):
    nx, ny = shape
    dx = 1.0 / 64
    gs = gs_struct(nx, ny, dx)
    dt = 0.2 * dx * dx / W.GRAY_SCOTT["Du"]
    u, v = small_state(nx, ny)
    ou, ov = u.copy(), v.copy()
    O.lib().oracle_gray_scott_rk4(C.byref(gs), 0.0, dt, steps, O.p(ou), O.p(ov), 4)
    gu, gv = gpu_rk4(gs, abi.FP64_PARITY, dt, steps, u, v)
    assert np.array_equal(gu, ou) and np.array_equal(gv, ov)


def test_gray_scott_fp64_fast_and_fp32_accuracy():
    nx, ny = 128, 128
    dx = 1.0 / 128
    gs = gs_struct(nx, ny, dx)
    dt = 0.2 * dx * dx / W.GRAY_SCOTT["Du"]
    u, v = small_state(nx, ny)
    ou, ov = u.copy(), v.copy()
    O.lib().oracle_gray_scott_rk4(C.byref(gs), 0.0, dt, 40, O.p(ou), O.p(ov), 4)
    fu, fv = gpu_rk4(gs, abi.FP64_FAST, dt, 40, u, v)
    assert np.max(np.abs(fu - ou)) < 1e-12 and np.max(np.abs(fv - ov)) < 1e-12
    su, sv = gpu_rk4(gs, abi.MIXED, dt, 40, u, v)
    assert np.max(np.abs(su - ou)) < 1e-5 and np.max(np.abs(sv - ov)) < 1e-5


def test_gray_scott_full_size_properties():
    """4096 x 4096 periodic grid, the benchmark's initial state: FP32 and FP64 stay finite and
    bounded over 50 steps, conserve the symmetry of a shifted start (periodic invariance: solving
    a cyclically shifted grid gives the cyclically shifted result), and agree to FP32 accuracy."""
    torch = pytest.importorskip("torch")
    n = 4096
    dx = 1.0 / 4096
    gs = gs_struct(n, n, dx)
    dt = 0.2 * dx * dx / W.GRAY_SCOTT["Du"]
    u, v = W.gray_scott_init(n, n)
    a_u, a_v = gpu_rk4(gs, abi.FP64_FAST, dt, 50, u, v)
    s_u, s_v = gpu_rk4(gs, abi.FP64_FAST, dt, 50, np.roll(u, (7, 13), (0, 1)), np.roll(v, (7, 13), (0, 1)))
    assert np.array_equal(np.roll(a_u, (7, 13), (0, 1)), s_u) and np.array_equal(np.roll(a_v, (7, 13), (0, 1)), s_v)
    assert np.all(np.isfinite(a_u)) and a_u.min() >= 0.0 and a_u.max() <= 1.0 + 1e-9
    f_u, f_v = gpu_rk4(gs, abi.MIXED, dt, 50, u, v)
    assert np.max(np.abs(f_u - a_u)) < 1e-4 and np.max(np.abs(f_v - a_v)) < 1e-4


def set_fused(on):
    fn = abi.load().degpu_internal_gs_fused_step
    fn.argtypes = [C.c_int]
    fn.restype = C.c_int
    return fn(1 if on else 0)


# (192, 96): fused tiles, but the passes take their one-node-per-thread kernel (nx % 128 != 0)
@pytest.mark.parametrize("shape,steps", [((4096, 4096), 7), ((256, 128), 5), ((192, 96), 3)])
def test_gray_scott_fused_fp32_step_equals_four_passes(shape, steps):
    """The fused FP32 RK4 step (one launch per step, tiles of 64 x 32 nodes with a 4-node halo in
    shared memory, periodic wrap across the grid's edges) against the four-pass kernels: the same
    arithmetic in the same order, so the states agree bit for bit, over an odd number of steps
    (the graph of two steps and a single step after it)."""
    nx, ny = shape
    dx = 1.0 / nx
    gs = gs_struct(nx, ny, dx)
    dt = 0.2 * dx * dx / W.GRAY_SCOTT["Du"]
    u, v = W.gray_scott_init(nx, ny) if nx == 4096 else small_state(nx, ny)
    prev = set_fused(True)
    try:
        fu, fv = gpu_rk4(gs, abi.MIXED, dt, steps, u, v)
        set_fused(False)
        pu, pv = gpu_rk4(gs, abi.MIXED, dt, steps, u, v)
    finally:
        set_fused(prev)
    assert np.array_equal(fu, pu) and np.array_equal(fv, pv)
    assert np.all(np.isfinite(fu)) and not np.array_equal(fu, u)
