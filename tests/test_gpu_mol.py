"""The general method-of-lines path on the device (degpu_mol_rhs / degpu_mol_rk4) against the
oracle's restatement of the crate's SemiDiscretePde::diff (src/pde/semi_discrete.rs:250-287) and
its fixed RK4 solve: the crate's own MOL tests (tests/pde/method_of_lines.rs:36-157), faces of
every kind on one and two axes, and Gray-Scott on the full 4096 x 4096 periodic grid for two
steps.  FP64 parity arithmetic equals the oracle bit for bit."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu

D, N, P = abi.BC_DIRICHLET, abi.BC_NEUMANN, abi.BC_PERIODIC


def dev(torch, a, dt=None):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt or torch.float64, device="cuda:0")


def gpu_rhs(m, y, t=0.0, precision=abi.FP64_PARITY):
    torch = pytest.importorskip("torch")
    dt = torch.float32 if precision == abi.MIXED else torch.float64
    yd = dev(torch, y, dt)
    dd = torch.full_like(yd, float("nan"))
    s = torch.cuda.Stream()
    rc = abi.load().degpu_mol_rhs(C.byref(m), precision, C.c_double(t), C.c_void_p(yd.data_ptr()),
                                  C.c_void_p(dd.data_ptr()), C.c_void_p(s.cuda_stream))
    s.synchronize()
    assert rc == abi.OK, rc
    return dd.cpu().numpy().astype(np.float64)


def gpu_rk4(m, y, t0, tf, h, precision=abi.FP64_PARITY):
    torch = pytest.importorskip("torch")
    dt = torch.float32 if precision == abi.MIXED else torch.float64
    yd = dev(torch, y, dt)
    st = C.c_int64(-1)
    s = torch.cuda.Stream()
    rc = abi.load().degpu_mol_rk4(C.byref(m), precision, C.c_double(t0), C.c_double(tf), C.c_double(h),
                                  C.c_void_p(yd.data_ptr()), C.byref(st), C.c_void_p(s.cuda_stream))
    s.synchronize()
    assert rc == abi.OK, rc
    return yd.cpu().numpy().astype(np.float64), st.value


def oracle_rhs(m, y, t=0.0):
    y = np.ascontiguousarray(y, dtype=np.float64)
    d = np.zeros_like(y)
    assert O.lib().oracle_mol_rhs(C.byref(m), t, O.p(y), O.p(d), 8) == 0
    return d


def oracle_rk4(m, y, t0, tf, h):
    y = np.array(y, dtype=np.float64)
    st = C.c_int64(-1)
    assert O.lib().oracle_mol_rk4(C.byref(m), t0, tf, h, O.p(y), C.byref(st), 8) == 0
    return y, st.value


def heat(n, faces, alpha=1.0):
    return abi.make_mol(abi.PDE_DIFFUSION, [n], [0.0], [1.0 / (n - 1)], [faces], [alpha], 1)


def test_heat_equation_mode():
    """method_of_lines_matches_heat_equation_mode: alpha = 0.1, 41 nodes, zero Dirichlet faces,
    u0 = sin(pi x), RK4 h = 1e-4 to t = 0.02; within 5e-4 of the decaying mode."""
    m = heat(41, [(D, [0.0]), (D, [0.0])], alpha=0.1)
    x = np.array([1.0 / 40 * i for i in range(41)])
    u0 = np.sin(np.pi * x)
    g, gs = gpu_rk4(m, u0, 0.0, 0.02, 1e-4)
    o, os_ = oracle_rk4(m, u0, 0.0, 0.02, 1e-4)
    assert gs == os_ == 200
    assert np.array_equal(g, o)
    assert np.max(np.abs(g - np.exp(-0.1 * np.pi ** 2 * 0.02) * np.sin(np.pi * x))) < 5e-4


def test_dirichlet_boundaries_are_held_fixed():
    m = heat(5, [(D, [2.0]), (D, [-1.0])])
    y = np.array([2.0, 1.0, 0.0, -0.5, -1.0])
    g = gpu_rhs(m, y)
    assert g[0] == 0.0 and g[-1] == 0.0
    assert np.array_equal(g, oracle_rhs(m, y))


def test_fixed_size_state():
    m = heat(5, [(D, [0.0]), (D, [0.0])])
    y = np.array([0.0, 1.0, 0.0, -1.0, 0.0])
    g = gpu_rhs(m, y)
    assert g[0] == 0.0 and g[4] == 0.0 and abs(g[2]) < 1e-12
    assert np.array_equal(g, oracle_rhs(m, y))


def test_vector_field_state():
    """method_of_lines_accepts_vector_field_state: CoupledDiffusion (diffusivities 1, 2), three
    nodes, Dirichlet faces (0, 1) and (1, 0): du/dt at the middle node is (-0.25, 4.25)."""
    m = abi.make_mol(abi.PDE_COUPLED_DIFFUSION, [3], [0.0], [0.5], [[(D, [0.0, 1.0]), (D, [1.0, 0.0])]],
                     [1.0, 2.0], 2)
    y = np.array([0.0, 1.0, 0.5, 0.25, 1.0, 0.0])
    g = gpu_rhs(m, y)
    assert list(g[[0, 1, 4, 5]]) == [0.0, 0.0, 0.0, 0.0]
    assert abs(g[2] + 0.25) < 1e-12 and abs(g[3] - 4.25) < 1e-12
    assert np.array_equal(g, oracle_rhs(m, y))


def test_neumann_boundary_uses_prescribed_gradient():
    m = heat(5, [(N, [0.0]), (N, [0.0])])
    dx = 1.0 / 4
    y = np.array([1.0, 2.0, 2.0, 2.0, 2.0])
    g = gpu_rhs(m, y)
    assert abs(g[0] - (1.0 / dx) / dx) < 1e-12
    assert np.array_equal(g, oracle_rhs(m, y))


FACES_2D = {
    "dirichlet_x_neumann_y": [[(D, [1.0, 0.5]), (D, [0.0, -0.5])], [(N, [0.25, 0.0]), (N, [-0.1, 0.3])]],
    "neumann_x_periodic_y": [[(N, [0.0, 0.1]), (N, [0.2, 0.0])], [(P, None), (P, None)]],
    "periodic_both": [[(P, None), (P, None)], [(P, None), (P, None)]],
}


@pytest.mark.parametrize("faces", list(FACES_2D), ids=list(FACES_2D))
@pytest.mark.parametrize("pde", [abi.PDE_DIFFUSION, abi.PDE_COUPLED_DIFFUSION, abi.PDE_GRAY_SCOTT])
def test_two_axes_every_face_kind(pde, faces):
    nx, ny = 37, 29
    params = {abi.PDE_DIFFUSION: [0.7, 1.3], abi.PDE_COUPLED_DIFFUSION: [1.0, 2.0],
              abi.PDE_GRAY_SCOTT: [2e-5, 1e-5, 0.037, 0.06]}[pde]
    dx = [1.0 / (nx - 1), 1.0 / 16]  # a spacing that is a power of two takes the multiplication
    m = abi.make_mol(pde, [nx, ny], [0.0, -0.5], dx, FACES_2D[faces], params, 2)
    rng = np.random.default_rng(pde * 10 + len(faces))
    y = rng.uniform(0.0, 1.0, 2 * nx * ny)
    assert np.array_equal(gpu_rhs(m, y, t=0.3), oracle_rhs(m, y, t=0.3))
    # within the explicit stability limits of diffusion and of the Gray-Scott reaction
    h = min(0.2 * min(dx) ** 2 / max(params[:2]), 0.05)
    g, gs = gpu_rk4(m, y, 0.0, 7.5 * h, h)  # the last of 8 steps is shortened to end at tf
    o, os_ = oracle_rk4(m, y, 0.0, 7.5 * h, h)
    assert gs == os_ == 8
    assert np.array_equal(g, o)


def test_other_precisions_track_parity():
    nx, ny = 64, 48
    m = abi.make_mol(abi.PDE_GRAY_SCOTT, [nx, ny], [0.0, 0.0], [1.0 / 64, 1.0 / 64],
                     FACES_2D["dirichlet_x_neumann_y"], [2e-5, 1e-5, 0.037, 0.06], 2)
    rng = np.random.default_rng(2)
    y = rng.uniform(0.2, 1.0, 2 * nx * ny)
    h = 0.05
    ref, _ = gpu_rk4(m, y, 0.0, 20 * h, h)
    assert np.all(np.isfinite(ref))
    for prec, tol in ((abi.FP64_FAST, 1e-13), (abi.FP64_PLAIN, 1e-13), (abi.MIXED, 1e-5)):
        g, _ = gpu_rk4(m, y, 0.0, 20 * h, h, precision=prec)
        assert np.max(np.abs(g - ref)) < tol, prec


def test_gray_scott_4096_fp64_parity_two_steps():
    """The Gray-Scott configuration (4096 x 4096 periodic, dx = 1/4096, dt = 0.2 dx^2 / Du) for two
    RK4 steps: the general path equals the oracle bit for bit, and equals the dedicated periodic
    Gray-Scott kernels (degpu_gray_scott_rk4) too."""
    torch = pytest.importorskip("torch")
    n = 4096
    p = W.GRAY_SCOTT
    dx = 1.0 / 4096
    dt = 0.2 * dx * dx / p["Du"]
    u0, v0 = W.gray_scott_init(n, n)
    y = np.empty(2 * n * n)
    y[0::2] = u0.ravel()
    y[1::2] = v0.ravel()
    m = abi.make_mol(abi.PDE_GRAY_SCOTT, [n, n], [0.0, 0.0], [dx, dx], FACES_2D["periodic_both"],
                     [p["Du"], p["Dv"], p["F"], p["k"]], 2)
    g, gs = gpu_rk4(m, y, 0.0, 2 * dt, dt)
    o, os_ = oracle_rk4(m, y, 0.0, 2 * dt, dt)
    assert gs == os_ == 2
    assert np.array_equal(g, o)
    gsp = abi.GrayScott(nx=n, ny=n, dx=dx, Du=p["Du"], Dv=p["Dv"], F=p["F"], k=p["k"])
    u = dev(torch, u0)
    v = dev(torch, v0)
    s = torch.cuda.Stream()
    assert abi.load().degpu_gray_scott_rk4(C.byref(gsp), abi.FP64_PARITY, C.c_double(0.0), C.c_double(dt), 2,
                                           C.c_void_p(u.data_ptr()), C.c_void_p(v.data_ptr()),
                                           C.c_void_p(s.cuda_stream)) == abi.OK
    s.synchronize()
    assert np.array_equal(u.cpu().numpy().ravel(), g[0::2]) and np.array_equal(v.cpu().numpy().ravel(), g[1::2])


def test_bad_inputs():
    m = heat(5, [(D, [0.0]), (D, [0.0])])
    y = np.zeros(5)
    lib = abi.load()
    torch = pytest.importorskip("torch")
    yd = dev(torch, y)
    bad_h = lib.degpu_mol_rk4(C.byref(m), abi.FP64_PARITY, C.c_double(0.0), C.c_double(1.0), C.c_double(-0.1),
                              C.c_void_p(yd.data_ptr()), None, None)
    assert bad_h == abi.BAD_INPUT
    m.bc_kind[0][0] = P  # one periodic face without the other
    assert lib.degpu_mol_rhs(C.byref(m), abi.FP64_PARITY, C.c_double(0.0), C.c_void_p(yd.data_ptr()),
                             C.c_void_p(yd.data_ptr()), None) == abi.BAD_INPUT
