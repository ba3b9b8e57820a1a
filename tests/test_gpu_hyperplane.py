"""Hyperplane crossing detection on the device (degpu_solve_ensemble_hyperplane) against the
oracle's restatement of the crate's HyperplaneCrossingSolout (src/solout/hyperplane.rs): with FP64
parity arithmetic every crossing count, time and state is bit for bit the oracle's (the normal's
scaling to unit length included); the fast and mixed forms find the same crossings within their
accuracy."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W
from test_gpu_crossing import assert_same, cfg_for, family_ensemble, gpu_solve_crossing

pytestmark = pytest.mark.gpu
R = abi.RHS


def gpu_plane(e, cfg, comps, point, normal, direction, max_points):
    hp = abi.make_hyperplane(comps, point, normal, direction, max_points)
    return gpu_solve_crossing(e, cfg, "degpu_solve_ensemble_hyperplane", hp, max_points)


def oracle_plane(e, cfg, comps, point, normal, direction, max_points):
    b = O.Batch(e.rhs_id, e.dim, e.params.shape[0], e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, family=e.family)
    return O.solve_hyperplane(b, cfg, comps, point, normal, direction, max_points)


# planes through each family's typical orbit, with unnormalised normals
PLANES = {
    "VAN_DER_POL": ([0, 1], [0.5, 0.0], [1.0, 0.7]),
    "PENDULUM": ([1, 0], [0.0, 0.0], [2.0, -0.3]),
    "LORENZ": ([0, 1, 2], [0.0, 0.0, 27.0], [0.4, 0.4, 1.0]),
}


@pytest.mark.parametrize("fam", ["VAN_DER_POL", "PENDULUM", "LORENZ"])
@pytest.mark.parametrize("method,h0", [(abi.DOPRI5, 0.0), (abi.DOP853, 0.0), (abi.RK4, 1e-3),
                                       (abi.RKF45, 0.0), (abi.CASH_KARP, 0.0)])
def test_hyperplane_parity(fam, method, h0):
    e = family_ensemble(fam, 600, first=3000)
    cfg = cfg_for(method, h0=h0)
    comps, point, normal = PLANES[fam]
    g = gpu_plane(e, cfg, comps, point, normal, abi.CROSS_BOTH, 3)
    o = oracle_plane(e, cfg, comps, point, normal, abi.CROSS_BOTH, 3)
    assert np.mean(o["cross_count"] > 0) > 0.5
    assert np.any(o["cross_count"] > 3)  # capacity overflow is exercised
    assert_same(g, o)


@pytest.mark.parametrize("direction", [abi.CROSS_POSITIVE, abi.CROSS_NEGATIVE])
def test_hyperplane_direction_and_family_map_parity(direction):
    e = W.config1(n=900, first=12000)
    e.tf = np.minimum(e.tf, 10.0)
    cfg = cfg_for(abi.DOP853, dense_mode=abi.DENSE_HAIRER)
    g = gpu_plane(e, cfg, [0, 1], [0.1, -0.2], [1.0, 1.0], direction, 6)
    o = oracle_plane(e, cfg, [0, 1], [0.1, -0.2], [1.0, 1.0], direction, 6)
    assert_same(g, o)


def test_hyperplane_cr3bp_example_parity():
    """The crate's CR3BP example (examples/ode/07_cr3bp/main.rs): plane through (1, 0, 0) with
    normal (0.5, 0.5, 0) on the position, DOP853; an ensemble around its near-rectilinear orbit."""
    n = 256
    rng = np.random.default_rng(7)
    mu = 0.012150585609624
    base = np.array([1.021881345465263, 0.0, -0.182, 0.0, -0.102950816739606, 0.0])
    y0 = base[:, None] * (1.0 + 1e-3 * rng.standard_normal((6, n)))
    y0[1] = 0.0
    y0[3] = 0.0
    y0[5] = 0.0
    period = 1.509263667286943
    rtol = 10.0 ** rng.uniform(-12, -8, n)
    e = W.Ensemble("cr3bp", abi.DOP853, n, 6, 1, np.zeros(n), np.full(n, 3.0 * period), np.ascontiguousarray(y0),
                   np.full((1, n), mu), rtol, rtol.copy(), rhs_id=R["CR3BP"])
    cfg = cfg_for(abi.DOP853)
    g = gpu_plane(e, cfg, [0, 1, 2], [1.0, 0.0, 0.0], [0.5, 0.5, 0.0], abi.CROSS_BOTH, 8)
    o = oracle_plane(e, cfg, [0, 1, 2], [1.0, 0.0, 0.0], [0.5, 0.5, 0.0], abi.CROSS_BOTH, 8)
    assert np.all(o["cross_count"] >= 3)
    assert_same(g, o)


@pytest.mark.parametrize("precision,tol", [(abi.FP64_FAST, 1e-7), (abi.MIXED, 3e-3)])
def test_hyperplane_fast_and_mixed(precision, tol):
    """Non-chaotic Van der Pol: the same crossings, at times within the form's accuracy."""
    e = family_ensemble("VAN_DER_POL", 500, first=20000)
    e.rtol[:] = 1e-8
    e.atol[:] = 1e-10
    comps, point, normal = PLANES["VAN_DER_POL"]
    g = gpu_plane(e, cfg_for(abi.DOPRI5, precision), comps, point, normal, abi.CROSS_BOTH, 10)
    o = oracle_plane(e, cfg_for(abi.DOPRI5), comps, point, normal, abi.CROSS_BOTH, 10)
    assert np.array_equal(g["cross_count"], o["cross_count"])
    m = ~np.isnan(o["cross_t"])
    assert np.array_equal(m, ~np.isnan(g["cross_t"]))
    assert np.max(np.abs(g["cross_t"][m] - o["cross_t"][m])) < tol


def test_hyperplane_bad_input():
    pytest.importorskip("torch")
    lib = abi.load()
    cfg = cfg_for(abi.DOPRI5)
    prob = abi.Problem(rhs_id=R["VAN_DER_POL"], dim=2, n_params=1)
    bi = abi.BatchIn(n=4)
    bo = abi.BatchOut()
    co = abi.CrossingOut()
    for hp in (abi.make_hyperplane([0, 2], [0, 0], [1, 1]),  # component >= dim
               abi.Hyperplane(dim=0, max_points=4),  # no component
               abi.Hyperplane(dim=9, max_points=4),  # beyond the maximum
               abi.make_hyperplane([0], [0], [1], direction=2)):
        assert lib.degpu_solve_ensemble_hyperplane(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(hp),
                                                   C.byref(bo), C.byref(co), None) == abi.BAD_INPUT
    assert lib.degpu_solve_ensemble_hyperplane(C.byref(prob), C.byref(cfg), C.byref(bi), None, C.byref(bo),
                                               C.byref(co), None) == abi.BAD_INPUT


def test_ivp_builder_hyperplane_and_host_entry():
    """IVP::ode(..).method(..).hyperplane_crossing(point, normal, extractor, Both).solve() on the
    harmonic oscillator: the plane x + v = 0 is crossed at pi/4 + j pi; the host entry point
    returns what the device entry point returns."""
    import degpu

    m = degpu.ExplicitRungeKutta.dop853().rtol(1e-11).atol(1e-11).dense_mode(abi.DENSE_HAIRER)
    sol = degpu.IVP.ode(degpu.System.harmonic(1.0), 0.0, 10.0, [1.0, 0.0]).method(m) \
        .hyperplane_crossing([0.0, 0.0], [1.0, 1.0], [0, 1]).solve()
    assert sol.status == "Complete"
    assert np.allclose(sol.t, [math.pi / 4 + j * math.pi for j in range(3)], rtol=0, atol=1e-9)

    e = family_ensemble("LORENZ", 300, first=777)
    cfg = cfg_for(abi.DOPRI5)
    comps, point, normal = PLANES["LORENZ"]
    g = gpu_plane(e, cfg, comps, point, normal, abi.CROSS_BOTH, 5)
    meth = degpu.ExplicitRungeKutta(abi.DOPRI5)
    meth.cfg = cfg
    r, (ct, cy, cc) = degpu.solve_ensemble_hyperplane(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol,
                                                      meth, comps, point, normal, abi.CROSS_BOTH, 5)
    assert np.array_equal(cc, g["cross_count"])
    assert np.array_equal(ct, g["cross_t"], equal_nan=True) and np.array_equal(cy, g["cross_y"], equal_nan=True)
    assert np.array_equal(r.accepted, g["accepted"]) and np.array_equal(r.y_final, g["y_final"])
