"""Crossing detection on the device (degpu_solve_ensemble_crossing) against the oracle's
restatement of the crate's CrossingSolout (src/solout/crossing.rs:200-330): with FP64 parity
arithmetic every crossing count, time and state is bit for bit the oracle's; the fast and mixed
forms locate the same crossings within their accuracy."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu
R = abi.RHS


def gpu_crossing(e, cfg, comp, thr, direction, max_points):
    cr = abi.Crossing(component=comp, direction=direction, max_points=max_points, threshold=thr)
    return gpu_solve_crossing(e, cfg, "degpu_solve_ensemble_crossing", cr, max_points)


def gpu_solve_crossing(e, cfg, fn, spec, max_points):
    """One device-pointer crossing entry point (component or hyperplane spec) on torch tensors."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    keep = dict(t0=T(e.t0), tf=T(e.tf), y0=T(e.y0), params=T(e.params), rtol=T(e.rtol), atol=T(e.atol))
    if e.family is not None:
        keep["family"] = T(e.family, torch.int32)
    bi = abi.BatchIn(n=e.n, t0=abi.ptr(keep["t0"]), tf=abi.ptr(keep["tf"]), y0=abi.ptr(keep["y0"]),
                     params=abi.ptr(keep["params"]), rtol=abi.ptr(keep["rtol"]), atol=abi.ptr(keep["atol"]),
                     family=abi.ptr(keep.get("family"), C.c_int32), n_eval=0)
    E = lambda *shape, dt=torch.float64: torch.empty(shape, dtype=dt, device=dev)
    out = dict(y_final=E(e.dim, e.n), t_final=E(e.n), accepted=E(e.n, dt=torch.int64),
               rejected=E(e.n, dt=torch.int64), fevals=E(e.n, dt=torch.int64), status=E(e.n, dt=torch.int32),
               cross_t=E(max_points, e.n), cross_y=E(max_points, e.dim, e.n), cross_count=E(e.n, dt=torch.int32))
    bo = abi.BatchOut(y_final=abi.ptr(out["y_final"]), t_final=abi.ptr(out["t_final"]),
                      accepted=abi.ptr(out["accepted"], C.c_int64), rejected=abi.ptr(out["rejected"], C.c_int64),
                      fevals=abi.ptr(out["fevals"], C.c_int64), status=abi.ptr(out["status"], C.c_int32))
    co = abi.CrossingOut(t=abi.ptr(out["cross_t"]), y=abi.ptr(out["cross_y"]),
                         count=abi.ptr(out["cross_count"], C.c_int32))
    prob = abi.Problem(rhs_id=e.rhs_id, dim=e.dim, n_params=e.params.shape[0])
    stream = torch.cuda.Stream()
    rc = getattr(abi.load(), fn)(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(spec), C.byref(bo), C.byref(co),
                                 C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    assert rc == abi.OK, rc
    return {k: v.cpu().numpy() for k, v in out.items()}


def oracle_crossing(e, cfg, comp, thr, direction, max_points):
    b = O.Batch(e.rhs_id, e.dim, e.params.shape[0], e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, family=e.family)
    return O.solve_crossing(b, cfg, comp, thr, direction, max_points)


def family_ensemble(fam, n, first=0, tf_max=12.0):
    e = W.config1(n=3 * n, first=first)
    e = e.subset(np.nonzero(e.family == R[fam])[0][:n])
    e.rhs_id = R[fam]
    e.family = None
    e.dim = 3 if fam == "LORENZ" else 2
    e.y0 = np.ascontiguousarray(e.y0[:e.dim])
    e.params = np.ascontiguousarray(e.params[:{"LORENZ": 3, "PENDULUM": 3, "VAN_DER_POL": 1}[fam]])
    e.tf = np.minimum(e.tf, tf_max)
    return e


def cfg_for(method, precision=abi.FP64_PARITY, h0=0.0, dense_mode=abi.DENSE_REFERENCE):
    c = abi.default_cfg(method)
    c.precision, c.h0, c.max_steps, c.dense_mode = precision, h0, 10_000_000, dense_mode
    return c


def assert_same(g, o):
    for k in ("status", "accepted", "rejected", "fevals", "cross_count"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["cross_t"], o["cross_t"], equal_nan=True)
    assert np.array_equal(g["cross_y"], o["cross_y"], equal_nan=True)
    assert np.array_equal(g["y_final"], o["y_final"])


@pytest.mark.parametrize("fam,comp,thr", [("VAN_DER_POL", 0, 0.0), ("PENDULUM", 1, 0.0), ("LORENZ", 2, 25.0)])
@pytest.mark.parametrize("method,h0", [(abi.DOPRI5, 0.0), (abi.DOP853, 0.0), (abi.RK4, 1e-3)])
def test_crossing_parity(fam, comp, thr, method, h0):
    e = family_ensemble(fam, 700)
    cfg = cfg_for(method, h0=h0)
    g = gpu_crossing(e, cfg, comp, thr, abi.CROSS_BOTH, 3)
    o = oracle_crossing(e, cfg, comp, thr, abi.CROSS_BOTH, 3)
    assert np.mean(o["cross_count"] > 0) > 0.5
    assert np.any(o["cross_count"] > 3)  # capacity overflow is exercised
    assert_same(g, o)


@pytest.mark.parametrize("direction", [abi.CROSS_POSITIVE, abi.CROSS_NEGATIVE])
def test_crossing_direction_parity(direction):
    e = family_ensemble("VAN_DER_POL", 400, first=5000)
    cfg = cfg_for(abi.DOP853, dense_mode=abi.DENSE_HAIRER)
    g = gpu_crossing(e, cfg, 1, 0.5, direction, 6)
    o = oracle_crossing(e, cfg, 1, 0.5, direction, 6)
    assert_same(g, o)


def test_crossing_family_map_parity():
    e = W.config1(n=900, first=9000)
    e.tf = np.minimum(e.tf, 10.0)
    cfg = cfg_for(abi.DOPRI5)
    g = gpu_crossing(e, cfg, 0, 0.0, abi.CROSS_BOTH, 8)
    o = oracle_crossing(e, cfg, 0, 0.0, abi.CROSS_BOTH, 8)
    assert_same(g, o)


@pytest.mark.parametrize("precision,tol", [(abi.FP64_FAST, 1e-7), (abi.MIXED, 3e-3)])
def test_crossing_fast_and_mixed(precision, tol):
    """Non-chaotic Van der Pol: the same crossings, at times within the form's accuracy."""
    e = family_ensemble("VAN_DER_POL", 500, first=20000)
    e.rtol[:] = 1e-8
    e.atol[:] = 1e-10
    g = gpu_crossing(e, cfg_for(abi.DOPRI5, precision), 0, 0.0, abi.CROSS_BOTH, 10)
    o = oracle_crossing(e, cfg_for(abi.DOPRI5), 0, 0.0, abi.CROSS_BOTH, 10)
    assert np.array_equal(g["cross_count"], o["cross_count"])
    m = ~np.isnan(o["cross_t"])
    assert np.array_equal(m, ~np.isnan(g["cross_t"]))
    assert np.max(np.abs(g["cross_t"][m] - o["cross_t"][m])) < tol


def test_crossing_bad_input():
    torch = pytest.importorskip("torch")
    lib = abi.load()
    e = family_ensemble("VAN_DER_POL", 4)
    cfg = cfg_for(abi.DOPRI5)
    prob = abi.Problem(rhs_id=e.rhs_id, dim=2, n_params=1)
    bi = abi.BatchIn(n=4)
    bo = abi.BatchOut()
    co = abi.CrossingOut()
    bad = abi.Crossing(component=2, direction=0, max_points=4, threshold=0.0)  # component >= dim
    assert lib.degpu_solve_ensemble_crossing(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bad), C.byref(bo),
                                             C.byref(co), None) == abi.BAD_INPUT
    assert lib.degpu_solve_ensemble_crossing(C.byref(prob), C.byref(cfg), C.byref(bi), None, C.byref(bo),
                                             C.byref(co), None) == abi.BAD_INPUT


def test_ivp_builder_crossing_and_host_entry():
    """IVP::ode(..).method(..).crossing(0, 0.0, Both).solve() on the harmonic oscillator: zeros of
    cos t on [0, 10]; the host entry point returns what the device entry point returns."""
    import math

    import degpu

    m = degpu.ExplicitRungeKutta.dop853().rtol(1e-11).atol(1e-11).dense_mode(abi.DENSE_HAIRER)
    sol = degpu.IVP.ode(degpu.System.harmonic(1.0), 0.0, 10.0, [1.0, 0.0]).method(m).crossing(0, 0.0).solve()
    assert sol.status == "Complete"
    assert np.allclose(sol.t, [math.pi / 2 + j * math.pi for j in range(3)], rtol=0, atol=1e-9)
    assert np.allclose([y[0] for y in sol.y], 0.0, atol=1e-9)

    e = family_ensemble("PENDULUM", 300, first=777)
    cfg = cfg_for(abi.DOPRI5)
    g = gpu_crossing(e, cfg, 1, 0.0, abi.CROSS_BOTH, 5)
    meth = degpu.ExplicitRungeKutta(abi.DOPRI5)
    meth.cfg = cfg
    r, (ct, cy, cc) = degpu.solve_ensemble_crossing(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol,
                                                    meth, 1, 0.0, abi.CROSS_BOTH, 5)
    assert np.array_equal(cc, g["cross_count"])
    assert np.array_equal(ct, g["cross_t"], equal_nan=True) and np.array_equal(cy, g["cross_y"], equal_nan=True)
    assert np.array_equal(r.accepted, g["accepted"]) and np.array_equal(r.y_final, g["y_final"])


@pytest.mark.parametrize("fam", ["VAN_DER_POL", "PENDULUM"])
def test_crossing_pair_stages_track_oracle(fam):
    """Mixed DOPRI5 below its bound (rtol 1e-9): the FP32-pair detecting lanes run the crate's FP64
    search on their pair interpolant and find the crate's crossings at the oracle's times, to the
    spread between the pair and FP64 trajectories."""
    e = family_ensemble(fam, 400, first=31000)
    e.rtol[:] = 1e-9
    e.atol[:] = 1e-11
    g = gpu_crossing(e, cfg_for(abi.DOPRI5, abi.MIXED), 0, 0.0, abi.CROSS_BOTH, 10)
    o = oracle_crossing(e, cfg_for(abi.DOPRI5), 0, 0.0, abi.CROSS_BOTH, 10)
    assert np.all(g["status"] == abi.COMPLETE)
    same = g["cross_count"] == o["cross_count"]
    assert same.mean() > 0.99
    m = ~np.isnan(o["cross_t"][:, same])
    dt = np.abs(g["cross_t"][:, same][m] - o["cross_t"][:, same][m])
    assert np.median(dt) < 1e-8 and np.max(dt) < 1e-5
