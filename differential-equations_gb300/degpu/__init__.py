"""degpu — Python bindings of the GB300 ensemble explicit Runge–Kutta integrator.

Thin ctypes layer over the C ABI (include/degpu.h).  The builder mirrors the crate's surface:

    m = ExplicitRungeKutta.dopri5().rtol(1e-8).atol(1e-10)       # src/methods/erk/mod.rs:165-174
    sol = IVP.ode(System.lorenz(10, 28, 8/3), 0.0, 20.0, [1, 1, 1]).method(m).t_eval(pts).solve()

and `solve_ensemble` solves many instances of a family in one call.  Every solve runs on the GPU
through libdegpu.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import abi

__all__ = ["abi", "ExplicitRungeKutta", "IVP", "System", "EnsembleResult", "solve_ensemble", "DegpuError",
           "Solution", "set_mixed_min_rtol", "mixed_min_rtol", "solve_ensemble_crossing", "solve_ensemble_hyperplane",
           "solve_ensemble_event", "solve_bvp", "BVP", "Shooting", "BvpResult", "write_csv", "rust_debug_f64"]

STATUS_NAMES = {abi.COMPLETE: "Complete", abi.ERR_BAD_INPUT: "BadInput", abi.ERR_MAX_STEPS: "MaxSteps",
                abi.ERR_STEP_SIZE: "StepSize", abi.ERR_STIFFNESS: "Stiffness", abi.INTERRUPTED: "Interrupted",
                abi.ERR_LINEAR_ALGEBRA: "LinearAlgebra"}


class DegpuError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        lib = abi.load()
        super().__init__(f"{what}: {lib.degpu_status_string(code).decode()} ({code})")
        self.code = code


class ExplicitRungeKutta:
    """Method configuration, mirroring ExplicitRungeKutta's constructors and setters
    (src/methods/erk/fixed/mod.rs:69-75, src/methods/erk/dormandprince/mod.rs:45-58,
    src/methods/erk/mod.rs:165-228)."""

    def __init__(self, method: int, h0: float = 0.0):
        self.cfg = abi.default_cfg(method)
        self.cfg.h0 = h0
        self._rtol = 1e-6
        self._atol = 1e-6

    @classmethod
    def rk4(cls, h0: float):
        return cls(abi.RK4, h0)

    @classmethod
    def dopri5(cls):
        return cls(abi.DOPRI5)

    @classmethod
    def dop853(cls):
        return cls(abi.DOP853)

    @classmethod
    def rkf45(cls):  # src/methods/erk/adaptive/mod.rs:43-50
        return cls(abi.RKF45)

    @classmethod
    def cash_karp(cls):  # src/methods/erk/adaptive/mod.rs:51-58
        return cls(abi.CASH_KARP)

    @classmethod
    def rkv655e(cls):
        """Verner's RKV655e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV655E)

    @classmethod
    def rkv656e(cls):
        """Verner's RKV656e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV656E)

    @classmethod
    def rkv766e(cls):
        """Verner's RKV766e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV766E)

    @classmethod
    def rkv767e(cls):
        """Verner's RKV767e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV767E)

    @classmethod
    def rkv877e(cls):
        """Verner's RKV877e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV877E)

    @classmethod
    def rkv878e(cls):
        """Verner's RKV878e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV878E)

    @classmethod
    def rkv988e(cls):
        """Verner's RKV988e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV988E)

    @classmethod
    def rkv989e(cls):
        """Verner's RKV989e pair (src/methods/erk/adaptive/mod.rs, src/tableau/verner.rs)."""
        return cls(abi.RKV989E)

    def rtol(self, v):
        self._rtol = v
        return self

    def atol(self, v):
        self._atol = v
        return self

    def h0(self, v):
        self.cfg.h0 = v
        return self

    def h_min(self, v):
        self.cfg.h_min = v
        return self

    def h_max(self, v):
        self.cfg.h_max = v
        return self

    def max_steps(self, v):
        self.cfg.max_steps = int(v)
        return self

    def safety_factor(self, v):
        self.cfg.safety_factor = v
        return self

    def min_scale(self, v):
        self.cfg.min_scale = v
        return self

    def max_scale(self, v):
        self.cfg.max_scale = v
        return self

    # GPU-specific knobs
    def precision(self, p: int):
        self.cfg.precision = p
        return self

    def kernel(self, k: int):
        self.cfg.kernel = k
        return self

    def dense_mode(self, d: int):
        self.cfg.dense_mode = d
        return self


@dataclass
class System:
    """A built-in right-hand side (a CUDA __device__ twin of `ODE::diff`) and its parameters."""
    rhs_id: int
    params: Sequence[float]
    dim: int

    @staticmethod
    def lorenz(sigma, rho, beta):
        return System(abi.RHS["LORENZ"], [sigma, rho, beta], 3)

    @staticmethod
    def van_der_pol(mu):
        return System(abi.RHS["VAN_DER_POL"], [mu], 2)

    @staticmethod
    def pendulum(gamma, A, Omega):
        return System(abi.RHS["PENDULUM"], [gamma, A, Omega], 2)

    @staticmethod
    def exponential_growth(k):
        return System(abi.RHS["EXP_GROWTH"], [k], 1)

    @staticmethod
    def harmonic(k):
        return System(abi.RHS["HARMONIC"], [k], 2)

    @staticmethod
    def fpu_beta(beta, masses):
        return System(abi.RHS["FPU_BETA"], [beta], 2 * masses)

    @staticmethod
    def brusselator(a, b):
        return System(abi.RHS["BRUSSELATOR"], [a, b], 2)

    @staticmethod
    def pipe_heat(heat_loss_rate, ambient):
        """T'' = b^2 (T - T_amb) as (T, T') (tests/bvp/systems.rs:25-57)."""
        return System(abi.RHS["PIPE_HEAT"], [heat_loss_rate, ambient], 2)

    @staticmethod
    def damped_quadrature(k, m, c):
        """Damped mass-spring system with the dissipated energy as a third component,
        (x, v, W) (examples/ode/17_quadrature/main.rs:41-55)."""
        return System(abi.RHS["DAMPED_QUADRATURE"], [k, m, c], 3)

    @staticmethod
    def cr3bp(mu):
        """Circular restricted three-body problem, state (x, y, z, vx, vy, vz)."""
        return System(abi.RHS["CR3BP"], [mu], 6)


@dataclass
class EnsembleResult:
    y_final: np.ndarray      # [dim, n]
    t_final: np.ndarray      # [n]
    dense: Optional[np.ndarray]  # [n_eval, dim, n]
    accepted: np.ndarray
    rejected: np.ndarray
    fevals: np.ndarray
    status: np.ndarray


def _solve_crossing_host(fn, spec, rhs_id, dim, t0, tf, y0, params, rtol, atol, method, max_points, family,
                         n_params, t_eval=None):
    """One host-pointer detection entry point `fn` (crossing, hyperplane or event) with its spec
    struct: host arrays in, (EnsembleResult, (t, y, count)) out."""
    lib = abi.load()
    y0 = np.asarray(y0, dtype=np.float64)
    n = y0.shape[1]
    bc = lambda v: _f64(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)).copy())
    t0, tf, rtol, atol = bc(t0), bc(tf), bc(rtol), bc(atol)
    y0 = _f64(y0)
    params = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, n)) if params is not None \
        and np.size(params) else np.zeros((1, n))
    np_ = n_params if n_params is not None else params.shape[0]
    fam_a = None if family is None else np.ascontiguousarray(family, dtype=np.int32)
    te = None if t_eval is None or len(t_eval) == 0 else _f64(np.asarray(t_eval, dtype=np.float64))
    ne = 0 if te is None else len(te)
    out = dict(y_final=np.empty((dim, n)), t_final=np.empty(n), dense=np.empty((ne, dim, n)) if ne else None,
               accepted=np.empty(n, np.int64), rejected=np.empty(n, np.int64), fevals=np.empty(n, np.int64),
               status=np.empty(n, np.int32))
    ct, cy, cc = np.empty((max_points, n)), np.empty((max_points, dim, n)), np.empty(n, np.int32)
    prob = abi.Problem(rhs_id=rhs_id, dim=dim, n_params=np_)
    bi = abi.BatchIn(n=n, t0=abi.ptr(t0), tf=abi.ptr(tf), y0=abi.ptr(y0), params=abi.ptr(params),
                     rtol=abi.ptr(rtol), atol=abi.ptr(atol), family=abi.ptr(fam_a, C.c_int32), n_eval=ne,
                     t_eval=abi.ptr(te))
    bo = abi.BatchOut(y_final=abi.ptr(out["y_final"]), t_final=abi.ptr(out["t_final"]), dense=abi.ptr(out["dense"]),
                      accepted=abi.ptr(out["accepted"], C.c_int64), rejected=abi.ptr(out["rejected"], C.c_int64),
                      fevals=abi.ptr(out["fevals"], C.c_int64), status=abi.ptr(out["status"], C.c_int32))
    co = abi.CrossingOut(t=abi.ptr(ct), y=abi.ptr(cy), count=abi.ptr(cc, C.c_int32))
    rc = getattr(lib, fn)(C.byref(prob), C.byref(method.cfg), C.byref(bi), C.byref(spec), C.byref(bo), C.byref(co))
    if rc != abi.OK:
        raise DegpuError(rc, fn)
    return EnsembleResult(**out), (ct, cy, cc)


def solve_ensemble_crossing(rhs_id: int, dim: int, t0, tf, y0, params, rtol, atol, method: ExplicitRungeKutta,
                            component: int, threshold: float, direction: int = abi.CROSS_BOTH,
                            max_points: int = 16, family=None, n_params: Optional[int] = None):
    """Solve n IVPs (host arrays) with crossing detection (degpu_solve_ensemble_crossing_host):
    the crate's `.crossing(component, threshold, direction)` output.  Returns the EnsembleResult
    and (t [max_points, n], y [max_points, dim, n], count [n])."""
    cr = abi.Crossing(component=component, direction=direction, max_points=max_points, threshold=threshold)
    return _solve_crossing_host("degpu_solve_ensemble_crossing_host", cr, rhs_id, dim, t0, tf, y0,
                                params, rtol, atol, method, max_points, family, n_params)


def solve_ensemble_hyperplane(rhs_id: int, dim: int, t0, tf, y0, params, rtol, atol, method: ExplicitRungeKutta,
                              components, point, normal, direction: int = abi.CROSS_BOTH, max_points: int = 16,
                              family=None, n_params: Optional[int] = None):
    """Solve n IVPs (host arrays) with hyperplane crossing detection
    (degpu_solve_ensemble_hyperplane_host): the crate's `.hyperplane_crossing(point, normal,
    extractor, direction)` output with the extractor given as state components
    (pos[j] = y[components[j]]).  Returns what solve_ensemble_crossing returns."""
    hp = abi.make_hyperplane(components, point, normal, direction, max_points)
    return _solve_crossing_host("degpu_solve_ensemble_hyperplane_host", hp, rhs_id, dim, t0, tf, y0,
                                params, rtol, atol, method, max_points, family, n_params)


def solve_ensemble_event(rhs_id: int, dim: int, t0, tf, y0, params, rtol, atol, method: ExplicitRungeKutta,
                         event: "abi.Event", t_eval=None, family=None, n_params: Optional[int] = None):
    """Solve n IVPs (host arrays) with event detection (degpu_solve_ensemble_event_host): the
    crate's `.event(&event)` wrapped around the output times (`t_eval`) or around the default
    per-step output.  Returns the EnsembleResult (dense = the output times) and the event points
    (t [max_points, n], y [max_points, dim, n], count [n]); a terminal event leaves the
    instance's status INTERRUPTED."""
    return _solve_crossing_host("degpu_solve_ensemble_event_host", event, rhs_id, dim, t0, tf, y0, params,
                                rtol, atol, method, event.max_points, family, n_params, t_eval)


@dataclass
class BvpResult:
    solution: EnsembleResult  # the final IVP from the converged y(t0): y_final = y(tf), dense
    y_a: np.ndarray           # [dim, n] converged initial states (NaN where a solve failed)
    iterations: np.ndarray    # [n] Newton iterations
    jacobian: np.ndarray      # [n] Jacobian columns formed


def solve_bvp(rhs_id: int, dim: int, t0, tf, y_guess, params, rtol, atol, method: ExplicitRungeKutta,
              bvp: "abi.Bvp", t_eval=None, n_params: Optional[int] = None) -> BvpResult:
    """Solve n two-point boundary value problems by shooting (degpu_solve_bvp_host): the crate's
    `BVP::ode(&problem, t0, tf, y_guess).method(Shooting::single(erk) | Shooting::multiple(erk))`
    with the boundary rows of `bvp` (abi.make_bvp).  Every IVP of a Newton iteration of the whole
    batch is one ensemble solve on the device."""
    lib = abi.load()
    y_guess = np.asarray(y_guess, dtype=np.float64)
    n = y_guess.shape[1]
    bc = lambda v: _f64(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)).copy())
    t0, tf, rtol, atol = bc(t0), bc(tf), bc(rtol), bc(atol)
    y_guess = _f64(y_guess)
    params = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, n)) if params is not None \
        and np.size(params) else np.zeros((1, n))
    np_ = n_params if n_params is not None else params.shape[0]
    te = None if t_eval is None or len(t_eval) == 0 else _f64(np.asarray(t_eval, dtype=np.float64))
    ne = 0 if te is None else len(te)
    out = dict(y_final=np.empty((dim, n)), t_final=np.empty(n), dense=np.empty((ne, dim, n)) if ne else None,
               accepted=np.empty(n, np.int64), rejected=np.empty(n, np.int64), fevals=np.empty(n, np.int64),
               status=np.empty(n, np.int32))
    ya, it, jac = np.empty((dim, n)), np.empty(n, np.int32), np.empty(n, np.int64)
    prob = abi.Problem(rhs_id=rhs_id, dim=dim, n_params=np_)
    bi = abi.BatchIn(n=n, t0=abi.ptr(t0), tf=abi.ptr(tf), y0=abi.ptr(y_guess), params=abi.ptr(params),
                     rtol=abi.ptr(rtol), atol=abi.ptr(atol), t_eval=abi.ptr(te), n_eval=ne)
    bo = abi.BatchOut(y_final=abi.ptr(out["y_final"]), t_final=abi.ptr(out["t_final"]), dense=abi.ptr(out["dense"]),
                      accepted=abi.ptr(out["accepted"], C.c_int64), rejected=abi.ptr(out["rejected"], C.c_int64),
                      fevals=abi.ptr(out["fevals"], C.c_int64), status=abi.ptr(out["status"], C.c_int32))
    vo = abi.BvpOut(y_a=abi.ptr(ya), iterations=abi.ptr(it, C.c_int32), jacobian=abi.ptr(jac, C.c_int64))
    rc = lib.degpu_solve_bvp_host(C.byref(prob), C.byref(method.cfg), C.byref(bi), C.byref(bvp), C.byref(bo),
                                  C.byref(vo))
    if rc != abi.OK:
        raise DegpuError(rc, "degpu_solve_bvp_host")
    return BvpResult(EnsembleResult(**out), ya, it, jac)


class Shooting:
    """The crate's shooting methods (src/methods/bvp/shooting): Shooting.single(erk) and
    Shooting.multiple(erk).segments(m), with .tolerance() and .max_iterations()."""

    def __init__(self, erk: ExplicitRungeKutta, method: int):
        self.erk, self.method_id, self._segments, self._tol, self._iters = erk, method, 4, 1e-6, 100

    @classmethod
    def single(cls, erk: ExplicitRungeKutta):
        return cls(erk, abi.BVP_SINGLE)

    @classmethod
    def multiple(cls, erk: ExplicitRungeKutta):
        return cls(erk, abi.BVP_MULTIPLE)

    def segments(self, m: int):
        self._segments = m
        return self

    def tolerance(self, tol: float):
        self._tol = tol
        return self

    def max_iterations(self, k: int):
        self._iters = k
        return self


class BVP:
    """Single-instance builder with the crate's shape (src/bvp.rs): BVP.ode(system, t0, tf,
    y_guess, boundary_rows).method(Shooting...).t_eval(pts).solve() -> Solution whose first point
    is y(t0) and last y(tf).  boundary_rows: (side, component, value) with r = y_side[c] - value."""

    def __init__(self, system: System, t0, tf, y_guess, rows):
        self.system, self.t0, self.tf = system, t0, tf
        self.y_guess = np.asarray(y_guess, dtype=np.float64).reshape(-1)
        self.rows = list(rows)
        self._method: Optional[Shooting] = None
        self._t_eval = None

    @classmethod
    def ode(cls, system: System, t0, tf, y_guess, rows):
        return cls(system, t0, tf, y_guess, rows)

    def method(self, m: Shooting):
        self._method = m
        return self

    def t_eval(self, pts):
        self._t_eval = list(pts)
        return self

    def solve(self) -> Solution:
        m = self._method or Shooting.single(ExplicitRungeKutta.dop853())
        d = len(self.y_guess)
        bvp = abi.make_bvp(self.rows, m.method_id, m._segments, m._iters, m._tol)
        r = solve_bvp(self.system.rhs_id, d, [self.t0], [self.tf], self.y_guess.reshape(d, 1),
                      np.asarray(self.system.params, dtype=np.float64).reshape(-1, 1), [m.erk._rtol], [m.erk._atol],
                      m.erk, bvp, t_eval=self._t_eval)
        s = r.solution
        st = STATUS_NAMES.get(int(s.status[0]), str(int(s.status[0])))
        if self._t_eval is not None:
            ts = [float(v) for i, v in enumerate(self._t_eval) if not np.isnan(s.dense[i, 0, 0])]
            ys = [s.dense[i, :, 0].copy() for i in range(len(self._t_eval)) if not np.isnan(s.dense[i, 0, 0])]
        else:
            ts = [float(self.t0), float(s.t_final[0])]
            ys = [r.y_a[:, 0].copy(), s.y_final[:, 0].copy()]
        return Solution(ts, ys, st, int(s.accepted[0]), int(s.rejected[0]), int(s.fevals[0]))


def set_mixed_min_rtol(method: int, min_rtol: float) -> None:
    """Mixed-precision bound of DOPRI5 / DOP853 (degpu_set_mixed_min_rtol): in a MIXED solve an
    instance with rtol below it runs in FP64_FAST arithmetic; 0 disables the split."""
    rc = abi.load().degpu_set_mixed_min_rtol(method, float(min_rtol))
    if rc != abi.OK:
        raise DegpuError(rc, "degpu_set_mixed_min_rtol")


def mixed_min_rtol(method: int) -> float:
    return abi.load().degpu_mixed_min_rtol(method)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape is not None else a


def solve_ensemble(rhs_id: int, dim: int, t0, tf, y0, params, rtol, atol, method: ExplicitRungeKutta,
                   t_eval=None, dims=None, family=None, n_params: Optional[int] = None, rtol_vec=None,
                   atol_vec=None) -> EnsembleResult:
    """Solve n IVPs (host arrays) through degpu_solve_ensemble_host.

    y0 is [dim, n] (structure of arrays), params [n_params, n]; t0, tf, rtol, atol are [n] or
    scalars broadcast to n.  rtol_vec / atol_vec ([dim, n], or [dim] broadcast to every instance)
    are per-component tolerances, the crate's Tolerance::Vector (`.rtol([..])`, `.atol([..])`);
    rtol / atol still order the work lists and choose the precision class of a mixed solve.
    """
    lib = abi.load()
    y0 = np.asarray(y0, dtype=np.float64)
    n = y0.shape[1]
    bc = lambda v: _f64(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)).copy())
    t0, tf, rtol, atol = bc(t0), bc(tf), bc(rtol), bc(atol)
    y0 = _f64(y0)
    params = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, n)) if params is not None \
        and np.size(params) else np.zeros((1, n))
    np_ = n_params if n_params is not None else (params.shape[0] if params is not None else 0)
    te = None if t_eval is None else _f64(t_eval)
    m = 0 if te is None else len(te)
    dims_a = None if dims is None else np.ascontiguousarray(dims, dtype=np.int32)
    fam_a = None if family is None else np.ascontiguousarray(family, dtype=np.int32)
    tv = lambda v: None if v is None else _f64(np.broadcast_to(
        np.asarray(v, dtype=np.float64).reshape(dim, -1), (dim, n)).copy())
    rtv, atv = tv(rtol_vec), tv(atol_vec)
    out = dict(y_final=np.empty((dim, n)), t_final=np.empty(n), dense=np.empty((m, dim, n)) if m else None,
               accepted=np.empty(n, np.int64), rejected=np.empty(n, np.int64), fevals=np.empty(n, np.int64),
               status=np.empty(n, np.int32))
    prob = abi.Problem(rhs_id=rhs_id, dim=dim, n_params=np_)
    bi = abi.BatchIn(n=n, t0=abi.ptr(t0), tf=abi.ptr(tf), y0=abi.ptr(y0), params=abi.ptr(params),
                     rtol=abi.ptr(rtol), atol=abi.ptr(atol), dims=abi.ptr(dims_a, C.c_int32),
                     family=abi.ptr(fam_a, C.c_int32), t_eval=abi.ptr(te), n_eval=m, rtol_vec=abi.ptr(rtv),
                     atol_vec=abi.ptr(atv))
    bo = abi.BatchOut(y_final=abi.ptr(out["y_final"]), t_final=abi.ptr(out["t_final"]), dense=abi.ptr(out["dense"]),
                      accepted=abi.ptr(out["accepted"], C.c_int64), rejected=abi.ptr(out["rejected"], C.c_int64),
                      fevals=abi.ptr(out["fevals"], C.c_int64), status=abi.ptr(out["status"], C.c_int32))
    rc = lib.degpu_solve_ensemble_host(C.byref(prob), C.byref(method.cfg), C.byref(bi), C.byref(bo))
    if rc != abi.OK:
        raise DegpuError(rc, "degpu_solve_ensemble_host")
    return EnsembleResult(**out)


@dataclass
class Solution:
    """Result of one solve: the crate's Solution fields (src/solution.rs:30-52) that the GPU
    produces — the requested output points (or the final point), counters and status."""
    t: list
    y: list
    status: str
    accepted: int
    rejected: int
    fevals: int

    def to_csv(self, filename: str) -> None:
        """The crate's Solution::to_csv (src/solution.rs:190-226): header t,y0,..,yN-1, one row per
        point, numbers in Rust's Debug format."""
        write_csv(filename, self.t, self.y)


def rust_debug_f64(x: float) -> str:
    """`format!("{:?}", x)` for an f64: the shortest digits that round-trip, in decimal notation
    for 1e-4 <= |x| < 1e16 (always with a fractional part) and in exponential notation otherwise
    ("1e-5", "1.5e16"); "NaN", "inf", "-inf"."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    r = repr(x)  # Python switches to exponential form at the same thresholds
    if "e" in r:
        mant, exp = r.split("e")
        return f"{mant}e{int(exp)}"
    return r


def write_csv(filename: str, t, y) -> None:
    """Write points (t[k], y[k]) in the crate's CSV format (src/solution.rs:190-226); the parent
    directory is created when missing."""
    import os

    parent = os.path.dirname(filename)
    if parent and not os.path.exists(parent):
        os.makedirs(parent)
    ys = [np.asarray(v, dtype=np.float64).reshape(-1) for v in y]
    n = len(ys[0]) if ys else 0
    with open(filename, "w") as f:
        f.write("t" + "".join(f",y{i}" for i in range(n)) + "\n")
        for tk, yk in zip(t, ys):
            f.write(rust_debug_f64(tk) + "".join("," + rust_debug_f64(v) for v in yk) + "\n")


class IVP:
    """Single-instance builder with the crate's shape (src/ivp.rs:279, 632, 656, 781-791)."""

    def __init__(self, system: System, t0: float, tf: float, y0):
        self.system, self.t0, self.tf, self.y0 = system, t0, tf, np.asarray(y0, dtype=np.float64).reshape(-1)
        self._method: Optional[ExplicitRungeKutta] = None
        self._t_eval = None
        self._crossing = None
        self._event = None

    @classmethod
    def ode(cls, system: System, t0, tf, y0):
        return cls(system, t0, tf, y0)

    def method(self, m: ExplicitRungeKutta):
        self._method = m
        return self

    def t_eval(self, pts):
        self._t_eval = list(pts)
        self._crossing = None
        return self

    def crossing(self, component: int, threshold: float, direction: int = abi.CROSS_BOTH, max_points: int = 1024):
        """The crate's IVP::crossing (src/ivp.rs:682-693): the solution holds the points where
        y[component] crosses `threshold` in `direction` (replaces t_eval)."""
        self._crossing = ("component", (component, threshold), direction, max_points)
        self._t_eval = None
        return self

    def hyperplane_crossing(self, point, normal, components, direction: int = abi.CROSS_BOTH,
                            max_points: int = 1024):
        """The crate's IVP::hyperplane_crossing (src/ivp.rs:695-706): the solution holds the
        points where pos = y[components] crosses the plane through `point` with `normal` in
        `direction` (replaces t_eval).  The crate's extractor function is given here as the list
        of state components it picks."""
        self._crossing = ("plane", (list(components), list(point), list(normal)), direction, max_points)
        self._t_eval = None
        return self

    def event(self, ev: "abi.Event"):
        """The crate's IVP::event (src/ivp.rs:661-679): wraps the current output (t_eval, or the
        final point) with event detection (abi.make_event).  The solution holds the output points
        and the recorded events in time order; a terminal event ends it with status
        "Interrupted"."""
        self._event = ev
        self._crossing = None
        return self

    def solve(self) -> Solution:
        m = self._method or ExplicitRungeKutta.dopri5()
        d = len(self.y0)
        if self._event is not None:
            r, (ct, cy, cc) = solve_ensemble_event(
                self.system.rhs_id, d, [self.t0], [self.tf], self.y0.reshape(d, 1),
                np.asarray(self.system.params, dtype=np.float64).reshape(-1, 1), [m._rtol], [m._atol], m,
                self._event, t_eval=self._t_eval)
            st = STATUS_NAMES.get(int(r.status[0]), str(int(r.status[0])))
            k = min(int(cc[0]), self._event.max_points)
            pts = [(float(ct[j, 0]), cy[j, :, 0].copy()) for j in range(k)]
            if self._t_eval is not None:
                pts += [(float(self._t_eval[i]), r.dense[i, :, 0].copy()) for i in range(len(self._t_eval))
                        if not np.isnan(r.dense[i, 0, 0])]
            else:
                pts.append((float(r.t_final[0]), r.y_final[:, 0].copy()))
            pts.sort(key=lambda p: p[0], reverse=self.tf < self.t0)
            return Solution([p[0] for p in pts], [p[1] for p in pts], st, int(r.accepted[0]), int(r.rejected[0]),
                            int(r.fevals[0]))
        if self._crossing is not None:
            kind, spec, direction, cap = self._crossing
            args = (self.system.rhs_id, d, [self.t0], [self.tf], self.y0.reshape(d, 1),
                    np.asarray(self.system.params, dtype=np.float64).reshape(-1, 1), [m._rtol], [m._atol], m)
            if kind == "plane":
                r, (ct, cy, cc) = solve_ensemble_hyperplane(*args, *spec, direction, cap)
            else:
                r, (ct, cy, cc) = solve_ensemble_crossing(*args, *spec, direction, cap)
            k = min(int(cc[0]), cap)
            st = STATUS_NAMES.get(int(r.status[0]), str(int(r.status[0])))
            return Solution([float(v) for v in ct[:k, 0]], [cy[j, :, 0].copy() for j in range(k)], st,
                            int(r.accepted[0]), int(r.rejected[0]), int(r.fevals[0]))
        r = solve_ensemble(self.system.rhs_id, d, [self.t0], [self.tf], self.y0.reshape(d, 1),
                           np.asarray(self.system.params, dtype=np.float64).reshape(-1, 1), [m._rtol], [m._atol], m,
                           t_eval=self._t_eval, dims=[d] if self.system.rhs_id == abi.RHS["FPU_BETA"] else None)
        st = STATUS_NAMES.get(int(r.status[0]), str(int(r.status[0])))
        if self._t_eval is not None:
            order = sorted(range(len(self._t_eval)), key=lambda i: self._t_eval[i],
                           reverse=self.tf < self.t0)
            ts = [self._t_eval[i] for i in order if not np.isnan(r.dense[i, 0, 0])]
            ys = [r.dense[i, :, 0].copy() for i in order if not np.isnan(r.dense[i, 0, 0])]
        else:
            ts, ys = [float(r.t_final[0])], [r.y_final[:, 0].copy()]
        return Solution(ts, ys, st, int(r.accepted[0]), int(r.rejected[0]), int(r.fevals[0]))
