"""Loader for the CPU oracle (oracle/liboracle.so) used as the parity checker by the tests.

The oracle is test infrastructure: it is a C++ restatement of the crate's explicit Runge–Kutta
path and is never on the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
sys.path.insert(0, os.path.join(REPO, "differential-equations_gb300"))

from degpu import abi  # noqa: E402  (boundary structs only)

DP = C.POINTER(C.c_double)
I64P = C.POINTER(C.c_int64)

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(ORACLE_SO)
        L.oracle_solve_ensemble.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.MethodCfg),
                                            C.POINTER(abi.BatchIn), C.POINTER(abi.BatchOut), C.c_int, C.c_int]
        L.oracle_solve_ensemble.restype = C.c_int
        L.oracle_solve_ensemble_crossing.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.MethodCfg),
                                                     C.POINTER(abi.BatchIn), C.POINTER(abi.Crossing),
                                                     C.POINTER(abi.BatchOut), C.POINTER(abi.CrossingOut), C.c_int,
                                                     C.c_int]
        L.oracle_solve_ensemble_crossing.restype = C.c_int
        L.oracle_solve_ensemble_hyperplane.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.MethodCfg),
                                                       C.POINTER(abi.BatchIn), C.POINTER(abi.Hyperplane),
                                                       C.POINTER(abi.BatchOut), C.POINTER(abi.CrossingOut),
                                                       C.c_int, C.c_int]
        L.oracle_solve_ensemble_hyperplane.restype = C.c_int
        L.oracle_solve_ensemble_event.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.MethodCfg),
                                                  C.POINTER(abi.BatchIn), C.POINTER(abi.Event),
                                                  C.POINTER(abi.BatchOut), C.POINTER(abi.CrossingOut), C.c_int,
                                                  C.c_int]
        L.oracle_solve_ensemble_event.restype = C.c_int
        L.oracle_solve_bvp.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.MethodCfg), C.POINTER(abi.BatchIn),
                                       C.POINTER(abi.Bvp), C.POINTER(abi.BatchOut), C.POINTER(abi.BvpOut), C.c_int,
                                       C.c_int]
        L.oracle_solve_bvp.restype = C.c_int
        L.oracle_eval_rhs.argtypes = [C.c_int32, C.c_int64, C.c_int32, C.c_int32, DP, DP, DP, DP, C.c_int]
        for nm in ("oracle_cr_pow", "oracle_libm_pow"):
            getattr(L, nm).argtypes = [C.c_double, C.c_double]
            getattr(L, nm).restype = C.c_double
        for nm in ("oracle_cr_sin", "oracle_cr_cos", "oracle_libm_sin", "oracle_libm_cos"):
            getattr(L, nm).argtypes = [C.c_double]
            getattr(L, nm).restype = C.c_double
        for nm in ("oracle_cr_pow_batch", "oracle_libm_pow_batch"):
            getattr(L, nm).argtypes = [DP, DP, DP, C.c_int64]
        L.oracle_cr_sincos_batch.argtypes = [DP, DP, DP, C.c_int64]
        L.oracle_heat1d_diff.argtypes = [C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                         C.c_int, C.c_double, DP, DP]
        L.oracle_coupled1d_diff.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, DP, DP,
                                            DP, DP]
        L.oracle_heat1d_solve.argtypes = [C.c_double, C.c_int, C.c_double, C.c_double, C.c_double, DP, DP, I64P]
        L.oracle_gray_scott_rhs.argtypes = [C.POINTER(abi.GrayScott), DP, DP, DP, DP, C.c_int]
        L.oracle_mol_rhs.argtypes = [C.POINTER(abi.Mol), C.c_double, DP, DP, C.c_int]
        L.oracle_mol_rk4.argtypes = [C.POINTER(abi.Mol), C.c_double, C.c_double, C.c_double, DP, I64P, C.c_int]
        L.oracle_gray_scott_rk4.argtypes = [C.POINTER(abi.GrayScott), C.c_double, C.c_double, C.c_int64, DP, DP,
                                            C.c_int]
        _lib = L
    return _lib


def p(a):
    return abi.ptr(a)


class Batch:
    """Host-side batch of IVPs in the ABI's structure-of-arrays layout."""

    def __init__(self, rhs_id, dim, n_params, t0, tf, y0, params, rtol, atol, t_eval=None, dims=None,
                 family=None, rtol_vec=None, atol_vec=None):
        self.n = len(t0)
        self.problem = abi.Problem(rhs_id=rhs_id, dim=dim, n_params=n_params)
        self.t0 = np.ascontiguousarray(t0, dtype=np.float64)
        self.tf = np.ascontiguousarray(tf, dtype=np.float64)
        self.y0 = np.ascontiguousarray(y0, dtype=np.float64).reshape(dim, self.n)
        self.params = np.ascontiguousarray(params, dtype=np.float64).reshape(max(n_params, 1), self.n) \
            if n_params else np.zeros((1, self.n))
        self.rtol = np.ascontiguousarray(rtol, dtype=np.float64)
        self.atol = np.ascontiguousarray(atol, dtype=np.float64)
        self.t_eval = None if t_eval is None else np.ascontiguousarray(t_eval, dtype=np.float64)
        self.dims = None if dims is None else np.ascontiguousarray(dims, dtype=np.int32)
        self.family = None if family is None else np.ascontiguousarray(family, dtype=np.int32)
        tv = lambda v: None if v is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(v, dtype=np.float64).reshape(dim, -1), (dim, self.n)))
        self.rtol_vec, self.atol_vec = tv(rtol_vec), tv(atol_vec)
        self.dim = dim

    def batch_in(self):
        return abi.BatchIn(
            n=self.n, t0=p(self.t0), tf=p(self.tf), y0=p(self.y0), params=p(self.params), rtol=p(self.rtol),
            atol=p(self.atol), dims=abi.ptr(self.dims, C.c_int32), family=abi.ptr(self.family, C.c_int32),
            t_eval=p(self.t_eval), n_eval=0 if self.t_eval is None else len(self.t_eval),
            rtol_vec=p(self.rtol_vec), atol_vec=p(self.atol_vec))

    def new_outputs(self):
        m = 0 if self.t_eval is None else len(self.t_eval)
        return dict(
            y_final=np.full((self.dim, self.n), np.nan), t_final=np.full(self.n, np.nan),
            dense=np.full((m, self.dim, self.n), np.nan) if m else None,
            accepted=np.zeros(self.n, np.int64), rejected=np.zeros(self.n, np.int64),
            fevals=np.zeros(self.n, np.int64), status=np.full(self.n, -1, np.int32))

    @staticmethod
    def batch_out(o):
        return abi.BatchOut(
            y_final=p(o["y_final"]), t_final=p(o["t_final"]), dense=p(o["dense"]),
            accepted=abi.ptr(o["accepted"], C.c_int64), rejected=abi.ptr(o["rejected"], C.c_int64),
            fevals=abi.ptr(o["fevals"], C.c_int64), status=abi.ptr(o["status"], C.c_int32))


def solve(batch: Batch, cfg, threads=None, math_mode=1):
    """Oracle solve of every instance.  math_mode 1 = correctly rounded pow/sin/cos, 0 = host libm."""
    out = batch.new_outputs()
    bi = batch.batch_in()
    bo = Batch.batch_out(out)
    threads = threads or os.cpu_count() or 1
    rc = lib().oracle_solve_ensemble(C.byref(batch.problem), C.byref(cfg), C.byref(bi), C.byref(bo), threads,
                                     math_mode)
    assert rc == 0
    return out


def solve_crossing(batch: Batch, cfg, component, threshold, direction=0, max_points=16, threads=None, math_mode=1):
    """Oracle solve with crossing detection (CrossingSolout): returns the ordinary outputs plus
    cross_t [max_points, n], cross_y [max_points, dim, n] and cross_count [n]."""
    out = batch.new_outputs()
    n, dim = batch.n, batch.problem.dim
    ct = np.empty((max_points, n))
    cy = np.empty((max_points, dim, n))
    cc = np.empty(n, np.int32)
    cr = abi.Crossing(component=component, direction=direction, max_points=max_points, threshold=threshold)
    co = abi.CrossingOut(t=p(ct), y=p(cy), count=abi.ptr(cc, C.c_int32))
    threads = threads or os.cpu_count() or 1
    rc = lib().oracle_solve_ensemble_crossing(C.byref(batch.problem), C.byref(cfg), C.byref(batch.batch_in()),
                                              C.byref(cr), C.byref(Batch.batch_out(out)), C.byref(co), threads,
                                              math_mode)
    assert rc == 0
    out.update(cross_t=ct, cross_y=cy, cross_count=cc)
    return out


def solve_hyperplane(batch: Batch, cfg, components, point, normal, direction=0, max_points=16, threads=None,
                     math_mode=1):
    """Oracle solve with hyperplane crossing detection (HyperplaneCrossingSolout): returns the
    ordinary outputs plus cross_t, cross_y and cross_count as solve_crossing does."""
    out = batch.new_outputs()
    n, dim = batch.n, batch.problem.dim
    ct = np.empty((max_points, n))
    cy = np.empty((max_points, dim, n))
    cc = np.empty(n, np.int32)
    hp = abi.make_hyperplane(components, point, normal, direction, max_points)
    co = abi.CrossingOut(t=p(ct), y=p(cy), count=abi.ptr(cc, C.c_int32))
    threads = threads or os.cpu_count() or 1
    rc = lib().oracle_solve_ensemble_hyperplane(C.byref(batch.problem), C.byref(cfg), C.byref(batch.batch_in()),
                                                C.byref(hp), C.byref(Batch.batch_out(out)), C.byref(co), threads,
                                                math_mode)
    assert rc == 0
    out.update(cross_t=ct, cross_y=cy, cross_count=cc)
    return out


def solve_event(batch: Batch, cfg, event, threads=None, math_mode=1):
    """Oracle solve with event detection (EventWrappedSolout over the batch's output times, or
    over the default per-step output): returns the ordinary outputs (dense included when the
    batch has output times) plus cross_t, cross_y and cross_count for the recorded events."""
    out = batch.new_outputs()
    n, dim = batch.n, batch.problem.dim
    mp = event.max_points
    ct = np.empty((mp, n))
    cy = np.empty((mp, dim, n))
    cc = np.empty(n, np.int32)
    co = abi.CrossingOut(t=p(ct), y=p(cy), count=abi.ptr(cc, C.c_int32))
    threads = threads or os.cpu_count() or 1
    rc = lib().oracle_solve_ensemble_event(C.byref(batch.problem), C.byref(cfg), C.byref(batch.batch_in()),
                                           C.byref(event), C.byref(Batch.batch_out(out)), C.byref(co), threads,
                                           math_mode)
    assert rc == 0
    out.update(cross_t=ct, cross_y=cy, cross_count=cc)
    return out


def solve_bvp(batch: Batch, cfg, bvp, threads=None, math_mode=1):
    """Oracle shooting solve of every instance (the batch's y0 are the guesses): the ordinary
    outputs of the final IVP (y_final = y(tf), dense at the batch's output times), totals in
    accepted / rejected / fevals, plus y_a [dim, n], iterations [n] and jacobian [n]."""
    out = batch.new_outputs()
    n, dim = batch.n, batch.problem.dim
    ya = np.empty((dim, n))
    it = np.empty(n, np.int32)
    jac = np.empty(n, np.int64)
    bo = abi.BvpOut(y_a=p(ya), iterations=abi.ptr(it, C.c_int32), jacobian=abi.ptr(jac, C.c_int64))
    threads = threads or os.cpu_count() or 1
    rc = lib().oracle_solve_bvp(C.byref(batch.problem), C.byref(cfg), C.byref(batch.batch_in()), C.byref(bvp),
                                C.byref(Batch.batch_out(out)), C.byref(bo), threads, math_mode)
    assert rc == 0
    out.update(y_a=ya, iterations=it, jacobian=jac)
    return out
