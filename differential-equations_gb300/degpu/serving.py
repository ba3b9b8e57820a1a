"""Python handle on the continuous-batching server (degpu_server_* in include/degpu.h).

    srv = Server(memory_budget_gb=150)
    rid = srv.submit(rhs_id, dim, t0, tf, y0, params, rtol, atol, method)   # returns at once
    res, latency_ms = srv.wait(rid)
    srv.close()

Host arrays of a request are kept alive by the handle until the request is done.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict

import numpy as np

from . import abi
from . import EnsembleResult, DegpuError, ExplicitRungeKutta


class Server:
    def __init__(self, memory_budget_gb: float = 150.0, max_active: int = 64, round_budget: int = 512):
        self.lib = abi.load()
        cfg = abi.ServerCfg(memory_budget_bytes=int(memory_budget_gb * (1 << 30)), max_active=max_active,
                            round_budget=round_budget)
        self.h = C.c_void_p()
        rc = self.lib.degpu_server_create(C.byref(cfg), C.byref(self.h))
        if rc != abi.OK:
            raise DegpuError(rc, "degpu_server_create")
        self.live: Dict[int, tuple] = {}

    def submit(self, rhs_id, dim, t0, tf, y0, params, rtol, atol, method: ExplicitRungeKutta, t_eval=None,
               dims=None, n_params=None) -> int:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        n = y0.shape[1]
        bc = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)))
        t0, tf, rtol, atol = bc(t0), bc(tf), bc(rtol), bc(atol)
        params = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, n))
        te = None if t_eval is None else np.ascontiguousarray(t_eval, dtype=np.float64)
        m = 0 if te is None else len(te)
        dims_a = None if dims is None else np.ascontiguousarray(dims, dtype=np.int32)
        out = dict(y_final=np.empty((dim, n)), t_final=np.empty(n), dense=np.empty((m, dim, n)) if m else None,
                   accepted=np.empty(n, np.int64), rejected=np.empty(n, np.int64), fevals=np.empty(n, np.int64),
                   status=np.empty(n, np.int32))
        prob = abi.Problem(rhs_id=rhs_id, dim=dim, n_params=params.shape[0] if n_params is None else n_params)
        bi = abi.BatchIn(n=n, t0=abi.ptr(t0), tf=abi.ptr(tf), y0=abi.ptr(y0), params=abi.ptr(params),
                         rtol=abi.ptr(rtol), atol=abi.ptr(atol), dims=abi.ptr(dims_a, C.c_int32), t_eval=abi.ptr(te),
                         n_eval=m)
        bo = abi.BatchOut(y_final=abi.ptr(out["y_final"]), t_final=abi.ptr(out["t_final"]),
                          dense=abi.ptr(out["dense"]), accepted=abi.ptr(out["accepted"], C.c_int64),
                          rejected=abi.ptr(out["rejected"], C.c_int64), fevals=abi.ptr(out["fevals"], C.c_int64),
                          status=abi.ptr(out["status"], C.c_int32))
        cfg = abi.MethodCfg()
        C.pointer(cfg)[0] = method.cfg
        rid = C.c_uint64(0)
        rc = self.lib.degpu_server_submit(self.h, C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo),
                                          C.byref(rid))
        if rc != abi.OK:
            raise DegpuError(rc, "degpu_server_submit")
        self.live[rid.value] = (t0, tf, y0, params, rtol, atol, te, dims_a, out, prob, cfg, bi, bo)
        return rid.value

    def poll(self, rid: int):
        done = C.c_int32(0)
        lat = C.c_double(0.0)
        rc = self.lib.degpu_server_poll(self.h, rid, C.byref(done), C.byref(lat))
        return bool(done.value), rc, lat.value

    def wait(self, rid: int):
        lat = C.c_double(0.0)
        rc = self.lib.degpu_server_wait(self.h, rid, C.byref(lat))
        if rc != abi.OK:
            raise DegpuError(rc, "request failed")
        out = self.live.pop(rid)[8]
        return EnsembleResult(**out), lat.value

    def close(self):
        if self.h:
            self.lib.degpu_server_destroy(self.h)
            self.h = C.c_void_p()
