"""Continuous-batching server: every request's result is the same alone and in the mix.

Requests of different families, methods, precisions and sizes are submitted together with a
small round budget (many resume/park cycles of the resident state); each result must equal, bit
for bit, the same request solved alone through degpu_solve_ensemble_host."""
import numpy as np
import pytest

import degpu
from degpu import abi, workloads as W
from degpu.serving import Server

pytestmark = pytest.mark.gpu


def method(m, prec, h0=0.0):
    e = degpu.ExplicitRungeKutta(m)
    e.cfg.precision = prec
    e.cfg.max_steps = 10_000_000
    e.cfg.h0 = h0
    return e


def requests():
    reqs = []
    fams = [abi.RHS["LORENZ"], abi.RHS["VAN_DER_POL"], abi.RHS["PENDULUM"]]
    rng = np.random.default_rng(5)
    for k in range(12):
        fam = fams[k % 3]
        m = [abi.DOPRI5, abi.DOP853, abi.RK4][(k // 3) % 3]
        prec = [abi.FP64_PARITY, abi.MIXED, abi.FP64_FAST][k % 3]
        n = int(rng.integers(1, 3000))
        e = W.config1(n=3 * n, first=1000 * k)
        e = e.subset(np.nonzero(e.family == fam)[0])
        e.tf = np.minimum(e.tf, 6.0)
        dim = 3 if fam == abi.RHS["LORENZ"] else 2
        reqs.append(dict(rhs=fam, dim=dim, e=e, m=method(m, prec, 1e-3 if m == abi.RK4 else 0.0)))
    # a mixed request whose rtol values straddle the mixed-precision bound: its instances run in
    # two round kernels (FP32 stages above the bound, FP32-pair stages below)
    e = W.config1(n=1500, first=123_000)
    e = e.subset(np.nonzero(e.family == abi.RHS["VAN_DER_POL"])[0])
    e.tf = np.minimum(e.tf, 6.0)
    e.rtol = W.logU(9, np.arange(e.n), 1, 1e-9, 1e-5)
    e.atol = 1e-2 * e.rtol
    assert 0 < (e.rtol < degpu.mixed_min_rtol(abi.DOPRI5)).sum() < e.n
    reqs.append(dict(rhs=abi.RHS["VAN_DER_POL"], dim=2, e=e, m=method(abi.DOPRI5, abi.MIXED)))
    # a dense-output request and a ragged FPU-chain request (solved by one launch inside the server)
    e = W.config1(n=600, first=99_000)
    e = e.subset(np.nonzero(e.family == abi.RHS["LORENZ"])[0])
    e.tf[:] = 4.0
    reqs.append(dict(rhs=abi.RHS["LORENZ"], dim=3, e=e, m=method(abi.DOP853, abi.FP64_PARITY),
                     t_eval=np.linspace(0, 4, 9)))
    f = W.config2(n=40)
    f.tf[:] = 5.0
    reqs.append(dict(rhs=abi.RHS["FPU_BETA"], dim=f.dim, e=f, m=method(abi.DOP853, abi.FP64_PARITY), dims=f.dims,
                     t_eval=np.linspace(0, 5, 6)))
    # ragged FPU-chain requests on the resumable group kernels: FP64 fast with output times, and
    # mixed with rtol values straddling the bounds of DOP853 (FP32 stages / FP64 fast parts) and
    # DOPRI5, so that one request runs several round kernels (one per precision and layout)
    for k, (m, prec, te) in enumerate(((abi.DOP853, abi.FP64_FAST, np.linspace(0, 5, 6)),
                                       (abi.DOP853, abi.MIXED, None),
                                       (abi.DOPRI5, abi.MIXED, np.linspace(0, 4, 5)))):
        f = W.config2(n=48, first=500 * (k + 1))
        f.tf[:] = 4.0 + k
        if prec == abi.MIXED:
            f.rtol = W.logU(11, np.arange(f.n), 1, 1e-9, 1e-5)
            f.atol = 1e-2 * f.rtol
            assert 0 < (f.rtol < degpu.mixed_min_rtol(m)).sum() < f.n
        reqs.append(dict(rhs=abi.RHS["FPU_BETA"], dim=f.dim, e=f, m=method(m, prec), dims=f.dims, t_eval=te))
    # mixed requests with output times that straddle the DOPRI5 bound (the dense round kernels,
    # FP32 stages above the bound and FP32-pair stages below)
    for fam, dim in ((abi.RHS["PENDULUM"], 2), (abi.RHS["LORENZ"], 3)):
        e = W.config1(n=900, first=77_000)
        e = e.subset(np.nonzero(e.family == fam)[0])
        e.tf = np.minimum(e.tf, 5.0)
        e.rtol = W.logU(12, np.arange(e.n), 1, 1e-9, 1e-5)
        e.atol = 1e-2 * e.rtol
        reqs.append(dict(rhs=fam, dim=dim, e=e, m=method(abi.DOPRI5, abi.MIXED), t_eval=np.linspace(5, 0, 11)))
    return reqs


def test_results_same_alone_and_in_the_mix():
    reqs = requests()
    srv = Server(memory_budget_gb=4.0, max_active=8, round_budget=32)
    try:
        ids = [srv.submit(r["rhs"], r["dim"], r["e"].t0, r["e"].tf, r["e"].y0[:r["dim"]], r["e"].params, r["e"].rtol,
                          r["e"].atol, r["m"], t_eval=r.get("t_eval"), dims=r.get("dims")) for r in reqs]
        got = [srv.wait(i) for i in ids]
    finally:
        srv.close()
    for r, (res, lat) in zip(reqs, got):
        e = r["e"]
        alone = degpu.solve_ensemble(r["rhs"], r["dim"], e.t0, e.tf, e.y0[:r["dim"]], e.params, e.rtol, e.atol, r["m"],
                                     t_eval=r.get("t_eval"), dims=r.get("dims"), n_params=e.params.shape[0])
        assert lat > 0.0
        assert np.array_equal(res.status, alone.status)
        assert np.array_equal(res.accepted, alone.accepted) and np.array_equal(res.rejected, alone.rejected)
        assert np.array_equal(res.fevals, alone.fevals)
        assert np.array_equal(res.y_final, alone.y_final)
        if r.get("t_eval") is not None:
            assert np.array_equal(res.dense, alone.dense, equal_nan=True)


def test_budget_smaller_than_request_still_admits_alone():
    """A request larger than the memory budget runs once nothing else is resident."""
    e = W.config0(n=2000)
    e.tf[:] = 2.0
    srv = Server(memory_budget_gb=1e-4, max_active=2, round_budget=64)
    try:
        a = srv.submit(abi.RHS["LORENZ"], 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, method(abi.DOPRI5, abi.MIXED))
        b = srv.submit(abi.RHS["LORENZ"], 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, method(abi.DOPRI5, abi.MIXED))
        ra, _ = srv.wait(a)
        rb, _ = srv.wait(b)
    finally:
        srv.close()
    assert np.array_equal(ra.y_final, rb.y_final)
    assert np.all(ra.status == abi.COMPLETE)
