"""GPU ensemble solves against the CPU oracle, through the C ABI.

Bar (FP64 parity path): every instance's accepted and rejected step counts, function
evaluations and status equal the oracle's, and the final state agrees within 1e-12 relative
(in practice bit for bit: both follow the crate's operation order without FMA contraction and
round pow/sin/cos correctly).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W
import degpu

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # parity tolerance on final states and dense outputs (FP64 parity path)


def oracle_solve(e: W.Ensemble, cfg, t_eval=None):
    b = O.Batch(e.rhs_id, e.dim, e.n_params, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol,
                t_eval=t_eval if t_eval is not None else e.t_eval, dims=e.dims, family=e.family)
    return O.solve(b, cfg, math_mode=1)


def gpu_solve(e: W.Ensemble, cfg, t_eval=None):
    m = degpu.ExplicitRungeKutta(cfg.method)
    m.cfg = cfg
    te = t_eval if t_eval is not None else e.t_eval
    return degpu.solve_ensemble(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m, t_eval=te,
                                dims=e.dims, family=e.family, n_params=e.n_params)


def rel_err(a, b):
    scale = np.maximum(np.abs(b), 1e-300)
    with np.errstate(invalid="ignore"):
        d = np.abs(a - b)
    d[(np.isnan(a) & np.isnan(b)) | (a == b)] = 0.0  # identical values, infinities included
    return d / scale


def assert_parity(g, o, dense=False, tol=REL_TOL):
    np.testing.assert_array_equal(g.status, o["status"])
    ok = o["status"] == abi.COMPLETE
    np.testing.assert_array_equal(g.accepted[ok], o["accepted"][ok])
    np.testing.assert_array_equal(g.rejected[ok], o["rejected"][ok])
    np.testing.assert_array_equal(g.fevals[ok], o["fevals"][ok])
    # A solution that overflowed (an unstable fixed step, say) is non-finite on both sides, but
    # its Inf/NaN pattern is not compared: the crate's 0*inf = NaN terms are skipped on the GPU.
    fin = np.isfinite(o["y_final"])
    assert np.all(~np.isfinite(g.y_final[~fin]))
    r = rel_err(g.y_final[fin], o["y_final"][fin])
    assert r.size == 0 or np.max(np.where(np.abs(o["y_final"][fin]) < 1e-300, 0, r)) <= tol, np.max(r)
    if dense:
        ofin = np.isfinite(o["dense"])
        assert np.all(np.isnan(g.dense[np.isnan(o["dense"]) & ~np.isinf(o["dense"])]) |
                      ~np.isfinite(g.dense[np.isnan(o["dense"]) & ~np.isinf(o["dense"])]))
        r = rel_err(g.dense[ofin], o["dense"][ofin])
        assert r.size == 0 or np.max(np.where(np.abs(o["dense"][ofin]) < 1e-300, 0, r)) <= tol


def cfg_for(method, precision=abi.FP64_PARITY, kernel=abi.KERNEL_THREAD, max_steps=10_000_000, h0=0.0):
    c = abi.default_cfg(method)
    c.precision, c.kernel, c.max_steps, c.h0 = precision, kernel, max_steps, h0
    return c


def test_lorenz_dopri5_4096_parity():
    """4096 Lorenz IVPs, DOPRI5 rtol=1e-8 atol=1e-10 on [0, 20] (the plain small configuration)."""
    e = W.config0()
    cfg = cfg_for(abi.DOPRI5)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o)
    # bit-for-bit in practice
    assert np.array_equal(g.y_final, o["y_final"])


@pytest.mark.parametrize("kernel", [abi.KERNEL_THREAD, abi.KERNEL_PERSISTENT])
def test_uneven_ensemble_parity(kernel):
    """A slice of the uneven ensemble (Van der Pol / pendulum / Lorenz, mixed horizons and
    tolerances) in one call, per-family work lists, thread and persistent kernels."""
    e = W.config1(n=3 * 700)
    e.tf = np.minimum(e.tf, 12.0)  # bounded oracle time
    cfg = cfg_for(abi.DOPRI5, kernel=kernel)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o)


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
def test_dense_output_parity(method):
    e = W.config1(n=3 * 200)
    e.tf = np.minimum(e.tf, 8.0)
    te = np.array([0.0, 0.37, 1.0, 2.5, 2.5, 5.0, 7.9, 8.0, 11.0])  # unsorted duplicates, beyond tf
    te = te[[3, 0, 5, 1, 2, 4, 8, 6, 7]]
    cfg = cfg_for(method)
    o = oracle_solve(e, cfg, t_eval=te)
    g = gpu_solve(e, cfg, t_eval=te)
    assert_parity(g, o, dense=True)


def test_dop853_hairer_dense_mode_parity():
    e = W.config0(n=256)
    e.tf[:] = 3.0
    te = np.linspace(0.0, 3.0, 17)
    cfg = cfg_for(abi.DOP853)
    cfg.dense_mode = abi.DENSE_HAIRER
    o = oracle_solve(e, cfg, t_eval=te)
    g = gpu_solve(e, cfg, t_eval=te)
    assert_parity(g, o, dense=True)


def test_rk4_parity_with_dense():
    e = W.config1(n=3 * 100)
    e.tf = np.minimum(e.tf, 5.0)
    te = np.linspace(0.0, 5.0, 11)
    cfg = cfg_for(abi.RK4, h0=1e-3)
    o = oracle_solve(e, cfg, t_eval=te)
    g = gpu_solve(e, cfg, t_eval=te)
    assert_parity(g, o, dense=True)


SYSTEMS = [
    # (name, rhs, params, y0, t0, tf)  tests/ode/systems.rs + accuracy.rs setups
    ("exp+", "EXP_GROWTH", [1.0], [1.0], 0.0, 10.0),
    ("exp-", "EXP_GROWTH", [1.0], [22026.46579479], 0.0, -10.0),
    ("linear", "LINEAR", [1.0, 1.0], [1.0], 0.0, 10.0),
    ("harmonic", "HARMONIC", [1.0], [1.0, 0.0], 0.0, 10.0),
    ("logistic", "LOGISTIC", [1.0, 10.0], [0.1], 0.0, 10.0),
    ("robertson", "ROBERTSON", [], [1.0, 0.0, 0.0], 0.0, 0.4),
    ("hires", "HIRES", [], [1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0057], 0.0, 5.0),
    ("brusselator", "BRUSSELATOR", [1.0, 3.0], [1.5, 3.0], 0.0, 10.0),
    ("cr3bp", "CR3BP", [0.012277471], [0.994, 0.0, 0.0, 0.0, -2.00158510637908, 0.0], 0.0, 5.0),
]


@pytest.mark.parametrize("method,h0", [(abi.DOPRI5, 0.0), (abi.DOP853, 0.0), (abi.RK4, 0.01)])
@pytest.mark.parametrize("sysdef", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_crate_test_systems_parity(sysdef, method, h0):
    name, rhs, p, y0, t0, tf = sysdef
    d = len(y0)
    n = 64
    rng = np.random.default_rng(7)
    y0s = np.array(y0, dtype=float)[:, None] * (1.0 + 1e-3 * rng.standard_normal((d, n)))
    rtol = np.exp(rng.uniform(np.log(1e-10), np.log(1e-5), n))
    params = np.array(p, dtype=float).reshape(-1, 1).repeat(n, axis=1) if p else np.zeros((0, n))
    e = W.Ensemble(name, method, n, d, len(p), np.full(n, t0), np.full(n, tf), y0s, params if p else np.zeros((1, n)),
                   rtol, 1e-2 * rtol, rhs_id=abi.RHS[rhs])
    cfg = cfg_for(method, h0=h0 if tf > t0 else -h0, max_steps=200_000)
    o = oracle_solve(e, cfg, t_eval=np.linspace(t0, tf, 5))
    g = gpu_solve(e, cfg, t_eval=np.linspace(t0, tf, 5))
    assert_parity(g, o, dense=True)


def test_error_statuses_parity():
    """MaxSteps, BadInput (h0 beyond the interval, tf == t0) per instance, batch not aborted."""
    e = W.config0(n=8)
    e.tf[2] = e.t0[2]              # tf == t0 -> BadInput
    cfg = cfg_for(abi.DOPRI5, max_steps=300)  # most instances hit MaxSteps
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o)
    assert g.status[2] == abi.ERR_BAD_INPUT
    assert (g.status == abi.ERR_MAX_STEPS).sum() >= 5
    cfg = cfg_for(abi.DOPRI5, h0=100.0)  # h0 > |tf - t0| -> BadInput everywhere
    g = gpu_solve(e, cfg)
    assert np.all(g.status == abi.ERR_BAD_INPUT)


def test_device_pointer_entry_point():
    """degpu_solve_ensemble with device pointers (torch CUDA tensors) on a stream equals the
    host entry point."""
    torch = pytest.importorskip("torch")
    e = W.config0(n=512)
    cfg = cfg_for(abi.DOPRI5, kernel=abi.KERNEL_PERSISTENT)
    g = gpu_solve(e, cfg)
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    t0, tf, y0, p, rt, at = T(e.t0), T(e.tf), T(e.y0), T(e.params), T(e.rtol), T(e.atol)
    yf = torch.empty((3, e.n), dtype=torch.float64, device=dev)
    acc = torch.empty(e.n, dtype=torch.int64, device=dev)
    rej = torch.empty_like(acc)
    fe = torch.empty_like(acc)
    st = torch.empty(e.n, dtype=torch.int32, device=dev)
    lib = abi.load()
    prob = abi.Problem(rhs_id=e.rhs_id, dim=3, n_params=3)
    bi = abi.BatchIn(n=e.n, t0=abi.ptr(t0), tf=abi.ptr(tf), y0=abi.ptr(y0), params=abi.ptr(p), rtol=abi.ptr(rt),
                     atol=abi.ptr(at), n_eval=0)
    bo = abi.BatchOut(y_final=abi.ptr(yf), accepted=abi.ptr(acc, C.c_int64), rejected=abi.ptr(rej, C.c_int64),
                      fevals=abi.ptr(fe, C.c_int64), status=abi.ptr(st, C.c_int32))
    s = torch.cuda.Stream()
    rc = lib.degpu_solve_ensemble(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), C.c_void_p(s.cuda_stream))
    assert rc == abi.OK
    s.synchronize()
    assert np.array_equal(yf.cpu().numpy(), g.y_final)
    assert np.array_equal(acc.cpu().numpy(), g.accepted)


def test_fast_fp64_accuracy():
    """FMA-contracted FP64 with the CUDA math library: same method, results differ only by
    rounding; compared on non-chaotic instances (Van der Pol / pendulum slice) at final time."""
    e = W.config1(n=3 * 300)
    keep = e.family != abi.RHS["LORENZ"]
    e = e.subset(np.nonzero(keep)[0])
    e.tf = np.minimum(e.tf, 10.0)
    o = oracle_solve(e, cfg_for(abi.DOPRI5))
    g = gpu_solve(e, cfg_for(abi.DOPRI5, precision=abi.FP64_FAST))
    assert np.all(g.status == abi.COMPLETE)
    err = np.max(np.abs(g.y_final - o["y_final"]), axis=0) / np.maximum(1.0, np.max(np.abs(o["y_final"]), axis=0))
    assert np.median(err) < 1e-9


def test_mixed_precision_error_vs_oracle():
    """The default mixed form (FP32 stages with Kahan-compensated y above the DOPRI5 bound,
    FP32-pair stages below it; the error norm, controller and accept decision in FP32, t as an
    FP32 pair) against a tight FP64 oracle (DOP853, rtol = atol = 1e-13), per rtol decade of the
    uneven ensemble's Van der Pol and pendulum instances.  In every decade where FP64 at the same
    tolerances reaches a median error of 1e-6, the mixed median may be at most 1.25 x FP64's and its
    share of instances within 1e-6 at most 3 points below FP64's (the accuracy rule of the
    benchmark's headline)."""
    e = W.config1(n=3 * 1600)
    e = e.subset(np.nonzero(e.family != abi.RHS["LORENZ"])[0])
    e.tf = np.minimum(e.tf, 10.0)
    tight = O.Batch(0, e.dim, e.n_params, e.t0, e.tf, e.y0, e.params, np.full(e.n, 1e-13), np.full(e.n, 1e-13),
                    family=e.family)
    c8 = cfg_for(abi.DOP853, max_steps=50_000_000)
    y_tight = O.solve(tight, c8, math_mode=1)["y_final"]
    g64 = gpu_solve(e, cfg_for(abi.DOPRI5, precision=abi.FP64_FAST, kernel=abi.KERNEL_PERSISTENT))
    gm = gpu_solve(e, cfg_for(abi.DOPRI5, precision=abi.MIXED, kernel=abi.KERNEL_PERSISTENT))
    assert np.all(g64.status == abi.COMPLETE) and np.all(gm.status == abi.COMPLETE)

    def rel(y):
        return np.max(np.abs(y - y_tight), axis=0) / np.maximum(np.max(np.abs(y_tight), axis=0), 1e-300)

    r64, rm = rel(g64.y_final), rel(gm.y_final)
    checked = 0
    for fam in (abi.RHS["VAN_DER_POL"], abi.RHS["PENDULUM"]):
        for lo, hi in ((1e-9, 1e-8), (1e-8, 1e-7), (1e-7, 1e-6), (1e-6, 1e-5)):
            m = (e.family == fam) & (e.rtol >= lo) & (e.rtol < hi)
            if m.sum() < 100 or np.median(r64[m]) > 1e-6:
                continue
            checked += 1
            assert np.median(rm[m]) <= 1.25 * np.median(r64[m]), (fam, lo, np.median(rm[m]), np.median(r64[m]))
            gap = np.mean(r64[m] <= 1e-6) - np.mean(rm[m] <= 1e-6)
            assert gap <= 0.03, (fam, lo, gap)
    assert checked >= 4


@pytest.mark.parametrize("precision", [abi.FP64_PARITY])
def test_fpu_chain_group_kernel_parity(precision):
    """FPU-beta chains of ragged dimension (2..256 components), DOP853 rtol=1e-10 atol=1e-12 with
    64 dense output times, through the group-per-system kernel; every dimension bucket
    (8/16/32 lanes per system, 1..8 components per lane) is exercised."""
    e = W.config2(n=96)
    # cover each bucket explicitly: masses 2, 4, 8, 16, 30, 64, 100, 128
    masses = np.array([2, 4, 8, 16, 30, 64, 100, 128] * 12)
    e.dims = (2 * masses).astype(np.int32)
    e.dim = 256
    rng = np.random.default_rng(3)
    e.y0 = np.zeros((256, 96))
    for i, m in enumerate(masses):
        e.y0[:m, i] = 0.1 * rng.standard_normal(m)
    e.tf[:] = 10.0
    e.t_eval = 10.0 * np.arange(64) / 63.0
    cfg = cfg_for(abi.DOP853, precision=precision)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o, dense=True)


def test_fpu_chain_dopri5_parity():
    e = W.config2(n=64)
    e.tf[:] = 5.0
    cfg = cfg_for(abi.DOPRI5)
    o = oracle_solve(e, cfg, t_eval=np.linspace(0.0, 5.0, 9))
    g = gpu_solve(e, cfg, t_eval=np.linspace(0.0, 5.0, 9))
    assert_parity(g, o, dense=True)


def test_fpu_chain_fast_and_mixed_accuracy():
    e = W.config2(n=128)
    e.tf[:] = 10.0
    e.t_eval = None
    o = oracle_solve(e, cfg_for(abi.DOP853))
    for prec, tol in ((abi.FP64_FAST, 1e-8), (abi.MIXED, 1e-4)):
        g = gpu_solve(e, cfg_for(abi.DOP853, precision=prec))
        assert np.all(g.status == abi.COMPLETE)
        err = np.max(np.abs(g.y_final - o["y_final"]), axis=0) / np.max(np.abs(o["y_final"]), axis=0)
        assert np.median(err) < tol, (prec, np.median(err))


@pytest.mark.parametrize("kernel", [abi.KERNEL_THREAD, abi.KERNEL_PERSISTENT])
def test_uneven_ensemble_full_horizon_parity(kernel):
    """6,000 instances of the uneven ensemble at their drawn horizons (t_end ~ U[5, 50], nothing
    clipped) and tolerances: the long-horizon regime in which a single rounding difference would
    flip an accept decision somewhere along the solve.  Bit for bit."""
    e = W.config1(n=6000)
    assert e.tf.max() > 45.0
    cfg = cfg_for(abi.DOPRI5, kernel=kernel)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o)
    assert np.all(g.status == abi.COMPLETE)
    assert np.array_equal(g.y_final, o["y_final"])


def test_fpu_chain_full_horizon_parity():
    """64 FPU-beta chains of the uneven-dimension configuration as drawn (2..128 masses, DOP853
    rtol 1e-10 atol 1e-12 over [0, 100], 64 uniformly spaced output times)."""
    e = W.config2(n=64)
    assert np.all(e.tf == 100.0) and len(e.t_eval) == 64
    cfg = cfg_for(abi.DOP853)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    assert_parity(g, o, dense=True)
    assert np.array_equal(g.y_final, o["y_final"])


def status_case(rhs, p, y0, tf, rtol, n=4):
    d = len(y0)
    rng = np.random.default_rng(11)
    y0s = np.array(y0, dtype=float)[:, None] * (1.0 + 1e-6 * rng.standard_normal((d, n)))
    return W.Ensemble(rhs, abi.DOPRI5, n, d, len(p), np.zeros(n), np.full(n, tf), y0s,
                      np.array(p, dtype=float).reshape(-1, 1).repeat(n, axis=1), np.full(n, rtol), np.full(n, rtol),
                      rhs_id=abi.RHS[rhs])


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
@pytest.mark.parametrize("case,expect", [
    # y' = y: the stiffness quotient's denominator |f(y_new) - y_stage|^2 is rounding noise, so
    # every 100th step counts as stiff and the 15th detection aborts (ordinary.rs:165-186)
    (("EXP_GROWTH", [1.0], [1.0], 600.0, 1e-12), "STIFFNESS"),
    # y' = 1000 y overflows; the step size then shrinks by min_scale per rejection until it is
    # below 1e-14 of the last accepted one (ordinary.rs:69-80)
    (("EXP_GROWTH", [1000.0], [1.0], 10.0, 1e-6), "STEP_SIZE"),
    (("EXP_GROWTH", [1.0], [1e300], 100.0, 1e-6), "STEP_SIZE"),
], ids=["stiffness", "step_size_growth", "step_size_overflow"])
def test_stiffness_and_step_size_statuses_parity(method, case, expect):
    """The crate's Error::Stiffness and Error::StepSize end instances on the device as they end
    them in the oracle: same status, counters, time and state at the abort."""
    e = status_case(*case)
    cfg = cfg_for(method)
    o = oracle_solve(e, cfg)
    g = gpu_solve(e, cfg)
    want = {"STIFFNESS": abi.ERR_STIFFNESS, "STEP_SIZE": abi.ERR_STEP_SIZE}[expect]
    assert np.all(o["status"] == want)
    np.testing.assert_array_equal(g.status, o["status"])
    np.testing.assert_array_equal(g.accepted, o["accepted"])
    np.testing.assert_array_equal(g.rejected, o["rejected"])
    np.testing.assert_array_equal(g.fevals, o["fevals"])
    np.testing.assert_array_equal(g.t_final, o["t_final"])
    np.testing.assert_array_equal(g.y_final, o["y_final"])
