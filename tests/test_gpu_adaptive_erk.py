"""The crate's Adaptive ERK family (RKF45, Cash-Karp: src/methods/erk/adaptive/ordinary.rs) on the
device against the oracle: FP64 parity reproduces status, step counts, function evaluations, final
states and cubic-Hermite dense output bit for bit; the fast and mixed forms agree within their
accuracy."""
import numpy as np
import pytest

from degpu import abi, workloads as W
from test_gpu_parity import assert_parity, cfg_for, gpu_solve, oracle_solve

pytestmark = pytest.mark.gpu

METHODS = [abi.RKF45, abi.CASH_KARP]

SYSTEMS = [  # (name, rhs, params, y0, t0, tf): the crate's accuracy-test systems
    ("exp+", "EXP_GROWTH", [1.0], [1.0], 0.0, 10.0),
    ("exp-", "EXP_GROWTH", [1.0], [22026.46579479], 0.0, -10.0),
    ("linear", "LINEAR", [1.0, 1.0], [1.0], 0.0, 10.0),
    ("harmonic", "HARMONIC", [1.0], [1.0, 0.0], 0.0, 10.0),
    ("logistic", "LOGISTIC", [1.0, 10.0], [0.1], 0.0, 10.0),
]


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("sysdef", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_adaptive_erk_test_systems_parity(sysdef, method):
    name, rhs, p, y0, t0, tf = sysdef
    d, n = len(y0), 64
    rng = np.random.default_rng(17)
    y0s = np.array(y0, dtype=float)[:, None] * (1.0 + 1e-3 * rng.standard_normal((d, n)))
    rtol = np.exp(rng.uniform(np.log(1e-10), np.log(1e-5), n))
    params = np.array(p, dtype=float).reshape(-1, 1).repeat(n, axis=1)
    e = W.Ensemble(name, method, n, d, len(p), np.full(n, t0), np.full(n, tf), y0s, params, rtol, 1e-2 * rtol,
                   rhs_id=abi.RHS[rhs])
    cfg = cfg_for(method, max_steps=200_000)
    te = np.linspace(t0, tf, 5)
    assert_parity(gpu_solve(e, cfg, t_eval=te), oracle_solve(e, cfg, t_eval=te), dense=True)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("kernel", [abi.KERNEL_THREAD, abi.KERNEL_PERSISTENT])
def test_adaptive_erk_uneven_ensemble_parity(method, kernel):
    e = W.config1(n=3 * 1500, first=40_000)
    e.tf = np.minimum(e.tf, 10.0)
    cfg = cfg_for(method, kernel=kernel)
    assert_parity(gpu_solve(e, cfg), oracle_solve(e, cfg))


def test_adaptive_erk_stiff_van_der_pol_parity():
    """Stiff Van der Pol (mu up to 1e3) under a step cap: whatever ends each solve (completion,
    MaxSteps, or Stiffness after 100 consecutive rejections) ends it alike on both sides."""
    n = 32
    mu = np.geomspace(10.0, 1e3, n)
    e = W.Ensemble("stiff", abi.RKF45, n, 2, 1, np.zeros(n), np.full(n, 50.0),
                   np.array([np.full(n, 2.0), np.zeros(n)]), mu[None, :], np.full(n, 1e-4), np.full(n, 1e-6),
                   rhs_id=abi.RHS["VAN_DER_POL"])
    for method in METHODS:
        cfg = cfg_for(method, max_steps=20_000)
        o = oracle_solve(e, cfg)
        assert_parity(gpu_solve(e, cfg), o)
        assert np.any(o["status"] != abi.COMPLETE)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("precision,tol", [(abi.FP64_FAST, 1e-9), (abi.MIXED, 1e-4)])
def test_adaptive_erk_fast_and_mixed_accuracy(method, precision, tol):
    e = W.config1(n=3 * 500, first=60_000)
    e = e.subset(np.nonzero(e.family == abi.RHS["VAN_DER_POL"])[0])
    e.rhs_id, e.family, e.dim, e.n_params = abi.RHS["VAN_DER_POL"], None, 2, 1
    e.y0 = np.ascontiguousarray(e.y0[:2])
    e.params = np.ascontiguousarray(e.params[:1])
    e.tf = np.minimum(e.tf, 10.0)
    e.rtol[:] = 1e-7
    e.atol[:] = 1e-9
    g = gpu_solve(e, cfg_for(method, precision))
    o = oracle_solve(e, cfg_for(method))
    assert np.all(g.status == abi.COMPLETE)
    rel = np.max(np.abs(g.y_final - o["y_final"]), axis=0) / np.maximum(np.max(np.abs(o["y_final"]), axis=0), 1e-300)
    assert np.median(rel) < tol


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("precision", [abi.FP64_FAST, abi.MIXED])
def test_adaptive_erk_persistent_equals_thread(method, precision):
    """The multi-family persistent kernel runs the same per-instance arithmetic as the
    one-system-per-thread launches: identical results, bit for bit, in both forms (the mixed one
    with its FP64 class below the bound)."""
    e = W.config1(n=3 * 3000, first=70_000)
    e.tf = np.minimum(e.tf, 10.0)
    g_p = gpu_solve(e, cfg_for(method, precision, kernel=abi.KERNEL_PERSISTENT))
    g_t = gpu_solve(e, cfg_for(method, precision, kernel=abi.KERNEL_THREAD))
    assert np.array_equal(g_p.status, g_t.status)
    assert np.array_equal(g_p.accepted, g_t.accepted) and np.array_equal(g_p.fevals, g_t.fevals)
    assert np.array_equal(g_p.y_final, g_t.y_final)
