"""Verner's pairs of the crate's Adaptive family (RKV655e ... RKV989e: src/tableau/verner.rs,
src/methods/erk/adaptive/ordinary.rs) on the device against the oracle: FP64 parity reproduces
status, step counts, function evaluations (the dense-output stages included), final states and
the high-order dense output bit for bit; the fast form agrees within its accuracy, and a mixed
solve runs these pairs in FP64."""
import math

import numpy as np
import pytest

from degpu import abi, workloads as W
from test_gpu_parity import assert_parity, cfg_for, gpu_solve, oracle_solve

pytestmark = pytest.mark.gpu

METHODS = [abi.RKV655E, abi.RKV656E, abi.RKV766E, abi.RKV767E, abi.RKV877E, abi.RKV878E, abi.RKV988E,
           abi.RKV989E]

SYSTEMS = [  # (name, rhs, params, y0, t0, tf): systems of the crate's accuracy tests
    ("exp+", "EXP_GROWTH", [1.0], [1.0], 0.0, 10.0),
    ("exp-", "EXP_GROWTH", [1.0], [22026.46579479], 0.0, -10.0),
    ("harmonic", "HARMONIC", [1.0], [1.0, 0.0], 0.0, 10.0),
]


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("sysdef", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_verner_test_systems_parity(sysdef, method):
    name, rhs, p, y0, t0, tf = sysdef
    d, n = len(y0), 64
    rng = np.random.default_rng(23)
    y0s = np.array(y0, dtype=float)[:, None] * (1.0 + 1e-3 * rng.standard_normal((d, n)))
    rtol = np.exp(rng.uniform(np.log(1e-12), np.log(1e-5), n))
    params = np.array(p, dtype=float).reshape(-1, 1).repeat(n, axis=1)
    e = W.Ensemble(name, method, n, d, len(p), np.full(n, t0), np.full(n, tf), y0s, params, rtol, 1e-2 * rtol,
                   rhs_id=abi.RHS[rhs])
    cfg = cfg_for(method, max_steps=200_000)
    te = np.linspace(t0, tf, 7)
    g = gpu_solve(e, cfg, t_eval=te)
    o = oracle_solve(e, cfg, t_eval=te)
    assert_parity(g, o, dense=True)
    if name == "harmonic":  # the interpolant is of high order: cos at the output times
        assert np.max(np.abs(o["dense"][:, 0, :] - np.cos(te)[:, None] * y0s[0][None, :])) < 1e-3


@pytest.mark.parametrize("method", METHODS)
def test_verner_uneven_ensemble_parity(method):
    e = W.config1(n=3 * 800, first=50_000)
    e.tf = np.minimum(e.tf, 10.0)
    cfg = cfg_for(method)
    assert_parity(gpu_solve(e, cfg), oracle_solve(e, cfg))
    te = np.array([0.0, 1.5, 4.0, 9.9])
    assert_parity(gpu_solve(e, cfg, t_eval=te), oracle_solve(e, cfg, t_eval=te), dense=True)


# At rtol 1e-6 a contracted multiply-add can flip one accept/reject decision of these high-order
# pairs, after which the two solutions differ at the tolerance level: the fast form is held to
# 10 rtol in the median.
@pytest.mark.parametrize("method", [abi.RKV656E, abi.RKV877E, abi.RKV989E])
def test_verner_fast_accuracy_and_mixed_runs_fp64(method):
    e = W.config1(n=3 * 400, first=61_000)
    e = e.subset(np.nonzero(e.family == abi.RHS["VAN_DER_POL"])[0])
    e.rhs_id, e.family, e.dim, e.n_params = abi.RHS["VAN_DER_POL"], None, 2, 1
    e.y0 = np.ascontiguousarray(e.y0[:2])
    e.params = np.ascontiguousarray(e.params[:1])
    e.tf = np.minimum(e.tf, 10.0)
    e.rtol[:] = 1e-6
    e.atol[:] = 1e-8
    te = np.array([1.0, 5.0])
    g = gpu_solve(e, cfg_for(method, abi.FP64_FAST), t_eval=te)
    o = oracle_solve(e, cfg_for(method), t_eval=te)
    assert np.all(g.status == abi.COMPLETE)
    rel = np.max(np.abs(g.y_final - o["y_final"]), axis=0) / np.maximum(np.max(np.abs(o["y_final"]), axis=0), 1e-300)
    assert np.median(rel) < 1e-5
    reld = np.max(np.abs(g.dense - o["dense"]), axis=(0, 1)) / np.max(np.abs(o["dense"]), axis=(0, 1))
    assert np.median(reld) < 1e-5
    # a mixed solve of a Verner pair runs every instance in FP64 (the bound is +infinity)
    assert abi.load().degpu_mixed_min_rtol(method) == float("inf")
    m = gpu_solve(e, cfg_for(method, abi.MIXED), t_eval=te)
    assert np.array_equal(m.y_final, g.y_final) and np.array_equal(m.dense, g.dense)
    assert np.array_equal(m.accepted, g.accepted)


def test_verner_ivp_builder():
    """IVP::ode(..).method(ExplicitRungeKutta::rkv989e()).solve(): tests/ode/accuracy.rs:395-422."""
    import degpu

    for ctor in (degpu.ExplicitRungeKutta.rkv655e, degpu.ExplicitRungeKutta.rkv989e):
        sol = degpu.IVP.ode(degpu.System.harmonic(1.0), 0.0, 10.0, [1.0, 0.0]).method(ctor()).solve()
        assert sol.status == "Complete"
        assert abs(sol.y[-1][0] - math.cos(10.0)) < 1e-3 and abs(sol.y[-1][1] + math.sin(10.0)) < 1e-3
