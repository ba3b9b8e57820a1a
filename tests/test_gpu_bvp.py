"""Boundary value problems by shooting over an ensemble (degpu_solve_bvp_host) against the oracle's
restatement of the crate's SingleShooting / MultipleShooting (src/methods/bvp/shooting): with FP64
parity arithmetic every status, Newton iteration count, Jacobian count, counter total, converged
initial state, final state and output time is bit for bit the oracle's; the crate's BVP tests
(tests/bvp/shooting.rs) hold through the builder."""
import math

import numpy as np
import pytest

import oracle_lib as O
import degpu
from degpu import abi

pytestmark = pytest.mark.gpu
R = abi.RHS
HALF_PI = math.pi / 2
HARMONIC_ROWS = [(0, 0, 0.0), (1, 0, 1.0)]
PIPE_ROWS = [(0, 0, 373.15), (1, 1, 0.0)]


def cfg_for(method=abi.DOP853, precision=abi.FP64_PARITY):
    c = abi.default_cfg(method)
    c.precision, c.max_steps = precision, 10_000_000
    return c


def both(rhs, dim, params, t0, tf, guess, rtol, atol, cfg, bvp, t_eval=None):
    n = guess.shape[1]
    m = degpu.ExplicitRungeKutta(cfg.method)
    m.cfg = cfg
    g = degpu.solve_bvp(R[rhs], dim, t0, tf, guess, params, rtol, atol, m, bvp, t_eval=t_eval)
    bc = lambda v: np.broadcast_to(np.asarray(v, dtype=float), (n,)).copy()
    b = O.Batch(R[rhs], dim, params.shape[0], bc(t0), bc(tf), guess, params, bc(rtol), bc(atol), t_eval=t_eval)
    o = O.solve_bvp(b, cfg, bvp)
    return g, o


def assert_bvp_same(g, o):
    s = g.solution
    assert np.array_equal(s.status, o["status"])
    ok = o["status"] == abi.COMPLETE
    for k in ("accepted", "rejected", "fevals"):
        assert np.array_equal(getattr(s, k)[ok], o[k][ok]), k
    assert np.array_equal(g.iterations[ok], o["iterations"][ok])
    assert np.array_equal(g.jacobian[ok], o["jacobian"][ok])
    assert np.array_equal(g.y_a, o["y_a"], equal_nan=True)
    assert np.array_equal(s.y_final, o["y_final"], equal_nan=True)
    assert np.array_equal(s.t_final, o["t_final"])
    if s.dense is not None:
        assert np.array_equal(s.dense, o["dense"], equal_nan=True)


@pytest.mark.parametrize("method,segments,tol", [(abi.BVP_SINGLE, 4, 1e-6), (abi.BVP_MULTIPLE, 4, 1e-8),
                                                 (abi.BVP_MULTIPLE, 3, 1e-8)])
@pytest.mark.parametrize("erk", [abi.DOP853, abi.DOPRI5, abi.RKF45])
def test_harmonic_bvp_ensemble_parity(method, segments, tol, erk):
    n = 300
    rng = np.random.default_rng(31)
    guess = np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 2, n)])
    k = rng.uniform(0.5, 2.0, n)[None, :]
    rtol = 10.0 ** rng.uniform(-12, -7, n)
    te = np.linspace(0.0, HALF_PI, 5)
    g, o = both("HARMONIC", 2, k, 0.0, HALF_PI, guess, rtol, 1e-2 * rtol, cfg_for(erk),
                abi.make_bvp(HARMONIC_ROWS, method, segments, tolerance=tol), t_eval=te)
    assert np.mean(o["status"] == abi.COMPLETE) > 0.9
    assert_bvp_same(g, o)


@pytest.mark.parametrize("method", [abi.BVP_SINGLE, abi.BVP_MULTIPLE])
def test_pipe_heat_bvp_ensemble_parity(method):
    n = 256
    rng = np.random.default_rng(37)
    beta = rng.uniform(0.05, 0.4, n)
    amb = rng.uniform(280.0, 300.0, n)
    guess = np.stack([np.full(n, 373.15), rng.uniform(-10.0, 0.0, n)])
    g, o = both("PIPE_HEAT", 2, np.stack([beta, amb]), 0.0, 10.0, guess, 1e-10, 1e-12, cfg_for(),
                abi.make_bvp(PIPE_ROWS, method, 5, tolerance=1e-8))
    assert np.all(o["status"] == abi.COMPLETE)
    assert_bvp_same(g, o)
    # the analytical solution (tests/bvp/systems.rs:31-42)
    theta0, bl = 373.15 - amb, beta * 10.0
    assert np.max(np.abs(g.y_a[1] + beta * theta0 * np.tanh(bl))) < 1e-4
    assert np.max(np.abs(g.solution.y_final[0] - (amb + theta0 / np.cosh(bl)))) < 1e-4


def test_bvp_failure_statuses_parity():
    """Singular Jacobian (LinearAlgebra), the iteration cap (MaxSteps) and a failing inner IVP
    (its own MaxSteps), side by side in one batch of each kind."""
    n = 16
    guess = np.stack([np.linspace(-1, 1, n), np.linspace(0, 2, n)])
    k = np.ones((1, n))
    for bvp in (abi.make_bvp([(0, 0, 0.0), (0, 0, 1.0)]),
                abi.make_bvp(HARMONIC_ROWS, max_iterations=1, tolerance=1e-14),
                abi.make_bvp(HARMONIC_ROWS, abi.BVP_MULTIPLE, 4, max_iterations=1, tolerance=1e-14)):
        g, o = both("HARMONIC", 2, k, 0.0, HALF_PI, guess, 1e-10, 1e-12, cfg_for(), bvp)
        assert np.all(o["status"] != abi.COMPLETE)
        assert_bvp_same(g, o)
    cfg = cfg_for()
    cfg.max_steps = 5  # every inner IVP runs out of steps
    g, o = both("HARMONIC", 2, k, 0.0, HALF_PI, guess, 1e-10, 1e-12, cfg, abi.make_bvp(HARMONIC_ROWS))
    assert np.all(o["status"] == abi.ERR_MAX_STEPS)
    assert_bvp_same(g, o)


def test_bvp_fast_and_mixed():
    """FP64 fast shots solve the BVP; a mixed configuration runs its shots in FP64 fast (the
    Jacobian's 1.5e-8 perturbation is below FP32 resolution), so it returns the same bits."""
    n = 128
    rng = np.random.default_rng(41)
    guess = np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 2, n)])
    res = []
    for precision in (abi.FP64_FAST, abi.MIXED):
        m = degpu.ExplicitRungeKutta(abi.DOPRI5)
        m.cfg = cfg_for(abi.DOPRI5, precision)
        r = degpu.solve_bvp(R["HARMONIC"], 2, 0.0, HALF_PI, guess, np.ones((1, n)), 1e-8, 1e-10, m,
                            abi.make_bvp(HARMONIC_ROWS, tolerance=1e-6))
        assert np.all(r.solution.status == abi.COMPLETE)
        assert np.max(np.abs(r.y_a[1] - 1.0)) < 1e-5 and np.max(np.abs(r.solution.y_final[0] - 1.0)) < 1e-5
        res.append(r)
    assert np.array_equal(res[0].y_a, res[1].y_a) and np.array_equal(res[0].iterations, res[1].iterations)


def test_bvp_builder_matches_crate_tests():
    """tests/bvp/shooting.rs: single and multiple shooting on the harmonic oscillator, even output."""
    m = degpu.ExplicitRungeKutta.dop853().rtol(1e-10).atol(1e-12)
    sys = degpu.System.harmonic(1.0)
    for sh in (degpu.Shooting.single(m), degpu.Shooting.multiple(m).segments(4).tolerance(1e-8)):
        sol = degpu.BVP.ode(sys, 0.0, HALF_PI, [0.0, 0.5], HARMONIC_ROWS).method(sh).solve()
        assert sol.status == "Complete"
        assert abs(sol.y[0][0]) < 1e-5 and abs(sol.y[0][1] - 1.0) < 1e-5
        assert abs(sol.y[-1][0] - 1.0) < 1e-5 and abs(sol.y[-1][1]) < 1e-5
    sol = degpu.BVP.ode(sys, 0.0, HALF_PI, [0.0, 0.5], HARMONIC_ROWS) \
        .method(degpu.Shooting.multiple(m).segments(3).tolerance(1e-8)).t_eval([i * HALF_PI / 4 for i in range(5)]) \
        .solve()
    assert len(sol.t) == 5 and abs(sol.t[0]) < 1e-12 and abs(sol.t[4] - HALF_PI) < 1e-12
