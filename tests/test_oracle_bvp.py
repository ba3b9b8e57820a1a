"""The oracle's restatement of the crate's shooting methods (src/methods/bvp/shooting/single.rs,
multiple.rs) and its dense LU (src/linalg/lu.rs), pinned against the crate's own BVP tests
(tests/bvp/shooting.rs with the systems of tests/bvp/systems.rs; the unit tests of single.rs):
  * harmonic oscillator y'' = -y, y(0) = 0, y(pi/2) = 1: y(0)' = 1, y(pi/2)' = 0;
  * pipe heat transfer T'' = b^2 (T - T_amb), T(0) = T_in, T'(L) = 0 against its analytical
    initial gradient and outlet temperature;
  * multiple shooting counts Jacobian columns and Newton iterations;
  * a singular Jacobian is LinearAlgebra, an iteration cap MaxSteps."""
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

R = abi.RHS
HALF_PI = math.pi / 2


def dop853(rtol=1e-10, atol=1e-12):
    cfg = abi.default_cfg(abi.DOP853)
    cfg.max_steps = 10_000_000
    return cfg, rtol, atol


def batch(rhs, params, t0, tf, guess, rtol, atol, t_eval=None):
    d = len(guess)
    return O.Batch(R[rhs], d, len(params), [t0], [tf], np.array(guess, dtype=float)[:, None],
                   np.array(params, dtype=float)[:, None], [rtol], [atol], t_eval=t_eval)


HARMONIC_ROWS = [(0, 0, 0.0), (1, 0, 1.0)]  # res[0] = y_a[0], res[1] = y_b[0] - target


@pytest.mark.parametrize("method,segments,tol", [(abi.BVP_SINGLE, 4, 1e-6), (abi.BVP_MULTIPLE, 4, 1e-8),
                                                 (abi.BVP_MULTIPLE, 3, 1e-8)])
def test_harmonic_oscillator_bvp(method, segments, tol):
    cfg, rtol, atol = dop853()
    b = batch("HARMONIC", [1.0], 0.0, HALF_PI, [0.0, 0.5], rtol, atol)
    o = O.solve_bvp(b, cfg, abi.make_bvp(HARMONIC_ROWS, method, segments, tolerance=tol))
    assert int(o["status"][0]) == abi.COMPLETE
    ya, yb = o["y_a"][:, 0], o["y_final"][:, 0]
    assert abs(ya[0]) < 1e-5 and abs(ya[1] - 1.0) < 1e-5          # shooting.rs:8-21
    assert abs(yb[0] - 1.0) < 1e-5 and abs(yb[1]) < 1e-5
    assert int(o["iterations"][0]) > 0 and int(o["jacobian"][0]) > 0  # shooting.rs:49-50
    unknowns = 2 if method == abi.BVP_SINGLE else 2 * (segments + 1)
    assert int(o["jacobian"][0]) == unknowns * int(o["iterations"][0])


def test_harmonic_even_output_and_default_tolerances():
    """shooting.rs:53-70: even output (pi/8 spacing) through the final solve; single.rs's unit
    test with DOP853 at its default tolerances."""
    cfg, rtol, atol = dop853()
    te = [i * HALF_PI / 4 for i in range(5)]
    b = batch("HARMONIC", [1.0], 0.0, HALF_PI, [0.0, 0.5], rtol, atol, t_eval=te)
    o = O.solve_bvp(b, cfg, abi.make_bvp(HARMONIC_ROWS, abi.BVP_MULTIPLE, 3, tolerance=1e-8))
    assert int(o["status"][0]) == abi.COMPLETE
    assert np.max(np.abs(o["dense"][:, 0, 0] - np.sin(te))) < 1e-5
    cfg6 = abi.default_cfg(abi.DOP853)
    b6 = batch("HARMONIC", [1.0], 0.0, HALF_PI, [0.0, 0.5], 1e-6, 1e-6)
    o6 = O.solve_bvp(b6, cfg6, abi.make_bvp(HARMONIC_ROWS))
    assert int(o6["status"][0]) == abi.COMPLETE
    assert abs(o6["y_a"][1, 0] - 1.0) < 1e-5 and abs(o6["y_final"][0, 0] - 1.0) < 1e-5


@pytest.mark.parametrize("method,segments,tol", [(abi.BVP_SINGLE, 4, 1e-6), (abi.BVP_MULTIPLE, 5, 1e-8)])
def test_pipe_heat_transfer_bvp(method, segments, tol):
    """shooting.rs:87-125: ambient 293.15, loss rate 0.2, inlet 373.15, L = 10."""
    amb, beta, t_in, length = 293.15, 0.2, 373.15, 10.0
    cfg, rtol, atol = dop853()
    b = batch("PIPE_HEAT", [beta, amb], 0.0, length, [t_in, -5.0], rtol, atol)
    rows = [(0, 0, t_in), (1, 1, 0.0)]  # res[0] = y_a[0] - T_in, res[1] = y_b[1]
    o = O.solve_bvp(b, cfg, abi.make_bvp(rows, method, segments, tolerance=tol))
    assert int(o["status"][0]) == abi.COMPLETE
    theta0, bl = t_in - amb, beta * length
    grad0 = -beta * theta0 * math.tanh(bl)
    outlet = amb + theta0 / math.cosh(bl)
    assert abs(o["y_a"][0, 0] - t_in) < 1e-8
    assert abs(o["y_final"][1, 0]) < 1e-5
    assert abs(o["y_a"][1, 0] - grad0) < 1e-4
    assert abs(o["y_final"][0, 0] - outlet) < 1e-4


def test_singular_jacobian_and_iteration_cap():
    cfg, rtol, atol = dop853()
    # both rows constrain y(t0)[0]: the Jacobian's second column is zero
    b = batch("HARMONIC", [1.0], 0.0, HALF_PI, [0.3, 0.5], rtol, atol)
    o = O.solve_bvp(b, cfg, abi.make_bvp([(0, 0, 0.0), (0, 0, 1.0)]))
    assert int(o["status"][0]) == abi.ERR_LINEAR_ALGEBRA
    # one Newton iteration is not enough from this guess: MaxSteps with the guess as state
    o = O.solve_bvp(b, cfg, abi.make_bvp(HARMONIC_ROWS, max_iterations=1, tolerance=1e-14))
    assert int(o["status"][0]) == abi.ERR_MAX_STEPS
    assert o["y_final"][0, 0] == 0.3 and o["t_final"][0] == 0.0


def test_linear_problem_converges_in_one_newton_step():
    """The harmonic oscillator is linear: from any guess Newton lands on the solution in one step
    (the second iteration only confirms it)."""
    rng = np.random.default_rng(5)
    cfg, rtol, atol = dop853()
    for guess in rng.uniform(-2, 2, (5, 2)):
        b = batch("HARMONIC", [1.0], 0.0, HALF_PI, list(guess), rtol, atol)
        o = O.solve_bvp(b, cfg, abi.make_bvp(HARMONIC_ROWS))
        assert int(o["status"][0]) == abi.COMPLETE and int(o["iterations"][0]) <= 2
