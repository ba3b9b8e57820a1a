"""The oracle's restatement of the crate's event detection (EventWrappedSolout with the Brent–Dekker
search, src/solout/event.rs:299-521), pinned against exact event times and the configurations of
the crate's event examples and tests:
  * examples/ode/03_logistic_growth: y' = k y (1 - y/m), k = 1, m = 10, y(0) = 1, terminal event
    y - 0.9 m; the exact solution reaches 9 at t = ln 81;
  * tests/ode/errors.rs: y' = y with the terminal event t - 10 attached; bad inputs still fail
    with BadInput, and a valid interval stops at t = 10;
  * examples/ode/05_damped_pendulum: max(|theta|, |omega|) - 0.01 with RKF45 over output times;
  * the harmonic oscillator's zeros pi/2 + j pi for non-terminal events and their directions;
  * the duplicate rule: an event within 1e-14 of the last point of the solution is counted
    (it can terminate) but not recorded."""
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

R = abi.RHS


def cfg_for(method, h0=0.0, dense_mode=abi.DENSE_REFERENCE):
    cfg = abi.default_cfg(method)
    cfg.h0 = h0
    cfg.dense_mode = dense_mode
    cfg.max_steps = 10_000_000
    return cfg


def one(rhs, y0, params, t0, tf, rtol, atol=None, t_eval=None):
    d = len(y0)
    return O.Batch(R[rhs], d, len(params), [t0], [tf], np.array(y0, dtype=float)[:, None],
                   np.array(params, dtype=float)[:, None] if params else None, [rtol],
                   [rtol if atol is None else atol], t_eval=t_eval)


def test_logistic_example_terminal_event():
    b = one("LOGISTIC", [1.0], [1.0, 10.0], 0.0, 10.0, 1e-12)
    ev = abi.make_event(abi.EVENT_LINEAR, [0], [1.0], offset=-(0.9 * 10.0), terminate=1)
    o = O.solve_event(b, cfg_for(abi.DOP853), ev)
    assert int(o["status"][0]) == abi.INTERRUPTED
    assert int(o["cross_count"][0]) == 1
    # the crate's DOP853 dense fold (not the published one) bounds the accuracy here
    assert abs(o["cross_t"][0, 0] - math.log(81.0)) < 1e-8
    assert abs(o["cross_y"][0, 0, 0] - 9.0) < 1e-8
    # the solve stops at the end of the step that holds the event
    assert math.log(81.0) < o["t_final"][0] < 10.0


def test_errors_rs_event_cases():
    ev = abi.make_event(abi.EVENT_LINEAR, [], t_weight=1.0, offset=-10.0, terminate=1)
    for method, h0 in [(abi.DOP853, 0.0), (abi.DOPRI5, 0.0), (abi.RKF45, 0.1), (abi.RK4, 0.1)]:
        bad_span = O.solve_event(one("EXP_GROWTH", [1.0], [1.0], 0.0, 0.0, 1e-6), cfg_for(method, h0), ev)
        assert int(bad_span["status"][0]) == abi.ERR_BAD_INPUT
        big_h0 = O.solve_event(one("EXP_GROWTH", [1.0], [1.0], 0.0, 1.0, 1e-6), cfg_for(method, 10.0), ev)
        assert int(big_h0["status"][0]) == abi.ERR_BAD_INPUT
        ok = O.solve_event(one("EXP_GROWTH", [1.0], [1.0], 0.0, 20.0, 1e-10),
                           cfg_for(method, 0.01 if method == abi.RK4 else h0), ev)
        assert int(ok["status"][0]) == abi.INTERRUPTED
        assert int(ok["cross_count"][0]) == 1 and abs(ok["cross_t"][0, 0] - 10.0) < 1e-12
        # the state interpolated at the event (DOP853 with the crate's dense fold is the loosest)
        assert abs(ok["cross_y"][0, 0, 0] / math.exp(10.0) - 1.0) < 1e-5


@pytest.mark.parametrize("method,h0,tol", [(abi.DOP853, 0.0, 1e-9), (abi.DOPRI5, 0.0, 1e-7),
                                           (abi.RKF45, 0.0, 1e-6), (abi.CASH_KARP, 0.0, 1e-6),
                                           (abi.RK4, 1e-3, 1e-8)])
def test_harmonic_event_times_and_directions(method, h0, tol):
    b = one("HARMONIC", [1.0, 0.0], [1.0], 0.0, 10.0, 1e-11)
    cfg = cfg_for(method, h0, abi.DENSE_HAIRER)
    exact = [math.pi / 2 + j * math.pi for j in range(3)]
    both = O.solve_event(b, cfg, abi.make_event(abi.EVENT_LINEAR, [0], [1.0]))
    assert int(both["status"][0]) == abi.COMPLETE and int(both["cross_count"][0]) == 3
    assert np.max(np.abs(both["cross_t"][:3, 0] - exact)) < tol
    neg = O.solve_event(b, cfg, abi.make_event(abi.EVENT_LINEAR, [0], [1.0], direction=abi.CROSS_NEGATIVE))
    pos = O.solve_event(b, cfg, abi.make_event(abi.EVENT_LINEAR, [0], [1.0], direction=abi.CROSS_POSITIVE))
    assert int(neg["cross_count"][0]) == 2 and int(pos["cross_count"][0]) == 1
    assert abs(pos["cross_t"][0, 0] - 1.5 * math.pi) < tol
    # terminate after the second event
    two = O.solve_event(b, cfg, abi.make_event(abi.EVENT_LINEAR, [0], [1.0], terminate=2))
    assert int(two["status"][0]) == abi.INTERRUPTED and int(two["cross_count"][0]) == 2
    assert 1.5 * math.pi < two["t_final"][0] < 2.5 * math.pi


def test_damped_pendulum_example_shape():
    """The example's event max(|theta|, |omega|) - 0.01 with RKF45 over output times, on the
    damped pendulum theta'' = -0.2 theta' - sin theta (the library's pendulum with no drive)."""
    t_out = [0.0, 1.0, 3.0, 4.5, 6.9, 10.0]
    b = one("PENDULUM", [1.0, 0.0], [0.2, 0.0, 0.0], 0.0, 100.0, 1e-6, t_eval=t_out)
    ev = abi.make_event(abi.EVENT_MAX_ABS, [0, 1], offset=-0.01, terminate=1)
    o = O.solve_event(b, cfg_for(abi.RKF45), ev)
    assert int(o["status"][0]) == abi.INTERRUPTED and int(o["cross_count"][0]) == 1
    te = o["cross_t"][0, 0]
    y = o["cross_y"][0, :, 0]
    # The crate's Brent–Dekker keeps no bracket after its first step (a is reset to c, which then
    # equals the previous b): it runs as a step-limited secant search and stops once a step is
    # below tolerance, which on this curved g leaves the time off the root by ~1e-5.
    assert abs(max(abs(y[0]), abs(y[1])) - 0.01) < 1e-6
    # the output times were all reached before the event, at the interpolated states
    assert te > 10.0 and not np.any(np.isnan(o["dense"][:, :, 0]))
    assert o["dense"][0, 0, 0] == 1.0


def test_duplicate_event_is_counted_not_recorded():
    # g = t - 1 with an output time at 1: the event coincides with the last output point
    b = one("HARMONIC", [1.0, 0.0], [1.0], 0.0, 5.0, 1e-9, t_eval=[0.5, 1.0, 2.0])
    ev = abi.make_event(abi.EVENT_LINEAR, [], t_weight=1.0, offset=-1.0, terminate=1)
    o = O.solve_event(b, cfg_for(abi.DOPRI5), ev)
    assert int(o["status"][0]) == abi.INTERRUPTED
    assert int(o["cross_count"][0]) == 0
    # without the output times (default output: every step's end) the event is recorded
    b2 = one("HARMONIC", [1.0, 0.0], [1.0], 0.0, 5.0, 1e-9)
    o2 = O.solve_event(b2, cfg_for(abi.DOPRI5), ev)
    assert int(o2["cross_count"][0]) == 1 and abs(o2["cross_t"][0, 0] - 1.0) < 1e-12
    # an event exactly at tf coincides with the final step's end: counted, not recorded
    b3 = one("HARMONIC", [1.0, 0.0], [1.0], 0.0, 1.0, 1e-9)
    o3 = O.solve_event(b3, cfg_for(abi.DOPRI5), ev)
    assert int(o3["status"][0]) == abi.INTERRUPTED and int(o3["cross_count"][0]) == 0
    assert o3["t_final"][0] == 1.0


def test_backward_integration_finds_no_event():
    """The crate's interpolator refuses every time inside a backward step (OutOfBounds), so the
    Brent–Dekker search gives up and no event is counted."""
    b = one("HARMONIC", [1.0, 0.0], [1.0], 0.0, -10.0, 1e-10)
    o = O.solve_event(b, cfg_for(abi.DOPRI5), abi.make_event(abi.EVENT_LINEAR, [0], [1.0], terminate=1))
    assert int(o["status"][0]) == abi.COMPLETE and int(o["cross_count"][0]) == 0
