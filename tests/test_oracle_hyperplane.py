"""The oracle's restatement of the crate's hyperplane crossing detection (HyperplaneCrossingSolout,
src/solout/hyperplane.rs), pinned against exact crossing times and the crate's CR3BP example
configuration (examples/ode/07_cr3bp/main.rs). The crate holds no test of hyperplane outputs, so
the pins are analytic:
  * the harmonic oscillator x = cos(w t), v = -w sin(w t) crosses the plane x + v/w = 0 at
    w t = pi/4 + j pi;
  * an axis-aligned plane monitors the same quantity as a component crossing;
  * a trajectory that starts on the plane records a crossing at t0 (hyperplane.rs's zero rule);
  * the CR3BP near-rectilinear orbit is periodic, so its crossings repeat with the period."""
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

R = abi.RHS


def harmonic_batch(ks, tf, rtol, y0=(1.0, 0.0)):
    n = len(ks)
    return O.Batch(R["HARMONIC"], 2, 1, np.zeros(n), np.full(n, tf), np.stack([np.full(n, y0[0]), np.full(n, y0[1])]),
                   np.array(ks)[None, :], np.full(n, rtol), np.full(n, rtol))


def dop853(dense_mode=abi.DENSE_HAIRER):
    cfg = abi.default_cfg(abi.DOP853)
    cfg.dense_mode = dense_mode
    cfg.max_steps = 10_000_000
    return cfg


@pytest.mark.parametrize("scale", [1.0, 3.5, 1e-3])
def test_harmonic_plane_crossings(scale):
    """The plane x + v / w = 0 (normal (1, 1/w), any length): crossings at (pi/4 + j pi) / w."""
    for k in [1.0, 4.0, 0.25]:
        w = math.sqrt(k)
        o = O.solve_hyperplane(harmonic_batch([k], 10.0, 1e-11), dop853(), [0, 1], [0.0, 0.0], [scale, scale / w],
                               abi.CROSS_BOTH, 16)
        exact = [(0.25 * math.pi + j * math.pi) / w for j in range(32) if (0.25 * math.pi + j * math.pi) / w < 10.0]
        cnt = int(o["cross_count"][0])
        assert cnt == len(exact)
        got = o["cross_t"][:cnt, 0]
        assert np.max(np.abs(got - exact)) < 1e-9
        # the recorded state lies on the plane
        y = o["cross_y"][:cnt, :, 0]
        assert np.max(np.abs(y[:, 0] + y[:, 1] / w)) < 1e-9


def test_normal_length_is_irrelevant():
    b = harmonic_batch([1.0], 10.0, 1e-10)
    a = O.solve_hyperplane(b, dop853(), [0, 1], [0.0, 0.0], [1.0, 1.0])
    c = O.solve_hyperplane(b, dop853(), [0, 1], [0.0, 0.0], [7.0, 7.0])
    assert np.array_equal(a["cross_count"], c["cross_count"])
    m = int(a["cross_count"][0])
    assert np.max(np.abs(a["cross_t"][:m] - c["cross_t"][:m])) < 1e-12


@pytest.mark.parametrize("direction", [abi.CROSS_BOTH, abi.CROSS_POSITIVE, abi.CROSS_NEGATIVE])
def test_axis_plane_matches_component_crossing(direction):
    """Normal e_0 through (thr, .): the signed distance is y0 - thr exactly, so the same crossings
    are found; the located times agree to the Newton tolerance."""
    b = harmonic_batch([1.0, 2.0], 12.0, 1e-10)
    cfg = dop853()
    hp = O.solve_hyperplane(b, cfg, [0, 1], [0.3, -5.0], [1.0, 0.0], direction)
    cr = O.solve_crossing(b, cfg, 0, 0.3, direction)
    assert np.array_equal(hp["cross_count"], cr["cross_count"])
    assert np.array_equal(hp["accepted"], cr["accepted"]) and np.array_equal(hp["y_final"], cr["y_final"])
    m = ~np.isnan(cr["cross_t"])
    assert np.array_equal(m, ~np.isnan(hp["cross_t"]))
    assert np.max(np.abs(hp["cross_t"][m] - cr["cross_t"][m])) < 1e-12


def test_start_on_plane_counts():
    """y(0) = (0, 1): x leaves the plane x = 0 upwards at t0. The hyperplane rule records a
    crossing at t0 (the previous distance is exactly zero); the component rule does not
    (signum(+0) = signum(positive))."""
    b = harmonic_batch([1.0], 5.0, 1e-10, y0=(0.0, 1.0))
    hp = O.solve_hyperplane(b, dop853(), [0], [0.0], [1.0])
    cr = O.solve_crossing(b, dop853(), 0, 0.0)
    # x = sin t: zero at pi (and at t0 for the plane rule)
    assert int(hp["cross_count"][0]) == 2 and int(cr["cross_count"][0]) == 1
    assert hp["cross_t"][0, 0] == 0.0
    assert abs(hp["cross_t"][1, 0] - math.pi) < 1e-9 and abs(cr["cross_t"][0, 0] - math.pi) < 1e-9


def cr3bp_example_batch(n_periods=3.0, rtol=1e-12):
    # examples/ode/07_cr3bp/main.rs: Earth-Moon mass ratio, near-rectilinear orbit, tf = 3 periods
    mu = 0.012150585609624
    y0 = np.array([1.021881345465263, 0.0, -0.182, 0.0, -0.102950816739606, 0.0])[:, None]
    period = 1.509263667286943
    return O.Batch(R["CR3BP"], 6, 1, np.zeros(1), np.array([n_periods * period]), y0, np.array([[mu]]),
                   np.array([rtol]), np.array([rtol])), period


def test_cr3bp_example_plane_crossings():
    """The example's plane (point (1, 0, 0), normal (0.5, 0.5, 0), position extracted) with DOP853
    at rtol = atol = 1e-12: the crossings lie on the plane and repeat with the orbit's period."""
    b, period = cr3bp_example_batch()
    o = O.solve_hyperplane(b, dop853(abi.DENSE_REFERENCE), [0, 1, 2], [1.0, 0.0, 0.0], [0.5, 0.5, 0.0],
                           abi.CROSS_BOTH, 32)
    cnt = int(o["cross_count"][0])
    assert int(o["status"][0]) == abi.COMPLETE
    assert cnt >= 3 and cnt % 3 == 0
    per = cnt // 3
    t = o["cross_t"][:cnt, 0]
    assert np.all(np.diff(t) > 0)
    # the same crossing one period later
    assert np.max(np.abs(t[per:] - t[:-per] - period)) < 1e-6
    y = o["cross_y"][:cnt, :, 0]
    dist = ((y[:, 0] - 1.0) * 0.5 + y[:, 1] * 0.5) / math.sqrt(0.5)
    assert np.max(np.abs(dist)) < 1e-9
