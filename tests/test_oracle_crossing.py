"""The oracle's restatement of the crate's crossing detection (CrossingSolout,
src/solout/crossing.rs:200-330), pinned against exact crossing times: the harmonic oscillator
x'' = -k x, x(0) = 1, x'(0) = 0 crosses zero at t_j = (pi/2 + j pi) / sqrt(k). The crate's own
tests do not pin crossing outputs (its crossing tests check construction only)."""
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

R = abi.RHS


def harmonic_batch(ks, tf, rtol):
    n = len(ks)
    return O.Batch(R["HARMONIC"], 2, 1, np.zeros(n), np.full(n, tf), np.stack([np.ones(n), np.zeros(n)]),
                   np.array(ks)[None, :], np.full(n, rtol), np.full(n, rtol))


# DOP853 with the crate's own dense fold (its alternation of s and 1 - s differs from the published
# continuous extension) locates crossings to about 1e-7; with the published fold to 1e-9.
@pytest.mark.parametrize("method,h0,dense_mode,tol", [(abi.DOP853, 0.0, abi.DENSE_REFERENCE, 1e-6),
                                                      (abi.DOP853, 0.0, abi.DENSE_HAIRER, 1e-9),
                                                      (abi.DOPRI5, 0.0, abi.DENSE_REFERENCE, 1e-7),
                                                      (abi.RK4, 1e-3, abi.DENSE_REFERENCE, 1e-9)])
def test_harmonic_zero_crossings(method, h0, dense_mode, tol):
    ks = [1.0, 2.0, 0.5]
    b = harmonic_batch(ks, 10.0, 1e-11)
    cfg = abi.default_cfg(method)
    cfg.h0 = h0
    cfg.dense_mode = dense_mode
    cfg.max_steps = 10_000_000
    o = O.solve_crossing(b, cfg, component=0, threshold=0.0, direction=abi.CROSS_BOTH, max_points=8)
    for i, k in enumerate(ks):
        w = math.sqrt(k)
        exact = [(math.pi / 2 + j * math.pi) / w for j in range(16) if (math.pi / 2 + j * math.pi) / w < 10.0]
        cnt = int(o["cross_count"][i])
        assert cnt == len(exact)
        got = o["cross_t"][:min(cnt, 8), i]
        assert np.max(np.abs(got - exact[:8])) < tol
        # the recorded state is the interpolant at the crossing: x ~ 0 there
        assert np.max(np.abs(o["cross_y"][:min(cnt, 8), 0, i])) < 10 * tol
        assert np.all(np.isnan(o["cross_t"][cnt:, i]))


def test_crossing_directions():
    b = harmonic_batch([1.0], 10.0, 1e-10)
    cfg = abi.default_cfg(abi.DOP853)
    cfg.dense_mode = abi.DENSE_HAIRER
    pos = O.solve_crossing(b, cfg, 0, 0.0, abi.CROSS_POSITIVE)
    neg = O.solve_crossing(b, cfg, 0, 0.0, abi.CROSS_NEGATIVE)
    both = O.solve_crossing(b, cfg, 0, 0.0, abi.CROSS_BOTH)
    # x = cos t goes down through 0 at pi/2, up at 3pi/2, down at 5pi/2 ...
    assert int(neg["cross_count"][0]) == 2 and int(pos["cross_count"][0]) == 1
    assert int(both["cross_count"][0]) == 3
    assert abs(pos["cross_t"][0, 0] - 1.5 * math.pi) < 1e-8
    assert np.allclose(np.sort(np.concatenate([pos["cross_t"][:1, 0], neg["cross_t"][:2, 0]])),
                       both["cross_t"][:3, 0], rtol=0, atol=0)


def test_threshold_and_capacity():
    # x = cos t crosses 0.5 at t = pi/3, 5pi/3, 7pi/3 on [0, 10]; capacity 2 keeps the first two
    b = harmonic_batch([1.0], 10.0, 1e-11)
    cfg = abi.default_cfg(abi.DOP853)
    cfg.dense_mode = abi.DENSE_HAIRER
    o = O.solve_crossing(b, cfg, 0, 0.5, abi.CROSS_BOTH, max_points=2)
    assert int(o["cross_count"][0]) == 3
    assert np.allclose(o["cross_t"][:, 0], [math.pi / 3, 5 * math.pi / 3], atol=1e-9)
    assert np.allclose(o["cross_y"][:, 0, 0], 0.5, atol=1e-9)


def test_verner_harmonic_zero_crossings():
    """Verner's pairs on the same oscillators: every crossing is found. Newton's search on the
    6(5) and 7(6) pairs' interpolants converges to the root; on the larger pairs the
    interpolant's rounding at some crossings stays above the crate's convergence test (100 eps)
    and the crate falls back to the linear estimate, up to ~5e-4 away."""
    ks = [1.0, 2.0, 0.5]
    b = harmonic_batch(ks, 10.0, 1e-11)
    for method in range(abi.RKV655E, abi.RKV989E + 1):
        cfg = abi.default_cfg(method)
        cfg.max_steps = 10_000_000
        o = O.solve_crossing(b, cfg, component=0, threshold=0.0, direction=abi.CROSS_BOTH, max_points=8)
        tol = 1e-11 if method <= abi.RKV766E else 1e-3
        for i, k in enumerate(ks):
            w = math.sqrt(k)
            exact = [(math.pi / 2 + j * math.pi) / w for j in range(16) if (math.pi / 2 + j * math.pi) / w < 10.0]
            assert int(o["cross_count"][i]) == len(exact)
            assert np.max(np.abs(o["cross_t"][:len(exact), i] - exact)) < tol
