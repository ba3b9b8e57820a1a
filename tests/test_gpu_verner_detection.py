"""Crossing, hyperplane and event detection with Verner's pairs (RKV655e … RKV989e) on the device
against the oracle: the detectors search the pairs' own interpolants (src/methods/erk/adaptive/
ordinary.rs:241-275) as the crate's CrossingSolout, HyperplaneCrossingSolout and
EventWrappedSolout do, and with FP64 parity arithmetic every count, time, state, counter and final
state is bit for bit the oracle's. A mixed configuration runs these pairs in FP64 fast arithmetic."""
import math

import numpy as np
import pytest

from degpu import abi, workloads as W
from test_gpu_crossing import assert_same, cfg_for, family_ensemble, gpu_crossing, oracle_crossing
from test_gpu_event import assert_same_event, gpu_event, oracle_event
from test_gpu_hyperplane import PLANES, gpu_plane, oracle_plane

pytestmark = pytest.mark.gpu
VERNER = [abi.RKV655E, abi.RKV656E, abi.RKV766E, abi.RKV767E, abi.RKV877E, abi.RKV878E, abi.RKV988E, abi.RKV989E]


@pytest.mark.parametrize("fam,comp,thr", [("VAN_DER_POL", 0, 0.0), ("LORENZ", 2, 25.0)])
@pytest.mark.parametrize("method", VERNER)
def test_verner_crossing_parity(fam, comp, thr, method):
    e = family_ensemble(fam, 300, first=1500)
    cfg = cfg_for(method)
    g = gpu_crossing(e, cfg, comp, thr, abi.CROSS_BOTH, 3)
    o = oracle_crossing(e, cfg, comp, thr, abi.CROSS_BOTH, 3)
    assert np.mean(o["cross_count"] > 0) > 0.5
    assert_same(g, o)


@pytest.mark.parametrize("method", [abi.RKV656E, abi.RKV877E, abi.RKV989E])
def test_verner_hyperplane_parity(method):
    e = family_ensemble("PENDULUM", 300, first=2500)
    cfg = cfg_for(method)
    comps, point, normal = PLANES["PENDULUM"]
    g = gpu_plane(e, cfg, comps, point, normal, abi.CROSS_BOTH, 4)
    o = oracle_plane(e, cfg, comps, point, normal, abi.CROSS_BOTH, 4)
    assert np.mean(o["cross_count"] > 0) > 0.5
    assert_same(g, o)


@pytest.mark.parametrize("method", [abi.RKV766E, abi.RKV878E, abi.RKV988E])
def test_verner_terminal_event_parity_with_output_times(method):
    """Output times as the base output, a terminal event, the family map."""
    e = W.config1(n=600, first=40000)
    e.tf = np.minimum(e.tf, 12.0)
    cfg = cfg_for(method)
    ev = abi.make_event(abi.EVENT_LINEAR, [0], [1.0], 0.0, -0.2, abi.CROSS_BOTH, 2, 4)
    t_eval = np.array([0.0, 0.7, 2.5, 6.0, 11.0, 3.3])
    g = gpu_event(e, cfg, ev, t_eval)
    o = oracle_event(e, cfg, ev, t_eval)
    assert np.any(o["status"] == abi.INTERRUPTED) and np.any(o["status"] == abi.COMPLETE)
    assert_same_event(g, o)


def test_verner_mixed_runs_fp64_fast():
    """A mixed crossing solve with a Verner pair returns the FP64 fast solve's bits."""
    e = family_ensemble("VAN_DER_POL", 400, first=6000)
    a = gpu_crossing(e, cfg_for(abi.RKV767E, abi.MIXED), 0, 0.0, abi.CROSS_BOTH, 6)
    b = gpu_crossing(e, cfg_for(abi.RKV767E, abi.FP64_FAST), 0, 0.0, abi.CROSS_BOTH, 6)
    assert_same(a, b)
    o = oracle_crossing(e, cfg_for(abi.RKV767E), 0, 0.0, abi.CROSS_BOTH, 6)
    assert np.array_equal(a["cross_count"], o["cross_count"])


def test_verner_builder_harmonic_crossings():
    """IVP::ode(..).method(rkv655e()).crossing(0, 0.0, Both) on the harmonic oscillator: zeros of
    cos t on [0, 10]."""
    import degpu

    m = degpu.ExplicitRungeKutta.rkv655e().rtol(1e-11).atol(1e-11)
    sol = degpu.IVP.ode(degpu.System.harmonic(1.0), 0.0, 10.0, [1.0, 0.0]).method(m).crossing(0, 0.0).solve()
    assert sol.status == "Complete"
    assert np.allclose(sol.t, [math.pi / 2 + j * math.pi for j in range(3)], rtol=0, atol=1e-11)
