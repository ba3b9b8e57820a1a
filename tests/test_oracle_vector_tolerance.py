"""Per-component tolerances in the oracle (the crate's Tolerance::Vector, src/tolerance.rs:11-68),
read per component by error_norm (src/traits.rs:394-410), the Adaptive family's infinity norm
(src/traits.rs:413-433) and the initial step (src/methods/h_init.rs:76-82).

  * a vector whose entries all equal the scalar gives the scalar's solve bit for bit;
  * examples/ode/17_quadrature (DOP853, rtol = atol = [1e-12, 1e-12, 1e-6] on a damped oscillator
    augmented with the dissipated energy W): the energy balance E(t_f) + W(t_f) = E0 holds, and
    the loose tolerance on W costs no steps over the tight one on (x, v) alone."""
import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W

R = abi.RHS


def cfg_for(method):
    c = abi.default_cfg(method)
    c.max_steps = 10_000_000
    return c


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853, abi.RKF45, abi.CASH_KARP, abi.RKV656E])
def test_uniform_vector_equals_scalar(method):
    e = W.config0(n=64)
    e.tf[:] = 5.0
    b = O.Batch(e.rhs_id, 3, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol)
    bv = O.Batch(e.rhs_id, 3, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol,
                 rtol_vec=np.repeat(e.rtol[None, :], 3, axis=0), atol_vec=np.repeat(e.atol[None, :], 3, axis=0))
    o, ov = O.solve(b, cfg_for(method)), O.solve(bv, cfg_for(method))
    for k in ("y_final", "accepted", "rejected", "fevals", "status"):
        assert np.array_equal(o[k], ov[k]), k


def quadrature_case(rtol_vec, atol_vec, n=1):
    k, m, c = 4.0, 1.0, 0.4
    return O.Batch(R["DAMPED_QUADRATURE"], 3, 3, np.zeros(n), np.full(n, 20.0),
                   np.array([[1.0], [0.0], [0.0]]).repeat(n, axis=1), np.array([[k], [m], [c]]).repeat(n, axis=1),
                   np.full(n, 1e-12), np.full(n, 1e-12), rtol_vec=rtol_vec, atol_vec=atol_vec)


def test_quadrature_example_energy_balance():
    tol = [1e-12, 1e-12, 1e-6]
    o = O.solve(quadrature_case(tol, tol), cfg_for(abi.DOP853))
    assert int(o["status"][0]) == abi.COMPLETE
    x, v, w = o["y_final"][:, 0]
    e0 = 0.5 * 4.0 * 1.0
    e_final = 0.5 * 4.0 * x * x + 0.5 * 1.0 * v * v
    assert abs(e0 - e_final - w) < 1e-6
    # W is integrated to its own, looser tolerance: its error is far above that of (x, v), whose
    # tolerance drives the step size; a tight tolerance on W too takes more steps
    tight = O.solve(quadrature_case(None, None), cfg_for(abi.DOP853))
    assert int(o["accepted"][0]) <= int(tight["accepted"][0])
    assert abs(tight["y_final"][0, 0] - x) < 1e-9 and abs(tight["y_final"][1, 0] - v) < 1e-9


def test_vector_changes_the_solve():
    """Loosening one component's tolerance changes the steps of a system whose error is led by
    that component."""
    e = W.config0(n=32)
    e.tf[:] = 5.0
    rv = np.repeat(e.rtol[None, :], 3, axis=0)
    rv[2] *= 1e3
    b = O.Batch(e.rhs_id, 3, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol)
    bv = O.Batch(e.rhs_id, 3, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, rtol_vec=rv)
    o, ov = O.solve(b, cfg_for(abi.DOPRI5)), O.solve(bv, cfg_for(abi.DOPRI5))
    assert np.all(ov["accepted"] <= o["accepted"]) and np.any(ov["accepted"] < o["accepted"])
