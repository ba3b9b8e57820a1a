"""Per-component tolerances (the crate's Tolerance::Vector, src/tolerance.rs:11-68) on the device:
error_norm (src/traits.rs:394-410), the Adaptive family's infinity norm and the initial step
(src/methods/h_init.rs:76-82) read one tolerance per component.  With FP64 parity arithmetic every
counter and final state equals the oracle's bit for bit, on the one-system-per-thread, persistent
multi-family and group-per-system kernels; the mixed form stays within its accuracy."""
import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W
from test_gpu_parity import assert_parity, cfg_for, gpu_solve

pytestmark = pytest.mark.gpu


def spread(e, seed):
    """Per-component tolerances around each instance's scalar: factors log-uniform in [0.1, 10]."""
    rng = np.random.default_rng(seed)
    f = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (e.dim, e.n)))
    return e.rtol[None, :] * f, e.atol[None, :] * f[::-1]


def oracle_vec(e, cfg, rv, av, t_eval=None):
    b = O.Batch(e.rhs_id, e.dim, e.n_params, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, t_eval=t_eval,
                dims=e.dims, family=e.family, rtol_vec=rv, atol_vec=av)
    return O.solve(b, cfg, math_mode=1)


def gpu_vec(e, cfg, rv, av, t_eval=None):
    import degpu

    m = degpu.ExplicitRungeKutta(cfg.method)
    m.cfg = cfg
    return degpu.solve_ensemble(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m, t_eval=t_eval,
                                dims=e.dims, family=e.family, n_params=e.n_params, rtol_vec=rv, atol_vec=av)


def test_quadrature_example_parity():
    """examples/ode/17_quadrature: DOP853, rtol = atol = [1e-12, 1e-12, 1e-6], output every 0.2."""
    n = 64
    rng = np.random.default_rng(5)
    k = 4.0 * (1.0 + 0.1 * rng.random(n))
    e = W.Ensemble("quadrature", abi.DOP853, n, 3, 3, np.zeros(n), np.full(n, 20.0),
                   np.array([[1.0], [0.0], [0.0]]).repeat(n, axis=1), np.stack([k, np.ones(n), np.full(n, 0.4)]),
                   np.full(n, 1e-12), np.full(n, 1e-12), rhs_id=abi.RHS["DAMPED_QUADRATURE"])
    tol = np.array([1e-12, 1e-12, 1e-6])
    te = np.arange(0.0, 20.0 + 1e-9, 0.2)
    cfg = cfg_for(abi.DOP853)
    o = oracle_vec(e, cfg, tol, tol, te)
    g = gpu_vec(e, cfg, tol, tol, te)
    assert_parity(g, o, dense=True)
    assert np.array_equal(g.y_final, o["y_final"])
    x, v, w = g.y_final
    assert np.max(np.abs(0.5 * k - (0.5 * k * x * x + 0.5 * v * v) - w)) < 1e-6


@pytest.mark.parametrize("kernel", [abi.KERNEL_THREAD, abi.KERNEL_PERSISTENT])
@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
def test_uneven_ensemble_vector_parity(kernel, method):
    e = W.config1(n=3 * 400, first=3000)
    e.tf = np.minimum(e.tf, 10.0)
    rv, av = spread(e, 1)
    cfg = cfg_for(method, kernel=kernel)
    o = oracle_vec(e, cfg, rv, av)
    g = gpu_vec(e, cfg, rv, av)
    assert_parity(g, o)
    assert np.array_equal(g.y_final, o["y_final"])
    # the vectors change the solve: not the scalar result
    s = gpu_solve(e, cfg)
    assert not np.array_equal(s.accepted, g.accepted)


@pytest.mark.parametrize("method", [abi.RKF45, abi.RKV656E])
def test_adaptive_family_vector_parity(method):
    e = W.config0(n=256)
    e.tf[:] = 8.0
    rv, av = spread(e, 2)
    cfg = cfg_for(method)
    o = oracle_vec(e, cfg, rv, av)
    g = gpu_vec(e, cfg, rv, av)
    assert_parity(g, o)
    assert np.array_equal(g.y_final, o["y_final"])


def test_fpu_chain_group_kernel_vector_parity():
    e = W.config2(n=48)
    e.tf[:] = 5.0
    te = np.linspace(0.0, 5.0, 6)
    rv, av = spread(e, 3)
    cfg = cfg_for(abi.DOP853)
    o = oracle_vec(e, cfg, rv, av, te)
    g = gpu_vec(e, cfg, rv, av, te)
    assert_parity(g, o, dense=True)


@pytest.mark.parametrize("precision", [abi.MIXED, abi.MIXED_FP64_CTRL, abi.FP64_PLAIN])
def test_vector_tolerances_other_precisions(precision):
    """Mixed and plain forms with vectors: non-chaotic slice, error against the FP64 oracle at the
    same vectors bounded as for scalar tolerances."""
    e = W.config1(n=3 * 300, first=9000)
    keep = e.family != abi.RHS["LORENZ"]
    e = e.subset(np.nonzero(keep)[0])
    e.tf = np.minimum(e.tf, 10.0)
    e.rtol[:] = 1e-6
    e.atol[:] = 1e-8
    rv, av = spread(e, 4)
    o = oracle_vec(e, cfg_for(abi.DOPRI5), rv, av)
    g = gpu_vec(e, cfg_for(abi.DOPRI5, precision=precision, kernel=abi.KERNEL_PERSISTENT), rv, av)
    assert np.all(g.status == abi.COMPLETE)
    err = np.max(np.abs(g.y_final - o["y_final"]), axis=0) / np.maximum(1.0, np.max(np.abs(o["y_final"]), axis=0))
    assert np.median(err) < (1e-9 if precision == abi.FP64_PLAIN else 1e-5)
