"""Mixed-precision bound (degpu_set_mixed_min_rtol): in a MIXED solve, instances with rtol below
the bound leave the FP32 stages for FP32-pair stages (DOPRI5, DOP853; other methods: the FP64_FAST
arithmetic) and the others run the FP32-stage form.  Each instance's result must equal, bit for bit, the same
instance solved by the arithmetic its rtol selects, on every kernel layout (persistent
multi-family, one system per thread, group per system).  The pair stages keep FP64-like accuracy
where the FP32 stages cannot."""
import numpy as np
import pytest

import degpu
from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu

BOUND = 1e-8


@pytest.fixture
def bound():
    old = {m: degpu.mixed_min_rtol(m) for m in (abi.DOPRI5, abi.DOP853)}
    yield
    for m, v in old.items():
        degpu.set_mixed_min_rtol(m, v)


def straddling(n, first=0):
    e = W.config1(n=n, first=first)
    e.tf = np.minimum(e.tf, 8.0)
    e.rtol = W.logU(7, np.arange(first, first + n), 1, 1e-10, 1e-6)
    e.atol = 1e-2 * e.rtol
    return e


def run(e, method, prec, kernel, rhs=None, dims=None, t_eval=None):
    m = degpu.ExplicitRungeKutta(method).precision(prec).kernel(kernel)
    return degpu.solve_ensemble(rhs if rhs is not None else e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol,
                                e.atol, m, family=e.family, dims=dims, t_eval=t_eval, n_params=e.params.shape[0])


def same(a, b, sel):
    assert np.array_equal(a.status[sel], b.status[sel])
    assert np.array_equal(a.accepted[sel], b.accepted[sel])
    assert np.array_equal(a.rejected[sel], b.rejected[sel])
    assert np.array_equal(a.fevals[sel], b.fevals[sel])
    assert np.array_equal(a.y_final[:, sel], b.y_final[:, sel])


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
@pytest.mark.parametrize("kernel", [abi.KERNEL_PERSISTENT, abi.KERNEL_THREAD])
def test_split_matches_the_selected_arithmetic(bound, method, kernel):
    e = straddling(6000)
    tight = e.rtol < BOUND
    assert 0 < tight.sum() < e.n
    degpu.set_mixed_min_rtol(method, BOUND)
    split = run(e, method, abi.MIXED, kernel)
    degpu.set_mixed_min_rtol(method, 1.0)  # every instance below the bound: pair stages
    low = run(e, method, abi.MIXED, kernel)
    degpu.set_mixed_min_rtol(method, 0.0)
    mixed = run(e, method, abi.MIXED, kernel)
    same(split, low, tight)
    same(split, mixed, ~tight)
    # the FP32-stage form below the bound is what the split avoids: it needs more steps there
    steps = lambda r: (r.accepted + r.rejected)[tight].mean()
    assert steps(mixed) > steps(low)


def test_split_on_ragged_group_kernel(bound):
    f = W.config2(n=96)
    f.tf[:] = 4.0
    f.rtol = W.logU(8, np.arange(f.n), 1, 1e-10, 1e-6)
    f.atol = 1e-2 * f.rtol
    tight = f.rtol < BOUND
    assert 0 < tight.sum() < f.n
    degpu.set_mixed_min_rtol(abi.DOP853, BOUND)
    split = run(f, abi.DOP853, abi.MIXED, abi.KERNEL_WARP, rhs=abi.RHS["FPU_BETA"], dims=f.dims)
    degpu.set_mixed_min_rtol(abi.DOP853, 1.0)  # every chain in the tight class: pair stages
    pair = run(f, abi.DOP853, abi.MIXED, abi.KERNEL_WARP, rhs=abi.RHS["FPU_BETA"], dims=f.dims)
    degpu.set_mixed_min_rtol(abi.DOP853, 0.0)
    mixed = run(f, abi.DOP853, abi.MIXED, abi.KERNEL_WARP, rhs=abi.RHS["FPU_BETA"], dims=f.dims)
    same(split, pair, tight)
    same(split, mixed, ~tight)
    # the pair stages follow FP64 at the same tolerances
    fast = run(f, abi.DOP853, abi.FP64_FAST, abi.KERNEL_WARP, rhs=abi.RHS["FPU_BETA"], dims=f.dims)
    ok = (pair.status == abi.COMPLETE) & (fast.status == abi.COMPLETE)
    assert ok.all()
    rel = np.max(np.abs(pair.y_final - fast.y_final), axis=0) / np.max(np.abs(fast.y_final), axis=0)
    assert np.median(rel[tight]) < 1e-9


def test_rk4_has_no_bound(bound):
    assert degpu.mixed_min_rtol(abi.RK4) == 0.0
    with pytest.raises(degpu.DegpuError):
        degpu.set_mixed_min_rtol(abi.RK4, 1e-8)


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853, abi.RKF45])
@pytest.mark.parametrize("kernel", [abi.KERNEL_PERSISTENT, abi.KERNEL_THREAD])
def test_mixed_time_pair_ends_at_tf_and_tracks_fp64(method, kernel):
    """The mixed form keeps t (and the pendulum's drive phase) as an FP32 pair when no output times
    are requested. With t0 far from zero (the pair's low part carries the offset's FP32 rounding)
    every completed instance ends exactly at tf, and the final states stay as close to the FP64
    solve as they are with t0 = 0."""
    errs = []
    for shift in (0.0, 1000.3):
        e = W.config1(n=3000, first=777)
        e.rtol = np.maximum(e.rtol, 1e-8)
        e.atol = 1e-2 * e.rtol
        nonchaotic = e.family != abi.RHS["LORENZ"]
        e.t0 = e.t0 + shift
        e.tf = e.t0 + np.minimum(e.tf - (e.t0 - shift), 20.0)
        mixed = run(e, method, abi.MIXED, kernel)
        fast = run(e, method, abi.FP64_FAST, kernel)
        ok = mixed.status == abi.COMPLETE
        assert ok.mean() > 0.99
        assert np.array_equal(mixed.t_final[ok], e.tf[ok])
        sel = ok & nonchaotic & (fast.status == abi.COMPLETE)
        rel = np.max(np.abs(mixed.y_final[:, sel] - fast.y_final[:, sel]), axis=0) / \
            np.maximum(np.max(np.abs(fast.y_final[:, sel]), axis=0), 1e-300)
        errs.append(np.median(rel))
    assert errs[0] < 1e-4 and errs[1] < 1e-4
    assert errs[1] < 10 * errs[0] + 1e-6


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
@pytest.mark.parametrize("kernel", [abi.KERNEL_PERSISTENT, abi.KERNEL_THREAD])
def test_pair_stages_track_fp64(bound, kernel, method):
    """The FP32-pair stages (the tight class of a mixed solve) against FP64 at the same
    tolerances on the non-chaotic families (Van der Pol, the damped driven pendulum), over the
    ensemble's full horizons: the FP32 stages' error floor (about 5e-7) is gone."""
    e = W.config1(n=3 * 1500, first=20_000)
    keep = e.family != abi.RHS["LORENZ"]
    e = e.subset(np.nonzero(keep)[0])
    e.rtol = W.logU(9, np.arange(e.n), 1, 1e-10, 1e-7)
    e.atol = 1e-2 * e.rtol
    degpu.set_mixed_min_rtol(method, 1.0)
    pair = run(e, method, abi.MIXED, kernel)
    degpu.set_mixed_min_rtol(method, 0.0)
    f32 = run(e, method, abi.MIXED, kernel)
    fast = run(e, method, abi.FP64_FAST, kernel)
    ok = (pair.status == abi.COMPLETE) & (fast.status == abi.COMPLETE)
    # at rtol 1e-10 over horizons up to 50 a few Van der Pol instances end on the crate's
    # stiffness test or the step limit in either arithmetic; the pairs must not end more often
    assert ok.mean() > 0.99
    assert (pair.status == abi.COMPLETE).sum() >= (fast.status == abi.COMPLETE).sum() - 0.002 * e.n
    rel = lambda r: np.max(np.abs(r.y_final[:, ok] - fast.y_final[:, ok]), axis=0) / \
        np.maximum(np.max(np.abs(fast.y_final[:, ok]), axis=0), 1e-300)
    # the pair stages follow FP64 to the rounding-driven spread of the step sequence (wider for
    # DOP853, whose longer steps amplify a rounding-level difference more)
    assert np.median(rel(pair)) < (1e-9 if method == abi.DOPRI5 else 3e-9)
    assert np.median(rel(pair)) < 0.05 * np.median(rel(f32))
    # the step counts of FP64
    steps = lambda r: (r.accepted + r.rejected)[ok].astype(float)
    assert abs(steps(pair).mean() / steps(fast).mean() - 1.0) < 0.01


@pytest.mark.parametrize("method", [abi.DOPRI5, abi.DOP853])
@pytest.mark.parametrize("kernel", [abi.KERNEL_PERSISTENT, abi.KERNEL_THREAD])
def test_pair_dense_output_tracks_fp64(bound, method, kernel):
    """Output times through the pair stages' interpolants (the tight class with dense output):
    the interpolated states follow FP64 at the same tolerances, on both kernel layouts."""
    e = W.config1(n=3 * 600, first=41_000)
    e = e.subset(np.nonzero(e.family != abi.RHS["LORENZ"])[0])
    e.tf = np.minimum(e.tf, 10.0)
    e.rtol = W.logU(14, np.arange(e.n), 1, 1e-10, 1e-7)
    e.atol = 1e-2 * e.rtol
    te = np.linspace(10.0, 0.0, 21)
    pair = run(e, method, abi.MIXED, kernel, t_eval=te)
    fast = run(e, method, abi.FP64_FAST, kernel, t_eval=te)
    ok = (pair.status == abi.COMPLETE) & (fast.status == abi.COMPLETE)
    assert ok.mean() > 0.99
    a, b = pair.dense[:, :, ok], fast.dense[:, :, ok]
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    rel = np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), 1e-3)
    assert np.median(rel) < (1e-9 if method == abi.DOPRI5 else 3e-9)
