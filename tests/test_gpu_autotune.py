"""Group-kernel layouts: every candidate (lanes per system, components per lane) gives bitwise the
same parity results, and the autotuner's choices are valid layouts for their buckets."""
import ctypes as C

import numpy as np
import pytest

import degpu
from degpu import abi, autotune, workloads as W

pytestmark = pytest.mark.gpu


def solve(e, prec=abi.FP64_PARITY):
    m = degpu.ExplicitRungeKutta(abi.DOP853)
    m.cfg.precision, m.cfg.max_steps = prec, 10_000_000
    return degpu.solve_ensemble(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m,
                                t_eval=np.linspace(0, 4, 5), dims=e.dims, n_params=1)


def test_layouts_give_identical_parity_results():
    lib = abi.load()
    pool = W.config2(n=4000)
    sel = np.nonzero((pool.dims > 32) & (pool.dims <= 64))[0][:64]
    e = pool.subset(sel)
    e.tf[:] = 4.0
    results = []
    for g, cpl in autotune.CANDIDATES[64]:
        autotune._set(lib, abi.DOP853, abi.FP64_PARITY, 1, 64, g, cpl)
        results.append(solve(e))
    autotune._set(lib, abi.DOP853, abi.FP64_PARITY, 1, 64, 32, 2)  # back to the default
    a, b = results
    assert np.array_equal(a.accepted, b.accepted) and np.array_equal(a.y_final, b.y_final)
    assert np.array_equal(a.dense, b.dense, equal_nan=True)


def test_autotune_choices_are_valid():
    ch = autotune.tune(abi.DOP853, abi.FP64_FAST, dense=False, per_bucket=64, horizon=2.0, reps=1)
    for c in ch:
        assert (c["g"], c["cpl"]) in autotune.CANDIDATES[c["dmax"]]
        assert c["g"] * c["cpl"] >= c["dmax"]
