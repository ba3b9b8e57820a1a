"""The crate's printed step counters (docs/ode.md:66-123) on the device.

DOP853 at rtol = atol = 1e-12 on logistic growth (k = 1, m = 10, y(0) = 1) over [0, 10], output
every 1.0 and the terminal event y - 0.9 m in the positive direction.  The crate prints 325
function evaluations, 20 accepted and 2 rejected steps, the states (1, 2.3197), (2, 4.5085),
(3, 6.9057), (4, 8.5849) and the event at (4.3944, 9.0000).  The FP64 parity path reproduces
them through degpu_solve_ensemble_event, bit for bit equal to the oracle; the FP64 fast path
(FMA contraction) reproduces the counters and the printed digits."""
import numpy as np
import pytest

import oracle_lib as O
from degpu import abi, workloads as W
from test_gpu_event import gpu_event

pytestmark = pytest.mark.gpu

DOC_STATES = [1.0000, 2.3197, 4.5085, 6.9057, 8.5849]


def logistic(n=32):
    return W.Ensemble("logistic", abi.DOP853, n, 1, 2, np.zeros(n), np.full(n, 10.0), np.ones((1, n)),
                      np.array([[1.0], [10.0]]).repeat(n, axis=1), np.full(n, 1e-12), np.full(n, 1e-12),
                      rhs_id=abi.RHS["LOGISTIC"])


@pytest.mark.parametrize("precision", [abi.FP64_PARITY, abi.FP64_FAST])
def test_docs_ode_md_counters_on_device(precision):
    e = logistic()
    te = np.arange(0.0, 10.5, 1.0)
    cfg = abi.default_cfg(abi.DOP853)
    cfg.precision = precision
    ev = abi.make_event(abi.EVENT_LINEAR, [0], [1.0], offset=-9.0, direction=abi.CROSS_POSITIVE, terminate=1)
    g = gpu_event(e, cfg, ev, t_eval=te)
    assert np.all(g["status"] == abi.INTERRUPTED)
    assert np.all(g["fevals"] == 325) and np.all(g["accepted"] == 20) and np.all(g["rejected"] == 2)
    for i in range(e.n):
        np.testing.assert_array_equal(np.round(g["dense"][:5, 0, i], 4), DOC_STATES)
        assert np.all(np.isnan(g["dense"][5:, 0, i]))
    assert np.all(g["cross_count"] == 1)
    assert np.all(np.round(g["cross_t"][0], 4) == 4.3944) and np.all(np.round(g["cross_y"][0, 0], 4) == 9.0)
    if precision == abi.FP64_PARITY:
        b = O.Batch(e.rhs_id, 1, 2, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, t_eval=te)
        o = O.solve_event(b, cfg, ev)
        for k in ("status", "fevals", "accepted", "rejected", "cross_count", "y_final", "t_final"):
            assert np.array_equal(g[k], o[k]), k
        assert np.array_equal(g["dense"], o["dense"], equal_nan=True)
        assert np.array_equal(g["cross_t"][:1], o["cross_t"][:1]) and np.array_equal(g["cross_y"][:1], o["cross_y"][:1])
