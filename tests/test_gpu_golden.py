"""The FP64 parity path against the frozen oracle fixtures of tests/golden: bit for bit, on the
run-to-completion and persistent kernels, independent of the oracle built on this machine."""
import os

import numpy as np
import pytest

import degpu
from degpu import abi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.mark.parametrize("kernel", [abi.KERNEL_THREAD, abi.KERNEL_PERSISTENT])
@pytest.mark.parametrize("name", ["uneven_dopri5_1500", "uneven_dop853_dense_600"])
def test_parity_path_matches_golden(name, kernel):
    f = load(name)
    m = degpu.ExplicitRungeKutta(int(f["method"]))
    m.cfg.precision, m.cfg.kernel, m.cfg.max_steps = abi.FP64_PARITY, kernel, 10_000_000
    te = f.get("t_eval")
    g = degpu.solve_ensemble(0, f["y0"].shape[0], f["t0"], f["tf"], f["y0"], f["params"], f["rtol"], f["atol"], m,
                             family=f["family"], t_eval=te, n_params=f["params"].shape[0])
    assert np.array_equal(g.status, f["status"])
    assert np.array_equal(g.accepted, f["accepted"]) and np.array_equal(g.rejected, f["rejected"])
    assert np.array_equal(g.fevals, f["fevals"])
    assert np.array_equal(g.y_final, f["y_final"])
    assert np.array_equal(g.t_final, f["t_final"])
    if te is not None:
        assert np.array_equal(g.dense, f["dense"], equal_nan=True)
