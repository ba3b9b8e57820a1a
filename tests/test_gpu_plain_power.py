"""The plain FP64 form's controller power x^(-0.2) and x^(-0.125) (pow_ctrl_neg in dd_math.cuh),
evaluated on the device as the plain form compiles it (FMA contraction on, CUDA's FP32 log2f and
exp2f in its starting value), against the oracle's binary128 evaluation rounded once: equal on
every input.  The power decides each step's size, so the plain form's accepted and rejected steps
follow the crate's only if this value is the correctly rounded one."""
import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("y", [-0.2, -0.125])
def test_plain_controller_power_correctly_rounded_on_device(y):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    n = 1 << 21
    x = np.exp(rng.uniform(np.log(2.0 ** -800), np.log(2.0 ** 800), n))
    x[: n // 2] = np.exp(rng.uniform(-40.0, 40.0, n // 2))     # error norms an integrator produces
    x[:4000] = 2.0 ** rng.integers(-790, 790, 4000)             # powers of two
    x[4000:8000] = 1.0 + rng.uniform(-1e-9, 1e-9, 4000)         # ln x near 0
    x[8000:12000] = np.nextafter(2.0 ** (40 * rng.integers(-19, 19, 4000)).astype(float), 0.0)
    x[12000:16000] = 2.0 ** rng.uniform(-800.0, -799.0, 4000)   # the ends of the direct range
    x[16000:20000] = 2.0 ** rng.uniform(799.0, 800.0, 4000)
    x[20000:20006] = [1e-300, 1e300, 0.0, np.inf, 1.0, 5e-324]  # handed to the general power
    dev = torch.device("cuda:0")
    tx = torch.as_tensor(x, device=dev)
    out = torch.empty_like(tx)
    assert abi.load_probe().degpu_internal_pow_ctrl_neg_check(n, tx.data_ptr(), y, out.data_ptr()) == 0
    got = out.cpu().numpy()
    ref = np.empty(n)
    O.lib().oracle_cr_pow_batch(O.p(x), O.p(np.full(n, y)), O.p(ref), n)
    bad = np.nonzero(~((got == ref) | (np.isnan(got) & np.isnan(ref))))[0]
    assert bad.size == 0, (bad.size, x[bad[:4]], got[bad[:4]], ref[bad[:4]])
