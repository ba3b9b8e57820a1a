"""Integer-op FP32<->FP64 conversions of the mixed form's per-step bookkeeping, checked on the
device against numpy: widening is exact; narrowing rounds toward zero."""

import numpy as np
import pytest

from degpu import abi

pytestmark = pytest.mark.gpu


def test_widen_exact_and_narrow_toward_zero():
    torch = pytest.importorskip("torch")
    fn = abi.load_probe().degpu_internal_conv_check
    rng = np.random.default_rng(3)
    n = 1 << 20
    f = (rng.standard_normal(n) * 10.0 ** rng.integers(-37, 38, n)).astype(np.float32)
    f[:6] = [0.0, -0.0, np.inf, -np.inf, np.float32(1.1754944e-38), np.float32(-3.4028235e38)]
    d = rng.standard_normal(n) * 10.0 ** rng.integers(-40, 40, n)
    d[:8] = [0.0, -0.0, 1e-300, -1e300, np.inf, 1.0, np.nextafter(1.0, 2.0), -np.nextafter(1.0, 2.0)]
    dev = torch.device("cuda:0")
    tf = torch.as_tensor(f, device=dev)
    td = torch.as_tensor(d, device=dev)
    wide = torch.empty(n, dtype=torch.float64, device=dev)
    narrow = torch.empty(n, dtype=torch.float32, device=dev)
    assert fn(n, tf.data_ptr(), wide.data_ptr(), td.data_ptr(), narrow.data_ptr()) == 0
    w = wide.cpu().numpy()
    sub = (f != 0) & (np.abs(f) < np.finfo(np.float32).tiny)  # subnormal inputs become signed zero
    assert sub.any()
    assert np.array_equal(w[~sub], f[~sub].astype(np.float64))
    assert np.all(w[sub] == 0.0)
    assert np.array_equal(np.signbit(w), np.signbit(f))
    nr = narrow.cpu().numpy()
    a = np.abs(d)
    fin = np.isfinite(a) & (a >= np.finfo(np.float32).tiny) & (a <= np.finfo(np.float32).max)
    # |narrow| <= |d| < next float32 above |narrow|
    assert np.all(np.abs(nr[fin]).astype(np.float64) <= a[fin])
    up = np.nextafter(np.abs(nr[fin]), np.float32(np.inf)).astype(np.float64)
    assert np.all(up > a[fin])
    assert np.array_equal(np.signbit(nr), np.signbit(d))
    small = a < np.finfo(np.float32).tiny
    assert np.all(nr[small] == 0.0)
    big = a > np.finfo(np.float32).max
    assert np.all(np.isinf(nr[big]))
