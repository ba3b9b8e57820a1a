"""degpu_solve_ensemble_noalloc against degpu_solve_ensemble.

The no-allocation entry point serves callers that must not allocate device memory while they
run, e.g. an application that has reserved the device memory pool for itself, or a loop whose
step cannot absorb an allocator call that may synchronise the device.  It must give the same
results as the ordinary entry point.  Two calls run back to back, the second on a different,
smaller batch, because the fixed work-list array keeps the previous call's contents.

CUDA loads the library's device code lazily, so the first call on a device loads the fixed array
there; a caller makes that call before it reserves its memory pool.  After it, a call must leave
the device's free memory and the default memory pool's high-water marks where they were.
"""
import ctypes as C
import ctypes.util

import numpy as np
import pytest

from degpu import abi, workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # same bar as the parity tests


def device_batch(torch, e, dev):
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ins = dict(t0=T(e.t0), tf=T(e.tf), y0=T(e.y0), params=T(e.params), rtol=T(e.rtol), atol=T(e.atol),
               family=T(e.family, torch.int32))
    bi = abi.BatchIn(n=e.n, t0=abi.ptr(ins["t0"]), tf=abi.ptr(ins["tf"]), y0=abi.ptr(ins["y0"]),
                     params=abi.ptr(ins["params"]), rtol=abi.ptr(ins["rtol"]), atol=abi.ptr(ins["atol"]),
                     family=abi.ptr(ins["family"], C.c_int32), n_eval=0)
    return ins, bi


def device_outputs(torch, n, dev):
    o = dict(y_final=torch.full((3, n), float("nan"), dtype=torch.float64, device=dev),
             t_final=torch.empty(n, dtype=torch.float64, device=dev),
             accepted=torch.empty(n, dtype=torch.int64, device=dev),
             rejected=torch.empty(n, dtype=torch.int64, device=dev),
             fevals=torch.empty(n, dtype=torch.int64, device=dev),
             status=torch.full((n,), -1, dtype=torch.int32, device=dev))
    bo = abi.BatchOut(y_final=abi.ptr(o["y_final"]), t_final=abi.ptr(o["t_final"]),
                      accepted=abi.ptr(o["accepted"], C.c_int64), rejected=abi.ptr(o["rejected"], C.c_int64),
                      fevals=abi.ptr(o["fevals"], C.c_int64), status=abi.ptr(o["status"], C.c_int32))
    return o, bo


def solve_both(torch, lib, e, precision, stream):
    dev = torch.device("cuda:0")
    cfg = abi.default_cfg(abi.DOPRI5)
    cfg.precision, cfg.kernel, cfg.max_steps = precision, abi.KERNEL_PERSISTENT, 10_000_000
    prob = abi.Problem(rhs_id=0, dim=3, n_params=3)
    ins, bi = device_batch(torch, e, dev)
    ref, bo_ref = device_outputs(torch, e.n, dev)
    got, bo_got = device_outputs(torch, e.n, dev)
    h = C.c_void_p(stream.cuda_stream)
    assert lib.degpu_solve_ensemble(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo_ref), h) == abi.OK
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo_got), h) == abi.OK
    stream.synchronize()
    return {k: v.cpu().numpy() for k, v in ref.items()}, {k: v.cpu().numpy() for k, v in got.items()}


def assert_same(ref, got):
    for k in ("status", "accepted", "rejected", "fevals"):
        assert np.array_equal(ref[k], got[k]), k
    scale = np.maximum(np.abs(ref["y_final"]), 1e-300)
    assert np.max(np.abs(got["y_final"] - ref["y_final"]) / scale) <= REL_TOL
    assert np.array_equal(ref["t_final"], got["t_final"])


@pytest.mark.parametrize("precision", [abi.FP64_PARITY, abi.MIXED])
def test_noalloc_matches_ordinary_entry_point_twice(precision):
    torch = pytest.importorskip("torch")
    lib = abi.load()
    stream = torch.cuda.Stream()
    first = W.config1(n=3 * 2000)
    first.tf = np.minimum(first.tf, 8.0)
    second = W.config1(n=3 * 500, first=50_000)  # different and smaller: stale lists must not leak
    second.tf = np.minimum(second.tf, 8.0)
    for e in (first, second):
        ref, got = solve_both(torch, lib, e, precision, stream)
        assert np.all(ref["status"] == abi.COMPLETE)
        assert_same(ref, got)


def test_noalloc_mixed_split_matches_ordinary_entry_point():
    """A mixed batch whose rtol values straddle the mixed-precision bound: the tight part (FP32-pair
    stages) and the FP32-stage part of the work lists both come from the fixed array."""
    torch = pytest.importorskip("torch")
    lib = abi.load()
    stream = torch.cuda.Stream()
    e = W.config1(n=3 * 1000, first=70_000)
    e.tf = np.minimum(e.tf, 8.0)
    e.rtol = W.logU(7, np.arange(e.n), 1, 1e-9, 1e-5)
    e.atol = 1e-2 * e.rtol
    bound = lib.degpu_mixed_min_rtol(abi.DOPRI5)
    assert 0 < (e.rtol < bound).sum() < e.n
    ref, got = solve_both(torch, lib, e, abi.MIXED, stream)
    assert_same(ref, got)


def test_noalloc_rejects_batches_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    lib = abi.load()
    e = W.config1(n=30)
    dev = torch.device("cuda:0")
    ins, bi = device_batch(torch, e, dev)
    out, bo = device_outputs(torch, e.n, dev)
    bi.n = abi_max = 262144 + 1  # DEGPU_NOALLOC_MAX_INSTANCES + 1: refused before anything runs
    cfg = abi.default_cfg(abi.DOPRI5)
    prob = abi.Problem(rhs_id=0, dim=3, n_params=3)
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), None) == \
        abi.BAD_INPUT
    assert abi_max > 262144


def cudart():
    """The CUDA runtime library, for the default memory pool's attributes."""
    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.skip("libcudart not found")


POOL_RESERVED_HIGH, POOL_USED_CURRENT, POOL_USED_HIGH = 0x6, 0x7, 0x8  # cudaMemPoolAttr


def pool_attr(rt, pool, attr):
    v = C.c_uint64(0)
    assert rt.cudaMemPoolGetAttribute(pool, C.c_int(attr), C.byref(v)) == 0
    return v.value


def test_noalloc_call_allocates_nothing_after_the_first():
    torch = pytest.importorskip("torch")
    lib = abi.load()
    rt = cudart()
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream()
    e = W.config1(n=3 * 1000, first=90_000)
    e.tf = np.minimum(e.tf, 8.0)
    cfg = abi.default_cfg(abi.DOPRI5)
    cfg.precision, cfg.kernel, cfg.max_steps = abi.MIXED, abi.KERNEL_PERSISTENT, 10_000_000
    prob = abi.Problem(rhs_id=0, dim=3, n_params=3)
    ins, bi = device_batch(torch, e, dev)
    out, bo = device_outputs(torch, e.n, dev)
    h = C.c_void_p(stream.cuda_stream)
    # the first call on the device loads the array (lazy module loading)
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), h) == abi.OK
    stream.synchronize()
    torch.cuda.synchronize()
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), C.c_int(0)) == 0
    zero = C.c_uint64(0)
    for attr in (POOL_RESERVED_HIGH, POOL_USED_HIGH):
        assert rt.cudaMemPoolSetAttribute(pool, C.c_int(attr), C.byref(zero)) == 0
    used_before = pool_attr(rt, pool, POOL_USED_CURRENT)
    free_before = torch.cuda.mem_get_info(0)[0]
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), h) == abi.OK
    stream.synchronize()
    free_after = torch.cuda.mem_get_info(0)[0]
    assert free_after == free_before
    assert pool_attr(rt, pool, POOL_USED_HIGH) <= used_before
    assert np.all(out["status"].cpu().numpy() == abi.COMPLETE)


def test_noalloc_unsupported_family_in_the_map():
    """An instance whose family is not Van der Pol, pendulum or Lorenz gets BadInput and a NaN
    final state; the others are solved as the ordinary entry point solves them.  Without a status
    array such a batch is refused as a whole."""
    torch = pytest.importorskip("torch")
    lib = abi.load()
    stream = torch.cuda.Stream()
    e = W.config1(n=3 * 100, first=120_000)
    e.tf = np.minimum(e.tf, 6.0)
    e.family = e.family.copy()
    e.family[::7] = abi.RHS["HARMONIC"]
    dev = torch.device("cuda:0")
    cfg = abi.default_cfg(abi.DOPRI5)
    cfg.precision, cfg.kernel, cfg.max_steps = abi.FP64_PARITY, abi.KERNEL_PERSISTENT, 10_000_000
    prob = abi.Problem(rhs_id=0, dim=3, n_params=3)
    ins, bi = device_batch(torch, e, dev)
    got, bo = device_outputs(torch, e.n, dev)
    h = C.c_void_p(stream.cuda_stream)
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), h) == abi.OK
    stream.synchronize()
    g = {k: v.cpu().numpy() for k, v in got.items()}
    bad = e.family == abi.RHS["HARMONIC"]
    assert np.all(g["status"][bad] == abi.ERR_BAD_INPUT)
    assert np.all(np.isnan(g["y_final"][:, bad])) and np.all(np.isnan(g["t_final"][bad]))
    good = np.nonzero(~bad)[0]
    ref, got2 = solve_both(torch, lib, e.subset(good), abi.FP64_PARITY, stream)
    for k in ("status", "accepted", "rejected", "fevals"):
        assert np.array_equal(g[k][good], ref[k]), k
    assert np.array_equal(g["y_final"][:, good], ref["y_final"])
    bo.status = None
    assert lib.degpu_solve_ensemble_noalloc(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), h) == \
        abi.BAD_INPUT
