"""CPU checks of the boundary: the C-ABI library loads and exports every function
include/degpu.h declares, and the host-side argument validation answers without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from degpu import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(REPO, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(degpu_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "degpu_solve_ensemble" in names and "degpu_solve_ensemble_host" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(abi.SIGNATURES)


def test_probe_library_is_separate_from_the_integrator():
    """The FMA peak probe and the device self-checks live in libdegpu_probe.so, which the benchmark
    and the tests load; the integrator library exports none of them."""
    probe = abi.load_probe()
    for name in ("degpu_internal_fma_peak", "degpu_internal_conv_check", "degpu_internal_pow_ctrl_neg_check"):
        assert hasattr(probe, name), name
        assert not hasattr(abi.load(), name), name


def test_rust_binding_declares_every_entry_point_and_struct():
    """The Rust sys crate a maintainer would add to the crate binds every function and struct of
    the header (it cannot be compiled here: no Rust toolchain)."""
    rs = open(os.path.join(REPO, "differential-equations_gb300", "rust", "degpu-sys", "src", "lib.rs")).read()
    bound = set(re.findall(r"pub fn (degpu_[a-z_0-9]+)\(", rs))
    assert set(declared_functions()) <= bound, sorted(set(declared_functions()) - bound)
    src = open(os.path.join(REPO, "include", "degpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    structs = set(re.findall(r"typedef struct\s*\{[^{}]*\}\s*(degpu_[a-z_0-9]+)\s*;", src))
    structs |= set(re.findall(r"typedef struct (degpu_[a-z_0-9]+) degpu_[a-z_0-9]+;", src))
    assert {"degpu_batch_in", "degpu_event", "degpu_bvp", "degpu_server"} <= structs
    rs_structs = set(re.findall(r"pub struct (degpu_[a-z_0-9]+)", rs))
    assert structs <= rs_structs, sorted(structs - rs_structs)
    # the field counts of the structs that cross the boundary by value agree with ctypes
    for name, cls in [("degpu_crossing", abi.Crossing), ("degpu_hyperplane", abi.Hyperplane),
                      ("degpu_event", abi.Event), ("degpu_bvp", abi.Bvp), ("degpu_method_cfg", abi.MethodCfg)]:
        body = re.search(r"pub struct %s \{(.*?)\}" % name, rs, flags=re.S).group(1)
        assert len(re.findall(r"pub \w+:", body)) == len(cls._fields_), name


def test_defaults_match_crate():
    lib = abi.load()
    cfg = abi.MethodCfg()
    lib.degpu_default_cfg(C.byref(cfg), abi.DOPRI5)
    # src/methods/erk/mod.rs:112-159
    assert cfg.h0 == 0.0 and cfg.h_min == 0.0 and np.isinf(cfg.h_max)
    assert cfg.max_steps == 10_000 and cfg.safety_factor == 0.9
    assert cfg.min_scale == 0.2 and cfg.max_scale == 10.0


def test_rhs_info():
    lib = abi.load()
    d, p = C.c_int32(), C.c_int32()
    assert lib.degpu_rhs_info(abi.RHS["LORENZ"], C.byref(d), C.byref(p)) == abi.OK
    assert (d.value, p.value) == (3, 3)
    assert lib.degpu_rhs_info(999, C.byref(d), C.byref(p)) == abi.BAD_INPUT


def test_bad_input_rejected_before_any_launch():
    lib = abi.load()
    cfg = abi.default_cfg(abi.DOPRI5)
    prob = abi.Problem(rhs_id=abi.RHS["LORENZ"], dim=3, n_params=3)
    bi = abi.BatchIn(n=4)  # null arrays
    bo = abi.BatchOut()
    assert lib.degpu_solve_ensemble(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo), None) == abi.BAD_INPUT
    assert lib.degpu_solve_ensemble(None, C.byref(cfg), C.byref(bi), C.byref(bo), None) == abi.BAD_INPUT
    cfg.method = 7
    assert lib.degpu_solve_ensemble_host(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo)) == abi.BAD_INPUT
    # an empty batch is a successful no-op
    cfg = abi.default_cfg(abi.DOPRI5)
    assert lib.degpu_solve_ensemble(C.byref(prob), C.byref(cfg), C.byref(abi.BatchIn(n=0)), C.byref(bo),
                                    None) == abi.OK
    assert lib.degpu_status_string(abi.BAD_INPUT) == b"bad input"


def test_mixed_min_rtol_setting():
    lib = abi.load()
    old5, old8 = lib.degpu_mixed_min_rtol(abi.DOPRI5), lib.degpu_mixed_min_rtol(abi.DOP853)
    assert old5 >= 0.0 and old8 >= 0.0
    assert lib.degpu_mixed_min_rtol(abi.RK4) == 0.0  # fixed step: no bound
    try:
        assert lib.degpu_set_mixed_min_rtol(abi.DOP853, 3e-9) == abi.OK
        assert lib.degpu_mixed_min_rtol(abi.DOP853) == 3e-9
        assert lib.degpu_mixed_min_rtol(abi.DOPRI5) == old5
        assert lib.degpu_set_mixed_min_rtol(abi.DOPRI5, 0.0) == abi.OK  # split off
        assert lib.degpu_set_mixed_min_rtol(abi.RK4, 1e-9) == abi.BAD_INPUT
        assert lib.degpu_set_mixed_min_rtol(9, 1e-9) == abi.BAD_INPUT
        assert lib.degpu_set_mixed_min_rtol(abi.DOPRI5, -1.0) == abi.BAD_INPUT
        assert lib.degpu_set_mixed_min_rtol(abi.DOPRI5, float("nan")) == abi.BAD_INPUT
    finally:
        lib.degpu_set_mixed_min_rtol(abi.DOPRI5, old5)
        lib.degpu_set_mixed_min_rtol(abi.DOP853, old8)
