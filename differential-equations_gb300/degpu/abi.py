"""ctypes mirror of include/degpu.h (the C ABI of the GB300 ensemble ERK integrator).

The structs here are byte-for-byte the C structs; `load()` opens the in-tree libdegpu.so and
declares every exported entry point.  There is no fallback: if the shared library is missing
the import of the solver API raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_ROOT, "csrc", "libdegpu.so")
# measurement and device self-checks (FMA peak probe, conversion and controller-power checks),
# built beside libdegpu.so and used by the benchmark and the tests only
PROBE_PATH = os.path.join(PKG_ROOT, "csrc", "libdegpu_probe.so")

# degpu_status
OK, BAD_INPUT, OOM, TIMEOUT, CUDA_ERROR, UNSUPPORTED = range(6)
# degpu_method
RK4, DOPRI5, DOP853, RKF45, CASH_KARP = 0, 1, 2, 3, 4
RKV655E, RKV656E, RKV766E, RKV767E, RKV877E, RKV878E, RKV988E, RKV989E = range(5, 13)
# degpu_precision
FP64_PARITY, FP64_FAST, MIXED, FP64_PLAIN, MIXED_FP64_CTRL = 0, 1, 2, 3, 4
# degpu_kernel
KERNEL_AUTO, KERNEL_THREAD, KERNEL_WARP, KERNEL_PERSISTENT = 0, 1, 2, 3
# degpu_dense_mode
DENSE_REFERENCE, DENSE_HAIRER = 0, 1
# degpu_instance_status
COMPLETE, ERR_BAD_INPUT, ERR_MAX_STEPS, ERR_STEP_SIZE, ERR_STIFFNESS, INTERRUPTED, ERR_LINEAR_ALGEBRA = range(7)
# degpu_rhs_id
RHS = dict(
    LORENZ=1, VAN_DER_POL=2, PENDULUM=3, FPU_BETA=4, EXP_GROWTH=5, LINEAR=6, HARMONIC=7,
    LOGISTIC=8, ROBERTSON=9, HIRES=10, BRUSSELATOR=11, CR3BP=12, PIPE_HEAT=13, DAMPED_QUADRATURE=14,
)
RHS_NVRTC_BASE = 1000

DP = C.POINTER(C.c_double)
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)


class MethodCfg(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("precision", C.c_int32), ("kernel", C.c_int32), ("dense_mode", C.c_int32),
        ("h0", C.c_double), ("h_min", C.c_double), ("h_max", C.c_double), ("max_steps", C.c_int64),
        ("safety_factor", C.c_double), ("min_scale", C.c_double), ("max_scale", C.c_double),
    ]


class Problem(C.Structure):
    _fields_ = [("rhs_id", C.c_int32), ("dim", C.c_int32), ("n_params", C.c_int32), ("reserved", C.c_int32)]


class BatchIn(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("t0", DP), ("tf", DP), ("y0", DP), ("params", DP), ("rtol", DP), ("atol", DP),
        ("dims", I32P), ("family", I32P), ("t_eval", DP), ("n_eval", C.c_int32), ("reserved", C.c_int32),
        ("rtol_vec", DP), ("atol_vec", DP),
    ]


class BatchOut(C.Structure):
    _fields_ = [
        ("y_final", DP), ("t_final", DP), ("dense", DP), ("accepted", I64P), ("rejected", I64P),
        ("fevals", I64P), ("status", I32P),
    ]


class Crossing(C.Structure):
    _fields_ = [("component", C.c_int32), ("direction", C.c_int32), ("max_points", C.c_int32),
                ("reserved", C.c_int32), ("threshold", C.c_double)]


class CrossingOut(C.Structure):
    _fields_ = [("t", DP), ("y", DP), ("count", I32P)]


CROSS_BOTH, CROSS_POSITIVE, CROSS_NEGATIVE = 0, 1, -1
HYPERPLANE_MAX_DIM = 8


class Hyperplane(C.Structure):
    _fields_ = [("dim", C.c_int32), ("direction", C.c_int32), ("max_points", C.c_int32),
                ("reserved", C.c_int32), ("components", C.c_int32 * HYPERPLANE_MAX_DIM),
                ("point", C.c_double * HYPERPLANE_MAX_DIM), ("normal", C.c_double * HYPERPLANE_MAX_DIM)]


EVENT_MAX_TERMS = 8
EVENT_LINEAR, EVENT_MAX_ABS = 0, 1


class Event(C.Structure):
    _fields_ = [("kind", C.c_int32), ("direction", C.c_int32), ("terminate", C.c_int32),
                ("max_points", C.c_int32), ("n_terms", C.c_int32), ("reserved", C.c_int32),
                ("components", C.c_int32 * EVENT_MAX_TERMS), ("weights", C.c_double * EVENT_MAX_TERMS),
                ("t_weight", C.c_double), ("offset", C.c_double)]


def make_event(kind=EVENT_LINEAR, components=(), weights=None, t_weight=0.0, offset=0.0, direction=CROSS_BOTH,
               terminate=0, max_points=16) -> Event:
    """degpu_event: LINEAR g = ((sum_j weights[j] y[components[j]]) + t_weight t) + offset, or
    MAX_ABS g = max_j |y[components[j]]| + offset; `terminate` events stop the solve (0: never)."""
    m = len(components)
    if m > EVENT_MAX_TERMS or (weights is not None and len(weights) != m):
        raise ValueError("event: at most 8 terms, one weight per term")
    ev = Event(kind=kind, direction=direction, terminate=terminate, max_points=max_points, n_terms=m,
               t_weight=float(t_weight), offset=float(offset))
    for j in range(m):
        ev.components[j] = int(components[j])
        ev.weights[j] = 1.0 if weights is None else float(weights[j])
    return ev


BVP_SINGLE, BVP_MULTIPLE = 0, 1
BVP_MAX_UNKNOWNS = 64


class Bvp(C.Structure):
    _fields_ = [("method", C.c_int32), ("segments", C.c_int32), ("max_iterations", C.c_int32),
                ("reserved", C.c_int32), ("tolerance", C.c_double), ("side", C.c_int32 * HYPERPLANE_MAX_DIM),
                ("component", C.c_int32 * HYPERPLANE_MAX_DIM), ("value", C.c_double * HYPERPLANE_MAX_DIM)]


class BvpOut(C.Structure):
    _fields_ = [("y_a", DP), ("iterations", I32P), ("jacobian", I64P)]


def make_bvp(rows, method=BVP_SINGLE, segments=4, max_iterations=100, tolerance=1e-6) -> Bvp:
    """degpu_bvp from residual rows (side, component, value): r_i = y_side[component] - value,
    side 0 = y(t0), 1 = y(tf); the crate's shooting defaults (100 iterations, tolerance 1e-6,
    4 segments)."""
    if not 1 <= len(rows) <= HYPERPLANE_MAX_DIM:
        raise ValueError("bvp: one residual row per state component (at most 8)")
    b = Bvp(method=method, segments=segments, max_iterations=max_iterations, tolerance=tolerance)
    for i, (side, comp, value) in enumerate(rows):
        b.side[i], b.component[i], b.value[i] = int(side), int(comp), float(value)
    return b


def make_hyperplane(components, point, normal, direction=CROSS_BOTH, max_points=16) -> Hyperplane:
    """degpu_hyperplane from sequences: pos[j] = y[components[j]], plane through `point` with
    `normal` (scaled to unit length by the library)."""
    m = len(components)
    if not (1 <= m <= HYPERPLANE_MAX_DIM) or len(point) != m or len(normal) != m:
        raise ValueError("hyperplane: 1..8 components, with a point and a normal of the same length")
    hp = Hyperplane(dim=m, direction=direction, max_points=max_points)
    for j in range(m):
        hp.components[j] = int(components[j])
        hp.point[j] = float(point[j])
        hp.normal[j] = float(normal[j])
    return hp


class GrayScott(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("dx", C.c_double), ("Du", C.c_double),
                ("Dv", C.c_double), ("F", C.c_double), ("k", C.c_double)]


# degpu_mol: the general method-of-lines problem
PDE_DIFFUSION, PDE_COUPLED_DIFFUSION, PDE_GRAY_SCOTT = 1, 2, 3
BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2
MOL_MAX_FIELDS, MOL_MAX_PARAMS = 4, 8


class Mol(C.Structure):
    _fields_ = [("pde_id", C.c_int32), ("dims", C.c_int32), ("fields", C.c_int32), ("reserved", C.c_int32),
                ("nodes", C.c_int32 * 2), ("lower", C.c_double * 2), ("dx", C.c_double * 2),
                ("bc_kind", (C.c_int32 * 2) * 2), ("bc_value", ((C.c_double * MOL_MAX_FIELDS) * 2) * 2),
                ("params", C.c_double * MOL_MAX_PARAMS)]


def make_mol(pde_id, nodes, lower, dx, faces, params, fields):
    """A degpu_mol: `faces` is [(lower kind, lower values), (upper kind, upper values)] per axis
    (values: one per field, the Dirichlet value or Neumann gradient)."""
    m = Mol(pde_id=pde_id, dims=len(nodes), fields=fields)
    for a, nd in enumerate(nodes):
        m.nodes[a] = nd
        m.lower[a] = lower[a]
        m.dx[a] = dx[a]
        for side, (kind, vals) in enumerate(faces[a]):
            m.bc_kind[a][side] = kind
            for c, v in enumerate(vals or []):
                m.bc_value[a][side][c] = v
    for q, v in enumerate(params):
        m.params[q] = v
    return m


class ServerCfg(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_uint64), ("max_active", C.c_int32), ("round_budget", C.c_int32)]


def default_cfg(method: int) -> MethodCfg:
    """The crate's defaults (src/methods/erk/mod.rs:112-159)."""
    return MethodCfg(method=method, precision=FP64_PARITY, kernel=KERNEL_AUTO, dense_mode=DENSE_REFERENCE,
                     h0=0.0, h_min=0.0, h_max=float("inf"), max_steps=10_000, safety_factor=0.9,
                     min_scale=0.2, max_scale=10.0)


_lib = None

# name -> (restype, argtypes) for every symbol include/degpu.h declares
SIGNATURES = {
    "degpu_default_cfg": (None, [C.POINTER(MethodCfg), C.c_int32]),
    "degpu_rhs_info": (C.c_int, [C.c_int32, I32P, I32P]),
    "degpu_set_mixed_min_rtol": (C.c_int, [C.c_int32, C.c_double]),
    "degpu_mixed_min_rtol": (C.c_double, [C.c_int32]),
    "degpu_solve_ensemble": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                       C.POINTER(BatchOut), C.c_void_p]),
    "degpu_solve_ensemble_host": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                            C.POINTER(BatchOut)]),
    "degpu_solve_ensemble_noalloc": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                               C.POINTER(BatchOut), C.c_void_p]),
    "degpu_solve_ensemble_crossing": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                                C.POINTER(Crossing), C.POINTER(BatchOut), C.POINTER(CrossingOut),
                                                C.c_void_p]),
    "degpu_solve_ensemble_crossing_host": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                                     C.POINTER(Crossing), C.POINTER(BatchOut), C.POINTER(CrossingOut)]),
    "degpu_solve_ensemble_hyperplane": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                                  C.POINTER(Hyperplane), C.POINTER(BatchOut),
                                                  C.POINTER(CrossingOut), C.c_void_p]),
    "degpu_solve_ensemble_hyperplane_host": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg),
                                                       C.POINTER(BatchIn), C.POINTER(Hyperplane),
                                                       C.POINTER(BatchOut), C.POINTER(CrossingOut)]),
    "degpu_solve_ensemble_event": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                             C.POINTER(Event), C.POINTER(BatchOut), C.POINTER(CrossingOut),
                                             C.c_void_p]),
    "degpu_solve_ensemble_event_host": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                                  C.POINTER(Event), C.POINTER(BatchOut), C.POINTER(CrossingOut)]),
    "degpu_solve_bvp_host": (C.c_int, [C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn), C.POINTER(Bvp),
                                       C.POINTER(BatchOut), C.POINTER(BvpOut)]),
    "degpu_eval_rhs": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_int32, C.c_int32, DP, DP, DP, DP,
                                 C.c_void_p]),
    "degpu_register_rhs_nvrtc": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, I32P, C.c_char_p,
                                           C.c_size_t]),
    "degpu_gray_scott_rk4": (C.c_int, [C.POINTER(GrayScott), C.c_int32, C.c_double, C.c_double, C.c_int64,
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
    "degpu_gray_scott_rhs": (C.c_int, [C.POINTER(GrayScott), DP, DP, DP, DP, C.c_void_p]),
    "degpu_mol_rhs": (C.c_int, [C.POINTER(Mol), C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    "degpu_mol_rk4": (C.c_int, [C.POINTER(Mol), C.c_int32, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                C.POINTER(C.c_int64), C.c_void_p]),
    "degpu_server_create": (C.c_int, [C.POINTER(ServerCfg), C.POINTER(C.c_void_p)]),
    "degpu_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(MethodCfg), C.POINTER(BatchIn),
                                      C.POINTER(BatchOut), C.POINTER(C.c_uint64)]),
    "degpu_server_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "degpu_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]),
    "degpu_server_destroy": (C.c_int, [C.c_void_p]),
    "degpu_status_string": (C.c_char_p, [C.c_int]),
    "degpu_version": (C.c_char_p, []),
}


def load(path: str = LIB_PATH):
    """Open libdegpu.so and declare its entry points.  Raises if it is not built."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libdegpu.so is not built ({path}); run __graft_entry__.build()")
    # group-kernel layouts chosen by the autotuner (degpu/autotune.py), read at the first ragged solve
    tuned = os.path.join(_HERE, "group_tune.txt")
    if os.path.exists(tuned):
        os.environ.setdefault("DEGPU_TUNE_FILE", tuned)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


_probe = None


def load_probe():
    """Open libdegpu_probe.so (the benchmark's FMA peak probe and the tests' device checks)."""
    global _probe
    if _probe is not None:
        return _probe
    if not os.path.exists(PROBE_PATH):
        raise RuntimeError(f"libdegpu_probe.so is not built ({PROBE_PATH}); run __graft_entry__.build()")
    lib = C.CDLL(PROBE_PATH)
    lib.degpu_internal_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    lib.degpu_internal_fma_peak.restype = C.c_int
    lib.degpu_internal_conv_check.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.degpu_internal_conv_check.restype = C.c_int
    lib.degpu_internal_pow_ctrl_neg_check.argtypes = [C.c_int64, C.c_void_p, C.c_double, C.c_void_p]
    lib.degpu_internal_pow_ctrl_neg_check.restype = C.c_int
    _probe = lib
    return lib


def ptr(arr, ctype=C.c_double):
    """ctypes pointer to a numpy array's data or a torch tensor's data_ptr (None -> NULL)."""
    if arr is None:
        return None
    if hasattr(arr, "data_ptr"):
        return C.cast(C.c_void_p(arr.data_ptr()), C.POINTER(ctype))
    return arr.ctypes.data_as(C.POINTER(ctype))
