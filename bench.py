"""Benchmark: IVP solves/sec on the 1,048,576-instance uneven ensemble (Van der Pol / damped
driven pendulum / Lorenz, t_end ~ U[5,50], rtol ~ logU[1e-9,1e-5], atol = 1e-2 rtol, DOPRI5)
on one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--variant V] [--impl ours|reference]

A step is one ensemble solve of the whole batch.  `value` is solves/s with inputs resident in
HBM (degpu_solve_ensemble on device pointers, CUDA events on the launch stream); `e2e` is the
same metric through degpu_solve_ensemble_host with pinned host buffers (host<->device copies
inside the timed region).  The CPU baseline is the oracle (a C++ restatement of the crate's
solver, the crate itself cannot be built here) on a bounded sample with all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "differential-equations_gb300"))

from degpu import abi, workloads as W  # noqa: E402

VARIANTS = {
    # name: (precision, kernel)
    "mixed-persistent": (abi.MIXED, abi.KERNEL_PERSISTENT),
    "fp64-persistent": (abi.FP64_PARITY, abi.KERNEL_PERSISTENT),
    "fp64-plain": (abi.FP64_PARITY, abi.KERNEL_THREAD),
    "fp64fast-persistent": (abi.FP64_FAST, abi.KERNEL_PERSISTENT),
    "mixed-thread": (abi.MIXED, abi.KERNEL_THREAD),
}

# Algorithmic FP operations of one attempted DOPRI5 step of a d-dimensional system whose
# right-hand side costs F operations (mul/add/div/sqrt = 1, pow/sin/cos not counted):
#   stage coefficients 20 + stage combinations 40d + stage times 12 + y_new 12d + t 1
#   + error estimate 12d + norm 5d + 5 + controller 3 + 6F;  an accepted step adds F.
RHS_FLOPS = {abi.RHS["LORENZ"]: (3, 8), abi.RHS["VAN_DER_POL"]: (2, 5), abi.RHS["PENDULUM"]: (2, 5)}


def step_flops(rhs_id):
    d, F = RHS_FLOPS[rhs_id]
    return 41 + 69 * d + 6 * F, F


def flops_of(family, accepted, rejected):
    tot = 0.0
    for rid in RHS_FLOPS:
        m = family == rid
        base, F = step_flops(rid)
        tot += base * float((accepted[m] + rejected[m]).sum()) + F * float(accepted[m].sum())
    return tot


def fp64_ops_mixed(family, accepted, rejected):
    """FP64 operations of the mixed form per attempted step: the norm accumulation (d adds), t and
    h bookkeeping (~10); the pendulum adds its FP64 stage times and drive phases (6*2 + 7*3)."""
    tot = 0.0
    for rid, (d, _F) in RHS_FLOPS.items():
        m = family == rid
        per = d + 10 + (33 if rid == abi.RHS["PENDULUM"] else 0)
        tot += per * float((accepted[m] + rejected[m]).sum())
    return tot


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(e: W.Ensemble, sample: int, threads: int):
    """The oracle (crate restatement, host libm) on the first `sample` instances."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib as O

    s = e.subset(np.arange(sample))
    b = O.Batch(0, s.dim, s.n_params, s.t0, s.tf, s.y0, s.params, s.rtol, s.atol, family=s.family)
    cfg = abi.default_cfg(abi.DOPRI5)
    cfg.max_steps = s.max_steps
    t = time.perf_counter()
    O.solve(b, cfg, threads=threads, math_mode=0)
    dt = time.perf_counter() - t
    return sample / dt, dt


def accuracy_report(e: W.Ensemble, y_gpu: np.ndarray, per_family: int = 1000, threads: int = 0):
    """Final-state error of the GPU result against (a) the FP64 oracle at the same tolerances
    (the crate's CPU solver, restated) and (b) an FP64 oracle run at rtol = atol = 1e-13
    (DOP853), on `per_family` instances of each family.  Relative error = max_c |a_c - b_c| /
    max_c |b_c|.  Lorenz instances with rho > ~24.7 are chaotic over these horizons, so their
    errors against any other trajectory grow to O(1); the table reports them as measured."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib as O

    threads = threads or (os.cpu_count() or 1)
    idx = np.concatenate([np.nonzero(e.family == f)[0][:per_family] for f in W.FAMILIES_C1])
    s = e.subset(idx)
    b = O.Batch(0, s.dim, s.n_params, s.t0, s.tf, s.y0, s.params, s.rtol, s.atol, family=s.family)
    cfg = abi.default_cfg(abi.DOPRI5)
    cfg.max_steps = s.max_steps
    same = O.solve(b, cfg, threads=threads, math_mode=1)["y_final"]
    bt = O.Batch(0, s.dim, s.n_params, s.t0, s.tf, s.y0, s.params, np.full(s.n, 1e-13), np.full(s.n, 1e-13),
                 family=s.family)
    cfg8 = abi.default_cfg(abi.DOP853)
    cfg8.max_steps = 50_000_000
    tight = O.solve(bt, cfg8, threads=threads, math_mode=1)["y_final"]
    g = y_gpu[:, idx]

    def rel(a, ref):
        return np.max(np.abs(a - ref), axis=0) / np.maximum(np.max(np.abs(ref), axis=0), 1e-300)

    out = {}
    names = {abi.RHS["VAN_DER_POL"]: "van_der_pol", abi.RHS["PENDULUM"]: "pendulum", abi.RHS["LORENZ"]: "lorenz"}
    for f in W.FAMILIES_C1:
        m = s.family == f
        r_same = rel(g[:, m], same[:, m])
        r_tight = rel(g[:, m], tight[:, m])
        r_fp64_tight = rel(same[:, m], tight[:, m])
        q = lambda v: {"median": float(np.median(v)), "p90": float(np.percentile(v, 90)), "max": float(np.max(v))}
        out[names[f]] = {"vs_fp64_oracle": q(r_same), "frac_le_1e-6_vs_fp64_oracle": float(np.mean(r_same <= 1e-6)),
                         "vs_tight_oracle": q(r_tight), "fp64_oracle_vs_tight": q(r_fp64_tight)}
        if f == abi.RHS["LORENZ"]:
            nc = s.params[1, m] < 24.0  # non-chaotic Lorenz (rho below the chaotic onset)
            out[names[f]]["nonchaotic_vs_fp64_oracle"] = q(r_same[nc]) if nc.any() else None
    out["sample"] = f"first {per_family} instances of each family; tight oracle = DOP853 rtol=atol=1e-13"
    return out


def run_profile_case(args):
    """A small case of the same workload for profiler captures: the first N instances (all three
    families), solved --steps times with the chosen variant through degpu_solve_ensemble_host."""
    import degpu

    e = W.config1(n=args.profile_case)
    prec, kern = VARIANTS[args.variant]
    m = degpu.ExplicitRungeKutta(abi.DOPRI5)
    m.cfg.precision, m.cfg.kernel, m.cfg.max_steps = prec, kern, e.max_steps
    for _ in range(max(1, args.steps)):
        t = time.perf_counter()
        g = degpu.solve_ensemble(0, 3, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m, family=e.family, n_params=3)
        print(json.dumps({"profile_case": e.n, "variant": args.variant, "wall_s": time.perf_counter() - t,
                          "step_attempts": int((g.accepted + g.rejected).sum()),
                          "complete": int((g.status == abi.COMPLETE).sum())}))


def run_reference(args):
    """--impl reference: the crate's CPU path (oracle restatement) on this host's cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n_all = args.n
    e = W.config1(n=n_all)
    threads = os.cpu_count() or 1
    sample = args.cpu_sample
    vals = []
    for i in range(args.warmup + args.steps):
        v, _ = cpu_baseline(e, sample, threads)
        if i >= args.warmup:
            vals.append(v)
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": "IVP solves/sec (uneven ensemble, DOPRI5)", "value": v, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": f"uneven ensemble {n_all} instances (VdP/pendulum/Lorenz), DOPRI5",
                   "sample_instances": sample},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} instances of the workload per step"},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--variant", default="mixed-persistent", choices=list(VARIANTS))
    ap.add_argument("--compare", default="fp64-plain", help="comma list of extra variants timed once each")
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--cpu-sample", type=int, default=12000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--profile-case", type=int, default=0,
                    help="solve only the first N instances once per --steps (a small case for ncu captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return run_profile_case(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = abi.load()

    # each rank solves its own slice of instances (weak scaling: instances are independent)
    e = W.config1(n=args.n, first=rank * args.n)
    n = e.n
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    d_in = dict(t0=T(e.t0), tf=T(e.tf), y0=T(e.y0), params=T(e.params), rtol=T(e.rtol), atol=T(e.atol),
                family=T(e.family, torch.int32))
    d_out = dict(y_final=torch.empty((3, n), dtype=torch.float64, device=dev),
                 t_final=torch.empty(n, dtype=torch.float64, device=dev),
                 accepted=torch.empty(n, dtype=torch.int64, device=dev),
                 rejected=torch.empty(n, dtype=torch.int64, device=dev),
                 fevals=torch.empty(n, dtype=torch.int64, device=dev),
                 status=torch.empty(n, dtype=torch.int32, device=dev))
    prob = abi.Problem(rhs_id=0, dim=3, n_params=3)
    bi = abi.BatchIn(n=n, t0=abi.ptr(d_in["t0"]), tf=abi.ptr(d_in["tf"]), y0=abi.ptr(d_in["y0"]),
                     params=abi.ptr(d_in["params"]), rtol=abi.ptr(d_in["rtol"]), atol=abi.ptr(d_in["atol"]),
                     family=abi.ptr(d_in["family"], C.c_int32), n_eval=0)
    bo = abi.BatchOut(y_final=abi.ptr(d_out["y_final"]), t_final=abi.ptr(d_out["t_final"]),
                      accepted=abi.ptr(d_out["accepted"], C.c_int64), rejected=abi.ptr(d_out["rejected"], C.c_int64),
                      fevals=abi.ptr(d_out["fevals"], C.c_int64), status=abi.ptr(d_out["status"], C.c_int32))
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # 256 MB > 129 MB L2

    def cfg_of(variant):
        prec, kern = VARIANTS[variant]
        c = abi.default_cfg(abi.DOPRI5)
        c.precision, c.kernel, c.max_steps = prec, kern, e.max_steps
        return c

    def solve_dev(cfg):
        rc = lib.degpu_solve_ensemble(C.byref(prob), C.byref(cfg), C.byref(bi), C.byref(bo),
                                      C.c_void_p(stream.cuda_stream))
        if rc != abi.OK:
            raise RuntimeError(f"degpu_solve_ensemble failed: {rc}")

    def timed(cfg, steps, warmup, clocks=None):
        for _ in range(warmup):
            solve_dev(cfg)
        stream.synchronize()
        ms = []
        if world > 1:
            torch.distributed.barrier()
        if clocks:
            clocks.start()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)  # L2 flush between timed iterations, outside the events
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            solve_dev(cfg)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        ck = clocks.stop() if clocks else None
        t = float(np.mean(ms))
        if world > 1:
            tt = torch.tensor([t], device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        return t, ck

    cfg = cfg_of(args.variant)
    clocks = Clocks()
    ms, ck = timed(cfg, args.steps, args.warmup, clocks)
    status = d_out["status"].cpu().numpy()
    acc = d_out["accepted"].cpu().numpy()
    rej = d_out["rejected"].cpu().numpy()
    value = n * world / (ms * 1e-3)
    steps_per_s = float((acc + rej).sum()) * world / (ms * 1e-3)
    fam = e.family

    # roofline of the dominant kernel: the persistent ensemble kernel is one launch per solve (the
    # three planning kernels before it take microseconds), so its duration is the solve's event
    # time.  Algorithmic operations are split by the pipe that executes them.
    pk = C.c_double(0.0)
    prec = VARIANTS[args.variant][0]
    lib.degpu_internal_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    lib.degpu_internal_fma_peak(1, C.byref(pk))
    fp64_peak = pk.value
    lib.degpu_internal_fma_peak(0, C.byref(pk))
    fp32_peak = pk.value
    total_ops = flops_of(fam, acc, rej)
    fp64_ops = total_ops if prec != abi.MIXED else fp64_ops_mixed(fam, acc, rej)
    fp32_ops = 0.0 if prec != abi.MIXED else total_ops - fp64_ops
    t_s = ms * 1e-3 / world
    a64 = fp64_ops / t_s / 1e12
    a32 = fp32_ops / t_s / 1e12
    f64, f32 = a64 / fp64_peak, (a32 / fp32_peak if fp32_peak else 0.0)
    kname = {abi.KERNEL_PERSISTENT: "erk_multi_kernel", abi.KERNEL_THREAD: "erk_thread_kernel"}[VARIANTS[args.variant][1]]
    bound64 = f64 >= f32
    roof = {"bound": "fp64" if bound64 else "fp32", "achieved": a64 if bound64 else a32,
            "peak": fp64_peak if bound64 else fp32_peak, "unit": "TFLOP/s", "frac": f64 if bound64 else f32,
            "traffic": None, "kernel": kname,
            "fp64": {"achieved": a64, "peak": fp64_peak, "frac": f64},
            "fp32": {"achieved": a32, "peak": fp32_peak, "frac": f32},
            "peak_source": "self-measured FMA probe (MEASURED_PEAKS.json has no FP64/FP32 figure); FMA = 2 ops",
            "note": "algorithmic ops of the whole ensemble solve / solve time (one kernel launch per solve)"}

    # end-to-end through the host-pointer entry point (pinned buffers, copies inside the timing)
    pin = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).pin_memory()
    h_in = dict(t0=pin(e.t0), tf=pin(e.tf), y0=pin(e.y0), params=pin(e.params), rtol=pin(e.rtol), atol=pin(e.atol),
                family=pin(e.family, torch.int32))
    h_out = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in d_out.items()}
    hbi = abi.BatchIn(n=n, t0=abi.ptr(h_in["t0"]), tf=abi.ptr(h_in["tf"]), y0=abi.ptr(h_in["y0"]),
                      params=abi.ptr(h_in["params"]), rtol=abi.ptr(h_in["rtol"]), atol=abi.ptr(h_in["atol"]),
                      family=abi.ptr(h_in["family"], C.c_int32), n_eval=0)
    hbo = abi.BatchOut(y_final=abi.ptr(h_out["y_final"]), t_final=abi.ptr(h_out["t_final"]),
                       accepted=abi.ptr(h_out["accepted"], C.c_int64), rejected=abi.ptr(h_out["rejected"], C.c_int64),
                       fevals=abi.ptr(h_out["fevals"], C.c_int64), status=abi.ptr(h_out["status"], C.c_int32))
    h2d = sum(v.numel() * v.element_size() for v in h_in.values())
    d2h = sum(v.numel() * v.element_size() for v in h_out.values())
    e2e_ms = []
    for i in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = lib.degpu_solve_ensemble_host(C.byref(prob), C.byref(cfg), C.byref(hbi), C.byref(hbo))
        e2e_ms.append((time.perf_counter() - t) * 1e3)
        assert rc == abi.OK
    e2e = n * world / (float(np.mean(e2e_ms)) * 1e-3)

    accuracy = None
    if rank == 0 and not args.no_accuracy:
        accuracy = accuracy_report(e, d_out["y_final"].cpu().numpy())

    extra = {}
    for v in [x for x in args.compare.split(",") if x in VARIANTS and x != args.variant]:
        t, _ = timed(cfg_of(v), 1, 1)
        extra[v] = {"solves_per_s": n * world / (t * 1e-3), "ms": t}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt = cpu_baseline(e, args.cpu_sample, threads)
        cpu = {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"first {args.cpu_sample} instances of the workload ({dt:.1f} s, host libm)"}

    # per solve: persistent variants = 3 planning kernels + 1 multi-family ensemble kernel;
    # thread variants = one ensemble kernel per family
    per_solve = 4 if VARIANTS[args.variant][1] == abi.KERNEL_PERSISTENT else 3
    launches = per_solve * args.steps
    line = {
        "metric": "IVP solves/sec (uneven ensemble, DOPRI5)", "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-stage/f64-control" if prec == abi.MIXED else "f64",
        "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": f"uneven ensemble {n} instances/GPU: 1/3 Van der Pol, 1/3 damped driven pendulum, "
                               f"1/3 Lorenz; t_end~U[5,50], rtol~logU[1e-9,1e-5], DOPRI5",
                   "variant": args.variant, "l2": "flushed (256 MB write) between timed iterations"},
        "steps_per_s": steps_per_s,
        "status_counts": {str(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "clocks": ck,
        "variants": extra,
        "accuracy": accuracy,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
