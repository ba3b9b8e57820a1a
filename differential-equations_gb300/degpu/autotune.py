"""Autotuner of the group-per-system kernel (ragged systems such as FPU-beta chains).

For every dimension bucket (d <= 8, 16, 32, 64, 128, 256) and a given (method, precision,
dense output), it times each candidate layout — G lanes per system (so 32/G systems per warp)
and CPL components per lane, which together set the register / shared-memory split — on a
sample of that bucket's instances, and keeps the fastest.  Results are written to a JSON file
(for people) and to the line format the library reads at start-up through DEGPU_TUNE_FILE
("method precision dense dmax G CPL").

    python -m degpu.autotune --method dop853 --precision parity --dense
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np

from . import abi
from . import workloads as W

CANDIDATES = {8: [(8, 1), (16, 1), (32, 1)], 16: [(16, 1), (32, 1)], 32: [(32, 1), (16, 2)],
              64: [(32, 2), (16, 4)], 128: [(32, 4)], 256: [(32, 8)]}
# DOPRI5 has no (16, CPL > 1) kernels: its buckets of 32 and 64 keep the 32-lane layouts
DOPRI5_MISSING = {(16, 2), (16, 4)}
HERE = os.path.dirname(os.path.abspath(__file__))
TUNE_TXT = os.path.join(HERE, "group_tune.txt")
TUNE_JSON = os.path.join(HERE, "group_tune.json")


def _set(lib, method, prec, dense, dmax, g, cpl):
    fn = lib.degpu_internal_group_config
    fn.argtypes = [C.c_int] * 6
    fn.restype = C.c_int
    if fn(method, prec, dense, dmax, g, cpl) != 0:
        raise RuntimeError(f"no bucket {dmax}")


def tune(method=abi.DOP853, precision=abi.FP64_PARITY, dense=True, per_bucket=1024, horizon=10.0, reps=2):
    import degpu

    lib = abi.load()
    pool = W.config2(n=16 * per_bucket)
    choices = []
    lo = 0
    for dmax, cands in CANDIDATES.items():
        if method == abi.DOPRI5:
            cands = [c for c in cands if c not in DOPRI5_MISSING]
        sel = np.nonzero((pool.dims > lo) & (pool.dims <= dmax))[0][:per_bucket]
        lo = dmax
        if len(sel) == 0:
            choices.append({"dmax": dmax, "g": cands[0][0], "cpl": cands[0][1], "timings_ms": {}})
            continue
        e = pool.subset(sel)
        e.tf[:] = horizon
        if precision == abi.MIXED:
            # the FP32-stage kernels run only above the mixed-precision bound: tune them there
            e.rtol[:] = max(1e-6, 10.0 * lib.degpu_mixed_min_rtol(method))
            e.atol = 1e-2 * e.rtol
        te = np.linspace(0.0, horizon, 8) if dense else None
        m = degpu.ExplicitRungeKutta(method)
        m.cfg.precision, m.cfg.max_steps = precision, 10_000_000
        timings = {}
        for g, cpl in cands:
            _set(lib, method, precision, 1 if dense else 0, dmax, g, cpl)
            best = float("inf")
            for _ in range(reps):
                t = time.perf_counter()
                degpu.solve_ensemble(e.rhs_id, e.dim, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, m, t_eval=te,
                                     dims=e.dims, n_params=1)
                best = min(best, time.perf_counter() - t)
            timings[f"{g}x{cpl}"] = best * 1e3
        g, cpl = min(cands, key=lambda c: timings[f"{c[0]}x{c[1]}"])
        _set(lib, method, precision, 1 if dense else 0, dmax, g, cpl)
        choices.append({"dmax": dmax, "g": g, "cpl": cpl, "timings_ms": timings, "instances": int(len(sel))})
    return choices


def save(results):
    """Merges `results` into the files: entries of other (method, precision, dense) keys stay."""
    merged = {}
    if os.path.exists(TUNE_JSON):
        with open(TUNE_JSON) as f:
            for b in json.load(f):
                merged[(b["method"], b["precision"], b["dense"])] = b["buckets"]
    merged.update(results)
    lines, blob = [], []
    for (method, prec, dense), choices in sorted(merged.items()):
        for c in choices:
            lines.append(f"{method} {prec} {dense} {c['dmax']} {c['g']} {c['cpl']}")
        blob.append({"method": method, "precision": prec, "dense": dense, "buckets": choices})
    with open(TUNE_TXT, "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(TUNE_JSON, "w") as f:
        json.dump(blob, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--method", default="dop853", choices=["dopri5", "dop853"])
    ap.add_argument("--precision", default="all", choices=["parity", "fast", "mixed", "all"])
    ap.add_argument("--dense", action="store_true")
    ap.add_argument("--per-bucket", type=int, default=1024)
    a = ap.parse_args()
    method = abi.DOP853 if a.method == "dop853" else abi.DOPRI5
    precs = {"parity": [abi.FP64_PARITY], "fast": [abi.FP64_FAST], "mixed": [abi.MIXED],
             "all": [abi.FP64_PARITY, abi.FP64_FAST, abi.MIXED]}[a.precision]
    results = {}
    for p in precs:
        results[(method, p, 1 if a.dense else 0)] = tune(method, p, a.dense, a.per_bucket)
        print(json.dumps({"method": method, "precision": p, "dense": a.dense,
                          "choices": results[(method, p, 1 if a.dense else 0)]}))
    save(results)


if __name__ == "__main__":
    main()
