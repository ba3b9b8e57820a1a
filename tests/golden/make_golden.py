"""Writes the golden fixtures of this directory: the oracle's results (correctly rounded math
mode, the mode the FP64 parity path matches bit for bit) on seeded slices of the uneven ensemble,
frozen so that a later change to the oracle, the workload generator or the device code shows up
as a difference against a fixed file.

    python tests/golden/make_golden.py      (from the repository root, after the oracle is built)

Fixtures:
  uneven_dopri5_1500.npz  the first 1,500 instances of the uneven ensemble (Van der Pol, pendulum,
                          Lorenz), horizons clipped to 8, DOPRI5 with the crate's defaults
  uneven_dop853_dense_600.npz  600 instances, DOP853, output times 0, 0.5, ..., 4 (unsorted,
                          with a duplicate), horizons clipped to 4
Each holds the inputs (t0, tf, y0, params, rtol, atol, family) and the outputs (y_final, t_final,
accepted, rejected, fevals, status, and dense where present)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "differential-equations_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import oracle_lib as O  # noqa: E402
from degpu import abi, workloads as W  # noqa: E402

T_EVAL_853 = np.array([4.0, 0.0, 2.5, 0.5, 1.0, 3.5, 1.5, 2.0, 1.0, 3.0])


def cases():
    e = W.config1(n=1500)
    e.tf = np.minimum(e.tf, 8.0)
    yield "uneven_dopri5_1500", e, abi.DOPRI5, None
    d = W.config1(n=600, first=3000)
    d.tf = np.minimum(d.tf, 4.0)
    yield "uneven_dop853_dense_600", d, abi.DOP853, T_EVAL_853


def solve(e, method, t_eval):
    b = O.Batch(0, e.dim, e.n_params, e.t0, e.tf, e.y0, e.params, e.rtol, e.atol, family=e.family, t_eval=t_eval)
    cfg = abi.default_cfg(method)
    cfg.max_steps = 10_000_000
    return O.solve(b, cfg, math_mode=1)


def main():
    for name, e, method, te in cases():
        o = solve(e, method, te)
        out = dict(t0=e.t0, tf=e.tf, y0=e.y0, params=e.params, rtol=e.rtol, atol=e.atol, family=e.family,
                   method=np.int32(method), y_final=o["y_final"], t_final=o["t_final"], accepted=o["accepted"],
                   rejected=o["rejected"], fevals=o["fevals"], status=o["status"])
        if te is not None:
            out["t_eval"] = te
            out["dense"] = o["dense"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, e.n, int(o["accepted"].sum()))


if __name__ == "__main__":
    main()
