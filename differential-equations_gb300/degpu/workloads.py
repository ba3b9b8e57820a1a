"""Seeded synthetic workloads of the benchmark configurations.

Every random draw is a counter-based SplitMix64 hash of (base seed, config, instance, draw
number), so any instance of any workload can be regenerated alone, on any machine, in any order.

  U[a,b]               a + (b-a) u,  u = top 53 bits / 2^53
  log-uniform [a,b]    exp(ln a + (ln b - ln a) u)
  N(0, s^2)            Box–Muller on two draws
  int log-uniform      floor(exp(U[ln lo, ln(hi+1))))
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M64
        return z ^ (z >> np.uint64(31))


def uniform01(config: int, inst: np.ndarray, draw: int, seed: int = 0x5EED0000) -> np.ndarray:
    """u in [0, 1) for each instance index."""
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed + config) * np.uint64(0x100000001B3) + np.uint64(draw))
        h = splitmix64(key ^ (inst.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03)))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def U(config, inst, draw, a, b):
    return a + (b - a) * uniform01(config, inst, draw)


def logU(config, inst, draw, a, b):
    return np.exp(math.log(a) + (math.log(b) - math.log(a)) * uniform01(config, inst, draw))


def normal(config, inst, draw, sigma):
    u1 = uniform01(config, inst, draw)
    u2 = uniform01(config, inst, draw + 1)
    return sigma * np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


@dataclass
class Ensemble:
    name: str
    method: int
    n: int
    dim: int            # maximum dimension (rows of y0)
    n_params: int
    t0: np.ndarray
    tf: np.ndarray
    y0: np.ndarray      # [dim, n]
    params: np.ndarray  # [n_params, n]
    rtol: np.ndarray
    atol: np.ndarray
    rhs_id: int = 0
    family: Optional[np.ndarray] = None
    dims: Optional[np.ndarray] = None
    t_eval: Optional[np.ndarray] = None
    max_steps: int = 10_000_000
    meta: dict = field(default_factory=dict)

    def subset(self, idx: np.ndarray) -> "Ensemble":
        idx = np.asarray(idx)
        return Ensemble(self.name, self.method, len(idx), self.dim, self.n_params, self.t0[idx].copy(),
                        self.tf[idx].copy(), np.ascontiguousarray(self.y0[:, idx]),
                        np.ascontiguousarray(self.params[:, idx]), self.rtol[idx].copy(), self.atol[idx].copy(),
                        self.rhs_id, None if self.family is None else self.family[idx].copy(),
                        None if self.dims is None else self.dims[idx].copy(), self.t_eval, self.max_steps,
                        dict(self.meta))


def lorenz_draws(config: int, inst: np.ndarray):
    rho = U(config, inst, 0, 10.0, 50.0)
    y0 = np.stack([1.0 + normal(config, inst, 1 + 2 * c, 0.1) for c in range(3)])
    p = np.stack([np.full(len(inst), 10.0), rho, np.full(len(inst), 8.0 / 3.0)])
    return y0, p


def config0(n: int = 4096) -> Ensemble:
    """4096 Lorenz IVPs (d=3), DOPRI5 rtol=1e-8 atol=1e-10, t in [0,20]; sigma=10, beta=8/3,
    rho ~ U[10,50], y0 = (1,1,1) + N(0, 0.1^2)."""
    inst = np.arange(n)
    y0, p = lorenz_draws(0, inst)
    return Ensemble("lorenz-dopri5-4096", abi.DOPRI5, n, 3, 3, np.zeros(n), np.full(n, 20.0), y0, p,
                    np.full(n, 1e-8), np.full(n, 1e-10), rhs_id=abi.RHS["LORENZ"])


FAMILIES_C1 = (abi.RHS["VAN_DER_POL"], abi.RHS["PENDULUM"], abi.RHS["LORENZ"])


def _family_draws(slot: int, i: np.ndarray):
    """(y0 [3, len(i)], params [3, len(i)]) of instances `i` of one family of the uneven ensemble
    (slot 0 Van der Pol, 1 pendulum, 2 Lorenz)."""
    y0 = np.zeros((3, len(i)))
    p = np.zeros((3, len(i)))
    if slot == 0:  # Van der Pol: mu ~ logU[0.1,5], y0 ~ U[-2,2]^2
        p[0] = logU(1, i, 10, 0.1, 5.0)
        y0[0] = U(1, i, 11, -2.0, 2.0)
        y0[1] = U(1, i, 12, -2.0, 2.0)
    elif slot == 1:  # pendulum: gamma ~ U[0.05,0.5], A ~ U[0.5,1.5], Omega ~ U[0.5,1], y0 ~ U[-2,2]^2
        p[0] = U(1, i, 20, 0.05, 0.5)
        p[1] = U(1, i, 21, 0.5, 1.5)
        p[2] = U(1, i, 22, 0.5, 1.0)
        y0[0] = U(1, i, 23, -2.0, 2.0)
        y0[1] = U(1, i, 24, -2.0, 2.0)
    else:  # Lorenz as config 0
        y0[:], p[:] = lorenz_draws(1, i)
    return y0, p


def config1(n: int = 1 << 20, first: int = 0) -> Ensemble:
    """Uneven ensemble: instance index mod 3 -> Van der Pol / damped driven pendulum / Lorenz;
    t_end ~ U[5,50], rtol ~ logU[1e-9,1e-5], atol = 1e-2 rtol, DOPRI5."""
    inst = np.arange(first, first + n)
    fam_idx = inst % 3
    family = np.array(FAMILIES_C1, dtype=np.int32)[fam_idx]
    y0 = np.zeros((3, n))
    p = np.zeros((3, n))
    for slot in range(3):
        m = fam_idx == slot
        y0[:, m], p[:, m] = _family_draws(slot, inst[m])
    tf = U(1, inst, 30, 5.0, 50.0)
    rtol = logU(1, inst, 31, 1e-9, 1e-5)
    return Ensemble("uneven-dopri5", abi.DOPRI5, n, 3, 3, np.zeros(n), tf, y0, p, rtol, 1e-2 * rtol,
                    family=family)


def config1_family(slot: int, n: int, first: int = 0) -> Ensemble:
    """n instances of one family of the uneven ensemble (slot 0 Van der Pol, 1 pendulum, 2 Lorenz):
    the instances first + 3 j + r (r the residue that gives the slot), with the draws config1 gives
    them, generated without the other families.  Single-family batch: rhs_id set, no family map,
    state and parameter rows of that family only."""
    inst = first + 3 * np.arange(n) + ((slot - first) % 3)
    y0, p = _family_draws(slot, inst)
    fid = FAMILIES_C1[slot]
    d = 3 if fid == abi.RHS["LORENZ"] else 2
    tf = U(1, inst, 30, 5.0, 50.0)
    rtol = logU(1, inst, 31, 1e-9, 1e-5)
    return Ensemble("uneven-family", abi.DOPRI5, n, d, 3, np.zeros(n), tf, np.ascontiguousarray(y0[:d]), p, rtol,
                    1e-2 * rtol, rhs_id=fid)


def config2(n: int = 131072, first: int = 0, max_masses: int = 128) -> Ensemble:
    """FPU-beta chains with fixed ends: masses ~ int log-uniform [2,128] (d = 2 masses),
    beta ~ U[0.1,1], x ~ N(0,0.1^2), p = 0; DOP853 rtol=1e-10 atol=1e-12, t in [0,100],
    64 output times 100 k / 63.  `max_masses` caps the draw (the serving configuration's
    chains have at most 64 masses)."""
    inst = np.arange(first, first + n)
    masses = np.floor(np.exp(U(2, inst, 0, math.log(2.0), math.log(129.0)))).astype(np.int32)
    masses = np.clip(masses, 2, max_masses)
    dims = 2 * masses
    dmax = int(dims.max()) if n else 2
    y0 = np.zeros((dmax, n))
    for j in range(128):
        sel = masses > j
        if not sel.any():
            break
        y0[j, sel] = normal(2, inst[sel], 10 + 2 * j, 0.1)
    # momenta are zero; rows [m, 2m) of each instance stay 0
    beta = U(2, inst, 1, 0.1, 1.0)
    te = 100.0 * np.arange(64) / 63.0
    return Ensemble("fpu-dop853", abi.DOP853, n, dmax, 1, np.zeros(n), np.full(n, 100.0), y0, beta.reshape(1, n),
                    np.full(n, 1e-10), np.full(n, 1e-12), rhs_id=abi.RHS["FPU_BETA"], dims=dims, t_eval=te)


def gray_scott_init(nx: int = 4096, ny: int = 4096, squares: int = 64, size: int = 32):
    """u = 1, v = 0 plus `squares` seeded size x size squares set to u = 0.5, v = 0.25, each cell
    multiplied by (1 + U[-0.01, 0.01])."""
    u = np.ones((ny, nx))
    v = np.zeros((ny, nx))
    sq = np.arange(squares)
    x0 = np.floor(U(3, sq, 0, 0, nx - size)).astype(np.int64)
    y0 = np.floor(U(3, sq, 1, 0, ny - size)).astype(np.int64)
    for s in range(squares):
        cells = (np.arange(size)[:, None] * size + np.arange(size)[None, :]).reshape(-1) + s * size * size
        nu = U(3, cells, 2, -0.01, 0.01).reshape(size, size)
        nv = U(3, cells, 3, -0.01, 0.01).reshape(size, size)
        u[y0[s]:y0[s] + size, x0[s]:x0[s] + size] = 0.5 * (1.0 + nu)
        v[y0[s]:y0[s] + size, x0[s]:x0[s] + size] = 0.25 * (1.0 + nv)
    return u, v


GRAY_SCOTT = dict(F=0.037, k=0.06, Du=2e-5, Dv=1e-5)


def rank_slice(n_per_rank: int, rank: int):
    """Instances [rank * n, (rank + 1) * n) of a workload: the replica partition used with several
    GPUs (instances are independent, so ranks share nothing but the timing reduction)."""
    return rank * n_per_rank, n_per_rank
