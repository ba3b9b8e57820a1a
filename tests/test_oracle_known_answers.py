"""The CPU oracle against the crate's own known-answer tests (expected values and tolerances
copied from the crate's test files, cited per case).  These pin the oracle before it is used as
the parity checker of the GPU path."""
import math

import numpy as np
import pytest

import oracle_lib as O
from degpu import abi

R = abi.RHS


def solve1(rhs, dim, params, t0, tf, y0, method, rtol=1e-6, atol=1e-6, h0=0.0, t_eval=None, math_mode=1,
           max_steps=10_000):
    b = O.Batch(rhs, dim, len(params), [t0], [tf], np.array(y0, dtype=float).reshape(dim, 1),
                np.array(params, dtype=float).reshape(-1, 1) if params else [], [rtol], [atol], t_eval=t_eval)
    cfg = abi.default_cfg(method)
    cfg.h0 = h0
    cfg.max_steps = max_steps
    return O.solve(b, cfg, threads=1, math_mode=math_mode)


# tests/ode/accuracy.rs: (system, t0, tf, y0, expected, [(method, rtol, atol, h0, tol)])
CASES = [
    ("exp+", R["EXP_GROWTH"], [1.0], 0.0, 10.0, [1.0], [22026.46579479],          # accuracy.rs:70-94
     [(abi.DOP853, 1e-12, 1e-12, 0.0, 1e-3), (abi.DOPRI5, 1e-6, 1e-6, 0.0, 1e1), (abi.RK4, 1e-6, 1e-6, 0.01, 1e3),
      (abi.RKF45, 1e-6, 1e-6, 0.0, 1e3), (abi.CASH_KARP, 1e-6, 1e-6, 0.0, 1e3)]),
    ("exp-", R["EXP_GROWTH"], [1.0], 0.0, -10.0, [22026.46579479], [1.0],          # accuracy.rs:177-204
     [(abi.DOP853, 1e-12, 1e-12, 0.0, 1e-3), (abi.DOPRI5, 1e-6, 1e-6, 0.0, 1e-2), (abi.RK4, 1e-6, 1e-6, -0.01, 1e-2),
      (abi.RKF45, 1e-6, 1e-6, 0.0, 1e-2), (abi.CASH_KARP, 1e-6, 1e-6, 0.0, 1e-2)]),
    ("linear", R["LINEAR"], [1.0, 1.0], 0.0, 10.0, [1.0], [44051.93158958],        # accuracy.rs:286-313
     [(abi.DOP853, 1e-12, 1e-12, 0.0, 1e-3), (abi.DOPRI5, 1e-6, 1e-6, 0.0, 1e1), (abi.RK4, 1e-6, 1e-6, 0.01, 1e3),
      (abi.RKF45, 1e-6, 1e-6, 0.0, 1e3), (abi.CASH_KARP, 1e-6, 1e-6, 0.0, 1e3)]),
    ("harmonic", R["HARMONIC"], [1.0], 0.0, 10.0, [1.0, 0.0], [-0.83907153, 0.54402111],  # accuracy.rs:395-422
     [(abi.DOP853, 1e-12, 1e-12, 0.0, 1e-3), (abi.DOPRI5, 1e-6, 1e-6, 0.0, 1e-2), (abi.RK4, 1e-6, 1e-6, 0.01, 1e-1),
      (abi.RKF45, 1e-6, 1e-6, 0.0, 1e-3), (abi.CASH_KARP, 1e-6, 1e-6, 0.0, 1e-3)]),
    ("logistic", R["LOGISTIC"], [1.0, 10.0], 0.0, 10.0, [0.1], [9.95525518],       # accuracy.rs:504-531
     [(abi.DOP853, 1e-12, 1e-12, 0.0, 1e-3), (abi.DOPRI5, 1e-6, 1e-6, 0.0, 1e-3), (abi.RK4, 1e-6, 1e-6, 0.01, 1e3),
      (abi.RKF45, 1e-6, 1e-6, 0.0, 1e-2), (abi.CASH_KARP, 1e-6, 1e-6, 0.0, 1e-2)]),
    ("robertson", R["ROBERTSON"], [], 0.0, 0.4, [1.0, 0.0, 0.0],                    # accuracy.rs:622-671
     [0.9851721139, 3.3863953790e-05, 0.0147940222],
     [(abi.DOP853, 1e-10, 1e-12, 0.0, 1e-1), (abi.DOPRI5, 1e-8, 1e-10, 0.0, 5e-1)]),
]


@pytest.mark.parametrize("math_mode", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_accuracy_known_answers(case, math_mode):
    name, rhs, p, t0, tf, y0, expected, runs = case
    for method, rtol, atol, h0, tol in runs:
        o = solve1(rhs, len(y0), p, t0, tf, y0, method, rtol, atol, h0, math_mode=math_mode)
        assert o["status"][0] == abi.COMPLETE
        for c, e in enumerate(expected):
            assert abs(o["y_final"][c, 0] - e) < tol, (name, method, c, o["y_final"][c, 0], e)


VERNER = [abi.RKV655E, abi.RKV766E, abi.RKV767E, abi.RKV877E, abi.RKV878E, abi.RKV988E, abi.RKV989E]
# tests/ode/accuracy.rs: the Verner pairs at their defaults (rtol = atol = 1e-6), one tolerance per
# system for all of them (accuracy.rs:124-151, 233-260, 342-369, 451-478, 560-587). RKV656e is not
# in the crate's tests; it is held to the same tolerances.
VERNER_CASES = [
    ("exp+", R["EXP_GROWTH"], [1.0], 0.0, 10.0, [1.0], [22026.46579479], 1e-1),
    ("exp-", R["EXP_GROWTH"], [1.0], 0.0, -10.0, [22026.46579479], [1.0], 1e-2),
    ("linear", R["LINEAR"], [1.0, 1.0], 0.0, 10.0, [1.0], [44051.93158958], 1e1),
    ("harmonic", R["HARMONIC"], [1.0], 0.0, 10.0, [1.0, 0.0], [-0.83907153, 0.54402111], 1e-3),
    ("logistic", R["LOGISTIC"], [1.0, 10.0], 0.0, 10.0, [0.1], [9.95525518], 1e-3),
]


@pytest.mark.parametrize("method", VERNER + [abi.RKV656E])
@pytest.mark.parametrize("case", VERNER_CASES, ids=[c[0] for c in VERNER_CASES])
def test_verner_accuracy_known_answers(case, method):
    name, rhs, p, t0, tf, y0, expected, tol = case
    o = solve1(rhs, len(y0), p, t0, tf, y0, method)
    assert o["status"][0] == abi.COMPLETE
    for c, e in enumerate(expected):
        assert abs(o["y_final"][c, 0] - e) < tol, (name, method, c, o["y_final"][c, 0], e)


def test_verner_counters():
    # adaptive/ordinary.rs: S - 1 stages per attempt, I - S dense-output stages and (without FSAL)
    # one derivative per acceptance, k0 plus the doubly counted h_init pair at init
    for method, S, I, fsal in [(abi.RKV655E, 9, 10, True), (abi.RKV656E, 9, 12, True), (abi.RKV766E, 10, 13, False),
                               (abi.RKV989E, 16, 26, False)]:
        o = solve1(R["HARMONIC"], 2, [1.0], 0.0, 10.0, [1.0, 0.0], method)
        acc, rej, fe = o["accepted"][0], o["rejected"][0], o["fevals"][0]
        assert fe == 5 + (S - 1) * (acc + rej) + (I - S) * acc + (0 if fsal else acc), (method, fe)


@pytest.mark.parametrize("method,h0", [(abi.DOP853, 0.0), (abi.DOPRI5, 0.0), (abi.RK4, 0.01), (abi.RKF45, 0.0),
                                       (abi.CASH_KARP, 0.0), (abi.RKV655E, 0.0), (abi.RKV877E, 0.0),
                                       (abi.RKV988E, 0.0)])
def test_interpolation_known_answer(method, h0):
    # tests/ode/interpolation.rs:14-87: t_eval [0.5, 1.0, 1.69] on exp growth, |y(0.5) - e^0.5| < 1e-3
    o = solve1(R["EXP_GROWTH"], 1, [1.0], 0.0, 2.0, [1.0], method, h0=h0, t_eval=[0.5, 1.0, 1.69])
    assert abs(o["dense"][0, 0, 0] - math.exp(0.5)) < 1e-3
    assert np.all(np.isfinite(o["dense"][:, 0, 0]))


@pytest.mark.parametrize("method,h0", [(abi.DOP853, 0.0), (abi.DOPRI5, 0.0), (abi.RK4, 0.1)])
def test_bad_input_tf_equals_t0(method, h0):
    # tests/ode/errors.rs:86-107: tf == t0 -> BadInput
    o = solve1(R["EXP_GROWTH"], 1, [1.0], 0.0, 0.0, [1.0], method, h0=h0)
    assert o["status"][0] == abi.ERR_BAD_INPUT


@pytest.mark.parametrize("method", [abi.DOP853, abi.DOPRI5, abi.RK4])
def test_bad_input_h0_too_big(method):
    # tests/ode/errors.rs:109-130: h0 = 10 on [0, 1] -> BadInput
    o = solve1(R["EXP_GROWTH"], 1, [1.0], 0.0, 1.0, [1.0], method, h0=10.0)
    assert o["status"][0] == abi.ERR_BAD_INPUT


def test_max_steps_error():
    # the attempted-step cap (src/methods/erk/mod.rs:139, dormandprince/ordinary.rs:82-92)
    o = solve1(R["LORENZ"], 3, [10.0, 28.0, 8.0 / 3.0], 0.0, 20.0, [1.0, 1.0, 1.0], abi.DOPRI5, 1e-8, 1e-10,
               max_steps=50)
    assert o["status"][0] == abi.ERR_MAX_STEPS
    assert o["accepted"][0] + o["rejected"][0] == 50


def test_step_counts_match_quirks():
    # DOPRI5 evaluates 6 stages per attempt + 1 on acceptance + 3 at init (2 h_init + k0),
    # dormandprince/ordinary.rs:122,163 and h_init.rs:68-101
    o = solve1(R["HARMONIC"], 2, [1.0], 0.0, 10.0, [1.0, 0.0], abi.DOPRI5)
    acc, rej, fe = o["accepted"][0], o["rejected"][0], o["fevals"][0]
    assert fe == 3 + 6 * (acc + rej) + acc
    # DOP853: 11 per attempt, +1 +3 dense stages per acceptance
    o = solve1(R["HARMONIC"], 2, [1.0], 0.0, 10.0, [1.0, 0.0], abi.DOP853)
    acc, rej, fe = o["accepted"][0], o["rejected"][0], o["fevals"][0]
    assert fe == 3 + 11 * (acc + rej) + 4 * acc
    # RK4: 4 per step + 1 at init (fixed/ordinary.rs:44,90,132)
    o = solve1(R["HARMONIC"], 2, [1.0], 0.0, 1.0, [1.0, 0.0], abi.RK4, h0=0.01)
    assert o["fevals"][0] == 1 + 4 * o["accepted"][0]


def test_dopri5_dense_is_cubic_part_only():
    # The crate's DOPRI5 dense coefficient cont[4] is zero (only row 0 of bi is filled,
    # dorman_prince.rs:95-101, row 4 is read, ordinary.rs:228-234): the interpolant at the step
    # midpoint equals the cubic cont0 + s(cont1 + s1(cont2 + s cont3)).  Check through a
    # t_eval point that interpolation is exact at the step ends and differs from the
    # DOP853 high-order value only at the interpolation-error level.
    o5 = solve1(R["EXP_GROWTH"], 1, [1.0], 0.0, 2.0, [1.0], abi.DOPRI5, 1e-10, 1e-10, t_eval=[0.5, 2.0])
    assert abs(o5["dense"][1, 0, 0] - o5["y_final"][0, 0]) == 0.0
    assert abs(o5["dense"][0, 0, 0] - math.exp(0.5)) < 1e-6


def test_mol_heat_known_answers():
    L = O.lib()
    # tests/pde/method_of_lines.rs:72-91: Dirichlet nodes have dydt = 0
    y = np.array([2.0, 1.0, 0.0, -0.5, -1.0])
    d = np.zeros(5)
    L.oracle_heat1d_diff(1.0, 5, 0.0, 1.0, 0, 2.0, 0, -1.0, O.p(y), O.p(d))
    assert d[0] == 0.0 and d[4] == 0.0
    # :93-113 fixed-size state: dydt[2] ~ 0
    y = np.array([0.0, 1.0, 0.0, -1.0, 0.0])
    L.oracle_heat1d_diff(1.0, 5, 0.0, 1.0, 0, 0.0, 0, 0.0, O.p(y), O.p(d))
    assert d[0] == 0.0 and d[4] == 0.0 and abs(d[2]) < 1e-12
    # :142-157 Neumann prescribed gradient: dydt[0] = (1/dx)/dx
    y = np.array([1.0, 2.0, 2.0, 2.0, 2.0])
    L.oracle_heat1d_diff(1.0, 5, 0.0, 1.0, 1, 0.0, 1, 0.0, O.p(y), O.p(d))
    dx = 0.25
    assert abs(d[0] - (1.0 / dx) / dx) < 1e-12
    # :115-140 vector field: dydt[2] = -0.25, dydt[3] = 4.25
    y = np.array([0.0, 1.0, 0.5, 0.25, 1.0, 0.0])
    dd = np.zeros(6)
    lo = np.array([0.0, 1.0])
    hi = np.array([1.0, 0.0])
    L.oracle_coupled1d_diff(1.0, 2.0, 3, 0.0, 1.0, O.p(lo), O.p(hi), O.p(y), O.p(dd))
    assert dd[0] == 0.0 and dd[1] == 0.0 and dd[4] == 0.0 and dd[5] == 0.0
    assert abs(dd[2] + 0.25) < 1e-12 and abs(dd[3] - 4.25) < 1e-12


def test_mol_heat_mode_decay():
    # tests/pde/method_of_lines.rs:36-70: heat alpha=0.1, 41 nodes, RK4(1e-4) to t=0.02
    L = O.lib()
    n = 41
    x = np.linspace(0.0, 1.0, n)
    x = np.array([0.0 + (1.0 / (n - 1)) * i for i in range(n)])
    u0 = np.sin(math.pi * x)
    uf = np.zeros(n)
    acc = np.zeros(1, np.int64)
    st = L.oracle_heat1d_solve(0.1, n, 0.0, 0.02, 1e-4, O.p(u0), O.p(uf), acc.ctypes.data_as(O.I64P))
    assert st == abi.COMPLETE
    decay = math.exp(-0.1 * math.pi ** 2 * 0.02)
    assert np.max(np.abs(uf - decay * np.sin(math.pi * x))) < 5e-4
