"""Step programs on the CPU. The batched kernels' (gpuklu_plan_steps): its
operations, executed step by step with each step's operations in reverse or
shuffled order, give bit for bit the factors and the solution of the
column-by-column path they replace, on the exact-pivot plans of the circuits
and matrices of the plan-parity tests; the solution also agrees with a dense
solve. The single-system solve's (gpuklu_plan_solve_steps): on the same
systems in both pivot modes, in any order within a step, it gives the device
solve's results bit for bit."""
import numpy as np
import pytest

from plan_emulator import EmulatedSolver, batch_region, factor_solve_columns, run_steps
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from test_plan_parity import SYSTEMS

from oracle import pyoracle as po

STEP_SYSTEMS = SYSTEMS + [("chain200", *po.mna(cz.inverter_chain(200, 0.6),
                                               wl.chain_nodeset(200, 0.6))[1:])]


@pytest.mark.parametrize("sysm", STEP_SYSTEMS, ids=[s[0] for s in STEP_SYSTEMS])
def test_step_program_matches_the_column_path(sysm):
    name, ap, ai, ax, rhs = sysm
    n = len(ap) - 1
    es = EmulatedSolver(N.PIVOT_EXACT)
    es.factor(n, ap, ai, ax)
    P = es.plan
    from plan_emulator import first_factor
    _, rperm = first_factor(N.Plan(n, ap, ai, N.PIVOT_EXACT), ax)
    # any region layout X[nc] T[n] DV[ndv] V[...]; offsets past 32767 too
    nc_hi = 32767 - 9 - (n + P.nslots + len(P.offd_raw)) - 1  # the last fitting layout
    for nc, ndv in ((7, 13), (nc_hi, 9)):
        prog = N.step_program(n, ap, ai, nc, ndv, N.PIVOT_EXACT, rperm)
        assert prog is not None
        ops, sp = prog
        assert sp[0] == 0 and sp[-1] == len(ops) and np.all(np.diff(sp) > 0)
        w0 = ops[:, 0].astype(np.int64) & 0xffffffff
        w1 = ops[:, 1].astype(np.int64) & 0xffffffff
        kinds = (w0 >> 30) | ((w1 >> 30) << 2)
        assert np.sum(kinds == 1) == n  # one reciprocal per column
        base = batch_region(P, ax, rhs, nc, ndv)
        want = factor_solve_columns(P, base.copy(), nc, ndv)
        for order in (None, "reverse", np.random.default_rng(5)):
            got = run_steps(ops, sp, base.copy(), order)
            assert np.array_equal(got, want), (order, np.max(np.abs(got - want)))
    x = want[nc + P.out_pos]
    a = np.zeros((n, n))
    for j in range(n):
        for t in range(ap[j], ap[j + 1]):
            a[ai[t], j] += ax[t]
    ref = np.linalg.solve(a, rhs)
    if name not in ("adder_dcop_01",):  # the reference's pivots leave it inaccurate
        assert np.max(np.abs(x - ref)) <= 1e-6 * max(1.0, np.max(np.abs(ref)))
    # fewer steps than operations: the schedule finds parallel work
    assert len(sp) - 1 < len(ops)


def test_step_program_absent_beyond_16_bit_offsets():
    c = cz.inverter_chain(8, 0.3)
    n, ap, ai, ax, rhs = po.mna(c, np.zeros(c.node_count))
    assert N.step_program(n, ap, ai, 32700, 13) is None
    assert N.step_program(n, ap, ai, 7, 13) is not None


def _run_solve_steps(ops, sp, P, ax, lu, rhs, order=None):
    """The single-system solve's step program (gpuklu_plan_solve_steps) on
    the CPU: products and differences separately rounded, the pivot division
    exact, a step's operations in the given order."""
    T = np.zeros(P.n)
    T[P.in_pos] = rhs
    for t in range(len(sp) - 1):
        idx = list(range(sp[t], sp[t + 1]))
        if order == "reverse":
            idx.reverse()
        elif order is not None:
            order.shuffle(idx)
        for p in idx:
            d, s, v, k = (int(x) for x in ops[p])
            if k == 1:
                T[d] = T[d] / lu[v]
            else:
                T[d] = T[d] - (ax[v] if k == 2 else lu[v]) * T[s]
    return T[P.out_pos]


@pytest.mark.parametrize("mode", [N.PIVOT_REFERENCE, N.PIVOT_EXACT], ids=["reference", "exact"])
@pytest.mark.parametrize("sysm", STEP_SYSTEMS, ids=[s[0] for s in STEP_SYSTEMS])
def test_solve_step_program_matches_the_sweeps(sysm, mode):
    """The solve's step program, run step by step with each step's
    operations in listed, reversed or shuffled order, gives the device
    solve's results bit for bit (the row-oriented emulation the plan-parity
    tests pin to the oracle): every row sees its updates in the sweeps'
    order."""
    from plan_emulator import first_factor, solve
    name, ap, ai, ax, rhs = sysm
    n = len(ap) - 1
    es = EmulatedSolver(mode)
    es.factor(n, ap, ai, ax)
    _, rperm = first_factor(N.Plan(n, ap, ai, mode), ax)
    prog = N.solve_step_program(n, ap, ai, mode, rperm)
    assert prog is not None
    ops, sp = prog
    assert sp[0] == 0 and sp[-1] == len(ops) and np.all(np.diff(sp) > 0)
    assert np.sum(ops[:, 3] == 1) == n  # one pivot division per row
    want = solve(es.plan, es.ax, es.lu, np.asarray(rhs, np.float64))
    for order in (None, "reverse", np.random.default_rng(3)):
        got = _run_solve_steps(ops, sp, es.plan, es.ax, es.lu, np.asarray(rhs, np.float64),
                               order)
        assert np.array_equal(got, want), (name, order, np.max(np.abs(got - want)))
    assert len(sp) - 1 <= len(ops)
