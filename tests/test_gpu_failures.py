"""Failure detection on the device, made without a GPU fault.

The reference's solver runs on the CPU and its error paths are SolverError
(crates/sim-core/src/solver.rs:76-92) and the Newton loop's SolverFailure
(crates/sim-core/src/newton.rs:85-91). The device adds one condition of its
own: a dependency wait (grid refactorization, grid and transpose solves, the
one-block refactorization) that runs out of polls. These tests make each
failure on the host:

- a spin limit of one poll, so a warp that finds a dependency unfinished
  gives up at once; the kernel ends normally, the call reports
  DEVICE_TIMEOUT and the handle, given its default limit back, factors and
  solves bit for bit as before;
- a NaN planted in a device parameter or a right-hand side, which the
  reference carries through (its convergence test is false for NaN, so the
  Newton loop runs to its cap) and which the device carries through the
  same way, or stops on at once when asked;
- singular blocks, which the reference's NativeKLU perturbs to +-1e-14
  (native_klu.rs:1229-1231, 1344-1348) instead of failing.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, SolverError, newton_dc

pytestmark = pytest.mark.gpu


def _factor_solve(g, ap, ai, ax, rhs):
    g.factor(ap, ai, ax)
    x = rhs.copy()
    g.solve(x)
    return x


def _timeouts(call, tries=8):
    """Runs call() `tries` times; returns how many raised DEVICE_TIMEOUT
    (any other error fails the test)."""
    hit = 0
    for _ in range(tries):
        try:
            call()
        except SolverError as e:
            assert e.status == N.DEVICE_TIMEOUT, e
            hit += 1
    return hit


@pytest.mark.parametrize("one_block", ["0", "1"], ids=["grid", "one_block"])
def test_spin_limit_runs_out_and_the_handle_recovers(one_block, monkeypatch):
    # the 32x32 diode mesh refactors on the grid (273k updates); a 256-stage
    # inverter chain refactors in one block
    monkeypatch.setenv("GPUKLU_ONE_BLOCK", one_block)
    if one_block == "0":
        c = cz.mesh_dc()
        x = np.zeros(c.node_count)
    else:
        c = cz.inverter_chain(256, 0.55)
        x = wl.chain_nodeset(256, 0.55)
    n, ap, ai, ax, rhs = po.mna(c, x)
    g = GpuKluSolver(n)
    o = po.Solver("nativeklu", n)
    o.prepare(n)
    o.analyze(ap, ai)
    # a first factorization, then the refactorization every later call runs
    # (in the reference's pivot mode the two differ: the first drops the
    # entries its row swaps move outside the pivot-free pattern)
    for _ in range(2):
        x_ref = _factor_solve(g, ap, ai, ax, rhs)
        o.factor(ap, ai, ax)
        assert np.array_equal(x_ref, o.solve(rhs)[1])

    g.set_spin_limit(1)
    hit = _timeouts(lambda: g.factor(ap, ai, ax))
    assert hit > 0, "no dependency wait ran out at a limit of one poll"
    if one_block == "0":  # the grid solve waits on per-row flags
        g.set_spin_limit(0)
        g.factor(ap, ai, ax)
        g.set_spin_limit(1)
        assert _timeouts(lambda: g.solve(rhs.copy())) > 0

    g.set_spin_limit(0)
    assert np.array_equal(_factor_solve(g, ap, ai, ax, rhs), x_ref)
    g.close()


def test_timeout_ends_the_device_newton_loop(monkeypatch):
    monkeypatch.setenv("GPUKLU_ONE_BLOCK", "0")
    c = cz.mesh_dc()
    cfg = N.newton_config(**dict(wl.TIGHT, gmin_steps=10))
    g = GpuKluSolver(1)
    dc = DeviceCircuit(c)
    ok = newton_dc(g, dc, cfg)
    assert ok.converged
    g.set_spin_limit(1)
    with pytest.raises(SolverError) as e:
        newton_dc(g, dc, cfg)
    assert e.value.status == N.DEVICE_TIMEOUT
    g.set_spin_limit(0)
    again = newton_dc(g, dc, cfg)
    assert again.iterations == ok.iterations and np.array_equal(again.x, ok.x)


def test_nan_parameter_runs_to_the_cap_as_the_reference():
    c = cz.mesh_dc()
    r = int(np.flatnonzero(c.type == cz.DEV_R)[7])
    c.p[r, 0] = np.nan
    cfg = dict(wl.TIGHT, max_iters=12, gmin_steps=2)
    ocfg = {k: cfg[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps",
                                "source_steps")}
    r_o, it_o, _ = po.dc_op(c, "nativeklu", **ocfg)
    assert r_o == "maxiters" and it_o == 12
    g = GpuKluSolver(1)
    dc = DeviceCircuit(c)
    res = newton_dc(g, dc, N.newton_config(**cfg))
    assert res.reason == "maxiters" and res.iterations == it_o
    assert res.iterations_total == 3 * 12
    assert np.isnan(res.x).any()
    # asked to stop: the first iterate is already non-finite
    g.set_stop_on_nonfinite(True)
    with pytest.raises(SolverError) as e:
        newton_dc(g, dc, N.newton_config(**cfg))
    assert e.value.status == N.NONFINITE
    assert "iteration 1" in str(e.value)
    # the handle keeps working on a finite circuit
    c.p[r, 0] = 1000.0
    good = newton_dc(g, DeviceCircuit(c), N.newton_config(**cfg))
    r_o, it_o, x_o = po.dc_op(c, "nativeklu", **ocfg)
    assert good.reason == r_o and good.iterations == it_o
    assert np.max(np.abs(good.x - x_o)) <= 1e-10 * np.max(np.abs(x_o))


@pytest.mark.parametrize("mode,kind", [(N.PIVOT_REFERENCE, "nativeklu"),
                                       (N.PIVOT_EXACT, "nativeklu_exact")])
def test_nan_rhs_propagates_as_in_the_oracle(mode, kind):
    c = cz.inverter_chain(40, 0.7)
    n, ap, ai, ax, rhs = po.mna(c, wl.chain_nodeset(40, 0.7))
    rhs = rhs.copy()
    rhs[n // 3] = np.nan
    g = GpuKluSolver(n, pivot_mode=mode)
    xg = _factor_solve(g, ap, ai, ax, rhs)
    o = po.Solver(kind, n)
    o.prepare(n)
    o.analyze(ap, ai)
    o.factor(ap, ai, ax)
    st, xo = o.solve(rhs)
    assert st == 0
    assert np.isnan(xg).any()
    assert np.array_equal(np.isnan(xg), np.isnan(xo))
    assert np.array_equal(xg[~np.isnan(xg)], xo[~np.isnan(xo)])


def _singular_system():
    """Block-diagonal 7x7: a singular 2x2 block [[1, 1], [1, 1]], a singleton
    stored as an explicit zero, and a regular 4x4 block."""
    A = np.zeros((7, 7))
    A[0:2, 0:2] = 1.0
    A[3:7, 3:7] = np.array([[4.0, 1, 0, 1], [1, 5, 2, 0], [0, 2, 6, 1], [1, 0, 1, 7]])
    ap = [0]
    ai = []
    ax = []
    for j in range(7):
        for i in range(7):
            if A[i, j] != 0.0 or (i == j == 2):
                ai.append(i)
                ax.append(A[i, j])
        ap.append(len(ai))
    return (7, np.array(ap, np.int64), np.array(ai, np.int64), np.array(ax),
            np.arange(1.0, 8.0))


@pytest.mark.parametrize("mode,kind", [(N.PIVOT_REFERENCE, "nativeklu"),
                                       (N.PIVOT_EXACT, "nativeklu_exact")])
def test_singular_blocks_perturbed_as_the_reference(mode, kind):
    n, ap, ai, ax, rhs = _singular_system()
    g = GpuKluSolver(n, pivot_mode=mode)
    xg = _factor_solve(g, ap, ai, ax, rhs)
    o = po.Solver(kind, n)
    o.prepare(n)
    o.analyze(ap, ai)
    assert o.factor(ap, ai, ax) == 0
    st, xo = o.solve(rhs)
    assert st == 0
    assert np.array_equal(xg, xo)
    # the perturbed pivots give solutions of order 1e14
    assert np.max(np.abs(xg)) > 1e13
    assert g.stats()["rcond"] == o.klu_stats()["rcond"]
