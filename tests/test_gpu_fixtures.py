"""The GPU solver on the reference's own fixtures (golden files).

Known-answer systems, the three Matrix Market matrices and the BeGAN power
grid go through GpuKluSolver / the device stamp and Newton path; the solver
results are compared with the oracle bit for bit (same algorithm, same
operation order), the stamps entry by entry.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, newton_dc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KATS = json.load(open(os.path.join(GOLD, "kats.json")))
MODES = [(N.PIVOT_REFERENCE, "nativeklu"), (N.PIVOT_EXACT, "nativeklu_exact")]


@pytest.fixture(params=["one_block", "grid"])
def kernels(request, monkeypatch):
    """Small factorizations refactor and solve in one thread block; "grid"
    switches that off so the grid-wide flag kernels run the same systems."""
    monkeypatch.setenv("GPUKLU_ONE_BLOCK", "1" if request.param == "one_block" else "0")
    return request.param


def _gpu_solve(g, ap, ai, ax, b):
    g.factor(ap, ai, ax)
    x = np.ascontiguousarray(b, np.float64).copy()
    g.solve(x)
    return x


def _oracle_solve(kind, ap, ai, ax, b):
    n = len(ap) - 1
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.factor(ap, ai, ax) == 0
    st, x = s.solve(b)
    assert st == 0
    return s, x


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_pivot_pass_refactorizations(mode, kind, kernels, monkeypatch):
    """The first factorization's pivot pass run as checked refactorizations
    (the default) and as the sequential one-warp kernel give the same
    pivots and factor: solutions equal bit for bit and equal to the
    oracle's, the same swap count, and the number of passes the CPU
    restatement of the host loop predicts. A second first factorization of
    the same pattern starts from the pivots found and settles in one pass."""
    from plan_emulator import staged_first_factor
    from test_plan_parity import PIVOT_SYSTEMS
    for name, ap, ai, ax in PIVOT_SYSTEMS:
        n = len(ap) - 1
        b = np.random.default_rng(n).uniform(-1, 1, n)
        r = staged_first_factor(N.Plan(n, ap, ai, mode), ax)
        expect = r[2] if r is not None else 0
        got = {}
        for pp in ("refactor", "sequential"):
            monkeypatch.setenv("GPUKLU_PIVOT_PASS", pp)
            g = GpuKluSolver(n, pivot_mode=mode)
            x = _gpu_solve(g, ap, ai, ax, b)
            got[pp] = (x, g.stats()["pivot_swaps"], g.pivot_passes())
            if pp == "refactor" and expect > 0:
                g.reset_pattern()
                x2 = _gpu_solve(g, ap, ai, ax, b)
                assert np.array_equal(x2, x) and g.pivot_passes() == 1, name
        _, xo = _oracle_solve(kind, ap, ai, ax, b)
        assert np.array_equal(got["refactor"][0], got["sequential"][0]), name
        assert np.array_equal(got["refactor"][0], xo), name
        assert got["refactor"][1] == got["sequential"][1], name
        assert got["sequential"][2] == 0 and got["refactor"][2] == expect, (name, got["refactor"][2])


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_grouped_one_block_solve(mode, kind, monkeypatch):
    """The one-block solve split over thread blocks (one per group of
    uncoupled BTF blocks), forced on systems whose whole plan would also fit
    one block: solutions equal to the oracle's bit for bit."""
    from test_plan_parity import GROUP_SYSTEMS
    monkeypatch.setenv("GPUKLU_SOLVE_GROUPS", "1")
    for name, ap, ai, ax, b in GROUP_SYSTEMS:
        n = len(ap) - 1
        g = GpuKluSolver(n, pivot_mode=mode)
        x = _gpu_solve(g, ap, ai, ax, b)
        _, xo = _oracle_solve(kind, ap, ai, ax, b)
        assert np.array_equal(x, xo), name
        ax2 = ax * (1.0 + 0.05 * np.random.default_rng(1).standard_normal(len(ax)))
        x = _gpu_solve(g, ap, ai, ax2, b)  # a refactorization, then the solve again
        s, _ = _oracle_solve(kind, ap, ai, ax, b)
        assert s.factor(ap, ai, ax2) == 0
        st, xo = s.solve(b)
        assert st == 0 and np.array_equal(x, xo), name


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_kats(mode, kind, kernels):
    for k in KATS["solve"]:
        n = len(k["ap"]) - 1
        g = GpuKluSolver(n, pivot_mode=mode)
        x = _gpu_solve(g, k["ap"], k["ai"], k["ax"], k["b"])
        _, xo = _oracle_solve(kind, k["ap"], k["ai"], k["ax"], k["b"])
        assert np.array_equal(x, xo), k["name"]
        if k["x"] is not None:
            assert np.max(np.abs(x - np.asarray(k["x"]))) < k["tol"], k["name"]
        g.close()


def test_refactor_counters_and_rcond():
    k = KATS["refactor"]
    g = GpuKluSolver(3)
    x1 = _gpu_solve(g, k["ap"], k["ai"], k["ax1"], k["b1"])
    st = g.stats()
    assert [st["factor_count"], st["refactor_count"]] == k["counts1"]
    x2 = _gpu_solve(g, k["ap"], k["ai"], k["ax2"], k["b2"])
    st = g.stats()
    assert [st["factor_count"], st["refactor_count"]] == k["counts2"]
    assert np.max(np.abs(x1 - x2)) < 1e-9
    r = KATS["rcond"]
    g2 = GpuKluSolver(3)
    g2.factor(r["ap"], r["ai"], r["ax_id"])
    assert abs(g2.stats()["rcond"] - 1.0) < 1e-10
    g2.factor(r["ap"], r["ai"], r["ax_ill"])
    assert g2.stats()["rcond"] < 1e-10


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
@pytest.mark.parametrize("name", ["adder_dcop_01", "circuit_1", "rajat01"])
def test_matrix_market_bit_exact(name, mode, kind, kernels):
    z = np.load(os.path.join(GOLD, f"mtx_{name}.npz"))
    ap, ai, ax, rhs = z["ap"].astype(np.int64), z["ai"].astype(np.int64), z["ax"], z["rhs"]
    n = len(ap) - 1
    g = GpuKluSolver(n, pivot_mode=mode)
    s = po.Solver(kind, n)
    s.prepare(n)
    ax2 = ax * (1.0 + 1e-3 * np.random.default_rng(1).standard_normal(len(ax)))
    for a in (ax, ax2):  # first factor, then a refactor on frozen pivots
        x = _gpu_solve(g, ap, ai, a, rhs)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert np.array_equal(x, xo), np.max(np.abs(x - xo))
    assert g.stats()["nblocks"] == s.klu_stats()["nblocks"]


@pytest.mark.parametrize("k", KATS["stamps"], ids=lambda k: k["name"])
def test_device_stamp_kats(k):
    t, a, b, p0, p1 = k["dev"]
    c = cz.Circuit(k["node_count"], np.array([t], np.int32), np.array([[a, b, 0, 0]], np.int32),
                   np.array([[p0, p1, 0, 0, 0, 0]], np.float64))
    g = GpuKluSolver(1)
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    ax, rhs = dc.stamp(g, np.asarray(k["x"], np.float64), gmin=k["gmin"], source_scale=k["scale"])
    A = sp.csc_matrix((ax, ai, ap), shape=(dc.n, dc.n)).toarray()
    for r, col, v in k.get("entries", []):
        pin = 1.0 if (r, col) == (0, 0) else 0.0
        assert abs(A[r, col] - (v + pin)) <= 1e-16 * (1.0 + pin)
    if "rhs" in k:
        assert np.allclose(rhs, k["rhs"], rtol=0, atol=1e-12)


def test_divider_and_began_newton():
    d = KATS["divider"]
    div = cz.Circuit(d["node_count"], np.array(d["type"], np.int32),
                     np.array(d["nodes"], np.int32), np.array(d["p"], np.float64))
    z = np.load(os.path.join(GOLD, "began_small_pgrid.npz"))
    grid = cz.Circuit(int(z["node_count"]), z["type"], z["nodes"], z["p"])
    cfg = dict(wl.TIGHT)
    ocfg = {k: cfg[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps",
                                "source_steps")}
    for c in (div, grid):
        g = GpuKluSolver(1)
        r = newton_dc(g, DeviceCircuit(c), N.newton_config(**cfg))
        ro, ito, xo = po.dc_op(c, "nativeklu", **ocfg)
        assert r.converged and ro == "converged" and r.iterations == ito
        assert np.max(np.abs(r.x - xo)) <= 1e-12 * np.max(np.abs(xo))
    g = GpuKluSolver(1)
    r = newton_dc(g, DeviceCircuit(div), N.newton_config(**cfg))
    for node, v in d["expect"].items():
        assert abs(r.x[int(node)] - v) < d["tol"]


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_mesh_solve_both_kernel_sets(mode, kind, kernels):
    """The 32x32 diode mesh (a dense 300-row separator at the end of its
    ordering; the one-block solve streams it in 13 chunks per sweep) solves
    bit for bit like the oracle with either kernel set, across a refactor."""
    c = cz.mesh_dc()
    n, ap, ai, ax, rhs = po.mna(c, np.random.default_rng(11).uniform(0, 0.8, c.node_count))
    g = GpuKluSolver(n, pivot_mode=mode)
    s = po.Solver(kind, n)
    s.prepare(n)
    ax2 = ax * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(len(ax)))
    for a in (ax, ax2):
        x = _gpu_solve(g, ap, ai, a, rhs)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert np.array_equal(x, xo), np.max(np.abs(x - xo))
    g.close()
