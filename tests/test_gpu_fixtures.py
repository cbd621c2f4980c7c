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
from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, SolverError, newton_dc

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


SPARSE_KINDS = ["sparselu", "sparselubtf"]


@pytest.mark.parametrize("kind", SPARSE_KINDS)
def test_sparselu_kinds_kats_and_mesh(kind, kernels):
    """The device handle as the reference's SparseLuSolver and
    SparseLuBtfSolver (no row exchanges, the +-1e-14 pivot rule in every
    block, SparseLU-BTF's BTF rule): bit for bit the oracle's, on the solver
    known answers and on the 32x32 diode mesh across a refactorization."""
    for k in KATS["solve"]:
        n = len(k["ap"]) - 1
        g = GpuKluSolver(n, kind=kind)
        x = _gpu_solve(g, k["ap"], k["ai"], k["ax"], k["b"])
        _, xo = _oracle_solve(kind, k["ap"], k["ai"], k["ax"], k["b"])
        assert np.array_equal(x, xo), k["name"]
        assert g.name() == ("GpuSparseLU" if kind == "sparselu" else "GpuSparseLU-BTF")
        g.close()
    c = cz.mesh_dc()
    n, ap, ai, ax, rhs = po.mna(c, np.random.default_rng(11).uniform(0, 0.8, c.node_count))
    g = GpuKluSolver(n, kind=kind)
    s = po.Solver(kind, n)
    s.prepare(n)
    ax2 = ax * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(len(ax)))
    for a in (ax, ax2):
        x = _gpu_solve(g, ap, ai, a, rhs)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert np.array_equal(x, xo), np.max(np.abs(x - xo))
    assert g.stats()["pivot_swaps"] == 0
    g.close()


@pytest.mark.parametrize("kind", SPARSE_KINDS)
@pytest.mark.parametrize("name", ["adder_dcop_01", "circuit_1", "rajat01"])
def test_sparselu_kinds_matrix_market(name, kind, kernels):
    z = np.load(os.path.join(GOLD, f"mtx_{name}.npz"))
    ap, ai, ax, rhs = z["ap"].astype(np.int64), z["ai"].astype(np.int64), z["ax"], z["rhs"]
    n = len(ap) - 1
    g = GpuKluSolver(n, kind=kind)
    s = po.Solver(kind, n)
    s.prepare(n)
    ax2 = ax * (1.0 + 1e-3 * np.random.default_rng(1).standard_normal(len(ax)))
    for a in (ax, ax2):
        x = _gpu_solve(g, ap, ai, a, rhs)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert np.array_equal(x, xo), np.max(np.abs(x - xo))
    g.close()


@pytest.mark.parametrize("kind", SPARSE_KINDS)
def test_sparselu_kinds_newton(kind):
    """The engine's DC loop on the device with the SparseLU kinds: the
    reference's iterations and operating point (the divider's known answer,
    the 32x32 diode mesh with gmin stepping)."""
    d = KATS["divider"]
    div = cz.Circuit(d["node_count"], np.array(d["type"], np.int32),
                     np.array(d["nodes"], np.int32), np.array(d["p"], np.float64))
    for c, extra in ((div, {}), (cz.mesh_dc(), {"gmin_steps": 10})):
        cfg = dict(wl.TIGHT, **extra)
        ocfg = {k: cfg[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps",
                                    "source_steps")}
        g = GpuKluSolver(1, kind=kind)
        r = newton_dc(g, DeviceCircuit(c), N.newton_config(**cfg))
        ro, ito, xo = po.dc_op(c, kind, **ocfg)
        assert r.reason == ro and r.iterations == ito
        assert np.max(np.abs(r.x - xo)) <= 1e-10 * np.max(np.abs(xo))
        g.close()


def test_dense_kind_matches_the_reference_dense_solver():
    """The device DenseSolver (solver.rs:596-724) bit for bit against the
    oracle's restatement: the known answers, small inverter chains, the
    32x32 diode mesh (n = 1026) across new values, and its failure paths."""
    from rustspice_gb300.solver import create_solver_auto, create_solver_for_matrix
    for k in KATS["solve"]:
        n = len(k["ap"]) - 1
        g = GpuKluSolver(n, kind="dense")
        x = _gpu_solve(g, k["ap"], k["ai"], k["ax"], k["b"])
        _, xo = _oracle_solve("dense", k["ap"], k["ai"], k["ax"], k["b"])
        assert np.array_equal(x, xo), k["name"]
        g.close()
    systems = [po.mna(cz.inverter_chain(s, v), wl.chain_nodeset(s, v)) for s, v in
               [(8, 0.3), (40, 0.7)]]
    c = cz.mesh_dc()
    systems.append(po.mna(c, np.random.default_rng(11).uniform(0, 0.8, c.node_count)))
    for n, ap, ai, ax, rhs in systems:
        g = GpuKluSolver(n, kind="dense")
        s = po.Solver("dense", n)
        s.prepare(n)
        for a in (ax, ax * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(len(ax)))):
            x = _gpu_solve(g, ap, ai, a, rhs)
            assert s.factor(ap, ai, a) == 0
            st, xo = s.solve(rhs)
            assert st == 0 and np.array_equal(x, xo), (n, np.max(np.abs(x - xo)))
        assert g.name() == "GpuDense"
        g.close()
    # a column without a nonzero candidate fails the factorization
    # (solver_tests.rs singular case: diag(1, 0, 1))
    g = GpuKluSolver(3, kind="dense")
    with pytest.raises(SolverError) as e:
        g.factor([0, 1, 2, 3], [0, 1, 2], [1.0, 0.0, 1.0])
    assert e.value.status == N.FACTOR_FAILED
    assert po.Solver("dense", 3).factor([0, 1, 2, 3], [0, 1, 2], [1.0, 0.0, 1.0]) == 2
    with pytest.raises(SolverError) as e:  # solve before a successful factorization
        g.solve(np.ones(3))
    assert e.value.status == N.SOLVE_FAILED
    g.factor([0, 1, 2, 3], [0, 1, 2], [1.0, 2.0, 4.0])
    with pytest.raises(SolverError) as e:  # wrong length: SolveFailed (solver.rs:689-691)
        g.solve(np.ones(4))
    assert e.value.status == N.SOLVE_FAILED
    g.analyze([0, 1], [0])  # analyze accepts any pattern
    with pytest.raises(SolverError) as e:
        g.factor([0, 1], [0], [1.0])
    assert e.value.status == N.ANALYZE_FAILED
    g.close()
    # the factory: auto picks Dense for 10 unknowns; the matrix selector's
    # example system (solver_tests.rs:95-110)
    a = create_solver_auto(10)
    assert a.name() == "GpuDense"
    a.close()
    m = create_solver_for_matrix(2, [0, 2, 4], [0, 1, 0, 1])
    m.prepare(2)
    m.analyze([0, 2, 4], [0, 1, 0, 1])
    m.factor([0, 2, 4], [0, 1, 0, 1], [3.0, 1.0, 1.0, 2.0])
    x = np.array([9.0, 8.0])
    m.solve(x)
    assert np.max(np.abs(x - [2.0, 3.0])) < 1e-9


@pytest.mark.parametrize("solver", ["dense", "auto", "sparselubtf", "nativeklu"])
def test_deck_solver_option_on_the_device(solver):
    """`.option solver=` picks the device solver kind as the engine picks its
    solver (engine.rs:971-984, solver.rs:169-246, by node count); the device
    Newton loop then gives the oracle's iterations and operating point with
    the same solver."""
    from rustspice_gb300 import netlist as nl
    deck = nl.compile_deck(f"""* divider with a diode
V1 in 0 1.0
R1 in out 1k
R2 out 0 2k
D1 out 0 dmod
.model dmod d is=1e-14 n=1
.option solver={solver} reltol=1e-10 vntol=1e-12 itl1=200
.end
""")
    kind = deck.solver_kind()
    assert kind == {"dense": "dense", "auto": "dense", "sparselubtf": "sparselubtf",
                    "nativeklu": "nativeklu"}[solver]
    opts = deck.newton_options()
    g = GpuKluSolver(1, kind=kind)
    r = newton_dc(g, DeviceCircuit(deck.circuit), N.newton_config(**opts))
    ro, ito, xo = po.dc_op(deck.circuit, kind, **opts)
    # NativeKLU's pivot rule drops entries on this deck and stalls at the cap
    # (the reference's Q6 behaviour); the others converge
    assert r.reason == ro and r.iterations == ito
    assert r.converged == (kind != "nativeklu")
    if r.converged:
        assert np.max(np.abs(r.x - xo)) <= 1e-12 * np.max(np.abs(xo))
    g.close()
