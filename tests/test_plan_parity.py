"""The library's host analysis against the oracle, without a GPU.

``plan_emulator`` runs the device kernels' exact operation sequence (first
factor with the reference pivot rule, frozen-pivot refactor, block solves)
over the integer plan that libgpuklu builds. Identical results to the
oracle's NativeKLU, bit for bit, in both pivot modes and across a refactor
with new values, show that the plan (BTF and AMD orderings, symbolic
patterns, slot maps, update lists, block coupling) is the reference's.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from plan_emulator import (SOLVE_CHUNK, EmulatedSolver, first_factor, solve_groups,
                            solve_one_block, staged_first_factor)
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MODES = [(N.PIVOT_REFERENCE, "nativeklu"), (N.PIVOT_EXACT, "nativeklu_exact")]


def _systems():
    out = []
    for k in json.load(open(os.path.join(GOLD, "kats.json")))["solve"]:
        out.append((k["name"], np.array(k["ap"], np.int64), np.array(k["ai"], np.int64),
                    np.array(k["ax"]), np.array(k["b"])))
    for name, c, seed in [("mesh12", cz.mesh_dc(side=12, ndiodes=10, seed=2), 0),
                          ("chain8", cz.inverter_chain(8, 0.3), 1),
                          ("chain40", cz.inverter_chain(40, 0.7), 2),
                          ("ring11", cz.ring_oscillator(11), 3)]:
        x = np.random.default_rng(seed).uniform(0, 1.2, c.node_count)
        transient = name.startswith("ring")
        n, ap, ai, ax, rhs = po.mna(c, x, dt=1e-12 if transient else 0.0,
                                    cap_v=np.zeros(c.ndev) if transient else None)
        out.append((name, ap, ai, ax, rhs))
    z = np.load(os.path.join(GOLD, "mtx_adder_dcop_01.npz"))
    out.append(("adder_dcop_01", z["ap"].astype(np.int64), z["ai"].astype(np.int64), z["ax"],
                z["rhs"]))
    return out


SYSTEMS = _systems()


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
@pytest.mark.parametrize("sysm", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_plan_emulation_bit_exact(sysm, mode, kind):
    name, ap, ai, ax, rhs = sysm
    n = len(ap) - 1
    ax2 = ax * (1.0 + 0.1 * np.random.default_rng(7).standard_normal(len(ax)))
    es = EmulatedSolver(mode)
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    for a in (ax, ax2):  # first factor, then a refactor with frozen pivots
        es.factor(n, ap, ai, a)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert st == 0
        xe = es.solve(rhs)
        assert np.array_equal(xe, xo), np.max(np.abs(xe - xo))
        xb = solve_one_block(es.plan, es.ax, es.lu, rhs)  # column sweeps, chunked
        assert np.array_equal(xb, xo), np.max(np.abs(xb - xo))
    st = s.klu_stats()
    assert es.plan.nblocks == st["nblocks"]
    if mode == N.PIVOT_REFERENCE:  # the pattern of the pivot-free symbolic pass
        assert es.plan.nnz_l == st["nnz_l"]


KINDS = ["sparselu", "sparselubtf"]
KIND_SYSTEMS = SYSTEMS + [("chain120", *po.mna(cz.inverter_chain(120, 0.4),
                                                np.random.default_rng(4).uniform(
                                                    0, 1.2, cz.inverter_chain(120, 0.4)
                                                    .node_count))[1:])]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("sysm", KIND_SYSTEMS, ids=[s[0] for s in KIND_SYSTEMS])
def test_plan_emulation_sparselu_kinds(sysm, kind):
    """The plan of the SparseLU kinds (no row exchanges, the general pivot
    perturbation in every block, SparseLU-BTF's BTF rule) run through the
    kernels' operation sequence equals the oracle's SparseLuSolver and
    SparseLuBtfSolver bit for bit, across a refactorization with new values."""
    name, ap, ai, ax, rhs = sysm
    n = len(ap) - 1
    ax2 = ax * (1.0 + 0.1 * np.random.default_rng(7).standard_normal(len(ax)))
    es = EmulatedSolver(N.PIVOT_REFERENCE, kind)
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    for a in (ax, ax2):
        es.factor(n, ap, ai, a)
        assert s.factor(ap, ai, a) == 0
        st, xo = s.solve(rhs)
        assert st == 0
        xe = es.solve(rhs)
        assert np.array_equal(xe, xo), np.max(np.abs(xe - xo))
        xb = solve_one_block(es.plan, es.ax, es.lu, rhs)
        assert np.array_equal(xb, xo), np.max(np.abs(xb - xo))
    assert es.plan.swaps == 0
    if kind == "sparselu" or n < 50:
        assert es.plan.nblocks == 1


def _weak_diagonal(n, seed):
    """Random sparse matrix whose diagonal is often far below its column:
    the threshold rule exchanges many rows, in chains."""
    rng = np.random.default_rng(seed)
    a = (rng.random((n, n)) < 0.12) * rng.uniform(-1, 1, (n, n))
    d = rng.uniform(-1, 1, n) * np.where(rng.random(n) < 0.4, 1e-5, 1.0)
    a[np.arange(n), np.arange(n)] = d
    ap = np.zeros(n + 1, np.int64)
    ai, ax = [], []
    for c in range(n):
        r = np.nonzero(a[:, c])[0]
        ai.extend(r)
        ax.extend(a[r, c])
        ap[c + 1] = len(ai)
    return ap, np.array(ai, np.int64), np.array(ax)


PIVOT_SYSTEMS = [(s[0], s[1], s[2], s[3]) for s in SYSTEMS] + [
    (f"weak_diag_{seed}", *_weak_diagonal(60, seed)) for seed in range(4)]


@pytest.mark.parametrize("mode", [N.PIVOT_REFERENCE, N.PIVOT_EXACT], ids=["reference", "exact"])
@pytest.mark.parametrize("sysm", PIVOT_SYSTEMS, ids=[s[0] for s in PIVOT_SYSTEMS])
def test_pivot_pass_as_refactorizations(sysm, mode):
    """The first factorization's pivot pass restated as refactorizations of
    the pivot-free pattern that check the threshold rule on every column (the
    host loop and the refactor kernel's pivot-pass mode) gives the sequential
    pass's pivots and factor bit for bit, with and without row exchanges."""
    name, ap, ai, ax = sysm
    n = len(ap) - 1
    P = N.Plan(n, ap, ai, mode)
    for a in (ax, ax * (1.0 + 0.1 * np.random.default_rng(7).standard_normal(len(ax)))):
        lu, rperm = first_factor(P, a)
        r = staged_first_factor(P, a, max_passes=n + 1)
        assert r is not None
        lu2, rperm2, passes, found = r
        assert np.array_equal(rperm2, rperm)
        assert np.array_equal(lu2, lu), np.max(np.abs(lu2 - lu))
        assert passes <= n + 1
        swaps = int(np.sum(rperm != np.arange(n) - P.block_ptr[P.pos_block]))
        assert (passes == 1) == (swaps == 0)
        # a start from the sequence found settles in one pass; a start from
        # arbitrary L slots still ends at the same pivots and factor
        r = staged_first_factor(P, a, max_passes=1, start=found)
        assert r is not None and np.array_equal(r[0], lu) and np.array_equal(r[1], rperm)
        rng = np.random.default_rng(n)
        junk = np.full(n, -1, np.int64)
        for k in range(n):
            if P.col_ptr[k + 1] > P.dslot[k] + 1 and rng.random() < 0.3:
                junk[k] = rng.integers(P.dslot[k] + 1, P.col_ptr[k + 1])
        r = staged_first_factor(P, a, max_passes=n + 2, start=junk)
        assert r is not None and np.array_equal(r[0], lu) and np.array_equal(r[1], rperm)


def test_mesh_dimensions():
    """32x32 diode mesh: n = 1026 and 8,201 raw CSC entries (duplicates kept,
    as the engine's finalize() keeps them: crates/sim-core/src/mna.rs:320-347)."""
    c = cz.mesh_dc()
    n, ap, ai, ax, rhs = po.mna(c, np.zeros(c.node_count))
    assert n == 1026 and len(ai) == 8201


def _star(n, seed):
    """A hub coupled to every other node: after ordering the hub's column holds
    n slots, more than one chunk of the one-block solve."""
    rng = np.random.default_rng(seed)
    cols = []
    for c in range(n):
        if c == 0:
            rows = list(range(n))
        else:
            rows = [0, c]
        cols.append(rows)
    ap = np.zeros(n + 1, np.int64)
    ap[1:] = np.cumsum([len(r) for r in cols])
    ai = np.concatenate([np.array(r, np.int64) for r in cols])
    ax = np.where(np.repeat(np.arange(n), [len(r) for r in cols]) == ai,
                  float(n) + rng.uniform(1, 2, len(ai)), rng.uniform(-1, 1, len(ai)))
    return ap, ai, ax, rng.uniform(-1, 1, n)


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_one_block_solve_direct_column(mode, kind):
    """A column longer than a chunk is read straight from memory; the result
    stays the oracle's bit for bit."""
    n = SOLVE_CHUNK + 300
    ap, ai, ax, rhs = _star(n, 5)
    es = EmulatedSolver(mode)
    es.factor(n, ap, ai, ax)
    op = es.plan.cs_op.reshape(-1, 3)
    assert np.any(op[:, 0] & 4), "expected a direct piece"
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    assert s.factor(ap, ai, ax) == 0
    st, xo = s.solve(rhs)
    assert st == 0
    xb = solve_one_block(es.plan, es.ax, es.lu, rhs)
    assert np.array_equal(xb, xo)


def _disjoint_meshes(sides, seed):
    """Block-diagonal MNA system of independent diode meshes (BTF finds one
    block per mesh, with no coupling between them)."""
    rng = np.random.default_rng(seed)
    aps, ais, axs, rhss, off = [], [], [], [], 0
    for side in sides:
        c = cz.mesh_dc(side=side, ndiodes=side, seed=int(rng.integers(1000)))
        n, ap, ai, ax, rhs = po.mna(c, rng.uniform(0, 0.7, c.node_count))
        aps.append(ap[1:] + (aps[-1][-1] if aps else 0))
        ais.append(ai + off)
        axs.append(ax)
        rhss.append(rhs)
        off += n
    ap = np.concatenate([[0], *aps]).astype(np.int64)
    return ap, np.concatenate(ais), np.concatenate(axs), np.concatenate(rhss)


GROUP_SYSTEMS = [s for s in SYSTEMS if s[0] in ("block_diagonal_4", "chain8", "chain40",
                                                 "adder_dcop_01")]
GROUP_SYSTEMS.append(("meshes", *_disjoint_meshes([6, 9, 4, 12, 7, 5, 10], 3)))


def _two_stars(n, seed):
    """Two independent hub systems of n rows each: every group holds a column
    longer than a chunk (a direct piece read straight from memory)."""
    ap1, ai1, ax1, b1 = _star(n, seed)
    ap2, ai2, ax2, b2 = _star(n, seed + 1)
    ap = np.concatenate([ap1, ap2[1:] + ap1[-1]])
    return ap, np.concatenate([ai1, ai2 + n]), np.concatenate([ax1, ax2]), np.concatenate([b1, b2])


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
def test_grouped_solve_direct_columns(mode, kind):
    """Groups whose blocks hold a column longer than a chunk: the direct
    pieces stay inside their group and the result is the oracle's."""
    n = SOLVE_CHUNK + 300
    ap, ai, ax, rhs = _two_stars(n, 5)
    es = EmulatedSolver(mode)
    es.factor(2 * n, ap, ai, ax)
    P = es.plan
    assert len(P.cs_grp) // 4 == 2 and np.any(P.cs_gop.reshape(-1, 3)[:, 0] & 4)
    xg = solve_groups(P, es.ax, es.lu, rhs)
    s = po.Solver(kind, 2 * n)
    s.prepare(2 * n)
    assert s.factor(ap, ai, ax) == 0
    st, xo = s.solve(rhs)
    assert st == 0 and np.array_equal(xg, xo)


@pytest.mark.parametrize("mode,kind", MODES, ids=["reference", "exact"])
@pytest.mark.parametrize("sysm", GROUP_SYSTEMS, ids=[s[0] for s in GROUP_SYSTEMS])
def test_grouped_one_block_solve(sysm, mode, kind):
    """The one-block solve split over thread blocks, one per group of
    uncoupled BTF blocks: the groups' schedules stay inside their rows, and
    the result is the row-ordered solve's (and the oracle's) bit for bit."""
    name, ap, ai, ax, rhs = sysm
    n = len(ap) - 1
    es = EmulatedSolver(mode)
    es.factor(n, ap, ai, ax)
    P = es.plan
    if len(P.cs_grp) == 0:  # the exact mode keeps BTF coupling: no groups
        assert P.noffdiag > 0 and mode == N.PIVOT_EXACT
        return
    assert P.noffdiag == 0 and len(P.cs_grp) // 4 >= 2
    xg = solve_groups(P, es.ax, es.lu, rhs)
    assert np.array_equal(xg, es.solve(rhs))
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.factor(ap, ai, ax) == 0
    st, xo = s.solve(rhs)
    assert st == 0 and np.array_equal(xg, xo)


def test_one_block_schedule_mesh():
    """The 32x32 diode mesh's schedule: several chunks, each within the
    buffer, and the sweeps bit-identical to the oracle's solve."""
    c = cz.mesh_dc()
    x = np.random.default_rng(4).uniform(0, 1.2, c.node_count)
    n, ap, ai, ax, rhs = po.mna(c, x)
    es = EmulatedSolver(N.PIVOT_EXACT)
    es.factor(n, ap, ai, ax)
    ch = es.plan.cs_chunk.reshape(-1, 4)
    assert ch.shape[0] > 4 and np.all(ch[:, 1] - ch[:, 0] <= SOLVE_CHUNK)
    s = po.Solver("nativeklu_exact", n)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    assert s.factor(ap, ai, ax) == 0
    st, xo = s.solve(rhs)
    assert st == 0
    assert np.array_equal(solve_one_block(es.plan, es.ax, es.lu, rhs), xo)


def _block_diagonal(nblocks, seed):
    """Independent meshes side by side: a factor with no block coupling."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(nblocks):
        m = int(rng.integers(3, 9))
        g = sp.random(m * m, m * m, density=0.05, random_state=int(rng.integers(1 << 30)))
        a = (g + g.T + sp.eye(m * m) * (m * m)).tocsc()
        mats.append(a)
    a = sp.block_diag(mats).tocsc()
    a.sort_indices()
    return a.shape[0], a.indptr.astype(np.int64), a.indices.astype(np.int64), a.data


@pytest.mark.parametrize("seed", [0, 1])
def test_grid_solve_task_order(seed):
    """Every task of the grid solve comes after the tasks it waits for (the
    dependency-flag kernels rely on it to finish), also when the tasks of
    independent blocks interleave."""
    n, ap, ai, ax = _block_diagonal(6, seed)
    for mode in (N.PIVOT_REFERENCE, N.PIVOT_EXACT):
        P = N.Plan(n, ap, ai, mode)
        assert P.nblocks > 1
        for name in ("task", "ttask"):
            t = getattr(P, name)
            assert len(t) == 2 * n and sorted(t) == list(range(2 * n))
            pos = np.empty(2 * n, np.int64)
            pos[t] = np.arange(2 * n)
            fwd, bwd = pos[0::2], pos[1::2]  # by plan position
            assert np.all(bwd > fwd)
            lower = name == "task"
            for i in range(n):
                if lower:  # L row i needs z of its columns; U row i needs x of its columns
                    deps_f = P.lrow_col[P.lrow_ptr[i]:P.lrow_ptr[i + 1]]
                    deps_b = P.urow_col[P.urow_ptr[i]:P.urow_ptr[i + 1]]
                else:  # transpose: U column i, then L column i
                    s0, ds, s1 = P.col_ptr[i], P.dslot[i], P.col_ptr[i + 1]
                    deps_f = P.slot_row[s0:ds]
                    deps_b = P.slot_row[ds + 1:s1]
                assert np.all(fwd[deps_f] < fwd[i])
                assert np.all(bwd[deps_b] < bwd[i])
        # and the interleaved order still solves bit for bit like the oracle
        es = EmulatedSolver(mode)
        es.factor(n, ap, ai, ax)
        rhs = np.random.default_rng(seed).standard_normal(n)
        s = po.Solver("nativeklu" if mode == N.PIVOT_REFERENCE else "nativeklu_exact", n)
        s.prepare(n)
        assert s.analyze(ap, ai) == 0 and s.factor(ap, ai, ax) == 0
        st, xo = s.solve(rhs)
        assert st == 0 and np.array_equal(es.solve(rhs), xo)
