"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Factor and solve results are compared bit for bit where the arithmetic is the
same (both compile without multiply-add contraction and follow the
reference's operation order); device stamps of diodes use CUDA's exp, so
those are compared to 1e-14 relative. Newton results use the required
tolerance: relative solution error <= 1e-10.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import Batch, DeviceCircuit, GpuKluSolver, SolverError, newton_dc

pytestmark = pytest.mark.gpu

MODES = [(N.PIVOT_REFERENCE, "nativeklu"), (N.PIVOT_EXACT, "nativeklu_exact")]


def _systems():
    out = []
    c = cz.mesh_dc()
    out.append(("mesh32", po.mna(c, np.zeros(c.node_count))))
    for s, v in [(8, 0.3), (40, 0.7), (256, 0.55)]:
        c = cz.inverter_chain(s, v)
        out.append((f"chain{s}", po.mna(c, wl.chain_nodeset(s, v))))
    return out


def _block_lower(n=300, seed=0):
    """Random diagonally dominant matrix in block lower triangular form with
    shuffled rows/columns, so BTF finds many blocks and coupling entries."""
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    b0 = 0
    while b0 < n:
        bs = int(rng.integers(1, 9))
        b1 = min(n, b0 + bs)
        A[b0:b1, b0:b1] = rng.standard_normal((b1 - b0, b1 - b0)) * (rng.random((b1 - b0, b1 - b0)) < 0.6)
        b0 = b1
    A += np.tril(rng.standard_normal((n, n)) * (rng.random((n, n)) < 0.01), -8)
    A[np.arange(n), np.arange(n)] += 5.0
    p = rng.permutation(n)
    q = rng.permutation(n)
    A = A[p][:, q]
    M = sp.csc_matrix(A)
    M.sort_indices()
    return n, M.indptr.astype(np.int64), M.indices.astype(np.int64), M.data.copy(), rng.standard_normal(n)


@pytest.mark.parametrize("mode,kind", MODES)
def test_factor_solve_bitexact(mode, kind):
    for name, (n, ap, ai, ax, rhs) in _systems() + [("blocklower", _block_lower())]:
        g = GpuKluSolver(n, pivot_mode=mode)
        o = po.Solver(kind, n)
        o.prepare(n)
        g.prepare(n)
        rng = np.random.default_rng(1)
        for it, a in enumerate([ax, ax * (1 + 0.05 * rng.standard_normal(len(ax))), ax]):
            g.analyze(ap, ai)
            assert o.analyze(ap, ai) == 0
            g.factor(ap, ai, a)
            assert o.factor(ap, ai, a) == 0
            xg = rhs.copy()
            g.solve(xg)
            st, xo = o.solve(rhs)
            assert st == 0
            assert np.array_equal(xg, xo), (name, kind, it, np.max(np.abs(xg - xo)))
        s = g.stats()
        ks = o.klu_stats()
        assert s["factor_count"] == 1 and s["refactor_count"] == 2
        assert s["nblocks"] == ks["nblocks"]
        if mode == N.PIVOT_REFERENCE:
            assert (s["nnz_l"], s["nnz_u"]) == (ks["nnz_l"], ks["nnz_u"])
        assert s["rcond"] == pytest.approx(ks["rcond"], rel=0, abs=0)
        g.close()


def test_exact_mode_solves_the_system():
    for name, (n, ap, ai, ax, rhs) in _systems() + [("blocklower", _block_lower())]:
        g = GpuKluSolver(n, pivot_mode=N.PIVOT_EXACT)
        g.factor(ap, ai, ax)
        x = rhs.copy()
        g.solve(x)
        A = sp.csc_matrix((ax, ai, ap), shape=(n, n))
        xr = np.linalg.solve(A.toarray(), rhs)
        assert np.max(np.abs(x - xr)) <= 1e-10 * max(1.0, np.max(np.abs(xr))), name
        # adjoint: A^T y = g
        if g.stats()["noffdiag"] == 0:
            y = rhs.copy()
            g.tsolve(y)
            yr = np.linalg.solve(A.toarray().T, rhs)
            assert np.max(np.abs(y - yr)) <= 1e-10 * max(1.0, np.max(np.abs(yr))), name


def test_error_behaviour():
    n, ap, ai, ax, rhs = _systems()[1][1]
    g = GpuKluSolver(n)
    with pytest.raises(SolverError) as e:
        g.solve(rhs.copy())
    assert e.value.status == N.SOLVE_FAILED
    with pytest.raises(SolverError) as e:
        g.analyze(ap[:-1], ai)
    assert e.value.status == N.INVALID_MATRIX
    g.factor(ap, ai, ax)
    with pytest.raises(SolverError) as e:
        g.solve(np.zeros(n + 1))
    assert e.value.status == N.INVALID_MATRIX
    assert g.name() == "GpuKLU"
    g.prepare(n + 1)  # size change resets the pattern
    with pytest.raises(SolverError):
        g.solve(np.zeros(n + 1))


@pytest.mark.parametrize("model", ["reference", "consistent"])
def test_device_stamps(model):
    rng = np.random.default_rng(2)
    cases = [cz.mesh_dc(), cz.inverter_chain(20, 0.4, mos_model=model),
             cz.ring_oscillator(11, mos_model=model)]
    g = GpuKluSolver(1)
    for c in cases:
        dc = DeviceCircuit(c)
        ap, ai = dc.pattern()
        x = rng.uniform(-0.2, 1.3, c.node_count)
        x[0] = 0.0
        for gmin in (1e-12, 1e-6):
            ax, rhs = dc.stamp(g, x, gmin=gmin)
            n, ap_o, ai_o, ax_o, rhs_o = po.mna(c, x, gmin=gmin)
            assert dc.n == n
            assert np.array_equal(ap, ap_o) and np.array_equal(ai, ai_o)
            np.testing.assert_allclose(ax, ax_o, rtol=1e-14, atol=0)
            np.testing.assert_allclose(rhs, rhs_o, rtol=1e-14, atol=1e-300)
            if not np.any(c.type == cz.DEV_D):
                assert np.array_equal(ax, ax_o) and np.array_equal(rhs, rhs_o)


def test_newton_dc_mesh():
    c = cz.mesh_dc()
    cfg = dict(wl.TIGHT, gmin_steps=10)
    ocfg = {k: cfg[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps",
                                "source_steps")}
    r_o, it_o, x_o = po.dc_op(c, "nativeklu_exact", **ocfg)
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    dc = DeviceCircuit(c)
    res = newton_dc(g, dc, N.newton_config(**cfg))
    assert res.converged and r_o == "converged"
    assert res.iterations == it_o
    assert np.max(np.abs(res.x - x_o)) <= 1e-10 * np.max(np.abs(x_o))
    assert po.residual(c, res.x, 1e-6) <= 1e-12
    # reference pivot rule: same iterates as the reference's NativeKLU
    r_r, it_r, x_r = po.dc_op(c, "nativeklu", **ocfg)
    g2 = GpuKluSolver(1, pivot_mode=N.PIVOT_REFERENCE)
    res2 = newton_dc(g2, DeviceCircuit(c), N.newton_config(**cfg))
    assert res2.iterations == it_r and res2.reason == r_r
    assert np.max(np.abs(res2.x - x_r)) <= 1e-10 * np.max(np.abs(x_r))


def test_batch_matches_oracle():
    _batch_against_oracle()


@pytest.mark.parametrize("switch", ["GPUKLU_CONT_M=2", "GPUKLU_CONT_KERNEL=0",
                                    "GPUKLU_STEP_PROGRAM=0", "GPUKLU_CONT_WARPS=4",
                                    "GPUKLU_LANE_CAP=1"])
def test_batch_paths_match_oracle(switch, monkeypatch):
    # the batch's other schedules (two instances per continuation warp, the
    # warp classes, column-order factorization, fewer resident warps, a lane
    # phase of one iteration) give the oracle's results as well
    name, value = switch.split("=")
    monkeypatch.setenv(name, value)
    _batch_against_oracle()


def _batch_against_oracle():
    B = wl.inverter_batch(12, 61, seed=11)
    it_o, rs_o, x_o = po.dc_batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val,
                                  "nativeklu_exact", nthreads=4,
                                  x_cap=max(c.n for c in B.circuits), x0=B.x0,
                                  x0_off=B.x0_off, **{k: v for k, v in wl.TIGHT.items()
                                                      if k in ("max_iters", "abs_tol",
                                                               "rel_tol", "gmin", "gmin_steps")})
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    bt.run(N.newton_config(**wl.TIGHT))
    it, itt, rs, x = bt.results()
    conv = rs_o == 0
    assert np.mean(conv) > 0.9
    assert np.array_equal(rs == 0, conv)
    agree = np.mean(it[conv] == it_o[conv])
    assert agree > 0.98, agree
    for i in np.flatnonzero(conv):
        n = B.circuits[B.inst_circ[i]].n
        xg = x[bt.x_off[i]:bt.x_off[i] + n]
        xo = x_o[i, :n]
        assert np.max(np.abs(xg - xo)) <= 1e-10 * max(1.0, np.max(np.abs(xo))), i


@pytest.mark.parametrize("lanes", ["1", "0"], ids=["two_phase", "warp_only"])
def test_batch_results_pinned_and_phase_times(lanes, monkeypatch):
    """The results land in a caller's pinned buffer exactly as in a new array,
    both batch schedules (the lane kernel with the warp kernel behind it, and
    the warp kernels alone) give the same operating points within 1e-10, and
    the per-kernel device times of a run are reported."""
    import torch
    monkeypatch.setenv("GPUKLU_BATCH_LANES", lanes)
    B = wl.inverter_batch(6, 21, seed=5)
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    cfg = N.newton_config(**wl.TIGHT)
    bt.run(cfg)
    it, itt, rs, x = bt.results()
    pinned = torch.empty(bt.x_len, dtype=torch.float64).pin_memory()
    it2, itt2, rs2, x2 = bt.results(x_out=pinned.numpy())
    assert np.array_equal(x, x2) and np.array_equal(itt, itt2) and np.array_equal(rs, rs2)
    ph = bt.phase_ms()
    assert ph["warps_ms"] >= 0.0 and ph["lanes_ms"] >= 0.0
    if lanes == "1":
        assert ph["lane_cap"] > 0 and ph["lanes_ms"] > 0.0
    else:
        assert ph["lane_cap"] == 0
    # the other schedule on the same batch
    monkeypatch.setenv("GPUKLU_BATCH_LANES", "0" if lanes == "1" else "1")
    bt2 = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    bt2.run(cfg)
    _, itt3, rs3, x3 = bt2.results()
    # the two schedules round differently (one instance per lane or per warp):
    # iteration counts may differ where a step lands on the tolerance
    assert np.mean(rs == rs3) >= 0.98
    conv = (rs == 0) & (rs3 == 0)
    assert np.mean(itt[conv] == itt3[conv]) >= 0.98
    for i in np.flatnonzero(conv):
        n = B.circuits[B.inst_circ[i]].n
        a, b = x[bt.x_off[i]:bt.x_off[i] + n], x3[bt.x_off[i]:bt.x_off[i] + n]
        assert np.max(np.abs(a - b)) <= 1e-10 * max(1.0, np.max(np.abs(a)))
    with pytest.raises(TypeError):
        bt.results(x_out=np.zeros(3))


def test_netlist_deck_on_the_device():
    """A deck read by the netlist compiler runs on the device Newton path with
    the oracle's iterations and solution (the deck's own .option settings)."""
    from rustspice_gb300 import netlist as nl
    deck = nl.compile_deck("""* two resistor-loaded NMOS stages beside a diode ladder
VDD vdd 0 DC 1.8
VIN in 0 DC 0.9
RL1 vdd mid 20k
MN1 mid in 0 0 nch W=2u L=1u
RL2 vdd out 20k
MN2 out mid 0 0 nch W=2u L=1u
V1 a 0 DC 1.0
R1 a b 1k
D1 b 0 dx
R2 b c 2k
D2 c 0 dx
.model nch nmos level=1 vto=0.45 u0=400
.model dx d is=1e-14
.option reltol=1e-10 vntol=1e-12 itl1=200
.op
.end
""")
    opts = deck.newton_options()
    r_o, it_o, x_o = po.dc_op(deck.circuit, "nativeklu_exact", **opts)
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    res = newton_dc(g, DeviceCircuit(deck.circuit), N.newton_config(**opts))
    assert r_o == "converged" and res.converged and res.iterations == it_o
    assert np.max(np.abs(res.x - x_o)) <= 1e-10 * max(1.0, np.max(np.abs(x_o)))


def test_batch_autotune_and_schedules():
    """The project's autotuner times the batch under candidate schedules and
    keeps the fastest; every schedule gives the default's operating points
    within 1e-10, and the default schedule set back reproduces the first
    run bit for bit."""
    B = wl.inverter_batch(16, 21, seed=7)
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    cfg = N.newton_config(**wl.TIGHT)
    bt.run(cfg)
    _, itt, rs, x = bt.results()
    ch = bt.autotune(cfg)
    assert ch["lane_cap"] in (0, 1, 2, 3, 4, 5, 6, 8, 10, 12) and ch["cont_tiles"] in (1, 2, 3, 4)
    assert ch["runs"] >= 10 and ch["best_ms"] > 0.0
    bt.run(cfg)
    _, itt2, rs2, x2 = bt.results()
    assert np.mean(rs == rs2) >= 0.98
    conv = (rs == 0) & (rs2 == 0)
    for i in np.flatnonzero(conv):
        n = B.circuits[B.inst_circ[i]].n
        a, b = x[bt.x_off[i]:bt.x_off[i] + n], x2[bt.x_off[i]:bt.x_off[i] + n]
        assert np.max(np.abs(a - b)) <= 1e-10 * max(1.0, np.max(np.abs(a)))
    for cap, ct in ((0, 2), (3, 1), (12, 4)):  # 0: the continuation starts every instance
        bt.set_schedule(cap, ct)
        bt.run(cfg)
        assert bt.phase_ms()["lane_cap"] == cap
        _, _, rs3, x3 = bt.results()
        assert np.mean(rs == rs3) >= 0.98
    bt.set_schedule(6, 2)
    bt.run(cfg)
    _, itt4, rs4, x4 = bt.results()
    assert np.array_equal(x, x4) and np.array_equal(itt, itt4) and np.array_equal(rs, rs4)
    with pytest.raises(SolverError) as e:
        bt.set_schedule(-1, 2)
    assert e.value.status == N.INVALID_MATRIX
