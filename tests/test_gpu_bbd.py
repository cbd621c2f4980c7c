"""The bordered-block-diagonal solver on the GPU.

Known-answer systems of the reference's BBD tests, seeded bordered meshes
against the oracle's BbdSolver (same decomposition, solutions to 1e-12), a
Newton DC solve against the oracle's engine loop with its BbdSolver, and the
full 64-mesh, 1024-border case against the plain GPU solver.
"""
import json
import os
import time

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import BbdSolver, DeviceCircuit, GpuKluSolver, newton_dc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KATS = json.load(open(os.path.join(GOLD, "kats.json")))
OCFG = {k: wl.TIGHT[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps")}


@pytest.mark.parametrize("k", KATS["bbd"], ids=lambda k: k["name"])
def test_bbd_kats(k):
    n = len(k["ap"]) - 1
    g = BbdSolver(k["ap"], k["ai"], k["assignment"], k["nblocks"])
    g.factor(k["ax"])
    x = np.array(k["b"], np.float64)
    g.solve(x)
    A = sp.csc_matrix((k["ax"], k["ai"], k["ap"]), shape=(n, n)).toarray()
    assert np.max(np.abs(x - np.linalg.solve(A, k["b"]))) < 1e-8
    assert g.info()["fallback"] == k["fallback"]


@pytest.mark.parametrize("nborder", [32, 80])
def test_bordered_meshes_match_oracle(nborder):
    c, asg, nb = cz.bordered_meshes(8, nborder, 6, 9, ndiodes=4, seed=3)
    x = np.random.default_rng(0).uniform(0, 0.7, c.node_count)
    n, ap, ai, ax, rhs = po.mna(c, x)
    s = po.Solver("bbd", n, asg, nb)
    s.prepare(n)
    s.factor(ap, ai, ax)
    _, xo = s.solve(rhs)
    g = BbdSolver(ap, ai, asg, nb)
    assert np.array_equal(g.perm(), s.bbd_info()["perm"])
    for a in (ax, ax * (1.0 + 0.01 * np.random.default_rng(1).standard_normal(len(ax)))):
        g.factor(a)
        xg = rhs.copy()
        g.solve(xg)
        s.factor(ap, ai, a)
        _, xo = s.solve(rhs)
        assert np.max(np.abs(xg - xo)) <= 1e-12 * np.max(np.abs(xo))
    info = g.info()
    assert info["num_blocks"] == 8 and info["inner_blocks"] == 8 and info["tiles"] >= 8


def test_newton_matches_oracle_bbd():
    c, asg, nb = cz.bordered_meshes(16, 256, 15, 25, ndiodes=16, seed=4)
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    g = BbdSolver(ap, ai, asg, nb)
    x0 = wl.bordered_nodeset(c)
    r = g.newton_dc(dc, N.newton_config(**wl.TIGHT), x0=x0)
    ro, ito, xo = po.dc_op_bbd(c, asg, nb, x0=x0, **OCFG)
    assert r.converged and ro == "converged" and r.iterations == ito
    assert np.max(np.abs(r.x - xo)) <= 1e-10 * np.max(np.abs(xo))


def test_full_bordered_case_against_oracle():
    c, asg, nb = cz.bordered_meshes()  # 64 meshes of 30..50 squared, 1024 border nodes
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    cfg = N.newton_config(**wl.TIGHT)
    g = BbdSolver(ap, ai, asg, nb)
    x0 = wl.bordered_nodeset(c)
    t0 = time.perf_counter()
    r = g.newton_dc(dc, cfg, x0=x0)
    t_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = g.newton_dc(dc, cfg, x0=x0)
    t_bbd = time.perf_counter() - t0
    info = g.info()
    t0 = time.perf_counter()
    ro, ito, xo = po.dc_op_bbd(c, asg, nb, x0=x0, **OCFG)
    t_cpu = time.perf_counter() - t0
    assert r.converged and ro == "converged" and r.iterations == ito
    assert np.max(np.abs(r.x - xo)) <= 1e-10 * np.max(np.abs(xo))
    print(f"bordered meshes n={c.n} blocks={info['num_blocks']} border={info['border_size']} "
          f"tiles={info['tiles']}: {r.iterations} Newton iterations, BBD "
          f"{t_bbd / r.iterations * 1e3:.2f} ms/iteration (first call {t_first:.2f} s); "
          f"oracle BbdSolver (1 core) {t_cpu / ito * 1e3:.0f} ms/iteration")


def test_plain_solver_refuses_the_whole_bordered_matrix():
    """Over the whole matrix the border couples every mesh, and the update
    lists of the plain solver's factorization would exceed 2^31 entries: it
    refuses with INVALID_MATRIX instead of indexing past them."""
    from rustspice_gb300.solver import SolverError
    c, asg, nb = cz.bordered_meshes()
    dc = DeviceCircuit(c)
    h = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    with pytest.raises(SolverError) as e:
        newton_dc(h, dc, N.newton_config(**wl.TIGHT), x0=wl.bordered_nodeset(c))
    assert "2^31" in str(e.value)


@pytest.mark.parametrize("n", [1, 31, 33, 100, 257, 1025])
def test_dense_schur_lu_variants(n):
    """The cooperative Schur LU (FMA or DMMA updates) within 1e-12 of the
    panel kernels' factor, and L U = A; a zero pivot takes the +-1e-14
    rule in all three."""
    from rustspice_gb300.solver import dense_lu_nopivot
    rng = np.random.default_rng(n)
    a = rng.uniform(-1.0, 1.0, (n, n))
    a[np.arange(n), np.arange(n)] += n
    if n >= 33:
        a[5, :] = 0.0  # a zero pivot: the +-1e-14 rule
        a[5, 5] = 0.0
    f0, _ = dense_lu_nopivot(a, 0)
    f1, _ = dense_lu_nopivot(a, 1)
    f2, _ = dense_lu_nopivot(a, 2)
    for f in (f1, f2):
        assert np.max(np.abs(f - f0)) <= 1e-12 * max(1.0, np.max(np.abs(f0)))
    if n < 33:
        for f in (f0, f1, f2):
            L = np.tril(f, -1) + np.eye(n)
            U = np.triu(f)
            assert np.max(np.abs(L @ U - a)) <= 1e-12 * np.max(np.abs(a))
    else:
        assert f0[5, 5] == f1[5, 5] == f2[5, 5] == 1e-14


def test_dmma_probe_and_bbd_newton_with_each_schur_lu(monkeypatch):
    from rustspice_gb300 import native as N
    assert N.lib().gpuklu_fp64_mma_peak_tflops() > 0.0
    c, asg, nb = cz.bordered_meshes(nblocks=6, nborder=96, side_lo=8, side_hi=14, ndiodes=4)
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    cfg = N.newton_config(**wl.TIGHT)
    x0 = wl.bordered_nodeset(c)
    res = {}
    for v in ("panels", "fma", "mma"):
        monkeypatch.setenv("GPUKLU_SCHUR_LU", v)
        bb = BbdSolver(ap, ai, asg, nb)
        res[v] = bb.newton_dc(dc, cfg, x0=x0)
        bb.close()
    assert res["panels"].iterations == res["fma"].iterations == res["mma"].iterations
    for v in ("fma", "mma"):
        assert np.max(np.abs(res[v].x - res["panels"].x)) <= 1e-10 * np.max(np.abs(res["panels"].x))
