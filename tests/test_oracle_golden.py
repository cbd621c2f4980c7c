"""The oracle against the reference's own known answers (CPU only).

The fixtures in tests/golden/ come from the reference's solver, stamp and
end-to-end tests and its Matrix Market / BeGAN fixtures (make_golden.py
there says how). Every oracle solver kind is held to the reference test's
own tolerance; the large fixtures are also checked against SciPy's
independent sparse solve.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KATS = json.load(open(os.path.join(GOLD, "kats.json")))
KINDS = ["dense", "sparselu", "sparselubtf", "nativeklu", "nativeklu_exact"]


def _solve(kind, ap, ai, ax, b):
    n = len(ap) - 1
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    assert s.factor(ap, ai, ax) == 0
    st, x = s.solve(b)
    assert st == 0
    return s, x


def _residual(ap, ai, ax, x, b):
    n = len(ap) - 1
    A = sp.csc_matrix((ax, ai, ap), shape=(n, n))
    return np.abs(A @ x - np.asarray(b))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("kat", KATS["solve"], ids=lambda k: k["name"])
def test_solve_kats(kind, kat):
    s, x = _solve(kind, kat["ap"], kat["ai"], kat["ax"], kat["b"])
    assert np.max(_residual(kat["ap"], kat["ai"], kat["ax"], x, kat["b"])) < kat["tol"]
    if kat["x"] is not None:
        assert np.max(np.abs(x - np.asarray(kat["x"]))) < kat["tol"]


@pytest.mark.parametrize("kind", ["nativeklu", "nativeklu_exact"])
def test_refactor_counters(kind):
    k = KATS["refactor"]
    n = len(k["ap"]) - 1
    s = po.Solver(kind, n)
    s.prepare(n)
    assert s.factor(k["ap"], k["ai"], k["ax1"]) == 0
    st = s.klu_stats()
    assert [st["factor_count"], st["refactor_count"]] == k["counts1"]
    _, x1 = s.solve(k["b1"])
    assert np.max(_residual(k["ap"], k["ai"], k["ax1"], x1, k["b1"])) < 1e-10
    assert s.factor(k["ap"], k["ai"], k["ax2"]) == 0
    st = s.klu_stats()
    assert [st["factor_count"], st["refactor_count"]] == k["counts2"]
    _, x2 = s.solve(k["b2"])
    assert np.max(_residual(k["ap"], k["ai"], k["ax2"], x2, k["b2"])) < 1e-10
    assert np.max(np.abs(x1 - x2)) < 1e-9


def test_rcond():
    k = KATS["rcond"]
    s = po.Solver("nativeklu", 3)
    s.prepare(3)
    assert s.factor(k["ap"], k["ai"], k["ax_id"]) == 0
    assert abs(s.klu_stats()["rcond"] - 1.0) < 1e-10
    assert s.factor(k["ap"], k["ai"], k["ax_ill"]) == 0
    assert s.klu_stats()["rcond"] < 1e-10


def _one_device_circuit(k):
    t, a, b, p0, p1 = k["dev"]
    return cz.Circuit(k["node_count"], np.array([t], np.int32),
                      np.array([[a, b, 0, 0]], np.int32),
                      np.array([[p0, p1, 0, 0, 0, 0]], np.float64))


@pytest.mark.parametrize("k", KATS["stamps"], ids=lambda k: k["name"])
def test_stamp_kats(k):
    """The engine's build adds the ground pin (0,0) += 1 after the devices
    (crates/sim-core/src/engine.rs:280); the builder tests have no pin."""
    c = _one_device_circuit(k)
    n, ap, ai, ax, rhs = po.mna(c, k["x"], gmin=k["gmin"], scale=k["scale"])
    A = sp.csc_matrix((ax, ai, ap), shape=(n, n)).toarray()
    for r, col, v in k.get("entries", []):
        pin = 1.0 if (r, col) == (0, 0) else 0.0
        assert abs(A[r, col] - (v + pin)) <= 1e-16 * (1.0 + pin)
    if "rhs" in k:
        assert np.allclose(rhs, k["rhs"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("kind", KINDS)
def test_divider_end_to_end(kind):
    d = KATS["divider"]
    c = cz.Circuit(d["node_count"], np.array(d["type"], np.int32), np.array(d["nodes"], np.int32),
                   np.array(d["p"], np.float64))
    r, it, x = po.dc_op(c, kind)
    assert r == "converged"
    for node, v in d["expect"].items():
        assert abs(x[int(node)] - v) < d["tol"]


def _mtx(name):
    z = np.load(os.path.join(GOLD, f"mtx_{name}.npz"))
    return int(z["n"]), z["ap"].astype(np.int64), z["ai"].astype(np.int64), z["ax"], z["rhs"]


@pytest.mark.parametrize("name,n,nnz,tol", [("adder_dcop_01", 1813, 11156, 1e-3),
                                            ("circuit_1", 2624, 35823, 1e-3),
                                            ("rajat01", 6833, 43250, 0.1)])
def test_matrix_market_fixtures(name, n, nnz, tol):
    """bbd_benchmark_tests.rs:289-330: the fixture sizes, and SparseLU (the
    solver that test compares against) within its tolerance of SciPy."""
    n_, ap, ai, ax, rhs = _mtx(name)
    assert (n_, len(ai)) == (n, nnz)
    A = sp.csc_matrix((ax, ai, ap), shape=(n, n))
    x_ref = spl.spsolve(A, rhs)
    _, x = _solve("sparselu", ap, ai, ax, rhs)
    assert np.max(np.abs(x - x_ref)) <= tol * np.max(np.abs(x_ref))
    if n < 3000:
        _, xd = _solve("dense", ap, ai, ax, rhs)
        assert np.max(np.abs(xd - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))


def test_btf_lower_coupling_defect_reproduced():
    """The reference's BTF orders the blocks so that the coupling lies BELOW
    the diagonal blocks, while its block solve (native_klu.rs:1491-1551,
    sparse_lu_btf.rs:461-561) walks the blocks last to first and applies only
    couplings above them. On adder_dcop_01 (469 BTF blocks) NativeKLU and
    SparseLU-BTF therefore miss the true solution by ~70 %; the restatement
    keeps that behaviour. The exact-pattern mode applies the lower coupling
    forward and agrees with SciPy to round-off."""
    n, ap, ai, ax, rhs = _mtx("adder_dcop_01")
    x_ref = spl.spsolve(sp.csc_matrix((ax, ai, ap), shape=(n, n)), rhs)
    sc = np.max(np.abs(x_ref))
    s, xk = _solve("nativeklu", ap, ai, ax, rhs)
    assert s.klu_stats()["nblocks"] == 469
    _, xb = _solve("sparselubtf", ap, ai, ax, rhs)
    assert np.max(np.abs(xk - x_ref)) > 0.5 * sc
    assert np.max(np.abs(xb - x_ref)) > 0.5 * sc
    _, xe = _solve("nativeklu_exact", ap, ai, ax, rhs)
    assert np.max(np.abs(xe - x_ref)) <= 1e-8 * sc


def test_began_small_pgrid():
    z = np.load(os.path.join(GOLD, "began_small_pgrid.npz"))
    c = cz.Circuit(int(z["node_count"]), z["type"], z["nodes"], z["p"])
    r, it, x = po.dc_op(c, "nativeklu", abs_tol=1e-12, rel_tol=1e-12)
    assert r == "converged"
    n, ap, ai, ax, rhs = po.mna(c, x[:c.node_count])
    x_ref = spl.spsolve(sp.csc_matrix((ax, ai, ap), shape=(n, n)), rhs)
    assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))
    v = c.device_index(cz.DEV_V)
    a, b = c.nodes[v, 0], c.nodes[v, 1]
    assert abs(x[a] - x[b] - 0.7) < 1e-12  # the 0.7 V supply
