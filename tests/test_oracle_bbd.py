"""The oracle's bordered-block-diagonal solver (CPU only).

Pinned to the reference's BBD unit tests (with the partition each test's
comment states), to SciPy on seeded bordered meshes through both Schur paths
(dense for a border of at most 64, sparse above), and to the reference's own
behaviour on duplicated border entries.
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


def _bbd(n, ap, ai, ax, b, asg, nb):
    s = po.Solver("bbd", n, asg, nb)
    s.prepare(n)
    assert s.analyze(ap, ai) == 0
    assert s.factor(ap, ai, ax) == 0
    st, x = s.solve(b)
    assert st == 0
    return s, x


@pytest.mark.parametrize("k", KATS["bbd"], ids=lambda k: k["name"])
def test_bbd_kats(k):
    n = len(k["ap"]) - 1
    s, x = _bbd(n, k["ap"], k["ai"], k["ax"], k["b"], k["assignment"], k["nblocks"])
    A = sp.csc_matrix((k["ax"], k["ai"], k["ap"]), shape=(n, n)).toarray()
    xd = np.linalg.solve(A, k["b"])
    assert np.max(np.abs(x - xd)) < 1e-8
    r = np.linalg.norm(A @ x - k["b"]) / np.linalg.norm(k["b"])
    assert r < 1e-10
    assert s.bbd_info()["fallback"] == k["fallback"]


def test_decomposition_promotes_cross_block_nodes():
    """bbd.rs:366-407: a node with an entry into another block joins the border."""
    # chain 0-1-2-3 with 0,1 in block 0 and 2,3 in block 1: 1-2 couples the blocks
    ap = [0, 2, 5, 8, 10]
    ai = [0, 1, 0, 1, 2, 1, 2, 3, 2, 3]
    ax = [2.0, -1.0, -1.0, 3.0, -1.0, -1.0, 3.0, -1.0, -1.0, 2.0]
    s, x = _bbd(4, ap, ai, ax, [1.0, 0.0, 0.0, 1.0], [0, 0, 1, 1], 2)
    info = s.bbd_info()
    # column pass promotes 1 (row 2 is in block 1), then 2 stays (its row 1 is border now)
    assert info["border_size"] >= 1 and 1 in set(info["perm"][info["border_start"]:])
    A = sp.csc_matrix((ax, ai, ap), shape=(4, 4)).toarray()
    assert np.max(np.abs(x - np.linalg.solve(A, [1.0, 0.0, 0.0, 1.0]))) < 1e-12


@pytest.mark.parametrize("nborder", [32, 80], ids=["dense_schur", "sparse_schur"])
def test_bordered_meshes_match_scipy(nborder):
    c, asg, nb = cz.bordered_meshes(8, nborder, 6, 9, ndiodes=4, seed=3)
    x = np.random.default_rng(0).uniform(0, 0.7, c.node_count)
    n, ap, ai, ax, rhs = po.mna(c, x)
    s, xb = _bbd(n, ap, ai, ax, rhs, asg, nb)
    info = s.bbd_info()
    assert info["num_blocks"] == 8 and not info["fallback"]
    assert info["border_size"] == nborder + 1  # the border nodes and ground
    xr = spl.spsolve(sp.csc_matrix((ax, ai, ap), shape=(n, n)), rhs)
    assert np.max(np.abs(xb - xr)) <= 1e-12 * np.max(np.abs(xr))


def test_duplicate_border_entries_defect_reproduced():
    """The reference's Schur assembly writes each entry of R_k into the block
    right-hand side by assignment (bbd_solver.rs:788, :867), so of two entries
    at one (block row, border column) only the last survives, while every
    other step sums duplicates. Two parallel resistors between a block node
    and a border node therefore give a wrong solution; the restatement keeps
    that, and the bordered-mesh workload never creates such pairs."""
    # blocks {1}, {2}; border {0 (ground), 3}; node 1 tied to 3 by two resistors
    c = cz.Circuit(4, np.array([0, 0, 0, 0, 0, 2], np.int32),
                   np.array([[1, 0, 0, 0], [2, 0, 0, 0], [1, 3, 0, 0], [1, 3, 0, 0],
                             [2, 3, 0, 0], [0, 3, 0, 0]], np.int32),
                   np.array([[1e3, 0, 0, 0, 0, 0], [1e3, 0, 0, 0, 0, 0], [2e3, 0, 0, 0, 0, 0],
                             [2e3, 0, 0, 0, 0, 0], [1e3, 0, 0, 0, 0, 0],
                             [1e-3, 0, 0, 0, 0, 0]], np.float64))
    n, ap, ai, ax, rhs = po.mna(c, np.zeros(4))
    s, xb = _bbd(n, ap, ai, ax, rhs, [-1, 0, 1, -1], 2)
    xr = np.linalg.solve(sp.csc_matrix((ax, ai, ap), shape=(n, n)).toarray(), rhs)
    assert not s.bbd_info()["fallback"]
    assert np.max(np.abs(xb - xr)) > 1e-3 * np.max(np.abs(xr))
