"""Writes the golden fixtures under tests/golden/ from the reference's own tests.

Run it with the reference checkout's root as its one argument; the fixtures
it writes are committed, so nothing at test time reads the reference.

* ``kats.json`` -- the known-answer systems of the reference's solver and
  stamp tests, restated as data with the file:line each comes from.
* ``mtx_<name>.npz`` -- the three Matrix Market fixtures
  (tests/fixtures/matrices/*.mtx) converted the way
  crates/sim-core/tests/bbd_benchmark_tests.rs:33-141 does it: 1-based
  coordinates, pattern files get 10 on the diagonal and -0.1 elsewhere,
  symmetric files are mirrored, entries sorted by (column, row) with
  duplicates summed. ``rhs`` is that file's LCG ``generate_rhs`` (:275-287)
  with seed 42.
* ``began_small_pgrid.npz`` -- the BeGAN power-grid netlist
  (tests/fixtures/netlists/began_small_pgrid.sp, R/I/V only) as a device
  list: nodes numbered by first appearance with ground "0" as node 0
  (crates/sim-core/src/circuit.rs:37-57), devices in netlist order.
* ``decks/`` -- the reference's fixture decks the netlist reader's tests read
  (tests/fixtures/netlists/{basic_dc,nmos_dc,include_parent,include_child}.cir
  and began_small_pgrid.sp), copied byte for byte.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

DEV_R, DEV_V, DEV_I = 0, 1, 2


def generate_rhs(n: int, seed: int) -> np.ndarray:
    """bbd_benchmark_tests.rs:275-287: 64-bit LCG, top 31 bits scaled to [-1, 1)."""
    out = np.zeros(n)
    s = seed & 0xFFFFFFFFFFFFFFFF
    for i in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
        out[i] = float(s >> 33) / float(1 << 31) - 1.0
    return out


def read_mtx(path: str):
    with open(path) as f:
        header = f.readline()
        assert header.startswith("%%MatrixMarket")
        low = header.lower()
        pattern, symmetric = "pattern" in low, "symmetric" in low
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, _ = (int(t) for t in line.split()[:3])
        assert nr == nc
        rows, cols, vals = [], [], []
        for line in f:
            t = line.split()
            if len(t) < 2 or t[0].startswith("%"):
                continue
            r, c = int(t[0]) - 1, int(t[1]) - 1
            v = (10.0 if r == c else -0.1) if pattern else float(t[2])
            rows.append(r)
            cols.append(c)
            vals.append(v)
            if symmetric and r != c:
                rows.append(c)
                cols.append(r)
                vals.append(v)
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals)
    order = np.lexsort((rows, cols))  # stable: equal (col,row) keep file order
    rows, cols, vals = rows[order], cols[order], vals[order]
    ap = np.zeros(nr + 1, np.int64)
    ai, ax = [], []
    last = (-1, -1)
    for r, c, v in zip(rows, cols, vals):
        if (r, c) == last:
            ax[-1] += v
            continue
        last = (r, c)
        ai.append(r)
        ax.append(v)
        ap[c + 1] += 1
    return nr, np.cumsum(ap), np.array(ai, np.int32), np.array(ax)


def read_rvi_netlist(path: str):
    names = {"0": 0}
    t, nd, p = [], [], []

    def node(s):
        if s not in names:
            names[s] = len(names)
        return names[s]

    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok or tok[0].startswith("*") or tok[0].startswith("."):
                continue
            kind = tok[0][0].upper()
            a, b = node(tok[1]), node(tok[2])
            vals = [x for x in tok[3:] if x.upper() != "DC"]
            v = float(vals[0])
            t.append({"R": DEV_R, "V": DEV_V, "I": DEV_I}[kind])
            nd.append((a, b, 0, 0))
            p.append((v, 0, 0, 0, 0, 0))
    return len(names), np.array(t, np.int32), np.array(nd, np.int32), np.array(p)


def kats():
    """Known-answer systems of the reference's tests (CSC, 0-based)."""
    sys3 = dict(ap=[0, 2, 5, 7], ai=[0, 1, 0, 1, 2, 1, 2], ax=[4.0, 1.0, 1.0, 5.0, 2.0, 2.0, 6.0],
                b=[5.0, 14.0, 14.0])

    def tridiag(n, diag_ends, diag_mid, off):
        ap, ai, ax = [0], [], []
        for c in range(n):
            if c > 0:
                ai.append(c - 1)
                ax.append(off)
            ai.append(c)
            ax.append(diag_ends if c in (0, n - 1) else diag_mid)
            if c < n - 1:
                ai.append(c + 1)
                ax.append(off)
            ap.append(len(ai))
        return ap, ai, ax

    out = [
        dict(name="lower_2x2", src="crates/sim-core/src/sparse_lu.rs:752-793; "
             "crates/sim-core/tests/native_klu_tests.rs:34-49",
             ap=[0, 2, 3], ai=[0, 1, 1], ax=[2.0, 1.0, 3.0], b=[4.0, 7.0],
             x=[2.0, 5.0 / 3.0], tol=1e-10),
        dict(name="diagonal_3", src="crates/sim-core/src/sparse_lu.rs:796-812; "
             "crates/sim-core/tests/native_klu_tests.rs:71-85",
             ap=[0, 1, 2, 3], ai=[0, 1, 2], ax=[2.0, 3.0, 4.0], b=[4.0, 9.0, 8.0],
             x=[2.0, 3.0, 2.0], tol=1e-10),
        dict(name="tridiag_3", src="crates/sim-core/src/sparse_lu.rs:815-853; "
             "crates/sim-core/tests/native_klu_tests.rs:52-68", x=None, tol=1e-10, **sys3),
        dict(name="block_diagonal_4", src="crates/sim-core/tests/native_klu_tests.rs:161-177",
             ap=[0, 2, 4, 6, 8], ai=[0, 1, 0, 1, 2, 3, 2, 3],
             ax=[2.0, 1.0, 1.0, 3.0, 4.0, 1.0, 1.0, 2.0], b=[7.0, 11.0, 17.0, 6.0],
             x=None, tol=1e-9),
        dict(name="upper_block_triangular_3",
             src="crates/sim-core/tests/native_klu_tests.rs:181-197",
             ap=[0, 1, 2, 5], ai=[0, 1, 0, 1, 2], ax=[2.0, 3.0, 1.0, 1.0, 4.0],
             b=[5.0, 10.0, 8.0], x=None, tol=1e-9),
    ]
    ap, ai, ax = tridiag(5, 4.0, 4.0, -1.0)
    out.append(dict(name="tridiag_5", src="crates/sim-core/tests/native_klu_tests.rs:88-125",
                    ap=ap, ai=ai, ax=ax, b=[1.0] * 5, x=None, tol=1e-10))
    for n, tol, src in ((20, 1e-9, ":336-367"), (100, 1e-8, ":370-401")):
        ap, ai, ax = tridiag(n, 2.0, 3.0, -1.0)
        out.append(dict(name=f"rc_ladder_{n}", src="crates/sim-core/tests/native_klu_tests.rs" + src,
                        ap=ap, ai=ai, ax=ax, b=[float(i + 1) for i in range(n)], x=None, tol=tol))
    refactor = dict(name="refactor_doubled", src="crates/sim-core/tests/native_klu_tests.rs:203-243",
                    ap=sys3["ap"], ai=sys3["ai"], ax1=sys3["ax"], ax2=[2 * v for v in sys3["ax"]],
                    b1=sys3["b"], b2=[2 * v for v in sys3["b"]], counts1=[1, 0], counts2=[1, 1])
    rcond = dict(name="rcond", src="crates/sim-core/tests/native_klu_tests.rs:246-264",
                 ap=[0, 1, 2, 3], ai=[0, 1, 2], ax_id=[1.0, 1.0, 1.0], ax_ill=[1.0, 1e-15, 1.0])
    stamps = [
        dict(name="diode_gmin_floor", src="crates/sim-core/tests/mna_builder_tests.rs:132-151",
             node_count=2, dev=[3, 1, 0, 1e-14, 1.0], x=[0.0, 0.0], gmin=1e-6, scale=1.0,
             entries=[[1, 1, 1e-6], [0, 0, 1e-6]]),
        dict(name="current_source_scale", src="crates/sim-core/tests/mna_builder_tests.rs:111-129",
             node_count=2, dev=[2, 1, 0, 1e-3, 0.0], x=[0.0, 0.0], gmin=0.0, scale=0.5,
             rhs=[0.0005, -0.0005]),
    ]
    divider = dict(name="divider", src="crates/sim-core/tests/dc_basic_end_to_end.rs:38-51 "
                   "(tests/fixtures/netlists/basic_dc.cir)",
                   node_count=3, type=[DEV_V, DEV_R, DEV_R],
                   nodes=[[1, 0, 0, 0], [1, 2, 0, 0], [2, 0, 0, 0]],
                   p=[[1.0, 0, 0, 0, 0, 0], [1e3, 0, 0, 0, 0, 0], [2e3, 0, 0, 0, 0, 0]],
                   expect={"1": 1.0, "2": 2.0 / 3.0}, tol=1e-6)
    bbd = [  # bbd_solver.rs tests, with the partition each test's comment states
        dict(name="bbd_block_diagonal", src="crates/sim-core/src/bbd_solver.rs:1173-1193",
             ap=[0, 2, 4, 6, 8], ai=[0, 1, 0, 1, 2, 3, 2, 3],
             ax=[2.0, 1.0, 1.0, 3.0, 4.0, 1.0, 1.0, 2.0], b=[7.0, 11.0, 17.0, 6.0],
             assignment=[0, 0, 1, 1], nblocks=2, fallback=True),
        dict(name="bbd_bordered_5", src="crates/sim-core/src/bbd_solver.rs:1231-1291",
             ap=[0, 2, 5, 7, 10, 13], ai=[0, 1, 0, 1, 4, 2, 3, 2, 3, 4, 1, 3, 4],
             ax=[4.0, 1.0, 1.0, 4.0, 1.0, 4.0, 1.0, 1.0, 4.0, 1.0, 1.0, 1.0, 3.0],
             b=[5.0, 10.0, 5.0, 10.0, 8.0], assignment=[0, 0, 1, 1, -1], nblocks=2,
             fallback=False),
        dict(name="bbd_bordered_8", src="crates/sim-core/src/bbd_solver.rs:1294-1363",
             ap=[0, 2, 5, 8, 10, 13, 16, 19, 22],
             ai=[0, 1, 0, 1, 2, 1, 2, 6, 3, 4, 3, 4, 5, 4, 5, 7, 2, 6, 7, 5, 6, 7],
             ax=[2.0, -1.0, -1.0, 2.0, -1.0, -1.0, 2.0, 1.0, 2.0, -1.0, -1.0, 2.0, -1.0, -1.0,
                 2.0, 1.0, 1.0, 3.0, 0.5, 1.0, 0.5, 3.0],
             b=[1.0, 2.0, 3.0, 1.0, 2.0, 3.0, 4.0, 4.0],
             assignment=[0, 0, 0, 1, 1, 1, -1, -1], nblocks=2, fallback=False),
    ]
    return dict(solve=out, refactor=refactor, rcond=rcond, stamps=stamps, divider=divider,
                bbd=bbd)


def main(ref: str) -> None:
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats(), f, indent=1)
    for name in ("adder_dcop_01", "circuit_1", "rajat01"):
        n, ap, ai, ax = read_mtx(os.path.join(ref, "tests/fixtures/matrices", name + ".mtx"))
        np.savez_compressed(os.path.join(HERE, f"mtx_{name}.npz"), n=n, ap=ap, ai=ai, ax=ax,
                            rhs=generate_rhs(n, 42))
        print(name, n, len(ai))
    nc, t, nd, p = read_rvi_netlist(os.path.join(ref, "tests/fixtures/netlists/began_small_pgrid.sp"))
    np.savez_compressed(os.path.join(HERE, "began_small_pgrid.npz"), node_count=nc, type=t,
                        nodes=nd, p=p)
    print("began_small_pgrid", nc, len(t))
    os.makedirs(os.path.join(HERE, "decks"), exist_ok=True)
    for name in DECKS:
        with open(os.path.join(ref, "tests/fixtures/netlists", name), "rb") as f:
            data = f.read()
        with open(os.path.join(HERE, "decks", name), "wb") as f:
            f.write(data)
        print("deck", name, len(data))


DECKS = ("basic_dc.cir", "nmos_dc.cir", "include_parent.cir", "include_child.cir",
         "began_small_pgrid.sp")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout root>")
    main(sys.argv[1])
