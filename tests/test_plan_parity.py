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
from plan_emulator import EmulatedSolver
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
                                    cap_v=np.zeros(c.node_count) if transient else None)
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
    st = s.klu_stats()
    assert es.plan.nblocks == st["nblocks"]
    if mode == N.PIVOT_REFERENCE:  # the pattern of the pivot-free symbolic pass
        assert es.plan.nnz_l == st["nnz_l"]


def test_mesh_dimensions():
    """32x32 diode mesh: n = 1026 and 8,201 raw CSC entries (duplicates kept,
    as the engine's finalize() keeps them: crates/sim-core/src/mna.rs:320-347)."""
    c = cz.mesh_dc()
    n, ap, ai, ax, rhs = po.mna(c, np.zeros(c.node_count))
    assert n == 1026 and len(ai) == 8201
