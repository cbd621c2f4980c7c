"""The batched headline workload against the oracle at scale.

The sample is stratified over the 4096-chain inverter workload: the first
chain of every stage count 8..256 (249 chains), each at all 61 input points
of the 0..1.2 V sweep, 15,189 DC operating points. A chain's 61 points are
its DC sweep as the reference runs one (crates/sim-core/src/engine.rs:
684-820): one solver for the whole sweep, so the pivots the first point's
first factorization chose are kept for every later point (native_klu.rs:
1020-1148), except that each point starts from its own logic-level nodeset.
The oracle runs exactly that (pyoracle.dc_batch, sweep=True). Both MOSFET
models run:

* ``consistent`` - the card with a consistent linearisation (the bench
  headline's model); about 98.7 % converge.
* ``reference`` - the reference's own level-1 evaluator
  (crates/sim-devices/src/bsim/evaluate.rs:285-356), whose PMOS
  linearisation is not the derivative of its current; about 59 % converge.

The instances that do not converge are the reference's Newton running out of
iterations (crates/sim-core/src/newton.rs:93-107: the damping factor only
halves, to its 0.1 floor, and the level-1 steps are not limited), so the
converged set is part of the result. With the consistent model the device
batch must converge on exactly the oracle's instances, and at most 1 % of
them may take a different iteration count (the batch kernels contract
multiply-adds and use a one-step reciprocal, so an iterate that lands on the
tolerance may take one iteration more or less); every converged operating
point must match to 1e-10 relative. With the reference's model 38 % of the
instances meet a kept pivot below 1e-14, which the reference replaces by
+-1e-14 (native_klu.rs:1344-1348), and none of those converge; the rest
converge linearly at best (the stamped PMOS conductances are not the
derivatives of the stamped current), so the damping rule's comparison of
successive step norms decides on near ties. There the contracted arithmetic
of the batch kernels and the oracle's part ways: the converged sets may
differ on at most 2 % of the instances and the iteration counts of the
instances both converge on may differ on at most 15 %. Converging linearly,
an iterate that passes the step test (1e-10 relative) can still be farther
than that from the fixed point, so the converged operating points are held
to 1e-9 relative for this model. test_device_sweep_matches_oracle runs
the same points through the bit-exact single-circuit kernels and agrees with
the oracle at every point.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import Batch

pytestmark = pytest.mark.gpu

NEWTON = {k: v for k, v in wl.TIGHT.items()
          if k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps")}


def _run(model):
    ids = wl.stratified_chains()
    B = wl.inverter_batch(chain_ids=ids, mos_model=model)
    assert B.ninst >= 10_000 and sorted(set(B.stages.tolist())) == list(range(8, 257))
    it_o, rs_o, x_o = po.dc_batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val,
                                  "nativeklu_exact", nthreads=os.cpu_count() or 1,
                                  x_cap=max(c.n for c in B.circuits), x0=B.x0,
                                  x0_off=B.x0_off, **NEWTON)
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    bt.run(N.newton_config(**wl.TIGHT))
    it, itt, rs, x = bt.results()
    return B, bt, it, rs, x, it_o, rs_o, x_o


@pytest.mark.parametrize("model,frac,set_diff,it_agree,xtol",
                         [("consistent", (0.98, 0.99), 0.0, 0.99, 1e-10),
                          ("reference", (0.55, 0.65), 0.02, 0.85, 1e-9)])
def test_stratified_batch_matches_oracle(model, frac, set_diff, it_agree, xtol):
    B, bt, it, rs, x, it_o, rs_o, x_o = _run(model)
    conv_o = rs_o == 0
    conv = rs == 0
    f = float(np.mean(conv_o))
    print(f"{model}: {B.ninst} instances, oracle converged {f:.4f}, device {np.mean(conv):.4f}, "
          f"oracle iterations {int(it_o.sum())}, device {int(it.sum())}, "
          f"converged sets differ on {int(np.sum(conv != conv_o))}")
    assert frac[0] <= f <= frac[1], f
    assert np.mean(conv != conv_o) <= set_diff, np.flatnonzero(conv != conv_o)[:20]
    both = conv & conv_o
    agree = float(np.mean(it[both] == it_o[both]))
    print(f"{model}: iteration counts equal on {agree:.4f} of the instances both converge")
    assert agree >= it_agree, agree
    # every non-converged instance ran to the iteration cap, on both sides
    assert np.all(it_o[~conv_o] == NEWTON["max_iters"])
    assert np.all(it[~conv] == NEWTON["max_iters"])
    worst = 0.0
    for i in np.flatnonzero(both):
        n = B.circuits[B.inst_circ[i]].n
        xg = x[bt.x_off[i]:bt.x_off[i] + n]
        xo = x_o[i, :n]
        worst = max(worst, float(np.max(np.abs(xg - xo)) / max(1.0, np.max(np.abs(xo)))))
    print(f"{model}: worst relative difference of a converged operating point {worst:.2e}")
    assert worst <= xtol
    # the failures sit where the first stage switches: by input point
    bad_vin = np.unique(B.vin[~conv_o])
    print(f"{model}: input points with a non-converged instance: {bad_vin.round(2).tolist()}")


@pytest.mark.parametrize("model,chains", [("reference", (0, 1, 2, 100, 248)),
                                          ("consistent", (3, 140))])
def test_device_sweep_matches_oracle(model, chains):
    """The reference's DC sweep on the device (gpuklu_dc_sweep: one handle,
    the first point's pivots kept, the bit-exact single-circuit kernels)
    against the oracle's sweep, point by point, from the points' nodesets and
    without stopping at a failed point: the same reason and iteration count
    at every point, including those whose kept pivots are perturbed, and the
    same converged operating points."""
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, dc_sweep
    ids = wl.stratified_chains()[list(chains)]
    B = wl.inverter_batch(chain_ids=ids, mos_model=model)
    cfg = N.newton_config(**wl.TIGHT)
    nvin = 61
    for k, c in enumerate(B.circuits):
        sl = slice(k * nvin, (k + 1) * nvin)
        x0 = np.stack([B.x0[B.x0_off[i]:B.x0_off[i] + c.node_count]
                       for i in range(k * nvin, (k + 1) * nvin)])
        rs_o, it_o, x_o, xl_o = po.dc_sweep(c, 1, B.inst_val[sl], "nativeklu_exact", x0=x0,
                                            stop_on_failure=False, **NEWTON)
        g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
        r = dc_sweep(g, DeviceCircuit(c), cfg, 1, B.inst_val[sl], x0=x0, stop_on_failure=False)
        assert np.array_equal(r.reason, rs_o), (k, r.reason, rs_o)
        assert np.array_equal(r.iterations, it_o), (k, r.iterations, it_o)
        for q in np.flatnonzero(rs_o == 0):
            assert np.max(np.abs(r.x[q] - x_o[q])) <= 1e-12 * max(1.0, np.max(np.abs(x_o[q])))
        g.close()


def test_device_sweep_continuation_matches_oracle():
    """The reference's .dc exactly: each point from the previous point's
    solution (with its aux currents, which the convergence test then covers)
    and a stop at the first failure. A diode ladder's source swept up from
    0 V beside two resistor-loaded NMOS stages converges at every point; a
    reference-model inverter chain from the engine's zero start fails at the
    first point and the sweep ends there, on the device as in the oracle."""
    from rustspice_gb300 import circuits as cz
    from rustspice_gb300 import netlist as nl
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, dc_sweep
    deck = nl.compile_deck("""* resistor-loaded NMOS stages beside a diode ladder
VDD vdd 0 DC 1.8
VIN in 0 DC 0.9
RL1 vdd mid 20k
MN1 mid in 0 0 nch W=2u L=1u
RL2 vdd out 20k
MN2 out mid 0 0 nch W=2u L=1u
V1 a 0 DC 0.0
R1 a b 1k
D1 b 0 dx
R2 b c 2k
D2 c 0 dx
.model nch nmos level=1 vto=0.45 u0=400
.model dx d is=1e-14
.end
""")
    chain = cz.inverter_chain(24, 0.0, seed=3, chain_id=7, mos_model="reference")
    cfg = N.newton_config(**wl.TIGHT)
    for name, c, src, vals in (("ladder", deck.circuit, deck.device_names.index("V1"),
                                np.linspace(0.0, 1.0, 21)),
                               ("chain", chain, 1, cz.vin_points(61))):
        rs_o, it_o, x_o, xl_o = po.dc_sweep(c, src, vals, "nativeklu_exact", **NEWTON)
        g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
        r = dc_sweep(g, DeviceCircuit(c), cfg, src, vals)
        assert np.array_equal(r.reason, rs_o) and np.array_equal(r.iterations, it_o), name
        assert np.array_equal(r.x_len, xl_o)
        for q in np.flatnonzero(rs_o == 0):
            assert np.max(np.abs(r.x[q] - x_o[q])) <= 1e-12 * max(1.0, np.max(np.abs(x_o[q])))
        if name == "ladder":
            assert np.all(rs_o == 0)
        else:
            assert rs_o[0] == 1 and np.all(rs_o[1:] == -1)
        g.close()
