"""The batched headline workload against the oracle at scale.

The sample is stratified over the 4096-chain inverter workload: the first
chain of every stage count 8..256 (249 chains), each at all 61 input points
of the 0..1.2 V sweep, 15,189 DC operating points. Both MOSFET models run:

* ``reference`` - the reference's own level-1 evaluator
  (crates/sim-devices/src/bsim/evaluate.rs:285-356), whose PMOS
  linearisation is not the derivative of its current; from the logic-level
  nodeset about 69 % of the instances converge.
* ``consistent`` - the same card with a consistent linearisation (the bench
  headline's model); about 98.6 % converge.

The instances that do not converge are the reference's Newton running out of
iterations (crates/sim-core/src/newton.rs:93-107: the damping factor only
halves, to its 0.1 floor, and the level-1 steps are not limited), so the
converged set is part of the result: the device batch must converge on the
same instances as the oracle, agree on the iteration count, and match every
converged operating point to 1e-10 relative. The batch kernels contract
multiply-adds and use a one-step reciprocal, so an iterate that lands on the
tolerance may take one iteration more or less: at most 1 % of the converged
instances may differ in iteration count, and at most 0.05 % in the converged
set (none differed when this was written).
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


@pytest.mark.parametrize("model,frac", [("consistent", (0.98, 0.99)),
                                        ("reference", (0.6, 0.75))])
def test_stratified_batch_matches_oracle(model, frac):
    B, bt, it, rs, x, it_o, rs_o, x_o = _run(model)
    conv_o = rs_o == 0
    conv = rs == 0
    f = float(np.mean(conv_o))
    print(f"{model}: {B.ninst} instances, oracle converged {f:.4f}, device {np.mean(conv):.4f}, "
          f"oracle iterations {int(it_o.sum())}, device {int(it.sum())}")
    assert frac[0] <= f <= frac[1], f
    assert np.mean(conv != conv_o) <= 5e-4, np.flatnonzero(conv != conv_o)[:20]
    both = conv & conv_o
    agree = float(np.mean(it[both] == it_o[both]))
    assert agree >= 0.99, agree
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
    assert worst <= 1e-10
    # the failures sit where the first stage switches: by input point
    bad_vin = np.unique(B.vin[~conv_o])
    print(f"{model}: input points with a non-converged instance: {bad_vin.round(2).tolist()}")
