"""The seeded workloads the bench and the parity tests run.

``inverter_batch`` is the batched Monte-Carlo DC case: uneven CMOS inverter
chains (8..256 stages), each solved at every input voltage of a 0..1.2 V
sweep as an independent DC operating point. The reference's Newton
(crates/sim-core/src/newton.rs:65-117) has no device limiting, so from the
engine's zero start it diverges on CMOS chains; each instance therefore
starts from a logic-level nodeset: every stage output at the rail an ideal
inverter with threshold ``vm`` would give. The instance's Newton then runs
exactly as the reference's.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import circuits as cz

VDD = 1.2


def chain_nodeset(stages: int, vin: float, vm: float = 0.585) -> np.ndarray:
    """Logic-level initial iterate of an inverter chain (node order of
    ``circuits.inverter_chain``)."""
    x = np.zeros(stages + 3)
    x[1] = VDD
    x[2] = vin
    v = vin
    for k in range(stages):
        v = VDD if v < vm else 0.0
        x[3 + k] = v
    return x


@dataclasses.dataclass
class InverterBatch:
    circuits: list
    inst_circ: np.ndarray
    inst_dev: np.ndarray
    inst_val: np.ndarray
    x0: np.ndarray
    x0_off: np.ndarray
    stages: np.ndarray
    vin: np.ndarray

    @property
    def ninst(self) -> int:
        return len(self.inst_circ)


def inverter_batch(nchains: int = 4096, nvin: int = 61, seed: int = 3,
                   lo: int = 8, hi: int = 256, mos_model: str = "consistent",
                   chain_ids=None) -> InverterBatch:
    """nchains chains x nvin input points; instance i = (chain i // nvin,
    vin point i % nvin). The input source is device 1 of every chain.
    chain_ids: only these chains of the nchains-chain workload (each keeps
    its stage count and its seeded parameters), in the order given."""
    stages = cz.chain_lengths(nchains, lo, hi, seed)
    ids = np.arange(nchains) if chain_ids is None else np.asarray(chain_ids, np.int64)
    stages = stages[ids]
    nchains = len(ids)
    vins = cz.vin_points(nvin)
    circuits = [cz.inverter_chain(int(s), 0.0, seed=seed, chain_id=int(i), mos_model=mos_model)
                for i, s in zip(ids, stages)]
    ninst = nchains * nvin
    inst_circ = np.repeat(np.arange(nchains, dtype=np.int64), nvin)
    inst_dev = np.full(ninst, 1, np.int64)
    inst_val = np.tile(vins, nchains)
    sizes = np.repeat(stages + 3, nvin)
    x0_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    x0 = np.concatenate([chain_nodeset(int(stages[i // nvin]), float(inst_val[i]))
                         for i in range(ninst)])
    return InverterBatch(circuits, inst_circ, inst_dev, inst_val, x0, x0_off, stages,
                         inst_val.copy())


def stratified_chains(nchains: int = 4096, seed: int = 3, lo: int = 8, hi: int = 256):
    """Ids of the first chain of every stage count lo..hi in the nchains-chain
    workload: a sample of it that covers each chain length once."""
    stages = cz.chain_lengths(nchains, lo, hi, seed)
    ids = []
    for s in range(lo, hi + 1):
        hit = np.flatnonzero(stages == s)
        if len(hit) == 0:
            raise ValueError(f"no chain of {s} stages among {nchains}")
        ids.append(int(hit[0]))
    return np.asarray(ids, np.int64)


# Newton settings of the parity and bench runs: the engine's option names
# (crates/sim-core/src/engine.rs:987-999) with tolerances tightened so the
# converged iterate's residual is at the FP64 floor.
TIGHT = dict(max_iters=100, abs_tol=1e-12, rel_tol=1e-10, gmin=1e-12, gmin_steps=0,
             source_steps=0, damping=1.0, damping_min=0.1)


# ---------------------------------------------------------------- rings
RING_DT = 1e-12         # backward-Euler step [s]
RING_STEPS = 2000
RING_CKPT = 50          # checkpoint interval of the adjoint
RING_TARGET = 0.6       # loss target of ring node 0 [V]
RING_PROBE = 2          # ring node 0 (node 1 is VDD)


def ring_stages(count: int = 1024, seed: int = 11) -> np.ndarray:
    """Uneven odd ring lengths in 11..101."""
    return 2 * cz.Stream(seed, 13).integers(5, 50, count) + 1


def ring_initial_state(c: cz.Circuit, vdd: float = 1.2) -> np.ndarray:
    """Logic levels alternating around the ring, VDD on node 1. With an odd
    length the first stage's input and output agree, which starts the
    oscillation (the `.ic` of a ring oscillator)."""
    stages = c.node_count - 2
    x = np.zeros(c.node_count)
    x[1] = vdd
    for s in range(stages):
        x[2 + s] = vdd if s % 2 == 0 else 0.0
    return x


@dataclasses.dataclass
class RingBatch:
    circuits: list
    x_init: np.ndarray      # concatenated initial states
    x_off: np.ndarray       # per instance offset into x_init

    @property
    def ninst(self) -> int:
        return len(self.circuits)


def ring_batch(count: int = 1024, seed: int = 5) -> RingBatch:
    """1024 CMOS rings (level-1 card, 10 fF per node with +-10 % jitter), one
    instance per ring."""
    stages = ring_stages(count)
    circuits = [cz.ring_oscillator(int(s), seed=seed, ring_id=i) for i, s in enumerate(stages)]
    xs = [ring_initial_state(c) for c in circuits]
    off = np.zeros(count, np.int64)
    off[1:] = np.cumsum([len(x) for x in xs])[:-1]
    return RingBatch(circuits, np.concatenate(xs), off)


def bordered_nodeset(c: cz.Circuit, v: float = 0.55) -> np.ndarray:
    """Initial iterate of the bordered-mesh case: every node but ground at
    0.55 V, inside the diodes' conduction knee (a `.nodeset`). From the zero
    start the first linear solve lifts the unloaded meshes to the supply
    voltage and the unlimited diode exponentials (the reference evaluates
    them at the raw iterate) stall Newton; the reference's source stepping
    would not help, because its schedule starts at scale 0 and returns the
    first converged step (crates/sim-core/src/newton.rs:164-179)."""
    x = np.full(c.node_count, v)
    x[0] = 0.0
    return x


# Adaptive transient workload: inverter chains of seeded lengths (the C3
# card, 20 fF per stage) driven by a 0 -> 1.2 V pulse train on the input
# source (device 1), from the chains' logic-level nodeset at Vin = 0.
ATRAN_TSTEP = 10e-12
ATRAN_TSTOP = 4e-9
ATRAN_PULSE = dict(v1=0.0, v2=1.2, td=0.1e-9, tr=50e-12, tf=50e-12, pw=0.95e-9, per=2e-9)


@dataclasses.dataclass
class AdaptiveBatch:
    circuits: list
    waves: list      # per circuit {device: Waveform}
    x_ic: list       # per circuit initial guess of the DC point
    probe: np.ndarray


def adaptive_batch(count: int = 1024, seed: int = 13, lo: int = 8, hi: int = 64) -> AdaptiveBatch:
    from . import waveforms as wf
    stages = cz.chain_lengths(count, lo, hi, seed)
    circuits, waves, xs, probe = [], [], [], []
    for i, s in enumerate(stages):
        c = cz.inverter_chain(int(s), 0.0, seed=seed, chain_id=i)
        circuits.append(c)
        waves.append({1: wf.pulse(**ATRAN_PULSE)})
        xs.append(chain_nodeset(int(s), 0.0))
        probe.append(c.node_count - 1)
    return AdaptiveBatch(circuits, waves, xs, np.asarray(probe, np.int64))
