"""Seeded synthetic circuits in the device-list form the stamp compiler takes.

A circuit is a flat list of device instances in netlist order, the order the
reference engine stamps them (crates/sim-core/src/engine.rs:262-279). Node 0 is
ground and stays in the matrix (crates/sim-core/src/circuit.rs:31-57); one
auxiliary unknown is appended per voltage source, in device order
(crates/sim-core/src/stamp.rs:290, crates/sim-core/src/mna.rs:472-480).

Device parameter slots (``p[dev, 0:6]``):

=====  ==========================================================
R      p0 = resistance [ohm]
V      p0 = volts
I      p0 = amps
D      p0 = Is, p1 = N
M      p0 = is_pmos (0/1), p1 = vth0, p2 = u0, p3 = tox, p4 = W, p5 = L
C      p0 = capacitance [F]
MC     as M
=====  ==========================================================

``M`` is the reference's level-1 evaluator exactly (crates/sim-devices/src/
bsim/evaluate.rs:285-356). Its PMOS branch negates and swaps the terminals
into a frame where the stamped gm and gds are not the derivatives of the
stamped current, so Newton diverges on CMOS inverters from a zero start, and
its linear region omits the (1 + lambda vds) factor, so the current steps by
~2 % where the linear and saturation regions meet (Newton can cycle on that
step in a transient). ``MC`` ("consistent") keeps the reference's constants
(lambda 0.02, beta from u0 and tox) in the Shichman-Hodges form (the factor
in both regions), applies the polarity to every terminal voltage and swaps
the drain/source roles for vds < 0, so the current is continuous and the
stamp is its exact linearisation. The CMOS workloads use ``MC`` by default;
``mos_model="reference"`` selects ``M``.

Random numbers come from a counter-based splitmix64 stream, so a circuit
depends only on its seed and is identical on every host.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

DEV_R, DEV_V, DEV_I, DEV_D, DEV_M, DEV_C, DEV_MC = 0, 1, 2, 3, 4, 5, 6
NPARAM = 6

# Level-1 card. The reference does not parse KP (crates/sim-devices/src/bsim/
# mod.rs:83-388); its level-1 beta is u0 * 1e-4 * EPSILON_OX / tox
# (mod.rs:445, params.rs:10, 460-462), so KP is expressed through u0 with the
# default tox of 1.5e-8 m. LAMBDA is fixed at 0.02 inside the reference's
# level-1 evaluator, which matches the card's 0.02.
EPSILON_OX = 3.9 * 8.854e-12
TOX = 1.5e-8
KP_N, KP_P = 120e-6, 40e-6
U0_N = KP_N / (1e-4 * (EPSILON_OX / TOX))
U0_P = KP_P / (1e-4 * (EPSILON_OX / TOX))
W_N, W_P, L_CH = 1e-6, 2e-6, 1e-6


@dataclasses.dataclass
class Circuit:
    node_count: int                 # includes ground
    type: np.ndarray                # int32 [ndev]
    nodes: np.ndarray               # int32 [ndev, 4]
    p: np.ndarray                   # float64 [ndev, 6]
    name: str = ""

    @property
    def ndev(self) -> int:
        return int(self.type.shape[0])

    @property
    def n_aux(self) -> int:
        return int(np.count_nonzero(self.type == DEV_V))

    @property
    def n(self) -> int:
        """Matrix dimension: nodes (with ground) plus one aux per V source."""
        return self.node_count + self.n_aux

    def device_index(self, kind: int, k: int = 0) -> int:
        """Index of the k-th device of a kind."""
        return int(np.flatnonzero(self.type == kind)[k])


class _Dev:
    """Append-only device list builder."""

    def __init__(self) -> None:
        self.t: list[int] = []
        self.nd: list[tuple] = []
        self.p: list[tuple] = []

    def add(self, kind, nodes, params):
        nodes = tuple(nodes) + (0,) * (4 - len(nodes))
        params = tuple(params) + (0.0,) * (NPARAM - len(params))
        self.t.append(kind)
        self.nd.append(nodes)
        self.p.append(params)

    def build(self, node_count, name="") -> Circuit:
        return Circuit(node_count, np.asarray(self.t, np.int32),
                       np.asarray(self.nd, np.int32).reshape(-1, 4),
                       np.asarray(self.p, np.float64).reshape(-1, NPARAM), name)


# ---------------------------------------------------------------- PRNG
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


class Stream:
    """Counter-based splitmix64: draw i of stream (seed, sub) is mix(key + i*phi)."""

    def __init__(self, seed: int, sub: int = 0) -> None:
        key = _mix64(np.array([(seed * 0x9E3779B97F4A7C15 + sub) & 0xFFFFFFFFFFFFFFFF],
                              dtype=np.uint64))[0]
        self.key = np.uint64(key)
        self.i = 0

    def bits(self, k: int) -> np.ndarray:
        idx = np.arange(self.i + 1, self.i + 1 + k, dtype=np.uint64)
        self.i += k
        with np.errstate(over="ignore"):
            return _mix64(self.key + idx * np.uint64(0x9E3779B97F4A7C15))

    def uniform(self, k: int) -> np.ndarray:
        """k doubles in [0, 1) with 53 random bits."""
        return (self.bits(k) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def integers(self, lo: int, hi: int, k: int) -> np.ndarray:
        """k integers in [lo, hi] inclusive."""
        return lo + np.floor(self.uniform(k) * (hi - lo + 1)).astype(np.int64)

    def normal(self, k: int) -> np.ndarray:
        """Box-Muller normals."""
        u1 = self.uniform(k)
        u2 = self.uniform(k)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)

    def log_uniform_r(self, k: int) -> np.ndarray:
        """R = 100 * 10^(2u): log-uniform 100 ohm .. 10 kohm."""
        return 100.0 * np.power(10.0, 2.0 * self.uniform(k))

    def choice(self, n: int, k: int) -> np.ndarray:
        """k distinct values from range(n) (partial Fisher-Yates)."""
        a = np.arange(n, dtype=np.int64)
        r = self.uniform(k)
        for i in range(k):
            j = i + int(r[i] * (n - i))
            a[i], a[j] = a[j], a[i]
        return a[:k].copy()


# ---------------------------------------------------------------- meshes
def _mesh_resistors(dev: _Dev, rows: int, cols: int, first_node: int, rs: Stream):
    """Horizontal then vertical neighbour resistors of a rows x cols grid."""
    nid = lambda r, c: first_node + r * cols + c  # noqa: E731
    nh = rows * (cols - 1)
    nv = (rows - 1) * cols
    rv = rs.log_uniform_r(nh + nv)
    k = 0
    for r in range(rows):
        for c in range(cols - 1):
            dev.add(DEV_R, (nid(r, c), nid(r, c + 1)), (rv[k],))
            k += 1
    for r in range(rows - 1):
        for c in range(cols):
            dev.add(DEV_R, (nid(r, c), nid(r + 1, c)), (rv[k],))
            k += 1
    return nid


def mesh_dc(side: int = 32, ndiodes: int = 64, seed: int = 1) -> Circuit:
    """Resistor mesh with a corner source, a grounded far corner and diodes.

    ``side`` x ``side`` nodes numbered 1..side^2 row-major; R log-uniform
    100 ohm .. 10 kohm between neighbours; 1.0 V source from node (0,0) to
    ground; node (side-1, side-1) to ground through 1 kohm; ``ndiodes`` diodes
    (Is=1e-14, N=1) from distinct seeded nodes to ground. For side=32 this is
    the 1024-node DC operating-point case: n = 1026, 8,201 raw CSC entries.
    """
    rs = Stream(seed, 1)
    dev = _Dev()
    nid = _mesh_resistors(dev, side, side, 1, rs)
    dev.add(DEV_R, (nid(side - 1, side - 1), 0), (1000.0,))
    dev.add(DEV_V, (nid(0, 0), 0), (1.0,))
    dn = Stream(seed, 2).choice(side * side, ndiodes) + 1
    for a in dn:
        dev.add(DEV_D, (int(a), 0), (1e-14, 1.0))
    return dev.build(side * side + 1, f"mesh{side}x{side}_d{ndiodes}_s{seed}")


# ---------------------------------------------------------------- inverters
def bordered_meshes(nblocks: int = 64, nborder: int = 1024, side_lo: int = 30,
                    side_hi: int = 50, ndiodes: int = 32, seed: int = 2):
    """Bordered-block-diagonal DC case: ``nblocks`` square resistor meshes
    (side uniform in [side_lo, side_hi], R log-uniform 100 ohm..10 kohm),
    ``ndiodes`` diodes per mesh from seeded mesh nodes to ground, and
    ``nborder`` border nodes, each tied by 4..8 resistors of 1 kohm to
    seeded nodes of seeded meshes. The supply is a Norton source on border
    node 0: 12 mA in parallel with 100 ohm to ground (1.2 V open circuit); a
    current source keeps the border free of voltage-source rows, whose zero
    diagonal the reference's no-pivot Schur factorisation cannot take.

    A border node ties to a mesh node at most once, and the diodes of a mesh
    sit on distinct nodes, so no block-border entry is duplicated (the
    reference's Schur assembly keeps only the last of duplicated entries of
    R, bbd_solver.rs:788, 867).

    Returns (circuit, assignment, nblocks): assignment[i] is node i's mesh,
    -1 for ground and the border nodes (the known partition).
    """
    rs = Stream(seed, 21)
    sides = rs.integers(side_lo, side_hi, nblocks)
    dev = _Dev()
    first = 1
    starts, sizes = [], []
    for k in range(nblocks):
        s = int(sides[k])
        _mesh_resistors(dev, s, s, first, Stream(seed, 1000 + k))
        dn = Stream(seed, 3000 + k).choice(s * s, ndiodes) + first
        for a in dn:
            dev.add(DEV_D, (int(a), 0), (1e-14, 1.0))
        starts.append(first)
        sizes.append(s * s)
        first += s * s
    b0 = first
    ties = Stream(seed, 22)
    nt = ties.integers(4, 8, nborder)
    blk = Stream(seed, 23)
    pos = Stream(seed, 24)
    for j in range(nborder):
        kk = blk.integers(0, nblocks - 1, int(nt[j]))
        uu = pos.uniform(int(nt[j]))
        seen = set()
        for k, u in zip(kk, uu):
            node = starts[int(k)] + int(u * sizes[int(k)])
            if node in seen:  # one tie per (border node, mesh node): no duplicate entries
                continue
            seen.add(node)
            dev.add(DEV_R, (b0 + j, node), (1000.0,))
    dev.add(DEV_I, (0, b0), (12e-3,))
    dev.add(DEV_R, (b0, 0), (100.0,))
    nc = b0 + nborder
    c = dev.build(nc, f"bbd{nblocks}_b{nborder}_s{seed}")
    assignment = -np.ones(nc, np.int64)
    for k in range(nblocks):
        assignment[starts[k]:starts[k] + sizes[k]] = k
    return c, assignment, nblocks


def _mos(model: str) -> int:
    if model == "consistent":
        return DEV_MC
    if model == "reference":
        return DEV_M
    raise ValueError(f"unknown MOSFET model {model!r}")


def _inverter_params(rs: Stream, k: int):
    vto_n = 0.45 + 0.03 * rs.normal(k)
    vto_p = -0.45 + 0.03 * rs.normal(k)
    wj_n = rs.uniform(k) * 0.1 + 0.95
    wj_p = rs.uniform(k) * 0.1 + 0.95
    return vto_n, vto_p, wj_n, wj_p


def inverter_chain(stages: int, vin: float = 0.0, seed: int = 1, chain_id: int = 0,
                   c_load: float = 20e-15, mos_model: str = "consistent") -> Circuit:
    """CMOS inverter chain on the level-1 card.

    Nodes: 0 ground, 1 VDD (1.2 V), 2 input, 3..stages+2 the stage outputs.
    Devices: VDD source, input source, then per stage NMOS (d=out, g=in,
    s=b=gnd), PMOS (d=out, g=in, s=b=VDD) and the load capacitor out->gnd.
    VTO_n ~ N(0.45, 0.03), VTO_p ~ N(-0.45, 0.03), W jittered U(0.95, 1.05).
    """
    rs = Stream(seed, 1000 + chain_id)
    vto_n, vto_p, wj_n, wj_p = _inverter_params(rs, stages)
    dev = _Dev()
    dev.add(DEV_V, (1, 0), (1.2,))
    dev.add(DEV_V, (2, 0), (vin,))
    for s in range(stages):
        gin = 2 + s
        out = 3 + s
        dev.add(_mos(mos_model), (out, gin, 0, 0), (0.0, vto_n[s], U0_N, TOX, W_N * wj_n[s], L_CH))
        dev.add(_mos(mos_model), (out, gin, 1, 1), (1.0, vto_p[s], U0_P, TOX, W_P * wj_p[s], L_CH))
        dev.add(DEV_C, (out, 0), (c_load,))
    return dev.build(stages + 3, f"inv{stages}_c{chain_id}_s{seed}")


def chain_lengths(count: int = 4096, lo: int = 8, hi: int = 256, seed: int = 3) -> np.ndarray:
    """Uneven stage counts, uniform in [lo, hi]."""
    return Stream(seed, 7).integers(lo, hi, count)


def vin_points(npts: int = 61, vmax: float = 1.2) -> np.ndarray:
    """Input sweep values 0, 0.02, ..., 1.2."""
    return np.array([i * (vmax / (npts - 1)) for i in range(npts)], dtype=np.float64)


def ring_oscillator(stages: int, seed: int = 5, ring_id: int = 0, c_node: float = 10e-15,
                    c_jitter: float = 0.1, mos_model: str = "consistent") -> Circuit:
    """CMOS ring oscillator of odd length on the level-1 card.

    Nodes: 0 ground, 1 VDD, 2..stages+1 the ring nodes; stage k drives node
    2+k from node 2+(k-1 mod stages). Per node a capacitor of
    ``c_node * U(1-c_jitter, 1+c_jitter)`` to ground.
    """
    rs = Stream(seed, 5000 + ring_id)
    vto_n, vto_p, wj_n, wj_p = _inverter_params(rs, stages)
    cj = 1.0 - c_jitter + 2.0 * c_jitter * rs.uniform(stages)
    dev = _Dev()
    dev.add(DEV_V, (1, 0), (1.2,))
    for s in range(stages):
        gin = 2 + (s - 1) % stages
        out = 2 + s
        dev.add(_mos(mos_model), (out, gin, 0, 0), (0.0, vto_n[s], U0_N, TOX, W_N * wj_n[s], L_CH))
        dev.add(_mos(mos_model), (out, gin, 1, 1), (1.0, vto_p[s], U0_P, TOX, W_P * wj_p[s], L_CH))
        dev.add(DEV_C, (out, 0), (c_node * cj[s],))
    return dev.build(stages + 2, f"ring{stages}_r{ring_id}_s{seed}")


def mesh_with_inverters(side: int = 120, ninv: int = 1000, seed: int = 4,
                        mos_model: str = "consistent") -> Circuit:
    """Resistor mesh driving level-1 inverters (the 20k-node adjoint case).

    ``side`` x ``side`` mesh (nodes 1..side^2, R log-uniform 100 ohm..10 kohm),
    a 1.2 V supply node driving the mesh corner (0,0), node (side-1,side-1) to
    ground through 1 kohm; ``ninv`` inverters whose gates are distinct seeded
    mesh nodes and whose outputs are new nodes, each loaded by 10 kohm to
    ground. For side=120, ninv=1000 this has 14,400 mesh nodes, 28,560 mesh
    resistors and 15,402 nodes in all.
    """
    rs = Stream(seed, 1)
    dev = _Dev()
    nid = _mesh_resistors(dev, side, side, 2, rs)
    nmesh = side * side
    vdd = 1
    dev.add(DEV_V, (vdd, 0), (1.2,))
    dev.add(DEV_R, (vdd, nid(0, 0)), (100.0,))
    dev.add(DEV_R, (nid(side - 1, side - 1), 0), (1000.0,))
    gates = Stream(seed, 2).choice(nmesh, ninv) + 2
    p = Stream(seed, 3)
    vto_n, vto_p, wj_n, wj_p = _inverter_params(p, ninv)
    out0 = 2 + nmesh
    for k in range(ninv):
        out = out0 + k
        dev.add(_mos(mos_model), (out, int(gates[k]), 0, 0), (0.0, vto_n[k], U0_N, TOX, W_N * wj_n[k], L_CH))
        dev.add(_mos(mos_model), (out, int(gates[k]), vdd, vdd), (1.0, vto_p[k], U0_P, TOX, W_P * wj_p[k], L_CH))
        dev.add(DEV_R, (out, 0), (10000.0,))
    return dev.build(out0 + ninv, f"mesh{side}_inv{ninv}_s{seed}")


def output_nodes(c: Circuit, count: int = 256, seed: int = 4) -> np.ndarray:
    """Seeded distinct non-ground nodes for the adjoint loss."""
    return Stream(seed, 9).choice(c.node_count - 1, count) + 1
