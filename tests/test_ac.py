"""AC small-signal sweep: the oracle's restatement of the reference's .ac on
analytic cases (no GPU), and the device sweep against the oracle (GPU)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import netlist as nl

RC = """* RC lowpass, 1 kOhm and 1 uF (fc = 159.15 Hz)
V1 in 0 DC 0 AC 1 0
R1 in out 1k
C1 out 0 1u
.ac dec 10 1 1meg
.end
"""


def _ladder(sections=100, seed=3):
    """An RC ladder driven by an AC source: n = sections + 3 (ground, the
    sections + 1 ladder nodes, the source's aux)."""
    rng = np.random.default_rng(seed)
    lines = ["V1 n0 0 DC 0 AC 1 30"]
    for k in range(sections):
        lines.append(f"R{k} n{k} n{k + 1} {rng.uniform(100, 1000):.6g}")
        lines.append(f"C{k} n{k + 1} 0 {rng.uniform(1e-12, 1e-9):.6g}")
    return nl.compile_deck("\n".join(lines) + "\n")


def _amp():
    """A resistor-loaded NMOS stage with a coupling capacitor and a load
    capacitor, then a diode-loaded divider, at its own DC operating point."""
    return nl.compile_deck("""VDD vdd 0 DC 1.8
VB bias 0 DC 0.9
VS src 0 DC 0 AC 1 0
RB bias gate 100k
CIN src gate 1n
RL vdd out 20k
M1 out gate 0 0 nch W=2u L=1u
CL out 0 100f
VD a 0 DC 1.0
R1 a b 1k
D1 b 0 dx
C2 b 0 10p
.model nch nmos level=1 vto=0.45 u0=400
.model dx d is=1e-14
.option reltol=1e-10 vntol=1e-12 itl1=200
""")


def test_netlist_ac_fields():
    d = nl.compile_deck(RC)
    assert d.circuit.p[0, :3].tolist() == [0.0, 1.0, 0.0]
    d2 = nl.compile_deck("I1 a 0 DC 1m AC 2 -45\nR1 a 0 1k\n")
    assert d2.circuit.p[0, :3].tolist() == [1e-3, 2.0, -45.0]


def test_oracle_rc_lowpass_analytic():
    from rustspice_gb300.solver import frequency_sweep
    d = nl.compile_deck(RC)
    f = frequency_sweep("dec", 10, 1.0, 1e6)
    assert len(f) == 61 and f[0] == 1.0 and abs(f[-1] - 1e6) < 1e-6
    x = po.ac_sweep(d.circuit, np.zeros(d.circuit.n), f)
    h = x[:, d.node_names.index("out")]
    w = 2 * np.pi * f * 1e3 * 1e-6
    want = 1.0 / (1.0 + 1j * w)
    assert np.max(np.abs(h - want)) < 1e-12
    assert abs(abs(h[22]) - 1.0 / np.sqrt(1 + (2 * np.pi * f[22] * 1e-3) ** 2)) < 1e-12


def test_oracle_ladder_against_numpy():
    d = _ladder(20)
    c = d.circuit
    f = np.array([10.0, 1e5, 3e7])
    x = po.ac_sweep(c, np.zeros(c.n), f)
    # the same system by nodal analysis with numpy
    for k, fk in enumerate(f):
        w = 2 * np.pi * fk
        n = c.n
        y = np.zeros((n, n), complex)
        b = np.zeros(n, complex)
        aux = c.node_count
        for dv in range(c.ndev):
            a, bb = c.nodes[dv, :2]
            if c.type[dv] == cz.DEV_R:
                g = 1.0 / c.p[dv, 0]
            elif c.type[dv] == cz.DEV_C:
                g = 1j * w * c.p[dv, 0]
            else:
                y[a, aux] += 1; y[bb, aux] -= 1; y[aux, a] += 1; y[aux, bb] -= 1
                b[aux] = c.p[dv, 1] * np.exp(1j * np.deg2rad(c.p[dv, 2]))
                aux += 1
                continue
            y[a, a] += g; y[bb, bb] += g; y[a, bb] -= g; y[bb, a] -= g
        y[0, :] = 0; y[0, 0] = 1; b[0] = 0
        ref = np.linalg.solve(y, b)
        assert np.max(np.abs(x[k] - ref)) <= 1e-9 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_device_ac_sweep_matches_oracle():
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import (DeviceCircuit, GpuKluSolver, ac_sweep,
                                        frequency_sweep, newton_dc)
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    # linear ladder: no device evaluation, the same arithmetic bit for bit
    d = _ladder(100)
    f = frequency_sweep("dec", 20, 1.0, 1e9)
    xo = po.ac_sweep(d.circuit, np.zeros(d.circuit.n), f)
    xg = ac_sweep(g, DeviceCircuit(d.circuit), np.zeros(d.circuit.n), f)
    assert np.array_equal(xg, xo)
    # amplifier at its operating point (the device stamp's exp may differ from
    # the host's by an ulp, so the bar is relative 1e-12)
    d = _amp()
    res = newton_dc(g, DeviceCircuit(d.circuit), N.newton_config(**d.newton_options()))
    assert res.converged
    f = frequency_sweep("dec", 10, 10.0, 1e10)
    xo = po.ac_sweep(d.circuit, res.x, f)
    xg = ac_sweep(g, DeviceCircuit(d.circuit), res.x, f)
    assert np.max(np.abs(xg - xo)) <= 1e-12 * np.max(np.abs(xo))
    # beyond one block's shared memory (n = 203 and 603): the matrices in
    # global scratch, the same arithmetic bit for bit
    for sections, nf in ((200, 24), (600, 5)):
        big = _ladder(sections, seed=sections)
        fb = frequency_sweep("dec", 3, 1.0, 1e8)[:nf]
        xo = po.ac_sweep(big.circuit, np.zeros(big.circuit.n), fb)
        xg = ac_sweep(g, DeviceCircuit(big.circuit), np.zeros(big.circuit.n), fb)
        assert xg.shape == (len(fb), sections + 3) and np.array_equal(xg, xo)
    # size limit (n = sections + 3: ground, sections + 1 nodes, the aux)
    huge = _ladder(N.AC_MAX_N)
    with pytest.raises(Exception):
        ac_sweep(g, DeviceCircuit(huge.circuit), np.zeros(huge.circuit.n), f[:2])
