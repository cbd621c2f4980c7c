"""The R/V/I/D/M/C netlist reader against the reference's reading of decks.

Small decks written here exercise each rule (numbers, continuation lines,
parameters, models, MOSFET level and polarity, node numbering); the
reference's own fixture decks, where the reference tree is present, are read
and solved with the oracle for the answers its tests expect. No GPU.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import netlist as nl

REF = "/root/reference/tests/fixtures/netlists"
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("tok,val", [("1k", 1e3), ("2.2MEG", 2.2e6), ("10u", 1e-5), ("3m", 3e-3),
                                     ("1e-3", 1e-3), ("5f", 5e-15), ("-4.7n", -4.7e-9),
                                     (".5", 0.5), ("7", 7.0), ("1g", 1e9), ("2t", 2e12)])
def test_numbers(tok, val):
    assert nl.parse_number(tok) == pytest.approx(val, rel=1e-15)


@pytest.mark.parametrize("tok", ["abc", "1x", "", "k", "1e"])
def test_not_numbers(tok):
    assert nl.parse_number(tok) is None


def test_divider_with_continuation_and_options():
    deck = nl.compile_deck("""* divider
V1 in 0
+ DC 3
  R1 in out 1k
R2 out 0 2k

.option reltol=1e-6 vntol=1e-9 itl1=50
.op
.end
""")
    c = deck.circuit
    assert deck.node_names == ["0", "in", "out"] and deck.device_names == ["V1", "R1", "R2"]
    assert list(c.type) == [cz.DEV_V, cz.DEV_R, cz.DEV_R]
    assert c.nodes[0, :2].tolist() == [1, 0] and c.p[0, 0] == 3.0
    assert c.p[1, 0] == 1e3 and c.p[2, 0] == 2e3
    assert deck.newton_options() == {"max_iters": 50, "abs_tol": 1e-9, "rel_tol": 1e-6,
                                     "gmin": 1e-12}
    r, it, x = po.dc_op(c, "nativeklu", **deck.newton_options())
    assert r == "converged" and abs(x[2] - 2.0) < 1e-9


def test_diode_and_level1_mosfets():
    deck = nl.compile_deck("""* inverter and a diode
VDD vdd 0 DC 1.2
VIN in 0 0.3
MN out in 0 0 nch W=2u L=1u
MP out in vdd vdd pch W=4u L=1u
D1 out 0 dx
.model nch nmos (level=1 vto=0.45 u0=400 tox=1.5e-8)
.model pch pmos level=1 vto=-0.45 u0=150 type=pmos
.model dx d is=2e-15 n=1.5
.end
""")
    c = deck.circuit
    mn, mp, d1 = 2, 3, 4
    assert list(c.type[[mn, mp, d1]]) == [cz.DEV_M, cz.DEV_M, cz.DEV_D]
    assert c.p[mn].tolist() == [0.0, 0.45, 400.0, 1.5e-8, 2e-6, 1e-6]
    assert c.p[mp].tolist() == [1.0, -0.45, 150.0, 1.5e-8, 4e-6, 1e-6]
    assert c.p[d1, :2].tolist() == [2e-15, 1.5]
    r, it, x = po.dc_op(c, "nativeklu_exact", max_iters=200, abs_tol=1e-12, rel_tol=1e-10)
    assert r == "converged"


def test_reference_polarity_rule():
    """A model card's own type word does not make a PMOS; a type parameter or
    a pmos key does (the reference's rule)."""
    base = "V1 d 0 1\nV2 g 0 1\nM1 d g 0 0 mx W=1u L=1u\n.model mx pmos level=1 %s\n"
    assert nl.compile_deck(base % "").circuit.p[2, 0] == 0.0
    assert nl.compile_deck(base % "type=pmos").circuit.p[2, 0] == 1.0
    assert nl.compile_deck(base % "pmos=1").circuit.p[2, 0] == 1.0


def test_three_terminal_mosfet_and_defaults():
    c = nl.compile_deck("M1 d g s mx\n.model mx nmos level=1\n").circuit
    assert c.nodes[0].tolist() == [1, 2, 3, 0]
    assert c.p[0].tolist() == [0.0, 0.7, 500.0, cz.TOX, 1e-6, 1e-6]


def test_ic_nodes_number_first():
    deck = nl.compile_deck("R1 a b 1k\n.ic v(b)=0.5\n")
    assert deck.node_names == ["0", "b", "a"]
    assert deck.transient_x0().tolist() == [0.0, 0.5, 0.0]


@pytest.mark.parametrize("text", ["M1 d g 0 0 mx\n.model mx nmos vto=0.4\n",  # level 49
                                  "L1 a 0 1n\n", "X1 a b sub\n", "V1 a 0 PULSE(0 1 0 1n)\n",
                                  ".include other.cir\n", "Q1 c b e qx\n", "+ R1 a 0 1\n"])
def test_outside_the_path(text):
    with pytest.raises(nl.NetlistError):
        nl.compile_deck(text)


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
def test_reference_fixture_decks():
    # the reference's end-to-end divider: vin = 1, vout = 2/3
    deck = nl.load(os.path.join(REF, "basic_dc.cir"))
    r, it, x = po.dc_op(deck.circuit, "nativeklu", **deck.newton_options())
    names = deck.node_names
    assert r == "converged"
    assert abs(x[names.index("in")] - 1.0) < 1e-6
    assert abs(x[names.index("out")] - 2.0 / 3.0) < 1e-6
    # the BeGAN grid reads into the committed fixture's device list
    z = np.load(os.path.join(GOLD, "began_small_pgrid.npz"))
    c = nl.load(os.path.join(REF, "began_small_pgrid.sp")).circuit
    assert c.node_count == int(z["node_count"])
    assert np.array_equal(c.type, z["type"]) and np.array_equal(c.nodes, z["nodes"])
    assert np.array_equal(c.p, z["p"])
    # the BSIM3 deck is outside this path
    with pytest.raises(nl.NetlistError):
        nl.load(os.path.join(REF, "nmos_dc.cir"))


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
def test_reference_include_fixture():
    """The reference's include test deck (netlist_tests.rs:111-127): the
    child's resistor is read in place of the .include line."""
    deck = nl.load(os.path.join(REF, "include_parent.cir"))
    assert deck.device_names == ["R1", "R2"]
    assert deck.node_names == ["0", "in", "out"]
    assert deck.circuit.nodes[:, :2].tolist() == [[1, 2], [2, 0]]
    assert deck.circuit.p[:, 0].tolist() == [1000.0, 2000.0]


def test_includes(tmp_path):
    """Includes resolve against the including file's directory, recursively,
    with quotes stripped; a cycle, a missing file and a missing path are
    errors."""
    sub = tmp_path / "lib"
    sub.mkdir()
    (sub / "leaf.cir").write_text("R3 b 0 3k\n")
    (sub / "mid.cir").write_text("R2 a b 2k\n.INCLUDE leaf.cir\n")
    (tmp_path / "top.cir").write_text('* top\nV1 a 0 DC 1\n.include "lib/mid.cir"\nR1 a 0 1k\n.end\n')
    deck = nl.load(str(tmp_path / "top.cir"))
    assert deck.device_names == ["V1", "R2", "R3", "R1"]
    assert deck.circuit.p[1:, 0].tolist() == [2000.0, 3000.0, 1000.0]
    (tmp_path / "a.cir").write_text("R1 x 0 1\n.include b.cir\n")
    (tmp_path / "b.cir").write_text("R2 x 0 1\n.include ./a.cir\n")
    with pytest.raises(nl.NetlistError, match="circular"):
        nl.load(str(tmp_path / "a.cir"))
    (tmp_path / "c.cir").write_text("R1 x 0 1\n.include nothere.cir\n")
    with pytest.raises(nl.NetlistError, match="cannot read file"):
        nl.load(str(tmp_path / "c.cir"))
    (tmp_path / "d.cir").write_text("R1 x 0 1\n.include\n")
    with pytest.raises(nl.NetlistError, match="missing path"):
        nl.load(str(tmp_path / "d.cir"))
