"""The R/V/I/D/M/C netlist reader against the reference's reading of decks.

Small decks written here exercise each rule (numbers, continuation lines,
parameters, models, MOSFET level and polarity, node numbering); the
reference's own fixture decks (copied into tests/golden/decks by
tests/golden/make_golden.py) are read and solved with the oracle for the
answers its tests expect. No GPU.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import netlist as nl

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF = os.path.join(GOLD, "decks")


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


def _elab(text):
    stmts, errors = nl.parse(text)
    assert not errors
    return nl.elaborate(stmts)[1]


@pytest.mark.parametrize("text,name,args", [
    # crates/sim-core/tests/netlist_tests.rs:80-90, 93-100, 103-109, 131-137, 148-154,
    # 157-163, 186-193, 321-327, 330-340
    (".subckt buf in out\nR1 in out 1k\n.ends\nX1 a b buf\n.end\n", "X1.R1", ["a", "b", "1000"]),
    (".param RVAL=5k\nR1 in out RVAL\n.end\n", "R1", ["in", "out", "5000"]),
    (".subckt buf in out RVAL=1k\nR1 in out RVAL\n.ends\nX1 a b buf RVAL=2k\n.end\n", "X1.R1",
     ["a", "b", "2000"]),
    (".param RVAL=1k+1k\nR1 in out RVAL\n.end\n", "R1", ["in", "out", "2000"]),
    (".param RVAL=max(1k,2k)\nR1 in out RVAL\n.end\n", "R1", ["in", "out", "2000"]),
    (".param RVAL=if(1,1k,2k)\nR1 in out RVAL\n.end\n", "R1", ["in", "out", "1000"]),
    (".param RVAL=-1k+2^3\nR1 in out RVAL\n.end\n", "R1", ["in", "out", "-992"]),
    (".subckt buf in out\n.param RVAL=3k\nR1 in out RVAL\n.ends\nX1 a b buf\n.end\n", "X1.R1",
     ["a", "b", "3000"]),
    (".subckt leaf a b\nR1 a b 1k\n.ends\n.subckt mid in out\nX1 in out leaf\n.ends\n"
     "Xtop n1 n2 mid\n.end\n", "Xtop.X1.R1", ["n1", "n2", "1000"]),
])
def test_reference_elaboration_vectors(text, name, args):
    d = _elab(text)
    assert len(d) == 1 and d[0].name == name and d[0].args == args


@pytest.mark.parametrize("expr,text", [
    ("2*-3", "-3"),            # a '-' after an operator is '0 -' placed after that operator
    ("2^3^2", "64"),           # '^' is left-associative
    ("(1k+1k)/4", "500"),
    ("min(3,abs(-7))", "3"),
    ("1/0", "inf"),
    ("1e-3", "1e-3"),          # the tokenizer splits at '-': no value, kept as written
    ("sqrt(4)", "sqrt(4)"),    # unknown function: kept as written
    ("(1+2", "(1+2"),          # unbalanced: kept as written
    ("1u*3", "0.000003"),
])
def test_expression_rules(expr, text):
    d = _elab(f".param P={expr}\nR1 a 0 P\n")
    assert d[0].args[2] == text


def test_subckt_deck_matches_flat_deck():
    """An inverter chain through a subcircuit compiles to exactly the flat
    deck's device list (names, nodes, values): ports map, parameters resolve
    in order (body .param, then the instance's)."""
    sub = (".model nm nmos level=1 vto=0.5\n"
           ".subckt inv in out vdd vss\nM1 out in vss vss nm W=2u\nR1 vdd out RL\n"
           ".param RL=20k\n.ends\n"
           "V1 vdd 0 DC 1.2\nV2 a 0 DC 0.9\nX1 a b vdd 0 inv\nX2 b c vdd 0 inv RL=10k\n.op\n")
    flat = (".model nm nmos level=1 vto=0.5\nV1 vdd 0 DC 1.2\nV2 a 0 DC 0.9\n"
            "M1 b a 0 0 nm W=2u\nR1 vdd b 20000\nM2 c b 0 0 nm W=2u\nR2 vdd c 10000\n.op\n")
    s, f = nl.compile_deck(sub), nl.compile_deck(flat)
    assert s.node_names == ["0", "vdd", "a", "b", "c"] == f.node_names
    assert s.device_names == ["V1", "V2", "X1.M1", "X1.R1", "X2.M1", "X2.R1"]
    assert np.array_equal(s.circuit.type, f.circuit.type)
    assert np.array_equal(s.circuit.nodes, f.circuit.nodes)
    assert np.array_equal(s.circuit.p, f.circuit.p)


def test_subckt_scoping_rules():
    """As the reference's expansion does it: a body node that is not a port,
    ground included, becomes <instance>:<node>; a body .model is kept as
    <instance>.<name>, which the body's devices do not reach (they see the
    global card of that name, or none); an instance parameter evaluates in
    the enclosing instance's scope."""
    deck = nl.compile_deck(".subckt s a\nR1 a 0 1k\n.ends\nX1 n s\nR2 n 0 1k\n")
    assert deck.node_names == ["0", "n", "X1:0"]
    text = (".subckt s a b\n.model dm d is=1e-9\nD1 a b dm\n.ends\n"
            "V1 p 0 DC 0.5\nX1 p 0 s\n")
    assert nl.compile_deck(text).circuit.p[1, 0] == 1e-14
    assert nl.compile_deck(text + ".model dm d is=2e-9\n").circuit.p[1, 0] == 2e-9
    d = _elab(".subckt leaf a b R=1\nR1 a b R\n.ends\n.subckt mid a b K=3\nX1 a b leaf R=K*2\n"
              ".ends\nXt p q mid K=5\n")
    assert d[0].name == "Xt.X1.R1" and d[0].args == ["p", "q", "10"]


@pytest.mark.parametrize("text", [".subckt s a\nR1 a 0 1\n", "X1 a b nosuch\n",
                                  ".subckt\nR1 a 0 1\n.ends\n",
                                  ".subckt s a\nX1 a q\n.ends\nX2 n s\n"])
def test_subckt_errors(text):
    with pytest.raises(nl.NetlistError):
        nl.compile_deck(text)


def test_three_node_mosfet_bulk_inside_a_subcircuit():
    """A MOSFET written with drain, gate and source gets the bulk "0" when
    the reader splits its line (netlist.rs:450-454), before the expansion
    maps nodes, so inside a body the bulk is "<instance>:0"
    (map_subckt_node, netlist.rs:1429-1439) while at the top level it is
    ground."""
    deck = nl.compile_deck("""* 3-node level-1 MOSFETs
.model nm nmos level=1 vto=0.5
.subckt cell d g
M1 d g 0 nm
.ends
VDD vdd 0 1.2
X1 vdd in cell
M2 vdd in 0 nm
.end
""")
    names = deck.node_names
    c = deck.circuit
    i1, i2 = deck.device_names.index("X1.M1"), deck.device_names.index("M2")
    assert [names[k] for k in c.nodes[i1]] == ["vdd", "in", "X1:0", "X1:0"]
    assert [names[k] for k in c.nodes[i2]] == ["vdd", "in", "0", "0"]


@pytest.mark.parametrize("text,lines", [
    ("", []), ("a", ["a"]), ("a\n", ["a"]), ("a\n\n", ["a", ""]),
    ("a\r\nb\r\n", ["a", "b"]), ("a\rb\n", ["a\rb"]), ("x\fy\nz\r", ["x\fy", "z\r"]),
    ("p\x85q\u2028r\vs\n", ["p\x85q\u2028r\vs"])])
def test_line_splitting_as_rust_str_lines(text, lines):
    """Only \\n ends a line; one \\r before it is dropped (Rust's
    str::lines, which the reference reads decks with, netlist.rs:150,1238)."""
    assert nl.rust_lines(text) == lines


def test_lone_carriage_return_keeps_one_line():
    """R1 and R2 written on one line split by a lone CR are one statement
    for the reference, so the deck has one resistor with extra tokens."""
    deck = nl.compile_deck("V1 a 0 1\nR1 a 0 1k\rR2 a 0 2k\n.end\n")
    assert deck.device_names == ["V1", "R1"]
