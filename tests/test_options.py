"""Simulator options, the Newton settings derived from them and the solver
factory and selector, against the reference's rules and its own unit tests
(crates/sim-core/src/options.rs:360-440, engine.rs:971-999, solver.rs:
169-562, tests/solver_tests.rs:10-120). Host only."""
import numpy as np
import pytest

from rustspice_gb300 import native as N
from rustspice_gb300 import netlist as nl
from rustspice_gb300.options import (OPTION_DEFS, SimOptions, newton_config_from_options,
                                     solver_type_from_options)
from rustspice_gb300.solver import MatrixProperties, SolverSelector, solver_kind


def test_defaults():  # options.rs:365-375
    o = SimOptions()
    assert o.get_float("abstol") == 1e-12
    assert o.get_float("reltol") == 1e-3
    assert o.get_float("vntol") == 1e-6
    assert o.get_float("gmin") == 1e-12
    assert o.get_int("itl1") == 100
    assert o.get_int("itl4") == 50
    assert o.get_float("temp") == 27.0 and o.get_float("tnom") == 27.0
    assert o.get_string("solver") == "auto"
    assert o.get_int("solver_parallel") == 0
    assert [d[0] for d in OPTION_DEFS] == ["abstol", "reltol", "vntol", "gmin", "itl1", "itl4",
                                           "temp", "tnom", "solver", "solver_parallel"]
    assert not o.is_set("abstol") and not o.is_set("itl1")


def test_set_parse_and_ranges():  # options.rs:377-440
    o = SimOptions()
    o.set("abstol", "1e-15")
    assert o.get_float("abstol") == 1e-15 and o.is_set("abstol")
    o.set("itl1", "200")
    assert o.get_int("itl1") == 200 and o.is_set("itl1")
    o.set("ABSTOL", "1e-14")
    assert o.get_float("abstol") == 1e-14
    o.set("vntol", "1u")  # SI suffix
    assert o.get_float("vntol") == 1e-6 and o.is_set("vntol")
    p = SimOptions()
    p.set("abstol", "1.0")  # float ranges are exclusive: (0, 1e-3)
    assert p.get_float("abstol") == 1e-12 and not p.is_set("abstol")
    p.set("reltol", "0")
    assert p.get_float("reltol") == 1e-3 and not p.is_set("reltol")
    p.set("itl1", "0")  # integer ranges inclusive: [1, 10000]
    assert p.get_int("itl1") == 100 and not p.is_set("itl1")
    p.set("itl1", "1")
    assert p.get_int("itl1") == 1
    p.set("itl4", "1e2")  # Rust's integer parse takes digits only
    assert p.get_int("itl4") == 50 and not p.is_set("itl4")
    p.set("nonexistent", "42")
    assert not p.is_set("nonexistent")
    p.set("solver", "gpu")  # not in the allowed set
    assert p.get_string("solver") == "auto" and not p.is_set("solver")
    p.set("solver", "SparseLU")
    assert p.get_string("solver") == "SparseLU"
    p.set("itl1", "300")  # a second definition replaces the first
    assert p.get_int("itl1") == 300
    assert p.get_float("itl1") == 0.0 and p.get_int("reltol") == 0  # typed lookups


def test_newton_config_from_options():  # engine.rs:986-999, newton.rs:13-26
    c = newton_config_from_options(SimOptions())
    assert (c.max_iters, c.abs_tol, c.rel_tol, c.gmin) == (100, 1e-6, 1e-3, 1e-12)
    assert (c.damping, c.damping_min, c.gmin_steps, c.source_steps) == (1.0, 0.1, 0, 0)
    o = SimOptions()
    o.set("itl1", "7")
    o.set("vntol", "1e-9")
    o.set("reltol", "1e-6")
    o.set("gmin", "1e-10")
    c = newton_config_from_options(o)
    assert (c.max_iters, c.abs_tol, c.rel_tol, c.gmin) == (7, 1e-9, 1e-6, 1e-10)


def test_deck_options_in_order():
    deck = nl.compile_deck("""* options
V1 1 0 1
R1 1 0 1k
.option itl1=200 reltol=1e-6
.option itl1=0 solver=sparselubtf
.option vntol=2.0
.end
""")
    assert deck.newton_options() == {"max_iters": 200, "abs_tol": 1e-6, "rel_tol": 1e-6,
                                     "gmin": 1e-12}
    assert solver_type_from_options(deck.sim_options()) == "sparselubtf"
    assert deck.solver_kind() == "sparselubtf"


def test_solver_types_and_kinds():  # engine.rs:971-984, solver.rs:169-246
    for s, t in [("dense", "dense"), ("sparse", "sparselu"), ("sparselu", "sparselu"),
                 ("sparselubtf", "sparselubtf"), ("bbd", "bbd"), ("faer", "faer"),
                 ("klu", "klu"), ("nativeklu", "nativeklu"), ("auto", "auto")]:
        o = SimOptions()
        o.set("solver", s)
        assert solver_type_from_options(o) == t
    assert solver_kind("auto", 10) == "dense" and solver_kind("auto", 50) == "dense"
    assert solver_kind("auto", 51) == "sparselu" and solver_kind("auto", 500) == "sparselu"
    assert solver_kind("auto", 501) == "sparselubtf"
    assert solver_kind("klu", 1000) == "sparselu" and solver_kind("faer", 10) == "sparselu"
    assert solver_kind("nativeklu", 3) == "nativeklu"
    with pytest.raises(NotImplementedError):
        solver_kind("bbd", 100)


def test_selector_reference_vectors():  # tests/solver_tests.rs:10-120
    s = SolverSelector.select(3, [0, 2, 4, 6], [0, 1, 0, 1, 1, 2])
    assert s.selected == "dense" and "Small" in s.reason
    n = 100
    ap, ai = [0], []
    for col in range(n):
        for row in range(n):
            if (row + col) % 5 != 0:
                ai.append(row)
        ap.append(len(ai))
    assert MatrixProperties.analyze_quick(n, ap, ai).density > 0.3
    assert SolverSelector.select_quick(n, ap, ai).selected == "dense"
    p = MatrixProperties.analyze(4, [0, 1, 2, 3, 4], [0, 1, 2, 3])
    assert (p.n, p.nnz) == (4, 4) and abs(p.density - 0.25) < 0.01 and abs(p.avg_degree - 1) < 0.01
    p = MatrixProperties.analyze(4, [0, 2, 4, 6, 8], [0, 1, 0, 1, 2, 3, 2, 3])
    assert p.num_blocks >= 2 and p.has_block_structure
    assert SolverSelector.select(3, [0, 1, 2, 3], [0, 1, 2]).reason


def _tridiag(n):
    ap, ai = [0], []
    for c in range(n):
        ai.extend(r for r in (c - 1, c, c + 1) if 0 <= r < n)
        ap.append(len(ai))
    return np.array(ap, np.int64), np.array(ai, np.int64)


def test_selector_decision_tree():  # solver.rs:423-520, default build
    ap, ai = _tridiag(150)  # one block, n < 200, sparse
    s = SolverSelector.select(150, ap, ai)
    assert s.selected == "sparselu" and "Medium" in s.reason
    ap, ai = _tridiag(300)  # one block, n >= 200, density < 0.15
    assert SolverSelector.select(300, ap, ai).selected == "bbd"
    # lower bidiagonal: n singleton blocks
    n = 120
    ap = np.array([0] + [2 * c + 2 if c < n - 1 else 2 * c + 1 for c in range(n)], np.int64)
    ai = np.array([r for c in range(n) for r in ((c, c + 1) if c < n - 1 else (c,))], np.int64)
    s = SolverSelector.select(n, ap, ai)
    assert s.selected == "sparselubtf" and s.properties.num_blocks == n
    assert SolverSelector.select_quick(600, *_tridiag(600)).selected == "bbd"
    # n > 500 at density >= 0.15: SparseLU-BTF (select_quick reads ap[n] only)
    ap = np.arange(601, dtype=np.int64) * 120
    assert SolverSelector.select_quick(600, ap).selected == "sparselubtf"
    assert N.KINDS["dense"] == 3
