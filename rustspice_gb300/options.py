"""Simulator options and the solver and Newton settings the engine derives
from them, restated from the reference:

- ``SimOptions``: the option table, parsing, range checks and lookups of
  crates/sim-core/src/options.rs:78-357 (unknown names, unparsable values
  and out-of-range values are ignored with a warning, keeping the default);
- ``newton_config_from_options``: engine.rs:986-999 (itl1, vntol, reltol,
  gmin; damping and stepping from NewtonConfig::default, newton.rs:13-26);
- ``solver_type_from_options``: engine.rs:971-984;
- the solver the engine then creates: ``solver.solver_kind`` (create_solver,
  solver.rs:169-230), sized by the node count (engine.rs:49, 191).
"""
from __future__ import annotations

import re

from . import native as N
from .netlist import parse_number

# name, type, default, range: (lo, hi) exclusive for floats and inclusive for
# integers (options.rs:325-336), or the allowed strings
OPTION_DEFS = [
    ("abstol", "float", 1e-12, (0.0, 1e-3)),
    ("reltol", "float", 1e-3, (0.0, 1.0)),
    ("vntol", "float", 1e-6, (0.0, 1.0)),
    ("gmin", "float", 1e-12, (0.0, 1e-3)),
    ("itl1", "int", 100, (1, 10000)),
    ("itl4", "int", 50, (1, 10000)),
    ("temp", "float", 27.0, (-273.15, 1000.0)),
    ("tnom", "float", 27.0, (-273.15, 1000.0)),
    ("solver", "str", "auto", ("auto", "dense", "sparse", "sparselu", "sparselubtf", "bbd",
                               "faer", "klu", "nativeklu")),
    ("solver_parallel", "int", 0, (0, 256)),
]
_DEFS = {d[0]: d for d in OPTION_DEFS}
_INT = re.compile(r"^[+-]?\d+$")


class SimOptions:
    """The reference's SimOptions: every known option with its default, and
    whether the deck set it."""

    def __init__(self, warn=None):
        self._v = {name: default for name, _, default, _ in OPTION_DEFS}
        self._set = set()
        self.warnings: list[str] = []
        self._warn = warn

    def _warning(self, msg):
        self.warnings.append(msg)
        if self._warn is not None:
            print(f"warning: {msg}", file=self._warn)

    def set(self, key: str, raw: str) -> None:
        """options.rs:185-258: parse by the option's type, check its range,
        store and mark as set."""
        k = key.lower()
        d = _DEFS.get(k)
        if d is None:
            self._warning(f"unknown option '{key}' ignored")
            return
        _, typ, default, rng = d
        if typ == "float":
            v = parse_number(raw)  # parse_number_with_suffix, then a plain parse
            if v is None:
                self._warning(f"option '{k}' value '{raw}' is not a valid number, ignored")
                return
            ok = rng[0] < v < rng[1]
        elif typ == "int":
            if not _INT.match(raw):  # Rust's i64 parse: optional sign, digits
                self._warning(f"option '{k}' value '{raw}' is not a valid integer, ignored")
                return
            v = int(raw)
            ok = rng[0] <= v <= rng[1]
        else:
            v = raw
            ok = any(a.lower() == v.lower() for a in rng)
        if not ok:
            self._warning(f"option '{k}' value {v} out of range, using default {default}")
            return
        if k in self._set:
            self._warning(f"option '{k}' redefined (was {self._v[k]}), using new value {v}")
        self._v[k] = v
        self._set.add(k)

    def get_float(self, key: str) -> float:
        v = self._v.get(key)
        return v if isinstance(v, float) else 0.0

    def get_int(self, key: str) -> int:
        v = self._v.get(key)
        return v if isinstance(v, int) else 0

    def get_string(self, key: str) -> str:
        v = self._v.get(key)
        return v if isinstance(v, str) else ""

    def is_set(self, key: str) -> bool:
        return key in self._set

    @classmethod
    def from_pairs(cls, pairs, warn=None) -> "SimOptions":
        """The options of a deck's .option lines, set in the order they came
        (key=value pairs; bare names as "true", netlist.rs:1044-1053)."""
        o = cls(warn)
        for k, v in pairs:
            o.set(k, v)
        return o


def newton_config_from_options(opts: SimOptions) -> N.NewtonConfig:
    """engine.rs:986-999."""
    return N.newton_config(max_iters=opts.get_int("itl1"), abs_tol=opts.get_float("vntol"),
                           rel_tol=opts.get_float("reltol"), gmin=opts.get_float("gmin"),
                           gmin_steps=0, source_steps=0, damping=1.0, damping_min=0.1)


def solver_type_from_options(opts: SimOptions) -> str:
    """engine.rs:971-984; anything unrecognised selects "auto"."""
    s = opts.get_string("solver").lower()
    return {"dense": "dense", "sparse": "sparselu", "sparselu": "sparselu",
            "sparselubtf": "sparselubtf", "bbd": "bbd", "faer": "faer", "klu": "klu",
            "nativeklu": "nativeklu"}.get(s, "auto")
