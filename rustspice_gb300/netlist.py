"""SPICE netlists of the R/V/I/D/M/C subset into the device-list Circuit.

A deck becomes the flat device list the stamp compiler takes (``Circuit`` in
circuits.py), with the reference's reading of every field, so a user deck
runs on ``DeviceCircuit`` / ``newton_dc`` / ``Batch`` as the reference engine
would run it:

* lines (crates/sim-core/src/netlist.rs:150-190): surrounding blanks are
  trimmed; ``*`` starts a comment; ``+`` continues the previous statement
  (joined with one space); a first token beginning with ``.`` is a control,
  any other a device named by its first letter;
* tokens (netlist.rs:322-370): ``key=value`` tokens are parameters (a token
  holding both ``=`` and ``,`` splits at top-level commas; a leading ``(`` and
  a trailing ``)`` around a parameter are dropped), the rest positional;
* device fields (netlist.rs:400-460, 1454-1476): R, C, V, I take two nodes
  and a value, the token after a ``DC`` keyword when there is one (a source
  without a DC value, which the reference leaves out of its DC system, is
  refused); V and I carry the magnitude and phase after an ``AC`` keyword
  (p[1], p[2]; 0 when absent); D takes two nodes and a model; M four nodes
  and a model, or three and a model with the bulk on ground;
* numbers (netlist.rs:1635-1660): one trailing ``f p n u m k g t`` scales by
  1e-15 ... 1e12 and ``meg`` by 1e6, case-insensitive;
* nodes (circuit.rs:31-57, netlist.rs:934-1100): ``0`` is ground (id 0),
  other names take ids in order of first use, ``.ic`` nodes before device
  nodes (controls are read first), names compared as written;
* models and parameters (netlist.rs:940-960, 1120-1135): ``.model name type
  params``, names and keys lower-cased; a device's parameters are its
  model's, overridden by its own;
* diode (crates/sim-core/src/stamp.rs:351-387): Is from ``is`` (1e-14), N
  from ``n`` or ``nj`` (1.0);
* MOSFET (stamp.rs:389-420, crates/sim-devices/src/bsim/mod.rs:83-200,
  params.rs:303-462): the level from ``level`` (49 when absent); PMOS only if
  parameter ``type`` contains ``pmos`` or equals ``p``, or a ``pmos`` key
  exists -- the model card's own type word does not count; vth0 from
  ``vth0``/``vto``/``vth`` (0.7, PMOS -0.7), u0 from ``u0``/``uo`` (500, PMOS
  150), tox from ``tox`` (1.5e-8), W and L from ``w``/``l`` (1e-6).
  Only level 1 is on this path; other levels raise ``NetlistError``;
* ``.option`` keys (crates/sim-core/src/engine.rs:987-999): ``itl1`` max
  iterations (100), ``vntol`` absolute (1e-6), ``reltol`` relative (1e-3),
  ``gmin`` (1e-12).

* ``.include`` (netlist.rs:1205-1260, ``load`` only, as the reference's
  ``parse_netlist_file``): a line whose trimmed, lower-cased text starts with
  ``.include`` is replaced by the named file (second token, quotes stripped,
  relative to the including file's directory), recursively; a file already
  on the include path is a circular reference. A missing path, an unreadable
  file and a cycle are errors.

* ``.param`` and subcircuits (netlist.rs:857-925, 1262-1460, 1557-1955):
  parameters evaluate in order (numbers with suffixes, names, ``+ - * / ^``
  left-associative, a ``-`` after no value taken as ``0 -``, ``max min abs
  if``); a device's value, model and parameter values resolve from its
  scope's table, the global one, or their own evaluation, else stay as
  written; ``X`` lines expand the subcircuit named by their last token:
  devices become ``<instance>.<name>``, ports map to the instance's nodes,
  other nodes become ``<instance>:<node>``, nested instances expand in the
  enclosing scope (its own, body ``.param`` and instance parameters), and a
  ``.model`` in a body is kept as ``<instance>.<name>``, which a device's
  unscoped model name does not reach. A ``.subckt`` ends at the first
  ``.ends``.

The other device kinds are outside this path and raise ``NetlistError`` (so
does ``.include`` in text given to ``compile_deck``, which has no directory
to resolve it against).
"""
from __future__ import annotations

import dataclasses
import os
import re

import numpy as np

from .circuits import (DEV_C, DEV_D, DEV_I, DEV_M, DEV_R, DEV_V, NPARAM, TOX, Circuit)


class NetlistError(ValueError):
    """A deck outside the subset this path runs (or a malformed line)."""


_SCALE = {"f": 1e-15, "p": 1e-12, "n": 1e-9, "u": 1e-6, "m": 1e-3, "k": 1e3, "g": 1e9,
          "t": 1e12}
_FLOAT = re.compile(r"^[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|infinity|nan)$",
                    re.I)


def parse_number(token: str):
    """A number with an optional SI suffix, or None."""
    t = token.strip().lower()
    mult = 1.0
    if t.endswith("meg"):
        t, mult = t[:-3], 1e6
    elif t and t[-1] in _SCALE:
        t, mult = t[:-1], _SCALE[t[-1]]
    if not _FLOAT.match(t):
        return None
    return float(t) * mult


def _split_top_commas(s: str):
    out, depth, start = [], 0, 0
    for i, ch in enumerate(s):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth = max(0, depth - 1)
        elif ch == "," and depth == 0:
            out.append(s[start:i])
            start = i + 1
    if start < len(s):
        out.append(s[start:])
    return out


def _args_params(tokens):
    args, params = [], []
    for tok in tokens:
        parts = _split_top_commas(tok) if ("=" in tok and "," in tok) else [tok]
        for raw in parts:
            part = raw.strip()
            if not part:
                continue
            if part.startswith("(") and "=" in part:
                part = part[1:]
            if part.endswith(")") and "=" in part and "(" not in part[part.index("=") + 1:]:
                part = part[:-1]
            if not part:
                continue
            if "=" in part:
                k, v = part.split("=", 1)
                params.append((k, v))
            else:
                args.append(part)
    return args, params


@dataclasses.dataclass
class Statement:
    line: int
    control: str = ""          # ".model", ".op", ... (lower-case) for a control
    name: str = ""             # device name for a device line
    kind: str = ""             # device letter, upper-case
    args: list = dataclasses.field(default_factory=list)
    params: list = dataclasses.field(default_factory=list)


def rust_lines(text: str):
    """Lines as Rust's ``str::lines`` gives them (the reference reads decks
    with it, netlist.rs:150, 1238): split on ``\n`` only, one trailing
    ``\r`` removed from each line, no empty line after a final newline."""
    parts = text.split("\n")
    last = parts.pop()  # the text after the final newline (no line ending)
    out = [q[:-1] if q.endswith("\r") else q for q in parts]
    if last:
        out.append(last)
    return out


def parse(text: str):
    """Statements of a deck and the errors the reader recorded (line, text)."""
    stmts, errors, pending, pending_line = [], [], "", 0

    def flush(line_text, line_no):
        toks = line_text.split()
        if not toks:
            return
        first = toks[0]
        args, params = _args_params(toks[1:])
        if first.startswith("."):
            stmts.append(Statement(line_no, control=first.lower(), args=args, params=params))
            return
        kind = first[0].upper()
        if kind not in "RCLVIDMEGFHX":
            errors.append((line_no, f"unknown device type: {first}"))
            return
        stmts.append(Statement(line_no, name=first, kind=kind, args=args, params=params))

    lines = rust_lines(text)
    for no, raw in enumerate(lines, 1):
        s = raw.strip()
        if not s or s.startswith("*"):
            continue
        if s.startswith("+"):
            if not pending:
                errors.append((no, "continuation line has no preceding line"))
                continue
            pending += " " + s.lstrip("+").strip()
            continue
        if pending:
            flush(pending, pending_line)
        pending, pending_line = s, no
    if pending:
        flush(pending, pending_line)
    return stmts, errors


# ------------------------------------------------------------ parameters
# .param values, subcircuit parameters and device fields are evaluated as the
# reference's elaboration does (crates/sim-core/src/netlist.rs:1262-1350,
# 1557-1860): tables map lower-cased names to text - an evaluated value in
# the text Rust's f64 Display gives it, or the raw text when the expression
# does not evaluate.

def _f64_text(v: float) -> str:
    """Rust's ``f64`` Display: the shortest round-trip digits, positional."""
    if v != v:
        return "NaN"
    if v in (float("inf"), float("-inf")):
        return "inf" if v > 0 else "-inf"
    import decimal
    t = format(decimal.Decimal(repr(v)), "f")
    if "." in t:
        t = t.rstrip("0").rstrip(".")
    return t


def _f64_parse(text: str):
    """Rust's ``str::parse::<f64>`` (no suffix)."""
    t = text.strip()
    return float(t) if _FLOAT.match(t) else None


def _tokens(expr: str):
    """netlist.rs:1589-1633: numbers (with suffix) and identifiers split at
    blanks and at ``+ - * / ^ , ( )``."""
    out, buf = [], []

    def push():
        if buf:
            word = "".join(buf)
            x = parse_number(word)
            out.append(("num", x) if x is not None else ("id", word))
            buf.clear()

    for ch in expr:
        if ch.isspace():
            push()
        elif ch in "+-*/^":
            push()
            out.append(("op", ch))
        elif ch == ",":
            push()
            out.append(("comma", None))
        elif ch == "(":
            push()
            out.append(("lp", None))
        elif ch == ")":
            push()
            out.append(("rp", None))
        else:
            buf.append(ch)
    push()
    return out


_PREC = {"+": 1, "-": 1, "*": 2, "/": 2, "^": 3}


def _rpn(tokens):
    """netlist.rs:1681-1772 (shunting-yard): a ``-`` after no value gets a 0
    pushed before it; operators of higher or equal precedence pop (all of
    them left-associative); an identifier before ``(`` is a function whose
    argument count the commas give; a parenthesis left at the end fails."""
    output, ops, argc = [], [], []
    prev_value = False
    for i, tok in enumerate(tokens):
        kind, val = tok
        nxt = tokens[i + 1] if i + 1 < len(tokens) else None
        if kind == "num":
            output.append(tok)
        elif kind == "id":
            if nxt is not None and nxt[0] == "lp":
                ops.append(("func", [val, 0]))
            else:
                output.append(tok)
        elif kind == "op":
            if not prev_value and val == "-":
                output.append(("num", 0.0))
            while ops and ops[-1][0] == "op" and _PREC[ops[-1][1]] >= _PREC[val]:
                output.append(ops.pop())
            ops.append(tok)
        elif kind == "comma":
            while ops and ops[-1][0] != "lp":
                output.append(ops.pop())
            if argc:
                argc[-1] += 1
        elif kind == "lp":
            if ops and ops[-1][0] == "func":
                argc.append(0)
            ops.append(tok)
        elif kind == "rp":
            while ops:
                top = ops.pop()
                if top[0] == "lp":
                    break
                output.append(top)
            if ops and ops[-1][0] == "func":
                name = ops.pop()[1][0]
                output.append(("call", (name, (argc.pop() if argc else 0) + 1)))
        prev_value = kind in ("num", "id", "rp")
    while ops:
        top = ops.pop()
        if top[0] in ("lp", "rp"):
            return None
        output.append(top)
    return output


def _lookup(name, local, parent, glob):
    key = name.lower()
    for table in (local, parent, glob):
        if key in table:
            text = table[key]
            x = parse_number(text)
            return x if x is not None else _f64_parse(text)
    return None


def _rmax(a, b):  # f64::max / f64::min: a NaN operand yields the other
    return b if a != a else (a if b != b else (a if a > b else b))


def _rmin(a, b):
    return b if a != a else (a if b != b else (a if a < b else b))


def _evaluate(expr, local, parent, glob):
    """netlist.rs:1564-1587, 1781-1845: the value of an expression, or None."""
    toks = _tokens(expr)
    if not toks:
        return None
    rpn = _rpn(toks)
    if rpn is None:
        return None
    stack = []
    with np.errstate(all="ignore"):
        for kind, val in rpn:
            if kind == "num":
                stack.append(val)
            elif kind == "id":
                x = _lookup(val, local, parent, glob)
                if x is None:
                    return None
                stack.append(x)
            elif kind == "op":
                if len(stack) < 2:
                    return None
                b, a = stack.pop(), stack.pop()
                fa, fb = np.float64(a), np.float64(b)
                r = {"+": fa + fb, "-": fa - fb, "*": fa * fb, "/": fa / fb,
                     "^": np.power(fa, fb)}[val]
                stack.append(float(r))
            elif kind == "call":
                name, n = val
                if len(stack) < n:
                    return None
                args = [stack.pop() for _ in range(n)][::-1]
                f = name.lower()
                if f == "max" and n == 2:
                    stack.append(_rmax(*args))
                elif f == "min" and n == 2:
                    stack.append(_rmin(*args))
                elif f == "abs" and n == 1:
                    stack.append(abs(args[0]))
                elif f == "if" and n == 3:
                    stack.append(args[1] if args[0] != 0.0 else args[2])
                else:
                    return None
            else:
                return None
    return stack[0] if len(stack) == 1 else None


def _param_entry(table, key, value, parent, glob):
    x = _evaluate(value, table, parent, glob)
    table[key.lower()] = _f64_text(x) if x is not None else value


def _resolve(local, glob, token):
    """netlist.rs:1338-1349: a field's text from the local table, the global
    one, or its own evaluation; None leaves the field as written."""
    key = token.lower()
    if key in local:
        return local[key]
    if key in glob:
        return glob[key]
    x = _evaluate(token, local, {}, glob)
    return None if x is None else _f64_text(x)


def _fields(st):
    """Positions of a device line's nodes, value and model in its positional
    tokens (split_device_fields, netlist.rs:398-520, for the kinds this
    reader maps; other kinds keep every token as written)."""
    a, k = st.args, st.kind
    if k in "RCLVI":
        if len(a) >= 3:
            if a[2].lower() == "dc" and len(a) >= 4:
                return [0, 1], 3, None
            if k in "VI" and _is_waveform(a[2]):
                return [0, 1], None, None
            return [0, 1], 2, None
        return list(range(len(a))), None, None
    if k == "D":
        return ([0, 1], None, 2) if len(a) >= 3 else (list(range(len(a))), None, None)
    if k == "M":
        if len(a) >= 5:
            return [0, 1, 2, 3], None, 4
        if len(a) == 4:
            return [0, 1, 2], None, 3
        return list(range(len(a))), None, None
    if k == "X":
        if len(a) >= 2:
            return list(range(len(a) - 1)), None, len(a) - 1
        return list(range(len(a))), None, None
    return [], None, None


def _is_waveform(tok):
    u = tok.upper()
    return u in ("AC", "SIN", "PULSE", "EXP", "SFFM", "PWL") or u.startswith(
        ("SIN(", "PULSE(", "EXP(", "SFFM(", "PWL("))


def _apply_params(st, local, glob):
    """netlist.rs:1316-1336: the value, the model and the parameter values
    of a device resolved in its scope."""
    _, vi, mi = _fields(st)
    args = list(st.args)
    for i in (vi, mi):
        if i is not None:
            r = _resolve(local, glob, args[i])
            if r is not None:
                args[i] = r
    params = []
    for k, v in st.params:
        r = _resolve(local, glob, v)
        params.append((k, v if r is None else r))
    return dataclasses.replace(st, args=args, params=params)


@dataclasses.dataclass
class Subckt:
    name: str
    ports: list
    params: list
    body: list
    line: int


def _extract_subckts(stmts):
    """netlist.rs:1351-1406: a ``.subckt`` takes the statements up to the
    next ``.ends`` (the first one: definitions do not nest)."""
    top, defs, i = [], [], 0
    while i < len(stmts):
        st = stmts[i]
        if st.control == ".subckt":
            if not st.args:
                raise NetlistError(f"line {st.line}: subckt statement missing name")
            body, i, closed = [], i + 1, False
            while i < len(stmts):
                if stmts[i].control == ".ends":
                    closed, i = True, i + 1
                    break
                body.append(stmts[i])
                i += 1
            if not closed:
                raise NetlistError(f"line {st.line}: subckt {st.args[0]} missing .ends")
            defs.append(Subckt(st.args[0], st.args[1:], list(st.params), body, st.line))
        else:
            top.append(st)
            i += 1
    return top, defs


def _body_params(body):
    """netlist.rs:1408-1427: the ``.param`` entries of a body outside the
    ``.subckt`` ... ``.ends`` ranges inside it."""
    out, depth = [], 0
    for st in body:
        if st.control == ".subckt":
            depth += 1
        elif st.control == ".ends":
            depth = max(0, depth - 1)
        elif st.control == ".param" and depth == 0:
            out.extend(st.params)
    return out


def _local_params(d, inst, parent, glob):
    """netlist.rs:1283-1314: the subcircuit's own parameters, then its body's
    ``.param`` entries, then the instance's, each evaluated in order."""
    table = {}
    for k, v in list(d.params) + _body_params(d.body) + list(inst.params):
        _param_entry(table, k, v, parent, glob)
    return table


def _expand(inst, d, defs, local, glob, models):
    """netlist.rs:1869-1955: the body's devices named ``<instance>.<name>``,
    ports mapped to the instance's nodes (case-insensitively), other nodes
    named ``<instance>:<node>``; nested instances expanded in the scope of
    this one; the body's ``.model`` cards kept as ``<instance>.<name>``."""
    body, nested = _extract_subckts(d.body)
    scope = {x.name: x for x in nested}
    for k, v in defs.items():
        scope.setdefault(k, v)
    inst_nodes = [inst.args[i] for i in _fields(inst)[0]]
    ports = {p.lower(): n for p, n in zip(d.ports, inst_nodes)}
    out = []
    for st in body:
        if st.control == ".model":
            if st.args:
                models.append(dataclasses.replace(st, args=[f"{inst.name}.{st.args[0]}"] +
                                                  st.args[1:]))
            continue
        if st.control:
            continue
        if st.kind == "M" and len(st.args) == 4:
            # drain gate source model: the reader adds the bulk "0" when it
            # splits the line (netlist.rs:450-454), before the expansion maps
            # the nodes, so inside a body it becomes "<instance>:0"
            st = dataclasses.replace(st, args=st.args[:3] + ["0"] + st.args[3:])
        nodes, _, mi = _fields(st)
        args = list(st.args)
        for i in nodes:
            args[i] = ports.get(args[i].lower(), f"{inst.name}:{args[i]}")
        sc = dataclasses.replace(st, name=f"{inst.name}.{st.name}", args=args)
        if st.kind == "X":
            child = scope.get(args[mi]) if mi is not None else None
            if child is None:
                raise NetlistError(f"line {st.line}: subcircuit not defined: {sc.name}")
            out.extend(_expand(sc, child, scope, _local_params(child, sc, local, glob), glob,
                               models))
            continue
        out.append(_apply_params(sc, local, glob))
    return out


def elaborate(stmts):
    """netlist.rs:857-925: the top-level controls, the flat device list
    (subcircuit instances expanded, parameters applied) and the ``.model``
    cards found inside subcircuits."""
    top, defs = _extract_subckts(stmts)
    glob = {}
    for st in top:
        if st.control == ".param":
            for k, v in st.params:
                _param_entry(glob, k, v, glob, glob)
    subckts = {d.name: d for d in defs}
    controls, devices, models = [], [], []
    for st in top:
        if st.control:
            controls.append(st)
        elif st.kind == "X":
            mi = _fields(st)[2]
            d = subckts.get(st.args[mi]) if mi is not None else None
            if d is None:
                raise NetlistError(f"line {st.line}: subcircuit not defined: {st.name}")
            devices.extend(_expand(st, d, subckts, _local_params(d, st, {}, glob), glob, models))
        else:
            devices.append(_apply_params(st, {}, glob))
    return controls, devices, models


@dataclasses.dataclass
class Deck:
    circuit: Circuit
    node_names: list           # node id -> name
    device_names: list         # device index -> instance name
    options: dict              # lower-case option -> value string
    initial: dict              # node id -> .ic voltage
    analyses: list             # control commands seen (".op", ".dc", ...)
    option_seq: list = dataclasses.field(default_factory=list)  # (key, value) in deck order

    def sim_options(self):
        """The deck's .option values as the reference's SimOptions holds them
        (types, ranges and defaults of options.rs), set in deck order."""
        from .options import SimOptions
        return SimOptions.from_pairs(self.option_seq)

    def newton_options(self) -> dict:
        """The Newton settings the reference derives from the options
        (engine.rs:986-999)."""
        o = self.sim_options()
        return {"max_iters": o.get_int("itl1"), "abs_tol": o.get_float("vntol"),
                "rel_tol": o.get_float("reltol"), "gmin": o.get_float("gmin")}

    def solver_kind(self) -> str:
        """The device solver kind for `.option solver=` (engine.rs:971-984,
        solver.rs:169-230), sized by the node count as the engine does."""
        from .options import solver_type_from_options
        from .solver import solver_kind
        return solver_kind(solver_type_from_options(self.sim_options()),
                           self.circuit.node_count)

    def transient_x0(self) -> np.ndarray:
        """A transient's starting point: zeros with the .ic voltages
        (crates/sim-core/src/engine.rs:340-348; the DC operating point starts
        from zeros)."""
        x = np.zeros(self.circuit.node_count)
        for k, v in self.initial.items():
            x[k] = v
        return x


def _pnum(params: dict, keys, default):
    for k in keys:
        if k in params:
            x = parse_number(params[k])
            if x is not None:
                return x
    return default


def compile_deck(text: str, name: str = "") -> Deck:
    """A deck of R, V, I, D, level-1 M and C into a Circuit."""
    stmts, errors = parse(text)
    if errors:
        raise NetlistError("; ".join(f"line {n}: {m}" for n, m in errors))
    controls, devices, sub_models = elaborate(stmts)
    names = {"0": 0}
    order = ["0"]

    def node(s):
        if s not in names:
            names[s] = len(order)
            order.append(s)
        return names[s]

    models, options, initial, analyses, option_seq = {}, {}, {}, [], []
    for st in controls:  # controls first (as the reference builds the circuit)
        if st.control == ".model":
            if len(st.args) < 2:
                raise NetlistError(f"line {st.line}: model statement missing name/type")
            models[st.args[0].lower()] = {k.lower(): v for k, v in st.params}
        elif st.control == ".option" or st.control == ".options":
            for k, v in st.params:
                options[k.lower()] = v
                option_seq.append((k, v))
            for a in st.args:
                options[a.lower()] = "true"
                option_seq.append((a, "true"))
        elif st.control == ".ic":
            for k, v in st.params:
                key = k.strip().lower()
                x = parse_number(v)
                if key.startswith("v(") and key.endswith(")") and x is not None:
                    initial[node(key[2:-1].strip())] = x
        elif st.control in (".include", ".inc", ".lib"):
            raise NetlistError(f"line {st.line}: {st.control} is outside this path")
        elif st.control in (".op", ".dc", ".tran", ".ac"):
            analyses.append(st.control)
    for st in sub_models:  # cards from subcircuit bodies, under <instance>.<name>
        if len(st.args) >= 2:
            models[st.args[0].lower()] = {k.lower(): v for k, v in st.params}
    t, nd, p, dev_names = [], [], [], []
    for st in devices:
        prm = {}
        a = st.args
        if st.kind in "RCVI":
            if len(a) < 3:
                raise NetlistError(f"line {st.line}: {st.name} needs two nodes and a value")
            val = a[3] if (a[2].lower() == "dc" and len(a) >= 4) else a[2]
            v = parse_number(val)
            if v is None:
                raise NetlistError(f"line {st.line}: {st.name} has no numeric (DC) value")
            kind = {"R": DEV_R, "C": DEV_C, "V": DEV_V, "I": DEV_I}[st.kind]
            nodes, params = (node(a[0]), node(a[1])), (v,)
            if st.kind in "VI":  # AC magnitude and phase after an AC keyword (netlist.rs:1454-1476)
                up = [x.upper() for x in a]
                if "AC" in up:
                    k = up.index("AC")
                    mag = parse_number(a[k + 1]) if k + 1 < len(a) else None
                    ph = parse_number(a[k + 2]) if k + 2 < len(a) else None
                    params = (v, 0.0 if mag is None else mag, 0.0 if ph is None else ph)
        elif st.kind in "DM":
            if st.kind == "D":
                if len(a) < 3:
                    raise NetlistError(f"line {st.line}: {st.name} needs two nodes and a model")
                terms, model = a[:2], a[2]
            elif len(a) >= 5:
                terms, model = a[:4], a[4]
            elif len(a) == 4:  # drain gate source model: the bulk is ground
                terms, model = a[:3] + ["0"], a[3]
            else:
                raise NetlistError(f"line {st.line}: {st.name} needs its nodes and a model")
            nodes = tuple(node(x) for x in terms)
            prm.update(models.get(model.lower(), {}))
            prm.update({k.lower(): v for k, v in st.params})
            if st.kind == "D":
                kind = DEV_D
                params = (_pnum(prm, ["is"], 1e-14), _pnum(prm, ["n", "nj"], 1.0))
            else:
                level = int(_pnum(prm, ["level"], 49.0))
                if level != 1:
                    raise NetlistError(f"line {st.line}: {st.name} is a level-{level} MOSFET;"
                                       " this path evaluates level 1")
                if "type" in prm:
                    tl = prm["type"].lower()
                    pmos = "pmos" in tl or tl == "p"
                else:
                    pmos = "pmos" in prm
                kind = DEV_M
                params = (1.0 if pmos else 0.0,
                          _pnum(prm, ["vth0", "vto", "vth"], -0.7 if pmos else 0.7),
                          _pnum(prm, ["u0", "uo"], 150.0 if pmos else 500.0),
                          _pnum(prm, ["tox"], TOX),
                          _pnum(prm, ["w"], 1e-6), _pnum(prm, ["l"], 1e-6))
        else:
            raise NetlistError(f"line {st.line}: device {st.name} ({st.kind}) is outside this path")
        t.append(kind)
        nd.append(tuple(nodes) + (0,) * (4 - len(nodes)))
        p.append(tuple(params) + (0.0,) * (NPARAM - len(params)))
        dev_names.append(st.name)
    c = Circuit(len(order), np.asarray(t, np.int32), np.asarray(nd, np.int32).reshape(-1, 4),
                np.asarray(p, np.float64).reshape(-1, NPARAM), name)
    return Deck(c, order, dev_names, options, initial, analyses or [".op"], option_seq)


def _path_key(path: str):
    """A path compared as the reference's PathBuf compares: by components,
    with ``.`` after the first one and empty components dropped."""
    parts = path.split("/")
    return (parts[0],) + tuple(q for q in parts[1:] if q not in ("", "."))


def read_with_includes(path: str, visited: set, errors: list) -> str:
    """The deck text with its ``.include`` lines replaced by the included
    files (netlist.rs:1205-1260): every other line is kept with a newline; an
    included file's text is followed by one more newline."""
    key = _path_key(path)
    if key in visited:
        errors.append(f"include circular reference: {path}")
        return ""
    visited.add(key)
    try:
        with open(path) as f:
            content = f.read()
    except OSError:
        errors.append(f"cannot read file: {path}")
        content = ""
    base = os.path.dirname(path) or "."
    out = []
    for line in rust_lines(content):
        t = line.strip()
        if t.lower().startswith(".include"):
            toks = t.split()
            inc = toks[1].strip('"') if len(toks) > 1 else ""
            if not inc:
                errors.append(f"include statement missing path: {path}")
                continue
            out.append(read_with_includes(os.path.join(base, inc), visited, errors))
            out.append("\n")
        else:
            out.append(line + "\n")
    return "".join(out)


def load(path: str) -> Deck:
    """A deck file with its includes resolved (the reference's
    ``parse_netlist_file``), compiled as ``compile_deck`` does."""
    errors: list = []
    text = read_with_includes(path, set(), errors)
    if errors:
        raise NetlistError("; ".join(errors))
    return compile_deck(text, name=path)
