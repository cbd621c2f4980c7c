"""Time-dependent source values for the transient (the reference's
crates/sim-core/src/waveform.rs): PULSE, PWL, SIN and EXP specifications,
their string parsers (waveform.rs:680-831) and the packed per-device form the
device kernels and the oracle take.

A circuit's waveforms are a dict {device index: Waveform}; the V or I source
at that index takes the waveform's value at the time of each transient solve
instead of its DC value p[0].
"""
from __future__ import annotations

import dataclasses

import numpy as np

KINDS = {"pulse": 1, "pwl": 2, "sin": 3, "exp": 4}
# parameter order and defaults of each kind (waveform.rs:60-72, 196-206, 246-257, 680-830)
DEFAULTS = {
    "pulse": (0.0, 1.0, 0.0, 1e-9, 1e-9, 1e-6, 0.0),   # v1 v2 td tr tf pw per
    "sin": (0.0, 1.0, 1e6, 0.0, 0.0),                    # vo va freq td theta
    "exp": (0.0, 1.0, 0.0, 1e-9, 1e-6, 1e-9),            # v1 v2 td1 tau1 td2 tau2
}


@dataclasses.dataclass
class Waveform:
    kind: str                      # "pulse", "pwl", "sin" or "exp"
    params: tuple = ()             # pulse / sin / exp parameters in the order above
    points: tuple = ()             # pwl: ((t0, v0), (t1, v1), ...)

    def __post_init__(self):
        if self.kind not in KINDS:
            raise ValueError(f"unknown waveform kind {self.kind!r}")
        if self.kind == "pwl":
            # PwlParams::new sorts by time (stable, waveform.rs:137-143)
            self.points = tuple(sorted(((float(t), float(v)) for t, v in self.points),
                                       key=lambda p: p[0]))
        else:
            d = DEFAULTS[self.kind]
            p = tuple(float(x) for x in self.params)
            self.params = p + d[len(p):]


def pulse(v1, v2, td=0.0, tr=1e-9, tf=1e-9, pw=1e-6, per=0.0) -> Waveform:
    return Waveform("pulse", (v1, v2, td, tr, tf, pw, per))


def pwl(points) -> Waveform:
    return Waveform("pwl", (), tuple(points))


def sin(vo, va, freq=1e6, td=0.0, theta=0.0) -> Waveform:
    return Waveform("sin", (vo, va, freq, td, theta))


def exp(v1, v2, td1=0.0, tau1=1e-9, td2=1e-6, tau2=1e-9) -> Waveform:
    return Waveform("exp", (v1, v2, td1, tau1, td2, tau2))


def _number(tok):
    from .netlist import parse_number
    return parse_number(tok)


def parse_source_value(spec: str):
    """parse_source_value (waveform.rs:793-823): a waveform, a DC value (as
    a float) or None. Each parser strips "KIND(" and ")" (upper or lower
    case) and splits on whitespace; missing or unparsable parameters take
    the defaults."""
    s = spec.strip()
    u = s.upper()
    for kind in ("PULSE", "PWL", "SIN", "EXP"):
        if u.startswith(kind):
            inner = None
            for pre in (kind + "(", kind.lower() + "("):
                if s.startswith(pre) and s.endswith(")"):
                    inner = s[len(pre):-1]
            if inner is None:
                return None
            parts = inner.split()
            k = kind.lower()
            if k == "pwl":
                if len(parts) < 2 or len(parts) % 2:
                    return None
                vals = [_number(x) for x in parts]
                if any(v is None for v in vals):
                    return None
                return pwl(zip(vals[0::2], vals[1::2]))
            if len(parts) < 2:
                return None
            d = DEFAULTS[k]
            vals = [(_number(parts[i]) if i < len(parts) else None) for i in range(len(d))]
            return Waveform(k, tuple(d[i] if v is None else v for i, v in enumerate(vals)))
    return _number(s)


def evaluate(w: Waveform, t: float) -> float:
    """WaveformSpec::evaluate restated in Python (for host-side checks)."""
    import math
    if w.kind == "pulse":
        v1, v2, td, tr, tf, pw, per = w.params
        if t < td:
            return v1
        trel = math.fmod(t - td, per) if per > 0.0 else t - td
        if trel < tr:
            return v1 + (v2 - v1) * trel / tr
        if trel < tr + pw:
            return v2
        if trel < tr + pw + tf:
            return v2 - (v2 - v1) * (trel - tr - pw) / tf
        return v1
    if w.kind == "pwl":
        pts = w.points
        if not pts:
            return 0.0
        if t <= pts[0][0]:
            return pts[0][1]
        if t >= pts[-1][0]:
            return pts[-1][1]
        for (t0, v0), (t1, v1) in zip(pts, pts[1:]):
            if t0 <= t < t1:
                return v0 + (v1 - v0) * ((t - t0) / (t1 - t0))
        return pts[-1][1]
    if w.kind == "sin":
        vo, va, freq, td, theta = w.params
        if t < td:
            return vo
        trel = t - td
        damp = math.exp(-theta * trel) if theta > 0.0 else 1.0
        return vo + va * math.sin(2.0 * math.pi * freq * trel) * damp
    v1, v2, td1, tau1, td2, tau2 = w.params
    if t < td1:
        return v1
    v = v1 + (v2 - v1) * (1.0 - math.exp(-(t - td1) / tau1))
    if t >= td2:
        v += (v1 - v2) * (1.0 - math.exp(-(t - td2) / tau2))
    return v


def pack(waves: dict, ndev: int):
    """Per-device arrays: kind (int32, 0 none), 7 parameters each, and the
    PWL points (pointer per device, times, values)."""
    kind = np.zeros(ndev, np.int32)
    p7 = np.zeros((ndev, 7))
    ptr = np.zeros(ndev + 1, np.int64)
    ts, vs = [], []
    for d in range(ndev):
        w = (waves or {}).get(d)
        if w is not None:
            kind[d] = KINDS[w.kind]
            if w.kind == "pwl":
                for t, v in w.points:
                    ts.append(t)
                    vs.append(v)
            else:
                p7[d, :len(w.params)] = w.params
        ptr[d + 1] = len(ts)
    return kind, p7.ravel(), ptr, np.asarray(ts, np.float64), np.asarray(vs, np.float64)
