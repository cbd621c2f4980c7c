"""ctypes wrapper over the oracle library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_solver_new.restype = _P
        L.orc_solver_new.argtypes = [C.c_char_p, _I64]
        L.orc_solver_free.argtypes = [_P]
        L.orc_bbd_new.restype = _P
        L.orc_bbd_new.argtypes = [_I64, _P, _I64]
        L.orc_bbd_info.restype = C.c_int
        L.orc_bbd_info.argtypes = [_P, _P, _P]
        L.orc_prepare.argtypes = [_P, _I64]
        L.orc_name.restype = C.c_char_p
        L.orc_name.argtypes = [_P]
        L.orc_reset.argtypes = [_P]
        L.orc_analyze.argtypes = [_P, _P, _I64, _P, _I64]
        L.orc_factor.argtypes = [_P, _P, _I64, _P, _P, _I64]
        L.orc_solve.argtypes = [_P, _P, _I64]
        L.orc_klu_stats.argtypes = [_P, _P, _P]
        L.orc_klu_pivots.restype = _I64
        L.orc_klu_pivots.argtypes = [_P, _P, _I64]
        L.orc_klu_block_values.restype = _I64
        L.orc_klu_block_values.argtypes = [_P, _I64, _P, _I64, _P, _I64, _P, _P]
        L.orc_amd.argtypes = [_I64, _P, _P, _P, _P]
        L.orc_btf.argtypes = [_I64, _P, _P, _P, _P, _P, _P]
        L.orc_mna.restype = _P
        L.orc_mna.argtypes = [_I64, _I64, _P, _P, _P, _P, _I64, _D, _D, _D, _P, _D, _D]
        L.orc_mna_dims.argtypes = [_P, _P, _P]
        L.orc_mna_get.argtypes = [_P, _P, _P, _P, _P]
        L.orc_mna_free.argtypes = [_P]
        L.orc_dc_op.restype = C.c_int
        L.orc_dc_op.argtypes = [_I64, _I64, _P, _P, _P, C.c_char_p, _I64, _D, _D, _D,
                                _I64, _I64, _P, _P, _I64, _P, _P]
        L.orc_dc_op_bbd.restype = C.c_int
        L.orc_dc_op_bbd.argtypes = [_I64, _I64, _P, _P, _P, _P, _I64, _I64, _D, _D, _D, _I64,
                                    _P, _P, _I64, _P, _P]
        L.orc_tran.restype = C.c_int
        L.orc_tran.argtypes = [_I64, _I64, _P, _P, _P, C.c_char_p, _I64, _D, _D, _D, _D, _I64,
                               _P, _P, _P]
        L.orc_ac_sweep.restype = C.c_int
        L.orc_ac_sweep.argtypes = [_I64, _I64, _P, _P, _P, _P, _I64, _P, _I64, _P, _P, _I64, _P]
        L.orc_tran_adjoint.restype = C.c_int
        L.orc_tran_adjoint.argtypes = [_I64, _I64, _P, _P, _P, _D, _I64, _P, _I64, _D, _D, _P]
        L.orc_dc_sweep.argtypes = [_I64, _I64, _P, _P, _P, C.c_char_p, _I64, _D, _D, _D, _I64,
                                   _I64, _P, _I64, _P, _I64, C.c_int, _P, _I64, _P, _P, _P]
        L.orc_residual.restype = _D
        L.orc_residual.argtypes = [_I64, _I64, _P, _P, _P, _P, _I64, _D]
        L.orc_dc_batch.argtypes = [_I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P, C.c_char_p,
                                   _I64, _D, _D, _D, _I64, _P, _P, _I64, _P, _P, _P, _I64,
                                   C.c_int, _P]
        L.orc_wave_eval.argtypes = [C.c_int32, _P, _I64, _P, _P, _I64, _P, _P]
        L.orc_breakpoints.restype = _I64
        L.orc_breakpoints.argtypes = [_I64, _P, _P, _P, _P, _P, _D, _P, _I64]
        L.orc_bp_limit_dt.restype = _D
        L.orc_bp_limit_dt.argtypes = [_P, _I64, _D, _D, _D]
        L.orc_bp_settling.argtypes = [_P, _I64, _I64, _D, _I64, _P, _P, _P]
        L.orc_lte.argtypes = [_P, _P, _I64, _D, _D, _P]
        L.orc_adaptive_sequence.argtypes = [_D, _D, _I64, _P, _P, _P]
        L.orc_tran_adaptive.restype = C.c_int
        L.orc_tran_adaptive.argtypes = [_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, C.c_char_p,
                                        _I64, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _P,
                                        _I64, _I64, _P, _P, _P]
        _lib = L
    return _lib


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Solver:
    """One of the reference's LinearSolver implementations, restated."""

    def __init__(self, kind: str, n: int, assignment=None, num_blocks: int = 0):
        if kind == "bbd":
            asg = _i64(assignment)
            self.h = lib().orc_bbd_new(n, _ptr(asg), num_blocks)
        else:
            self.h = lib().orc_solver_new(kind.encode(), n)
        self.n = n

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_solver_free(self.h)
            self.h = None

    def prepare(self, n):
        self.n = n
        lib().orc_prepare(self.h, n)

    def name(self):
        return lib().orc_name(self.h).decode()

    def reset_pattern(self):
        lib().orc_reset(self.h)

    def analyze(self, ap, ai):
        ap, ai = _i64(ap), _i64(ai)
        return lib().orc_analyze(self.h, _ptr(ap), len(ap), _ptr(ai), len(ai))

    def factor(self, ap, ai, ax):
        ap, ai, ax = _i64(ap), _i64(ai), _f64(ax)
        return lib().orc_factor(self.h, _ptr(ap), len(ap), _ptr(ai), _ptr(ax), len(ai))

    def solve(self, rhs):
        """Solves in place on a float64 copy; returns (status, x)."""
        x = _f64(rhs).copy()
        st = lib().orc_solve(self.h, _ptr(x), len(x))
        return st, x

    def klu_stats(self):
        out = np.zeros(7, np.int64)
        rc = C.c_double()
        if lib().orc_klu_stats(self.h, _ptr(out), C.byref(rc)) != 0:
            return None
        keys = ["factor_count", "refactor_count", "nnz_l", "nnz_u", "nblocks", "noffdiag",
                "repivots"]
        d = {k: int(v) for k, v in zip(keys, out)}
        d["rcond"] = rc.value
        return d

    def bbd_info(self):
        out = np.zeros(4, np.int64)
        perm = np.zeros(max(self.n, 1), np.int64)
        if lib().orc_bbd_info(self.h, _ptr(out), _ptr(perm)) != 0:
            return None
        return dict(num_blocks=int(out[0]), border_start=int(out[1]), border_size=int(out[2]),
                    fallback=bool(out[3]), perm=perm[:self.n])

    def klu_pivots(self):
        cap = max(self.n, 1)
        out = np.zeros(cap, np.int64)
        w = lib().orc_klu_pivots(self.h, _ptr(out), cap)
        return out[:w]


def amd(n, ap, ai):
    ap, ai = _i64(ap), _i64(ai)
    perm = np.zeros(n, np.int64)
    inv = np.zeros(n, np.int64)
    lib().orc_amd(n, _ptr(ap), _ptr(ai), _ptr(perm), _ptr(inv))
    return perm, inv


def btf(n, ap, ai):
    ap, ai = _i64(ap), _i64(ai)
    rp = np.zeros(n, np.int64)
    cp = np.zeros(n, np.int64)
    bp = np.zeros(n + 1, np.int64)
    info = np.zeros(4, np.int64)
    lib().orc_btf(n, _ptr(ap), _ptr(ai), _ptr(rp), _ptr(cp), _ptr(bp), _ptr(info))
    nb = int(info[0])
    return dict(row_perm=rp, col_perm=cp, block_ptr=bp[:nb + 1], num_blocks=nb,
                structural_rank=int(info[1]), num_singletons=int(info[2]),
                max_block_size=int(info[3]))


def _circ_arrays(c):
    return (_i64([0]) if False else None, np.ascontiguousarray(c.type, np.int32),
            np.ascontiguousarray(c.nodes, np.int32), _f64(c.p))


def mna(c, x, gmin=1e-12, scale=1.0, dt=0.0, cap_v=None, be_sign=-1.0, gdev=1e-12):
    """The reference engine's MNA build at x: (n, ap, ai, ax, rhs)."""
    _, t, nd, p = _circ_arrays(c)
    x = _f64(x)
    cv = _f64(cap_v) if cap_v is not None else None
    if cv is not None and len(cv) != c.ndev:  # one previous voltage per device
        raise ValueError(f"cap_v has {len(cv)} values, the circuit {c.ndev} devices")
    h = lib().orc_mna(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), _ptr(x), len(x),
                      gmin, scale, dt, _ptr(cv) if cv is not None else None, be_sign, gdev)
    n = C.c_int64()
    nnz = C.c_int64()
    lib().orc_mna_dims(h, C.byref(n), C.byref(nnz))
    ap = np.zeros(n.value + 1, np.int64)
    ai = np.zeros(nnz.value, np.int64)
    ax = np.zeros(nnz.value)
    rhs = np.zeros(n.value)
    lib().orc_mna_get(h, _ptr(ap), _ptr(ai), _ptr(ax), _ptr(rhs))
    lib().orc_mna_free(h)
    return n.value, ap, ai, ax, rhs


REASONS = {0: "converged", 1: "maxiters", 2: "solver_failure"}


def dc_op(c, solver="nativeklu", max_iters=100, abs_tol=1e-6, rel_tol=1e-3,
          gmin=1e-12, gmin_steps=0, source_steps=0, x0=None):
    """Engine DC operating point. Returns (reason, iterations, x)."""
    _, t, nd, p = _circ_arrays(c)
    x0a = _f64(x0) if x0 is not None else None
    cap = c.n
    x = np.zeros(cap)
    xl = C.c_int64()
    it = C.c_int64()
    r = lib().orc_dc_op(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), solver.encode(),
                        max_iters, abs_tol, rel_tol, gmin, gmin_steps, source_steps,
                        _ptr(x0a) if x0a is not None else None, _ptr(x), cap, C.byref(xl),
                        C.byref(it))
    return REASONS[r], it.value, x[:xl.value]


def tran(c, x_init, dt, steps, solver="nativeklu_exact", max_iters=100, abs_tol=1e-12,
         rel_tol=1e-10, gmin=1e-12):
    """Fixed-step backward Euler. Returns (reason, iterations, states[steps+1, nc])."""
    _, t, nd, p = _circ_arrays(c)
    xi = _f64(x_init)
    st = np.zeros((steps + 1) * c.node_count)
    it = C.c_int64()
    r = lib().orc_tran(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), solver.encode(),
                       max_iters, abs_tol, rel_tol, gmin, dt, steps, _ptr(xi), _ptr(st),
                       C.byref(it))
    return r, it.value, st.reshape(steps + 1, c.node_count)


def ac_sweep(c, x_dc, freqs):
    """AC solutions at a DC point: complex array [len(freqs), n] (n = nodes
    plus one aux per V source). V and I carry the AC magnitude in p[:, 1]
    and the phase in degrees in p[:, 2]."""
    _, t, nd, p = _circ_arrays(c)
    xd = _f64(x_dc)
    fr = _f64(freqs)
    cap = c.n
    re = np.zeros(len(fr) * cap)
    im = np.zeros(len(fr) * cap)
    n = C.c_int64()
    r = lib().orc_ac_sweep(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), _ptr(xd), len(xd),
                           _ptr(fr), len(fr), _ptr(re), _ptr(im), cap, C.byref(n))
    if r != 0:
        raise RuntimeError("singular AC system" if r == 1 else "AC system larger than expected")
    return (re + 1j * im).reshape(len(fr), cap)[:, :n.value]


def tran_adjoint(c, states, dt, probe, target, gmin=1e-12):
    """dL/dC per device (capacitors) for L = sum_t (x_t[probe] - target)^2."""
    _, t, nd, p = _circ_arrays(c)
    st = _f64(states).ravel()
    steps = states.shape[0] - 1
    g = np.zeros(c.ndev)
    r = lib().orc_tran_adjoint(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), dt, steps,
                               _ptr(st), probe, target, gmin, _ptr(g))
    if r != 0:
        raise RuntimeError("singular Jacobian in the transient adjoint")
    return g


def dc_op_bbd(c, assignment, num_blocks, max_iters=100, abs_tol=1e-6, rel_tol=1e-3,
              gmin=1e-12, gmin_steps=0, x0=None):
    """Engine DC operating point through the BbdSolver (known partition)."""
    _, t, nd, p = _circ_arrays(c)
    asg = _i64(assignment)
    x0a = _f64(x0) if x0 is not None else None
    x = np.zeros(c.n)
    xl = C.c_int64()
    it = C.c_int64()
    r = lib().orc_dc_op_bbd(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), _ptr(asg),
                            num_blocks, max_iters, abs_tol, rel_tol, gmin, gmin_steps,
                            _ptr(x0a) if x0a is not None else None, _ptr(x), c.n, C.byref(xl),
                            C.byref(it))
    return REASONS[r], it.value, x[:xl.value]


def dc_sweep(c, src_dev, values, solver="nativeklu", max_iters=100, abs_tol=1e-6,
             rel_tol=1e-3, gmin=1e-12, gmin_steps=0, x0=None, stop_on_failure=True):
    """The reference's .dc sweep (engine.rs:684-820). Returns (reason,
    iterations, x [points, n], x_len) per point; reason -1: not run."""
    _, t, nd, p = _circ_arrays(c)
    vals = _f64(values)
    npts = len(vals)
    x0a = None
    stride = 0
    if x0 is not None:
        x0a = _f64(np.asarray(x0).reshape(npts, -1))
        stride = x0a.shape[1]
    xo = np.zeros((npts, c.n))
    xl = np.zeros(npts, np.int64)
    it = np.zeros(npts, np.int64)
    rs = np.zeros(npts, np.int32)
    lib().orc_dc_sweep(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), solver.encode(),
                       max_iters, abs_tol, rel_tol, gmin, gmin_steps, src_dev, _ptr(vals), npts,
                       _ptr(x0a) if x0a is not None else None, stride, int(bool(stop_on_failure)),
                       _ptr(xo), c.n, _ptr(xl), _ptr(it), _ptr(rs))
    return rs, it, xo, xl


def residual(c, x, gmin=1e-12):
    _, t, nd, p = _circ_arrays(c)
    x = _f64(x)
    return lib().orc_residual(c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p),
                              _ptr(x), len(x), gmin)


def dc_batch(circuits, inst_circ, inst_dev, inst_val, solver="nativeklu", max_iters=100,
             abs_tol=1e-6, rel_tol=1e-3, gmin=1e-12, gmin_steps=0, nthreads=1, x_cap=0,
             x0=None, x0_off=None, sweep=True, perturbed_out=None):
    """DC operating points over a thread pool, circuit by circuit.

    sweep=True: the instances of a circuit are the points of its DC sweep,
    one solver for all of them, so the pivots of the first point are kept
    (the reference's .dc, engine.rs:684-820), each point from its own x0.
    sweep=False: every instance a separate .op with pivots of its own
    (engine.rs:249-283). perturbed_out (int64, one per instance): how many
    pivots NativeKLU replaced by +-1e-14 during the instance's solve."""
    x0a = _f64(x0) if x0 is not None else None
    x0o = _i64(x0_off) if x0_off is not None else None
    dev_off = np.zeros(len(circuits) + 1, np.int64)
    for i, c in enumerate(circuits):
        dev_off[i + 1] = dev_off[i] + c.ndev
    ncs = _i64([c.node_count for c in circuits])
    t = np.ascontiguousarray(np.concatenate([c.type for c in circuits]), np.int32)
    nd = np.ascontiguousarray(np.concatenate([c.nodes for c in circuits]), np.int32)
    p = _f64(np.concatenate([c.p for c in circuits]))
    ic, idv, iv = _i64(inst_circ), _i64(inst_dev), _f64(inst_val)
    ninst = len(ic)
    iters = np.zeros(ninst, np.int64)
    reason = np.zeros(ninst, np.int32)
    xo = np.zeros((ninst, max(x_cap, 1)))
    lib().orc_dc_batch(len(circuits), _ptr(dev_off), _ptr(ncs), _ptr(t), _ptr(nd), _ptr(p),
                       ninst, _ptr(ic), _ptr(idv), _ptr(iv), solver.encode(), max_iters,
                       abs_tol, rel_tol, gmin, gmin_steps,
                       _ptr(x0a) if x0a is not None else None,
                       _ptr(x0o) if x0o is not None else None, nthreads, _ptr(iters),
                       _ptr(reason), _ptr(xo) if x_cap > 0 else None, x_cap, int(sweep),
                       _ptr(perturbed_out) if perturbed_out is not None else None)
    return iters, reason, (xo if x_cap > 0 else None)


# ---------------------------------------------------------------- adaptive transient
def _waves(waves, ndev):
    from rustspice_gb300 import waveforms as wf
    return wf.pack(waves, ndev)


def wave_eval(w, ts):
    """WaveformSpec::evaluate of one waveform at the times ts."""
    from rustspice_gb300 import waveforms as wf
    kind, p7, ptr, pt, pv = wf.pack({0: w}, 1)
    ts = _f64(ts)
    out = np.zeros(len(ts))
    lib().orc_wave_eval(int(kind[0]), _ptr(p7), int(ptr[1]), _ptr(pt), _ptr(pv), len(ts),
                        _ptr(ts), _ptr(out))
    return out


def breakpoints(waves_list, tstop):
    """Sorted unique breakpoint times of the sources' PULSE and PWL waveforms."""
    kind, p7, ptr, pt, pv = _waves({i: w for i, w in enumerate(waves_list)}, len(waves_list))
    out = np.zeros(100000)
    n = lib().orc_breakpoints(len(waves_list), _ptr(kind), _ptr(p7), _ptr(ptr), _ptr(pt),
                              _ptr(pv), tstop, _ptr(out), len(out))
    return out[:n]


def bp_limit_dt(times, t, dt, margin):
    ts = _f64(times)
    return lib().orc_bp_limit_dt(_ptr(ts), len(ts), t, dt, margin)


def bp_settling(times, steps, factor, pairs):
    ts = _f64(times)
    tp = _f64([a for a, _ in pairs])
    tn = _f64([b for _, b in pairs])
    out = np.zeros(2 * len(pairs), np.int32)
    lib().orc_bp_settling(_ptr(ts), len(ts), steps, factor, len(pairs), _ptr(tp), _ptr(tn),
                          _ptr(out))
    return [(bool(out[2 * i]), bool(out[2 * i + 1])) for i in range(len(pairs))]


def lte_milne(x_be, x_trap, abs_tol, rel_tol):
    be, tr = _f64(x_be), _f64(x_trap)
    out = np.zeros(5)
    lib().orc_lte(_ptr(be), _ptr(tr), len(be), abs_tol, rel_tol, _ptr(out))
    return {"error_norm": out[0], "max_error_node": int(out[1]), "accept": bool(out[2]),
            "suggested_factor": out[3], "raw_lte": out[4]}


def adaptive_sequence(dt_min, dt_max, errors, dts):
    """Feeds error ratios through the adaptive controller; per step
    (accept, next_dt, struggling, PI suggestion)."""
    e, d = _f64(errors), _f64(dts)
    out = np.zeros(4 * len(e))
    lib().orc_adaptive_sequence(dt_min, dt_max, len(e), _ptr(e), _ptr(d), _ptr(out))
    o = out.reshape(-1, 4)
    return [(bool(r[0]), r[1], bool(r[2]), r[3]) for r in o]


def tran_adaptive(c, waves, tstep, tstop, tstart=0.0, tmax=None, solver="nativeklu_exact",
                  max_iters=100, abs_tol=1e-6, rel_tol=1e-3, gmin=1e-12, lte_abs=None,
                  lte_rel=None, be_sign=1.0, x_ic=None, cap=100000):
    """The engine's adaptive transient. Returns dict(status, times,
    solutions[points, n], accepted, rejected, newton_iterations)."""
    _, t, nd, p = _circ_arrays(c)
    kind, p7, ptr, pt, pv = _waves(waves, c.ndev)
    xi = _f64(x_ic if x_ic is not None else np.zeros(c.node_count))
    n = c.n
    times = np.zeros(cap)
    sols = np.zeros(cap * n)
    st = np.zeros(4, np.int64)
    r = lib().orc_tran_adaptive(
        c.node_count, c.ndev, _ptr(t), _ptr(nd), _ptr(p), _ptr(kind), _ptr(p7), _ptr(ptr),
        _ptr(pt), _ptr(pv), solver.encode(), max_iters, abs_tol, rel_tol, gmin, tstep, tstop,
        tstart, tstop if tmax is None else tmax, abs_tol if lte_abs is None else lte_abs,
        rel_tol if lte_rel is None else lte_rel, be_sign, _ptr(xi), cap, n, _ptr(times),
        _ptr(sols), _ptr(st))
    npts = min(int(st[3]), cap)
    return {"status": r, "times": times[:npts], "solutions": sols.reshape(cap, n)[:npts],
            "accepted": int(st[0]), "rejected": int(st[1]), "newton_iterations": int(st[2])}
