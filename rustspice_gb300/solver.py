"""Python face of libgpuklu, shaped like the reference's Rust API.

* ``GpuKluSolver`` mirrors the ``LinearSolver`` trait
  (crates/sim-core/src/solver.rs:141-166): prepare / analyze / factor /
  solve / reset_pattern / name / set_parallel_threads, with the same error
  behaviour (``SolverError`` is raised with the status of the C ABI).
* ``DeviceCircuit`` is the compiled device-stamp plan and ``newton_dc`` the
  device-resident DC operating point (crates/sim-core/src/engine.rs:249-311).
* ``Batch`` runs many independent operating points in one kernel launch.

Everything numeric runs on the GPU; constructing any of these without a CUDA
device raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import native as N
from .circuits import Circuit

STATUS_NAMES = {0: "Ok", 1: "AnalyzeFailed", 2: "FactorFailed", 3: "SolveFailed",
                4: "SingularMatrix", 5: "IllConditioned", 6: "InvalidMatrix",
                7: "DeviceTimeout", 8: "NonFinite", 9: "CudaError"}


class SolverError(RuntimeError):
    """Mirror of SolverError (crates/sim-core/src/solver.rs:76-92)."""

    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class GpuKluSolver:
    """Drop-in for NativeKluSolver / KluSolver behind the LinearSolver trait."""

    def __init__(self, n: int = 0, pivot_mode: int = N.PIVOT_REFERENCE,
                 kind: str = "nativeklu"):
        """kind: the reference solver restated - "nativeklu" (NativeKluSolver),
        "sparselu" (SparseLuSolver) or "sparselubtf" (SparseLuBtfSolver)."""
        L = N.lib()
        self._h = L.gpuklu_create(n)
        if not self._h:
            raise RuntimeError("gpuklu_create failed: no usable CUDA device")
        self._n = n
        if pivot_mode != N.PIVOT_REFERENCE:
            L.gpuklu_set_pivot_mode(self._h, pivot_mode)
        if kind != "nativeklu":
            self._check(L.gpuklu_set_solver_kind(self._h, N.KINDS[kind]))

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, st: int):
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_last_error(self._h).decode())

    # -- trait
    def prepare(self, n: int) -> None:
        self._n = n
        N.lib().gpuklu_prepare(self._h, n)

    def analyze(self, ap, ai) -> None:
        ap, ai = N.i64(ap), N.i64(ai)
        self._check(N.lib().gpuklu_analyze(self._h, N.ptr(ap), len(ap), N.ptr(ai), len(ai)))

    def factor(self, ap, ai, ax) -> None:
        ap, ai, ax = N.i64(ap), N.i64(ai), N.f64(ax)
        if len(ax) != len(ai):
            raise SolverError(N.INVALID_MATRIX, "ax and ai lengths differ")
        self._check(N.lib().gpuklu_factor(self._h, N.ptr(ap), len(ap), N.ptr(ai), len(ai),
                                          N.ptr(ax)))

    def solve(self, rhs: np.ndarray) -> None:
        """Overwrites ``rhs`` (a float64 numpy array) with x."""
        if not (isinstance(rhs, np.ndarray) and rhs.dtype == np.float64 and rhs.flags.c_contiguous):
            raise TypeError("rhs must be a contiguous float64 numpy array")
        self._check(N.lib().gpuklu_solve(self._h, N.ptr(rhs), len(rhs)))

    def tsolve(self, g: np.ndarray) -> None:
        """Overwrites ``g`` with y solving A^T y = g (adjoint)."""
        self._check(N.lib().gpuklu_tsolve(self._h, N.ptr(g), len(g)))

    def reset_pattern(self) -> None:
        N.lib().gpuklu_reset_pattern(self._h)

    def name(self) -> str:
        return N.lib().gpuklu_name(self._h).decode()

    def set_parallel_threads(self, threads: int) -> None:
        N.lib().gpuklu_set_parallel_threads(self._h, threads)

    # -- extensions
    def set_pivot_mode(self, mode: int) -> None:
        self._check(N.lib().gpuklu_set_pivot_mode(self._h, mode))

    def set_repivot(self, on: bool) -> None:
        """Growth-triggered re-pivot after refactorizations (off: the
        reference's kept pivots)."""
        self._check(N.lib().gpuklu_set_repivot(self.handle, int(bool(on))))

    def repivots(self) -> int:
        return int(N.lib().gpuklu_repivot_count(self.handle))

    def set_spin_limit(self, polls: int) -> None:
        """Polls of a device dependency flag before the waiting warp gives up
        and the call raises SolverError(DEVICE_TIMEOUT); 0: the default."""
        self._check(N.lib().gpuklu_set_spin_limit(self.handle, int(polls)))

    def set_stop_on_nonfinite(self, on: bool) -> None:
        """End the device Newton loop at the first NaN/Inf iterate with
        SolverError(NONFINITE) (off: run on to the iteration cap, as the
        reference does)."""
        self._check(N.lib().gpuklu_set_stop_on_nonfinite(self.handle, int(bool(on))))

    def stats(self) -> dict:
        s = N.Stats()
        self._check(N.lib().gpuklu_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.Stats._fields_}

    def pivot_passes(self) -> int:
        """Refactorizations the last first factorization used to find its
        pivots (0: the sequential pivot pass ran)."""
        return int(N.lib().gpuklu_pivot_pass_count(self._h))


class DeviceCircuit:
    """A circuit compiled into its stamp-to-slot map on the device."""

    def __init__(self, c: Circuit, transient: bool = False):
        self.circuit = c
        t, nd, p = N.i32(c.type), N.i32(c.nodes), N.f64(c.p)
        self._h = N.lib().gpuklu_compile_devices(c.node_count, c.ndev, N.ptr(t), N.ptr(nd),
                                                 N.ptr(p), 1 if transient else 0)
        if not self._h:
            raise RuntimeError("gpuklu_compile_devices failed")
        n = C.c_int64()
        nnz = C.c_int64()
        N.lib().gpuklu_circuit_dims(self._h, C.byref(n), C.byref(nnz))
        self.n, self.nnz_raw = n.value, nnz.value

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_circuit_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def pattern(self):
        ap = np.zeros(self.n + 1, np.int64)
        ai = np.zeros(self.nnz_raw, np.int64)
        N.lib().gpuklu_circuit_pattern(self._h, N.ptr(ap), N.ptr(ai))
        return ap, ai

    def set_params(self, p):
        p = N.f64(p)
        if N.lib().gpuklu_circuit_set_params(self._h, N.ptr(p)) != N.OK:
            raise RuntimeError("set_params failed")

    def stamp(self, solver: GpuKluSolver, x, gmin=1e-12, source_scale=1.0, dt=0.0,
              cap_v=None, be_sign=-1.0):
        """Device stamp at x: (ax_raw, rhs) copied back."""
        x = N.f64(x)
        ax = np.zeros(self.nnz_raw)
        rhs = np.zeros(self.n)
        cv = N.f64(cap_v) if cap_v is not None else None
        if cv is not None and len(cv) != self.circuit.ndev:  # one previous voltage per device
            raise ValueError(f"cap_v has {len(cv)} values, the circuit {self.circuit.ndev} devices")
        st = N.lib().gpuklu_stamp(solver.handle, self._h, N.ptr(x), len(x), gmin, source_scale,
                                  dt, N.ptr(cv) if cv is not None else None, be_sign,
                                  N.ptr(ax), N.ptr(rhs))
        solver._check(st)
        return ax, rhs


@dataclasses.dataclass
class NewtonResult:
    converged: bool
    iterations: int
    iterations_total: int
    reason: str
    x: np.ndarray


REASONS = {0: "converged", 1: "maxiters", 2: "solver_failure"}


def newton_dc(solver: GpuKluSolver, dc: DeviceCircuit, cfg: N.NewtonConfig,
              x0=None) -> NewtonResult:
    """Device-resident DC operating point through ``solver``."""
    n = dc.n
    x = np.zeros(n)
    xl = C.c_int64()
    it = C.c_int64()
    itt = C.c_int64()
    rs = C.c_int()
    x0a = N.f64(x0) if x0 is not None else None
    st = N.lib().gpuklu_newton_dc(solver.handle, dc.handle, C.byref(cfg),
                                  N.ptr(x0a) if x0a is not None else None, N.ptr(x), n,
                                  C.byref(xl), C.byref(it), C.byref(itt), C.byref(rs))
    solver._check(st)
    return NewtonResult(rs.value == 0, it.value, itt.value, REASONS[rs.value], x[:xl.value])


@dataclasses.dataclass
class SweepResult:
    reason: np.ndarray          # per point: 0 converged, 1 max iterations, 2 solver failure,
    iterations: np.ndarray      # -1 not run (the sweep stopped before it)
    iterations_total: np.ndarray
    x: np.ndarray               # [points, n]; zero beyond x_len
    x_len: np.ndarray


def dc_sweep(solver: GpuKluSolver, dc: DeviceCircuit, cfg: N.NewtonConfig, src_dev: int,
             values, x0=None, stop_on_failure: bool = True) -> SweepResult:
    """The reference's .dc sweep of one source on the device
    (engine.rs:684-820): one solver for all points, so the first point's
    pivots are kept. x0 None: continuation from the previous point; else an
    array [points, node_count] of initial iterates."""
    vals = N.f64(values)
    npts = len(vals)
    n = dc.n
    xo = np.zeros((npts, n))
    xl = np.zeros(npts, np.int64)
    it = np.zeros(npts, np.int64)
    itt = np.zeros(npts, np.int64)
    rs = np.zeros(npts, np.int32)
    x0a = None
    stride = 0
    if x0 is not None:
        x0a = N.f64(np.asarray(x0).reshape(npts, -1))
        stride = x0a.shape[1]
    st = N.lib().gpuklu_dc_sweep(solver.handle, dc.handle, C.byref(cfg), int(src_dev),
                                 N.ptr(vals), npts, N.ptr(x0a) if x0a is not None else None,
                                 stride, int(bool(stop_on_failure)), N.ptr(xo), n, N.ptr(xl),
                                 N.ptr(it), N.ptr(itt), N.ptr(rs))
    solver._check(st)
    return SweepResult(rs, it, itt, xo, xl)


def ac_sweep(solver: GpuKluSolver, dc: DeviceCircuit, x_dc, freqs) -> np.ndarray:
    """AC small-signal solutions at the operating point x_dc for every
    frequency (the reference's .ac): complex array [len(freqs), n]. V and I
    sources carry the AC magnitude in p[:, 1] and the phase [deg] in p[:, 2]."""
    x = N.f64(x_dc)
    fr = N.f64(freqs)
    re = np.zeros(len(fr) * dc.n)
    im = np.zeros(len(fr) * dc.n)
    n = C.c_int64()
    solver._check(N.lib().gpuklu_ac_sweep(solver.handle, dc.handle, N.ptr(x), len(x), N.ptr(fr),
                                          len(fr), N.ptr(re), N.ptr(im), C.byref(n)))
    return (re + 1j * im).reshape(len(fr), dc.n)


def frequency_sweep(kind: str, points: int, fstart: float, fstop: float) -> np.ndarray:
    """The reference's .ac frequency list (crates/sim-core/src/engine.rs:
    1002-1042): "dec" and "oct" points per decade / octave, "lin" points."""
    import math
    kind = kind.lower()
    if kind == "oct":
        octaves = math.log2(fstop / fstart)
        total = int(math.ceil(octaves * points)) + 1
        return np.array([fstart * 2.0 ** ((i * octaves) / max(total - 1, 1))
                         for i in range(total)])
    if kind == "lin":
        step = (fstop - fstart) / max(points - 1, 1)
        return np.array([fstart + i * step for i in range(points)])
    ls, lt = math.log10(fstart), math.log10(fstop)
    dec = lt - ls
    total = int(math.ceil(dec * points)) + 1
    return np.array([10.0 ** (ls + (i * dec) / max(total - 1, 1)) for i in range(total)])


def dc_forward(solver: GpuKluSolver, dc: DeviceCircuit, cfg: N.NewtonConfig,
               x0=None) -> NewtonResult:
    """Forward half of the DC operating-point function pair (newton_dc)."""
    return newton_dc(solver, dc, cfg, x0)


def dc_backward(solver: GpuKluSolver, dc: DeviceCircuit, x, dl_dx, gmin: float = 1e-12):
    """Backward half: (lambda, dL/dp per device) at the converged x."""
    x = N.f64(x)
    g = N.f64(dl_dx)
    if len(g) != dc.n:
        raise ValueError("dl_dx must have n values")
    lam = np.zeros(dc.n)
    grad = np.zeros(dc.circuit.ndev)
    solver._check(N.lib().gpuklu_dc_backward(solver.handle, dc.handle, N.ptr(x), len(x),
                                             N.ptr(g), gmin, N.ptr(lam), N.ptr(grad)))
    return lam, grad


class Batch:
    """Independent DC operating points of many circuit instances.

    ``circuits``: list of Circuit; ``inst_circ[i]``: circuit of instance i
    (instances of one circuit must be consecutive); ``inst_dev[i]`` / ``inst_val[i]``:
    device whose first parameter is overridden and its value (-1: none);
    ``x0``/``x0_off``: flat initial iterates and their offsets (-1: zero start).
    """

    def __init__(self, circuits, inst_circ, inst_dev=None, inst_val=None, x0=None, x0_off=None):
        self.circuits = circuits
        ninst = len(inst_circ)
        dev_off = np.zeros(len(circuits) + 1, np.int64)
        for i, c in enumerate(circuits):
            dev_off[i + 1] = dev_off[i] + c.ndev
        ncs = N.i64([c.node_count for c in circuits])
        t = N.i32(np.concatenate([c.type for c in circuits]))
        nd = N.i32(np.concatenate([c.nodes for c in circuits]))
        p = N.f64(np.concatenate([c.p for c in circuits]))
        self.inst_circ = N.i64(inst_circ)
        idev = N.i64(inst_dev if inst_dev is not None else -np.ones(ninst))
        ival = N.f64(inst_val if inst_val is not None else np.zeros(ninst))
        x0a = N.f64(x0) if x0 is not None else None
        x0o = N.i64(x0_off) if x0_off is not None else None
        self._h = N.lib().gpuklu_batch_create(
            len(circuits), N.ptr(dev_off), N.ptr(ncs), N.ptr(t), N.ptr(nd), N.ptr(p), ninst,
            N.ptr(self.inst_circ), N.ptr(idev), N.ptr(ival),
            N.ptr(x0a) if x0a is not None else None, N.ptr(x0o) if x0o is not None else None,
            len(x0a) if x0a is not None else 0)
        if not self._h:
            raise RuntimeError("gpuklu_batch_create failed")
        self.ninst = ninst
        ns = np.array([c.n for c in circuits], np.int64)[self.inst_circ]
        self.x_off = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
        self.x_len = int(ns.sum())

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, cfg: N.NewtonConfig):
        st = N.lib().gpuklu_batch_run(self._h, C.byref(cfg))
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())

    def update_inputs(self, inst_val=None, x0=None):
        iv = N.f64(inst_val) if inst_val is not None else None
        xa = N.f64(x0) if x0 is not None else None
        st = N.lib().gpuklu_batch_update_inputs(self._h, N.ptr(iv) if iv is not None else None,
                                                N.ptr(xa) if xa is not None else None)
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())

    def results(self, with_x: bool = True, x_out: np.ndarray = None):
        """Iterations, total iterations, exit reasons and (with_x) the
        solutions, concatenated per instance. x_out: a float64 buffer of
        x_len values to fill instead of a new array (pinned memory makes
        the copy a DMA)."""
        it = np.zeros(self.ninst, np.int64)
        itt = np.zeros(self.ninst, np.int64)
        rs = np.zeros(self.ninst, np.int32)
        if with_x and x_out is not None:
            if not (x_out.dtype == np.float64 and x_out.flags.c_contiguous
                    and len(x_out) >= self.x_len):
                raise TypeError("x_out must be a contiguous float64 array of x_len values")
            x = x_out
        else:
            x = np.zeros(self.x_len) if with_x else None
        st = N.lib().gpuklu_batch_results(self._h, N.ptr(it), N.ptr(itt), N.ptr(rs),
                                          N.ptr(x) if with_x else None,
                                          N.ptr(self.x_off) if with_x else None)
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())
        return it, itt, rs, x

    def info(self) -> dict:
        out = np.zeros(8, np.int64)
        N.lib().gpuklu_batch_info(self._h, N.ptr(out))
        return dict(grid=int(out[0]), block=int(out[1]), groups=int(out[2]),
                    smem_per_warp=int(out[3]), regs=int(out[4]), blocks_per_sm=int(out[5]),
                    launches=int(out[6]), cont_kernel=bool(out[7]))

    def work(self):
        """Per instance: FP64 operations and on-chip value bytes of one iteration."""
        f = np.zeros(self.ninst, np.int64)
        b = np.zeros(self.ninst, np.int64)
        N.lib().gpuklu_batch_work(self._h, N.ptr(f), N.ptr(b))
        return f, b

    def stream(self) -> int:
        return N.lib().gpuklu_batch_stream(self._h) or 0

    def phase_ms(self) -> dict:
        """Device time of the last run by kernel (CUDA events; waits for the
        run): the lane-per-instance kernel, the warp kernels after it, and
        the lane kernel's iteration cap."""
        out = np.zeros(3)
        st = N.lib().gpuklu_batch_phase_ms(self._h, N.ptr(out))
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())
        return {"lanes_ms": float(out[0]), "warps_ms": float(out[1]), "lane_cap": int(out[2])}

    def set_schedule(self, lane_cap: int, cont_tiles: int) -> None:
        """Lane-phase iteration cap and continuation tiles per program."""
        st = N.lib().gpuklu_batch_set_schedule(self._h, int(lane_cap), int(cont_tiles))
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())

    def autotune(self, cfg: N.NewtonConfig) -> dict:
        """Times the batch under candidate schedules and keeps the fastest
        (the results afterwards are the last trial's: run again)."""
        out = np.zeros(3, np.int64)
        ms = C.c_double()
        st = N.lib().gpuklu_batch_autotune(self._h, C.byref(cfg), N.ptr(out), C.byref(ms))
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())
        return {"lane_cap": int(out[0]), "cont_tiles": int(out[1]), "runs": int(out[2]),
                "best_ms": ms.value}


@dataclasses.dataclass
class ATranResult:
    status: np.ndarray          # per instance: 0 completed, 1 rejections, 2 DC failed, 3 budget
    times: list                 # per instance: accepted times (the DC point first)
    probe: list                 # per instance: the probe node's voltage at those times
    npoints: np.ndarray
    accepted: np.ndarray
    rejected: np.ndarray
    iterations: np.ndarray
    x: list                     # per instance: the last accepted solution (n values)


class ATranBatch:
    """The engine's adaptive transient (engine.rs:332-602) on many circuits
    at once, one warp per circuit, the time loop on the device. waves: per
    circuit a dict {device: rustspice_gb300.waveforms.Waveform} of time
    dependent V / I sources; x_ic: per circuit the .ic initial guess of the
    DC point (node_count values) or None; probe: recorded node per circuit."""

    def __init__(self, circuits, waves=None, x_ic=None, probe=1):
        from . import waveforms as wf
        self.circuits = circuits
        n = len(circuits)
        dev_off = np.zeros(n + 1, np.int64)
        for i, c in enumerate(circuits):
            dev_off[i + 1] = dev_off[i] + c.ndev
        ncs = N.i64([c.node_count for c in circuits])
        t = N.i32(np.concatenate([c.type for c in circuits]))
        nd = N.i32(np.concatenate([c.nodes for c in circuits]))
        p = N.f64(np.concatenate([c.p for c in circuits]))
        kinds, p7s, pts_t, pts_v, ptr = [], [], [], [], [0]
        for i, c in enumerate(circuits):
            k, q, pp, pt, pv = wf.pack((waves or [None] * n)[i] or {}, c.ndev)
            kinds.append(k)
            p7s.append(q)
            pts_t.append(pt)
            pts_v.append(pv)
            ptr.extend(ptr[-1] + pp[1:])
        self._wk = N.i32(np.concatenate(kinds))
        self._wp = N.f64(np.concatenate(p7s))
        self._pp = N.i64(ptr)
        self._pt = N.f64(np.concatenate(pts_t) if pts_t else np.zeros(0))
        self._pv = N.f64(np.concatenate(pts_v) if pts_v else np.zeros(0))
        xs = [np.zeros(c.node_count) if (x_ic is None or x_ic[i] is None) else
              np.asarray(x_ic[i], np.float64) for i, c in enumerate(circuits)]
        xo = np.zeros(n, np.int64)
        for i in range(1, n):
            xo[i] = xo[i - 1] + circuits[i - 1].node_count
        xi = N.f64(np.concatenate(xs))
        pr = N.i64(np.broadcast_to(np.asarray(probe, np.int64), (n,)).copy())
        self._h = N.lib().gpuklu_atran_create(
            n, N.ptr(dev_off), N.ptr(ncs), N.ptr(t), N.ptr(nd), N.ptr(p), N.ptr(self._wk),
            N.ptr(self._wp), N.ptr(self._pp), N.ptr(self._pt), N.ptr(self._pv), N.ptr(xi),
            N.ptr(N.i64(xo)), len(xi), N.ptr(pr))
        if not self._h:
            raise RuntimeError("gpuklu_atran_create failed")
        self.x_off = np.cumsum([0] + [c.n for c in circuits])[:-1]

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, cfg: N.NewtonConfig, tstep, tstop, tstart=0.0, tmax=None, lte_abs=None,
            lte_rel=None, be_sign=1.0, max_points=4096, max_steps=1_000_000) -> ATranResult:
        """lte_abs / lte_rel default to the Newton config's abs_tol / rel_tol
        (the engine passes vntol and reltol to both)."""
        n = len(self.circuits)
        times = np.zeros(n * max_points)
        probe = np.zeros(n * max_points)
        npts, acc, rej, its = (np.zeros(n, np.int64) for _ in range(4))
        st = np.zeros(n, np.int32)
        xo = np.zeros(int(sum(c.n for c in self.circuits)))
        r = N.lib().gpuklu_atran_run(
            self._h, C.byref(cfg), tstep, tstop, tstart, tstop if tmax is None else tmax,
            cfg.abs_tol if lte_abs is None else lte_abs, cfg.rel_tol if lte_rel is None else lte_rel,
            be_sign, max_points, max_steps, N.ptr(times), N.ptr(probe), N.ptr(npts), N.ptr(acc),
            N.ptr(rej), N.ptr(st), N.ptr(its), N.ptr(xo))
        if r != N.OK:
            raise SolverError(r, N.lib().gpuklu_batch_last_error(self._h).decode())
        k = np.minimum(npts, max_points)
        return ATranResult(
            st, [times[i * max_points:i * max_points + k[i]] for i in range(n)],
            [probe[i * max_points:i * max_points + k[i]] for i in range(n)], npts, acc, rej, its,
            [xo[self.x_off[i]:self.x_off[i] + c.n] for i, c in enumerate(self.circuits)])


class TranBatch:
    """Fixed-step backward-Euler transient of many circuits (one instance per
    circuit) with the checkpointed adjoint of
    L_i = sum_t (x_t[probe_i] - target)^2 with respect to every capacitance."""

    def __init__(self, circuits, x_init, x_off, dt, steps, ckpt_every, probe, target):
        self.circuits = circuits
        n = len(circuits)
        dev_off = np.zeros(n + 1, np.int64)
        for i, c in enumerate(circuits):
            dev_off[i + 1] = dev_off[i] + c.ndev
        self.dev_off = dev_off
        ncs = N.i64([c.node_count for c in circuits])
        t = N.i32(np.concatenate([c.type for c in circuits]))
        nd = N.i32(np.concatenate([c.nodes for c in circuits]))
        p = N.f64(np.concatenate([c.p for c in circuits]))
        xi, xo = N.f64(x_init), N.i64(x_off)
        pr = N.i64(np.broadcast_to(np.asarray(probe, np.int64), (n,)).copy())
        self.steps = int(steps)
        self._h = N.lib().gpuklu_tran_create(n, N.ptr(dev_off), N.ptr(ncs), N.ptr(t), N.ptr(nd),
                                             N.ptr(p), N.ptr(xi), N.ptr(xo), len(xi), dt, steps,
                                             ckpt_every, N.ptr(pr), target)
        if not self._h:
            raise RuntimeError("gpuklu_tran_create failed")

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _err(self, st):
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_batch_last_error(self._h).decode())

    def forward(self, cfg: N.NewtonConfig, with_wave: bool = False):
        """(loss, wave or None, iterations, reason) per instance."""
        n = len(self.circuits)
        loss = np.zeros(n)
        wave = np.zeros((n, self.steps)) if with_wave else None
        it = np.zeros(n, np.int64)
        rs = np.zeros(n, np.int32)
        self._err(N.lib().gpuklu_tran_forward(self._h, C.byref(cfg), N.ptr(loss),
                                              N.ptr(wave) if with_wave else None, N.ptr(it),
                                              N.ptr(rs)))
        return loss, wave, it, rs

    def backward(self, cfg: N.NewtonConfig):
        """dL_i/dp[d][0] per device of every instance (list of arrays), and the
        Newton iterations of the recomputation."""
        g = np.zeros(int(self.dev_off[-1]))
        it = np.zeros(len(self.circuits), np.int64)
        self._err(N.lib().gpuklu_tran_backward(self._h, C.byref(cfg), N.ptr(g), N.ptr(it)))
        return [g[self.dev_off[i]:self.dev_off[i + 1]] for i in range(len(self.circuits))], it

    def stream(self) -> int:
        return N.lib().gpuklu_batch_stream(self._h) or 0


class BbdSolver:
    """The reference's BbdSolver with a known partition, on the GPU.

    ``assignment[i]``: block of node i, -1 for the border. ``factor`` /
    ``solve`` follow the LinearSolver calls (host arrays, original order);
    ``newton_dc`` runs the device Newton loop of a compiled circuit whose
    pattern is the solver's."""

    def __init__(self, ap, ai, assignment, num_blocks):
        ap, ai, asg = N.i64(ap), N.i64(ai), N.i64(assignment)
        self.n = len(ap) - 1
        self._h = N.lib().gpuklu_bbd_create(self.n, N.ptr(ap), len(ap), N.ptr(ai), len(ai),
                                            N.ptr(asg), num_blocks)
        if not self._h:
            raise RuntimeError("gpuklu_bbd_create failed")
        self.nnz = len(ai)

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gpuklu_bbd_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, st):
        if st != N.OK:
            raise SolverError(st, N.lib().gpuklu_bbd_last_error(self._h).decode())

    def info(self) -> dict:
        out = np.zeros(6, np.int64)
        self._check(N.lib().gpuklu_bbd_info(self._h, N.ptr(out)))
        return dict(num_blocks=int(out[0]), border_start=int(out[1]), border_size=int(out[2]),
                    fallback=bool(out[3]), tiles=int(out[4]), inner_blocks=int(out[5]))

    def perm(self) -> np.ndarray:
        p = np.zeros(self.n, np.int64)
        self._check(N.lib().gpuklu_bbd_perm(self._h, N.ptr(p)))
        return p

    def factor(self, ax) -> None:
        ax = N.f64(ax)
        if len(ax) != self.nnz:
            raise SolverError(N.INVALID_MATRIX, "ax and ai lengths differ")
        self._check(N.lib().gpuklu_bbd_factor(self._h, N.ptr(ax)))

    def solve(self, rhs: np.ndarray) -> None:
        """Overwrites ``rhs`` (contiguous float64) with x."""
        if not (isinstance(rhs, np.ndarray) and rhs.dtype == np.float64 and rhs.flags.c_contiguous):
            raise TypeError("rhs must be a contiguous float64 numpy array")
        self._check(N.lib().gpuklu_bbd_solve(self._h, N.ptr(rhs), len(rhs)))

    def newton_dc(self, dc: "DeviceCircuit", cfg: N.NewtonConfig, x0=None) -> NewtonResult:
        n = dc.n
        x = np.zeros(n)
        xl = C.c_int64()
        it = C.c_int64()
        itt = C.c_int64()
        rs = C.c_int()
        x0a = N.f64(x0) if x0 is not None else None
        self._check(N.lib().gpuklu_bbd_newton_dc(self._h, dc.handle, C.byref(cfg),
                                                 N.ptr(x0a) if x0a is not None else None,
                                                 N.ptr(x), n, C.byref(xl), C.byref(it),
                                                 C.byref(itt), C.byref(rs)))
        return NewtonResult(rs.value == 0, it.value, itt.value, REASONS[rs.value], x[:xl.value])



# ---------------------------------------------------------------- selection
# The reference's solver factory and selector (crates/sim-core/src/solver.rs:
# 169-258, 262-562) for its default build, which has neither the `klu`
# feature nor faer: KLU and Faer requests fall back to SparseLU (:174-196),
# and "auto" is Dense up to 50 unknowns, SparseLU up to 500, SparseLU-BTF
# beyond (:215-246). Every kind runs on the device through GpuKluSolver.
SOLVER_TYPES = ("dense", "sparselu", "sparselubtf", "bbd", "faer", "klu", "nativeklu", "auto")


def solver_kind(solver_type: str, n: int) -> str:
    """The device solver kind create_solver(solver_type, n) amounts to."""
    if solver_type not in SOLVER_TYPES:
        raise ValueError(f"unknown solver type {solver_type!r}")
    if solver_type == "auto":
        if n <= 50:
            return "dense"
        return "sparselubtf" if n > 500 else "sparselu"
    if solver_type in ("klu", "faer"):
        return "sparselu"
    if solver_type == "bbd":
        raise NotImplementedError("the BBD solver here takes a known partition: use BbdSolver")
    return solver_type


def create_solver(solver_type: str, n: int) -> GpuKluSolver:
    """create_solver (solver.rs:169-200)."""
    return GpuKluSolver(n, kind=solver_kind(solver_type, n))


def create_solver_auto(n: int) -> GpuKluSolver:
    """create_solver_auto (solver.rs:215-246)."""
    return create_solver("auto", n)


@dataclasses.dataclass
class MatrixProperties:
    """MatrixProperties (solver.rs:243-338)."""
    n: int
    nnz: int
    density: float
    avg_degree: float
    has_block_structure: bool
    num_blocks: int
    max_block_ratio: float

    @classmethod
    def analyze(cls, n: int, ap, ai) -> "MatrixProperties":
        if n == 0:
            return cls(0, 0, 0.0, 0.0, False, 0, 0.0)
        ap, ai = N.i64(ap), N.i64(ai)
        nnz = int(ap[n])
        out = np.zeros(2, np.int64)
        st = N.lib().gpuklu_btf_info(n, N.ptr(ap), N.ptr(ai), N.ptr(out))
        if st != N.OK:
            raise SolverError(st, "btf analysis")
        nb, mx = int(out[0]), int(out[1])
        return cls(n, nnz, nnz / float(n * n), nnz / float(n), nb > 1 and mx < n, nb, mx / float(n))

    @classmethod
    def analyze_quick(cls, n: int, ap, _ai=None) -> "MatrixProperties":
        if n == 0:
            return cls(0, 0, 0.0, 0.0, False, 1, 1.0)
        nnz = int(np.asarray(ap)[n])
        return cls(n, nnz, nnz / float(n * n), nnz / float(n), False, 1, 1.0)


@dataclasses.dataclass
class SolverSelector:
    """SolverSelector (solver.rs:383-527): the decision tree of the default
    build on a matrix's properties, with the reason text."""
    properties: MatrixProperties
    selected: str
    reason: str

    @classmethod
    def select(cls, n: int, ap, ai) -> "SolverSelector":
        return cls.select_from_properties(MatrixProperties.analyze(n, ap, ai))

    @classmethod
    def select_quick(cls, n: int, ap, ai=None) -> "SolverSelector":
        return cls.select_from_properties(MatrixProperties.analyze_quick(n, ap, ai))

    @classmethod
    def select_from_properties(cls, p: MatrixProperties) -> "SolverSelector":
        n, density = p.n, p.density
        if n <= 50:
            return cls(p, "dense", f"Small matrix (n={n}) - Dense solver has lowest overhead")
        if density > 0.3 and n <= 200:
            return cls(p, "dense", f"Dense matrix ({density * 100.0:.1f}% fill, n={n}) - "
                                   "Dense solver efficient")
        if p.has_block_structure and p.num_blocks > 1:
            est = p.num_blocks ** 2 / (1.0 + p.max_block_ratio ** 3 * p.num_blocks)
            return cls(p, "sparselubtf",
                       f"Block structure detected ({p.num_blocks} blocks, max "
                       f"{p.max_block_ratio * 100.0:.0f}% of n) - SparseLU-BTF "
                       f"~{max(est, 1.0):.1f}x faster")
        if n >= 200 and density < 0.15:
            return cls(p, "bbd", f"Large sparse matrix (n={n}, {density * 100.0:.1f}% fill) - "
                                 "BBD partitioning")
        if n > 500:
            return cls(p, "sparselubtf",
                       f"Large matrix (n={n}) - SparseLU-BTF may find hidden structure")
        return cls(p, "sparselu", f"Medium sparse matrix (n={n}, {density * 100.0:.1f}% fill) - "
                                  "SparseLU selected")

    def create_solver(self) -> GpuKluSolver:
        return create_solver(self.selected, self.properties.n)


def create_solver_for_matrix(n: int, ap, ai) -> GpuKluSolver:
    """create_solver_for_matrix (solver.rs:551-554)."""
    return SolverSelector.select(n, ap, ai).create_solver()


def dense_lu_nopivot(a, variant: int = 1):
    """The BBD solver's dense Schur LU (no pivoting, +-1e-14 rule) of a square
    matrix on the device: returns (lu, ms) with L below the diagonal (unit
    diagonal implied) and U on and above it, and the factorization's device
    time. variant 0: panel kernels; 1: one cooperative launch, FP64 FMA
    updates; 2: the same with DMMA updates (1 and 2 agree with 0 to
    rounding)."""
    a = np.asarray(a, np.float64)
    n = a.shape[0]
    work = np.asfortranarray(a.copy())  # column-major on the device
    buf = work.ravel(order="F").copy()
    ms = C.c_double()
    st = N.lib().gpuklu_dense_lu_nopivot(N.ptr(buf), n, int(variant), C.byref(ms))
    if st != N.OK:
        raise SolverError(st, "dense_lu_nopivot")
    return buf.reshape((n, n), order="F"), ms.value
