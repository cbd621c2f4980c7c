"""Benchmark: batched circuit-Newton iterations/s on one GB300 (FP64).

Workload (one "step"): the batched Monte-Carlo DC case - 4096 CMOS inverter
chains of 8..256 stages (level-1 card, KP_n=120u, KP_p=40u, VTO ~ N(+-0.45,
0.03), W jittered +-5%), each solved at 61 input voltages 0..1.2 V as an
independent DC operating point: 249,856 Newton solves, every Newton iteration
= device stamp + frozen-pivot refactor + forward/backward solve + update, all
in one kernel launch. Synthetic seeded data (the reference publishes none).

``value``   Newton iterations/s with inputs resident in device memory.
``e2e``     the same through the public API from pinned host buffers: the
            per-step copy of the inputs (input voltages and initial iterates)
            and the read-back of every solution are inside the timed region.
``--impl reference`` times the reference's CPU algorithm (the oracle's C++
restatement of NativeKLU, the exact-pivot variant, with the same Newton
loop) on the host cores over a bounded sample of the same instances.
"""
from __future__ import annotations

import argparse
import json
import re
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "circuit-Newton iters/s, batched vs one-at-a-time on GB300 (FP64, resid<=1e-10)"
UNIT = "iters/s"
WORKLOAD = "batched Monte-Carlo DC: 4096 CMOS inverter chains (8-256 stages) x 61 Vin"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpuklu", choices=["gpuklu", "reference"])
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--nvin", type=int, default=61)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="instances timed on the host cores (0: sized for ~15 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the batch's default schedule instead of tuning it first")
    ap.add_argument("--lane-cap", type=int, default=0,
                    help="fix the lane phase's iteration cap instead of tuning it (profiling)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the single-circuit, adjoint, transient and bordered-block lines")
    ap.add_argument("--only", choices=SECONDARY,
                    help="run just this one of the other workloads (one JSON line, no batch)")
    return ap.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _alg_bytes_per_iter(batch_circuits):
    """Algorithmic bytes of one Newton iteration of one instance, as defined
    for the roofline: stamp 8*nnz_A + 8*n + per-device bytes (diode 104 B,
    level-1 MOSFET 184 B); refactor 8*nnz_A + 12*(nnz_L+nnz_U); solve
    12*(nnz_L+nnz_U) + 24*n; update 32*n. nnz counts from the GPU solver's
    own symbolic analysis (host-side plan, no device work)."""
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import DeviceCircuit
    out = {}
    for c in batch_circuits:
        key = (c.ndev, c.node_count)
        if key in out:
            continue
        dc = DeviceCircuit(c)
        ap, ai = dc.pattern()
        n = dc.n
        dc.close()
        plan = N.Plan(n, ap, ai, N.PIVOT_EXACT)
        nnz_a = len(ai)
        nlu = plan.nnz_l + plan.nnz_u
        nmos = int(np.count_nonzero((c.type == 4) | (c.type == 6)))
        ndio = int(np.count_nonzero(c.type == 3))
        b = (8 * nnz_a + 8 * n + 104 * ndio + 184 * nmos) + (8 * nnz_a + 12 * nlu) + \
            (12 * nlu + 24 * n) + 32 * n
        out[key] = b
    return out


def _residual_sample(B, bt, rs, count=64):
    import scipy.sparse as sp
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver
    _, _, _, xs = bt.results(with_x=True)
    conv = np.flatnonzero(rs == 0)
    idx = conv[:: max(1, len(conv) // count)][:count]
    g = GpuKluSolver(1)
    worst = 0.0
    for i in idx:
        c0 = B.circuits[B.inst_circ[i]]
        c = c0.__class__(**{**c0.__dict__})
        c.p = c0.p.copy()
        c.p[B.inst_dev[i], 0] = B.inst_val[i]
        dc = DeviceCircuit(c)
        x = xs[bt.x_off[i]:bt.x_off[i] + dc.n]
        ax, rhs = dc.stamp(g, x[:c.node_count])
        ap, ai = dc.pattern()
        A = sp.csc_matrix((ax, ai, ap), shape=(dc.n, dc.n))
        r = A @ x - rhs
        den = abs(A).sum(axis=1).max() * np.max(np.abs(x)) + np.max(np.abs(rhs))
        worst = max(worst, float(np.max(np.abs(r)) / den))
        dc.close()
    g.close()
    return worst


PROFILE = os.path.join(ROOT, "profiles", "batch_kernels_inverter_chains.txt")


def _ncu_traffic(kernel, iters):
    """DRAM bytes of one launch of `kernel` that runs `iters` Newton
    iterations, scaled from the committed ncu summary (dram__bytes_read.sum +
    dram__bytes_write.sum of one launch on a 2048-chain batch, per iteration
    that launch ran)."""
    try:
        with open(PROFILE) as f:
            m = re.search(r"^dram_bytes_per_iteration %s:\s*([0-9.eE+-]+)" % re.escape(kernel),
                          f.read(), re.M)
        per = float(m.group(1))
    except (OSError, AttributeError, ValueError):
        return None, "no ncu summary"
    return per * iters, f"{os.path.relpath(PROFILE, ROOT)} ({per:.1f} B per iteration)"


SECONDARY = ("mesh_dc", "dc_adjoint", "transient_adjoint", "adaptive_transient", "bbd",
             "ac_sweep")


def secondary(with_cpu=True, parts=SECONDARY):
    """The other workloads of the path, each timed once warm (CUDA-synchronised
    wall clock around the public call): the 32x32 diode mesh with gmin
    stepping, the 20k-node adjoint, the 1024-ring transient adjoint and the
    64-mesh bordered-block-diagonal DC solve, with the oracle's time for the
    same work on one host core where it is short. `parts` selects among
    them."""
    import torch
    from rustspice_gb300 import workloads as wl

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    out = {}
    ocfg = {k: wl.TIGHT[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps")}
    if "mesh_dc" in parts:
        _mesh_dc(out, with_cpu, timed, ocfg)
    if "dc_adjoint" in parts:
        _dc_adjoint(out, timed, with_cpu, ocfg)
    if "transient_adjoint" in parts:
        _transient_adjoint(out, timed, with_cpu)
    if "adaptive_transient" in parts:
        _adaptive_transient(out, timed, with_cpu)
    if "bbd" in parts:
        _bbd(out, with_cpu, timed, ocfg)
    if "ac_sweep" in parts:
        _ac(out, with_cpu, timed)
    return out


def _ac(out, with_cpu, timed):
    """AC sweep of a 100-section RC ladder (n = 103), 500 points per decade
    from 1 Hz to 1 GHz; the oracle's dense complex LU timed on 64 of the
    points on one host core and scaled."""
    from oracle import pyoracle as po
    from rustspice_gb300 import netlist as nl
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, ac_sweep, frequency_sweep
    rng = np.random.default_rng(3)
    lines = ["V1 n0 0 DC 0 AC 1 30"]
    for k in range(100):
        lines.append(f"R{k} n{k} n{k + 1} {rng.uniform(100, 1000):.6g}")
        lines.append(f"C{k} n{k + 1} 0 {rng.uniform(1e-12, 1e-9):.6g}")
    c = nl.compile_deck("\n".join(lines) + "\n").circuit
    f = frequency_sweep("dec", 500, 1.0, 1e9)
    g = GpuKluSolver(1)
    dc = DeviceCircuit(c)
    x0 = np.zeros(c.n)
    ac_sweep(g, dc, x0, f)
    _, t = timed(lambda: ac_sweep(g, dc, x0, f))
    e = {"workload": "100-section RC ladder, 4501 frequencies (dec 500, 1 Hz - 1 GHz)",
         "n": c.n, "frequencies": len(f), "gpu_ms": t * 1e3}
    if with_cpu:
        sample = f[::max(1, len(f) // 64)][:64]
        t0 = time.perf_counter()
        po.ac_sweep(c, x0, sample)
        e["oracle_ms_1core_est"] = (time.perf_counter() - t0) / len(sample) * len(f) * 1e3
    out["ac_sweep"] = e


def _mesh_dc(out, with_cpu, timed, ocfg):
    """Diode mesh, gmin stepping (one circuit, device-resident Newton)."""
    from oracle import pyoracle as po
    from rustspice_gb300 import circuits as cz
    from rustspice_gb300 import native as N
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, newton_dc
    c = cz.mesh_dc()
    cfg = N.newton_config(**dict(wl.TIGHT, gmin_steps=10))
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    dc = DeviceCircuit(c)
    newton_dc(g, dc, cfg)
    r, t = timed(lambda: newton_dc(g, dc, cfg))
    e = {"workload": "32x32 diode mesh, gmin stepping (10 steps)", "n": dc.n,
         "newton_iterations": r.iterations_total, "gpu_ms": t * 1e3,
         "pivot_passes": g.pivot_passes()}
    if with_cpu:
        t0 = time.perf_counter()
        ro = po.dc_op(c, "nativeklu_exact", **dict(ocfg, gmin_steps=10))
        e["oracle_ms_1core"] = (time.perf_counter() - t0) * 1e3
    out["mesh_dc"] = e


def _dc_adjoint(out, timed, with_cpu, ocfg):
    """DC adjoint of the 20k-node mesh with inverters; the oracle's forward
    (the reference's Newton loop with NativeKLU) on one host core beside it."""
    from rustspice_gb300 import circuits as cz
    from rustspice_gb300 import native as N
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, dc_backward, dc_forward
    c = cz.mesh_with_inverters(120, 1000)
    outs = cz.output_nodes(c, 256)
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    dc = DeviceCircuit(c)
    cfg = N.newton_config(**wl.TIGHT)
    f = dc_forward(g, dc, cfg)
    f, t_f = timed(lambda: dc_forward(g, dc, cfg))
    dl = np.zeros(dc.n)
    dl[outs] = 2.0 * (f.x[outs] - 0.6)
    dc_backward(g, dc, f.x, dl)
    _, t_b = timed(lambda: dc_backward(g, dc, f.x, dl))
    out["dc_adjoint"] = {"workload": "120x120 mesh + 1000 inverters, loss on 256 nodes",
                         "n": dc.n, "forward_ms": t_f * 1e3, "newton_iterations": f.iterations,
                         "pivot_passes": g.pivot_passes(),
                         "backward_ms": t_b * 1e3, "backward_over_forward": t_b / t_f}
    if with_cpu:
        from oracle import pyoracle as po
        t0 = time.perf_counter()
        po.dc_op(c, "nativeklu_exact", **ocfg)
        out["dc_adjoint"]["oracle_forward_ms_1core"] = (time.perf_counter() - t0) * 1e3


def _transient_adjoint(out, timed, with_cpu):
    """Transient adjoint of 1024 rings; beside it the oracle's backward-Euler
    forward run (the reference's transient Newton loop with NativeKLU) on one
    host core, timed on 16 rings and scaled to the 1024."""
    from rustspice_gb300 import native as N
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import TranBatch
    B = wl.ring_batch(1024)
    tb = TranBatch(B.circuits, B.x_init, B.x_off, wl.RING_DT, wl.RING_STEPS, wl.RING_CKPT,
                   wl.RING_PROBE, wl.RING_TARGET)
    cfg = N.newton_config(**wl.TIGHT)
    tb.forward(cfg)
    (loss, _, it, rs), t_f = timed(lambda: tb.forward(cfg))
    _, t_b = timed(lambda: tb.backward(cfg))
    out["transient_adjoint"] = {
        "workload": "1024 CMOS rings (11-101 stages) x 2000 BE steps of 1 ps, checkpoint 50",
        "forward_ms": t_f * 1e3, "backward_ms": t_b * 1e3, "backward_over_forward": t_b / t_f,
        "newton_iterations_forward": int(it.sum()), "converged_fraction": float(np.mean(rs == 0))}
    tb.close()
    if with_cpu:
        from oracle import pyoracle as po
        sample = np.random.default_rng(2).choice(len(B.circuits), 16, replace=False)
        t0 = time.perf_counter()
        for i in sample:
            c = B.circuits[i]
            po.tran(c, B.x_init[B.x_off[i]:B.x_off[i] + c.node_count], wl.RING_DT,
                    wl.RING_STEPS)
        per = (time.perf_counter() - t0) / len(sample)
        out["transient_adjoint"]["oracle_forward_ms_1core_est"] = per * len(B.circuits) * 1e3
        out["transient_adjoint"]["oracle_sample"] = "16 rings (seed 2), scaled to 1024"


def _adaptive_transient(out, timed, with_cpu):
    """The engine's adaptive transient (BE + trapezoidal solves, Milne's LTE,
    PI control, breakpoints) on 1024 inverter chains of 8-64 stages driven by
    a pulse train, 0 to 4 ns, the engine's default LTE tolerances; the
    oracle's restatement on one host core timed on 16 chains and scaled."""
    from rustspice_gb300 import native as N
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import ATranBatch
    B = wl.adaptive_batch(1024)
    ab = ATranBatch(B.circuits, B.waves, B.x_ic, B.probe)
    cfg = N.newton_config(max_iters=100, abs_tol=1e-9, rel_tol=1e-6, gmin=1e-12)
    kw = dict(lte_abs=1e-6, lte_rel=1e-3, be_sign=1.0, max_points=1)
    ab.run(cfg, wl.ATRAN_TSTEP, wl.ATRAN_TSTOP, **kw)
    r, t = timed(lambda: ab.run(cfg, wl.ATRAN_TSTEP, wl.ATRAN_TSTOP, **kw))
    its = int(r.iterations.sum())
    out["adaptive_transient"] = {
        "workload": "1024 CMOS inverter chains (8-64 stages) x pulse train, 0-4 ns, "
                    "tstep 10 ps, LTE vntol 1e-6 / reltol 1e-3, physical BE sign",
        "gpu_ms": t * 1e3, "completed_fraction": float(np.mean(r.status == 0)),
        "accepted_steps": int(r.accepted.sum()), "rejected_steps": int(r.rejected.sum()),
        "newton_iterations": its, "newton_iters_per_s": its / t}
    ab.close()
    if with_cpu:
        from oracle import pyoracle as po
        sample = np.random.default_rng(2).choice(len(B.circuits), 16, replace=False)
        t0 = time.perf_counter()
        for i in sample:
            po.tran_adaptive(B.circuits[i], B.waves[i], wl.ATRAN_TSTEP, wl.ATRAN_TSTOP,
                             x_ic=B.x_ic[i], max_iters=100, abs_tol=1e-9, rel_tol=1e-6,
                             lte_abs=1e-6, lte_rel=1e-3, cap=1)
        per = (time.perf_counter() - t0) / len(sample)
        out["adaptive_transient"]["oracle_ms_1core_est"] = per * len(B.circuits) * 1e3
        out["adaptive_transient"]["oracle_sample"] = "16 chains (seed 2), scaled to 1024"


def _bbd(out, with_cpu, timed, ocfg):
    """Bordered block diagonal DC solve."""
    from oracle import pyoracle as po
    from rustspice_gb300 import circuits as cz
    from rustspice_gb300 import native as N
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import BbdSolver, DeviceCircuit
    c, asg, nb = cz.bordered_meshes()
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    bb = BbdSolver(ap, ai, asg, nb)
    x0 = wl.bordered_nodeset(c)
    cfg = N.newton_config(**wl.TIGHT)
    bb.newton_dc(dc, cfg, x0=x0)
    r, t = timed(lambda: bb.newton_dc(dc, cfg, x0=x0))
    info = bb.info()
    e = {"workload": "64 meshes (side 30-50) + 1024 border nodes, known partition",
         "n": dc.n, "border": info["border_size"], "newton_iterations": r.iterations,
         "gpu_ms_per_iteration": t * 1e3 / max(r.iterations, 1)}
    if with_cpu:
        ts = []
        for k in (1, 3):  # the difference removes the analysis
            t0 = time.perf_counter()
            po.dc_op_bbd(c, asg, nb, x0=x0, **dict(ocfg, max_iters=k))
            ts.append(time.perf_counter() - t0)
        e["oracle_ms_per_iteration_1core"] = (ts[1] - ts[0]) * 1e3 / 2
    e["schur_lu"] = _schur_lu(info["border_size"])
    out["bbd"] = e


def _schur_lu(bs):
    """The dense LU of a border-sized Schur complement on its own, each
    variant timed with CUDA events (best of three, S resident in L2 as in the
    BBD iteration), against the measured FP64 FMA and DMMA peaks."""
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import dense_lu_nopivot
    rng = np.random.default_rng(5)
    a = rng.uniform(-1.0, 1.0, (bs, bs))
    a[np.arange(bs), np.arange(bs)] += bs  # no pivoting needed
    flops = 2.0 * bs ** 3 / 3.0 - bs ** 2 / 2.0 - bs / 6.0
    dfma = float(N.lib().gpuklu_fp64_peak_tflops())
    dmma = float(N.lib().gpuklu_fp64_mma_peak_tflops())
    r = {"n": bs, "flops": flops, "dfma_peak_tflops": dfma, "dmma_peak_tflops": dmma}
    for name, v in (("panels", 0), ("coop_fma", 1), ("coop_dmma", 2)):
        dense_lu_nopivot(a, v)
        ms = min(dense_lu_nopivot(a, v)[1] for _ in range(3))
        tf = flops / (ms * 1e-3) / 1e12
        r[name] = {"ms": ms, "tflops": tf, "frac_of_dfma_peak": tf / dfma if dfma else None,
                   "frac_of_dmma_peak": tf / dmma if dmma else None}
    return r


def run_gpu(a):
    import torch
    from rustspice_gb300 import native as N
    from rustspice_gb300 import ranks
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import Batch, DeviceCircuit, GpuKluSolver, newton_dc

    ws, rank, lrank = _dist()
    torch.cuda.set_device(lrank)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", lrank)
    # every rank solves its own seeded batch of the same size (weak scaling)
    B = wl.inverter_batch(a.chains, a.nvin, seed=ranks.shard_seed(rank))
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    cfg = N.newton_config(**wl.TIGHT)
    stream = torch.cuda.ExternalStream(bt.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def step():
        flush.fill_(1)
        bt.run(cfg)

    with torch.cuda.stream(stream):
        # the project's autotuner picks the lane-phase cap and the
        # continuation's tiles per program from timed runs of this batch
        if a.lane_cap > 0:
            bt.set_schedule(a.lane_cap, 2)
            tune = {"lane_cap": a.lane_cap, "cont_tiles": 2, "runs": 0, "autotuned": False}
        elif a.no_autotune:
            tune = {"lane_cap": 6, "cont_tiles": 2, "runs": 0, "autotuned": False}
        else:
            tune = dict(bt.autotune(cfg), autotuned=True)
        for _ in range(a.warmup):
            step()
        stream.synchronize()
        it, itt, rs, _ = bt.results(with_x=False)
        iters_per_step = int(itt.sum())
        # device-resident timing
        clk = ClockSampler(lrank)
        clk.start()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        evs = []
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            flush.fill_(1)
            e0.record(stream)
            bt.run(cfg)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clocks = clk.stop()
        kern_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
        ms_step = ranks.max_over_ranks(float(np.mean(kern_ms)), dev)
        iters_all = int(ranks.sum_over_ranks(iters_per_step, dev))
        value = iters_all / (ms_step * 1e-3)

        # end-to-end: pinned host inputs -> device, run, every solution -> host
        val_h = torch.from_numpy(np.ascontiguousarray(B.inst_val)).pin_memory()
        x0_h = torch.from_numpy(np.ascontiguousarray(B.x0)).pin_memory()
        xout_h = torch.empty(bt.x_len, dtype=torch.float64).pin_memory()
        e2e_ms = []
        for _ in range(max(2, a.steps)):
            flush.fill_(1)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            bt.update_inputs(val_h.numpy(), x0_h.numpy())
            bt.run(cfg)
            it2, itt2, rs2, x2 = bt.results(with_x=True, x_out=xout_h.numpy())
            e2e_ms.append((time.perf_counter() - t1) * 1e3)
        e2e_step = ranks.max_over_ranks(float(np.median(e2e_ms)), dev)

        # per-kernel device time (CUDA events the library records on its
        # launching streams around the lane kernel and the warp kernels)
        phases = []
        for _ in range(max(3, a.steps)):
            step()
            phases.append(bt.phase_ms())
        h2d = val_h.numel() * 8 + x0_h.numel() * 8
        d2h = len(x2) * 8 + 3 * 8 * len(it2)
    conv = float(np.mean(rs == 0))
    it_final = it

    # Newton residual F(x) = A(x) x - b(x) of a sample of converged solutions,
    # stamped at x by the device and evaluated on the host, normwise relative
    resid = _residual_sample(B, bt, rs)

    # roofline of the dominant kernel. Both kernels keep an instance's
    # values on chip or in L2 and run FP64 dependency chains: the bound is
    # the FP64 rate (the DFMA peak measured in this run), with the HBM view
    # beside it. Per kernel: the iterations an instance runs in the lane
    # kernel (min(total, cap)) or after it, their algorithmic bytes and FP64
    # operations, over the kernel's own event-timed duration.
    hbm_peak, peak_src = _measured_peaks()
    per_key = _alg_bytes_per_iter(B.circuits)
    keys = [(B.circuits[c].ndev, B.circuits[c].node_count) for c in B.inst_circ]
    b_inst = np.array([per_key[k] for k in keys], np.float64)
    alg_bytes = float(np.sum(b_inst * itt))
    flops, _ = bt.work()
    f_inst = flops.astype(np.float64)
    fp64 = float(np.sum(f_inst * itt))
    fp64_tflops = fp64 / (ms_step * 1e-3) / 1e12
    fp64_peak = float(N.lib().gpuklu_fp64_peak_tflops())
    cap = phases[0]["lane_cap"]
    lane_it = np.minimum(itt, cap) if cap > 0 else np.zeros_like(itt)
    second = "k_batch_cont" if bt.info()["cont_kernel"] else "k_batch_newton"
    kern = {}
    phases_run = ([("k_batch_lanes", "lanes_ms", lane_it)] if cap > 0 else []) + \
        [(second, "warps_ms", itt - lane_it)]
    for name, ms_k, its in phases_run:
        t_ms = float(np.median([p[ms_k] for p in phases]))
        kb = float(np.sum(b_inst * its))
        kf = float(np.sum(f_inst * its))
        tr, tr_src = _ncu_traffic(name, int(its.sum()))
        kern[name] = {"ms_per_launch": t_ms, "newton_iterations": int(its.sum()),
                      "algorithmic_bytes_per_launch": kb,
                      "achieved_gbs": kb / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None,
                      "fp64_ops_per_launch": kf,
                      "achieved_tflops": kf / (t_ms * 1e-3) / 1e12 if t_ms > 0 else None,
                      "dram_bytes_per_launch": tr, "traffic_source": tr_src}
    dom = max(kern, key=lambda k: kern[k]["ms_per_launch"])
    achieved = kern[dom]["achieved_tflops"]
    traffic, traffic_src = kern[dom]["dram_bytes_per_launch"], kern[dom]["traffic_source"]

    # converged-only rates, and the time of the instances that run to the
    # iteration cap: the same step with only the converged instances, timed
    # the same way (the difference is what the capped ones cost)
    conv_mask = rs == 0
    conv_iters = int(itt[conv_mask].sum())
    capped = _converged_only_step(B, conv_mask, cfg, flush, dev, a.steps, tune)
    # one-at-a-time GpuKluSolver: the engine's DC sweep of a chain over the
    # 61 input points, one handle per chain, the pattern analysed on the
    # sweep's first point and reused for the others (engine.rs:684-820)
    one = _one_at_a_time(B, cfg, torch)
    one_at_a_time = one["value"]

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded circuits; the reference publishes no dataset)",
        "config": {"workload": WORKLOAD, "chains": a.chains, "vin_points": a.nvin,
                   "instances": int(B.ninst), "newton_iterations_per_step": iters_per_step,
                   "converged_fraction": conv, "max_final_residual": resid,
                   "newton": dict(wl.TIGHT),
                   "mos_model": "level-1, consistent linearisation (MC)",
                   "pivot_mode": "exact pattern (nativeklu_exact)",
                   "initial_iterate": "logic-level nodeset",
                   "l2": "256 MB buffer written before every timed step; inputs 270 MB > L2",
                   "parallelism": f"replicas x{ws}",
                   "schedule": tune},
        "e2e": {"value": iters_all / (e2e_step * 1e-3), "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_step},
        "gpu_launches": a.steps * bt.info()["launches"],
        "converged_iters_per_s": conv_iters / (ms_step * 1e-3),
        "converged_solves_per_s": int(conv_mask.sum()) / (ms_step * 1e-3),
        "capped_instances": capped,
        "one_at_a_time": dict(one, batched_over_one_at_a_time=value / one_at_a_time),
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak else None,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": "measured DFMA microbenchmark in this run "
                                    "(gpuklu_fp64_peak_tflops; MEASURED_PEAKS.json has no FP64)",
                     "hbm_view": {"achieved": kern[dom]["achieved_gbs"], "peak": hbm_peak,
                                  "unit": "GB/s",
                                  "frac": kern[dom]["achieved_gbs"] / hbm_peak,
                                  "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
                     "algorithmic_bytes_per_step": alg_bytes, "fp64_ops_per_step": fp64,
                     "kernels": kern},
        "roofline_fp64": {"achieved": fp64_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                          "frac": fp64_tflops / fp64_peak if fp64_peak else None,
                          "peak_source": "measured DFMA microbenchmark (gpuklu_fp64_peak_tflops)",
                          "fp64_ops_per_step": fp64},
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    if not a.no_secondary:
        line["reference_level1"] = _reference_model_line(a, cfg, flush, dev, rank)
    if not a.no_cpu_baseline and rank == 0:
        line["cpu_baseline"] = cpu_baseline(B, a, cfg_dict=wl.TIGHT)
    if not a.no_secondary and rank == 0:
        line["secondary"] = secondary(with_cpu=not a.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def _timed_runs(bt, cfg, flush, steps):
    """Mean device time [ms] of `steps` runs of a batch, each behind an L2
    flush, with CUDA events on the batch's stream."""
    import torch
    stream = torch.cuda.ExternalStream(bt.stream(), device=flush.device)
    with torch.cuda.stream(stream):
        for _ in range(3):
            flush.fill_(1)
            bt.run(cfg)
        evs = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            flush.fill_(1)
            e0.record(stream)
            bt.run(cfg)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
    return float(np.mean([e0.elapsed_time(e1) for e0, e1 in evs]))


def _converged_only_step(B, conv, cfg, flush, dev, steps, sched=None):
    """The batch restricted to the instances that converged, timed like the
    full step (with the same schedule): what the instances that run to the
    iteration cap cost is the difference."""
    from rustspice_gb300.solver import Batch
    idx = np.flatnonzero(conv)
    x0 = np.concatenate([B.x0[B.x0_off[i]:B.x0_off[i] + B.circuits[B.inst_circ[i]].node_count]
                         for i in idx])
    off = np.concatenate([[0], np.cumsum([B.circuits[B.inst_circ[i]].node_count
                                          for i in idx])[:-1]]).astype(np.int64)
    bt = Batch(B.circuits, B.inst_circ[idx], B.inst_dev[idx], B.inst_val[idx], x0, off)
    if sched is not None:
        bt.set_schedule(sched["lane_cap"], sched["cont_tiles"])
    ms = _timed_runs(bt, cfg, flush, max(3, steps // 2))
    _, itt, rs, _ = bt.results(with_x=False)
    ph = bt.phase_ms()
    bt.close()
    return {"instances": int(B.ninst - len(idx)), "converged_only_ms_per_step": ms,
            "converged_only_iterations": int(itt.sum()),
            "converged_only_kernel_ms": {"k_batch_lanes": ph["lanes_ms"],
                                         "continuation": ph["warps_ms"]},
            "how": "the same batch with only the converged instances, timed the same way; "
                   "the capped instances cost the difference to ms_per_step"}


def _one_at_a_time(B, cfg, torch, chains=4):
    """The plain GpuKluSolver, one operating point at a time, as the
    reference's DC sweep runs it (gpuklu_dc_sweep, engine.rs:684-820): per
    sampled chain one handle, the input source stepped through the sweep's
    points in order, one Newton solve per point on the device from the
    point's nodeset, the pattern and pivots of the first point kept. The
    first point (pattern analysis and pivot pass) is timed apart, from a
    one-point sweep, and taken out of the value."""
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, dc_sweep
    rng = np.random.default_rng(0)
    nvin = int(np.sum(B.inst_circ == 0))
    picks = rng.choice(len(B.circuits), chains, replace=False)
    t_all = t_first = 0.0
    it_all = it_first = 0
    for ci in picks:
        c = B.circuits[ci]
        g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
        dc = DeviceCircuit(c)
        idx = np.arange(ci * nvin, (ci + 1) * nvin)
        x0 = np.stack([B.x0[B.x0_off[i]:B.x0_off[i] + c.node_count] for i in idx])
        vals = B.inst_val[idx]
        for npts in (1, nvin):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            r = dc_sweep(g, dc, cfg, 1, vals[:npts], x0=x0[:npts], stop_on_failure=False)
            dt = time.perf_counter() - t1
            if npts == 1:
                t_first += dt
                it_first += int(r.iterations_total.sum())
            else:
                t_all += dt
                it_all += int(r.iterations_total.sum())
        dc.close()
        g.close()
    t_rest, it_rest = t_all - t_first, it_all - it_first
    return {"value": it_rest / t_rest, "unit": UNIT,
            "first_point_iters_per_s": it_first / t_first,
            "first_point_ms": t_first * 1e3 / chains,
            "how": f"gpuklu_dc_sweep over the {nvin}-point input sweep of {chains} sampled "
                   "chains (one handle per sweep, pivots of the first point kept); the first "
                   "point's time, from a one-point sweep, is taken out of the value"}


def _reference_model_line(a, cfg, flush, dev, rank):
    """The same workload with the reference's own level-1 evaluator (M),
    from the same nodeset: its converged fraction and rates."""
    from rustspice_gb300 import ranks
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import Batch
    B = wl.inverter_batch(a.chains, a.nvin, seed=ranks.shard_seed(rank),
                          mos_model="reference")
    bt = Batch(B.circuits, B.inst_circ, B.inst_dev, B.inst_val, B.x0, B.x0_off)
    ms = _timed_runs(bt, cfg, flush, max(3, a.steps // 2))
    _, itt, rs, _ = bt.results(with_x=False)
    bt.close()
    conv = rs == 0
    return {"mos_model": "level-1 as the reference evaluates it (M)",
            "ms_per_step": ms, "value": float(itt.sum()) / (ms * 1e-3), "unit": UNIT,
            "newton_iterations_per_step": int(itt.sum()),
            "converged_fraction": float(np.mean(conv)),
            "converged_iters_per_s": float(itt[conv].sum()) / (ms * 1e-3),
            "converged_solves_per_s": int(conv.sum()) / (ms * 1e-3)}


def _cpu_sample(B, count, seed=1):
    """Whole chains sampled at random, each with all its input points (the
    points of one chain's sweep share one solver on the CPU as on the
    device), about `count` instances in all."""
    rng = np.random.default_rng(seed)
    nchains = len(B.circuits)
    per = max(1, B.ninst // nchains)
    k = max(1, min(nchains, -(-count // per)))
    chains = np.sort(rng.choice(nchains, k, replace=False))
    return np.flatnonzero(np.isin(B.inst_circ, chains))


def _cpu_run(B, idx, threads, cfg_dict):
    from oracle import pyoracle as po
    circ_ids = np.unique(B.inst_circ[idx])
    remap = {c: k for k, c in enumerate(circ_ids)}
    circuits = [B.circuits[c] for c in circ_ids]
    order = np.argsort(B.inst_circ[idx], kind="stable")
    idx = idx[order]
    ic = np.array([remap[c] for c in B.inst_circ[idx]], np.int64)
    x0 = np.concatenate([B.x0[B.x0_off[i]:B.x0_off[i] + B.circuits[B.inst_circ[i]].node_count]
                         for i in idx])
    off = np.concatenate([[0], np.cumsum([B.circuits[B.inst_circ[i]].node_count
                                          for i in idx])[:-1]]).astype(np.int64)
    kw = {k: cfg_dict[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps")}
    t0 = time.perf_counter()
    it, rs, _ = po.dc_batch(circuits, ic, B.inst_dev[idx], B.inst_val[idx], "nativeklu_exact",
                            nthreads=threads, x0=x0, x0_off=off, **kw)
    dt = time.perf_counter() - t0
    _cpu_run.last_converged_iters = int(it[rs == 0].sum())
    _cpu_run.last_converged = int(np.sum(rs == 0))
    return int(it.sum()), dt, float(np.mean(rs == 0))


def cpu_baseline(B, a, cfg_dict):
    threads = os.cpu_count() or 1
    count = a.cpu_sample or 4000
    idx = _cpu_sample(B, count)
    iters, dt, conv = _cpu_run(B, idx, threads, cfg_dict)
    if not a.cpu_sample and dt < 10.0:  # grow the sample towards ~15 s of CPU work
        count = int(min(B.ninst, count * max(1.0, 15.0 / max(dt, 1e-3))))
        idx = _cpu_sample(B, count)
        iters, dt, conv = _cpu_run(B, idx, threads, cfg_dict)
    return {"value": iters / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "converged_iters_per_s": _cpu_run.last_converged_iters / dt,
            "converged_solves_per_s": _cpu_run.last_converged / dt,
            "sample": f"{len(idx)} of {B.ninst} instances (whole chains at random, seed 1), "
                      f"{iters} Newton iterations in {dt:.2f} s, converged {conv:.4f}; "
                      "oracle C++ NativeKLU (exact pivots) + reference Newton loop"}


def run_reference(a):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from rustspice_gb300 import workloads as wl
    B = wl.inverter_batch(a.chains, a.nvin, seed=3)
    threads = os.cpu_count() or 1
    count = a.cpu_sample or 3000
    idx = _cpu_sample(B, count)
    for _ in range(max(0, min(a.warmup, 1))):
        _cpu_run(B, idx[: max(1, len(idx) // 10)], threads, wl.TIGHT)
    per = []
    tot_it = 0
    for _ in range(a.steps):
        iters, dt, conv = _cpu_run(B, idx, threads, wl.TIGHT)
        per.append(dt)
        tot_it = iters
    ms = float(np.mean(per)) * 1e3
    value = tot_it / (ms * 1e-3)
    conv_rates = {"converged_iters_per_s": _cpu_run.last_converged_iters / (ms * 1e-3),
                  "converged_solves_per_s": _cpu_run.last_converged / (ms * 1e-3),
                  "converged_fraction": conv}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded circuits)",
        "config": {"workload": WORKLOAD, "chains": a.chains, "vin_points": a.nvin,
                   "step": f"bounded sample of {len(idx)} instances per step"},
        "impl": "reference",
        **conv_rates,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(idx)} of {B.ninst} instances per step (whole chains "
                                   "at random, seed 1); "
                                   "oracle C++ restatement of NativeKLU (exact pivots) and the "
                                   "reference Newton loop"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    args = _args()
    if args.only:
        print(json.dumps({"only": args.only,
                          "secondary": secondary(with_cpu=not args.no_cpu_baseline,
                                                 parts=(args.only,))}))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)
