"""Batched backward-Euler transient and its checkpointed adjoint on the GPU
(CMOS ring oscillators).

Forward: probe waveforms and losses against the oracle's transient. Backward:
dL/dC against the oracle's discrete adjoint, and against central finite
differences through the GPU forward on 8 sampled instances (relative steps
1e-4 strict, 1e-6 with the measured loss noise). The full 1024-ring,
2000-step case is timed.
"""
import time

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import TranBatch

pytestmark = pytest.mark.gpu

EXACT = dict(wl.TIGHT, abs_tol=1e-15, rel_tol=1e-14)


def _batch(circuits, steps, ckpt=wl.RING_CKPT):
    xs = [wl.ring_initial_state(c) for c in circuits]
    off = np.zeros(len(xs), np.int64)
    off[1:] = np.cumsum([len(x) for x in xs])[:-1]
    return TranBatch(circuits, np.concatenate(xs), off, wl.RING_DT, steps, ckpt,
                     wl.RING_PROBE, wl.RING_TARGET), xs


def test_forward_and_adjoint_match_oracle():
    circuits = [cz.ring_oscillator(s, seed=5, ring_id=i)
                for i, s in enumerate([11, 13, 21, 31, 51, 101])]
    steps = 230  # five segments of 50 (the last one partial)
    tb, xs = _batch(circuits, steps)
    cfg = N.newton_config(**EXACT)
    loss, wave, it, rs = tb.forward(cfg, with_wave=True)
    assert np.all(rs == 0)
    grads, _ = tb.backward(cfg)
    ocfg = {k: EXACT[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin")}
    for i, c in enumerate(circuits):
        r, ito, st = po.tran(c, xs[i], wl.RING_DT, steps, **ocfg)
        assert r == 0
        w_o = st[1:, wl.RING_PROBE]
        assert np.max(np.abs(wave[i] - w_o)) <= 1e-9
        l_o = float(np.sum((w_o - wl.RING_TARGET) ** 2))
        assert abs(loss[i] - l_o) <= 1e-9 * l_o
        g_o = po.tran_adjoint(c, st, wl.RING_DT, wl.RING_PROBE, wl.RING_TARGET)
        caps = c.type == cz.DEV_C
        scale = np.max(np.abs(g_o[caps]))
        assert np.max(np.abs(grads[i][caps] - g_o[caps])) <= 1e-7 * scale, i
        assert np.all(grads[i][~caps] == 0.0)


def test_full_batch_timing_and_finite_differences():
    B = wl.ring_batch(1024)
    steps = wl.RING_STEPS
    tb = TranBatch(B.circuits, B.x_init, B.x_off, wl.RING_DT, steps, wl.RING_CKPT,
                   wl.RING_PROBE, wl.RING_TARGET)
    cfg = N.newton_config(**EXACT)
    tb.forward(cfg)  # warm-up
    t0 = time.perf_counter()
    loss, _, it, rs = tb.forward(cfg)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    grads, it_b = tb.backward(cfg)
    t_bwd = time.perf_counter() - t0
    assert np.all(rs == 0)
    assert np.all(np.isfinite(loss))
    print(f"1024 rings x {steps} BE steps: forward {t_fwd*1e3:.0f} ms "
          f"({int(it.sum())} Newton iterations, {it.sum() / t_fwd / 1e6:.2f} M/s), "
          f"backward {t_bwd*1e3:.0f} ms (ratio {t_bwd / t_fwd:.2f})")
    # finite differences on 8 sampled instances, the largest capacitance gradient of each
    rng = np.random.default_rng(8)
    sample = rng.choice(len(B.circuits), 8, replace=False)
    circ, dev, gsel = [], [], []
    for i in sample:
        c = B.circuits[i]
        caps = np.flatnonzero(c.type == cz.DEV_C)
        d = caps[np.argmax(np.abs(grads[i][caps]))]
        dev.append(d)
        gsel.append(grads[i][d])
        circ.append(c)
    rows = []
    for rel in (1e-4, 1e-6):
        pert = []
        for c, d in zip(circ, dev):
            for sgn in (1.0, -1.0):
                cc = cz.Circuit(c.node_count, c.type, c.nodes, c.p.copy(), c.name)
                cc.p[d, 0] *= 1.0 + sgn * rel
                pert.append(cc)
        # noise probe: each instance unperturbed, twice (the loss is deterministic,
        # so the spread comes from re-running with capacitances 1e-13 apart)
        for c, d in zip(circ, dev):
            for k in (1, 2):
                cc = cz.Circuit(c.node_count, c.type, c.nodes, c.p.copy(), c.name)
                cc.p[d, 0] *= 1.0 + k * 1e-13
                pert.append(cc)
        tp, _ = _batch(pert, steps)
        lp, _, _, rsp = tp.forward(cfg)
        tp.close()
        assert np.all(rsp == 0)
        for k, (c, d, g) in enumerate(zip(circ, dev, gsel)):
            h = rel * c.p[d, 0]
            fd = (lp[2 * k] - lp[2 * k + 1]) / (2 * h)
            noise = abs(lp[2 * len(circ) + 2 * k] - lp[2 * len(circ) + 2 * k + 1])
            tol = 1e-6 * abs(fd) + (0.0 if rel == 1e-4 else 4.0 * noise / (2 * h))
            rows.append((rel, abs(g - fd) / abs(fd)))
            assert abs(g - fd) <= tol, (rel, k, g, fd, noise)
    print("FD worst rel diff: step 1e-4 %.2e, step 1e-6 %.2e" % (
        max(r for s, r in rows if s == 1e-4), max(r for s, r in rows if s == 1e-6)))
