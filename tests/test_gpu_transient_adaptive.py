"""The adaptive transient on the device (gpuklu_atran_*) against the
oracle's restatement of the reference's engine loop (oracle/transient.cpp)
on the same circuits: step counts, accepted times, waveforms, status; the
analytic RC response; the reference's backward-Euler sign reproduced as the
reference behaves (every step with a charged capacitor rejected)."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import waveforms as wf
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import ATranBatch, SolverError

pytestmark = pytest.mark.gpu

CFG = dict(max_iters=100, abs_tol=1e-9, rel_tol=1e-6, gmin=1e-12)
LTE = dict(lte_abs=1e-6, lte_rel=1e-3)  # the engine's defaults (vntol, reltol)


def _rc(vsrc, r=1000.0, c=1e-9):
    dev = cz._Dev()
    dev.add(cz.DEV_V, (1, 0), (vsrc,))
    dev.add(cz.DEV_R, (1, 2), (r,))
    dev.add(cz.DEV_C, (2, 0), (c,))
    return dev.build(3)


def _oracle(c, w, tstep, tstop, be_sign, x_ic=None, lte=None):
    return po.tran_adaptive(c, w, tstep, tstop, be_sign=be_sign, x_ic=x_ic, **CFG, **(lte or {}))


def _compare(dev, i, orc, probe, wave_tol, exact=False):
    """Device run i against the oracle's run. The device's solves round
    differently (FMA and a one-step reciprocal in the batched factor, CUDA's
    exp): Milne's estimate subtracts two nearly equal solutions, so those
    1e-14 differences become ~1e-9 in the error ratio and the PI controller
    carries them into the step sizes - the two time grids drift apart by up
    to ~1e-6 of tstop over thousands of steps. So: the same status, the same
    step counts (exact for short runs, within 1 % otherwise), both ending at
    tstop (or where the run failed), and the probe waveform within wave_tol of the oracle's (linearly
    interpolated at the device's times)."""
    assert dev.status[i] == orc["status"], (i, dev.status[i], orc["status"])
    acc, rej = int(dev.accepted[i]), int(dev.rejected[i])
    if exact:
        assert (acc, rej) == (orc["accepted"], orc["rejected"]), (i, acc, rej, orc)
    else:
        assert abs(acc - orc["accepted"]) <= max(2, 0.01 * orc["accepted"]), (i, acc, orc)
        assert abs(rej - orc["rejected"]) <= max(3, 0.05 * orc["rejected"]), (i, rej, orc)
    ts, td = orc["times"], dev.times[i]
    end_tol = 1e-15 if orc["status"] == 0 else 1e-9  # a failed run stops where it failed
    assert td[0] == ts[0] and abs(td[-1] - ts[-1]) <= end_tol * abs(ts[-1]) + 1e-300
    assert np.all(np.diff(td) > 0)
    v = orc["solutions"][:, probe]
    scale = max(1.0, np.max(np.abs(v)))
    assert np.max(np.abs(dev.probe[i] - np.interp(td, ts, v))) <= wave_tol * scale


def test_rc_pulse_matches_the_oracle_and_the_analytic_response():
    c = _rc(0.0)
    w = {0: wf.pulse(0.0, 1.0, 1e-6, 1e-9, 1e-9, 5e-6, 0.0)}
    b = ATranBatch([c], [w], probe=2)
    r = b.run(N.newton_config(**CFG), 1e-7, 10e-6, be_sign=1.0, max_points=20000)
    o = _oracle(c, w, 1e-7, 10e-6, 1.0)
    assert r.status[0] == 0 and r.npoints[0] == r.accepted[0] + 1
    _compare(r, 0, o, 2, 2e-5)
    ts, v = r.times[0], r.probe[0]
    m = (ts > 1.1e-6) & (ts < 6e-6)
    assert np.max(np.abs(v[m] - (1.0 - np.exp(-(ts[m] - 1e-6 - 0.5e-9) / 1e-6)))) < 5e-4
    b.close()


def test_reference_be_sign_as_the_reference_behaves():
    cp = _rc(0.0)
    w = {0: wf.pulse(0.0, 1.0, 1e-6, 1e-9, 1e-9, 5e-6, 0.0)}
    cd = _rc(1.0)
    b = ATranBatch([cp, cd], [w, {}], probe=2)
    r = b.run(N.newton_config(**CFG), 1e-7, 10e-6, be_sign=-1.0)
    for i, (c, ww) in enumerate(((cp, w), (cd, {}))):
        o = _oracle(c, ww, 1e-7, 10e-6, -1.0)
        assert o["status"] == 1
        _compare(r, i, o, 2, 1e-9, exact=True)
    assert r.accepted[1] == 0 and r.rejected[1] == 10
    b.close()


def _mixed():
    """Circuits of different sizes and sources: RC ladders driven by PWL,
    SIN and EXP sources, a diode clipper behind a pulse, and short CMOS
    inverter chains (the consistent level-1 model, 20 fF per stage) driven
    by pulses of different periods."""
    out = []
    for k, w in enumerate([wf.pwl([(0, 0), (2e-7, 1.0), (6e-7, 1.0), (8e-7, 0.2)]),
                           wf.sin(0.5, 0.4, 4e6, 1e-7, 1e5),
                           wf.exp(0.0, 1.0, 1e-7, 1e-7, 5e-7, 2e-7)]):
        dev = cz._Dev()
        dev.add(cz.DEV_V, (1, 0), (0.0,))
        nodes = 4 + k
        for j in range(1, nodes):
            dev.add(cz.DEV_R, (j, j + 1), (200.0 * (j + 1),))
            dev.add(cz.DEV_C, (j + 1, 0), (1e-11 * (j + 1),))
        out.append((dev.build(nodes + 1), {0: w}, nodes, None))
    dev = cz._Dev()
    dev.add(cz.DEV_V, (1, 0), (0.0,))
    dev.add(cz.DEV_R, (1, 2), (500.0,))
    dev.add(cz.DEV_D, (2, 0), (1e-14, 1.0))
    dev.add(cz.DEV_C, (2, 0), (5e-12,))
    out.append((dev.build(3), {0: wf.pulse(-1.0, 2.0, 1e-7, 2e-8, 2e-8, 3e-7, 6e-7)}, 2, None))
    for stages, per in ((3, 4e-7), (5, 6e-7)):
        c = cz.inverter_chain(stages, 0.0)  # device 1 is the input source
        out.append((c, {1: wf.pulse(0.0, 1.2, 5e-8, 1e-8, 1e-8, per / 2, per)},
                    c.node_count - 1, wl.chain_nodeset(stages, 0.0)))
    return out


def test_mixed_batch_matches_the_oracle():
    cases = _mixed()
    b = ATranBatch([c for c, _, _, _ in cases], [w for _, w, _, _ in cases],
                   x_ic=[x for _, _, _, x in cases], probe=[p for _, _, p, _ in cases])
    r = b.run(N.newton_config(**CFG), 1e-8, 1.5e-6, be_sign=1.0, max_points=20000, **LTE)
    for i, (c, w, p, x) in enumerate(cases):
        o = _oracle(c, w, 1e-8, 1.5e-6, 1.0, x_ic=x, lte=LTE)
        assert o["status"] == 0, i
        _compare(r, i, o, p, 2e-3)
        n = c.n
        assert np.max(np.abs(r.x[i][:c.node_count] - o["solutions"][-1][:c.node_count])) <= \
            2e-3 * max(1.0, np.max(np.abs(o["solutions"][-1])))
    b.close()


def test_points_beyond_the_buffer_and_bad_arguments():
    c = _rc(0.0)
    w = {0: wf.pulse(0.0, 1.0, 1e-6, 1e-9, 1e-9, 5e-6, 0.0)}
    b = ATranBatch([c], [w], probe=2)
    full = b.run(N.newton_config(**CFG), 1e-7, 10e-6, max_points=20000)
    part = b.run(N.newton_config(**CFG), 1e-7, 10e-6, max_points=16)
    assert part.npoints[0] == full.npoints[0] and len(part.times[0]) == 16
    assert np.array_equal(part.times[0], full.times[0][:16])
    few = b.run(N.newton_config(**CFG), 1e-7, 10e-6, max_steps=40)
    assert few.status[0] == 3 and few.accepted[0] + few.rejected[0] <= 40
    with pytest.raises(SolverError) as e:
        b.run(N.newton_config(**CFG), 0.0, 10e-6)
    assert e.value.status == N.INVALID_MATRIX
    b.close()
