"""The adaptive transient's pieces on the CPU: the oracle's restatement of
the reference's waveforms, breakpoints, Milne's LTE estimate and PI step
controller, pinned by the reference's own unit tests
(crates/sim-core/tests/adaptive_timestep_tests.rs:33-410, analysis.rs:
760-840), and its transient loop on RC circuits against the analytic
response. The device kernel is checked against this oracle in
test_gpu_transient_adaptive.py."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import waveforms as wf


def test_pulse_full_cycle():  # adaptive_timestep_tests.rs:33-65
    p = wf.pulse(0.0, 3.3, 1e-9, 100e-12, 100e-12, 5e-9, 10e-9)
    ts = [0.0, 0.5e-9, 1e-9 + 50e-12, 3e-9, 6.1e-9 + 50e-12, 7e-9, 13e-9]
    v = po.wave_eval(p, ts)
    assert abs(v[0]) < 1e-10 and abs(v[1]) < 1e-10
    assert 1.5 < v[2] < 1.8
    assert abs(v[3] - 3.3) < 1e-10
    assert 1.5 < v[4] < 1.8
    assert abs(v[5]) < 1e-10 and abs(v[6] - 3.3) < 1e-10
    assert np.array_equal(v, [wf.evaluate(p, t) for t in ts])


def test_pwl_sin_exp():  # :68-137
    w = wf.pwl([(0.0, 0.0), (1e-6, 1.0), (2e-6, 2.0), (3e-6, 2.0), (4e-6, 0.0)])
    v = po.wave_eval(w, [0.5e-6, 1.5e-6, 2.5e-6, 3.5e-6, 5e-6])
    assert np.allclose(v, [0.5, 1.5, 2.0, 1.0, 0.0], rtol=0, atol=1e-10)
    s = wf.sin(0.0, 1.0, 1e6, 0.0, 0.0)
    v = po.wave_eval(s, [0.0, 0.25e-6, 0.5e-6, 0.75e-6, 1e-6])
    assert np.allclose(v, [0.0, 1.0, 0.0, -1.0, 0.0], rtol=0, atol=1e-10)
    e = wf.exp(0.0, 5.0, 0.0, 1e-6, 10e-6, 1e-6)
    v = po.wave_eval(e, [0.0, 1e-6, 5e-6])
    assert abs(v[0]) < 1e-10 and abs(v[1] - 5.0 * (1.0 - math.exp(-1.0))) < 0.01 and v[2] > 4.9
    for w_ in (w, s, e):  # the Python restatement agrees with the oracle's
        ts = np.linspace(0.0, 12e-6, 97)
        assert np.allclose(po.wave_eval(w_, ts), [wf.evaluate(w_, t) for t in ts], rtol=1e-15,
                           atol=1e-15)


def test_parse_source_value():  # waveform.rs:680-831
    p = wf.parse_source_value("PULSE(0 3.3 1n 100p 100p 5n 10n)")
    assert p.kind == "pulse" and np.allclose(p.params, (0, 3.3, 1e-9, 1e-10, 1e-10, 5e-9, 1e-8))
    q = wf.parse_source_value("pulse(0 1)")
    assert q.params == (0.0, 1.0, 0.0, 1e-9, 1e-9, 1e-6, 0.0)
    r = wf.parse_source_value("PWL(2u 1 0 0 1u 2)")
    assert r.points == ((0.0, 0.0), (1e-6, 2.0), (2e-6, 1.0))
    assert wf.parse_source_value("PWL(0 0 1u)") is None
    s = wf.parse_source_value("SIN(0.5 1 1meg)")
    assert s.kind == "sin" and s.params == (0.5, 1.0, 1e6, 0.0, 0.0)
    assert wf.parse_source_value("EXP(0 5 0 1u 10u 1u)").params[3] == 1e-6
    assert wf.parse_source_value("2.5k") == 2500.0


def test_breakpoints():  # :145-223
    v1 = wf.pulse(0.0, 5.0, 0.0, 10e-9, 10e-9, 50e-9, 100e-9)
    v2 = wf.pwl([(0.0, 0.0), (25e-9, 3.3), (75e-9, 3.3), (100e-9, 0.0)])
    times = po.breakpoints([v1, v2], 200e-9)
    assert len(times) >= 8
    assert np.all(np.diff(times) > 0)
    assert any(abs(t - 25e-9) < 1e-15 for t in times) and any(abs(t - 75e-9) < 1e-15 for t in times)
    bp = [10e-9, 20e-9, 30e-9]
    assert abs(po.bp_limit_dt(bp, 0.0, 15e-9, 1e-15) - 10e-9) < 1e-15
    assert abs(po.bp_limit_dt(bp, 10e-9, 15e-9, 1e-15) - 10e-9) < 1e-15
    assert abs(po.bp_limit_dt(bp, 0.0, 5e-9, 1e-15) - 5e-9) < 1e-15
    # within 10 % of the step: go to the breakpoint
    assert po.bp_limit_dt(bp, 0.0, 9.5e-9, 1e-15) == 10e-9
    s = po.bp_settling([10e-9], 3, 0.1, [(0.0, 5e-9), (5e-9, 10e-9), (10e-9, 11e-9),
                                         (11e-9, 12e-9), (12e-9, 13e-9)])
    assert s == [(False, False), (True, True), (True, True), (True, False), (False, False)]


def test_lte_milne():  # :266-320
    a = po.lte_milne([1, 2, 3, 4, 5], [1.001, 2.002, 3.003, 4.004, 5.005], 1e-6, 1e-3)
    assert 0.0 < a["error_norm"] < 1.0 and a["accept"]
    assert a["max_error_node"] == 4
    b = po.lte_milne([1, 2, 3], [1.1, 2.2, 3.3], 1e-9, 1e-6)
    assert b["error_norm"] > 1.0 and not b["accept"] and b["suggested_factor"] < 1.0
    assert b["suggested_factor"] == 0.1  # 0.9 / sqrt(large), clamped to 0.1
    c = po.lte_milne([1, 2, 3, 4, 5], [1, 2, 3.5, 4, 5], 1e-9, 1e-6)
    assert c["max_error_node"] == 2
    d = po.lte_milne([0, 1e-31, 2], [0, 2e-31, 2], 1e-9, 1e-6)  # zeros skipped, no error
    assert d["error_norm"] == 0.0 and d["suggested_factor"] == 2.0
    # the definition itself
    ratio = (0.5 / 3.0) / (1e-9 + 1e-6 * 3.5)
    assert c["error_norm"] == pytest.approx(ratio, rel=1e-15)
    assert c["suggested_factor"] == pytest.approx(min(max(0.9 * ratio ** -0.5, 0.1), 2.0))


def test_pi_controller():  # :327-410, analysis.rs:497-583, 720-743
    seq = po.adaptive_sequence(1e-15, 1e-6, [0.1], [1e-9])
    assert seq[0][0] and seq[0][1] > 1e-9  # small error: the step grows
    seq = po.adaptive_sequence(1e-15, 1e-6, [2.0], [1e-9])
    assert not seq[0][0] and seq[0][1] < 1e-9
    # history: after errors 0.8 and 0.5 the suggestion for 0.3 grows > 1.1x
    seq = po.adaptive_sequence(1e-15, 1e-6, [0.8, 0.5, 0.3], [1e-9, 1e-9, 1e-9])
    assert seq[2][3] > 1.1e-9
    assert seq[2][3] == pytest.approx(1e-9 * min(max((1 / 0.3) ** 0.35 * (1 / 0.5) ** 0.2 * 0.9,
                                                     0.1), 2.0), rel=1e-15)
    # five rejections: struggling, emergency dt below 0.3 dt
    seq = po.adaptive_sequence(1e-15, 1e-6, [2.0] * 5, [1e-9] * 5)
    assert seq[4][2] and seq[4][1] < 0.3e-9
    assert [s[2] for s in seq] == [False, False, True, True, True]
    assert seq[2][1] == 0.25e-9  # the third rejection: emergency 0.25 dt
    # an accepted step clears the struggle
    seq = po.adaptive_sequence(1e-15, 1e-6, [2.0, 2.0, 2.0, 0.5], [1e-9] * 4)
    assert seq[3][0] and not seq[3][2]


def _rc(vsrc, r=1000.0, c=1e-9):
    dev = cz._Dev()
    dev.add(cz.DEV_V, (1, 0), (vsrc,))
    dev.add(cz.DEV_R, (1, 2), (r,))
    dev.add(cz.DEV_C, (2, 0), (c,))
    return dev.build(3)


def test_rc_pulse_against_the_analytic_response():
    """A 1 kOhm / 1 nF low-pass driven by a 0 -> 1 V pulse (1 ns ramp at
    1 us): the accepted points follow 1 - exp(-(t - t0)/RC) (t0 the ramp's
    midpoint), the run completes and the breakpoints are hit exactly. The
    reference keeps the trapezoidal history current as the backward
    difference C (v_n - v_(n-1)) / dt (stamp.rs:631-647), which leaves the
    accepted solution first order: its global error grows to about 1e-4
    over the 5 us plateau (the oracle restates this)."""
    c = _rc(0.0)
    w = {0: wf.pulse(0.0, 1.0, 1e-6, 1e-9, 1e-9, 5e-6, 0.0)}
    r = po.tran_adaptive(c, w, 1e-7, 10e-6, abs_tol=1e-9, rel_tol=1e-6, be_sign=1.0)
    assert r["status"] == 0 and r["accepted"] > 100
    ts, v = r["times"], r["solutions"][:, 2]
    assert ts[0] == 0.0 and abs(ts[-1] - 10e-6) < 1e-18 and np.all(np.diff(ts) > 0)
    for bp in (1e-6, 1e-6 + 1e-9, 6e-6 + 1e-9, 6e-6 + 2e-9):
        assert np.min(np.abs(ts - bp)) < 1e-18, bp
    tau, t0 = 1e-6, 1e-6 + 0.5e-9
    m = (ts > 1.1e-6) & (ts < 6e-6)
    ana = 1.0 - np.exp(-(ts[m] - t0) / tau)
    assert np.max(np.abs(v[m] - ana)) < 5e-4
    # after the fall the capacitor discharges from its value at 6 us
    m2 = ts > 6.2e-6
    v6 = 1.0 - math.exp(-(6e-6 + 1e-9 - t0) / tau)
    ana2 = v6 * np.exp(-(ts[m2] - (6e-6 + 1.5e-9)) / tau)
    assert np.max(np.abs(v[m2] - ana2)) < 5e-4


def test_reference_be_sign_rejects_every_step_once_the_source_moves():
    """With the reference's backward-Euler companion (rhs[a] -= (C/dt) v),
    x_be is near -x_trap as soon as the capacitor holds a voltage, so every
    step is rejected and the run fails after ten rejections in a row
    (engine.rs:556-565): the steps before the pulse are accepted."""
    c = _rc(0.0)
    w = {0: wf.pulse(0.0, 1.0, 1e-6, 1e-9, 1e-9, 5e-6, 0.0)}
    r = po.tran_adaptive(c, w, 1e-7, 10e-6, abs_tol=1e-9, rel_tol=1e-6, be_sign=-1.0)
    assert r["status"] == 1 and r["rejected"] >= 10
    assert r["times"][-1] <= 1e-6 + 1e-9
    # a DC source charging the capacitor at the DC point: with the physical
    # sign nothing moves and every step is accepted; with the reference's
    # the very first steps are rejected, ten in a row
    r = po.tran_adaptive(_rc(1.0), {}, 1e-7, 10e-6, be_sign=1.0)
    assert r["status"] == 0 and r["rejected"] == 0
    assert np.allclose(r["solutions"][:, 2], 1.0, rtol=0, atol=1e-9)
    r = po.tran_adaptive(_rc(1.0), {}, 1e-7, 10e-6, be_sign=-1.0)
    assert r["status"] == 1 and r["accepted"] == 0 and r["rejected"] == 10
