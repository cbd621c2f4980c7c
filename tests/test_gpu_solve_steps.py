"""The single-system solve as a step program (k_solve_steps): bit for bit
the column sweeps' results (and so the oracle's), with each pivot division
done by Markstein's correction from the pivot's reciprocal; a diagonal
system over a wide exponent range checks every quotient against IEEE
division."""
import numpy as np
import pytest

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import GpuKluSolver

pytestmark = pytest.mark.gpu


def _diag_values(n, seed):
    """Pivots and right-hand sides: random significands over exponents
    +-250 (pivots) and +-300 (right-hand sides), significands of all ones,
    powers of two, values next to them, and zeros on the right."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-250, 250, n).astype(float))
    d *= rng.choice([-1.0, 1.0], n)
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-300, 300, n).astype(float))
    b *= rng.choice([-1.0, 1.0], n)
    k = n // 8
    ones = np.nextafter(2.0, 0.0)  # 1.111...1 in binary
    d[:k] = np.where(rng.random(k) < 0.5, ones, 1.0) * np.exp2(rng.integers(-40, 40, k).astype(float))
    b[k:2 * k] = np.where(rng.random(k) < 0.5, ones, 1.0) * np.exp2(rng.integers(-40, 40, k).astype(float))
    d[2 * k:3 * k] = np.nextafter(d[2 * k:3 * k], np.inf)
    b[3 * k:3 * k + 64] = 0.0
    b[3 * k + 64:3 * k + 128] = -0.0
    d[3 * k + 128:3 * k + 192] = 1e-299  # below the exponent guard: the division itself
    b[3 * k + 192:3 * k + 256] = 1e-308  # subnormal right-hand sides
    return d, b


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pivot_division_is_ieee(seed):
    n = 20000
    d, b = _diag_values(n, seed)
    ap = np.arange(n + 1, dtype=np.int64)
    ai = np.arange(n, dtype=np.int64)
    g = GpuKluSolver(n, pivot_mode=N.PIVOT_EXACT)
    g.factor(ap, ai, d)
    x = b.copy()
    g.solve(x)
    with np.errstate(over="ignore", under="ignore"):
        want = b / d
    bad = np.flatnonzero(x.view(np.int64) != want.view(np.int64))
    assert len(bad) == 0, (bad[:5], x[bad[:5]], want[bad[:5]], b[bad[:5]], d[bad[:5]])
    g.close()


def _systems():
    out = []
    c = cz.mesh_dc()
    out.append(("mesh32", po.mna(c, np.zeros(c.node_count))))
    for s, v in [(8, 0.3), (256, 0.55)]:
        c = cz.inverter_chain(s, v)
        out.append((f"chain{s}", po.mna(c, wl.chain_nodeset(s, v))))
    return out


@pytest.mark.parametrize("mode", [N.PIVOT_REFERENCE, N.PIVOT_EXACT], ids=["reference", "exact"])
def test_step_solve_equals_the_sweeps(mode, monkeypatch):
    from test_gpu_solver import _block_lower
    for name, (n, ap, ai, ax, rhs) in _systems() + [("blocklower", _block_lower())]:
        xs = []
        for steps in ("1", "0"):
            monkeypatch.setenv("GPUKLU_SOLVE_STEPS", steps)
            g = GpuKluSolver(n, pivot_mode=mode)
            g.factor(ap, ai, ax)
            x = rhs.copy()
            g.solve(x)
            xs.append(x)
            g.close()
        assert np.array_equal(xs[0], xs[1]), (name, np.max(np.abs(xs[0] - xs[1])))
