"""DC adjoint sensitivities on the GPU (the 20k-node mesh + inverter case).

Forward: the device-resident DC operating point against the oracle. Backward:
lambda from the transpose solve against a SciPy solve with A(x*)^T, the
parameter gradients against the same formula evaluated on the host, and the
largest gradients against central finite differences through the plain GPU
solver (relative steps 1e-6 and 1e-4).
"""
import time

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from oracle import pyoracle as po
from rustspice_gb300 import circuits as cz
from rustspice_gb300 import native as N
from rustspice_gb300 import workloads as wl
from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver, dc_backward, dc_forward

pytestmark = pytest.mark.gpu

OCFG = {k: wl.TIGHT[k] for k in ("max_iters", "abs_tol", "rel_tol", "gmin", "gmin_steps",
                                 "source_steps")}


def _loss_grad(x, outs):
    g = np.zeros(len(x))
    g[outs] = 2.0 * (x[outs] - 0.6)
    return float(np.sum((x[outs] - 0.6) ** 2)), g


def _host_grads(c, x, lam):
    """dL/dp = -lambda^T dF/dp, evaluated with numpy (R and MC only)."""
    out = np.zeros(c.ndev)
    nd, p = c.nodes, c.p
    for d in range(c.ndev):
        t = c.type[d]
        if t == cz.DEV_R:
            a, b = nd[d, 0], nd[d, 1]
            out[d] = (lam[a] - lam[b]) * (x[a] - x[b]) / (p[d, 0] ** 2)
        elif t == cz.DEV_MC:
            dr, gt, sr = nd[d, 0], nd[d, 1], nd[d, 2]
            pol = -1.0 if p[d, 0] != 0 else 1.0
            vgs, vds = pol * (x[gt] - x[sr]), pol * (x[dr] - x[sr])
            rev = vds < 0
            if rev:
                vgs, vds = vgs - vds, -vds
            vth = abs(p[d, 1])
            beff = p[d, 2] * 1e-4 * ((3.9 * 8.854e-12) / p[d, 3]) * p[d, 4] / p[d, 5]
            gm = 0.0
            if vgs > vth:
                gm = (beff * vds * (1 + 0.02 * vds) if vds < vgs - vth
                      else beff * (vgs - vth) * (1 + 0.02 * vds))
            sgn = -pol if rev else pol
            did = sgn * (-gm) * (1.0 if p[d, 1] >= 0 else -1.0)
            out[d] = -(lam[dr] - lam[sr]) * did
    return out


def test_dc_adjoint_mesh_inverters():
    c = cz.mesh_with_inverters(120, 1000)
    outs = cz.output_nodes(c, 256)
    g = GpuKluSolver(1, pivot_mode=N.PIVOT_EXACT)
    dc = DeviceCircuit(c)
    cfg = N.newton_config(**wl.TIGHT)
    t0 = time.perf_counter()
    fwd = dc_forward(g, dc, cfg)
    t_fwd = time.perf_counter() - t0
    assert fwd.converged
    r_o, it_o, x_o = po.dc_op(c, "nativeklu_exact", **OCFG)
    assert r_o == "converged" and fwd.iterations == it_o
    assert np.max(np.abs(fwd.x - x_o)) <= 1e-10 * np.max(np.abs(x_o))
    x = fwd.x
    loss, dl_dx = _loss_grad(x, outs)
    t0 = time.perf_counter()
    lam, grad = dc_backward(g, dc, x, dl_dx)
    t_bwd = time.perf_counter() - t0
    # lambda against a host transpose solve of the exact Jacobian at x*
    n, ap, ai, ax, rhs = po.mna(c, x[:c.node_count], gdev=0.0)
    A = sp.csc_matrix((ax, ai, ap), shape=(n, n))
    lam_ref = spl.spsolve(A.T.tocsc(), dl_dx)
    assert np.max(np.abs(lam - lam_ref)) <= 1e-9 * np.max(np.abs(lam_ref))
    # gradient formula
    ref = _host_grads(c, x, lam_ref)
    sel = (c.type == cz.DEV_R) | (c.type == cz.DEV_MC)
    scale = np.max(np.abs(ref[sel]))
    assert np.max(np.abs(grad[sel] - ref[sel])) <= 1e-8 * scale
    print(f"forward {t_fwd*1e3:.1f} ms ({fwd.iterations} iterations), backward "
          f"{t_bwd*1e3:.1f} ms, ratio {t_bwd / t_fwd:.2f}")
    # Central finite differences through the plain solver, largest gradients.
    # The converged fixed point carries the rounding of the residual
    # evaluation amplified by lambda (which reaches 6e4 here): about 1e-12 on
    # a loss of 9, so a quotient at relative step 1e-6 holds ~1e-6 relative
    # noise of its own.  Each device therefore samples L at p0 + k*h,
    # k = +-1..+-4, h = 1e-6*|p0|: the quotient from k = +-1 is the
    # step-1e-6 FD, and the rms residual of a cubic fit to the eight samples
    # is the loss noise sigma, which bounds the quotient's own error by
    # 4*sqrt(2)*sigma/(2h).  At relative step 1e-4 that term is negligible
    # and the check is a strict 1e-6 relative.
    fd_cfg = N.newton_config(**dict(wl.TIGHT, abs_tol=1e-15, rel_tol=1e-14))

    def loss_at(d, slot, val):
        pp = c.p.copy()
        pp[d, slot] = val
        dc.set_params(pp)
        r = dc_forward(g, dc, fd_cfg, x0=x[:c.node_count])
        assert r.converged
        return _loss_grad(r.x, outs)[0]

    checks = []
    ks = np.array([-4, -3, -2, -1, 1, 2, 3, 4], np.float64)
    for kind, slot in ((cz.DEV_R, 0), (cz.DEV_MC, 1)):
        idx = np.flatnonzero(c.type == kind)
        top = idx[np.argsort(-np.abs(grad[idx]))[:6]]
        for d in top:
            p0 = c.p[d, slot]
            h = 1e-6 * abs(p0)
            ls = np.array([loss_at(d, slot, p0 + k * h) for k in ks])
            coef, res, *_ = np.polyfit(ks, ls - loss, 3, full=True)
            sigma = float(np.sqrt(res[0] / (len(ks) - 4))) if len(res) else 0.0
            fd = (ls[4] - ls[3]) / (2 * h)
            noise = 4.0 * np.sqrt(2.0) * sigma / (2 * h)
            checks.append((1e-6, d, grad[d], fd, abs(grad[d] - fd) / abs(fd), sigma))
            assert abs(grad[d] - fd) <= 1e-6 * abs(fd) + noise, (1e-6, d, grad[d], fd, sigma)
            h4 = 1e-4 * abs(p0)
            fd4 = (loss_at(d, slot, p0 + h4) - loss_at(d, slot, p0 - h4)) / (2 * h4)
            checks.append((1e-4, d, grad[d], fd4, abs(grad[d] - fd4) / abs(fd4), 0.0))
            assert abs(grad[d] - fd4) <= 1e-6 * abs(fd4), (1e-4, d, grad[d], fd4)
    dc.set_params(c.p)
    w6 = max(ch[4] for ch in checks if ch[0] == 1e-6)
    w4 = max(ch[4] for ch in checks if ch[0] == 1e-4)
    sig = max(ch[5] for ch in checks)
    print(f"{len(checks)} FD checks: worst rel diff {w6:.2e} at step 1e-6 (loss noise up to "
          f"{sig:.1e}), {w4:.2e} at step 1e-4")
