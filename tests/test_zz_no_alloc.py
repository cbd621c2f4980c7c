"""The no-allocation solve entry point, against the regular solve.

gpuklu_solve_device_noalloc exists for callers that cannot call cudaMalloc
where they solve (for example inside a runtime that owns all device memory
and only lends buffers, or a loop with a fixed device-memory budget); its kernel
scratch is a fixed array inside the library. This test drives it through the
C ABI with device buffers the test owns, twice in a row with different
right-hand sides, and requires results identical to gpuklu_solve (the same
kernel, so bit for bit). It lives in its own file, collected last, and needs
nothing from the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system():
    from rustspice_gb300 import circuits as cz
    from rustspice_gb300 import workloads as wl
    from rustspice_gb300.solver import DeviceCircuit, GpuKluSolver
    c = cz.mesh_dc(side=24, ndiodes=20, seed=9)
    g = GpuKluSolver(1)
    dc = DeviceCircuit(c)
    ap, ai = dc.pattern()
    x = np.random.default_rng(3).uniform(0.0, 0.8, c.node_count)
    ax, rhs = dc.stamp(g, x)
    g.close()
    return dc.n, ap, ai, ax, rhs


@pytest.mark.parametrize("one_block", ["1", "0"], ids=["one_block", "grid"])
def test_noalloc_solve_matches_solve(one_block, monkeypatch):
    monkeypatch.setenv("GPUKLU_ONE_BLOCK", one_block)
    import torch
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import GpuKluSolver

    n, ap, ai, ax, rhs = _system()
    L = N.lib()
    for mode in (N.PIVOT_REFERENCE, N.PIVOT_EXACT):
        g = GpuKluSolver(n, pivot_mode=mode)
        g.factor(ap, ai, ax)
        rng = np.random.default_rng(mode)
        for call in range(2):  # two calls in a row share the library's scratch
            b = rhs if call == 0 else rng.standard_normal(n)
            want = np.ascontiguousarray(b, np.float64).copy()
            g.solve(want)
            d_b = torch.tensor(b, dtype=torch.float64, device="cuda")
            d_x = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            st = L.gpuklu_solve_device_noalloc(g.handle, C.c_void_p(d_b.data_ptr()),
                                               C.c_void_p(d_x.data_ptr()))
            assert st == N.OK, L.gpuklu_last_error(g.handle).decode()
            got = d_x.cpu().numpy()
            assert np.array_equal(got, want), np.max(np.abs(got - want))
        g.close()


def test_noalloc_rejects_oversize():
    import torch
    import scipy.sparse as sp
    from rustspice_gb300 import native as N
    from rustspice_gb300.solver import GpuKluSolver

    n = N.lib() and 65536 + 8
    A = sp.diags(np.full(n, 2.0)).tocsc()
    g = GpuKluSolver(n)
    g.factor(A.indptr.astype(np.int64), A.indices.astype(np.int64), A.data)
    d_b = torch.ones(n, dtype=torch.float64, device="cuda")
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = N.lib().gpuklu_solve_device_noalloc(g.handle, C.c_void_p(d_b.data_ptr()),
                                             C.c_void_p(d_x.data_ptr()))
    assert st == N.INVALID_MATRIX
    assert b"GPUKLU_NOALLOC_MAX_N" in N.lib().gpuklu_last_error(g.handle)
    g.close()
