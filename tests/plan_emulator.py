"""Scalar CPU emulation of the device algorithms over a host Plan.

Test infrastructure: it runs the exact operation sequence of the CUDA kernels
(first factor with the reference pivot rule, frozen-pivot refactor, block
solve) on the integer plan the library builds, so the plan itself (slot maps,
update lists, permutations, block coupling) can be checked against the
oracle on a machine without a GPU.
"""
from __future__ import annotations

import numpy as np

from rustspice_gb300 import native


def _perturb(d, single):
    if single:
        return 1e-14 if abs(d) < 1e-300 else d
    if abs(d) < 1e-14:
        return 1e-14 if d >= 0.0 else -1e-14
    return d


def first_factor(P: native.Plan, ax, tol=0.001):
    n = P.n
    lu = np.zeros(P.nslots)
    work = np.zeros(n)
    b0s = P.block_ptr[P.pos_block]
    rperm = (np.arange(n) - b0s).astype(np.int64)
    rinv = rperm.copy()
    for k in range(n):
        b0 = b0s[k]
        s0, ds, s1 = P.col_ptr[k], P.dslot[k], P.col_ptr[k + 1]
        t0, t1 = P.pcol_ptr[k], P.pcol_ptr[k + 1]
        if P.col_single[k]:
            d = 0.0
            for t in range(t0, t1):
                d += ax[P.pcol_raw[t]]
            lu[ds] = _perturb(d, True)
            continue
        for t in range(t0, t1):
            work[b0 + rinv[b0 + P.pcol_q[t]]] += ax[P.pcol_raw[t]]
        for s in range(s0, ds):
            j = P.slot_row[s]
            u = work[j]
            if u != 0.0:
                for q in range(P.dslot[j] + 1, P.col_ptr[j + 1]):
                    r = P.slot_row[q]
                    work[r] = work[r] - lu[q] * u
        dabs = abs(work[k])
        best, bq = -1.0, -1
        for q in range(ds + 1, s1):
            v = abs(work[P.slot_row[q]])
            if v > best:
                best, bq = v, q
        if bq >= 0 and best > dabs and dabs < tol * best:
            mr = P.slot_row[bq]
            work[k], work[mr] = work[mr], work[k]
            ok, om = rperm[k], rperm[mr]
            rperm[k], rperm[mr] = om, ok
            rinv[b0 + ok] = mr - b0
            rinv[b0 + om] = k - b0
        for s in range(s0, ds):
            lu[s] = work[P.slot_row[s]]
        diag = _perturb(work[k], False)
        lu[ds] = diag
        for q in range(ds + 1, s1):
            lu[q] = work[P.slot_row[q]] / diag
        for t in range(t0, t1):
            work[b0 + rinv[b0 + P.pcol_q[t]]] = 0.0
        for q in range(s0, s1):
            work[P.slot_row[q]] = 0.0
        work[k] = 0.0
    return lu, rperm


def staged_amap(P: native.Plan, swaps):
    """Raw entries summed into each slot when column k scatters A(:,k)
    through the row order the pivot pass has reached at column k: the swaps
    {column: row position} of earlier columns applied to the identity.
    Entries that land outside the column's pattern are dropped (the pivot
    pass adds them to working positions it never reads)."""
    n = P.n
    b0s = P.block_ptr[P.pos_block]
    rperm = (np.arange(n) - b0s).astype(np.int64)
    rinv = rperm.copy()
    lists = [[] for _ in range(P.nslots)]
    for k in range(n):
        b0 = b0s[k]
        where = {int(P.slot_row[s]): s for s in range(P.col_ptr[k], P.col_ptr[k + 1])}
        for t in range(P.pcol_ptr[k], P.pcol_ptr[k + 1]):
            s = where.get(int(b0 + rinv[b0 + P.pcol_q[t]]))
            if s is not None:
                lists[s].append(int(P.pcol_raw[t]))
        if k in swaps:
            mr = swaps[k]
            ok, om = rperm[k], rperm[mr]
            rperm[k], rperm[mr] = om, ok
            rinv[b0 + ok] = mr - b0
            rinv[b0 + om] = k - b0
    return lists, rperm


def staged_refactor(P: native.Plan, ax, lists, cand, tol):
    """The refactorization kernel in its pivot-pass mode: before scaling
    column k it applies the pass's threshold rule to the column's finished
    values, writes the choice to want[k] (an L slot, or -1 for the diagonal)
    and swaps the candidate's row (cand[k], an L slot or -1) into the
    pivot."""
    lu = np.zeros(P.nslots)
    want = np.full(P.n, -1, np.int64)
    for k in range(P.n):
        s0, ds, s1 = P.col_ptr[k], P.dslot[k], P.col_ptr[k + 1]
        for s in range(s0, s1):
            v = 0.0
            for t in lists[s]:
                v += ax[t]
            lu[s] = v
        for s in range(s0, ds):
            j = P.slot_row[s]
            u = lu[s]
            if u != 0.0:
                q0 = P.dslot[j] + 1
                for q in range(q0, P.col_ptr[j + 1]):
                    d = P.upd_dst[P.upd_ptr[s] + q - q0]
                    lu[d] = lu[d] - lu[q] * u
        if not P.col_single[k]:
            dabs = abs(lu[ds])
            best, bq = -1.0, -1
            for q in range(ds + 1, s1):
                v = abs(lu[q])
                if v > best:
                    best, bq = v, q
            if bq >= 0 and best > dabs and dabs < tol * best:
                want[k] = bq
            c = cand[k]
            if c >= 0:
                lu[ds], lu[c] = lu[c], lu[ds]
        diag = _perturb(lu[ds], bool(P.col_single[k]))
        lu[ds] = diag
        for q in range(ds + 1, s1):
            lu[q] = lu[q] / diag
    return lu, want


def staged_first_factor(P: native.Plan, ax, tol=0.001, max_passes=8, start=None):
    """The pivot pass as the host runs it on the device: refactorizations of
    the pivot-free pattern with a candidate pivot sequence (start: per column
    an L slot or -1, e.g. the last sequence found for this pattern; default
    none); from the first column whose choice disagrees with the candidate
    on, the choices become the next candidate, until a pass agrees
    everywhere. Returns (lu, rperm, passes, cand), or None when max_passes
    did not settle it (the sequential pass runs then)."""
    n = P.n
    cand = np.full(n, -1, np.int64) if start is None else np.array(start, np.int64)
    for p in range(max_passes):
        rows = {k: int(P.slot_row[c]) for k, c in enumerate(cand) if c >= 0}
        lists, rperm = staged_amap(P, rows)
        lu, want = staged_refactor(P, ax, lists, cand, tol)
        bad = np.nonzero(want != cand)[0]
        if len(bad) == 0:
            return lu, rperm, p + 1, cand
        cand[bad[0]:] = want[bad[0]:]
    return None


def refactor(P: native.Plan, ax):
    lu = np.zeros(P.nslots)
    for k in range(P.n):
        s0, ds, s1 = P.col_ptr[k], P.dslot[k], P.col_ptr[k + 1]
        for s in range(s0, s1):
            v = 0.0
            for t in range(P.amap_ptr[s], P.amap_ptr[s + 1]):
                v += ax[P.amap_idx[t]]
            lu[s] = v
        for s in range(s0, ds):
            j = P.slot_row[s]
            u = lu[s]
            if u != 0.0:
                q0 = P.dslot[j] + 1
                for q in range(q0, P.col_ptr[j + 1]):
                    d = P.upd_dst[P.upd_ptr[s] + q - q0]
                    lu[d] = lu[d] - lu[q] * u
        diag = _perturb(lu[ds], bool(P.col_single[k]))
        lu[ds] = diag
        for q in range(ds + 1, s1):
            lu[q] = lu[q] / diag
    return lu


def solve(P: native.Plan, ax, lu, rhs):
    """Row-oriented dependency order, as the device solve computes it."""
    n = P.n
    in_row = np.zeros(n, np.int64)
    in_row[P.in_pos] = np.arange(n)
    z = np.zeros(n)
    x = np.zeros(n)
    nb = P.nblocks
    order = range(nb) if P.offd_lower else range(nb - 1, -1, -1)
    for b in order:
        b0, b1 = P.block_ptr[b], P.block_ptr[b + 1]
        for i in range(b0, b1):
            v = rhs[in_row[i]]
            for e in range(P.offd_ptr[i], P.offd_ptr[i + 1]):
                v = v - ax[P.offd_raw[e]] * x[P.offd_col[e]]
            for e in range(P.lrow_ptr[i], P.lrow_ptr[i + 1]):
                v = v - lu[P.lrow_slot[e]] * z[P.lrow_col[e]]
            z[i] = v
        for i in range(b1 - 1, b0 - 1, -1):
            v = z[i]
            for e in range(P.urow_ptr[i], P.urow_ptr[i + 1]):
                v = v - lu[P.urow_slot[e]] * x[P.urow_col[e]]
            x[i] = v / lu[P.dslot[i]]
    out = np.zeros(n)
    out[:] = x[P.out_pos]
    return out


SOLVE_CHUNK = 2048  # slots per chunk of the one-block solve (kSolveChunk)


def solve_one_block(P: native.Plan, ax, lu, rhs):
    """The one-block solve's column sweeps over its chunk schedule, with the
    double buffer's index arithmetic checked: every slot an op reads lies in
    its chunk's range, and no chunk is longer than the buffer."""
    n = P.n
    in_row = np.zeros(n, np.int64)
    in_row[P.in_pos] = np.arange(n)
    w = np.asarray(rhs, np.float64)[in_row].copy()
    ch, op = P.cs_chunk.reshape(-1, 4), P.cs_op.reshape(-1, 3)
    assert ch.shape[0] > 0 and ch[0, 2] == 0 and ch[-1, 3] == op.shape[0]
    for c in range(ch.shape[0]):
        lo, hi, o0, o1 = (int(v) for v in ch[c])
        assert 0 <= lo <= hi <= P.nslots and hi - lo <= SOLVE_CHUNK
        if c + 1 < ch.shape[0]:
            assert ch[c + 1, 2] == o1
        buf_v = lu[lo:hi]
        buf_r = P.slot_row[lo:hi]

        def at(q, direct):
            if direct:
                return lu[q], P.slot_row[q]
            assert lo <= q < hi
            return buf_v[q - lo], buf_r[q - lo]

        for o in range(o0, o1):
            code, a, b = (int(v) for v in op[o])
            direct = bool(code & 4)
            assert 0 <= a < b <= n
            if code & 3 == 0:
                for i in range(a, b):
                    v = w[i]
                    for e in range(P.offd_ptr[i], P.offd_ptr[i + 1]):
                        v = v - ax[P.offd_raw[e]] * w[P.offd_col[e]]
                    w[i] = v
            elif code & 3 == 1:
                for j in range(a, b):
                    xj = w[j]
                    for q in range(P.dslot[j] + 1, P.col_ptr[j + 1]):
                        val, r = at(q, direct)
                        assert j < r < n
                        w[r] = w[r] - val * xj
            else:
                for j in range(b - 1, a - 1, -1):
                    ds = P.dslot[j]
                    dv, _ = at(ds, direct)
                    xj = w[j] / dv
                    for q in range(P.col_ptr[j], ds):
                        val, r = at(q, direct)
                        assert 0 <= r < j
                        w[r] = w[r] - val * xj
                    w[j] = xj
    out = np.zeros(n)
    out[:] = w[P.out_pos]
    return out


def solve_groups(P: native.Plan, ax, lu, rhs):
    """The one-block solve split over thread blocks (cs_grp): every group
    sweeps its own chunks with its rows in a local array indexed by position
    minus its first row. Checks that the groups cover the rows in order, that
    their chunk ranges cover the schedule in order, and that every op and
    every row an update writes lies inside its group."""
    n = P.n
    grp = P.cs_grp.reshape(-1, 4)
    ch, op = P.cs_gchunk.reshape(-1, 4), P.cs_gop.reshape(-1, 3)
    assert grp.shape[0] > 0 and grp[0, 0] == 0 and grp[-1, 1] == n
    assert grp[0, 2] == 0 and grp[-1, 3] == ch.shape[0] and ch[-1, 3] == op.shape[0]
    in_row = np.zeros(n, np.int64)
    in_row[P.in_pos] = np.arange(n)
    x = np.zeros(n)
    for g in range(grp.shape[0]):
        r0, r1, c0, c1 = (int(v) for v in grp[g])
        if g + 1 < grp.shape[0]:
            assert grp[g + 1, 0] == r1 and grp[g + 1, 2] == c1
        w = np.asarray(rhs, np.float64)[in_row[r0:r1]].copy()
        for c in range(c0, c1):
            lo, hi, o0, o1 = (int(v) for v in ch[c])
            assert 0 <= lo <= hi <= P.nslots and hi - lo <= SOLVE_CHUNK

            def at(q, direct):
                if not direct:
                    assert lo <= q < hi
                return lu[q], int(P.slot_row[q])

            for o in range(o0, o1):
                code, a, b = (int(v) for v in op[o])
                direct = bool(code & 4)
                assert r0 <= a < b <= r1 and code & 3 != 0
                if code & 3 == 1:
                    for j in range(a, b):
                        xj = w[j - r0]
                        for q in range(P.dslot[j] + 1, P.col_ptr[j + 1]):
                            val, r = at(q, direct)
                            assert j < r < r1
                            w[r - r0] = w[r - r0] - val * xj
                else:
                    for j in range(b - 1, a - 1, -1):
                        ds = P.dslot[j]
                        dv, _ = at(ds, direct)
                        xj = w[j - r0] / dv
                        for q in range(P.col_ptr[j], ds):
                            val, r = at(q, direct)
                            assert r0 <= r < j
                            w[r - r0] = w[r - r0] - val * xj
                        w[j - r0] = xj
        x[r0:r1] = w
    return x[P.out_pos]


class EmulatedSolver:
    """LinearSolver call sequence over the emulated kernels."""

    def __init__(self, mode=native.PIVOT_REFERENCE, kind="nativeklu"):
        self.mode = mode
        self.kind = kind
        # the SparseLU kinds never exchange rows
        self.tol = 0.001 if kind == "nativeklu" else 0.0
        self.plan = None
        self.key = None
        self.lu = None
        self.factored = False

    def factor(self, n, ap, ai, ax):
        key = (n, ap.tobytes(), ai.tobytes())
        if key != self.key:
            self.key = key
            self.plan = native.Plan(n, ap, ai, self.mode, kind=self.kind)
            self.factored = False
        if not self.factored:
            lu, rperm = first_factor(self.plan, ax, self.tol)
            self.plan = native.Plan(n, ap, ai, self.mode, row_perm=rperm, kind=self.kind)
            self.lu = lu if self.mode == native.PIVOT_REFERENCE else refactor(self.plan, ax)
            self.factored = True
        else:
            self.lu = refactor(self.plan, ax)
        self.ax = np.asarray(ax, np.float64)

    def solve(self, rhs):
        return solve(self.plan, self.ax, self.lu, np.asarray(rhs, np.float64))


def batch_region(P: native.Plan, ax, rhs, nc, ndv):
    """An instance region of the batched warp kernel (X[nc], T[n], DV[ndv],
    V[nslots + noffd]) with the LU slots, the coupling values and the
    permuted right-hand side assembled from a matrix and a right-hand side."""
    n = P.n
    tb, vb = nc, nc + n + ndv
    R = np.zeros(vb + P.nslots + len(P.offd_raw))
    for s in range(P.nslots):
        v = 0.0
        for t in range(P.amap_ptr[s], P.amap_ptr[s + 1]):
            v += ax[P.amap_idx[t]]
        R[vb + s] = v
    for e in range(len(P.offd_raw)):
        R[vb + P.nslots + e] = ax[P.offd_raw[e]]
    R[tb + P.in_pos] = rhs
    return R


def factor_solve_columns(P: native.Plan, R, nc, ndv):
    """The batched kernels' column-by-column factorization with the forward
    substitution fused, then the backward substitution, block by block
    (bt::factor_solve_columns), on a region; a fused multiply-add is
    emulated as a product then a difference."""
    n, ns = P.n, P.nslots
    T = lambda i: nc + i  # noqa: E731
    V = lambda v: nc + n + ndv + v  # noqa: E731
    for b in range(P.nblocks):
        b0, b1 = P.block_ptr[b], P.block_ptr[b + 1]
        for i in range(b0, b1):
            for e in range(P.offd_ptr[i], P.offd_ptr[i + 1]):
                R[T(i)] = R[T(i)] - R[V(ns + e)] * R[T(P.offd_col[e])]
        for k in range(b0, b1):
            s0, ds, s1 = P.col_ptr[k], P.dslot[k], P.col_ptr[k + 1]
            for s in range(s0, ds):
                u = R[V(s)]
                if u != 0.0:
                    j = P.slot_row[s]
                    q0 = P.dslot[j] + 1
                    for qq in range(q0, P.col_ptr[j + 1]):
                        d = P.upd_dst[P.upd_ptr[s] - q0 + qq]
                        R[V(d)] = R[V(d)] - R[V(qq)] * u
            r = 1.0 / _perturb(R[V(ds)], bool(P.col_single[k]))
            zk = R[T(k)]
            for qq in range(ds + 1, s1):
                lv = R[V(qq)] * r
                R[V(qq)] = lv
                R[T(P.slot_row[qq])] = R[T(P.slot_row[qq])] - lv * zk
            R[V(ds)] = r
        for k in range(b1 - 1, b0 - 1, -1):
            s0, ds = P.col_ptr[k], P.dslot[k]
            xk = R[T(k)] * R[V(ds)]
            for s in range(s0, ds):
                R[T(P.slot_row[s])] = R[T(P.slot_row[s])] - R[V(s)] * xk
            R[T(k)] = xk
    return R


def run_steps(ops, sp, R, order=None):
    """A step program (native.step_program) on a region, the operations of
    each step in the given order ("reverse", a numpy Generator for a
    shuffle, or None for the listed order): the results do not depend on it
    when the operations of a step are independent."""
    for t in range(len(sp) - 1):
        idx = list(range(sp[t], sp[t + 1]))
        if order == "reverse":
            idx.reverse()
        elif order is not None:
            order.shuffle(idx)
        for p in idx:
            x, y = int(ops[p, 0]) & 0xffffffff, int(ops[p, 1]) & 0xffffffff
            d, a = x & 0x7fff, (x >> 15) & 0x7fff
            b, c = y & 0x7fff, (y >> 15) & 0x7fff
            k = (x >> 30) | ((y >> 30) << 2)
            if k == 1:
                R[d] = 1.0 / _perturb(R[d], a != 0)
            elif k == 2:
                R[d] = R[a] * R[b]
            elif k in (4, 5):
                t = R[d] - R[a] * R[b] if R[b] != 0.0 else R[d]
                R[d] = t * R[c] if k == 5 else t
            elif k in (0, 6):
                t = R[d] - R[a] * R[b]
                R[d] = t * R[c] if k == 6 else t
    return R
