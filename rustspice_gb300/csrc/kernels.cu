// CUDA kernels of the Newton inner loop (sm_103a).
//
//  * first_factor  - the reference's first numeric factorization with its
//                    threshold pivot rule (crates/sim-core/src/native_klu.rs:
//                    1194-1382), one warp walking the columns in order; it
//                    discovers the pivot sequence. k_first_factor_s keeps the
//                    working column and each column's update operands in
//                    shared memory; k_first_factor is the fallback for blocks
//                    too large for that. From 512 rows on the host runs the
//                    same pass as refactorizations in their pivot-pass mode
//                    (PivotCheck) instead, and these kernels only when that
//                    does not settle.
//  * refactor      - left-looking refactorization with frozen pivots. Warps
//                    take columns in increasing order from an atomic counter
//                    and wait on per-column completion flags of exactly the
//                    columns they depend on (the U pattern), so independent
//                    columns run concurrently without level barriers; a
//                    warp's column sits in shared memory while it is updated.
//                    k_refactor_cta is the same in one block, for small plans.
//  * solve         - the forward (L) and backward (U) substitutions and the
//                    BTF block coupling. k_solve_cta sweeps the columns in one
//                    block (solution vector in shared memory); k_solve runs
//                    one warp per row task driven by per-row flags (large
//                    plans); k_tsolve solves A^T y = g for the adjoint.
//  * stamp         - one thread per device instance writes its conductances
//                    into the raw CSC slots given by the stamp-to-slot map and
//                    its currents into per-contribution slots; a second pass
//                    sums the right-hand side row by row in stamping order.
//  * newton_update - convergence test, damping and the iterate update of
//                    crates/sim-core/src/newton.rs:93-107, 187-201.
//  * batch_newton  - batched Newton over many circuit instances, one warp per
//                    instance (or 2, 4 per warp for small programs) with the
//                    instance's whole state in shared memory; behind the lane
//                    kernel (lanes.cu) it finishes the instances still
//                    iterating.
//
// All floating-point work of the single-circuit kernels is FP64 and compiled
// without multiply-add contraction, so every product is rounded before it is
// added exactly as in the reference; their factor and solve results are
// bit-identical to a scalar CPU evaluation in the reference's order. The
// batched kernels use fused multiply-adds and agree with the oracle within
// the Newton tolerance.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "batch_common.cuh"
#include "device.cuh"
#include "kernels.cuh"

namespace gk {

namespace {
constexpr unsigned FULL = 0xffffffffu;

// --------------------------------------------------------------- first factor
__global__ void k_first_factor(DPlan P, const double* __restrict__ ax, double* lu,
                               double* work, int* rperm, int* rinv, double tol,
                               int* status) {
  const int lane = threadIdx.x;
  const int n = P.n;
  for (int i = lane; i < n; i += 32) {
    int b0 = P.block_ptr[P.pos_block[i]];
    rperm[i] = i - b0;
    rinv[i] = i - b0;
    work[i] = 0.0;
  }
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    const int b0 = P.block_ptr[P.pos_block[k]];
    const int s0 = P.col_ptr[k], ds = P.dslot[k], s1 = P.col_ptr[k + 1];
    const int t0 = P.pcol_ptr[k], t1 = P.pcol_ptr[k + 1];
    if (P.col_single[k]) {
      if (lane == 0) {
        double d = 0.0;
        for (int t = t0; t < t1; ++t) d += ax[P.pcol_raw[t]];
        lu[ds] = perturb(d, true);
      }
      __syncwarp();
      continue;
    }
    if (lane == 0)  // duplicates accumulate in CSC order
      for (int t = t0; t < t1; ++t) {
        int w = b0 + rinv[b0 + P.pcol_q[t]];
        work[w] += ax[P.pcol_raw[t]];
      }
    __syncwarp();
    for (int s = s0; s < ds; ++s) {
      const int j = P.slot_row[s];
      const double u = work[j];
      if (u != 0.0) {
        const int q1 = P.col_ptr[j + 1];
        for (int q = P.dslot[j] + 1 + lane; q < q1; q += 32) {
          int r = P.slot_row[q];
          work[r] = work[r] - lu[q] * u;
        }
      }
      __syncwarp();
    }
    // threshold pivot search inside the symbolic pattern: the first row with
    // the largest magnitude wins; the diagonal wins ties
    const double dabs = fabs(work[k]);
    double best = -1.0;
    int bidx = 0x7fffffff;
    for (int q = ds + 1 + lane; q < s1; q += 32) {
      double v = fabs(work[P.slot_row[q]]);
      if (v > best) {
        best = v;
        bidx = q;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      double ov = __shfl_down_sync(FULL, best, off);
      int oi = __shfl_down_sync(FULL, bidx, off);
      if (ov > best || (ov == best && oi < bidx)) {
        best = ov;
        bidx = oi;
      }
    }
    best = __shfl_sync(FULL, best, 0);
    bidx = __shfl_sync(FULL, bidx, 0);
    if (lane == 0 && bidx != 0x7fffffff && best > dabs && dabs < tol * best) {
      const int mr = P.slot_row[bidx];
      double tmp = work[k];
      work[k] = work[mr];
      work[mr] = tmp;
      int ok = rperm[k], om = rperm[mr];
      rperm[k] = om;
      rperm[mr] = ok;
      rinv[b0 + ok] = mr - b0;
      rinv[b0 + om] = k - b0;
    }
    __syncwarp();
    for (int s = s0 + lane; s < ds; s += 32) lu[s] = work[P.slot_row[s]];
    const double diag = perturb(work[k], false);
    if (lane == 0) lu[ds] = diag;
    for (int q = ds + 1 + lane; q < s1; q += 32) lu[q] = work[P.slot_row[q]] / diag;
    __syncwarp();
    if (lane == 0)
      for (int t = t0; t < t1; ++t) work[b0 + rinv[b0 + P.pcol_q[t]]] = 0.0;
    for (int q = s0 + lane; q < s1; q += 32) work[P.slot_row[q]] = 0.0;
    __syncwarp();
    if (lane == 0) work[k] = 0.0;
    __syncwarp();
  }
  (void)status;
}

// The same first factorization with the working column, the block's row
// inverse and the operands of each column's updates in shared memory. The
// operations and their order are those of k_first_factor (and therefore the
// reference's); only where the operands sit differs. Per column:
//   1. A(:,k) is loaded by all lanes and lane 0 adds it into the working
//      column in CSC order;
//   2. the U entries are taken in chunks of 32, and a chunk in runs whose
//      L columns (rows and values, all of them final) fit the buffer: a run's
//      operands are copied into shared memory by cp.async, every lane issuing
//      its copies at once, and its updates then run in order out of shared
//      memory;
//   3. the threshold pivot search, the swap and the scaling follow.
// Shared layout: work[maxblk] f64, bl[cap] f64, rinv[maxblk] i32, br[cap]
// i32, kpat[kcap] i32, then the chunk table.
constexpr int kPatCap = 1024;

__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

__global__ void k_first_factor_s(DPlan P, const double* __restrict__ ax, double* lu,
                                 int* rperm, int* rinv, double tol, int maxblk, int cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* const work = reinterpret_cast<double*>(smem_raw);
  double* const bl = work + maxblk;
  int* const srinv = reinterpret_cast<int*>(bl + cap);
  int* const br = srinv + maxblk;
  int* const kpat = br + cap;
  int* const soff = kpat + kPatCap;  // [33]
  int* const sq0 = soff + 33;        // [32]
  int* const sj = sq0 + 32;          // [32]
  const int lane = threadIdx.x;
  const int n = P.n;
  for (int i = lane; i < n; i += 32) rperm[i] = i - P.block_ptr[P.pos_block[i]];
  for (int i = lane; i < maxblk; i += 32) work[i] = 0.0;
  for (int b = 0; b < P.nblocks; ++b) {
    const int b0 = P.block_ptr[b], b1 = P.block_ptr[b + 1];
    for (int i = lane; i < b1 - b0; i += 32) srinv[i] = i;
    __syncwarp();
    for (int k = b0; k < b1; ++k) {
      const int s0 = P.col_ptr[k], ds = P.dslot[k], s1 = P.col_ptr[k + 1];
      const int t0 = P.pcol_ptr[k], t1 = P.pcol_ptr[k + 1];
      if (P.col_single[k]) {
        double d = 0.0;
        for (int tc = t0; tc < t1; tc += 32) {
          const double v = tc + lane < t1 ? ax[P.pcol_raw[tc + lane]] : 0.0;
          const int cnt = min(32, t1 - tc);
          for (int i = 0; i < cnt; ++i) d += __shfl_sync(FULL, v, i);
        }
        if (lane == 0) lu[ds] = perturb(d, true);
        continue;
      }
      const bool staged = s1 - s0 <= kPatCap;
      if (staged)
        for (int s = s0 + lane; s < s1; s += 32) cp_async4(&kpat[s - s0], &P.slot_row[s]);
      // 1. A(:,k), duplicates added in CSC order
      for (int tc = t0; tc < t1; tc += 32) {
        int q = 0;
        double v = 0.0;
        if (tc + lane < t1) {
          q = P.pcol_q[tc + lane];
          v = ax[P.pcol_raw[tc + lane]];
        }
        const int cnt = min(32, t1 - tc);
        for (int i = 0; i < cnt; ++i) {
          const int qi = __shfl_sync(FULL, q, i);
          const double vi = __shfl_sync(FULL, v, i);
          if (lane == 0) work[srinv[qi]] += vi;
        }
      }
      cp_async_wait_all();
      __syncwarp();
      auto row = [&](int s) { return staged ? kpat[s - s0] : P.slot_row[s]; };
      // 2. updates by the U entries, in order
      for (int sc = s0; sc < ds; sc += 32) {
        const int cnt = min(32, ds - sc);
        int j = 0, q0 = 0, len = 0;
        if (lane < cnt) {
          j = row(sc + lane);
          q0 = P.dslot[j] + 1;
          len = P.col_ptr[j + 1] - q0;
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        soff[lane] = incl - len;
        sq0[lane] = q0;
        sj[lane] = j;
        if (lane == 31) soff[32] = total;
        __syncwarp();
        // runs of consecutive U entries whose operands fit the buffer
        for (int i0 = 0; i0 < cnt;) {
          int i1 = i0 + 1;
          while (i1 < cnt && soff[i1 + 1] - soff[i0] <= cap) ++i1;
          const int e0 = soff[i0], e1 = soff[i1];
          if (e1 - e0 <= cap) {
            int si = i0;
            for (int e = e0 + lane; e < e1; e += 32) {
              while (soff[si + 1] <= e) ++si;
              const int q = sq0[si] + (e - soff[si]);
              cp_async4(&br[e - e0], &P.slot_row[q]);
              cp_async8(&bl[e - e0], &lu[q]);
            }
            cp_async_wait_all();
            __syncwarp();
            for (int i = i0; i < i1; ++i) {
              const double u = work[sj[i] - b0];
              if (u != 0.0) {
                const int ea = soff[i] - e0, eb = soff[i + 1] - e0;
                for (int e = ea + lane; e < eb; e += 32) {
                  const int r = br[e] - b0;
                  work[r] = work[r] - bl[e] * u;
                }
              }
              __syncwarp();
            }
          } else {  // one L column longer than the buffer: straight from memory
            const double u = work[sj[i0] - b0];
            const int qa = sq0[i0], qb = qa + (e1 - e0);
            if (u != 0.0)
              for (int q = qa + lane; q < qb; q += 32) {
                const int r = P.slot_row[q] - b0;
                work[r] = work[r] - lu[q] * u;
              }
            __syncwarp();
          }
          i0 = i1;
        }
      }
      // 3. threshold pivot search inside the symbolic pattern: the first row
      // with the largest magnitude wins; the diagonal wins ties
      const double dabs = fabs(work[k - b0]);
      double best = -1.0;
      int bidx = 0x7fffffff;
      for (int q = ds + 1 + lane; q < s1; q += 32) {
        const double v = fabs(work[row(q) - b0]);
        if (v > best) {
          best = v;
          bidx = q;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_down_sync(FULL, best, off);
        const int oi = __shfl_down_sync(FULL, bidx, off);
        if (ov > best || (ov == best && oi < bidx)) {
          best = ov;
          bidx = oi;
        }
      }
      best = __shfl_sync(FULL, best, 0);
      bidx = __shfl_sync(FULL, bidx, 0);
      if (lane == 0 && bidx != 0x7fffffff && best > dabs && dabs < tol * best) {
        const int mr = row(bidx);
        const double tmp = work[k - b0];
        work[k - b0] = work[mr - b0];
        work[mr - b0] = tmp;
        const int ok = rperm[k], om = rperm[mr];
        rperm[k] = om;
        rperm[mr] = ok;
        srinv[ok] = mr - b0;
        srinv[om] = k - b0;
      }
      __syncwarp();
      for (int s = s0 + lane; s < ds; s += 32) lu[s] = work[row(s) - b0];
      const double diag = perturb(work[k - b0], false);
      if (lane == 0) lu[ds] = diag;
      for (int q = ds + 1 + lane; q < s1; q += 32) lu[q] = work[row(q) - b0] / diag;
      __syncwarp();
      for (int t = t0 + lane; t < t1; t += 32) work[srinv[P.pcol_q[t]]] = 0.0;
      for (int q = s0 + lane; q < s1; q += 32) work[row(q) - b0] = 0.0;
      __syncwarp();
      if (lane == 0) work[k - b0] = 0.0;
      __syncwarp();
    }
    for (int i = lane; i < b1 - b0; i += 32) rinv[b0 + i] = srinv[i];
    __syncwarp();
  }
}

// --------------------------------------------------------------- refactor
// A warp's column lives in shared memory while it is updated (columns of up
// to kColBuf slots; longer ones stay in memory). The U entries are taken in
// chunks of 32: one acquire per entry, all lanes at once, finds the columns
// already final; those need no further wait, and the L column of the next
// entry (its first 32 values and destinations) is loaded while the current
// one is applied. The operations and their order are the reference's.
constexpr int kColBuf = 768;

// Pivot-pass mode of the refactorization (PivotCheck): the first
// factorization's threshold rule on column k's finished values - the first L
// slot of largest magnitude takes the pivot when it beats the diagonal and
// the diagonal is below tol times it - written to want[k]; then the
// candidate's row is swapped into the pivot. get(q) / put(q, v) access the
// column by slot.
template <class Get, class Put>
__device__ __forceinline__ void pivot_check(const PivotCheck& pc, int k, int ds, int s1,
                                            bool single, Get get, Put put) {
  const int lane = threadIdx.x & 31;
  double best = -1.0;
  int bq = 0x7fffffff;
  if (!single)
    for (int q = ds + 1 + lane; q < s1; q += 32) {
      const double v = fabs(get(q));
      if (v > best) {
        best = v;
        bq = q;
      }
    }
  for (int off = 16; off > 0; off >>= 1) {
    const double ov = __shfl_down_sync(FULL, best, off);
    const int oq = __shfl_down_sync(FULL, bq, off);
    if (ov > best || (ov == best && oq < bq)) {
      best = ov;
      bq = oq;
    }
  }
  if (lane == 0) {
    const double dabs = fabs(get(ds));
    pc.want[k] = (!single && bq != 0x7fffffff && best > dabs && dabs < pc.tol * best) ? bq : -1;
    const int c = pc.cand[k];
    if (c > ds && c < s1) {
      const double t = get(ds);
      put(ds, get(c));
      put(c, t);
    }
  }
  __syncwarp();
}

__global__ void k_refactor(DPlan P, const double* __restrict__ ax, double* lu,
                           unsigned* flags, unsigned epoch, unsigned* counter,
                           int* status, PivotCheck pc) {
  extern __shared__ double scol[];
  const int lane = threadIdx.x & 31;
  double* const cbuf = scol + (threadIdx.x >> 5) * kColBuf;
  const int n = P.n;
  while (true) {
    int k = 0;
    if (lane == 0) k = (int)atomicAdd(counter, 1u);
    k = __shfl_sync(FULL, k, 0);
    if (k >= n) return;
    const int s0 = P.col_ptr[k], ds = P.dslot[k], s1 = P.col_ptr[k + 1];
    const bool staged = s1 - s0 <= kColBuf;
    double* const C = staged ? cbuf - s0 : lu;  // the column, indexed by slot
    // A(:,k) into the column's slots; duplicates summed in CSC order
    for (int s = s0 + lane; s < s1; s += 32) {
      double v = 0.0;
      for (int t = P.amap_ptr[s]; t < P.amap_ptr[s + 1]; ++t) v += ax[P.amap_idx[t]];
      C[s] = v;
    }
    __syncwarp();
    for (int sc = s0; sc < ds; sc += 32) {
      const int cnt = min(32, ds - sc);
      int jl = 0;
      bool rdy = true;
      if (lane < cnt) {
        jl = P.slot_row[sc + lane];
        rdy = ld_acquire(&flags[jl]) == epoch;
      }
      const unsigned ready = __ballot_sync(FULL, rdy);
      __syncwarp();  // orders every lane's later loads after the acquires
      int j = 0, qa = 0, qb = 0, d0 = 0;
      const int* dst = nullptr;
      double v0 = 0.0;
      auto fetch = [&](int i) {
        j = __shfl_sync(FULL, jl, i);
        qa = P.dslot[j] + 1;
        qb = P.col_ptr[j + 1];
        dst = P.upd_dst + P.upd_ptr[sc + i] - qa;
        v0 = 0.0;
        d0 = 0;
        const int q = qa + lane;
        if (q < qb && ((ready >> i) & 1u)) {
          v0 = ld_cg(&lu[q]);
          d0 = dst[q];
        }
      };
      fetch(0);
      for (int i = 0; i < cnt; ++i) {
        const int s = sc + i, cqa = qa, cqb = qb;
        const int* const cdst = dst;
        int cd0 = d0;
        double cv0 = v0;
        const int cj = j;
        if (i + 1 < cnt) fetch(i + 1);  // independent of this entry's update
        if (!((ready >> i) & 1u)) {
          int ok = 1;
          if (lane == 0) ok = wait_flag(&flags[cj], epoch, status, P.spin_limit);
          if (!__shfl_sync(FULL, ok, 0)) return;
          __syncwarp();
          const int q = cqa + lane;
          if (q < cqb) {
            cv0 = ld_cg(&lu[q]);
            cd0 = cdst[q];
          }
        }
        const double u = staged ? C[s] : ld_cg(&lu[s]);
        if (u != 0.0) {
          int q = cqa + lane;
          if (q < cqb) {
            const double c = staged ? C[cd0] : ld_cg(&lu[cd0]);
            C[cd0] = c - cv0 * u;
          }
          for (q += 32; q < cqb; q += 32) {
            const int d = cdst[q];
            const double c = staged ? C[d] : ld_cg(&lu[d]);
            C[d] = c - ld_cg(&lu[q]) * u;
          }
        }
        __syncwarp();
      }
    }
    if (pc.want != nullptr)
      pivot_check(
          pc, k, ds, s1, P.col_single[k] != 0,
          [&](int q) { return staged ? C[q] : ld_cg(&lu[q]); },
          [&](int q, double v) { C[q] = v; });
    const double diag = perturb(staged ? C[ds] : ld_cg(&lu[ds]), P.col_single[k] != 0);
    for (int q = ds + 1 + lane; q < s1; q += 32)
      lu[q] = (staged ? C[q] : ld_cg(&lu[q])) / diag;
    if (staged)
      for (int q = s0 + lane; q < ds; q += 32) lu[q] = C[q];
    if (lane == 0) lu[ds] = diag;
    __syncwarp();
    __threadfence();
    if (lane == 0) st_release(&flags[k], epoch);
  }
}

// --------------------------------------------------------------- solve
// v - sum_e coef(e) * val(dep(e)) over e in [e0, e1), subtracted in order.
// Each lane waits for and multiplies one entry of a 32-entry chunk; lane 0
// then subtracts the rounded products in order.
template <class Coef, class Dep>
__device__ __forceinline__ bool ordered_dot(double& v, int e0, int e1, Coef coef, Dep dep,
                                            const unsigned* flag, const double* val,
                                            unsigned epoch, int* status, unsigned limit) {
  const int lane = threadIdx.x & 31;
  for (int base = e0; base < e1; base += 32) {
    const int e = base + lane;
    double prod = 0.0;
    int ok = 1;
    if (e < e1) {
      const int d = dep(e);
      ok = wait_flag(&flag[d], epoch, status, limit);
      if (ok) prod = coef(e) * ld_cg(&val[d]);
    }
    if (!__all_sync(FULL, ok)) return false;
    const int cnt = min(32, e1 - base);
    for (int t = 0; t < cnt; ++t) {
      double pt = __shfl_sync(FULL, prod, t);
      v = v - pt;
    }
  }
  return true;
}

__global__ void k_solve(DPlan P, const double* __restrict__ rhs, const double* __restrict__ ax,
                        const double* __restrict__ lu, double* z, double* x, double* out,
                        unsigned* zflag, unsigned* xflag, unsigned epoch, unsigned* counter,
                        int* status) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int t = 0;
    if (lane == 0) t = (int)atomicAdd(counter, 1u);
    t = __shfl_sync(FULL, t, 0);
    if (t >= P.ntask) return;
    const int code = P.task[t];
    const int i = code >> 1;
    if ((code & 1) == 0) {  // forward: block coupling, then L
      double v = rhs[P.in_row[i]];
      bool ok = ordered_dot(
          v, P.offd_ptr[i], P.offd_ptr[i + 1], [&](int e) { return ax[P.offd_raw[e]]; },
          [&](int e) { return P.offd_col[e]; }, xflag, x, epoch, status, P.spin_limit);
      if (ok)
        ok = ordered_dot(
            v, P.lrow_ptr[i], P.lrow_ptr[i + 1], [&](int e) { return lu[P.lrow_slot[e]]; },
            [&](int e) { return P.lrow_col[e]; }, zflag, z, epoch, status, P.spin_limit);
      if (!ok) return;
      if (lane == 0) {
        z[i] = v;
        __threadfence();
        st_release(&zflag[i], epoch);
      }
    } else {  // backward: U
      int ok = 1;
      if (lane == 0) ok = wait_flag(&zflag[i], epoch, status, P.spin_limit);
      if (!__shfl_sync(FULL, ok, 0)) return;
      double v = ld_cg(&z[i]);
      ok = ordered_dot(
          v, P.urow_ptr[i], P.urow_ptr[i + 1], [&](int e) { return lu[P.urow_slot[e]]; },
          [&](int e) { return P.urow_col[e]; }, xflag, x, epoch, status, P.spin_limit);
      if (!ok) return;
      if (lane == 0) {
        v = v / lu[P.dslot[i]];
        x[i] = v;
        out[P.out_col[i]] = v;
        __threadfence();
        st_release(&xflag[i], epoch);
      }
    }
  }
}

// A^T y = g with the same factors: U^T forward (U columns as rows), then
// L^T backward (L columns as rows). Task codes as in k_solve; the input is
// indexed by original column and the output by original row.
__global__ void k_tsolve(DPlan P, const double* __restrict__ g, const double* __restrict__ ax,
                         const double* __restrict__ lu, double* z, double* x, double* out,
                         unsigned* zflag, unsigned* xflag, unsigned epoch, unsigned* counter,
                         int* status) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int t = 0;
    if (lane == 0) t = (int)atomicAdd(counter, 1u);
    t = __shfl_sync(FULL, t, 0);
    if (t >= P.ntask) return;
    const int code = P.task[t];
    const int k = code >> 1;
    if ((code & 1) == 0) {  // coupling^T, then U^T row k = U column k
      double v = g[P.out_col[k]];
      bool ok = ordered_dot(
          v, P.offdT_ptr[k], P.offdT_ptr[k + 1], [&](int e) { return ax[P.offdT_raw[e]]; },
          [&](int e) { return P.offdT_row[e]; }, xflag, x, epoch, status, P.spin_limit);
      if (ok)
        ok = ordered_dot(
            v, P.col_ptr[k], P.dslot[k], [&](int e) { return lu[e]; },
            [&](int e) { return P.slot_row[e]; }, zflag, z, epoch, status, P.spin_limit);
      if (!ok) return;
      if (lane == 0) {
        v = v / lu[P.dslot[k]];
        z[k] = v;
        __threadfence();
        st_release(&zflag[k], epoch);
      }
    } else {  // L^T row k = L column k
      int ok = 1;
      if (lane == 0) ok = wait_flag(&zflag[k], epoch, status, P.spin_limit);
      if (!__shfl_sync(FULL, ok, 0)) return;
      double v = ld_cg(&z[k]);
      ok = ordered_dot(
          v, P.dslot[k] + 1, P.col_ptr[k + 1], [&](int e) { return lu[e]; },
          [&](int e) { return P.slot_row[e]; }, xflag, x, epoch, status, P.spin_limit);
      if (!ok) return;
      if (lane == 0) {
        x[k] = v;
        out[P.in_row[k]] = v;
        __threadfence();
        st_release(&xflag[k], epoch);
      }
    }
  }
}

// --------------------------------------------------------------- one-block factor and solve
// For factorizations small enough that one SM does their arithmetic faster
// than the dependency hops of the grid-wide kernels cost, the refactor and
// the solve run in one thread block, where a hop is a shared-memory flag (or
// a warp barrier) instead of a round trip through L2.

__device__ __forceinline__ unsigned ld_acquire_cta(const unsigned* p) {
  unsigned v;
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta(unsigned* p, unsigned v) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// k_refactor in one block, with the factor itself in shared memory: the
// column code is k_refactor's (same operations, same order); the completion
// flags also live in shared memory, so a warp waiting for a column sees it
// finish within a few hundred cycles. The static metadata of the U entries is
// fetched in a pipeline - the row two entries ahead, the L range and update
// list one entry ahead, the first update destinations before the wait - so a
// step costs shared-memory latency only. All warps of the block are resident
// and a warp only waits for columns handed out before its own, so the warp
// holding the lowest unfinished column always proceeds. Shared: lu[nslots]
// f64, done[n] u32.
__global__ void __launch_bounds__(1024) k_refactor_cta(DPlan P, const double* __restrict__ ax,
                                                       double* lu_out, int* status,
                                                       PivotCheck pc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* const lu = reinterpret_cast<double*>(smem_raw);
  unsigned* const sdone = reinterpret_cast<unsigned*>(lu + P.nslots);
  __shared__ unsigned snext;
  const int lane = threadIdx.x & 31;
  const int n = P.n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sdone[i] = 0u;
  if (threadIdx.x == 0) snext = 0u;
  __syncthreads();
  bool failed = false;
  while (!failed) {
    int k = 0;
    if (lane == 0) k = (int)atomicAdd(&snext, 1u);
    k = __shfl_sync(FULL, k, 0);
    if (k >= n) break;
    const int s0 = P.col_ptr[k], ds = P.dslot[k], s1 = P.col_ptr[k + 1];
    for (int s = s0 + lane; s < s1; s += 32) {
      double v = 0.0;
      for (int t = P.amap_ptr[s]; t < P.amap_ptr[s + 1]; ++t) v += ax[P.amap_idx[t]];
      lu[s] = v;
    }
    int j0 = s0 < ds ? P.slot_row[s0] : 0;
    int j1 = s0 + 1 < ds ? P.slot_row[s0 + 1] : 0;
    int qa = 0, qb = 0, up = 0;
    if (s0 < ds) {
      qa = P.dslot[j0] + 1;
      qb = P.col_ptr[j0 + 1];
      up = P.upd_ptr[s0];
    }
    __syncwarp();
    for (int s = s0; s < ds; ++s) {
      int nqa = 0, nqb = 0, nup = 0, j2 = 0;
      if (s + 1 < ds) {
        nqa = P.dslot[j1] + 1;
        nqb = P.col_ptr[j1 + 1];
        nup = P.upd_ptr[s + 1];
      }
      if (s + 2 < ds) j2 = P.slot_row[s + 2];
      const int q = qa + lane;
      const int d0 = q < qb ? P.upd_dst[up + lane] : 0;
      int ok = 1;
      if (lane == 0) {
        unsigned spins = 0;
        while (ld_acquire_cta(&sdone[j0]) == 0u) {
          if (++spins > P.spin_limit) {
            atomicCAS(status, DS_OK, DS_TIMEOUT);
            ok = 0;
            break;
          }
          if ((spins & 63u) == 0 && *(volatile int*)status != DS_OK) {
            ok = 0;
            break;
          }
          if (spins > 256) __nanosleep(20);  // shared-memory polls first
        }
      }
      if (!__shfl_sync(FULL, ok, 0)) {
        failed = true;
        break;
      }
      const double u = lu[s];
      if (u != 0.0) {
        if (q < qb) lu[d0] = lu[d0] - lu[q] * u;
        for (int qq = q + 32; qq < qb; qq += 32) {
          const int d = P.upd_dst[up + qq - qa];
          lu[d] = lu[d] - lu[qq] * u;
        }
      }
      __syncwarp();
      j0 = j1;
      j1 = j2;
      qa = nqa;
      qb = nqb;
      up = nup;
    }
    if (failed) break;
    if (pc.want != nullptr)
      pivot_check(
          pc, k, ds, s1, P.col_single[k] != 0, [&](int q) { return lu[q]; },
          [&](int q, double v) { lu[q] = v; });
    const double diag = perturb(lu[ds], P.col_single[k] != 0);
    for (int q = ds + 1 + lane; q < s1; q += 32) lu[q] = lu[q] / diag;
    if (lane == 0) lu[ds] = diag;
    __syncwarp();
    __threadfence_block();
    if (lane == 0) st_release_cta(&sdone[k], 1u);
  }
  __syncthreads();
  for (int s = threadIdx.x; s < P.nslots; s += blockDim.x) lu_out[s] = lu[s];
}

// The solve of k_solve in one block, column by column: the forward sweep
// takes the L columns in ascending order and subtracts l(r,j) x(j) from each
// row r below, the backward sweep the U columns in descending order, so every
// row receives its terms in the order of its row lists (L ascending, U
// descending) - the reference's order - and the results are those of k_solve
// bit for bit. The block coupling of a BTF block is subtracted, row by row in
// its list order, before the block's first column.
//
// Warp 0 does the arithmetic; the other warps copy the factor's slots (rows
// and values) chunk by chunk into a double buffer ahead of it. The host cuts
// the sweeps into chunks of contiguous slots (CtaSolve in capi.cu):
//   chunk c: cs_chunk[4c..4c+3] = slot_lo, slot_hi, op_lo, op_hi
//   op o:    cs_op[3o..3o+2]    = kind | direct << 2, a, b
// kind 0: coupling of rows [a, b); 1: forward over columns [a, b); 2:
// backward over columns [a, b); direct: a column larger than a chunk, read
// from memory. Shared: w[n] f64, 2 x chunk values f64, then (i32) 2 x chunk
// rows, col_ptr[n+1], dslot[n], offd_ptr[n+1] (when there is coupling).
//
// With grouped != 0 the block is one of P.cs_ngrp: it solves rows [r0, r1)
// (whole uncoupled BTF blocks) with its own chunk range; the shared arrays
// then cover only those rows and are indexed by position - r0.
__global__ void __launch_bounds__(256) k_solve_cta(DPlan P, const double* __restrict__ rhs,
                                                   const double* __restrict__ ax,
                                                   const double* __restrict__ lu, double* out,
                                                   int chunk, int grouped) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31;
  int r0 = 0, r1 = P.n, c0 = 0, c1 = P.cs_nchunk;
  const int *CH = P.cs_chunk, *OP = P.cs_op;
  if (grouped) {
    const int* g = P.cs_grp + 4 * blockIdx.x;
    r0 = g[0];
    r1 = g[1];
    c0 = g[2];
    c1 = g[3];
    CH = P.cs_gchunk;
    OP = P.cs_gop;
  }
  const int m = r1 - r0;
  const bool coupled = P.noffd > 0;
  double* const w = reinterpret_cast<double*>(smem_raw);
  double* const bval = w + m;
  int* const brow = reinterpret_cast<int*>(bval + 2 * chunk);
  int* const scp = brow + 2 * chunk;
  int* const sds = scp + m + 1;
  int* const sop = sds + m;
  for (int i = tid; i <= m; i += blockDim.x) {
    cp_async4(&scp[i], &P.col_ptr[r0 + i]);
    if (i < m) cp_async4(&sds[i], &P.dslot[r0 + i]);
    if (coupled) cp_async4(&sop[i], &P.offd_ptr[r0 + i]);
  }
  for (int i = tid; i < m; i += blockDim.x) w[i] = rhs[P.in_row[r0 + i]];
  cp_async_wait_all();
  const int nprod = blockDim.x - 32;
  auto load = [&](int c) {
    const int lo = CH[4 * c], hi = CH[4 * c + 1];
    double* const bv = bval + (c & 1) * chunk;
    int* const br = brow + (c & 1) * chunk;
    for (int s = lo + tid - 32; s < hi; s += nprod) {  // all copies in flight at once
      cp_async8(&bv[s - lo], &lu[s]);
      cp_async4(&br[s - lo], &P.slot_row[s]);
    }
    cp_async_wait_all();
  };
  if (tid >= 32 && c1 > c0) load(c0);
  __syncthreads();
  for (int c = c0; c < c1; ++c) {
    if (tid >= 32) {
      if (c + 1 < c1) load(c + 1);
    } else {
      const int lo = CH[4 * c], o0 = CH[4 * c + 2], o1 = CH[4 * c + 3];
      const double* const bv = bval + (c & 1) * chunk - lo;  // indexed by slot
      const int* const br = brow + (c & 1) * chunk - lo;
      for (int o = o0; o < o1; ++o) {
        const int code = OP[3 * o], a = OP[3 * o + 1] - r0, b = OP[3 * o + 2] - r0;
        // forward: L columns ascending. The next column's range is read, and
        // this column's first rows and values are loaded, before the value
        // of x(j) is: only the subtraction waits for the previous column.
        auto fwd = [&](const auto* V, const auto* R) {
          int q0 = sds[a] + 1, q1 = scp[a + 1];
          for (int j = a; j < b; ++j) {
            const int cq0 = q0, cq1 = q1;
            if (j + 1 < b) {
              q0 = sds[j + 1] + 1;
              q1 = scp[j + 2];
            }
            const int q = cq0 + lane;
            int r = 0;
            double v = 0.0;
            if (q < cq1) {
              r = R[q] - r0;
              v = V[q];
            }
            const double xj = w[j];
            if (q < cq1) w[r] = w[r] - v * xj;
            for (int qq = q + 32; qq < cq1; qq += 32) {
              const int rr = R[qq] - r0;
              w[rr] = w[rr] - V[qq] * xj;
            }
            __syncwarp();
          }
        };
        // backward: U columns descending
        auto bwd = [&](const auto* V, const auto* R) {
          for (int j = b - 1; j >= a; --j) {
            const int ds = sds[j], q = scp[j] + lane;
            int r = 0;
            double v = 0.0;
            if (q < ds) {
              r = R[q] - r0;
              v = V[q];
            }
            const double xj = w[j] / V[ds];
            if (q < ds) w[r] = w[r] - v * xj;
            for (int qq = q + 32; qq < ds; qq += 32) {
              const int rr = R[qq] - r0;
              w[rr] = w[rr] - V[qq] * xj;
            }
            __syncwarp();
            if (lane == 0) w[j] = xj;
          }
        };
        // separate instantiations keep the buffered sweeps on shared-memory
        // loads (a pointer that may be either space would make them generic)
        if ((code & 3) == 0) {  // coupling to the blocks solved before
          for (int i = a + lane; i < b; i += 32) {
            double v = w[i];
            for (int e = sop[i]; e < sop[i + 1]; ++e)
              v = v - ax[P.offd_raw[e]] * w[P.offd_col[e] - r0];
            w[i] = v;
          }
        } else if ((code & 3) == 1) {
          if (code & 4)
            fwd(lu, P.slot_row);
          else
            fwd(bv, br);
        } else {
          if (code & 4)
            bwd(lu, P.slot_row);
          else
            bwd(bv, br);
        }
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < m; i += blockDim.x) out[P.out_col[r0 + i]] = w[i];
}

// a / b correctly rounded, from y = 1/b correctly rounded, by Markstein's
// correction (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = a y is
// within an ulp of a / b, the residual r = a - b q is exact in one fma, and
// q + r y rounded to nearest is the correctly rounded quotient. Three
// dependent FP64 operations instead of a division's sequence. Operands or a
// quotient near the ends of the exponent range (zeros, subnormals,
// infinities, NaN included) take the division itself; the exponent tests are
// integer operations.
__device__ __forceinline__ double div_markstein(double a, double b, double y) {
  const double q = a * y;
  const unsigned ea = (unsigned)(__double_as_longlong(a) >> 52) & 0x7ffu;
  const unsigned eb = (unsigned)(__double_as_longlong(b) >> 52) & 0x7ffu;
  const unsigned eq = (unsigned)(__double_as_longlong(q) >> 52) & 0x7ffu;
  if (ea - 64u > 1919u || eb - 64u > 1919u || eq - 64u > 1919u) return a / b;
  const double r = fma(-b, q, a);
  return fma(r, y, q);
}

// The solve as a step program, one thread block: the solution vector in
// shared memory, the pivots' reciprocals computed first (n divisions in
// parallel), then step by step the operations the column sweeps perform, in
// the reference's order for every row (each row's updates separately rounded
// products and differences, the pivot division exact), the operations of a
// step spread over the block's threads. A step's operation, its matrix value
// and (for a division) its reciprocal are loaded two steps ahead: none of
// them depends on the solution.
constexpr int kSolveStepsThreads = 128;

struct SolveOp {
  int4 o;
  double v, y;
};

__global__ void __launch_bounds__(kSolveStepsThreads)
    k_solve_steps(DPlan P, const double* __restrict__ rhs, const double* __restrict__ ax,
                  const double* __restrict__ lu, double* rec, double* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* const T = reinterpret_cast<double*>(smem_raw);
  const int tid = threadIdx.x, n = P.n;
  for (int i = tid; i < n; i += blockDim.x) {
    T[i] = rhs[P.in_row[i]];
    rec[i] = 1.0 / lu[P.dslot[i]];
  }
  __syncthreads();
  const int4* const ops = P.ss_ops;
  const int* const sp = P.ss_ptr;
  const int ns = P.ss_nsteps;
  const int nops = sp[ns];
  auto fetch = [&](int p) {
    SolveOp f;
    f.o = make_int4(0, -1, 0, 3);
    f.v = 0.0;
    f.y = 0.0;
    if (p < nops) {
      f.o = __ldg(ops + p);
      f.v = f.o.w == 2 ? __ldg(ax + f.o.z) : __ldg(lu + f.o.z);
      if (f.o.w == 1) f.y = __ldcg(rec + f.o.x);  // written above by this block
    }
    return f;
  };
  auto exec = [&](const SolveOp& f) {
    const int d = f.o.x;
    if (f.o.w == 1)
      T[d] = div_markstein(T[d], f.v, f.y);
    else if (f.o.w != 3)
      T[d] = __dsub_rn(T[d], __dmul_rn(f.v, T[f.o.y]));
  };
  int s0 = sp[0], s1 = ns >= 1 ? sp[1] : s0, s2 = ns >= 2 ? sp[2] : s1, s3 = ns >= 3 ? sp[3] : s2;
  SolveOp f0 = fetch(s0 + tid), f1 = fetch(s1 + tid);
  for (int t = 0; t < ns; ++t) {
    const SolveOp f2 = fetch(s2 + tid);
    const int s4 = t + 4 <= ns ? sp[t + 4] : s3;
    if (s0 + tid < s1) exec(f0);
    for (int p = s0 + tid + kSolveStepsThreads; p < s1; p += kSolveStepsThreads) exec(fetch(p));
    __syncthreads();
    s0 = s1;
    s1 = s2;
    s2 = s3;
    s3 = s4;
    f0 = f1;
    f1 = f2;
  }
  for (int i = tid; i < n; i += blockDim.x) out[P.out_col[i]] = T[i];
}

// --------------------------------------------------------------- devices
// Level-1 MOSFET exactly as the reference evaluates it
// (crates/sim-devices/src/bsim/evaluate.rs:285-356 via mod.rs:440-455).
__device__ void mos_reference(const double* p, double vd, double vg, double vs, double& gm,
                              double& gds, double& ieq) {
  const double lambda = 0.02, gmin_dev = 1e-12;
  const bool pm = p[0] != 0.0;
  const double beta = p[2] * 1e-4 * ((3.9 * 8.854e-12) / p[3]);
  double vdi = pm ? -vs : vd, vgi = pm ? -vg : vg, vsi = pm ? -vd : vs;
  double vgs = vgi - vsi, vds = vdi - vsi;
  if (vds < 0.0) {
    vds = -vds;
    vgs = vgi - vdi;
  }
  const double vth = pm ? -fabs(p[1]) : fabs(p[1]);
  const double beff = beta * p[4] / p[5];
  double ids;
  if (vgs <= vth) {
    ids = 0.0;
    gm = 0.0;
    gds = gmin_dev;
  } else if (vds < vgs - vth) {
    ids = beff * ((vgs - vth) * vds - 0.5 * vds * vds);
    gm = beff * vds;
    gds = fmax(beff * ((vgs - vth) - vds), gmin_dev);
  } else {
    const double t = vgs - vth;
    ids = 0.5 * beff * (t * t) * (1.0 + lambda * vds);
    gm = beff * (vgs - vth) * (1.0 + lambda * vds);
    gds = fmax(0.5 * beff * (t * t) * lambda, gmin_dev);
  }
  const double ids_s = pm ? -ids : ids;
  ieq = ids_s - gm * (vg - vs) - gds * (vd - vs);
}

// Level-1 MOSFET in the Shichman-Hodges form (the (1 + lambda vds) factor in
// both regions, so the current is continuous where they meet) with a
// self-consistent linearisation: drain current and its partials with respect
// to (vg, vd, vs).
__device__ void mos_consistent(const double* p, double vd, double vg, double vs, double& id,
                               double& ddg, double& ddd, double& dds, double gmin_dev) {
  const double lambda = 0.02;
  const double pol = p[0] != 0.0 ? -1.0 : 1.0;
  const double beta = p[2] * 1e-4 * ((3.9 * 8.854e-12) / p[3]);
  const double vgs = pol * (vg - vs), vds = pol * (vd - vs);
  const bool rev = vds < 0.0;
  const double vgse = rev ? vgs - vds : vgs, vdse = rev ? -vds : vds;
  const double vth = fabs(p[1]);
  const double beff = beta * p[4] / p[5];
  double ids, gm, gds;
  if (vgse <= vth) {
    ids = 0.0;
    gm = 0.0;
    gds = gmin_dev;
  } else if (vdse < vgse - vth) {  // Shichman-Hodges: (1 + lambda vds) here too
    const double k = 1.0 + lambda * vdse;
    const double q = (vgse - vth) * vdse - 0.5 * vdse * vdse;
    ids = beff * q * k;
    gm = beff * vdse * k;
    gds = fmax(beff * ((vgse - vth) - vdse) * k + lambda * beff * q, gmin_dev);
  } else {
    const double t = vgse - vth;
    ids = 0.5 * beff * (t * t) * (1.0 + lambda * vdse);
    gm = beff * (vgse - vth) * (1.0 + lambda * vdse);
    gds = fmax(0.5 * beff * (t * t) * lambda, gmin_dev);
  }
  if (!rev) {
    id = pol * ids;
    ddg = gm;
    ddd = gds;
    dds = -(gm + gds);
  } else {
    id = -pol * ids;
    ddg = -gm;
    ddd = gm + gds;
    dds = -gds;
  }
}

// One device's matrix inserts (in the reference's insert order) and its
// right-hand-side contributions. Returns the number of matrix values.
// gdev is the level-1 conductance floor of the consistent model: 1e-12 as
// the reference's evaluator uses, or 0 for the exact Jacobian of the
// residual (the floor cancels in the residual but not in the matrix).
template <class XGet>
__device__ __forceinline__ int eval_device(int type, const int* nd, const double* p, XGet xg,
                                           double gmin, double scale, double dt, double vprev,
                                           double be_sign, double* m, double* r, int& nr,
                                           double gdev = 1e-12) {
  nr = 0;
  switch (type) {
    case 0: {  // R
      const double g = 1.0 / p[0];
      m[0] = g;
      m[1] = g;
      m[2] = -g;
      m[3] = -g;
      return 4;
    }
    case 1: {  // V
      m[0] = 1.0;
      m[1] = -1.0;
      m[2] = 1.0;
      m[3] = -1.0;
      r[0] = p[0] * scale;
      nr = 1;
      return 4;
    }
    case 2: {  // I
      const double v = p[0] * scale;
      r[0] = -v;
      r[1] = v;
      nr = 2;
      return 0;
    }
    case 3: {  // D, crates/sim-core/src/stamp.rs:351-387
      const double gf = gmin > 0.0 ? gmin : 1e-12;
      const double vt = 0.02585 * p[1];
      const double vd = xg(nd[0]) - xg(nd[1]);
      const double e = exp(vd / vt);
      const double id = p[0] * (e - 1.0);
      const double gd = (p[0] / vt) * e;
      const double g = fmax(gd, gf);
      const double ieq = id - gd * vd;
      m[0] = g;
      m[1] = g;
      m[2] = -g;
      m[3] = -g;
      r[0] = -ieq;
      r[1] = ieq;
      nr = 2;
      return 4;
    }
    case 4: {  // M, crates/sim-core/src/stamp.rs:511-545
      const double gf = gmin > 0.0 ? gmin : 1e-12;
      double gm, gds, ieq;
      mos_reference(p, xg(nd[0]), xg(nd[1]), xg(nd[2]), gm, gds, ieq);
      gds = fmax(gds, gf);
      m[0] = gds;
      m[1] = gds;
      m[2] = -gds;
      m[3] = -gds;
      m[4] = gm;
      m[5] = -gm;
      m[6] = -gm;
      m[7] = gm;
      r[0] = -ieq;
      r[1] = ieq;
      nr = 2;
      return 8;
    }
    case 6: {  // MC: same 8 inserts, exact partials
      const double vd = xg(nd[0]), vg = xg(nd[1]), vs = xg(nd[2]);
      double id, ddg, ddd, dds;
      mos_consistent(p, vd, vg, vs, id, ddg, ddd, dds, gdev);
      const double ieq = id - (ddg * vg + ddd * vd + dds * vs);
      m[0] = ddd;
      m[1] = -dds;
      m[2] = dds;
      m[3] = -ddd;
      m[4] = ddg;
      m[5] = 0.0;
      m[6] = -ddg;
      m[7] = 0.0;
      r[0] = -ieq;
      r[1] = ieq;
      nr = 2;
      return 8;
    }
    case 5: {  // C: backward Euler companion in transient, open in DC
      if (dt <= 0.0) return 0;
      const double g = p[0] / dt;
      const double ieq = g * vprev;
      m[0] = g;
      m[1] = g;
      m[2] = -g;
      m[3] = -g;
      r[0] = be_sign * ieq;
      r[1] = -be_sign * ieq;
      nr = 2;
      return 4;
    }
  }
  return 0;
}

__global__ void k_stamp(DCircuit C, const double* __restrict__ x, int xlen, double gmin,
                        double scale, double dt, const double* __restrict__ cap_v,
                        double be_sign, double* ax, double* rhs_c, double gdev) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d == 0 && C.pin_raw >= 0) ax[C.pin_raw] = 1.0;
  if (d >= C.ndev) return;
  const int* nd = C.nodes + 4 * d;
  auto xg = [&](int i) { return (i >= 0 && i < xlen) ? x[i] : 0.0; };
  double m[8], r[2];
  int nr;
  const double vprev = cap_v ? cap_v[d] : 0.0;
  const int nm = eval_device(C.type[d], nd, C.p + 6 * d, xg, gmin, scale, dt, vprev, be_sign,
                             m, r, nr, gdev);
  const int* raw = C.raw + 8 * d;
  for (int e = 0; e < nm; ++e)
    if (raw[e] >= 0) ax[raw[e]] = m[e];
  const int* rs = C.rhs_slot + 2 * d;
  for (int e = 0; e < nr; ++e)
    if (rs[e] >= 0) rhs_c[rs[e]] = r[e];
}

// dL/dp of every device at a DC solution x, given the adjoint lambda
// (A^T lambda = dL/dx): dL/dp = -lambda^T dF/dp with F(x, p) = A(x) x - b(x)
// the stamped KCL residual. p is the resistance for R, the value for V and
// I, Is for D, and VTO for the MOSFETs (threshold |VTO| for both models).
__global__ void k_param_grad(DCircuit C, const double* __restrict__ x, int xlen,
                             const double* __restrict__ lam, double* grad) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= C.ndev) return;
  const int* nd = C.nodes + 4 * d;
  const double* p = C.p + 6 * d;
  auto xg = [&](int i) { return (i >= 0 && i < xlen) ? x[i] : 0.0; };
  auto lg = [&](int i) { return (i >= 0 && i < C.n) ? lam[i] : 0.0; };
  double gr = 0.0;
  switch (C.type[d]) {
    case 0: {  // F_a += (va - vb)/R
      const double v = xg(nd[0]) - xg(nd[1]);
      gr = (lg(nd[0]) - lg(nd[1])) * v / (p[0] * p[0]);
      break;
    }
    case 1:  // aux row: va - vb - V
      gr = lg(nd[2]);
      break;
    case 2:  // F_a += I, F_b -= I
      gr = -(lg(nd[0]) - lg(nd[1]));
      break;
    case 3: {  // F_a += Is (exp(vd/vt) - 1)
      const double vt = 0.02585 * p[1];
      const double e = exp((xg(nd[0]) - xg(nd[1])) / vt);
      gr = -(lg(nd[0]) - lg(nd[1])) * (e - 1.0);
      break;
    }
    case 4:
    case 6: {  // F_d += id, F_s -= id; d id / d vth = -(frame sign) * gm
      const bool pm = p[0] != 0.0;
      const double vd = xg(nd[0]), vg = xg(nd[1]), vs = xg(nd[2]);
      const double beff = p[2] * 1e-4 * ((3.9 * 8.854e-12) / p[3]) * p[4] / p[5];
      double vgs, vds, vth, sgn;
      if (C.type[d] == 6) {
        const double pol = pm ? -1.0 : 1.0;
        vgs = pol * (vg - vs);
        vds = pol * (vd - vs);
        const bool rev = vds < 0.0;
        if (rev) {
          vgs = vgs - vds;
          vds = -vds;
        }
        vth = fabs(p[1]);
        sgn = rev ? -pol : pol;
      } else {  // the reference's frame (evaluate.rs:299-316)
        double vdi = pm ? -vs : vd, vgi = pm ? -vg : vg, vsi = pm ? -vd : vs;
        vgs = vgi - vsi;
        vds = vdi - vsi;
        if (vds < 0.0) {
          vds = -vds;
          vgs = vgi - vdi;
        }
        vth = pm ? -fabs(p[1]) : fabs(p[1]);
        sgn = pm ? -1.0 : 1.0;
      }
      double gm = 0.0;
      if (vgs > vth)
        gm = vds < vgs - vth ? beff * vds * (C.type[d] == 6 ? 1.0 + 0.02 * vds : 1.0)
                             : beff * (vgs - vth) * (1.0 + 0.02 * vds);
      // dvth/dVTO: |VTO| -> sign(VTO); the reference's PMOS uses -|VTO|
      double dvth = p[1] >= 0.0 ? 1.0 : -1.0;
      if (C.type[d] == 4 && pm) dvth = -dvth;
      const double did = sgn * (-gm) * dvth;
      gr = -(lg(nd[0]) - lg(nd[2])) * did;
      break;
    }
    default:
      break;
  }
  grad[d] = gr;
}

__global__ void k_rhs_sum(DCircuit C, const double* __restrict__ rhs_c, double* rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C.n) return;
  double v = 0.0;
  for (int t = C.rhs_ptr[i]; t < C.rhs_ptr[i + 1]; ++t) v += rhs_c[C.rhs_src[t]];
  rhs[i] = v;
}

// --------------------------------------------------------------- Newton
__global__ void k_newton_update(int m, int n, double* x, const double* __restrict__ xn,
                                NewtonState* st, NewtonCfg cfg, int* status) {
  __shared__ double ssum[32];
  __shared__ int sconv[32], sfin[32];
  const int tid = threadIdx.x;
  double acc = 0.0;
  int conv = 1, fin = 1;
  for (int i = tid; i < m; i += blockDim.x) {
    const double a = xn[i], dx = a - x[i];
    acc += dx * dx;
    if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = 0;
    if (!isfinite(a)) fin = 0;
  }
  for (int off = 16; off > 0; off >>= 1) {
    acc += __shfl_down_sync(FULL, acc, off);
    conv &= __shfl_down_sync(FULL, conv, off);
    fin &= __shfl_down_sync(FULL, fin, off);
  }
  if ((tid & 31) == 0) {
    ssum[tid >> 5] = acc;
    sconv[tid >> 5] = conv;
    sfin[tid >> 5] = fin;
  }
  __syncthreads();
  if (tid < 32) {
    const int nw = blockDim.x >> 5;
    acc = tid < nw ? ssum[tid] : 0.0;
    conv = tid < nw ? sconv[tid] : 1;
    fin = tid < nw ? sfin[tid] : 1;
    for (int off = 16; off > 0; off >>= 1) {
      acc += __shfl_down_sync(FULL, acc, off);
      conv &= __shfl_down_sync(FULL, conv, off);
      fin &= __shfl_down_sync(FULL, fin, off);
    }
    if (tid == 0) {
      const double dxn = sqrt(acc);
      st->iter += 1;
      st->converged = conv;
      if (!fin) atomicCAS(status, DS_OK, DS_NONFINITE);
      if (!conv) {
        if (dxn > st->prev_dx_norm && st->damping > cfg.damping_min)
          st->damping = fmax(st->damping * 0.5, cfg.damping_min);
        st->prev_dx_norm = dxn;
      }
      ssum[0] = st->damping;
      sconv[0] = conv;
    }
  }
  __syncthreads();
  const double damp = ssum[0];
  if (sconv[0]) {
    for (int i = tid; i < n; i += blockDim.x) x[i] = xn[i];
  } else {
    for (int i = tid; i < m; i += blockDim.x) x[i] = x[i] + damp * (xn[i] - x[i]);
  }
}

// FP64 pipe throughput probe: every thread runs 8 independent chains of
// fused multiply-adds (explicit fma, 2 flops each); the result is stored so
// the work cannot be removed.
__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = threadIdx.x * 1e-7 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += v[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_rcond(DPlan P, const double* __restrict__ lu, double* out) {
  __shared__ double smin[32], smax[32];
  const int tid = threadIdx.x;
  double mn = 1.7976931348623157e308, mx = 0.0;
  for (int k = tid; k < P.n; k += blockDim.x) {
    const double a = fabs(lu[P.dslot[k]]);
    mn = fmin(mn, a);
    mx = fmax(mx, a);
  }
  for (int off = 16; off > 0; off >>= 1) {
    mn = fmin(mn, __shfl_down_sync(FULL, mn, off));
    mx = fmax(mx, __shfl_down_sync(FULL, mx, off));
  }
  if ((tid & 31) == 0) {
    smin[tid >> 5] = mn;
    smax[tid >> 5] = mx;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mn = fmin(mn, smin[w]);
      mx = fmax(mx, smax[w]);
    }
    out[0] = fmin(mn, smin[0]);
    out[1] = fmax(mx, smax[0]);
  }
}

// Pivot growth after a refactorization with kept pivots: one thread per
// column scans its multipliers (L slots after the pivot); a block with one
// above lim - the kept pivot is below 1/lim of the largest entry under it,
// the rule the first factorization swaps on - is marked.
__global__ void k_growth(DPlan P, const double* __restrict__ lu, double lim, int* grow) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n) return;
  const int s1 = P.col_ptr[k + 1];
  for (int s = P.dslot[k] + 1; s < s1; ++s)
    if (!(fabs(lu[s]) <= lim)) {
      grow[P.pos_block[k]] = 1;
      return;
    }
}

// --------------------------------------------------------------- batched
// One warp owns M instances of one circuit program at a time and keeps all
// of their state in shared memory (batch_common.cuh); each Newton iteration
// touches global memory only for the program and the circuit constants.
//   stamp     - lanes evaluate devices (strided) into their value records
//   assemble  - lanes sum each LU slot's and each rhs row's contributions in
//               stamping order (bit-identical to the reference's scatter)
//   factor    - left-looking, column by column; a column's U entries in
//               order, each applying L(:,j) across lanes; the forward
//               substitution of the right-hand side is fused in
//   backward  - U sweep, lanes over a column's U entries
//   update    - convergence test, damping and iterate update
// M instances per warp, 32/M lanes each; the M instances run the same
// program (one group), so the warp's control flow is shared and every FP64
// warp instruction of the sequential factor and solve serves M instances.
// SHARED: the warps of a block work on one group at a time and share one
// staged program (more instances per SM when the program is large); the
// block moves to its next tile when every warp has run out of instances.
// The block's shared memory is carved per group: as many warps as the
// group's own program and instance regions fit take instances, the others
// sit the tile out, so groups smaller than the largest of their class keep
// more instances resident.
template <int M, bool SHARED>
__global__ void k_batch_newton(BatchArgs A) {
  constexpr int LPI = 32 / M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LPI, sl = lane % LPI, lead = sub * LPI;
  const unsigned leaders =
      M == 1 ? 1u : (M == 2 ? 0x00010001u : (M == 4 ? 0x01010101u : 0x11111111u));
  // per-warp slice (the staged program, then M instance regions), or one
  // program for the block followed by every warp's regions
  unsigned char* const slice =
      SHARED ? smem_raw
             : smem_raw + (size_t)warp * ((size_t)A.prog_ints * 4 + (size_t)M * A.region * 8);
  int* const prog = reinterpret_cast<int*>(slice);
  const NewtonCfg cfg = A.cfg;
  const double gstart = fmax(cfg.gmin * 1e3, 1e-6);
  while (true) {
    int ti = 0;
    if (SHARED) {
      // a continuation tile whose group has no parked instance left is
      // skipped before its program is staged: most groups park none
      if (threadIdx.x == 0) {
        int t = (int)atomicAdd(A.counter, 1u);
        while (A.cont_mode && t < A.ntiles) {
          const int gg = A.tile_group[t];
          if (*(volatile unsigned*)&A.gnext2[gg] < *(volatile unsigned*)&A.cont_count[gg])
            break;
          t = (int)atomicAdd(A.counter, 1u);
        }
        s_tile = t;
      }
      __syncthreads();
      ti = s_tile;
    } else {
      if (lane == 0) ti = (int)atomicAdd(A.counter, 1u);
      ti = __shfl_sync(FULL, ti, 0);
    }
    if (ti >= A.ntiles) return;
    const int g = A.tile_group[ti];
    const GroupHdr G = A.groups[g];
    const int pg = SHARED ? G.prog : A.prog_ints;
    const int rg = SHARED ? G.region : A.region;
    const int active =
        SHARED ? min((int)(blockDim.x >> 5), (A.shared_bytes - pg * 4) / (rg * 8 * M)) : 1;
    double* const region = reinterpret_cast<double*>(slice + (size_t)pg * 4) +
                           (size_t)((SHARED ? warp * M : 0) + sub) * rg;
    bt::Prog P = SHARED ? bt::stage_program(A, G, prog, threadIdx.x, blockDim.x, true, true)
                        : bt::stage_program(A, G, prog, lane, 32, false, true);
    const int n = P.n, nc = P.nc;
    // region: X[nc] T[n] V[nslots + noffd] DV[ndv], then the row -> slot map
    // (the step program addresses X, T and V from the region's start)
    double* const X = region;
    double* const T = X + nc;
    double* const V = T + n;
    double* const DV = V + G.nslots + G.noffd;
    P.map = reinterpret_cast<int*>(DV + G.ndv);

    int inst = -1, it = 0, total = 0, gstep = 0, ov_dev = -1;
    bool exhausted = warp >= active;  // no room for this warp's instances in this group
    double damp = 0.0, prev = 0.0, gmin = 0.0, ov_val = 0.0;
    const double* dparams = nullptr;
    while (true) {
      // ---- idle sub-groups take the group's next instances (one atomic per warp)
      const bool need = inst < 0 && !exhausted;
      const unsigned want = __ballot_sync(FULL, need) & leaders;
      if (want) {
        const int first_lane = __ffs(want) - 1;
        unsigned* const ctr = A.cont_mode ? &A.gnext2[g] : &A.gnext[g];
        int base = 0;
        if (lane == first_lane) base = (int)atomicAdd(ctr, (unsigned)__popc(want));
        base = __shfl_sync(FULL, base, first_lane);
        if (need) {
          const int k = base + __popc(want & ((1u << lead) - 1));
          const int count = A.cont_mode ? (int)A.cont_count[g] : G.inst_count;
          if (k < count) {
            inst = A.cont_mode ? A.cont_list[G.inst_begin + k] : A.order[G.inst_begin + k];
            dparams = A.dparams + A.inst_p_off[inst];
            ov_dev = A.inst_ov_dev[inst];
            ov_val = A.inst_ov_val[inst];
            if (A.cont_mode) {  // resume where the lane phase parked it
              const long long xo = A.inst_x_off[inst];
              for (int i = sl; i < nc; i += LPI) X[i] = A.x_out[xo + i];
              it = A.cont_it[inst];
              total = A.cont_total[inst];
              gstep = A.cont_gstep[inst];
              damp = A.cont_damp[inst];
              prev = A.cont_prev[inst];
              gmin = cfg.gmin_steps == 0
                         ? cfg.gmin
                         : gstart + (cfg.gmin - gstart) * ((double)gstep / (double)cfg.gmin_steps);
            } else {
              const long long xo = A.inst_x0_off[inst];
              for (int i = sl; i < nc; i += LPI) X[i] = xo >= 0 ? A.x0[xo + i] : 0.0;
              it = total = gstep = 0;
              damp = cfg.damping;
              prev = 1.7976931348623157e308;
              gmin = cfg.gmin_steps == 0 ? cfg.gmin : gstart;
            }
          } else {
            exhausted = true;
          }
        }
      }
      if (!__any_sync(FULL, inst >= 0)) break;
      __syncwarp();
      const bool live = inst >= 0;
      if (live) bt::stamp_devices<LPI>(P, dparams, ov_dev, ov_val, X, X, gmin, 1e-12, false, DV, sl);
      __syncwarp();
      bt::assemble<LPI>(P, DV, V, T, sl);
      __syncwarp();
      if (P.nsteps > 0)
        bt::run_steps<LPI>(P, X, sl);
      else
        bt::factor_solve<LPI>(P, V, T, sl);
      // ---- Newton update (crates/sim-core/src/newton.rs:93-107)
      bool conv = true, fin = true;
      for (int c = sl; c < nc; c += LPI) {
        const double a = T[P.out_pos[c]];
        const double dx = a - X[c];
        DV[c] = dx * dx;
        if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
        if (!isfinite(a)) fin = false;
      }
      const unsigned smask = (LPI == 32 ? FULL : (((1u << LPI) - 1u) << lead));
      const unsigned nconv = __ballot_sync(FULL, !conv) & smask;
      const unsigned nfin = __ballot_sync(FULL, !fin) & smask;
      __syncwarp();
      if (live) {
        ++it;
        ++total;
        int rsn = -1;
        if (!nconv) {
          rsn = 0;
          const long long xo = A.inst_x_off[inst];
          if (xo >= 0)
            for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = T[P.out_pos[c]];
        } else {
          double ss = 0.0;  // norm2 of dx, reduced across the instance's lanes
          for (int c = sl; c < nc; c += LPI) ss += DV[c];
#pragma unroll
          for (int o = LPI / 2; o > 0; o >>= 1) ss += __shfl_xor_sync(smask, ss, o);
          const double dxn = sqrt(ss);
          if (dxn > prev && damp > cfg.damping_min) damp = fmax(damp * 0.5, cfg.damping_min);
          prev = dxn;
          for (int c = sl; c < nc; c += LPI) X[c] = fma(damp, T[P.out_pos[c]] - X[c], X[c]);
          if (nfin) {
            rsn = 1;
          } else if (it >= cfg.max_iters) {
            if (gstep < cfg.gmin_steps) {  // next gmin step, fresh damping state
              ++gstep;
              gmin = gstart + (cfg.gmin - gstart) * ((double)gstep / (double)cfg.gmin_steps);
              it = 0;
              damp = cfg.damping;
              prev = 1.7976931348623157e308;
            } else {
              rsn = 1;
            }
          }
          if (rsn == 1) {
            const long long xo = A.inst_x_off[inst];
            if (xo >= 0)
              for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = c < nc ? X[c] : 0.0;
          }
        }
        if (rsn >= 0) {
          if (sl == 0) {  // non-finite: the reference's run ends at the cap
            A.iters[inst] = (rsn == 1 && nfin) ? cfg.max_iters : it;
            A.iters_total[inst] = total;
            A.reason[inst] = rsn;
          }
          inst = -1;
        }
      }
      __syncwarp();
    }
    if (SHARED)
      __syncthreads();  // every warp is done with the block's staged program
    else
      __syncwarp();  // done with this group's staged program
  }
}

}  // namespace

// ------------------------------------------------------------------ launches
void launch_first_factor(const DPlan& P, int maxblk, const double* ax, double* lu,
                         double* work, int* rperm, int* rinv, double tol, int* status,
                         cudaStream_t s) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t fixed = (size_t)12 * maxblk + 4 * (size_t)(kPatCap + 33 + 32 + 32) + 16;
  int cap = 4096;
  while (cap > 256 && fixed + (size_t)12 * cap > (size_t)optin) cap >>= 1;
  const size_t bytes = fixed + (size_t)12 * cap;
  if (maxblk > 0 && bytes <= (size_t)optin) {
    cudaFuncSetAttribute(k_first_factor_s, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
    k_first_factor_s<<<1, 32, bytes, s>>>(P, ax, lu, rperm, rinv, tol, maxblk, cap);
    return;
  }
  k_first_factor<<<1, 32, 0, s>>>(P, ax, lu, work, rperm, rinv, tol, status);
}

void launch_refactor(const DPlan& P, const double* ax, double* lu, unsigned* flags,
                     unsigned epoch, unsigned* counter, int* status, int grid,
                     cudaStream_t s, const PivotCheck& pc) {
  cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
  k_refactor<<<grid, 128, 4 * kColBuf * sizeof(double), s>>>(P, ax, lu, flags, epoch, counter,
                                                             status, pc);
}

namespace {
size_t refactor_cta_bytes(const DPlan& P) {
  return (size_t)8 * P.nslots + (size_t)4 * P.n + 16;
}
int smem_optin() {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return optin;
}
}  // namespace

bool refactor_cta_fits(const DPlan& P) {
  return P.n > 0 && refactor_cta_bytes(P) + 64 <= (size_t)smem_optin();
}

void launch_refactor_cta(const DPlan& P, const double* ax, double* lu, int* status,
                         cudaStream_t s, const PivotCheck& pc) {
  const size_t bytes = refactor_cta_bytes(P);
  cudaFuncSetAttribute(k_refactor_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_refactor_cta<<<1, 1024, bytes, s>>>(P, ax, lu, status, pc);
}

namespace {
size_t solve_cta_bytes(const DPlan& P, int rows) {
  return (size_t)8 * rows + (size_t)24 * kSolveChunk + (size_t)4 * (2 * (size_t)rows + 1) +
         (P.noffd > 0 ? (size_t)4 * (rows + 1) : 0) + 16;
}
size_t solve_cta_bytes(const DPlan& P) { return solve_cta_bytes(P, P.n); }
}  // namespace

bool solve_cta_fits(const DPlan& P) {
  return P.n > 0 && solve_cta_bytes(P) <= (size_t)smem_optin();
}

void launch_solve_cta(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                      double* out, cudaStream_t s) {
  const size_t bytes = solve_cta_bytes(P);
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(k_solve_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_solve_cta<<<1, 256, bytes, s>>>(P, rhs, ax, lu, out, kSolveChunk, 0);
}

bool solve_steps_fits(const DPlan& P) {
  return P.n > 0 && P.ss_nsteps > 0 && (size_t)8 * P.n + 16 <= (size_t)smem_optin();
}

void launch_solve_steps(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                        double* rec, double* out, cudaStream_t s) {
  const size_t bytes = (size_t)8 * P.n + 16;
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(k_solve_steps, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_solve_steps<<<1, kSolveStepsThreads, bytes, s>>>(P, rhs, ax, lu, rec, out);
}

bool solve_groups_fit(const DPlan& P) {
  return P.cs_ngrp > 0 && P.noffd == 0 &&
         solve_cta_bytes(P, P.cs_grp_rows) <= (size_t)smem_optin();
}

void launch_solve_groups(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                         double* out, cudaStream_t s) {
  const size_t bytes = solve_cta_bytes(P, P.cs_grp_rows);
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(k_solve_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_solve_cta<<<P.cs_ngrp, 256, bytes, s>>>(P, rhs, ax, lu, out, kSolveChunk, 1);
}

void launch_solve(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                  double* z, double* x, double* out, unsigned* zflag, unsigned* xflag,
                  unsigned epoch, unsigned* counter, int* status, int grid, bool transpose,
                  cudaStream_t s) {
  cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
  if (transpose)
    k_tsolve<<<grid, 128, 0, s>>>(P, rhs, ax, lu, z, x, out, zflag, xflag, epoch, counter,
                                  status);
  else
    k_solve<<<grid, 128, 0, s>>>(P, rhs, ax, lu, z, x, out, zflag, xflag, epoch, counter,
                                 status);
}

void launch_stamp(const DCircuit& C, const double* x, int xlen, double gmin, double scale,
                  double dt, const double* cap_v, double be_sign, double* ax, double* rhs_c,
                  double* rhs, cudaStream_t s, double gdev) {
  const int nb = (C.ndev + 255) / 256;
  k_stamp<<<nb > 0 ? nb : 1, 256, 0, s>>>(C, x, xlen, gmin, scale, dt, cap_v, be_sign, ax,
                                          rhs_c, gdev);
  k_rhs_sum<<<(C.n + 255) / 256, 256, 0, s>>>(C, rhs_c, rhs);
}

void launch_param_grad(const DCircuit& C, const double* x, int xlen, const double* lam,
                       double* grad, cudaStream_t s) {
  k_param_grad<<<(C.ndev + 255) / 256 > 0 ? (C.ndev + 255) / 256 : 1, 256, 0, s>>>(C, x, xlen, lam,
                                                                                  grad);
}

void launch_newton_update(int m, int n, double* x, const double* xnew, NewtonState* st,
                          NewtonCfg cfg, int* status, cudaStream_t s) {
  k_newton_update<<<1, 1024, 0, s>>>(m, n, x, xnew, st, cfg, status);
}

void launch_growth(const DPlan& P, const double* lu, double lim, int* grow, cudaStream_t s) {
  if (P.n <= 0) return;
  k_growth<<<(P.n + 255) / 256, 256, 0, s>>>(P, lu, lim, grow);
}

void launch_rcond(const DPlan& P, const double* lu, double* out2, cudaStream_t s) {
  k_rcond<<<1, 1024, 0, s>>>(P, lu, out2);
}

double fp64_peak_tflops() {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8, block = 256, iters = 4096;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * sizeof(double)) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_peak<<<grid, block>>>(out, 64, 0.999999, 1e-9);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_dfma_peak<<<grid, block>>>(out, iters, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)grid * block;
  return flops / (best * 1e-3) / 1e12;
}

template <int M, bool SHARED>
static size_t smem_bytes(const BatchArgs& a, int warps_per_block) {
  if (SHARED) return (size_t)a.shared_bytes;
  return ((size_t)a.prog_ints * 4 + (size_t)a.region * M * sizeof(double)) * warps_per_block;
}

// The dynamic shared-memory limit of an instantiation is one attribute for
// every launch of it; launches of different sizes (the batch's classes)
// raise it to the largest size any of them needs.
template <int M, bool SHARED>
static void raise_smem_limit(size_t bytes) {
  static std::mutex mu;
  static size_t set = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (bytes > set) {
    cudaFuncSetAttribute(k_batch_newton<M, SHARED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
    set = bytes;
  }
}

template <int M, bool SHARED>
static void launch_m(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  const size_t sm = smem_bytes<M, SHARED>(a, warps_per_block);
  raise_smem_limit<M, SHARED>(sm);
  k_batch_newton<M, SHARED><<<grid, 32 * warps_per_block, sm, s>>>(a);
}

// The tile counter and the per-group instance counters are reset by the
// caller before the classes start (the classes share the group counter
// array and run concurrently).
void launch_batch_newton(const BatchArgs& a, int m, int grid, int warps_per_block,
                         cudaStream_t s, bool shared) {
  if (shared) {
    switch (m) {
      case 8: launch_m<8, true>(a, grid, warps_per_block, s); break;
      case 4: launch_m<4, true>(a, grid, warps_per_block, s); break;
      case 2: launch_m<2, true>(a, grid, warps_per_block, s); break;
      default: launch_m<1, true>(a, grid, warps_per_block, s); break;
    }
    return;
  }
  switch (m) {
    case 8: launch_m<8, false>(a, grid, warps_per_block, s); break;
    case 4: launch_m<4, false>(a, grid, warps_per_block, s); break;
    case 2: launch_m<2, false>(a, grid, warps_per_block, s); break;
    default: launch_m<1, false>(a, grid, warps_per_block, s); break;
  }
}

template <int M, bool SHARED>
static void info_m(int warps_per_block, int region, int prog_ints, int* regs,
                   int* blocks_per_sm, size_t shared_bytes) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_batch_newton<M, SHARED>);
  *regs = fa.numRegs;
  const size_t per = (size_t)region * M * sizeof(double);
  const size_t sm = SHARED ? shared_bytes : ((size_t)prog_ints * 4 + per) * warps_per_block;
  raise_smem_limit<M, SHARED>(sm);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_batch_newton<M, SHARED>,
                                                32 * warps_per_block, sm);
}

void batch_kernel_info(int m, int warps_per_block, int region, int prog_ints, int* regs,
                       int* blocks_per_sm, bool shared, size_t shared_bytes) {
  auto run = [&](auto fn) {
    fn(warps_per_block, region, prog_ints, regs, blocks_per_sm, shared_bytes);
  };
  if (shared) {
    switch (m) {
      case 8: run(info_m<8, true>); break;
      case 4: run(info_m<4, true>); break;
      case 2: run(info_m<2, true>); break;
      default: run(info_m<1, true>); break;
    }
    return;
  }
  switch (m) {
    case 8: run(info_m<8, false>); break;
    case 4: run(info_m<4, false>); break;
    case 2: run(info_m<2, false>); break;
    default: run(info_m<1, false>); break;
  }
}

}  // namespace gk
