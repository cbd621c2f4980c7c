// Batched fixed-step backward-Euler transient and its checkpointed adjoint.
//
// One warp owns one instance (a circuit with its own constants) for the whole
// run and keeps its state in shared memory (layout in batch_common.cuh).
//
//  * k_tran_fwd - time steps t = 1..steps, each a Newton solve from the
//    previous time point with the capacitor companions built from it; the
//    loss sum_t (x_t[probe] - target)^2 accumulates on the fly and the state
//    is written every ckpt_every steps.
//  * k_tran_bwd - segments in reverse: the states of a segment are recomputed
//    from its checkpoint with the same Newton iterations (so they are the
//    forward's states bit for bit), then for t descending the exact Jacobian
//    J_t (level-1 floor 0) is stamped and factored and
//        J_t^T lambda_t = dL/dx_t + G_C lambda_{t+1}
//    is solved with the factors; dL/dC_d = -sum_t (lambda_t[a] -
//    lambda_t[b]) (dv_t - dv_{t-1}) / dt accumulates per capacitor.
#include <cfloat>

#include "batch_common.cuh"
#include "kernels.cuh"

namespace gk {
namespace {

constexpr int LPI = 32;

// One Newton solve of the time step (crates/sim-core/src/newton.rs:65-117):
// X holds the initial iterate on entry and the solution on exit (node
// voltages). Returns 0 when converged, 1 otherwise.
__device__ int newton_step(const BatchArgs& A, const bt::Prog& P, const double* dparams,
                           double* X, const double* XP, double* T, double* DV, double* V,
                           int sl, int& iters) {
  const NewtonCfg& cfg = A.cfg;
  const int nc = P.nc;
  double damp = cfg.damping, prev = DBL_MAX;
  for (int it = 0; it < cfg.max_iters; ++it) {
    bt::stamp_devices<LPI>(P, dparams, -1, 0.0, X, XP, cfg.gmin, 1e-12, true, DV, sl);
    __syncwarp();
    bt::assemble<LPI>(P, DV, V, T, sl);
    __syncwarp();
    bt::factor_solve<LPI>(P, V, T, sl);
    bool conv = true, fin = true;
    double ss = 0.0;
    for (int c = sl; c < nc; c += LPI) {
      const double a = T[P.out_pos[c]];
      const double dx = a - X[c];
      ss = fma(dx, dx, ss);
      if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
      if (!isfinite(a)) fin = false;
    }
    conv = __all_sync(bt::kFull, conv);
    fin = __all_sync(bt::kFull, fin);
    ++iters;
    if (conv) {
      for (int c = sl; c < nc; c += LPI) X[c] = T[P.out_pos[c]];
      __syncwarp();
      return 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(bt::kFull, ss, o);
    const double dxn = sqrt(ss);
    if (dxn > prev && damp > cfg.damping_min) damp = fmax(damp * 0.5, cfg.damping_min);
    prev = dxn;
    for (int c = sl; c < nc; c += LPI) X[c] = fma(damp, T[P.out_pos[c]] - X[c], X[c]);
    __syncwarp();
    if (!fin) return 1;
  }
  return 1;
}

__device__ __forceinline__ void copy_vec(double* dst, const double* src, int n, int sl) {
  for (int i = sl; i < n; i += LPI) dst[i] = src[i];
}

struct Slice {
  int* prog;
  double* region;
};

__device__ __forceinline__ Slice warp_slice(const BatchArgs& A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* const s =
      smem_raw + (size_t)(threadIdx.x >> 5) * ((size_t)A.prog_ints * 4 + (size_t)A.region * 8);
  return {reinterpret_cast<int*>(s), reinterpret_cast<double*>(s + (size_t)A.prog_ints * 4)};
}

__device__ __forceinline__ int next_instance(const BatchArgs& A, int lane) {
  int i = 0;
  if (lane == 0) i = (int)atomicAdd(A.counter, 1u);
  return __shfl_sync(bt::kFull, i, 0);
}

__global__ void k_tran_fwd(BatchArgs A) {
  const int lane = threadIdx.x & 31, sl = lane;
  const Slice S = warp_slice(A);
  while (true) {
    const int inst = next_instance(A, lane);
    if (inst >= A.ninst) return;
    const GroupHdr G = A.groups[A.inst_group[inst]];
    bt::Prog P = bt::stage_program(A, G, S.prog, lane);
    const int nc = P.nc, n = P.n;
    double* const X = S.region;
    double* const XP = X + nc;
    double* const T = XP + nc;
    double* const DV = T + n;
    double* const V = DV + G.ndv;
    P.map = reinterpret_cast<int*>(V + P.nv);
    const double* dparams = A.dparams + A.inst_p_off[inst];
    copy_vec(X, A.x0 + A.inst_x0_off[inst], nc, sl);
    double* ck = A.ckpt + A.ckpt_off[inst];
    __syncwarp();
    copy_vec(ck, X, nc, sl);
    const int probe = A.probe[inst];
    double loss = 0.0;
    int iters = 0, reason = 0;
    for (int t = 1; t <= A.steps; ++t) {
      copy_vec(XP, X, nc, sl);
      __syncwarp();
      if (newton_step(A, P, dparams, X, XP, T, DV, V, sl, iters)) {
        reason = 1;
        break;
      }
      const double v = X[probe];
      loss = fma(v - A.target, v - A.target, loss);
      if (A.wave && sl == 0) A.wave[(long long)inst * A.steps + (t - 1)] = v;
      if (t % A.ckpt_every == 0) copy_vec(ck + (long long)(t / A.ckpt_every) * nc, X, nc, sl);
      __syncwarp();
    }
    if (sl == 0) {
      A.loss[inst] = reason ? __longlong_as_double(0x7ff8000000000000ll) : loss;
      A.iters_total[inst] = iters;
      A.reason[inst] = reason;
    }
    const long long xo = A.inst_x_off[inst];
    for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = c < nc ? X[c] : 0.0;
    __syncwarp();
  }
}

__global__ void k_tran_bwd(BatchArgs A) {
  const int lane = threadIdx.x & 31, sl = lane;
  const Slice S = warp_slice(A);
  while (true) {
    const int inst = next_instance(A, lane);
    if (inst >= A.ninst) return;
    const GroupHdr G = A.groups[A.inst_group[inst]];
    bt::Prog P = bt::stage_program(A, G, S.prog, lane);
    const int nc = P.nc, n = P.n, ndev = P.ndev;
    double* const X = S.region;
    double* const XP = X + nc;
    double* const T = XP + nc;
    double* const DV = T + n;
    double* const V = DV + G.ndv;
    double* const LAM = V + P.nv;  // lambda_{t+1}, original row order
    double* const GR = LAM + n;    // dL/dC per device
    P.map = reinterpret_cast<int*>(GR + ndev);
    const double* dparams = A.dparams + A.inst_p_off[inst];
    const double* ck = A.ckpt + A.ckpt_off[inst];
    double* const seg = A.seg + A.seg_off[inst];
    const int probe = A.probe[inst];
    const int K = A.ckpt_every;
    for (int i = sl; i < n; i += LPI) LAM[i] = 0.0;
    for (int d = sl; d < ndev; d += LPI) GR[d] = 0.0;
    int iters = 0, failed = A.reason[inst];
    const int nseg = (A.steps + K - 1) / K;
    for (int s = nseg - 1; s >= 0 && !failed; --s) {
      const int t0 = s * K, t1 = min((s + 1) * K, A.steps);
      // recompute the segment's states from its checkpoint
      copy_vec(X, ck + (long long)s * nc, nc, sl);
      __syncwarp();
      copy_vec(seg, X, nc, sl);
      for (int t = t0 + 1; t <= t1; ++t) {
        copy_vec(XP, X, nc, sl);
        __syncwarp();
        if (newton_step(A, P, dparams, X, XP, T, DV, V, sl, iters)) {
          failed = 1;
          break;
        }
        copy_vec(seg + (long long)(t - t0) * nc, X, nc, sl);
        __syncwarp();
      }
      if (failed) break;
      for (int t = t1; t > t0; --t) {
        copy_vec(X, seg + (long long)(t - t0) * nc, nc, sl);
        copy_vec(XP, seg + (long long)(t - 1 - t0) * nc, nc, sl);
        __syncwarp();
        bt::stamp_devices<LPI>(P, dparams, -1, 0.0, X, XP, A.cfg.gmin, 0.0, true, DV, sl);
        __syncwarp();
        bt::assemble<LPI>(P, DV, V, T, sl);
        __syncwarp();
        bt::factor_solve<LPI>(P, V, T, sl);
        // right-hand side dL/dx_t + G_C lambda_{t+1}, in permuted column order
        for (int i = sl; i < n; i += LPI) T[i] = 0.0;
        __syncwarp();
        if (sl == 0) {
          T[P.out_pos[probe]] = 2.0 * (X[probe] - A.target);
          for (int d = 0; d < ndev; ++d) {
            if (P.dev_type[d] != 5) continue;
            const int a = P.dev_nodes[4 * d], b = P.dev_nodes[4 * d + 1];
            const double gl = __ldg(dparams + 4 * d + 1) * (LAM[a] - LAM[b]);
            T[P.out_pos[a]] += gl;
            T[P.out_pos[b]] -= gl;
          }
        }
        __syncwarp();
        bt::tsolve<LPI>(P, V, T, sl);
        for (int i = sl; i < n; i += LPI) LAM[P.in_row[i]] = T[i];
        __syncwarp();
        for (int d = sl; d < ndev; d += LPI) {
          if (P.dev_type[d] != 5) continue;
          const int a = P.dev_nodes[4 * d], b = P.dev_nodes[4 * d + 1];
          const double dv = (X[a] - X[b]) - (XP[a] - XP[b]);
          GR[d] = fma(-(LAM[a] - LAM[b]) * dv, A.inv_dt, GR[d]);
        }
        __syncwarp();
      }
    }
    double* const go = A.grad + A.grad_off[inst];
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    for (int d = sl; d < ndev; d += LPI) go[d] = failed ? nan : GR[d];
    if (sl == 0) A.iters[inst] = iters;
    __syncwarp();
  }
}

size_t tran_smem(const BatchArgs& a, int warps_per_block) {
  return (size_t)warps_per_block * ((size_t)a.prog_ints * 4 + (size_t)a.region * 8);
}

}  // namespace

void launch_tran_forward(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  k_tran_fwd<<<grid, 32 * warps_per_block, tran_smem(a, warps_per_block), s>>>(a);
}

void launch_tran_backward(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  k_tran_bwd<<<grid, 32 * warps_per_block, tran_smem(a, warps_per_block), s>>>(a);
}

void tran_kernel_info(bool backward, int warps_per_block, int region, int prog_ints, int* regs,
                      int* blocks_per_sm) {
  const void* fn = backward ? (const void*)k_tran_bwd : (const void*)k_tran_fwd;
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, fn);
  *regs = fa.numRegs;
  const size_t sm = (size_t)warps_per_block * ((size_t)prog_ints * 4 + (size_t)region * 8);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, 32 * warps_per_block, sm);
}

}  // namespace gk
