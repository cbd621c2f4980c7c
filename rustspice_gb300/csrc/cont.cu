// Continuation of the instances the lane phase parked (the second phase of
// a batched DC run).
//
// The lane phase gives up on an instance after a few iterations; what is
// left is mostly the few instances per circuit program that never converge
// and run to the iteration cap. Here each warp takes one parked instance at
// a time from a queue over every program (most expensive programs first)
// and runs its Newton loop to the end: the iterate, the permuted right-hand
// side and the LU values in the warp's slice of shared memory (the serial
// factorization chain runs at shared-memory latency), the device records in
// the warp's slice of a global scratch (written and read by the warp's own
// lanes, L2 resident), the factorization and substitutions as the program's
// step program read through the read-only path. A warp that finishes an
// instance takes the next one at once: no warp waits for the others of its
// block, and no block stages a program.
#include <cfloat>

#include "batch_common.cuh"
#include "kernels.cuh"

namespace gk {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;

// The program view of a group without staging (global arrays only).
__device__ __forceinline__ bt::Prog global_view(const BatchArgs& A, const GroupHdr& G) {
  bt::Prog P;
  P.colrec = nullptr;
  P.srow = nullptr;
  P.uptr = A.upd_ptr + G.slot_off;
  P.udst = A.upd_dst + G.upd_off;
  P.map = nullptr;
  P.dev_type = A.dev_type + G.dev_off;
  P.dev_nodes = A.dev_nodes + 4 * G.dev_off;
  P.dev_dv = A.dev_dv + G.dev_off;
  P.amap_ptr = A.amap_ptr + G.amap_off;
  P.amap_code = A.amap_code + G.amap_code_off;
  P.rmap_ptr = A.rmap_ptr + G.rmap_off;
  P.rmap_code = A.rmap_code + G.rmap_code_off;
  P.in_row = A.in_row + G.col_off;
  P.out_pos = A.out_pos + G.col_off;
  P.offd_ptr = A.offd_ptr + G.col_off;
  P.offd_col = A.offd_col + G.offd_off;
  P.bptr = A.block_ptr + G.blk_off;
  P.heavy = A.heavy + G.heavy_off;
  P.lvl_col = A.lvl_col + G.col_off;
  P.lseg_ptr = A.lseg_ptr + G.blk_off;
  P.lseg = A.lseg + 3 * G.seg_off;
  P.amap4 = reinterpret_cast<const int4*>(A.amap4 + G.amap4_off);
  P.rmap4 = reinterpret_cast<const int4*>(A.rmap4 + G.rmap4_off);
  P.lng = A.lng + G.lng_off;
  P.nlng = G.nlng;
  P.ops = A.ops + G.ops_off;
  P.sp = A.step_ptr + G.step_off;
  P.n = G.n;
  P.nc = G.node_count;
  P.nslots = G.nslots;
  P.nv = G.nslots + G.noffd;
  P.ndev = G.ndev;
  P.nblocks = G.nblocks;
  P.nheavy = G.nheavy;
  P.nsteps = G.nsteps;
  return P;
}

// bt::run_steps with the program in global memory (read-only path): the
// next step's operation and pointer are loaded a step ahead.
__device__ __forceinline__ void run_steps_global(const bt::Prog& P, double* R, int lane) {
  const int2 nop = make_int2((int)(3u << 30), 0);  // kind 3: nothing
  const int2* const ops = P.ops;
  const int* const sp = P.sp;
  int p0 = __ldg(sp), p1 = __ldg(sp + 1);
  int2 op = p0 + lane < p1 ? __ldg(ops + p0 + lane) : nop;
  for (int t = 0; t < P.nsteps; ++t) {
    const int q0 = p1, q1 = t + 2 <= P.nsteps ? __ldg(sp + t + 2) : p1;
    const int2 next = q0 + lane < q1 ? __ldg(ops + q0 + lane) : nop;
    bt::exec_op(op, R);
    for (int p = p0 + lane + 32; p < p1; p += 32) bt::exec_op(__ldg(ops + p), R);
    __syncwarp();
    p0 = q0;
    p1 = q1;
    op = next;
  }
}

__global__ void k_batch_cont(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  double* const S = reinterpret_cast<double*>(smem_raw) + (size_t)warp * A.slice;
  double* const DV = A.dv_scratch + gw * A.dv_stride;
  const NewtonCfg cfg = A.cfg;
  const double gstart = fmax(cfg.gmin * 1e3, 1e-6);
  while (true) {
    // ---- the next parked instance: the cursor's group, or the next group
    // once it has none left (every pass either takes an instance or moves
    // the cursor on, so the loop ends)
    int inst = -1, g = -1;
    if (lane == 0) {
      while (true) {
        const unsigned c = *(volatile unsigned*)A.cont_cursor;
        if (c >= (unsigned)A.cont_ngroups) break;
        const int gg = A.cont_groups[c];
        const unsigned k = atomicAdd(&A.gnext2[gg], 1u);
        if (k < A.cont_count[gg]) {
          inst = A.cont_list[A.groups[gg].inst_begin + (int)k];
          g = gg;
          break;
        }
        atomicCAS(A.cont_cursor, c, c + 1);
      }
    }
    inst = __shfl_sync(kFullMask, inst, 0);
    g = __shfl_sync(kFullMask, g, 0);
    if (inst < 0) return;
    const GroupHdr G = A.groups[g];
    const bt::Prog P = global_view(A, G);
    const int n = P.n, nc = P.nc;
    double* const X = S;
    double* const T = X + nc;
    double* const V = T + n;
    const double* dparams = A.dparams + A.inst_p_off[inst];
    const int ov_dev = A.inst_ov_dev[inst];
    const double ov_val = A.inst_ov_val[inst];
    const long long xo = A.inst_x_off[inst];
    for (int i = lane; i < nc; i += 32) X[i] = A.x_out[xo + i];
    int it = A.cont_it[inst], total = A.cont_total[inst], gstep = A.cont_gstep[inst];
    double damp = A.cont_damp[inst], prev = A.cont_prev[inst];
    double gmin = cfg.gmin_steps == 0
                      ? cfg.gmin
                      : gstart + (cfg.gmin - gstart) * ((double)gstep / (double)cfg.gmin_steps);
    __syncwarp();
    while (true) {
      bt::stamp_devices<32>(P, dparams, ov_dev, ov_val, X, X, gmin, 1e-12, false, DV, lane);
      __syncwarp();
      bt::assemble<32>(P, DV, V, T, lane);
      __syncwarp();
      run_steps_global(P, X, lane);
      // ---- Newton update (crates/sim-core/src/newton.rs:93-107), as the
      // warp kernel does it for one instance per warp
      bool conv = true, fin = true;
      double ss = 0.0;
      for (int c = lane; c < nc; c += 32) {
        const double a = T[P.out_pos[c]];
        const double dx = a - X[c];
        ss += dx * dx;
        if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
        if (!isfinite(a)) fin = false;
      }
      const bool nconv = __any_sync(kFullMask, !conv);
      const bool nfin = __any_sync(kFullMask, !fin);
      ++it;
      ++total;
      int rsn = -1;
      if (!nconv) {
        rsn = 0;
        if (xo >= 0)
          for (int c = lane; c < n; c += 32) A.x_out[xo + c] = T[P.out_pos[c]];
      } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(kFullMask, ss, o);
        const double dxn = sqrt(ss);
        if (dxn > prev && damp > cfg.damping_min) damp = fmax(damp * 0.5, cfg.damping_min);
        prev = dxn;
        __syncwarp();
        for (int c = lane; c < nc; c += 32) X[c] = fma(damp, T[P.out_pos[c]] - X[c], X[c]);
        if (nfin) {
          rsn = 1;
        } else if (it >= cfg.max_iters) {
          if (gstep < cfg.gmin_steps) {  // next gmin step, fresh damping state
            ++gstep;
            gmin = gstart + (cfg.gmin - gstart) * ((double)gstep / (double)cfg.gmin_steps);
            it = 0;
            damp = cfg.damping;
            prev = DBL_MAX;
          } else {
            rsn = 1;
          }
        }
        if (rsn == 1 && xo >= 0)
          for (int c = lane; c < n; c += 32) A.x_out[xo + c] = c < nc ? X[c] : 0.0;
      }
      __syncwarp();
      if (rsn >= 0) {
        if (lane == 0) {  // non-finite: the reference's run ends at the cap
          A.iters[inst] = (rsn == 1 && nfin) ? cfg.max_iters : it;
          A.iters_total[inst] = total;
          A.reason[inst] = rsn;
        }
        break;
      }
    }
  }
}

}  // namespace

void launch_batch_cont(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  const size_t bytes = (size_t)warps_per_block * a.slice * sizeof(double);
  static size_t set = 0;
  if (bytes > set) {
    cudaFuncSetAttribute(k_batch_cont, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    set = bytes;
  }
  k_batch_cont<<<grid, 32 * warps_per_block, bytes, s>>>(a);
}

void cont_kernel_info(int warps_per_block, int slice, int* regs, int* blocks_per_sm) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_batch_cont);
  *regs = fa.numRegs;
  const size_t bytes = (size_t)warps_per_block * slice * sizeof(double);
  cudaFuncSetAttribute(k_batch_cont, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_batch_cont,
                                                32 * warps_per_block, bytes);
}

}  // namespace gk
