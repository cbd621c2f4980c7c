// Continuation of the instances the lane phase parked (the second phase of
// a batched DC run).
//
// The lane phase gives up on an instance after a few iterations; what is
// left is mostly the few instances per circuit program that never converge
// and run to the iteration cap. Here each warp takes one parked instance at
// a time from a queue over every program (most expensive programs first)
// and runs its Newton loop to the end: the permuted right-hand side and the
// LU values in the warp's slice of shared memory (the serial factorization
// chain runs at shared-memory latency), the device records and the iterate
// in the warp's slice of a global scratch (written and read by the warp's
// own lanes, L2 resident), the factorization and substitutions as the
// program's step program read through the read-only path. A warp that finishes an
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

// bt::run_steps with the program in global memory (read-only path). A
// step's operation and its step pointer are independent loads issued two
// steps ahead (the operation load bounded by the program's length, not by
// the next pointer), so neither waits on the other and both have two steps
// to arrive; the instance's LPI lanes take a step's operations.
template <int LPI>
__device__ __forceinline__ void run_steps_global(const bt::Prog& P, double* R, int sl) {
  const int2 nop = make_int2((int)(3u << 30), 0);  // kind 3: nothing
  const int2* const ops = P.ops;
  const int* const sp = P.sp;
  const int ns = P.nsteps;
  const int nops = __ldg(sp + ns);
  int s0 = __ldg(sp), s1 = __ldg(sp + 1);
  int s2 = ns >= 2 ? __ldg(sp + 2) : s1, s3 = ns >= 3 ? __ldg(sp + 3) : s2;
  int2 o0 = s0 + sl < nops ? __ldg(ops + s0 + sl) : nop;
  int2 o1 = s1 + sl < nops ? __ldg(ops + s1 + sl) : nop;
  for (int t = 0; t < ns; ++t) {
    const int2 o2 = s2 + sl < nops ? __ldg(ops + s2 + sl) : nop;
    const int s4 = t + 4 <= ns ? __ldg(sp + t + 4) : s3;
    if (s0 + sl < s1) bt::exec_op(o0, R);
    for (int p = s0 + sl + LPI; p < s1; p += LPI) bt::exec_op(__ldg(ops + p), R);
    __syncwarp();
    s0 = s1;
    s1 = s2;
    s2 = s3;
    s3 = s4;
    o0 = o1;
    o1 = o2;
  }
}

// M instances of one program per warp (32 / M lanes each, in step: one FP64
// instruction of a step serves all M); a sub-warp whose instance ends takes
// the program's next parked instance, and the warp moves to the next
// program when every sub-warp has run out.
template <int M>
__global__ void k_batch_cont(BatchArgs A) {
  constexpr int LPI = 32 / M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LPI, sl = lane % LPI;
  const unsigned smask = M == 1 ? kFullMask : (((1u << LPI) - 1u) << (sub * LPI));
  const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  double* const S = reinterpret_cast<double*>(smem_raw) + ((size_t)warp * M + sub) * A.slice;
  double* const DV = A.dv_scratch + (gw * M + sub) * A.dv_stride;
  const NewtonCfg cfg = A.cfg;
  const double gstart = fmax(cfg.gmin * 1e3, 1e-6);
  while (true) {
    // ---- the next program with parked instances, and up to M of them
    // (every pass either takes instances or moves the cursor on, so the
    // loop ends)
    int g = -1;
    unsigned k0 = 0, cnt = 0;
    if (lane == 0) {
      while (true) {
        const unsigned c = *(volatile unsigned*)A.cont_cursor;
        if (c >= (unsigned)A.cont_ngroups) break;
        const int gg = A.cont_groups[c];
        const unsigned k = atomicAdd(&A.gnext2[gg], (unsigned)M);
        const unsigned count = A.cont_fresh ? (unsigned)A.groups[gg].inst_count : A.cont_count[gg];
        if (k < count) {
          g = gg;
          k0 = k;
          cnt = count;
          break;
        }
        atomicCAS(A.cont_cursor, c, c + 1);
      }
    }
    g = __shfl_sync(kFullMask, g, 0);
    k0 = __shfl_sync(kFullMask, k0, 0);
    cnt = __shfl_sync(kFullMask, cnt, 0);
    if (g < 0) return;
    const GroupHdr G = A.groups[g];
    const bt::Prog P = global_view(A, G);
    const int n = P.n, nc = P.nc;
    // shared: T, V; global (L2): the records and the iterate. The step
    // program addresses T at nc and V at nc + n from a base nc doubles
    // before the slice (it touches no X entry).
    double* const X = DV + A.dv_x;
    double* const T = S;
    double* const V = T + n;
    double* const R = S - nc;
    // a program's instances: those the lane phase parked, or all of them
    const int* const list = A.cont_fresh ? A.order : A.cont_list;
    int inst = k0 + sub < cnt ? list[G.inst_begin + (int)(k0 + sub)] : -1;
    bool exhausted = inst < 0;
    int it = 0, total = 0, gstep = 0, ov_dev = -1;
    long long xo = 0;
    double damp = 0.0, prev = 0.0, gmin = 0.0, ov_val = 0.0;
    const double* dparams = nullptr;
    auto resume = [&]() {  // where the lane phase parked the instance, or its start
      dparams = A.dparams + A.inst_p_off[inst];
      ov_dev = A.inst_ov_dev[inst];
      ov_val = A.inst_ov_val[inst];
      xo = A.inst_x_off[inst];
      if (A.cont_fresh) {
        const long long x0o = A.inst_x0_off[inst];
        for (int i = sl; i < nc; i += LPI) X[i] = x0o >= 0 ? A.x0[x0o + i] : 0.0;
        it = total = gstep = 0;
        damp = cfg.damping;
        prev = DBL_MAX;
        gmin = cfg.gmin_steps == 0 ? cfg.gmin : gstart;
        return;
      }
      for (int i = sl; i < nc; i += LPI) X[i] = A.x_out[xo + i];
      it = A.cont_it[inst];
      total = A.cont_total[inst];
      gstep = A.cont_gstep[inst];
      damp = A.cont_damp[inst];
      prev = A.cont_prev[inst];
      gmin = cfg.gmin_steps == 0
                 ? cfg.gmin
                 : gstart + (cfg.gmin - gstart) * ((double)gstep / (double)cfg.gmin_steps);
    };
    if (inst >= 0) resume();
    while (true) {
      if (M > 1) {  // idle sub-warps take the program's next instances
        const bool need = inst < 0 && !exhausted;
        const unsigned want = __ballot_sync(kFullMask, need && sl == 0);
        if (want) {
          const int first = __ffs(want) - 1;
          unsigned base = 0;
          if (lane == first) base = atomicAdd(&A.gnext2[g], (unsigned)__popc(want));
          base = __shfl_sync(kFullMask, base, first);
          if (need) {
            const unsigned kk = base + __popc(want & ((1u << (sub * LPI)) - 1u));
            if (kk < cnt) {
              inst = A.cont_list[G.inst_begin + (int)kk];
              resume();
            } else {
              exhausted = true;
            }
          }
        }
      }
      if (!__any_sync(kFullMask, inst >= 0)) break;
      __syncwarp();
      const bool live = inst >= 0;
      if (live) bt::stamp_devices<LPI>(P, dparams, ov_dev, ov_val, X, X, gmin, 1e-12, false, DV, sl);
      __syncwarp();
      bt::assemble<LPI>(P, DV, V, T, sl);
      __syncwarp();
      run_steps_global<LPI>(P, R, sl);
      // ---- Newton update (crates/sim-core/src/newton.rs:93-107), as the
      // warp kernel does it
      bool conv = true, fin = true;
      double ss = 0.0;
      for (int c = sl; c < nc; c += LPI) {
        const double a = T[P.out_pos[c]];
        const double dx = a - X[c];
        ss += dx * dx;
        if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
        if (!isfinite(a)) fin = false;
      }
      const unsigned nconv = __ballot_sync(kFullMask, !conv) & smask;
      const unsigned nfin = __ballot_sync(kFullMask, !fin) & smask;
#pragma unroll
      for (int o = LPI / 2; o > 0; o >>= 1) ss += __shfl_xor_sync(kFullMask, ss, o);
      __syncwarp();
      if (live) {
        ++it;
        ++total;
        int rsn = -1;
        if (!nconv) {
          rsn = 0;
          if (xo >= 0)
            for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = T[P.out_pos[c]];
        } else {
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
              prev = DBL_MAX;
            } else {
              rsn = 1;
            }
          }
          if (rsn == 1 && xo >= 0)
            for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = c < nc ? X[c] : 0.0;
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
  }
}

template <int M>
void launch_m(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  const size_t bytes = (size_t)warps_per_block * M * a.slice * sizeof(double);
  static size_t set = 0;
  if (bytes > set) {
    cudaFuncSetAttribute(k_batch_cont<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
    set = bytes;
  }
  k_batch_cont<M><<<grid, 32 * warps_per_block, bytes, s>>>(a);
}

template <int M>
void info_m(int warps_per_block, int slice, int* regs, int* blocks_per_sm) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_batch_cont<M>);
  *regs = fa.numRegs;
  const size_t bytes = (size_t)warps_per_block * M * slice * sizeof(double);
  cudaFuncSetAttribute(k_batch_cont<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_batch_cont<M>,
                                                32 * warps_per_block, bytes);
}

}  // namespace

void launch_batch_cont(const BatchArgs& a, int m, int grid, int warps_per_block,
                       cudaStream_t s) {
  if (m == 2)
    launch_m<2>(a, grid, warps_per_block, s);
  else
    launch_m<1>(a, grid, warps_per_block, s);
}

void cont_kernel_info(int m, int warps_per_block, int slice, int* regs, int* blocks_per_sm) {
  if (m == 2)
    info_m<2>(warps_per_block, slice, regs, blocks_per_sm);
  else
    info_m<1>(warps_per_block, slice, regs, blocks_per_sm);
}

}  // namespace gk
