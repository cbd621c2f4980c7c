// Lane-per-instance batched Newton (the first phase of a batch run).
//
// A warp takes a group (one circuit program) and each of its 32 lanes runs
// its own instance's Newton loop: every FP64 instruction of the device
// evaluation, assembly, factorization and solves does useful work for 32
// instances, which matters on a part whose FP64 pipe issues one warp
// instruction per 16 cycles per SM. The state of the 32 instances lives in a
// per-warp global scratch, element i of lane l at [i * 32 + l], so every
// access of the warp is one coalesced 256-byte transaction; the program is
// read with warp-uniform addresses (broadcast, L1 resident).
//
// Lanes refill from the group's instance counter as their instances finish.
// An instance still iterating after `cap` iterations is parked: its iterate
// goes to its output slot, its Newton state to the continuation arrays, its
// id to the group's continuation list, and the lane moves on. The warp
// kernel (one instance per warp, state in shared memory, a much shorter
// iteration latency) then finishes the parked instances, so the long-running
// few do not hold 31 idle lanes each.
#include <cfloat>

#include "batch_common.cuh"
#include "kernels.cuh"

namespace gk {
namespace {

constexpr unsigned kAllLanes = 0xffffffffu;
constexpr int kPad = 4;  // the +0.0 contribution code that pads the four-code lists

__global__ void k_batch_lanes(BatchArgs A) {
  const int lane = threadIdx.x & 31;
  const long long wid = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  double* const W = A.scratch + wid * A.warp_stride + lane;  // element i at W[i * 32]
  const NewtonCfg cfg = A.cfg;
  const double gstart = fmax(cfg.gmin * 1e3, 1e-6);
  while (true) {
    int ti = 0;
    if (lane == 0) ti = (int)atomicAdd(A.lcounter, 1u);
    ti = __shfl_sync(kAllLanes, ti, 0);
    if (ti >= A.nltiles) return;
    const int g = A.ltile_group[ti];
    const GroupHdr G = A.groups[g];
    const int n = G.n, nc = G.node_count, nv = G.nslots + G.noffd, ndev = G.ndev;
    const int* dev_type = A.dev_type + G.dev_off;
    const int* dev_nodes = A.dev_nodes + 4 * G.dev_off;
    const int* dev_dv = A.dev_dv + G.dev_off;
    const int* amap_ptr = A.amap_ptr + G.amap_off;
    const int* amap_code = A.amap_code + G.amap_code_off;
    const int* rmap_ptr = A.rmap_ptr + G.rmap_off;
    const int* rmap_code = A.rmap_code + G.rmap_code_off;
    const int* col_ptr = A.col_ptr + G.col_off;
    const int* dslot = A.dslot + G.col_off;
    const int* col_single = A.col_single + G.col_off;
    const int* in_row = A.in_row + G.col_off;
    const int* out_pos = A.out_pos + G.col_off;
    const int* offd_ptr = A.offd_ptr + G.col_off;
    const int* slot_row = A.slot_row + G.slot_off;
    const int* upd_ptr = A.upd_ptr + G.slot_off;
    const int* upd_dst = A.upd_dst + G.upd_off;
    const int* offd_col = A.offd_col + G.offd_off;
    const int* bptr = A.block_ptr + G.blk_off;
    // disjoint views of the scratch (restrict: loads may pass earlier stores)
    double* __restrict__ const X = W;
    double* __restrict__ const T = X + (long long)nc * 32;
    double* __restrict__ const DV = T + (long long)n * 32;
    double* __restrict__ const V = DV + (long long)G.ndv * 32;
    double* __restrict__ const K = V + (long long)nv * 32;  // 4 constants per device
    const int* amap4 = A.amap4 + G.amap4_off;
    const int* rmap4 = A.rmap4 + G.rmap4_off;
    const int* lng = A.lng + G.lng_off;
#define AT(base, i) (base)[(long long)(i) * 32]

    int inst = -1, it = 0, total = 0, gstep = 0, nphase = 0;
    bool exhausted = false;
    double damp = 0.0, prev = 0.0, gmin = 0.0;
    while (true) {
      const bool need = inst < 0 && !exhausted;
      const unsigned want = __ballot_sync(kAllLanes, need);
      if (want) {
        const int first = __ffs(want) - 1;
        int base = 0;
        if (lane == first) base = (int)atomicAdd(&A.gnext[g], (unsigned)__popc(want));
        base = __shfl_sync(kAllLanes, base, first);
        if (need) {
          const int k = base + __popc(want & ((1u << lane) - 1));
          if (k < G.inst_count) {
            inst = A.order[G.inst_begin + k];
            const double* dp = A.dparams + A.inst_p_off[inst];
            const int ov = A.inst_ov_dev[inst];
            for (int d = 0; d < ndev; ++d)
#pragma unroll
              for (int q = 0; q < 4; ++q)
                AT(K, 4 * d + q) = (q == 0 && d == ov) ? A.inst_ov_val[inst] : __ldg(dp + 4 * d + q);
            const long long xo = A.inst_x0_off[inst];
            for (int i = 0; i < nc; ++i) AT(X, i) = xo >= 0 ? A.x0[xo + i] : 0.0;
            it = total = gstep = nphase = 0;
            damp = cfg.damping;
            prev = DBL_MAX;
            gmin = cfg.gmin_steps == 0 ? cfg.gmin : gstart;
          } else {
            exhausted = true;
          }
        }
      }
      const bool live = inst >= 0;
      if (!__any_sync(kAllLanes, live)) break;
      // ---- device evaluation into the value records
#pragma unroll 2
      for (int d = 0; d < ndev; ++d) {
        const int type = dev_type[d];
        const int nd[4] = {dev_nodes[4 * d], dev_nodes[4 * d + 1], dev_nodes[4 * d + 2],
                           dev_nodes[4 * d + 3]};
        double dp[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) dp[q] = AT(K, 4 * d + q);
        double rec[4];
        bt::eval_record<32>(type, nd, dp, X, X, nc, gmin, 1e-12, rec);
        const int o = dev_dv[d];
        const int nrec = bt::record_len(type, false);
        for (int q = 0; q < nrec; ++q) AT(DV, o + q) = rec[q];
      }
      // ---- assembly, in stamping order per slot and per row: up to four
      // codes each (the loads of a slot issue together), padded with +0.0
      // codes that are not added (the branches are the warp's: one program),
      // longer lists after
#pragma unroll 2
      for (int v = 0; v < nv; ++v) {
        const int4 c4 = *reinterpret_cast<const int4*>(amap4 + 4 * v);
        const double a0 = bt::contrib<32>(DV, c4.x), a1 = bt::contrib<32>(DV, c4.y);
        const double a2 = bt::contrib<32>(DV, c4.z), a3 = bt::contrib<32>(DV, c4.w);
        double acc = a0;
        if (c4.y != kPad) {
          acc += a1;
          if (c4.z != kPad) {
            acc += a2;
            if (c4.w != kPad) acc += a3;
          }
        }
        AT(V, v) = acc;
      }
#pragma unroll 2
      for (int i = 0; i < n; ++i) {
        const int4 c4 = *reinterpret_cast<const int4*>(rmap4 + 4 * i);
        const double a0 = bt::contrib<32>(DV, c4.x), a1 = bt::contrib<32>(DV, c4.y);
        const double a2 = bt::contrib<32>(DV, c4.z), a3 = bt::contrib<32>(DV, c4.w);
        double acc = a0;
        if (c4.y != kPad) {
          acc += a1;
          if (c4.z != kPad) {
            acc += a2;
            if (c4.w != kPad) acc += a3;
          }
        }
        AT(T, i) = acc;
      }
      for (int h = 0; h < G.nlng; ++h) {
        const int code = lng[h];
        const int idx = code >> 1;
        double acc = 0.0;
        if (code & 1) {
          const int r = in_row[idx];
          for (int t = rmap_ptr[r]; t < rmap_ptr[r + 1]; ++t) acc += bt::contrib<32>(DV, rmap_code[t]);
          AT(T, idx) = acc;
        } else {
          for (int t = amap_ptr[idx]; t < amap_ptr[idx + 1]; ++t) acc += bt::contrib<32>(DV, amap_code[t]);
          AT(V, idx) = acc;
        }
      }
      // ---- factor + forward substitution, backward substitution, per block
      for (int b = 0; b < G.nblocks; ++b) {
        const int b0 = bptr[b], b1 = bptr[b + 1];
        for (int i = b0; i < b1; ++i)
          for (int e = offd_ptr[i]; e < offd_ptr[i + 1]; ++e)
            AT(T, i) = fma(-AT(V, G.nslots + e), AT(T, offd_col[e]), AT(T, i));
        for (int k = b0; k < b1; ++k) {
          const int s0 = col_ptr[k], ds = dslot[k], s1 = col_ptr[k + 1];
          for (int s = s0; s < ds; ++s) {
            const double u = AT(V, s);
            const int j = slot_row[s];
            const int q0 = dslot[j] + 1, q1 = col_ptr[j + 1];
            const int* dst = upd_dst + upd_ptr[s] - q0;
            for (int qq = q0; qq < q1; ++qq) {
              const int dd = dst[qq];
              AT(V, dd) = fma(-AT(V, qq), u, AT(V, dd));
            }
          }
          const double r = bt::fast_rcp(bt::perturb_bits(AT(V, ds), col_single[k] != 0));
          const double zk = AT(T, k);
          for (int qq = ds + 1; qq < s1; ++qq) {
            const double l = AT(V, qq) * r;
            AT(V, qq) = l;
            const int row = slot_row[qq];
            AT(T, row) = fma(-l, zk, AT(T, row));
          }
          AT(V, ds) = r;
        }
        for (int k = b1 - 1; k >= b0; --k) {
          const int s0 = col_ptr[k], ds = dslot[k];
          const double xk = AT(T, k) * AT(V, ds);
          for (int s = s0; s < ds; ++s) {
            const int row = slot_row[s];
            AT(T, row) = fma(-AT(V, s), xk, AT(T, row));
          }
          AT(T, k) = xk;
        }
      }
      // ---- Newton update (crates/sim-core/src/newton.rs:93-107)
      bool conv = true, fin = true;
      double ss = 0.0;
      for (int c = 0; c < nc; ++c) {
        const double a = AT(T, out_pos[c]);
        const double dx = a - AT(X, c);
        ss = fma(dx, dx, ss);
        if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
        if (!isfinite(a)) fin = false;
      }
      if (live) {
        ++it;
        ++total;
        ++nphase;
        int rsn = -1;
        const long long xo = A.inst_x_off[inst];
        if (conv) {
          rsn = 0;
          if (xo >= 0)
            for (int c = 0; c < n; ++c) A.x_out[xo + c] = AT(T, out_pos[c]);
        } else {
          const double dxn = sqrt(ss);
          if (dxn > prev && damp > cfg.damping_min) damp = fmax(damp * 0.5, cfg.damping_min);
          prev = dxn;
          for (int c = 0; c < nc; ++c) AT(X, c) = fma(damp, AT(T, out_pos[c]) - AT(X, c), AT(X, c));
          if (!fin) {
            rsn = 1;
          } else if (it >= cfg.max_iters) {
            if (gstep < cfg.gmin_steps) {
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
            for (int c = 0; c < n; ++c) A.x_out[xo + c] = c < nc ? AT(X, c) : 0.0;
          if (rsn < 0 && A.cap > 0 && nphase >= A.cap) {  // park for the warp kernel
            for (int c = 0; c < nc; ++c) A.x_out[xo + c] = AT(X, c);
            A.cont_it[inst] = it;
            A.cont_total[inst] = total;
            A.cont_gstep[inst] = gstep;
            A.cont_damp[inst] = damp;
            A.cont_prev[inst] = prev;
            const unsigned pos = atomicAdd(&A.cont_count[g], 1u);
            A.cont_list[G.inst_begin + pos] = inst;
            inst = -1;
          }
        }
        if (rsn >= 0) {
          // a run stopped at a non-finite iterate ends, in the reference, at
          // the iteration cap (a non-finite entry never turns finite again);
          // that is the count reported, iters_total counts executed ones
          A.iters[inst] = (rsn == 1 && !fin) ? cfg.max_iters : it;
          A.iters_total[inst] = total;
          A.reason[inst] = rsn;
          inst = -1;
        }
      }
    }
#undef AT
  }
}

}  // namespace

void launch_batch_lanes(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s) {
  k_batch_lanes<<<grid, 32 * warps_per_block, 0, s>>>(a);
}

void lanes_kernel_info(int warps_per_block, int* regs, int* blocks_per_sm) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_batch_lanes);
  *regs = fa.numRegs;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_batch_lanes,
                                                32 * warps_per_block, 0);
}

}  // namespace gk
