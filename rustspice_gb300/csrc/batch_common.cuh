// Building blocks of the batched kernels (DC Newton, transient forward and
// transient adjoint). One warp works on M instances of one circuit program
// at a time, LPI = 32/M lanes per instance, with every value of an instance
// in shared memory:
//   X[nc]   iterate (node voltages)      XP[nc] previous time point
//   T[n]    permuted right-hand side / solution
//   DV[ndv] device value records         V[nv]  LU values + BTF coupling
// The group's program (column records, slot rows, update lists) is staged in
// the warp's shared memory; everything else of the program is read through
// the read-only path.
#pragma once

#include "kernels.cuh"

namespace gk {
namespace bt {

constexpr unsigned kFull = 0xffffffffu;

// Contribution lists longer than this are summed across the instance's
// lanes instead of by one lane.
constexpr int kHeavy = 12;

// S: element stride of dv (1 in shared memory; 32 in a lane-interleaved
// scratch, where element i of a lane's array sits at [i * 32])
template <int S = 1>
__device__ __forceinline__ double contrib(const double* dv, int code) {
  const int kind = code & 7, idx = code >> 3;
  switch (kind) {
    case 0: return dv[idx * S];
    case 1: return -dv[idx * S];
    case 2: return 1.0;
    case 3: return -1.0;
    default: return 0.0;
  }
}

// x with its sign bit flipped where m has it (m: 0 or the sign bit); on the
// integer pipe.
__device__ __forceinline__ double flip_sign(double x, unsigned long long m) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)m);
}

// Device value record: R [g]; V [value]; I [value]; D [g, ieq];
// M [gds, gm, ieq]; MC [ddd, dds, ddg, ieq]; C (transient) [g, ieq].
// Circuit constants per device: R [1/R]; V, I [value]; D [Is, vt, Is/vt];
// M [is_pmos, vth0, beff]; MC [polarity, |vth0|, beff]; C [C, C/dt].
// gdev is the level-1 conductance floor (1e-12 as the reference has it; 0
// for the exact Jacobian of the adjoint).
template <int S = 1>
__device__ __forceinline__ void eval_record(int type, const int* nd, const double* dp,
                                            const double* X, const double* XP, int nc,
                                            double gmin, double gdev, double* rec) {
  auto xg = [&](int i) { return (i >= 0 && i < nc) ? X[i * S] : 0.0; };
  switch (type) {
    case 0:
    case 1:
    case 2:
      rec[0] = dp[0];
      break;
    case 3: {  // crates/sim-core/src/stamp.rs:351-387
      const double gf = gmin > 0.0 ? gmin : 1e-12;
      const double vd = xg(nd[0]) - xg(nd[1]);
      const double e = exp(vd / dp[1]);
      const double id = dp[0] * (e - 1.0);
      const double gd = dp[2] * e;
      rec[0] = fmax(gd, gf);
      rec[1] = id - gd * vd;
      break;
    }
    case 4: {  // level 1 as the reference evaluates it (evaluate.rs:285-356)
      const double lambda = 0.02;
      const double gf = gmin > 0.0 ? gmin : 1e-12;
      const bool pm = dp[0] != 0.0;
      const double vd = xg(nd[0]), vg = xg(nd[1]), vs = xg(nd[2]);
      double vdi = pm ? -vs : vd, vgi = pm ? -vg : vg, vsi = pm ? -vd : vs;
      double vgs = vgi - vsi, vds = vdi - vsi;
      if (vds < 0.0) {
        vds = -vds;
        vgs = vgi - vdi;
      }
      const double vth = pm ? -fabs(dp[1]) : fabs(dp[1]);
      const double beff = dp[2];
      double ids, gm, gds;
      if (vgs <= vth) {
        ids = 0.0;
        gm = 0.0;
        gds = gdev;
      } else if (vds < vgs - vth) {
        ids = beff * ((vgs - vth) * vds - 0.5 * vds * vds);
        gm = beff * vds;
        gds = fmax(beff * ((vgs - vth) - vds), gdev);
      } else {
        const double t = vgs - vth;
        ids = 0.5 * beff * (t * t) * (1.0 + lambda * vds);
        gm = beff * (vgs - vth) * (1.0 + lambda * vds);
        gds = fmax(0.5 * beff * (t * t) * lambda, gdev);
      }
      const double ids_s = pm ? -ids : ids;
      rec[0] = fmax(gds, gf);
      rec[1] = gm;
      rec[2] = ids_s - gm * (vg - vs) - gds * (vd - vs);
      break;
    }
    case 5: {  // backward-Euler capacitor companion, physical sign
      const double g = dp[1];
      const double vp = ((nd[0] >= 0 && nd[0] < nc) ? XP[nd[0] * S] : 0.0) -
                        ((nd[1] >= 0 && nd[1] < nc) ? XP[nd[1] * S] : 0.0);
      rec[0] = g;
      rec[1] = g * vp;
      break;
    }
    case 6: {  // consistent level 1, Shichman-Hodges form
      // One formula for the three regions, with the region tests, signs,
      // absolute values and maxima on the integer pipe (on this part an FP64
      // warp instruction costs the SM sub-partition's FP64 unit 64 cycles,
      // and lanes of a warp evaluate devices in different regions): with
      // vde = 0 (cutoff), vds_eff (linear) or vgs_eff - vth (saturation),
      //   q = vde (vov - vde / 2), ids = beff q (1 + lambda vds_eff),
      //   gm = beff (1 + lambda vds_eff) vde,
      //   gds = max(beff (1 + lambda vds_eff) (vov - vde) + lambda beff q, gdev),
      // which are the Shichman-Hodges current and its partials in each
      // region (in cutoff gds comes out as the floor gdev).
      const unsigned long long sg = 0x8000000000000000ull;
      const double lambda = 0.02;
      const double vd = xg(nd[0]), vg = xg(nd[1]), vs = xg(nd[2]);
      const unsigned long long fm = (unsigned long long)__double_as_longlong(dp[0]) & sg;
      const double vgs = flip_sign(vg - vs, fm), vds = flip_sign(vd - vs, fm);
      const unsigned long long bds = (unsigned long long)__double_as_longlong(vds);
      const bool rev = (bds & sg) != 0 && (bds << 1) != 0;  // vds < 0
      const double vgse = vgs - (rev ? vds : 0.0);
      const long long bdse = (long long)(bds & ~sg);
      const double vdse = __longlong_as_double(bdse);
      const double vth = dp[1], beff = dp[2];
      const double vov = vgse - vth;
      const long long bov = __double_as_longlong(vov);
      // non-negative doubles order as their bit patterns
      const double vde = bov <= 0 ? 0.0 : (bdse < bov ? vdse : vov);
      const double k = fma(lambda, vdse, 1.0);
      const double q = vde * fma(-0.5, vde, vov);
      const double bq = beff * q, bk = beff * k;
      const double ids = bq * k, gm = bk * vde;
      const double g0 = fma(lambda, bq, bk * (vov - vde));
      const long long b0 = __double_as_longlong(g0);
      const double gds = (b0 < 0 || b0 < __double_as_longlong(gdev)) ? gdev : g0;
      const unsigned long long rm = rev ? sg : 0ull;
      const double sum = gm + gds;
      rec[0] = rev ? sum : gds;                  // ddd
      rec[1] = flip_sign(rev ? gds : sum, sg);   // dds
      rec[2] = flip_sign(gm, rm);                // ddg
      rec[3] = flip_sign(ids, fm ^ rm) - fma(rec[2], vg, fma(rec[0], vd, rec[1] * vs));
      break;
    }
    default:
      break;
  }
}

__device__ __forceinline__ int record_len(int type, bool transient) {
  return type == 6 ? 4 : type == 4 ? 3 : type == 3 ? 2 : type == 5 ? (transient ? 2 : 0) : 1;
}

// 1/d for the batched factorization: a single-precision seed built from d's
// bits on the integer pipe, the hardware float reciprocal, and one FP64
// Newton step (relative error about 1e-14). FP64 operations have a 64-cycle
// dependent latency on this part, so this is about half the latency of the
// correctly rounded reciprocal, which serves magnitudes outside the
// single-precision range.
__device__ __forceinline__ double fast_rcp(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 1023 - 120 || e > 1023 + 120) return __drcp_rn(d);
  const unsigned fb = (unsigned)((b >> 32) & 0x80000000u) | ((unsigned)(e - 1023 + 127) << 23) |
                      (unsigned)((b >> 29) & 0x7fffffu);
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fb)));
  const unsigned rb = __float_as_uint(rf);
  const unsigned long long r64 =
      ((unsigned long long)(rb & 0x80000000u) << 32) |
      ((unsigned long long)(((rb >> 23) & 0xff) - 127 + 1023) << 52) |
      ((unsigned long long)(rb & 0x7fffffu) << 29);
  const double r = __longlong_as_double((long long)r64);
  return fma(r, fma(-d, r, 1.0), r);
}

__device__ __forceinline__ bool nonzero(double u) {
  return (__double_as_longlong(u) << 1) != 0;
}

// The reference's pivot perturbation (native_klu.rs:1229-1231, :1345-1348)
// on the bit pattern: integer compares instead of FP64 pipe compares.
__device__ __forceinline__ double perturb_bits(double d, bool singleton) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned long long a = b & 0x7fffffffffffffffull;
  if (singleton)
    return a < (unsigned long long)__double_as_longlong(1e-300) ? 1e-14 : d;
  if (a < (unsigned long long)__double_as_longlong(1e-14))
    return (a == 0 || (b >> 63) == 0) ? 1e-14 : -1e-14;
  return d;
}

// One group's program as the phases below read it.
struct Prog {
  const int4* colrec;  // staged: (s0, dslot, s1, singleton) per column
  const int* srow;     // staged: slot rows
  const int* uptr;     // update-list offsets per slot (staged when leveled)
  const int* udst;     // update destinations (staged when leveled)
  int* map;            // per instance: row -> slot of the column being factored
  const int *dev_type, *dev_nodes, *dev_dv, *amap_ptr, *amap_code, *rmap_ptr, *rmap_code,
      *in_row, *out_pos, *offd_ptr, *offd_col, *bptr, *heavy;
  const int *lvl_col, *lseg_ptr, *lseg;  // level schedule of the factorization
  const int4 *amap4, *rmap4;             // four padded codes per slot / permuted row
  const int* lng;                        // slots and rows with more: (index << 1) | is_row
  int nlng;
  const int2* ops;                       // staged step program (or null)
  const int* sp;                         //   and its step pointers
  int n, nc, nv, nslots, ndev, nblocks, nheavy, nsteps;
};

// Stages the group's factor and solve structure into shared memory and
// returns the program view: by one warp (tid = lane, nthr = 32) or by the
// whole block (block = true; every thread of the block calls it). steps:
// a group with a step program stages that instead of the column records.
__device__ __forceinline__ Prog stage_program(const BatchArgs& A, const GroupHdr& G, int* prog,
                                              int lane, int nthr = 32, bool block = false,
                                              bool steps = false) {
  Prog P;
  const int n = G.n;
  int4* const colrec = reinterpret_cast<int4*>(prog);
  int* const srow = prog + 4 * n;
  P.ops = nullptr;
  P.sp = nullptr;
  P.nsteps = 0;
  if (steps && G.nsteps > 0) {
    int2* const ops = reinterpret_cast<int2*>(prog);
    int* const sp = prog + 2 * G.nops;
    const int2* gops = A.ops + G.ops_off;
    const int* gsp = A.step_ptr + G.step_off;
    for (int q = lane; q < G.nops; q += nthr) ops[q] = gops[q];
    for (int q = lane; q <= G.nsteps; q += nthr) sp[q] = gsp[q];
    P.ops = ops;
    P.sp = sp;
    P.nsteps = G.nsteps;
  } else {
    const int* cp = A.col_ptr + G.col_off;
    const int* dsl = A.dslot + G.col_off;
    const int* cs = A.col_single + G.col_off;
    for (int k = lane; k < n; k += nthr) colrec[k] = make_int4(cp[k], dsl[k], cp[k + 1], cs[k]);
    const int* sr = A.slot_row + G.slot_off;
    for (int q = lane; q < G.nslots; q += nthr) srow[q] = sr[q];
    if (G.nseg > 0) {  // the level path reads the update lists per lane: stage them too
      int* const uptr = srow + G.nslots;
      int* const udst = uptr + G.nslots;
      const int* up = A.upd_ptr + G.slot_off;
      for (int q = lane; q < G.nslots; q += nthr) uptr[q] = up[q];
      const int* ud = A.upd_dst + G.upd_off;
      for (int q = lane; q < G.nupd; q += nthr) udst[q] = ud[q];
    }
  }
  if (block)
    __syncthreads();
  else
    __syncwarp();
  const bool cols = P.nsteps == 0;
  P.colrec = cols ? colrec : nullptr;
  P.srow = cols ? srow : nullptr;
  P.uptr = cols && G.nseg > 0 ? srow + G.nslots : A.upd_ptr + G.slot_off;
  P.udst = cols && G.nseg > 0 ? srow + 2 * G.nslots : A.upd_dst + G.upd_off;
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
  P.n = n;
  P.nc = G.node_count;
  P.nslots = G.nslots;
  P.nv = G.nslots + G.noffd;
  P.ndev = G.ndev;
  P.nblocks = G.nblocks;
  P.nheavy = G.nheavy;
  return P;
}

// Device evaluation of one instance into its value records (lanes over
// devices). ov_dev/ov_val override the first constant of one device.
template <int LPI>
__device__ __forceinline__ void stamp_devices(const Prog& P, const double* dparams, int ov_dev,
                                              double ov_val, const double* X, const double* XP,
                                              double gmin, double gdev, bool transient,
                                              double* DV, int sl) {
#pragma unroll 2
  for (int d = sl; d < P.ndev; d += LPI) {
    double dp[4];
    const double* src = dparams + 4 * d;
#pragma unroll
    for (int k = 0; k < 4; ++k) dp[k] = __ldg(src + k);
    if (d == ov_dev) dp[0] = ov_val;
    double rec[4];
    const int type = P.dev_type[d];
    eval_record(type, P.dev_nodes + 4 * d, dp, X, XP, P.nc, gmin, gdev, rec);
    const int o = P.dev_dv[d];
    const int nrec = record_len(type, transient);
    for (int k = 0; k < nrec; ++k) DV[o + k] = rec[k];
  }
}

// LU slot values and the permuted right-hand side from the value records,
// each the sum of its contributions in stamping order: lists of up to four
// as one padded 16-byte record (code 4 pads, never added), two slots per
// lane in flight; longer lists afterwards, one lane each, and the longest
// (the ground and supply rows and columns) reduced across the instance's
// lanes.
constexpr int kPadCode = 4;

__device__ __forceinline__ double sum4(const double* DV, int4 c) {
  double acc = contrib(DV, c.x);
  if (c.y != kPadCode) {
    acc += contrib(DV, c.y);
    if (c.z != kPadCode) {
      acc += contrib(DV, c.z);
      if (c.w != kPadCode) acc += contrib(DV, c.w);
    }
  }
  return acc;
}

template <int LPI>
__device__ __forceinline__ void assemble(const Prog& P, const double* DV, double* V, double* T,
                                         int sl) {
#pragma unroll 2
  for (int v = sl; v < P.nv; v += LPI) V[v] = sum4(DV, __ldg(P.amap4 + v));
#pragma unroll 2
  for (int i = sl; i < P.n; i += LPI) T[i] = sum4(DV, __ldg(P.rmap4 + i));
  __syncwarp();  // the longer lists below overwrite their all-pad records' zeros
  for (int h = sl; h < P.nlng; h += LPI) {
    const int code = P.lng[h];  // (index << 1) | is_row
    const int idx = code >> 1;
    const int* ptr = (code & 1) ? P.rmap_ptr : P.amap_ptr;
    const int* cds = (code & 1) ? P.rmap_code : P.amap_code;
    const int key = (code & 1) ? P.in_row[idx] : idx;
    const int t0 = ptr[key], t1 = ptr[key + 1];
    if (t1 - t0 > kHeavy) continue;
    double acc = contrib(DV, cds[t0]);
    for (int t = t0 + 1; t < t1; ++t) acc += contrib(DV, cds[t]);
    if (code & 1)
      T[idx] = acc;
    else
      V[idx] = acc;
  }
  for (int h = 0; h < P.nheavy; ++h) {
    const int code = P.heavy[h];  // (index << 1) | is_row
    const int idx = code >> 1;
    const int* ptr = (code & 1) ? P.rmap_ptr : P.amap_ptr;
    const int* cds = (code & 1) ? P.rmap_code : P.amap_code;
    const int key = (code & 1) ? P.in_row[idx] : idx;
    const int t0 = ptr[key], t1 = ptr[key + 1];
    double acc = 0.0;
    for (int t = t0 + sl; t < t1; t += LPI) acc += contrib(DV, cds[t]);
#pragma unroll
    for (int o = LPI / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (sl == 0) {
      if (code & 1)
        T[idx] = acc;
      else
        V[idx] = acc;
    }
  }
}

// Factor, forward substitution, backward substitution, block by block
// (blocks in order; the BTF coupling lies below the diagonal blocks).
// The factorization follows the program's level schedule: in a parallel
// segment every lane factors whole columns of one level (each column reads
// only finished columns and writes only its own slots, its U entries in
// order), in a sequential segment (the rails) the lanes share each update.
// Afterwards V[dslot] holds the reciprocal of the (perturbed) pivot and T
// the permuted solution.
__device__ __forceinline__ void factor_column(const Prog& P, double* V, int k) {
  const int4 ck = P.colrec[k];
  for (int s = ck.x; s < ck.y; ++s) {
    const double u = V[s];
    if (nonzero(u)) {
      const int4 cj = P.colrec[P.srow[s]];
      const int q0 = cj.y + 1;
      const int* dst = P.udst + P.uptr[s] - q0;
      for (int qq = q0; qq < cj.z; ++qq) {
        const int dd = dst[qq];
        V[dd] = fma(-V[qq], u, V[dd]);
      }
    }
  }
  const double r = fast_rcp(perturb_bits(V[ck.y], ck.w != 0));
  for (int qq = ck.y + 1; qq < ck.z; ++qq) V[qq] = V[qq] * r;
  V[ck.y] = r;
}

// Column by column, lanes over each update, forward substitution fused.
template <int LPI>
__device__ __forceinline__ void factor_solve_columns(const Prog& P, double* V, double* T,
                                                     int sl) {
  for (int b = 0; b < P.nblocks; ++b) {
    const int b0 = P.bptr[b], b1 = P.bptr[b + 1];
    for (int i = b0 + sl; i < b1; i += LPI)
      for (int e = P.offd_ptr[i]; e < P.offd_ptr[i + 1]; ++e)
        T[i] = fma(-V[P.nslots + e], T[P.offd_col[e]], T[i]);
    __syncwarp();
    int* const map = P.map;
    for (int k = b0; k < b1; ++k) {
      const int4 ck = P.colrec[k];
      // destination slots of this column's updates: row -> slot
      for (int q = ck.x + sl; q < ck.z; q += LPI) map[P.srow[q]] = q;
      __syncwarp();
      // The update structure of U entry s (its L column, this lane's first
      // destination) does not depend on values: it is loaded one entry
      // ahead, so its latency overlaps the previous update and its warp
      // synchronisation.
      int4 cj = make_int4(0, 0, 0, 0);
      int dd0 = 0;
      if (ck.x < ck.y) {
        cj = P.colrec[P.srow[ck.x]];
        if (cj.y + 1 + sl < cj.z) dd0 = map[P.srow[cj.y + 1 + sl]];
      }
      for (int s = ck.x; s < ck.y; ++s) {
        const int4 cur = cj;
        const int cdd0 = dd0;
        if (s + 1 < ck.y) {
          cj = P.colrec[P.srow[s + 1]];
          if (cj.y + 1 + sl < cj.z) dd0 = map[P.srow[cj.y + 1 + sl]];
        }
        const double u = V[s];
        if (nonzero(u)) {
          const int q0 = cur.y + 1;
          int qq = q0 + sl;
          if (qq < cur.z) {
            V[cdd0] = fma(-V[qq], u, V[cdd0]);
            for (qq += LPI; qq < cur.z; qq += LPI) {
              const int dd = map[P.srow[qq]];
              V[dd] = fma(-V[qq], u, V[dd]);
            }
          }
        }
        __syncwarp();
      }
      const double r = fast_rcp(perturb_bits(V[ck.y], ck.w != 0));
      const double zk = T[k];
      for (int qq = ck.y + 1 + sl; qq < ck.z; qq += LPI) {
        const double l = V[qq] * r;
        V[qq] = l;
        const int row = P.srow[qq];
        T[row] = fma(-l, zk, T[row]);
      }
      if (sl == 0) V[ck.y] = r;
      __syncwarp();
    }
    for (int k = b1 - 1; k >= b0; --k) {
      const int4 ck = P.colrec[k];
      const double xk = T[k] * V[ck.y];
      for (int s = ck.x + sl; s < ck.y; s += LPI) {
        const int row = P.srow[s];
        T[row] = fma(-V[s], xk, T[row]);
      }
      __syncwarp();
      if (sl == 0) T[k] = xk;
      __syncwarp();
    }
  }
}

template <int LPI>
__device__ __forceinline__ void factor_solve(const Prog& P, double* V, double* T, int sl) {
  if (P.lseg_ptr[P.nblocks] == 0) {  // no level schedule for this program
    factor_solve_columns<LPI>(P, V, T, sl);
    return;
  }
  for (int b = 0; b < P.nblocks; ++b) {
    const int b0 = P.bptr[b], b1 = P.bptr[b + 1];
    for (int i = b0 + sl; i < b1; i += LPI)
      for (int e = P.offd_ptr[i]; e < P.offd_ptr[i + 1]; ++e)
        T[i] = fma(-V[P.nslots + e], T[P.offd_col[e]], T[i]);
    for (int g = P.lseg_ptr[b]; g < P.lseg_ptr[b + 1]; ++g) {
      const int start = P.lseg[3 * g], end = P.lseg[3 * g + 1];
      if (P.lseg[3 * g + 2] == 0) {
        for (int idx = start + sl; idx < end; idx += LPI) factor_column(P, V, P.lvl_col[idx]);
        __syncwarp();
        continue;
      }
      for (int idx = start; idx < end; ++idx) {
        const int k = P.lvl_col[idx];
        const int4 ck = P.colrec[k];
        for (int s = ck.x; s < ck.y; ++s) {
          const double u = V[s];
          if (nonzero(u)) {
            const int4 cj = P.colrec[P.srow[s]];
            const int q0 = cj.y + 1;
            const int* dst = P.udst + P.uptr[s] - q0;
            for (int qq = q0 + sl; qq < cj.z; qq += LPI) {
              const int dd = dst[qq];
              V[dd] = fma(-V[qq], u, V[dd]);
            }
          }
          __syncwarp();
        }
        const double r = fast_rcp(perturb_bits(V[ck.y], ck.w != 0));
        for (int qq = ck.y + 1 + sl; qq < ck.z; qq += LPI) V[qq] = V[qq] * r;
        __syncwarp();
        if (sl == 0) V[ck.y] = r;
        __syncwarp();
      }
    }
    for (int k = b0; k < b1; ++k) {  // L z = b, column order
      const int4 ck = P.colrec[k];
      const double zk = T[k];
      for (int qq = ck.y + 1 + sl; qq < ck.z; qq += LPI) {
        const int row = P.srow[qq];
        T[row] = fma(-V[qq], zk, T[row]);
      }
      __syncwarp();
    }
    for (int k = b1 - 1; k >= b0; --k) {
      const int4 ck = P.colrec[k];
      const double xk = T[k] * V[ck.y];
      for (int s = ck.x + sl; s < ck.y; s += LPI) {
        const int row = P.srow[s];
        T[row] = fma(-V[s], xk, T[row]);
      }
      __syncwarp();
      if (sl == 0) T[k] = xk;
      __syncwarp();
    }
  }
}

// One operation of a step program on an instance region R (X, T, V), two
// 32-bit words: d | a << 15 | kind bits 0-1 << 30 and b | c << 15 | kind
// bits 2-3 << 30. Kinds: 0 R[d] -= R[a] R[b] (one fma); 4 the same unless
// R[b] is zero (a factor update by a zero U entry is skipped); 2 R[d] =
// R[a] R[b]; 1 R[d] = 1 / perturbed R[d] (a: the column is a singleton); 5
// kind 4 then R[d] *= R[c] (an L entry's last update and its scaling); 6
// kind 0 then R[d] *= R[c] (a row's last backward update and its pivot);
// 3 nothing.
__device__ __forceinline__ void exec_op(int2 o, double* R) {
  const unsigned x = (unsigned)o.x, y = (unsigned)o.y;
  const int d = x & 0x7fff, a = (x >> 15) & 0x7fff, b = y & 0x7fff, c = (y >> 15) & 0x7fff;
  const int k = (int)((x >> 30) | ((y >> 30) << 2));
  if (k == 1) {
    R[d] = fast_rcp(perturb_bits(R[d], a != 0));
    return;
  }
  // The other kinds as one fma, so that lanes of a step that mix them issue
  // one FP64 instruction (and the product only where a lane needs it): kind 2
  // is fma(a, b, -0), which rounds like a b; kinds 0, 4, 5 and 6 are fma(-a,
  // b, d), with d kept where kind 4 or 5 skips a zero b. The signs and the
  // selections are integer operations.
  const bool mul = k == 2, fused = k >= 5;
  const double va = R[a], vb = R[b], vd = R[d];
  const double na = flip_sign(va, mul ? 0ull : 0x8000000000000000ull);
  const double t = fma(na, vb, mul ? -0.0 : vd);
  const bool skip = (k == 4 || k == 5) && !nonzero(vb);
  double r = skip ? vd : t;
  if (fused) r = r * R[c];
  if (k != 3) R[d] = r;
}

// The factorization, forward and backward substitution as the group's step
// program: the host lists every operation of factor_solve_columns in its
// order and places each in the first step after the steps that write its
// operands or read its destination, so the operations of one step are
// independent and every value sees the same operations in the same order
// as in the column-by-column path (the same results; fused pairs keep both
// roundings). The instance's lanes take a step's operations in parallel;
// the next step's operations are loaded while the current one runs. The
// warp's instances run the same program in step.
template <int LPI>
__device__ __forceinline__ void run_steps(const Prog& P, double* R, int sl) {
  const int2 nop = make_int2((int)(3u << 30), 0);  // kind 3: nothing
  const int2* const ops = P.ops;
  const int* const sp = P.sp;
  const int ns = P.nsteps;
  const int nops = sp[ns];
  // a step's operation and pointer load independently, a step ahead
  int s0 = sp[0], s1 = sp[1], s2 = ns >= 2 ? sp[2] : s1;
  int2 o0 = s0 + sl < nops ? ops[s0 + sl] : nop;
  for (int t = 0; t < ns; ++t) {
    const int2 o1 = s1 + sl < nops ? ops[s1 + sl] : nop;
    const int s3 = t + 3 <= ns ? sp[t + 3] : s2;
    if (s0 + sl < s1) exec_op(o0, R);
    for (int p = s0 + sl + LPI; p < s1; p += LPI) exec_op(ops[p], R);
    __syncwarp();
    s0 = s1;
    s1 = s2;
    s2 = s3;
    o0 = o1;
  }
}

// Transpose solve with the factors factor_solve left in V: on entry T holds
// the right-hand side in permuted column order (T[out_pos[c]] = g[c]); on
// exit T holds w with lambda[in_row[i]] = w[i]. Blocks in reverse order:
// U^T forward, L^T backward, then the block's coupling scattered into the
// earlier blocks by one lane (few entries).
template <int LPI>
__device__ __forceinline__ void tsolve(const Prog& P, const double* V, double* T, int sl) {
  constexpr unsigned smask = kFull;  // all M instances of the warp run in step
  for (int b = P.nblocks - 1; b >= 0; --b) {
    const int b0 = P.bptr[b], b1 = P.bptr[b + 1];
    for (int k = b0; k < b1; ++k) {  // U^T y = r
      const int4 ck = P.colrec[k];
      double acc = 0.0;
      for (int s = ck.x + sl; s < ck.y; s += LPI) acc = fma(V[s], T[P.srow[s]], acc);
#pragma unroll
      for (int o = LPI / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(smask, acc, o);
      const double yk = (T[k] - acc) * V[ck.y];
      __syncwarp(smask);
      if (sl == 0) T[k] = yk;
      __syncwarp(smask);
    }
    for (int k = b1 - 1; k >= b0; --k) {  // L^T w = y
      const int4 ck = P.colrec[k];
      double acc = 0.0;
      for (int q = ck.y + 1 + sl; q < ck.z; q += LPI) acc = fma(V[q], T[P.srow[q]], acc);
#pragma unroll
      for (int o = LPI / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(smask, acc, o);
      const double wk = T[k] - acc;
      __syncwarp(smask);
      if (sl == 0) T[k] = wk;
      __syncwarp(smask);
    }
    if (sl == 0)
      for (int i = b0; i < b1; ++i)
        for (int e = P.offd_ptr[i]; e < P.offd_ptr[i + 1]; ++e)
          T[P.offd_col[e]] = fma(-V[P.nslots + e], T[i], T[P.offd_col[e]]);
    __syncwarp(smask);
  }
}

}  // namespace bt
}  // namespace gk
