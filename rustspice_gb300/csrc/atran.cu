// Batched adaptive transient: the reference engine's transient analysis
// (crates/sim-core/src/engine.rs:332-602) with one warp per circuit
// instance, state in shared memory (layout below), the whole time loop on
// the device:
//   DC operating point from the instance's initial guess (the .ic values),
//   then per step: the step limited to the next breakpoint and by settling
//   after one (waveform.rs:567-641), a backward-Euler Newton solve and a
//   trapezoidal one from the last accepted point, Milne's estimate
//   |x_trap - x_be| / 3 against vntol + reltol max(|x|) over the whole
//   iterate (analysis.rs:147-206), the PI controller (analysis.rs:497-583,
//   720-743) and, on acceptance, the trapezoidal point with the companion
//   history update (stamp.rs:572-668); ten rejections in a row end the run.
// The per-device value records are the batched kernels' (batch_common.cuh);
// capacitors and time-dependent sources are re-evaluated here for the mode
// of each solve: DC (capacitor open), BE (g = C/dt, rhs += be_sign g v_prev;
// be_sign -1 is the reference's sign, +1 the physical one), trapezoidal
// (g = 2C/dt, rhs += g v_prev + i_prev).
#include <cfloat>

#include "batch_common.cuh"
#include "kernels.cuh"

namespace gk {
namespace {

constexpr int LPI = 32;
enum Mode { DC = 0, BE = 1, TRAP = 2 };

__device__ double wave_value(const AtranArgs& T, int r, double t) {
  const double* p = T.wave_p + 7 * (long long)r;
  switch (T.wave_kind[r]) {
    case 1: {  // PULSE
      const double v1 = p[0], v2 = p[1], td = p[2], tr = p[3], tf = p[4], pw = p[5], per = p[6];
      if (t < td) return v1;
      const double trl = per > 0.0 ? fmod(t - td, per) : t - td;
      if (trl < tr) return v1 + (v2 - v1) * trl / tr;
      if (trl < tr + pw) return v2;
      if (trl < tr + pw + tf) return v2 - (v2 - v1) * (trl - tr - pw) / tf;
      return v1;
    }
    case 2: {  // PWL
      const int q0 = T.pwl_ptr[r], q1 = T.pwl_ptr[r + 1];
      if (q1 <= q0) return 0.0;
      if (t <= T.pwl_t[q0]) return T.pwl_v[q0];
      if (t >= T.pwl_t[q1 - 1]) return T.pwl_v[q1 - 1];
      for (int q = q0; q + 1 < q1; ++q) {
        const double t0 = T.pwl_t[q], t1 = T.pwl_t[q + 1];
        if (t >= t0 && t < t1) {
          const double v0 = T.pwl_v[q], v1 = T.pwl_v[q + 1];
          return v0 + (v1 - v0) * ((t - t0) / (t1 - t0));
        }
      }
      return T.pwl_v[q1 - 1];
    }
    case 3: {  // SIN
      if (t < p[3]) return p[0];
      const double trl = t - p[3];
      const double damp = p[4] > 0.0 ? exp(-p[4] * trl) : 1.0;
      return p[0] + p[1] * sin(2.0 * 3.141592653589793 * p[2] * trl) * damp;
    }
    case 4: {  // EXP
      if (t < p[2]) return p[0];
      double v = p[0] + (p[1] - p[0]) * (1.0 - exp(-(t - p[2]) / p[3]));
      if (t >= p[4]) v += (p[0] - p[1]) * (1.0 - exp(-(t - p[4]) / p[5]));
      return v;
    }
    default:
      return 0.0;
  }
}

struct Step {  // the companion state and the solve's mode
  int mode;
  double t, dt;
  const double *capv, *capi;
};

// Value records at X for the solve: the batched records, then capacitors
// and time-dependent sources for the mode.
__device__ void stamp_step(const BatchArgs& A, const AtranArgs& T, const bt::Prog& P,
                           const double* dparams, int w0, int w1, const double* X, const Step& s,
                           double* DV, int sl) {
  bt::stamp_devices<LPI>(P, dparams, -1, 0.0, X, X, A.cfg.gmin, 1e-12, true, DV, sl);
  __syncwarp();
  for (int d = sl; d < P.ndev; d += LPI) {
    if (P.dev_type[d] != 5) continue;
    const double C = __ldg(dparams + 4 * d);
    double g = 0.0, ieq = 0.0;
    if (s.mode == BE) {
      g = C / s.dt;
      ieq = T.be_sign * (g * s.capv[d]);
    } else if (s.mode == TRAP) {
      g = 2.0 * C / s.dt;
      ieq = g * s.capv[d] + s.capi[d];
    }
    DV[P.dev_dv[d]] = g;
    DV[P.dev_dv[d] + 1] = ieq;
  }
  for (int r = w0 + sl; r < w1; r += LPI) DV[P.dev_dv[T.wave_dev[r]]] = wave_value(T, r, s.t);
  __syncwarp();
}

// run_newton (newton.rs:65-117) on X: m entries enter the convergence test
// and the damping (node_count on the DC point's fresh start, n afterwards);
// on convergence X takes the whole solution. Returns 0 when converged.
__device__ int newton_atran(const BatchArgs& A, const AtranArgs& T, const bt::Prog& P,
                            const double* dparams, int w0, int w1, double* X, int m,
                            const Step& s, double* TS, double* DV, double* V, int sl,
                            int& iters) {
  const NewtonCfg& cfg = A.cfg;
  double damp = cfg.damping, prev = DBL_MAX;
  for (int it = 0; it < cfg.max_iters; ++it) {
    stamp_step(A, T, P, dparams, w0, w1, X, s, DV, sl);
    bt::assemble<LPI>(P, DV, V, TS, sl);
    __syncwarp();
    bt::factor_solve<LPI>(P, V, TS, sl);
    bool conv = true;
    double ss = 0.0;
    for (int c = sl; c < m; c += LPI) {
      const double a = TS[P.out_pos[c]];
      const double dx = a - X[c];
      ss = fma(dx, dx, ss);
      if (!(fabs(dx) <= cfg.abs_tol + cfg.rel_tol * fabs(a))) conv = false;
    }
    conv = __all_sync(bt::kFull, conv);
    ++iters;
    if (conv) {
      for (int c = sl; c < P.n; c += LPI) X[c] = TS[P.out_pos[c]];
      __syncwarp();
      return 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(bt::kFull, ss, o);
    const double dxn = sqrt(ss);
    if (dxn > prev && damp > cfg.damping_min) damp = fmax(damp * 0.5, cfg.damping_min);
    prev = dxn;
    for (int c = sl; c < m; c += LPI) X[c] = X[c] + damp * (TS[P.out_pos[c]] - X[c]);
    __syncwarp();
  }
  return 1;
}

__global__ void k_atran(BatchArgs A, AtranArgs T) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, sl = lane;
  unsigned char* const sbase =
      smem_raw + (size_t)(threadIdx.x >> 5) * ((size_t)A.prog_ints * 4 + (size_t)A.region * 8);
  int* const sprog = reinterpret_cast<int*>(sbase);
  double* const sreg = reinterpret_cast<double*>(sbase + (size_t)A.prog_ints * 4);
  while (true) {
    int inst = 0;
    if (lane == 0) inst = (int)atomicAdd(A.counter, 1u);
    inst = __shfl_sync(bt::kFull, inst, 0);
    if (inst >= A.ninst) return;
    const GroupHdr G = A.groups[A.inst_group[inst]];
    bt::Prog P = bt::stage_program(A, G, sprog, lane);
    const int nc = P.nc, n = P.n, ndev = P.ndev;
    double* const X = sreg;        // the last accepted point (n)
    double* const XB = X + n;      // backward-Euler solve (n)
    double* const XT = XB + n;     // trapezoidal solve (n)
    double* const TS = XT + n;     // right-hand side / solution (n)
    double* const CV = TS + n;     // capacitor voltage at the last point (ndev)
    double* const CI = CV + ndev;  // trapezoidal history current (ndev)
    double* const DV = CI + ndev;
    double* const V = DV + G.ndv;
    P.map = reinterpret_cast<int*>(V + P.nv);
    const double* dparams = A.dparams + A.inst_p_off[inst];
    const int w0 = T.wave_ptr[inst], w1 = T.wave_ptr[inst + 1];
    const int b0 = T.bp_ptr[inst], b1 = T.bp_ptr[inst + 1];
    const double* x0 = A.x0 + A.inst_x0_off[inst];
    for (int c = sl; c < n; c += LPI) X[c] = c < nc ? x0[c] : 0.0;
    for (int d = sl; d < ndev; d += LPI) CV[d] = CI[d] = 0.0;
    __syncwarp();
    const long long o0 = (long long)inst * T.max_points;
    const int probe = T.probe[inst];
    int iters = 0, status = 0, npts = 0, acc = 0, rej = 0;
    // ---- DC operating point at tstart (engine.rs:412-451)
    Step st{DC, T.tstart, 0.0, CV, CI};
    if (newton_atran(A, T, P, dparams, w0, w1, X, nc, st, TS, DV, V, sl, iters)) status = 2;
    const double min_dt = fmax(T.tstep * 1e-6, 1e-15);
    const double max_dt = fmin(T.tmax, T.tstop / 10.0);
    double t = T.tstart, dt = fmin(T.tstep, max_dt);
    if (status == 0) {
      for (int d = sl; d < ndev; d += LPI)
        if (P.dev_type[d] == 5) {
          const int a = P.dev_nodes[4 * d], b = P.dev_nodes[4 * d + 1];
          CV[d] = (a < nc ? X[a] : 0.0) - (b < nc ? X[b] : 0.0);
        }
      if (sl == 0 && T.max_points > 0) {
        T.times[o0] = t;
        T.probe_out[o0] = X[probe];
      }
      npts = 1;
      __syncwarp();
    }
    // controller state: PI history, its and the engine's reject counters,
    // settling, the first breakpoint after t
    bool has_prev = false;
    double prev_err = 0.0;
    int pi_rej = 0, consecutive = 0, settling = 0, bi = b0, attempts = 0;
    while (status == 0 && t < T.tstop) {
      if (++attempts > T.max_steps) {
        status = 3;
        break;
      }
      while (bi < b1 && T.bp_t[bi] <= t) ++bi;
      if (bi < b1) {  // limit_dt (waveform.rs:567-600)
        const double to_bp = T.bp_t[bi] - t;
        if (dt >= to_bp)
          dt = fmax(to_bp, min_dt);
        else if (dt > 0.9 * to_bp)
          dt = to_bp;
        else if (to_bp - dt < 0.1 * dt && to_bp - dt < min_dt * 10.0)
          dt = to_bp;
      }
      if (settling > 0) dt = fmax(dt * 0.1, min_dt);
      if (t + dt > T.tstop) dt = T.tstop - t;
      const double tt = t + dt;
      for (int c = sl; c < n; c += LPI) XB[c] = XT[c] = X[c];
      __syncwarp();
      Step sb{BE, tt, dt, CV, CI};
      Step sr{TRAP, tt, dt, CV, CI};
      bool fail = newton_atran(A, T, P, dparams, w0, w1, XB, n, sb, TS, DV, V, sl, iters) != 0;
      if (!fail)
        fail = newton_atran(A, T, P, dparams, w0, w1, XT, n, sr, TS, DV, V, sl, iters) != 0;
      if (fail) {  // Newton failed: a quarter of the step, at least min_dt
        ++consecutive;
        ++rej;
        if (consecutive >= 10) {
          status = 1;
          break;
        }
        dt = fmax(dt * 0.25, min_dt);
        continue;
      }
      // Milne's estimate over the whole iterate
      double mr = 0.0;
      for (int c = sl; c < n; c += LPI) {
        const double be = XB[c], tr = XT[c];
        if (fabs(be) < 1e-30 && fabs(tr) < 1e-30) continue;
        const double lte = fabs(tr - be) / 3.0;
        const double tol = T.lte_abs + T.lte_rel * fmax(fabs(be), fabs(tr));
        const double ratio = tol > 0.0 ? lte / tol : 0.0;
        mr = fmax(mr, ratio);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mr = fmax(mr, __shfl_xor_sync(bt::kFull, mr, o));
      const bool accept = mr <= 1.0;  // lte.accept and !should_reject (both: mr <= 1)
      double dt_new;
      if (accept) {  // suggest_dt, then record the accepted step
        const double p_f = pow(1.0 / fmax(mr, 1e-10), 0.35);
        const double i_f = has_prev ? pow(1.0 / fmax(prev_err, 1e-10), 0.2) : 1.0;
        dt_new = dt * fmin(fmax(p_f * i_f * 0.9, 0.1), 2.0);
        dt_new = fmin(fmax(dt_new, min_dt), max_dt);
        has_prev = true;
        prev_err = mr;
        pi_rej = 0;
      } else {
        ++pi_rej;
        if (pi_rej >= 3) {  // emergency_dt (struggling)
          dt_new = pi_rej <= 5 ? dt * 0.25 : (pi_rej <= 10 ? dt * 0.1 : min_dt);
        } else {
          const double f = mr > 1e-10 ? fmin(fmax(pow(1.0 / mr, 0.5) * 0.9, 0.1), 2.0) : 2.0;
          dt_new = fmin(fmax(dt * f, min_dt), max_dt);
        }
      }
      if (accept) {
        const double t_new = t + dt;
        // update_settling: a breakpoint in (t, t_new] starts five steps
        const bool crossed = bi < b1 && T.bp_t[bi] <= t_new;
        if (crossed) settling = 5;
        if (settling > 0) --settling;
        for (int c = sl; c < n; c += LPI) X[c] = XT[c];
        __syncwarp();
        for (int d = sl; d < ndev; d += LPI)
          if (P.dev_type[d] == 5) {  // update_transient_state_full
            const int a = P.dev_nodes[4 * d], b = P.dev_nodes[4 * d + 1];
            const double v = (a < n ? X[a] : 0.0) - (b < n ? X[b] : 0.0);
            CI[d] = __ldg(dparams + 4 * d) * (v - CV[d]) / dt;
            CV[d] = v;
          }
        if (sl == 0 && npts < T.max_points) {
          T.times[o0 + npts] = t_new;
          T.probe_out[o0 + npts] = X[probe];
        }
        __syncwarp();
        ++npts;
        t = t_new;
        ++acc;
        consecutive = 0;
        dt = fmin(fmax(dt_new, min_dt), max_dt);
      } else {
        ++rej;
        ++consecutive;
        if (consecutive >= 10) {
          status = 1;
          break;
        }
        dt = fmin(fmax(dt_new, min_dt), max_dt);
      }
    }
    if (sl == 0) {
      T.status[inst] = status;
      T.npoints[inst] = npts;
      T.accepted[inst] = acc;
      T.rejected[inst] = rej;
      A.iters_total[inst] = iters;
    }
    const long long xo = A.inst_x_off[inst];
    for (int c = sl; c < n; c += LPI) A.x_out[xo + c] = X[c];
    __syncwarp();
  }
}

size_t atran_smem(const BatchArgs& a) { return (size_t)a.prog_ints * 4 + (size_t)a.region * 8; }

}  // namespace

void launch_atran(const BatchArgs& a, const AtranArgs& t, int grid, cudaStream_t s) {
  k_atran<<<grid, 32, atran_smem(a), s>>>(a, t);
}

void atran_kernel_info(int region, int prog_ints, int* regs, int* blocks_per_sm) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_atran);
  *regs = fa.numRegs;
  const size_t sm = (size_t)prog_ints * 4 + (size_t)region * 8;
  cudaFuncSetAttribute(k_atran, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_atran, 32, sm);
}

}  // namespace gk
