// Oracle (test infrastructure only): a flat C interface over the CPU
// restatement so that tests/ and bench.py's CPU-baseline leg can drive it
// through ctypes. Nothing in the product links this library.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "oracle.h"

using namespace oracle;

namespace {
Circuit make_circuit(int64_t node_count, int64_t ndev, const int32_t* type,
                     const int32_t* nodes, const double* p) {
  Circuit c;
  c.node_count = (size_t)node_count;
  c.type.assign(type, type + ndev);
  c.nodes.assign(nodes, nodes + ndev * 4);
  c.p.assign(p, p + ndev * NPARAM);
  return c;
}
IVec ivec(const int64_t* p, int64_t n) { return IVec(p, p + n); }
// The DC build closure of the sweep (engine.rs:761-775) over the current
// source value.
struct DcSweepCtx {
  const Circuit* c;
};
MnaSystem dc_sweep_build(void* p, const Vec& x, double gmin, double scale) {
  return build_mna(*static_cast<DcSweepCtx*>(p)->c, x, gmin, scale);
}
}  // namespace

extern "C" {

void* orc_solver_new(const char* kind, int64_t n) {
  return make_solver(kind, (size_t)n).release();
}
void orc_solver_free(void* h) { delete static_cast<LinearSolver*>(h); }

// BbdSolver with a known partition: assignment[i] = block or -1 (border).
void* orc_bbd_new(int64_t n, const int64_t* assignment, int64_t num_blocks) {
  return static_cast<LinearSolver*>(
      new BbdSolver((size_t)n, std::vector<int64_t>(assignment, assignment + n), (size_t)num_blocks));
}
// out[0..3] = num_blocks, border_start, border_size, uses_fallback; perm[n]
int orc_bbd_info(void* h, int64_t* out, int64_t* perm) {
  auto* b = dynamic_cast<BbdSolver*>(static_cast<LinearSolver*>(h));
  if (!b) return -1;
  const BbdDecomposition& d = b->decomposition();
  out[0] = (int64_t)d.num_blocks;
  out[1] = (int64_t)d.border_start;
  out[2] = (int64_t)d.border_size;
  out[3] = b->uses_fallback() ? 1 : 0;
  if (perm)
    for (size_t i = 0; i < d.perm.size(); ++i) perm[i] = (int64_t)d.perm[i];
  return 0;
}
void orc_prepare(void* h, int64_t n) { static_cast<LinearSolver*>(h)->prepare((size_t)n); }
const char* orc_name(void* h) { return static_cast<LinearSolver*>(h)->name(); }
void orc_reset(void* h) { static_cast<LinearSolver*>(h)->reset_pattern(); }

int orc_analyze(void* h, const int64_t* ap, int64_t aplen, const int64_t* ai,
                int64_t nnz) {
  return static_cast<LinearSolver*>(h)->analyze(ivec(ap, aplen), ivec(ai, nnz));
}
int orc_factor(void* h, const int64_t* ap, int64_t aplen, const int64_t* ai,
               const double* ax, int64_t nnz) {
  return static_cast<LinearSolver*>(h)->factor(ivec(ap, aplen), ivec(ai, nnz),
                                               Vec(ax, ax + nnz));
}
int orc_solve(void* h, double* rhs, int64_t len) {
  Vec r(rhs, rhs + len);
  int st = static_cast<LinearSolver*>(h)->solve(r);
  if (st == ST_OK) std::memcpy(rhs, r.data(), sizeof(double) * (size_t)len);
  return st;
}

// NativeKLU counters: out[0..5] = factor, refactor, nnz_l, nnz_u, nblocks,
// noffdiag; *rcond = rcond.
// out[0..6]: factor and refactor counts, nnz(L), nnz(U), blocks, coupling
// entries, growth-triggered re-pivots
int orc_klu_stats(void* h, int64_t* out, double* rcond) {
  auto* k = dynamic_cast<NativeKluSolver*>(static_cast<LinearSolver*>(h));
  if (!k) return -1;
  const KluStats& s = k->stats();
  out[0] = (int64_t)s.factor_count;
  out[1] = (int64_t)s.refactor_count;
  out[2] = (int64_t)s.nnz_l;
  out[3] = (int64_t)s.nnz_u;
  out[4] = (int64_t)s.nblocks;
  out[5] = (int64_t)s.noffdiag;
  out[6] = (int64_t)s.repivots;
  *rcond = s.rcond;
  return 0;
}

// NativeKLU pivot sequence: concatenation over blocks of row_perm (block
// local). Returns the number written, or -1.
int64_t orc_klu_pivots(void* h, int64_t* out, int64_t cap) {
  auto* k = dynamic_cast<NativeKluSolver*>(static_cast<LinearSolver*>(h));
  if (!k) return -1;
  int64_t w = 0;
  for (auto& nm : k->numeric())
    for (size_t r : nm.row_perm) {
      if (w < cap) out[w] = (int64_t)r;
      ++w;
    }
  return w;
}

// NativeKLU factor values for inspection: l values then u values of block b.
int64_t orc_klu_block_values(void* h, int64_t b, double* l, int64_t lcap,
                             double* u, int64_t ucap, int64_t* nl, int64_t* nu) {
  auto* k = dynamic_cast<NativeKluSolver*>(static_cast<LinearSolver*>(h));
  if (!k || b < 0 || (size_t)b >= k->numeric().size()) return -1;
  auto& nm = k->numeric()[(size_t)b];
  *nl = (int64_t)nm.l_val.size();
  *nu = (int64_t)nm.u_val.size();
  for (int64_t i = 0; i < *nl && i < lcap; ++i) l[i] = nm.l_val[(size_t)i];
  for (int64_t i = 0; i < *nu && i < ucap; ++i) u[i] = nm.u_val[(size_t)i];
  return 0;
}

void orc_amd(int64_t n, const int64_t* ap, const int64_t* ai, int64_t* perm,
             int64_t* inv) {
  AmdResult r = amd_order((size_t)n, ap, ai);
  for (int64_t i = 0; i < n; ++i) {
    perm[i] = (int64_t)r.perm[(size_t)i];
    inv[i] = (int64_t)r.inv_perm[(size_t)i];
  }
}

// info[0..3] = num_blocks, structural_rank, num_singletons, max_block_size
void orc_btf(int64_t n, const int64_t* ap, const int64_t* ai, int64_t* row_perm,
             int64_t* col_perm, int64_t* block_ptr, int64_t* info) {
  Btf b = btf_decompose((size_t)n, ap, ai);
  for (int64_t i = 0; i < n; ++i) {
    row_perm[i] = (int64_t)b.row_perm[(size_t)i];
    col_perm[i] = (int64_t)b.col_perm[(size_t)i];
  }
  for (size_t i = 0; i < b.block_ptr.size(); ++i) block_ptr[i] = (int64_t)b.block_ptr[i];
  info[0] = (int64_t)b.num_blocks;
  info[1] = (int64_t)b.structural_rank;
  info[2] = (int64_t)b.num_singletons;
  info[3] = (int64_t)b.max_block_size;
}

// MNA system of a circuit at x.
void* orc_mna(int64_t node_count, int64_t ndev, const int32_t* type,
              const int32_t* nodes, const double* p, const double* x,
              int64_t xlen, double gmin, double scale, double dt,
              const double* cap_v, double be_sign, double gdev) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  TranState st;
  if (cap_v) st.cap_v.assign(cap_v, cap_v + ndev);
  auto* s = new MnaSystem(build_mna(c, Vec(x, x + xlen), gmin, scale, dt,
                                    cap_v ? &st : nullptr, be_sign, gdev));
  return s;
}
void orc_mna_dims(void* h, int64_t* n, int64_t* nnz) {
  auto* s = static_cast<MnaSystem*>(h);
  *n = (int64_t)s->n;
  *nnz = (int64_t)s->ai.size();
}
void orc_mna_get(void* h, int64_t* ap, int64_t* ai, double* ax, double* rhs) {
  auto* s = static_cast<MnaSystem*>(h);
  std::memcpy(ap, s->ap.data(), sizeof(int64_t) * s->ap.size());
  std::memcpy(ai, s->ai.data(), sizeof(int64_t) * s->ai.size());
  std::memcpy(ax, s->ax.data(), sizeof(double) * s->ax.size());
  std::memcpy(rhs, s->rhs.data(), sizeof(double) * s->rhs.size());
}
void orc_mna_free(void* h) { delete static_cast<MnaSystem*>(h); }

// One DC operating point. cfg: max_iters, abs_tol, rel_tol, gmin, gmin_steps,
// source_steps. Returns the Newton exit reason; x_out gets min(n, x_cap)
// entries of the final x.
int orc_dc_op(int64_t node_count, int64_t ndev, const int32_t* type,
              const int32_t* nodes, const double* p, const char* solver_kind,
              int64_t max_iters, double abs_tol, double rel_tol, double gmin,
              int64_t gmin_steps, int64_t source_steps, const double* x0, double* x_out,
              int64_t x_cap, int64_t* x_len, int64_t* iters) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  cfg.gmin_steps = (size_t)gmin_steps;
  cfg.source_steps = (size_t)source_steps;
  auto solver = make_solver(solver_kind, c.node_count);
  Vec x;
  NewtonResult r = dc_op(c, cfg, *solver, x, x0);
  *x_len = (int64_t)x.size();
  for (int64_t i = 0; i < x_cap && (size_t)i < x.size(); ++i) x_out[i] = x[(size_t)i];
  *iters = (int64_t)r.iterations;
  return r.reason;
}

// DC operating point through the BbdSolver with a known partition.
int orc_dc_op_bbd(int64_t node_count, int64_t ndev, const int32_t* type, const int32_t* nodes,
                  const double* p, const int64_t* assignment, int64_t num_blocks,
                  int64_t max_iters, double abs_tol, double rel_tol, double gmin,
                  int64_t gmin_steps, const double* x0, double* x_out, int64_t x_cap,
                  int64_t* x_len, int64_t* iters) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  cfg.gmin_steps = (size_t)gmin_steps;
  size_t naux = 0;
  for (size_t d = 0; d < c.ndev(); ++d) naux += c.type[d] == DEV_V;
  std::vector<int64_t> asg(assignment, assignment + node_count);
  asg.resize(node_count + naux, -1);  // aux rows join the border
  BbdSolver solver(node_count + naux, asg, (size_t)num_blocks);
  Vec x;
  NewtonResult r = dc_op(c, cfg, solver, x, x0);
  *x_len = (int64_t)x.size();
  for (int64_t i = 0; i < x_cap && (size_t)i < x.size(); ++i) x_out[i] = x[(size_t)i];
  *iters = (int64_t)r.iterations;
  return r.reason;
}

// Fixed-step backward Euler (tran_be). states: (steps+1) * node_count.
int orc_tran(int64_t node_count, int64_t ndev, const int32_t* type, const int32_t* nodes,
             const double* p, const char* solver_kind, int64_t max_iters, double abs_tol,
             double rel_tol, double gmin, double dt, int64_t steps, const double* x_init,
             double* states, int64_t* iters) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  Vec st;
  size_t it = 0;
  int r = tran_be(c, cfg, solver_kind, dt, (size_t)steps, x_init, st, it);
  std::copy(st.begin(), st.end(), states);
  *iters = (int64_t)it;
  return r;
}

// AC sweep (ac_sweep): out_re/out_im hold nf x cap values; *n_out = n.
int orc_ac_sweep(int64_t node_count, int64_t ndev, const int32_t* type, const int32_t* nodes,
                 const double* p, const double* xdc, int64_t xlen, const double* freqs,
                 int64_t nf, double* out_re, double* out_im, int64_t cap, int64_t* n_out) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  std::vector<double> re, im;
  size_t n = 0;
  int r = ac_sweep(c, Vec(xdc, xdc + xlen), Vec(freqs, freqs + nf), re, im, n);
  *n_out = (int64_t)n;
  if (r != 0 || (int64_t)n > cap) return r != 0 ? r : 2;
  for (int64_t f = 0; f < nf; ++f)
    for (size_t i = 0; i < n; ++i) {
      out_re[f * cap + (int64_t)i] = re[(size_t)f * n + i];
      out_im[f * cap + (int64_t)i] = im[(size_t)f * n + i];
    }
  return 0;
}

// Discrete adjoint of orc_tran's loss (tran_adjoint); grad has ndev entries.
int orc_tran_adjoint(int64_t node_count, int64_t ndev, const int32_t* type,
                     const int32_t* nodes, const double* p, double dt, int64_t steps,
                     const double* states, int64_t probe, double target, double gmin,
                     double* grad) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  Vec st(states, states + (size_t)(steps + 1) * (size_t)node_count), g;
  int r = tran_adjoint(c, dt, (size_t)steps, st, (size_t)probe, target, gmin, g);
  std::copy(g.begin(), g.end(), grad);
  return r;
}

double orc_residual(int64_t node_count, int64_t ndev, const int32_t* type,
                    const int32_t* nodes, const double* p, const double* x,
                    int64_t xlen, double gmin) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  return residual_inf(c, Vec(x, x + xlen), gmin);
}

// Many independent DC operating points over a thread pool: instance i runs
// circuit inst_circ[i] with device inst_dev[i]'s first parameter replaced by
// inst_val[i] (inst_dev < 0: no override). Circuits are concatenated device
// lists delimited by dev_off[ncirc + 1]. Per instance: iterations, exit
// reason, and x (x_cap entries, zero padded).
// The reference's DC sweep (engine.rs:684-820): one solver, prepare(
// node_count) once (engine.rs:747) and x = zeros(node_count); per value the
// source's value is set and run_newton_with_stepping runs from x (the
// previous point's final iterate) or, when x0 is given, from that point's
// own initial iterate; a point that does not converge ends the sweep when
// stop != 0 (engine.rs:785-796). Points not run get reason -1.
void orc_dc_sweep(int64_t node_count, int64_t ndev, const int32_t* type, const int32_t* nodes,
                  const double* p, const char* solver_kind, int64_t max_iters, double abs_tol,
                  double rel_tol, double gmin, int64_t gmin_steps, int64_t src_dev,
                  const double* values, int64_t npts, const double* x0, int64_t x0_stride,
                  int stop, double* x_out, int64_t x_stride, int64_t* x_len, int64_t* iters,
                  int32_t* reason) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  cfg.gmin_steps = (size_t)gmin_steps;
  auto s = make_solver(solver_kind, c.node_count);
  for (int64_t k = 0; k < npts; ++k) {
    iters[k] = 0;
    reason[k] = -1;
    x_len[k] = 0;
  }
  s->prepare(c.node_count);
  Vec x(c.node_count, 0.0);
  for (int64_t k = 0; k < npts; ++k) {
    c.p[(size_t)src_dev * NPARAM] = values[k];
    NewtonResult r;
    if (x0) {
      r = dc_sweep_point(c, cfg, *s, x, x0 + k * x0_stride);
    } else {
      DcSweepCtx ctx{&c};
      r = run_newton_with_stepping(cfg, x, dc_sweep_build, &ctx, *s);
    }
    iters[k] = (int64_t)r.iterations;
    reason[k] = r.reason;
    x_len[k] = (int64_t)x.size();
    for (int64_t i = 0; i < x_stride; ++i)
      x_out[k * x_stride + i] = (size_t)i < x.size() ? x[(size_t)i] : 0.0;
    if (r.reason != NR_CONVERGED && stop) break;
  }
}

void orc_dc_batch(int64_t ncirc, const int64_t* dev_off, const int64_t* node_counts,
                  const int32_t* type, const int32_t* nodes, const double* p,
                  int64_t ninst, const int64_t* inst_circ, const int64_t* inst_dev,
                  const double* inst_val, const char* solver_kind, int64_t max_iters,
                  double abs_tol, double rel_tol, double gmin, int64_t gmin_steps,
                  const double* x0, const int64_t* x0_off, int64_t nthreads, int64_t* iters,
                  int32_t* reason, double* x_out, int64_t x_cap, int sweep,
                  int64_t* perturbed) {
  std::vector<Circuit> circs((size_t)ncirc);
  for (int64_t c = 0; c < ncirc; ++c) {
    int64_t d0 = dev_off[c], d1 = dev_off[c + 1];
    circs[(size_t)c] = make_circuit(node_counts[c], d1 - d0, type + d0,
                                    nodes + d0 * 4, p + d0 * NPARAM);
  }
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  cfg.gmin_steps = (size_t)gmin_steps;
  // sweep != 0: each circuit's instances are the points of that circuit's
  // DC sweep. As in the reference's sweep (engine.rs:684-820) one solver
  // serves every point and prepare(node_count) runs once before the first,
  // so the solver keeps the pattern and the pivots the first point's first
  // factorization chose (native_klu.rs:1020-1148) for all later points.
  // Unlike that sweep, every point starts from its own initial iterate and a
  // point that fails does not end the others.
  // sweep == 0: every instance is its own DC operating point (engine.rs:
  // 249-283), whose prepare(node_count) resets the pattern (a size other
  // than the matrix's, which has one aux row per voltage source), so each
  // instance's pivots come from its own first matrix.
  std::string kind(solver_kind);
  std::vector<std::vector<int64_t>> by_circ((size_t)ncirc);
  for (int64_t i = 0; i < ninst; ++i) by_circ[(size_t)inst_circ[i]].push_back(i);
  std::atomic<int64_t> next(0);
  auto worker = [&]() {
    while (true) {
      int64_t ci = next.fetch_add(1);
      if (ci >= ncirc) break;
      if (by_circ[(size_t)ci].empty()) continue;
      auto s = make_solver(kind, circs[(size_t)ci].node_count);
      s->prepare(circs[(size_t)ci].node_count);
      for (int64_t i : by_circ[(size_t)ci]) {
        Circuit c = circs[(size_t)ci];
        if (inst_dev[i] >= 0) c.p[(size_t)inst_dev[i] * NPARAM] = inst_val[i];
        Vec x;
        const double* xi = (x0 && x0_off && x0_off[i] >= 0) ? x0 + x0_off[i] : nullptr;
        const size_t p0 = perturbed_pivots;
        NewtonResult r = sweep ? dc_sweep_point(c, cfg, *s, x, xi) : dc_op(c, cfg, *s, x, xi);
        if (perturbed) perturbed[i] = (int64_t)(perturbed_pivots - p0);
        iters[i] = (int64_t)r.iterations;
        reason[i] = r.reason;
        double* xo = x_out ? x_out + i * x_cap : nullptr;
        if (xo)
          for (int64_t k = 0; k < x_cap; ++k)
            xo[k] = (size_t)k < x.size() ? x[(size_t)k] : 0.0;
      }
    }
  };
  int64_t nt = nthreads < 1 ? 1 : nthreads;
  std::vector<std::thread> th;
  for (int64_t t = 1; t < nt; ++t) th.emplace_back(worker);
  worker();
  for (auto& t : th) t.join();
}

}  // extern "C"

// ---------------------------------------------------------------- adaptive transient
namespace {
std::vector<Waveform> make_waves(int64_t n, const int32_t* kind, const double* p7,
                                 const int64_t* pwl_ptr, const double* pwl_t,
                                 const double* pwl_v) {
  std::vector<Waveform> w((size_t)n);
  for (int64_t d = 0; d < n; ++d) {
    w[d].kind = kind ? kind[d] : 0;
    if (p7)
      for (int k = 0; k < 7; ++k) w[d].p[k] = p7[d * 7 + k];
    if (pwl_ptr)
      for (int64_t q = pwl_ptr[d]; q < pwl_ptr[d + 1]; ++q) w[d].pwl.push_back({pwl_t[q], pwl_v[q]});
    // PwlParams::new sorts the points by time (a stable sort, waveform.rs:137-143)
    std::stable_sort(w[d].pwl.begin(), w[d].pwl.end(),
                     [](const std::pair<double, double>& a, const std::pair<double, double>& b) {
                       return a.first < b.first;
                     });
  }
  return w;
}
}  // namespace

extern "C" {

// Waveform values at nt times (kind and 7 parameters; PWL points).
void orc_wave_eval(int32_t kind, const double* p7, int64_t npwl, const double* pwl_t,
                   const double* pwl_v, int64_t nt, const double* ts, double* out) {
  int64_t ptr[2] = {0, npwl};
  std::vector<Waveform> w = make_waves(1, &kind, p7, ptr, pwl_t, pwl_v);
  for (int64_t i = 0; i < nt; ++i) out[i] = w[0].eval(ts[i]);
}

// Breakpoint times of nw sources (sorted, unique); returns their count.
int64_t orc_breakpoints(int64_t nw, const int32_t* kind, const double* p7,
                        const int64_t* pwl_ptr, const double* pwl_t, const double* pwl_v,
                        double tstop, double* out, int64_t cap) {
  std::vector<Waveform> w = make_waves(nw, kind, p7, pwl_ptr, pwl_t, pwl_v);
  Breakpoints b;
  for (const Waveform& x : w) b.extract(x, tstop);
  for (size_t i = 0; i < b.times.size() && (int64_t)i < cap; ++i) out[i] = b.times[i];
  return (int64_t)b.times.size();
}

// limit_dt over a breakpoint set.
double orc_bp_limit_dt(const double* times, int64_t n, double t, double dt, double margin) {
  Breakpoints b;
  for (int64_t i = 0; i < n; ++i) b.add(times[i]);
  return b.limit_dt(t, dt, margin);
}

// update_settling over a sequence of (t_prev, t) pairs; settling[i] gets
// the return value and is_settling afterwards (2 * i, 2 * i + 1).
void orc_bp_settling(const double* times, int64_t n, int64_t steps, double factor,
                     int64_t m, const double* tp, const double* tn, int32_t* out) {
  Breakpoints b;
  for (int64_t i = 0; i < n; ++i) b.add(times[i]);
  b.settling_steps = (size_t)steps;
  b.settling_factor = std::min(std::max(factor, 0.01), 1.0);
  for (int64_t i = 0; i < m; ++i) {
    out[2 * i] = b.update_settling(tp[i], tn[i]) ? 1 : 0;
    out[2 * i + 1] = b.is_settling() ? 1 : 0;
  }
}

// Milne's estimate: out = error_norm, max_error_node, accept, suggested_factor, raw_lte.
void orc_lte(const double* be, const double* tr, int64_t n, double abs_tol, double rel_tol,
             double* out) {
  Lte l = estimate_lte_milne(Vec(be, be + n), Vec(tr, tr + n), abs_tol, rel_tol);
  out[0] = l.error_norm;
  out[1] = (double)l.max_error_node;
  out[2] = l.accept ? 1.0 : 0.0;
  out[3] = l.suggested_factor;
  out[4] = l.raw_lte;
}

// A sequence of steps through the adaptive controller: step i feeds an LTE
// of error_norm err[i] (accept and suggested factor as Milne's estimate
// gives them) at dt[i] (dt[i] < 0: the previous step's next dt); out gets
// (accept, next_dt, struggling, pi_suggest) per step.
void orc_adaptive_sequence(double dt_min, double dt_max, int64_t m, const double* err,
                           const double* dt, double* out) {
  AdaptiveController c(dt_min, dt_max);
  double cur = 0.0;
  for (int64_t i = 0; i < m; ++i) {
    if (dt[i] >= 0.0) cur = dt[i];
    Lte l;
    l.error_norm = err[i];
    l.accept = err[i] <= 1.0;
    l.suggested_factor = err[i] > 1e-10 ? std::min(std::max(std::pow(1.0 / err[i], 0.5) * 0.9, 0.1), 2.0) : 2.0;
    const double s = c.pi.suggest_dt(err[i], cur);
    std::pair<bool, double> r = c.process_lte(l, cur);
    out[4 * i] = r.first ? 1.0 : 0.0;
    out[4 * i + 1] = r.second;
    out[4 * i + 2] = c.pi.is_struggling() ? 1.0 : 0.0;
    out[4 * i + 3] = s;
    cur = r.second;
  }
}

// The engine's adaptive transient (tran_adaptive). Per device a waveform
// (kind, 7 parameters, PWL points). times_out / sols_out: up to cap points,
// sols_out cap x n_cap values; stats = accepted, rejected, newton iterations,
// points; returns the status (0 completed, 1 rejections, 2 DC point failed).
int orc_tran_adaptive(int64_t node_count, int64_t ndev, const int32_t* type, const int32_t* nodes,
                      const double* p, const int32_t* wkind, const double* wp7,
                      const int64_t* pwl_ptr, const double* pwl_t, const double* pwl_v,
                      const char* solver_kind, int64_t max_iters, double abs_tol, double rel_tol,
                      double gmin, double tstep, double tstop, double tstart, double tmax,
                      double lte_abs, double lte_rel, double be_sign, const double* x_ic,
                      int64_t cap, int64_t n_cap, double* times_out, double* sols_out,
                      int64_t* stats) {
  Circuit c = make_circuit(node_count, ndev, type, nodes, p);
  std::vector<Waveform> w = make_waves(ndev, wkind, wp7, pwl_ptr, pwl_t, pwl_v);
  NewtonConfig cfg;
  cfg.max_iters = (size_t)max_iters;
  cfg.abs_tol = abs_tol;
  cfg.rel_tol = rel_tol;
  cfg.gmin = gmin;
  Vec xi(x_ic ? x_ic : nullptr, x_ic ? x_ic + node_count : nullptr);
  TranAdaptiveResult r = tran_adaptive(c, w, cfg, solver_kind, tstep, tstop, tstart, tmax,
                                       lte_abs, lte_rel, be_sign, xi);
  const int64_t np = (int64_t)r.times.size();
  for (int64_t i = 0; i < np && i < cap; ++i) {
    times_out[i] = r.times[i];
    const Vec& s = r.solutions[i];
    for (int64_t j = 0; j < n_cap; ++j) sols_out[i * n_cap + j] = j < (int64_t)s.size() ? s[j] : 0.0;
  }
  stats[0] = (int64_t)r.accepted;
  stats[1] = (int64_t)r.rejected;
  stats[2] = (int64_t)r.newton_iterations;
  stats[3] = np;
  return r.status;
}

}  // extern "C"
