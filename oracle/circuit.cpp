// Oracle (test infrastructure only): MNA assembly, device stamps and the
// Newton loop restated from the reference.
//   SparseBuilder / StampContext   crates/sim-core/src/mna.rs:89-168, 320-347, 452-525
//   stamps                         crates/sim-core/src/stamp.rs:242-297, 351-545, 759-787
//   level-1 MOSFET                 crates/sim-devices/src/bsim/evaluate.rs:285-356,
//                                  crates/sim-devices/src/bsim/mod.rs:430-476,
//                                  crates/sim-devices/src/bsim/params.rs:10, 460-462
//   Newton                         crates/sim-core/src/newton.rs:65-265
//   DC operating point             crates/sim-core/src/engine.rs:249-311
#include <algorithm>
#include <cmath>

#include "oracle.h"

namespace oracle {

namespace {
const double kEpsOx = 3.9 * 8.854e-12;  // params.rs:10
const double kGmin = 1e-12;             // evaluate.rs:50

// SparseBuilder in dynamic mode with the non-merging finalize().
struct Builder {
  size_t n;
  std::vector<std::vector<std::pair<size_t, double>>> cols;
  explicit Builder(size_t n_) : n(n_), cols(n_) {}
  void insert(size_t col, size_t row, double v) {  // mna.rs:151-168
    if (col >= n || row >= n) return;
    cols[col].push_back({row, v});
  }
  void resize(size_t nn) {  // mna.rs:235-255
    if (nn <= n) return;
    cols.resize(nn);
    n = nn;
  }
  void finalize(IVec& ap, IVec& ai, Vec& ax) {  // mna.rs:320-347
    ap.assign(1, 0);
    ai.clear();
    ax.clear();
    for (auto& c : cols) {
      std::stable_sort(c.begin(), c.end(),
                       [](const std::pair<size_t, double>& a,
                          const std::pair<size_t, double>& b) {
                         return a.first < b.first;
                       });
      for (auto& e : c) {
        ai.push_back((i64)e.first);
        ax.push_back(e.second);
      }
      ap.push_back((i64)ai.size());
    }
  }
};

struct Ctx {  // StampContext, mna.rs:452-481
  Builder& b;
  Vec& rhs;
  size_t node_count;
  size_t naux = 0;
  double gmin, scale;
  void add(size_t i, size_t j, double v) { b.insert(j, i, v); }
  void add_rhs(size_t i, double v) {
    if (i < rhs.size()) rhs[i] += v;
  }
  size_t allocate_aux() {  // every voltage source has its own name
    size_t id = naux++;
    b.resize(node_count + naux);
    rhs.resize(b.n, 0.0);
    return node_count + id;
  }
};

inline double xget(const Vec& x, size_t i) { return i < x.size() ? x[i] : 0.0; }
}  // namespace

MosOut eval_level1(double vth0, double u0, double tox, double w, double l,
                   double vd, double vg, double vs, bool is_pmos) {
  // evaluate_mos level 1 (mod.rs:440-455) -> evaluate_level1_dc (evaluate.rs:285-356)
  const double lambda = 0.02;
  double cox = kEpsOx / tox;
  double beta = u0 * 1e-4 * cox;
  double vd_i, vg_i, vs_i, sign;
  if (is_pmos) {
    vd_i = -vs;
    vg_i = -vg;
    vs_i = -vd;
    sign = -1.0;
  } else {
    vd_i = vd;
    vg_i = vg;
    vs_i = vs;
    sign = 1.0;
  }
  double vgs = vg_i - vs_i;
  double vds = vd_i - vs_i;
  if (vds < 0.0) {
    vds = -vds;
    vgs = vg_i - vd_i;
  }
  double vth = is_pmos ? -std::fabs(vth0) : std::fabs(vth0);
  double beff = beta * w / l;
  double ids, gm, gds;
  if (vgs <= vth) {
    ids = 0.0;
    gm = 0.0;
    gds = kGmin;
  } else if (vds < vgs - vth) {
    ids = beff * ((vgs - vth) * vds - 0.5 * vds * vds);
    gm = beff * vds;
    gds = std::fmax(beff * ((vgs - vth) - vds), kGmin);
  } else {
    double t = vgs - vth;
    ids = 0.5 * beff * (t * t) * (1.0 + lambda * vds);
    gm = beff * (vgs - vth) * (1.0 + lambda * vds);
    gds = std::fmax(0.5 * beff * (t * t) * lambda, kGmin);
  }
  MosOut o;
  o.ids = ids * sign;
  o.gm = gm;
  o.gds = gds;
  o.gmbs = 0.0;
  double vgs_o = vg - vs, vds_o = vd - vs;
  o.ieq = o.ids - gm * vgs_o - gds * vds_o;
  return o;
}

MosJ eval_level1_consistent(double vth0, double u0, double tox, double w,
                            double l, double vd, double vg, double vs,
                            bool is_pmos, double gdev) {
  // Level 1 with the constants of eval_level1 (lambda 0.02, beta from u0
  // and tox) in the Shichman-Hodges form: the (1 + lambda vds) factor
  // multiplies the current in the linear region too, so the current and its
  // partials are continuous where the linear and saturation regions meet
  // (the reference's linear region omits the factor, a 2 % current step
  // there on which Newton can cycle). The polarity is applied to every
  // terminal voltage and the drain/source roles swap when vds < 0, so
  // (ddg, ddd, dds) are the exact partials of id.
  const double lambda = 0.02;
  double beta = u0 * 1e-4 * (kEpsOx / tox);
  double pol = is_pmos ? -1.0 : 1.0;
  double vgs = pol * (vg - vs), vds = pol * (vd - vs);
  bool rev = vds < 0.0;
  double vgse = rev ? vgs - vds : vgs;
  double vdse = rev ? -vds : vds;
  double vth = std::fabs(vth0);
  double beff = beta * w / l;
  double ids, gm, gds;
  if (vgse <= vth) {
    ids = 0.0;
    gm = 0.0;
    gds = gdev;
  } else if (vdse < vgse - vth) {
    const double k = 1.0 + lambda * vdse;
    const double q = (vgse - vth) * vdse - 0.5 * vdse * vdse;
    ids = beff * q * k;
    gm = beff * vdse * k;
    gds = std::fmax(beff * ((vgse - vth) - vdse) * k + lambda * beff * q, gdev);
  } else {
    double t = vgse - vth;
    ids = 0.5 * beff * (t * t) * (1.0 + lambda * vdse);
    gm = beff * (vgse - vth) * (1.0 + lambda * vdse);
    gds = std::fmax(0.5 * beff * (t * t) * lambda, gdev);
  }
  MosJ j;
  if (!rev) {
    j.id = pol * ids;
    j.ddg = gm;
    j.ddd = gds;
    j.dds = -(gm + gds);
  } else {
    j.id = -pol * ids;
    j.ddg = -gm;
    j.ddd = gm + gds;
    j.dds = -gds;
  }
  return j;
}

namespace {
// A source's value: its waveform at the state's time, else its DC value.
double src_value(const Circuit& c, size_t d, const TranState* st) {
  if (st && st->waves && d < st->waves->size() && (*st->waves)[d].kind != 0)
    return (*st->waves)[d].eval(st->t);
  return c.p[d * NPARAM];
}
}  // namespace

MnaSystem build_mna(const Circuit& c, const Vec& x, double gmin,
                    double source_scale, double dt, const TranState* st,
                    double be_sign, double gdev) {
  MnaSystem s;
  Builder b(c.node_count);
  s.rhs.assign(c.node_count, 0.0);
  Ctx ctx{b, s.rhs, c.node_count, 0, gmin, source_scale};
  for (size_t d = 0; d < c.ndev(); ++d) {
    const int32_t* nd = &c.nodes[d * 4];
    const double* p = &c.p[d * NPARAM];
    size_t a = (size_t)nd[0], bb = (size_t)nd[1];
    switch (c.type[d]) {
      case DEV_R: {  // stamp.rs:242-259
        double g = 1.0 / p[0];
        ctx.add(a, a, g);
        ctx.add(bb, bb, g);
        ctx.add(a, bb, -g);
        ctx.add(bb, a, -g);
        break;
      }
      case DEV_I: {  // stamp.rs:261-276 (at time t: :331-349)
        double v = src_value(c, d, st) * ctx.scale;
        ctx.add_rhs(a, -v);
        ctx.add_rhs(bb, v);
        break;
      }
      case DEV_V: {  // stamp.rs:278-297 (at time t: :303-325)
        double v = src_value(c, d, st) * ctx.scale;
        size_t k = ctx.allocate_aux();
        ctx.add(a, k, 1.0);
        ctx.add(bb, k, -1.0);
        ctx.add(k, a, 1.0);
        ctx.add(k, bb, -1.0);
        ctx.add_rhs(k, v);
        break;
      }
      case DEV_D: {  // stamp.rs:351-387
        double gm_ = ctx.gmin > 0.0 ? ctx.gmin : 1e-12;
        double isat = p[0], vt = 0.02585 * p[1];
        double vdd = xget(x, a) - xget(x, bb);
        double e = std::exp(vdd / vt);
        double id = isat * (e - 1.0);
        double gd = (isat / vt) * e;
        double g = std::fmax(gd, gm_);
        double ieq = id - gd * vdd;
        ctx.add(a, a, g);
        ctx.add(bb, bb, g);
        ctx.add(a, bb, -g);
        ctx.add(bb, a, -g);
        ctx.add_rhs(a, -ieq);
        ctx.add_rhs(bb, ieq);
        break;
      }
      case DEV_M: {  // stamp.rs:389-545 (level-1 branch)
        size_t dr = (size_t)nd[0], gt = (size_t)nd[1], sr = (size_t)nd[2];
        double gm_ = ctx.gmin > 0.0 ? ctx.gmin : 1e-12;
        MosOut o = eval_level1(p[1], p[2], p[3], p[4], p[5], xget(x, dr),
                               xget(x, gt), xget(x, sr), p[0] != 0.0);
        double gm = o.gm, gds = std::fmax(o.gds, gm_);
        ctx.add(dr, dr, gds);
        ctx.add(sr, sr, gds);
        ctx.add(dr, sr, -gds);
        ctx.add(sr, dr, -gds);
        ctx.add(dr, gt, gm);
        ctx.add(dr, sr, -gm);
        ctx.add(sr, gt, -gm);
        ctx.add(sr, sr, gm);
        // gmbs is 0 for level 1, below gmin*0.01: not stamped (:519-524)
        ctx.add_rhs(dr, -o.ieq);
        ctx.add_rhs(sr, o.ieq);
        break;
      }
      case DEV_MC: {  // consistent level-1, same 8 matrix slots as DEV_M
        size_t dr = (size_t)nd[0], gt = (size_t)nd[1], sr = (size_t)nd[2];
        double vd = xget(x, dr), vg = xget(x, gt), vs = xget(x, sr);
        MosJ j = eval_level1_consistent(p[1], p[2], p[3], p[4], p[5], vd, vg, vs,
                                        p[0] != 0.0, gdev);
        double ieq = j.id - (j.ddg * vg + j.ddd * vd + j.dds * vs);
        ctx.add(dr, dr, j.ddd);
        ctx.add(sr, sr, -j.dds);
        ctx.add(dr, sr, j.dds);
        ctx.add(sr, dr, -j.ddd);
        ctx.add(dr, gt, j.ddg);
        ctx.add(dr, sr, 0.0);
        ctx.add(sr, gt, -j.ddg);
        ctx.add(sr, sr, 0.0);
        ctx.add_rhs(dr, -ieq);
        ctx.add_rhs(sr, ieq);
        break;
      }
      case DEV_C: {
        if (dt > 0.0 && st && st->method == 1) {  // trapezoidal, stamp.rs:871-915
          double g = 2.0 * p[0] / dt;
          double vprev = st->cap_v[d];
          double iprev = st->cap_i.empty() ? 0.0 : st->cap_i[d];
          double ieq = g * vprev + iprev;
          ctx.add(a, a, g);
          ctx.add(bb, bb, g);
          ctx.add(a, bb, -g);
          ctx.add(bb, a, -g);
          ctx.add_rhs(a, ieq);
          ctx.add_rhs(bb, -ieq);
        } else if (dt > 0.0) {  // backward Euler companion, stamp.rs:759-787
          double g = p[0] / dt;
          double vprev = st ? st->cap_v[d] : 0.0;
          double ieq = g * vprev;
          ctx.add(a, a, g);
          ctx.add(bb, bb, g);
          ctx.add(a, bb, -g);
          ctx.add(bb, a, -g);
          ctx.add_rhs(a, be_sign * ieq);
          ctx.add_rhs(bb, -be_sign * ieq);
        }
        break;  // DC: open circuit (stamp.rs:137)
      }
      default:
        break;
    }
  }
  b.insert(0, 0, 1.0);  // ground pin, engine.rs:280
  b.finalize(s.ap, s.ai, s.ax);
  s.n = b.n;
  return s;
}

// ---------------------------------------------------------------- Newton
static double norm2(const double* v, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += v[i] * v[i];
  return std::sqrt(s);
}

NewtonResult run_newton(const NewtonConfig& cfg, Vec& x, BuildFn build,
                        void* ctx, double gmin, double source_scale,
                        LinearSolver& solver) {  // newton.rs:65-117
  NewtonResult res;
  double damping = cfg.damping;
  double prev = 1.7976931348623157e308;
  res.reason = NR_MAXITERS;
  size_t iter = 0;
  for (size_t it = 0; it < cfg.max_iters; ++it) {
    iter = it + 1;
    MnaSystem s = build(ctx, x, gmin, source_scale);
    solver.prepare(s.n);
    if (solver.analyze(s.ap, s.ai) != ST_OK ||
        solver.factor(s.ap, s.ai, s.ax) != ST_OK || solver.solve(s.rhs) != ST_OK) {
      res.reason = NR_SOLVER_FAILURE;
      break;
    }
    Vec& xn = s.rhs;
    size_t m = std::min(xn.size(), x.size());
    Vec dx(m);
    for (size_t i = 0; i < m; ++i) dx[i] = xn[i] - x[i];
    double dxn = norm2(dx.data(), m);
    res.final_norm = norm2(xn.data(), xn.size());
    bool conv = true;  // check_convergence :187-191
    for (size_t i = 0; i < m; ++i)
      if (!(std::fabs(dx[i]) <= cfg.abs_tol + cfg.rel_tol * std::fabs(xn[i]))) {
        conv = false;
        break;
      }
    if (conv) {
      x = xn;
      res.converged = true;
      res.reason = NR_CONVERGED;
      break;
    }
    if (dxn > prev && damping > cfg.damping_min)
      damping = std::fmax(damping * 0.5, cfg.damping_min);
    prev = dxn;
    for (size_t i = 0; i < m; ++i) x[i] = x[i] + damping * (xn[i] - x[i]);
  }
  res.iterations = iter;
  return res;
}

NewtonResult run_newton_with_stepping(const NewtonConfig& cfg, Vec& x,
                                      BuildFn build, void* ctx,
                                      LinearSolver& solver) {  // :142-185
  double gstart = std::fmax(cfg.gmin * 1e3, 1e-6);
  NewtonResult last;
  last.reason = NR_MAXITERS;
  size_t total = 0;
  for (size_t gi = 0; gi <= cfg.gmin_steps; ++gi) {
    double gmin = cfg.gmin_steps == 0
                      ? cfg.gmin
                      : gstart + (cfg.gmin - gstart) * ((double)gi / (double)cfg.gmin_steps);
    for (size_t si = 0; si <= cfg.source_steps; ++si) {
      double scale = cfg.source_steps == 0 ? 1.0 : (double)si / (double)cfg.source_steps;
      NewtonResult r = run_newton(cfg, x, build, ctx, gmin, scale, solver);
      total += r.iterations;
      if (r.converged) {
        r.iterations = r.iterations;
        return r;
      }
      last = r;
    }
  }
  (void)total;
  return last;
}

namespace {
struct DcCtx {
  const Circuit* c;
};
MnaSystem dc_build(void* p, const Vec& x, double gmin, double scale) {
  return build_mna(*static_cast<DcCtx*>(p)->c, x, gmin, scale);
}
}  // namespace

NewtonResult dc_op(const Circuit& c, const NewtonConfig& cfg,
                   LinearSolver& solver, Vec& x, const double* x0) {  // engine.rs:249-283
  x.assign(c.node_count, 0.0);
  if (x0)  // an initial iterate (nodeset) in place of the zero start
    for (size_t i = 0; i < c.node_count; ++i) x[i] = x0[i];
  solver.prepare(c.node_count);
  DcCtx ctx{&c};
  return run_newton_with_stepping(cfg, x, dc_build, &ctx, solver);
}

NewtonResult dc_sweep_point(const Circuit& c, const NewtonConfig& cfg, LinearSolver& solver,
                            Vec& x, const double* x0) {  // engine.rs:750-775
  x.assign(c.node_count, 0.0);
  if (x0)
    for (size_t i = 0; i < c.node_count; ++i) x[i] = x0[i];
  DcCtx ctx{&c};
  return run_newton_with_stepping(cfg, x, dc_build, &ctx, solver);
}

double residual_inf(const Circuit& c, const Vec& x, double gmin) {
  MnaSystem s = build_mna(c, x, gmin, 1.0);
  size_t n = s.n;
  Vec r(n, 0.0), arow(n, 0.0);
  for (size_t col = 0; col < n; ++col) {
    double xc = col < x.size() ? x[col] : 0.0;
    for (i64 idx = s.ap[col]; idx < s.ap[col + 1]; ++idx) {
      r[(size_t)s.ai[idx]] += s.ax[idx] * xc;
      arow[(size_t)s.ai[idx]] += std::fabs(s.ax[idx]);
    }
  }
  double rn = 0.0, an = 0.0, xn = 0.0, bn = 0.0;
  for (size_t i = 0; i < n; ++i) {
    rn = std::fmax(rn, std::fabs(r[i] - s.rhs[i]));
    an = std::fmax(an, arow[i]);
    bn = std::fmax(bn, std::fabs(s.rhs[i]));
    xn = std::fmax(xn, std::fabs(i < x.size() ? x[i] : 0.0));
  }
  double den = an * xn + bn;
  return den > 0.0 ? rn / den : rn;
}


// ---------------------------------------------------------------- transient
namespace {
struct TranCtx {
  const Circuit* c;
  double dt;
  TranState st;
};
MnaSystem tran_build(void* p, const Vec& x, double gmin, double scale) {
  auto* t = static_cast<TranCtx*>(p);
  return build_mna(*t->c, x, gmin, scale, t->dt, &t->st, 1.0);
}

// Dense LU with partial pivoting (row-major), in place; piv[k] = row swapped
// into k. Returns false on an exactly zero pivot.
bool dense_lu(std::vector<double>& a, size_t n, std::vector<size_t>& piv) {
  piv.resize(n);
  for (size_t k = 0; k < n; ++k) {
    size_t p = k;
    double best = std::fabs(a[k * n + k]);
    for (size_t i = k + 1; i < n; ++i)
      if (std::fabs(a[i * n + k]) > best) {
        best = std::fabs(a[i * n + k]);
        p = i;
      }
    if (best == 0.0) return false;
    piv[k] = p;
    if (p != k)
      for (size_t j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
    for (size_t i = k + 1; i < n; ++i) {
      const double l = a[i * n + k] / a[k * n + k];
      a[i * n + k] = l;
      for (size_t j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
    }
  }
  return true;
}

// Solves A^T y = b with P A = L U: U^T z = b, L^T w = z, y = P^T w.
void dense_tsolve(const std::vector<double>& lu, size_t n, const std::vector<size_t>& piv,
                  Vec& b) {
  for (size_t k = 0; k < n; ++k) {
    double s = b[k];
    for (size_t j = 0; j < k; ++j) s -= lu[j * n + k] * b[j];
    b[k] = s / lu[k * n + k];
  }
  for (size_t k = n; k-- > 0;) {
    double s = b[k];
    for (size_t i = k + 1; i < n; ++i) s -= lu[i * n + k] * b[i];
    b[k] = s;
  }
  for (size_t k = n; k-- > 0;)
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
}
}  // namespace

int tran_be(const Circuit& c, const NewtonConfig& cfg, const std::string& solver_kind,
            double dt, size_t steps, const double* x_init, Vec& states, size_t& iters) {
  const size_t nc = c.node_count;
  states.assign((steps + 1) * nc, 0.0);
  Vec x(x_init, x_init + nc);
  std::copy(x.begin(), x.end(), states.begin());
  TranCtx ctx{&c, dt, {}};
  ctx.st.cap_v.assign(c.ndev(), 0.0);
  auto solver = make_solver(solver_kind, nc);
  iters = 0;
  for (size_t t = 1; t <= steps; ++t) {
    for (size_t d = 0; d < c.ndev(); ++d)
      if (c.type[d] == DEV_C) {
        const int a = c.nodes[d * 4], b = c.nodes[d * 4 + 1];
        ctx.st.cap_v[d] = x[(size_t)a] - x[(size_t)b];
      }
    Vec xn(x.begin(), x.begin() + nc);
    NewtonResult r = run_newton(cfg, xn, tran_build, &ctx, cfg.gmin, 1.0, *solver);
    iters += r.iterations;
    if (!r.converged) return r.reason == NR_CONVERGED ? NR_MAXITERS : r.reason;
    std::copy(xn.begin(), xn.begin() + nc, x.begin());
    std::copy(x.begin(), x.end(), states.begin() + t * nc);
  }
  return 0;
}

int tran_adjoint(const Circuit& c, double dt, size_t steps, const Vec& states, size_t probe,
                 double target, double gmin, Vec& grad) {
  const size_t nc = c.node_count;
  grad.assign(c.ndev(), 0.0);
  Vec lam_next;  // lambda_{t+1}
  TranState st;
  st.cap_v.assign(c.ndev(), 0.0);
  for (size_t t = steps; t >= 1; --t) {
    Vec xt(states.begin() + t * nc, states.begin() + (t + 1) * nc);
    MnaSystem s = build_mna(c, xt, gmin, 1.0, dt, &st, 1.0, 0.0);
    const size_t n = s.n;
    std::vector<double> a(n * n, 0.0);
    for (size_t col = 0; col < n; ++col)
      for (i64 q = s.ap[col]; q < s.ap[col + 1]; ++q) a[(size_t)s.ai[q] * n + col] += s.ax[q];
    std::vector<size_t> piv;
    if (!dense_lu(a, n, piv)) return 1;
    if (lam_next.empty()) lam_next.assign(n, 0.0);
    Vec rhs(n, 0.0);
    rhs[probe] += 2.0 * (xt[probe] - target);
    for (size_t d = 0; d < c.ndev(); ++d)
      if (c.type[d] == DEV_C) {
        const size_t ca = (size_t)c.nodes[d * 4], cb = (size_t)c.nodes[d * 4 + 1];
        const double gl = c.p[d * NPARAM] / dt * (lam_next[ca] - lam_next[cb]);
        rhs[ca] += gl;
        rhs[cb] -= gl;
      }
    dense_tsolve(a, n, piv, rhs);
    const double* xp = &states[(t - 1) * nc];
    for (size_t d = 0; d < c.ndev(); ++d)
      if (c.type[d] == DEV_C) {
        const size_t ca = (size_t)c.nodes[d * 4], cb = (size_t)c.nodes[d * 4 + 1];
        const double dv = (xt[ca] - xt[cb]) - (xp[ca] - xp[cb]);
        grad[d] -= (rhs[ca] - rhs[cb]) * dv / dt;
      }
    lam_next = rhs;
  }
  return 0;
}

}  // namespace oracle
