// Oracle (test infrastructure only): the reference's adaptive transient
// restated.
//   waveforms                    crates/sim-core/src/waveform.rs:31-330
//   breakpoints, settling        crates/sim-core/src/waveform.rs:417-660
//   Milne's LTE estimate         crates/sim-core/src/analysis.rs:147-206
//   PI controller                crates/sim-core/src/analysis.rs:380-760
//   transient loop               crates/sim-core/src/engine.rs:332-602, 635-680
//   companion state              crates/sim-core/src/stamp.rs:572-668
#include <algorithm>
#include <cmath>

#include "oracle.h"

namespace oracle {

// ---------------------------------------------------------------- waveforms
double Waveform::eval(double t) const {
  switch (kind) {
    case 1: {  // PULSE (waveform.rs:82-112)
      const double v1 = p[0], v2 = p[1], td = p[2], tr = p[3], tf = p[4], pw = p[5], per = p[6];
      if (t < td) return v1;
      const double tr_ = per > 0.0 ? std::fmod(t - td, per) : t - td;
      if (tr_ < tr) return v1 + (v2 - v1) * tr_ / tr;
      if (tr_ < tr + pw) return v2;
      if (tr_ < tr + pw + tf) {
        const double tfall = tr_ - tr - pw;
        return v2 - (v2 - v1) * tfall / tf;
      }
      return v1;
    }
    case 2: {  // PWL (waveform.rs:147-176)
      if (pwl.empty()) return 0.0;
      if (t <= pwl.front().first) return pwl.front().second;
      if (t >= pwl.back().first) return pwl.back().second;
      for (size_t i = 0; i + 1 < pwl.size(); ++i) {
        const double t0 = pwl[i].first, v0 = pwl[i].second;
        const double t1 = pwl[i + 1].first, v1 = pwl[i + 1].second;
        if (t >= t0 && t < t1) {
          const double ratio = (t - t0) / (t1 - t0);
          return v0 + (v1 - v0) * ratio;
        }
      }
      return pwl.back().second;
    }
    case 3: {  // SIN (waveform.rs:212-226)
      const double vo = p[0], va = p[1], freq = p[2], td = p[3], theta = p[4];
      if (t < td) return vo;
      const double trel = t - td;
      const double phase = 2.0 * 3.141592653589793 * freq * trel;
      const double damping = theta > 0.0 ? std::exp(-theta * trel) : 1.0;
      return vo + va * std::sin(phase) * damping;
    }
    case 4: {  // EXP (waveform.rs:268-289)
      const double v1 = p[0], v2 = p[1], td1 = p[2], tau1 = p[3], td2 = p[4], tau2 = p[5];
      if (t < td1) return v1;
      double v = v1;
      const double e1 = 1.0 - std::exp(-(t - td1) / tau1);
      v += (v2 - v1) * e1;
      if (t >= td2) {
        const double e2 = 1.0 - std::exp(-(t - td2) / tau2);
        v += (v1 - v2) * e2;
      }
      return v;
    }
    default:
      return 0.0;
  }
}

// ---------------------------------------------------------------- breakpoints
void Breakpoints::add(double t) {  // add_breakpoint: a BTreeSet of times
  if (t < 0.0) return;
  auto it = std::lower_bound(times.begin(), times.end(), t);
  if (it == times.end() || *it != t) times.insert(it, t);
}

void Breakpoints::extract(const Waveform& w, double tstop) {
  if (w.kind == 1) {  // extract_pulse_breakpoints (waveform.rs:474-519)
    const double td = w.p[2], tr = w.p[3], tf = w.p[4], pw = w.p[5], per = w.p[6];
    double t = td;
    int count = 0;
    if (td > 0.0) add(td);
    while (t <= tstop && count < 10000) {
      add(t);
      const double t_high = t + tr;
      if (t_high > tstop) break;
      add(t_high);
      const double t_fall = t_high + pw;
      if (t_fall > tstop) break;
      add(t_fall);
      const double t_low = t_fall + tf;
      if (t_low > tstop) break;
      add(t_low);
      if (per > 0.0) {
        t = td + per * (double)(count + 1);
        count += 1;
      } else {
        break;
      }
    }
  } else if (w.kind == 2) {  // extract_pwl_breakpoints
    for (const auto& pt : w.pwl) add(pt.first);
  }
}

bool Breakpoints::next(double t, double& out) const {
  auto it = std::upper_bound(times.begin(), times.end(), t);
  if (it == times.end()) return false;
  out = *it;
  return true;
}

double Breakpoints::limit_dt(double t, double dt, double min_margin) const {  // :567-600
  double bp;
  if (next(t, bp)) {
    const double to_bp = bp - t;
    if (dt >= to_bp) return std::fmax(to_bp, min_margin);
    if (dt > 0.9 * to_bp) return to_bp;
    const double remaining = to_bp - dt;
    if (remaining < 0.1 * dt && remaining < min_margin * 10.0) return to_bp;
  }
  return dt;
}

bool Breakpoints::crossed(double t_prev, double t) const {  // (t_prev, t]
  auto it = std::upper_bound(times.begin(), times.end(), t_prev);
  return it != times.end() && *it <= t;
}

bool Breakpoints::update_settling(double t_prev, double t) {  // :617-633
  if (crossed(t_prev, t)) current_settling = settling_steps;
  if (current_settling > 0) {
    current_settling -= 1;
    return true;
  }
  return false;
}

double Breakpoints::settling_dt(double dt, double dt_min) const {
  return std::fmax(dt * settling_factor, dt_min);
}

// ---------------------------------------------------------------- LTE
Lte estimate_lte_milne(const Vec& x_be, const Vec& x_trap, double abs_tol, double rel_tol) {
  Lte r;
  double max_ratio = 0.0, max_raw = 0.0;
  size_t max_node = 0;
  const size_t m = std::min(x_be.size(), x_trap.size());
  for (size_t i = 0; i < m; ++i) {
    const double be = x_be[i], tr = x_trap[i];
    if (std::fabs(be) < 1e-30 && std::fabs(tr) < 1e-30) continue;
    const double lte = std::fabs(tr - be) / 3.0;
    const double tol = abs_tol + rel_tol * std::fmax(std::fabs(be), std::fabs(tr));
    const double ratio = tol > 0.0 ? lte / tol : 0.0;
    if (ratio > max_ratio) {
      max_ratio = ratio;
      max_node = i;
      max_raw = lte;
    }
  }
  double factor = 2.0;
  if (max_ratio > 1e-10) {
    const double raw = std::pow(1.0 / max_ratio, 0.5);
    factor = std::min(std::max(raw * 0.9, 0.1), 2.0);
  }
  r.error_norm = max_ratio;
  r.max_error_node = max_node;
  r.accept = max_ratio <= 1.0;
  r.suggested_factor = factor;
  r.raw_lte = max_raw;
  return r;
}

// ---------------------------------------------------------------- PI controller
double StepController::suggest_dt(double err, double dt) const {  // :497-523
  const double e_n = std::fmax(err, 1e-10);
  const double p_factor = std::pow(1.0 / e_n, k_p);
  const double i_factor = has_prev ? std::pow(1.0 / std::fmax(prev_error, 1e-10), k_i) : 1.0;
  const double raw = p_factor * i_factor * safety;
  return dt * std::min(std::max(raw, shrink), growth);
}

void StepController::record_step(double err, double dt, bool acc) {  // :533-551
  if (acc) {
    has_prev = true;
    prev_error = err;
    consecutive_rejects = 0;
    accepted += 1;
    min_dt_used = std::fmin(min_dt_used, dt);
    max_dt_used = std::fmax(max_dt_used, dt);
  } else {
    consecutive_rejects += 1;
    rejected += 1;
  }
}

double StepController::emergency_dt(double dt, double dt_min) const {  // :576-583
  if (consecutive_rejects <= 2) return dt * 0.5;
  if (consecutive_rejects <= 5) return dt * 0.25;
  if (consecutive_rejects <= 10) return dt * 0.1;
  return dt_min;
}

std::pair<bool, double> AdaptiveController::process_lte(const Lte& lte, double dt) {  // :720-743
  const bool accept = lte.accept && !pi.should_reject(lte.error_norm);
  double next;
  if (accept) {
    const double s = pi.suggest_dt(lte.error_norm, dt);
    pi.record_step(lte.error_norm, dt, true);
    next = std::min(std::max(s, dt_min), dt_max);
  } else {
    pi.record_step(lte.error_norm, dt, false);
    if (pi.is_struggling()) {
      next = pi.emergency_dt(dt, dt_min);
    } else {
      next = std::min(std::max(dt * lte.suggested_factor, dt_min), dt_max);
    }
  }
  return {accept, next};
}

// ---------------------------------------------------------------- the loop
namespace {
struct ATranCtx {
  const Circuit* c;
  double dt, be_sign;
  TranState st;
};
MnaSystem atran_build(void* p, const Vec& x, double gmin, double scale) {
  auto* t = static_cast<ATranCtx*>(p);
  return build_mna(*t->c, x, gmin, scale, t->dt, &t->st, t->be_sign);
}
double clampd(double v, double lo, double hi) { return std::min(std::max(v, lo), hi); }
}  // namespace

TranAdaptiveResult tran_adaptive(const Circuit& c, const std::vector<Waveform>& waves,
                                 const NewtonConfig& cfg, const std::string& solver_kind,
                                 double tstep, double tstop, double tstart, double tmax,
                                 double abs_tol, double rel_tol, double be_sign,
                                 const Vec& x_ic) {
  TranAdaptiveResult R;
  const size_t nc = c.node_count;
  Vec x(nc, 0.0);
  for (size_t i = 0; i < nc && i < x_ic.size(); ++i) x[i] = x_ic[i];
  auto solver = make_solver(solver_kind, nc);
  solver->prepare(nc);
  const double min_dt = std::fmax(tstep * 1e-6, 1e-15);
  const double max_dt = std::fmin(tmax, tstop / 10.0);
  AdaptiveController ctrl(min_dt, max_dt);
  Breakpoints bps;
  for (const Waveform& w : waves) bps.extract(w, tstop);
  double t = tstart, dt = std::fmin(tstep, max_dt);
  size_t consecutive = 0;
  const size_t max_consecutive = 10;
  // DC operating point (engine.rs:412-451), sources at tstart
  ATranCtx ctx{&c, 0.0, be_sign, {}};
  ctx.st.waves = &waves;
  ctx.st.t = tstart;
  ctx.st.cap_v.assign(c.ndev(), 0.0);
  ctx.st.cap_i.assign(c.ndev(), 0.0);
  NewtonResult dc = run_newton_with_stepping(cfg, x, atran_build, &ctx, *solver);
  R.newton_iterations += dc.iterations;
  if (!dc.converged) {
    R.status = 2;
    return R;
  }
  R.times.push_back(t);
  R.solutions.push_back(x);
  auto cap_voltage = [&](const Vec& v, size_t d) {
    const size_t a = (size_t)c.nodes[d * 4], b = (size_t)c.nodes[d * 4 + 1];
    return (a < v.size() ? v[a] : 0.0) - (b < v.size() ? v[b] : 0.0);
  };
  std::vector<double> cap_v(c.ndev(), 0.0), cap_i(c.ndev(), 0.0);  // both states' history
  for (size_t d = 0; d < c.ndev(); ++d)
    if (c.type[d] == DEV_C) cap_v[d] = cap_voltage(x, d);
  while (t < tstop) {
    dt = bps.limit_dt(t, dt, min_dt);
    if (bps.is_settling()) dt = bps.settling_dt(dt, min_dt);
    if (t + dt > tstop) dt = tstop - t;
    const double t_target = t + dt;
    ATranCtx be{&c, dt, be_sign, {}};
    be.st.waves = &waves;
    be.st.t = t_target;
    be.st.cap_v = cap_v;
    be.st.method = 0;
    Vec x_be = x;
    NewtonResult rb = run_newton_with_stepping(cfg, x_be, atran_build, &be, *solver);
    R.newton_iterations += rb.iterations;
    if (!rb.converged) {
      consecutive += 1;
      R.rejected += 1;
      if (consecutive >= max_consecutive) {
        R.status = 1;
        break;
      }
      dt = std::fmax(dt * 0.25, min_dt);
      continue;
    }
    ATranCtx tr{&c, dt, be_sign, {}};
    tr.st.waves = &waves;
    tr.st.t = t_target;
    tr.st.cap_v = cap_v;
    tr.st.cap_i = cap_i;
    tr.st.method = 1;
    Vec x_tr = x;
    NewtonResult rt = run_newton_with_stepping(cfg, x_tr, atran_build, &tr, *solver);
    R.newton_iterations += rt.iterations;
    if (!rt.converged) {
      consecutive += 1;
      R.rejected += 1;
      if (consecutive >= max_consecutive) {
        R.status = 1;
        break;
      }
      dt = std::fmax(dt * 0.25, min_dt);
      continue;
    }
    const Lte lte = estimate_lte_milne(x_be, x_tr, abs_tol, rel_tol);
    const std::pair<bool, double> pr = ctrl.process_lte(lte, dt);
    if (pr.first) {
      const double t_new = t + dt;
      bps.update_settling(t, t_new);
      x = x_tr;
      for (size_t d = 0; d < c.ndev(); ++d)  // update_transient_state_full / _state
        if (c.type[d] == DEV_C) {
          const double v = cap_voltage(x, d);
          cap_i[d] = c.p[d * NPARAM] * (v - cap_v[d]) / dt;
          cap_v[d] = v;
        }
      R.times.push_back(t_new);
      R.solutions.push_back(x);
      t = t_new;
      R.accepted += 1;
      consecutive = 0;
      dt = clampd(pr.second, min_dt, max_dt);
    } else {
      R.rejected += 1;
      consecutive += 1;
      if (consecutive >= max_consecutive) {
        R.status = 1;
        break;
      }
      dt = clampd(pr.second, min_dt, max_dt);
    }
  }
  return R;
}

}  // namespace oracle
