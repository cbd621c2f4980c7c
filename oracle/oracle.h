// Oracle: a CPU restatement of RustSpice's Newton inner loop.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product (rustspice_gb300/, include/)
// links, includes or calls this code. It is the checker that the CUDA path is
// compared against, and the timed CPU baseline in bench.py. Each function
// cites the reference file:line (paths inside easyfly007/rustspice) it
// restates.
//
// Arithmetic follows the reference exactly: no fused multiply-add (the build
// uses -ffp-contract=off, matching Rust, which never contracts), the same
// loop orders, the same pivot and perturbation rules.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace oracle {

using i64 = int64_t;
using Vec = std::vector<double>;
using IVec = std::vector<i64>;
using UVec = std::vector<size_t>;

// ---------------------------------------------------------------- statuses
// Mirrors SolverError (crates/sim-core/src/solver.rs:76-92) as integers.
enum Status : int {
  ST_OK = 0,
  ST_ANALYZE_FAILED = 1,
  ST_FACTOR_FAILED = 2,
  ST_SOLVE_FAILED = 3,
  ST_SINGULAR = 4,
  ST_ILL_CONDITIONED = 5,
  ST_INVALID_MATRIX = 6,
};

// ---------------------------------------------------------------- AMD
// crates/sim-core/src/amd.rs:143-412
struct AmdResult {
  UVec perm;      // perm[old] = new
  UVec inv_perm;  // inv_perm[new] = old
};
AmdResult amd_order(size_t n, const i64* ap, const i64* ai);

// ---------------------------------------------------------------- BTF
// crates/sim-core/src/btf.rs:59-177, 202-550, 560-573
struct Btf {
  UVec row_perm, col_perm, row_perm_inv, col_perm_inv, block_ptr;
  size_t num_blocks = 0, structural_rank = 0, num_singletons = 0,
         max_block_size = 0;
  size_t block_size(size_t k) const {
    return k < num_blocks ? block_ptr[k + 1] - block_ptr[k] : 0;
  }
};
Btf btf_decompose(size_t n, const i64* ap, const i64* ai);
bool should_use_btf(size_t n, size_t nnz);

// ---------------------------------------------------------------- solvers
// The LinearSolver trait, crates/sim-core/src/solver.rs:141-166.
class LinearSolver {
 public:
  virtual ~LinearSolver() = default;
  virtual void prepare(size_t n) = 0;
  virtual int analyze(const IVec& ap, const IVec& ai) = 0;
  virtual int factor(const IVec& ap, const IVec& ai, const Vec& ax) = 0;
  virtual int solve(Vec& rhs) = 0;
  virtual void reset_pattern() = 0;
  virtual const char* name() const = 0;
  virtual void set_parallel_threads(size_t) {}
};

// DenseSolver, crates/sim-core/src/solver.rs:596-724
class DenseSolver : public LinearSolver {
 public:
  explicit DenseSolver(size_t n);
  void prepare(size_t n) override;
  int analyze(const IVec&, const IVec&) override { return ST_OK; }
  int factor(const IVec& ap, const IVec& ai, const Vec& ax) override;
  int solve(Vec& rhs) override;
  void reset_pattern() override {}
  const char* name() const override { return "Dense"; }

 private:
  size_t n_;
  Vec lu_;
  UVec pivots_;
};

// SparseLuSolver, crates/sim-core/src/sparse_lu.rs:118-745
class SparseLuSolver : public LinearSolver {
 public:
  explicit SparseLuSolver(size_t n);
  void prepare(size_t n) override;
  int analyze(const IVec& ap, const IVec& ai) override;
  int factor(const IVec& ap, const IVec& ai, const Vec& ax) override;
  int solve(Vec& rhs) override;
  void reset_pattern() override;
  const char* name() const override { return "SparseLU"; }
  size_t nnz_l() const { return nnz_l_; }
  size_t nnz_u() const { return nnz_u_; }
  size_t factor_count = 0;

 private:
  void symbolic(const IVec& ap, const IVec& ai);
  void numeric(const IVec& ap, const IVec& ai, const Vec& ax);
  size_t n_;
  UVec perm_, inv_perm_, l_ptr_, l_idx_, u_ptr_, u_idx_;
  Vec l_val_, u_val_, work_;
  UVec mark_;
  size_t cur_mark_ = 0;
  bool analyzed_ = false, factored_ = false;
  IVec last_ap_, last_ai_;
  size_t nnz_l_ = 0, nnz_u_ = 0;
};

// SparseLuBtfSolver, crates/sim-core/src/sparse_lu_btf.rs:71-690
class SparseLuBtfSolver : public LinearSolver {
 public:
  explicit SparseLuBtfSolver(size_t n);
  void prepare(size_t n) override;
  int analyze(const IVec& ap, const IVec& ai) override;
  int factor(const IVec& ap, const IVec& ai, const Vec& ax) override;
  int solve(Vec& rhs) override;
  void reset_pattern() override;
  const char* name() const override {
    return has_btf_ ? "SparseLU-BTF" : "SparseLU";
  }
  bool uses_btf() const { return has_btf_; }
  size_t factor_count = 0;

 private:
  struct OffDiag {
    size_t block_row, block_col, row_start, col_start, nrows, ncols;
    UVec col_ptr, row_idx;
    Vec values;
  };
  int analyze_btf(const IVec& ap, const IVec& ai);
  size_t n_;
  bool has_btf_ = false;
  Btf btf_;
  std::vector<SparseLuSolver> blocks_;
  std::vector<OffDiag> off_;
  Vec work_;
  bool use_btf_ = true;
  bool has_fallback_ = false;
  std::vector<SparseLuSolver> fallback_;  // 0 or 1 element
  IVec last_ap_, last_ai_;
  bool analyzed_ = false, factored_ = false;
};

// NativeKluSolver, crates/sim-core/src/native_klu.rs:49-71, 605-1685
struct KluConfig {
  double pivot_tol = 0.001;
  int ordering = 0;  // 0 = AMD, 3 = natural
  bool use_btf = true;
  size_t btf_min_blocks = 2;
  // false: the reference's rule (Q6): threshold row swaps are applied inside
  // the symbolic pattern computed without pivoting, so entries that a swap
  // moves outside that pattern are dropped.
  // true: "static pivoting with re-analysis": the same first-factor pass
  // chooses the row permutation, then the symbolic pattern is recomputed for
  // the row-permuted block and every factorization (the first included)
  // refactors that exact pattern with the frozen pivots.
  bool exact_pivots = false;
  // Growth-triggered re-pivot (not in the reference, whose refactorization
  // always keeps the first pivots): after a refactorization, a BTF block
  // with a multiplier |l_ik| above 1 / pivot_tol (its kept pivot is smaller
  // than pivot_tol times the column's largest entry below it, the threshold
  // the first factorization swaps on) is factored afresh: new pivots by the
  // first-factorization pass and, in exact mode, its exact pattern for them.
  // In the reference's mode a trigger refactors every block afresh.
  bool repivot = false;
};

// Pivots the NativeKLU factorization replaced by its +-1e-14 perturbation
// (native_klu.rs:1229-1231, 1344-1348) on this thread so far (a diagnostic
// of the oracle; the reference keeps no such count).
extern thread_local size_t perturbed_pivots;

struct KluStats {
  size_t factor_count = 0, refactor_count = 0, nnz_l = 0, nnz_u = 0,
         nblocks = 0, noffdiag = 0, repivots = 0;
  double rcond = 0.0;
};

class NativeKluSolver : public LinearSolver {
 public:
  struct Symbolic {
    size_t n = 0;
    UVec col_perm, col_perm_inv, l_ptr, l_idx, u_ptr, u_idx;
  };
  struct Numeric {
    Vec l_val, u_val, u_diag;
    UVec row_perm, row_perm_inv;
  };
  struct OffDiag {
    size_t block_row, block_col, row_start, col_start, nrows, ncols;
    UVec col_ptr, row_idx;
    Vec values;
  };

  explicit NativeKluSolver(size_t n, KluConfig cfg = KluConfig());
  void prepare(size_t n) override;
  int analyze(const IVec& ap, const IVec& ai) override;
  int factor(const IVec& ap, const IVec& ai, const Vec& ax) override;
  int solve(Vec& rhs) override;
  void reset_pattern() override;
  const char* name() const override { return "NativeKLU"; }
  const KluStats& stats() const { return stats_; }

  // Introspection used by the parity tests.
  bool has_btf() const { return has_btf_; }
  const Btf& btf() const { return btf_; }
  const std::vector<Symbolic>& symbolic() const { return sym_; }
  const std::vector<Numeric>& numeric() const { return num_; }

 private:
  enum State { EMPTY, ANALYZED, FACTORED };
  int do_analyze(const IVec& ap, const IVec& ai);
  int do_factor(const IVec& ap, const IVec& ai, const Vec& ax);
  bool growth(const Numeric& nm) const;
  int refactor_afresh(const IVec& ap, const IVec& ai, const Vec& ax);
  Symbolic symbolic_for_block(size_t n, const IVec& ap, const IVec& ai) const;
  static void symbolic_dfs(size_t n, const IVec& pap, const IVec& pai,
                           Symbolic& s);
  Symbolic resymbolic(const Symbolic& sym, const Numeric& num, const IVec& ap,
                      const IVec& ai) const;
  Numeric factor_block(const Symbolic& sym, const IVec& ap, const IVec& ai,
                       const Vec& ax, const Numeric* old, bool refactor) const;
  void solve_block(const Symbolic& sym, const Numeric& num, double* rhs) const;
  bool pattern_matches(const IVec& ap, const IVec& ai) const {
    return last_ap_ == ap && last_ai_ == ai;
  }

  size_t n_;
  KluConfig cfg_;
  bool has_btf_ = false;
  Btf btf_;
  std::vector<Symbolic> sym_;
  std::vector<Symbolic> sym_free_;  // the pivot-free patterns (re-pivot)
  std::vector<Numeric> num_;
  std::vector<OffDiag> off_;
  IVec last_ap_, last_ai_;
  State state_ = EMPTY;
  KluStats stats_;
  Vec work_;
};

// ---------------------------------------------------------------- circuits
// A circuit is a flat list of device instances in netlist order (the order
// the engine stamps them, crates/sim-core/src/engine.rs:262-279). Node 0 is
// ground and stays in the matrix (crates/sim-core/src/circuit.rs:31-57).
enum DevType : int32_t {
  DEV_R = 0,  // p[0] = resistance
  DEV_V = 1,  // p[0] = volts
  DEV_I = 2,  // p[0] = amps
  DEV_D = 3,  // p[0] = Is, p[1] = N
  DEV_M = 4,  // p[0] = is_pmos, p[1] = vth0, p[2] = u0, p[3] = tox, p[4] = W, p[5] = L
  DEV_C = 5,  // p[0] = capacitance
  // Level-1 MOSFET with a self-consistent Jacobian: polarity applied to all
  // terminal voltages and the drain/source roles swapped when vds < 0. The
  // reference's evaluator flips PMOS into a frame where the stamped gm/gds are
  // not the derivatives of the stamped current, so its Newton diverges on
  // CMOS circuits; this type is the documented physical alternative, in the
  // Shichman-Hodges form (lambda factor in the linear region too, so the
  // current is continuous between regions). Same parameters as DEV_M.
  DEV_MC = 6,
};
constexpr int NPARAM = 6;

struct Circuit {
  size_t node_count = 0;           // includes ground
  std::vector<int32_t> type;       // [ndev]
  std::vector<int32_t> nodes;      // [ndev * 4]
  std::vector<double> p;           // [ndev * NPARAM]
  size_t ndev() const { return type.size(); }
};

// SparseBuilder (non-merging finalize) and StampContext,
// crates/sim-core/src/mna.rs:89-168, 320-347, 452-525.
struct MnaSystem {
  size_t n = 0;
  IVec ap, ai;
  Vec ax, rhs;
};

// Time-dependent source value (crates/sim-core/src/waveform.rs:31-330):
// kind 0 none (the device's DC value), 1 PULSE(v1 v2 td tr tf pw per),
// 2 PWL (points), 3 SIN(vo va freq td theta), 4 EXP(v1 v2 td1 tau1 td2 tau2).
struct Waveform {
  int kind = 0;
  double p[7] = {0, 0, 0, 0, 0, 0, 0};
  std::vector<std::pair<double, double>> pwl;  // sorted by time
  double eval(double t) const;
};

// Companion state of the transient (crates/sim-core/src/stamp.rs:572-668):
// the capacitor voltage at the last accepted point and, for the trapezoidal
// rule, its current; the integration method; the time the sources are
// evaluated at.
struct TranState {
  std::vector<double> cap_v;  // indexed by device id (0 for non-capacitors)
  std::vector<double> cap_i;  // trapezoidal history current (empty: 0)
  int method = 0;             // 0 backward Euler, 1 trapezoidal
  double t = 0.0;
  const std::vector<Waveform>* waves = nullptr;  // per device, or null
};

// Builds the MNA system at x the way the engine's build closure does
// (crates/sim-core/src/engine.rs:262-283): stamp every instance, pin ground,
// finalize without merging. `x` may be shorter than n (node voltages only).
// When `dt > 0` capacitors use the backward-Euler companion
// (crates/sim-core/src/stamp.rs:759-787) with `be_sign` = -1 for the
// reference's sign and +1 for the physical one; dt <= 0 is DC (C open).
// gdev: the consistent MOSFET model's conductance floor (1e-12; 0 gives the
// exact Jacobian of the residual).
MnaSystem build_mna(const Circuit& c, const Vec& x, double gmin,
                    double source_scale, double dt = 0.0,
                    const TranState* st = nullptr, double be_sign = -1.0,
                    double gdev = 1e-12);

// Level-1 MOSFET, crates/sim-devices/src/bsim/evaluate.rs:285-356 via
// evaluate_mos, crates/sim-devices/src/bsim/mod.rs:430-476.
struct MosOut {
  double ids, gm, gds, gmbs, ieq;
};
MosOut eval_level1(double vth0, double u0, double tox, double w, double l,
                   double vd, double vg, double vs, bool is_pmos);
// Consistent level-1: current into the drain and its partial derivatives
// with respect to (vg, vd, vs).
struct MosJ {
  double id, ddg, ddd, dds;
};
MosJ eval_level1_consistent(double vth0, double u0, double tox, double w,
                            double l, double vd, double vg, double vs,
                            bool is_pmos, double gdev = 1e-12);

// AC small-signal sweep at a DC solution (crates/sim-core/src/engine.rs:
// 829-930 with the AC stamps and the dense complex LU; ac.cpp). V and I
// sources carry the AC magnitude in p[1] and the phase [deg] in p[2]. out_re
// and out_im get freqs.size() x n values; returns 0, or 1 on a pivot below
// 1e-30.
int ac_sweep(const Circuit& c, const Vec& xdc, const Vec& freqs, std::vector<double>& out_re,
             std::vector<double>& out_im, size_t& n_out);

// ---------------------------------------------------------------- Newton
// crates/sim-core/src/newton.rs:1-265
struct NewtonConfig {
  size_t max_iters = 50;
  double abs_tol = 1e-9, rel_tol = 1e-6, gmin = 1e-12, damping = 1.0,
         damping_min = 0.1;
  size_t gmin_steps = 0, source_steps = 0;
};
enum NewtonReason { NR_CONVERGED = 0, NR_MAXITERS = 1, NR_SOLVER_FAILURE = 2 };
struct NewtonResult {
  bool converged = false;
  size_t iterations = 0;
  double final_norm = 0.0;
  int reason = NR_MAXITERS;
};

// build(x, gmin, source_scale) -> system
using BuildFn = MnaSystem (*)(void* ctx, const Vec& x, double gmin,
                              double source_scale);

NewtonResult run_newton(const NewtonConfig& cfg, Vec& x, BuildFn build,
                        void* ctx, double gmin, double source_scale,
                        LinearSolver& solver);
NewtonResult run_newton_with_stepping(const NewtonConfig& cfg, Vec& x,
                                      BuildFn build, void* ctx,
                                      LinearSolver& solver);

// Engine DC operating point (crates/sim-core/src/engine.rs:249-311) on a
// circuit. `x` returns the solution (length n when converged).
// One point of the engine's DC sweep (engine.rs:684-820): the sweep calls
// prepare(node_count) once before its first point, so its solver keeps the
// pattern and pivots the first point found; each point here starts from x0
// (or zero) instead of the previous point's solution.
NewtonResult dc_sweep_point(const Circuit& c, const NewtonConfig& cfg, LinearSolver& solver,
                            Vec& x, const double* x0);
NewtonResult dc_op(const Circuit& c, const NewtonConfig& cfg,
                   LinearSolver& solver, Vec& x, const double* x0 = nullptr);

// Nonlinear residual F(x) = A(x) x - b(x) with the stamps at x, in the
// infinity norm, divided by max(|b|_inf, 1).
double residual_inf(const Circuit& c, const Vec& x, double gmin);

std::unique_ptr<LinearSolver> make_solver(const std::string& kind, size_t n);

// ---------------------------------------------------------------- adaptive transient
// Breakpoints of PULSE and PWL sources (waveform.rs:417-660; the engine
// extracts only those two kinds, engine.rs:635-680): sorted, unique.
struct Breakpoints {
  std::vector<double> times;
  size_t settling_steps = 5, current_settling = 0;
  double settling_factor = 0.1;
  void add(double t);
  void extract(const Waveform& w, double tstop);
  bool next(double t, double& out) const;
  double limit_dt(double t, double dt, double min_margin) const;
  bool crossed(double t_prev, double t) const;
  bool update_settling(double t_prev, double t);
  double settling_dt(double dt, double dt_min) const;
  bool is_settling() const { return current_settling > 0; }
};

// Milne's device (analysis.rs:147-206).
struct Lte {
  double error_norm = 0.0, suggested_factor = 2.0, raw_lte = 0.0;
  size_t max_error_node = 0;
  bool accept = true;
};
Lte estimate_lte_milne(const Vec& x_be, const Vec& x_trap, double abs_tol, double rel_tol);

// PI step controller and the adaptive controller around it
// (analysis.rs:380-760), trapezoidal gains k_p = 0.35, k_i = 0.2.
struct StepController {
  double k_p = 0.35, k_i = 0.2, growth = 2.0, shrink = 0.1, safety = 0.9, reject = 1.0;
  bool has_prev = false;
  double prev_error = 0.0, min_dt_used = 1.7976931348623157e308, max_dt_used = 0.0;
  size_t consecutive_rejects = 0, accepted = 0, rejected = 0;
  double suggest_dt(double err, double dt) const;
  void record_step(double err, double dt, bool accepted);
  bool should_reject(double err) const { return err > reject; }
  double emergency_dt(double dt, double dt_min) const;
  bool is_struggling() const { return consecutive_rejects >= 3; }
};
struct AdaptiveController {
  StepController pi;
  double dt_min, dt_max;
  AdaptiveController(double mn, double mx) : dt_min(mn), dt_max(mx) {}
  std::pair<bool, double> process_lte(const Lte& lte, double dt);
};

// The engine's adaptive transient (engine.rs:332-602): DC operating point
// from the .ic guess, then per step a backward-Euler and a trapezoidal
// Newton solve, Milne's estimate, the PI controller, breakpoints and
// settling; 10 rejections in a row end the run as failed. be_sign: -1 the
// reference's BE companion (rhs[a] -= g v_prev), +1 the physical one. Time
// dependent sources take their value at tstart in the DC point (the
// reference's stamp_voltage cannot parse a waveform string and leaves such
// a source out of the DC point; not restated). status: 0 completed, 1 a run
// of rejections, 2 the DC point did not converge.
struct TranAdaptiveResult {
  int status = 0;
  std::vector<double> times;
  std::vector<Vec> solutions;
  size_t accepted = 0, rejected = 0, newton_iterations = 0;
};
TranAdaptiveResult tran_adaptive(const Circuit& c, const std::vector<Waveform>& waves,
                                 const NewtonConfig& cfg, const std::string& solver_kind,
                                 double tstep, double tstop, double tstart, double tmax,
                                 double abs_tol, double rel_tol, double be_sign,
                                 const Vec& x_ic);

// ---------------------------------------------------------------- BBD
// bbd_decompose (crates/sim-core/src/bbd.rs:355-485) on a given partition
// (the Partitioner trait's result, bbd.rs:44-72): assignment[i] = block id,
// or -1 for the border. Nodes with an entry coupling them to another block
// are promoted to the border in the reference's two passes; empty blocks
// are dropped; perm[new] = old with the blocks first, then the border.
struct BbdDecomposition {
  size_t num_blocks = 0, border_start = 0, border_size = 0;
  UVec perm, inv_perm, block_ptr;
};
BbdDecomposition bbd_decompose_known(size_t n, const i64* ap, const i64* ai,
                                     const std::vector<int64_t>& assignment,
                                     size_t num_blocks);

// BbdSolver (crates/sim-core/src/bbd_solver.rs:86-1095): one SparseLU per
// diagonal block; the Schur complement S = B_T - sum_k C_k B_k^-1 R_k built
// column by column of R_k; dense partial-pivot LU for a border of at most 64
// (singular below 1e-30), otherwise SparseLU on the structural Schur pattern;
// a trivial decomposition or a border above half of n falls back to SparseLU.
class BbdSolver : public LinearSolver {
 public:
  BbdSolver(size_t n, std::vector<int64_t> assignment, size_t num_blocks);
  void prepare(size_t n) override;
  int analyze(const IVec& ap, const IVec& ai) override;
  int factor(const IVec& ap, const IVec& ai, const Vec& ax) override;
  int solve(Vec& rhs) override;
  void reset_pattern() override;
  const char* name() const override { return "BBD"; }
  const BbdDecomposition& decomposition() const { return dec_; }
  bool uses_fallback() const { return fallback_ != nullptr; }

 private:
  struct Sparse {  // CSC with values in pattern order
    size_t nrows = 0, ncols = 0;
    UVec col_ptr, row_idx;
    Vec values;
  };
  int analyze_bbd(const IVec& ap, const IVec& ai);
  int factor_bbd(const IVec& ap, const IVec& ai, const Vec& ax);
  int solve_bbd(Vec& rhs);
  size_t n_;
  std::vector<int64_t> assign_;
  size_t nblk_target_;
  BbdDecomposition dec_;
  bool have_dec_ = false, analyzed_ = false, factored_ = false;
  std::vector<SparseLuSolver> blocks_;
  std::vector<Sparse> c_, r_;
  Vec block_work_;
  // Schur: dense (border <= 64) or sparse
  bool dense_schur_ = true;
  Vec bt_dense_, schur_dense_, schur_lu_;
  UVec schur_piv_;
  std::unique_ptr<SparseLuSolver> schur_sparse_;
  IVec schur_ap_, schur_ai_;
  Vec schur_ax_;
  std::unique_ptr<SparseLuSolver> fallback_;
  IVec last_ap_, last_ai_;
};

// ---------------------------------------------------------------- transient
// Fixed-step backward Euler with the physical companion sign (the transient
// the reference's engine would run with `.tran dt` and BE, crates/sim-core/
// src/engine.rs:463-602 with stamp.rs:759-787, fixed step, no LTE control):
// every step is a Newton solve from the previous time point, capacitor
// voltages from the previous time point, one solver whose pivots freeze at
// the first factorization. `states` returns (steps + 1) x node_count values
// (the initial state first). Returns the first failing step's Newton reason
// (0 when every step converged); `iters` sums the Newton iterations.
int tran_be(const Circuit& c, const NewtonConfig& cfg, const std::string& solver_kind,
            double dt, size_t steps, const double* x_init, Vec& states, size_t& iters);

// Discrete adjoint of tran_be for L = sum_{t=1..steps} (x_t[probe] - target)^2:
// lambda_t solves J_t^T lambda_t = dL/dx_t + G_C lambda_{t+1} with the exact
// Jacobian J_t at x_t (level-1 floor 0) and G_C the capacitor conductances;
// dL/dC_d = -sum_t (lambda_t[a] - lambda_t[b]) (dv_t - dv_{t-1}) / dt.
// grad[d] receives dL/dp[d][0] for capacitors (0 elsewhere). Dense LU with
// partial pivoting for the transposed solves. Returns 0, or 1 on a singular
// Jacobian.
int tran_adjoint(const Circuit& c, double dt, size_t steps, const Vec& states, size_t probe,
                 double target, double gmin, Vec& grad);

}  // namespace oracle
