/* gpuklu.h - C ABI of the GB300 Newton inner loop for RustSpice.
 *
 * A drop-in for the reference's `LinearSolver` trait
 * (crates/sim-core/src/solver.rs:141-166) plus a device-stamp Newton path and
 * a batched path. Plain pointers and sizes only; every function is callable
 * from a Rust `extern "C"` block, ctypes, or C/C++.
 *
 * Threading: a handle is used by one thread at a time (the trait is `Send`,
 * not `Sync`); many handles may coexist, each with its own CUDA stream.
 * Host pointers are host memory unless a name ends in _device.
 */
#ifndef GPUKLU_H
#define GPUKLU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. 0..6 mirror SolverError (crates/sim-core/src/solver.rs:76-92):
 * AnalyzeFailed, FactorFailed, SolveFailed, SingularMatrix{pivot},
 * IllConditioned{rcond}, InvalidMatrix{reason}. 7.. are device conditions. */
enum {
  GPUKLU_OK = 0,
  GPUKLU_ANALYZE_FAILED = 1,
  GPUKLU_FACTOR_FAILED = 2,
  GPUKLU_SOLVE_FAILED = 3,
  GPUKLU_SINGULAR = 4,
  GPUKLU_ILL_CONDITIONED = 5,
  GPUKLU_INVALID_MATRIX = 6,
  GPUKLU_DEVICE_TIMEOUT = 7, /* a dependency wait hit its spin limit */
  GPUKLU_NONFINITE = 8,      /* NaN/Inf in a Newton iterate */
  GPUKLU_CUDA_ERROR = 9      /* CUDA runtime error; see gpuklu_last_error */
};

/* Pivot handling of the first factorization.
 * REFERENCE: NativeKLU's rule exactly (crates/sim-core/src/native_klu.rs:
 *   1295-1334): threshold row swaps inside the symbolic pattern computed
 *   without pivoting; entries a swap moves outside that pattern are dropped,
 *   and later refactorizations reuse the pivots.
 * EXACT: the same first pass chooses the pivots, then the pattern is
 *   recomputed for the row-permuted blocks and every factorization refactors
 *   that exact pattern; BTF coupling blocks are applied where BTF puts them
 *   (below the diagonal blocks). */
enum { GPUKLU_PIVOT_REFERENCE = 0, GPUKLU_PIVOT_EXACT = 1 };

typedef struct gpuklu_handle gpuklu_handle;

typedef struct {
  int64_t factor_count;   /* full factorizations (pivot discovery) */
  int64_t refactor_count; /* refactorizations with frozen pivots */
  int64_t nnz_l, nnz_u;   /* symbolic pattern sizes (U includes the diagonal) */
  int64_t nblocks;        /* BTF diagonal blocks */
  int64_t noffdiag;       /* entries in the BTF coupling blocks used by solve */
  int64_t pivot_swaps;    /* rows whose pivot differs from the diagonal */
  int64_t refactor_flops; /* multiply/add/divide count of one refactorization */
  double rcond;           /* min|u_kk| / max|u_kk| (native_klu.rs:1406-1427) */
} gpuklu_stats;

/* ------------------------------------------------ LinearSolver (solver.rs:141-166) */

/* NativeKluSolver::new (native_klu.rs:659-674). Returns NULL if no CUDA
 * device is usable (the reason is printed to stderr). */
gpuklu_handle* gpuklu_create(int64_t n);
void gpuklu_destroy(gpuklu_handle* h);
/* prepare (native_klu.rs:1608-1614): a new n resets the cached pattern. */
void gpuklu_prepare(gpuklu_handle* h, int64_t n);
/* analyze (native_klu.rs:1616-1632): no-op when (ap, ai) equal the cached
 * pattern; ap_len != n + 1 gives GPUKLU_INVALID_MATRIX. */
int gpuklu_analyze(gpuklu_handle* h, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                   int64_t ai_len);
/* factor (native_klu.rs:1634-1641): re-analyzes on a pattern change, else
 * refactors with the frozen pivots. ax has ai_len values (host memory). */
int gpuklu_factor(gpuklu_handle* h, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                  int64_t ai_len, const double* ax);
/* solve (native_klu.rs:1643-1655): rhs (length n) is overwritten with x.
 * Before a factorization: GPUKLU_SOLVE_FAILED. */
int gpuklu_solve(gpuklu_handle* h, double* rhs, int64_t len);
/* reset_pattern (native_klu.rs:1657-1666). */
void gpuklu_reset_pattern(gpuklu_handle* h);
/* name (native_klu.rs:1668-1670) -> "GpuKLU". */
const char* gpuklu_name(const gpuklu_handle* h);
/* set_parallel_threads (native_klu.rs:1672-1674): accepted and ignored; the
 * device decides its own parallelism. */
void gpuklu_set_parallel_threads(gpuklu_handle* h, size_t threads);

/* ------------------------------------------------ extensions */

/* Pivot mode for the next analysis (default GPUKLU_PIVOT_REFERENCE). */
int gpuklu_set_pivot_mode(gpuklu_handle* h, int mode);
/* Which of the reference's LinearSolver implementations the handle
 * restates (default NATIVEKLU); a change resets the pattern. Each is a drop-
 * in for its namesake, bit for bit:
 * NATIVEKLU     NativeKluSolver (native_klu.rs:659-1675);
 * SPARSELU      SparseLuSolver (sparse_lu.rs:217-745): one block, AMD, no
 *               row exchanges, pivots below 1e-14 set to +-1e-14;
 * SPARSELU_BTF  SparseLuBtfSolver (sparse_lu_btf.rs:137-672): BTF when
 *               should_use_btf (btf.rs:560-573) gives >= 2 blocks below n,
 *               one SparseLU per block, the block coupling applied as its
 *               solve_btf does (:441-561); else one SparseLU;
 * DENSE         DenseSolver (solver.rs:596-724): the values summed into a
 *               row-major n x n array, LU with partial pivoting (the first
 *               row of largest magnitude), GPUKLU_FACTOR_FAILED for a column
 *               without a nonzero candidate; any pattern is accepted by
 *               analyze, a wrong ap length fails the factorization with
 *               GPUKLU_ANALYZE_FAILED; n up to GPUKLU_DENSE_MAX_N; no
 *               transpose solve. */
enum {
  GPUKLU_KIND_NATIVEKLU = 0,
  GPUKLU_KIND_SPARSELU = 1,
  GPUKLU_KIND_SPARSELU_BTF = 2,
  GPUKLU_KIND_DENSE = 3
};
#define GPUKLU_DENSE_MAX_N 2048
int gpuklu_set_solver_kind(gpuklu_handle* h, int kind);
/* Growth-triggered re-pivot, off by default (the reference's refactorization
 * always keeps the first factorization's pivots, native_klu.rs:1020-1148,
 * and only perturbs a tiny one to +-1e-14, :1344-1348). On: after every
 * refactorization the device checks each BTF block's multipliers; a block
 * with one above 1/0.001 (its kept pivot below a thousandth of the largest
 * entry under it, the threshold the first factorization swaps on,
 * :1295-1334) is factored afresh on the device - the first factorization's
 * pivot choice for the current values and, in GPUKLU_PIVOT_EXACT, that
 * block's exact pattern, the other blocks keeping their pivots; in
 * GPUKLU_PIVOT_REFERENCE every block afresh, as after reset_pattern. The
 * factor then equals a fresh first factorization of those values. Costs a
 * growth scan and a device-to-host read after each refactorization. */
int gpuklu_set_repivot(gpuklu_handle* h, int on);
/* Re-pivots since the last pattern change (the count reset_pattern clears). */
int64_t gpuklu_repivot_count(const gpuklu_handle* h);
/* Failure detection; no counterpart in the reference, whose solver runs on
 * the CPU and cannot stall (its error paths are SolverError, solver.rs:
 * 76-92, and the Newton loop's SolverFailure, newton.rs:85-91).
 * Spin limit: polls of a dependency flag (grid refactorization, grid and
 * transpose solves, the one-block refactorization) before the waiting warp
 * gives up; the kernel then ends normally and the call returns
 * GPUKLU_DEVICE_TIMEOUT, with the handle still usable. 0 restores the
 * default, 2^22 polls (seconds of waiting). */
int gpuklu_set_spin_limit(gpuklu_handle* h, uint32_t polls);
/* Off (default): a Newton iterate with a NaN or an infinity runs on to the
 * iteration cap and ends with reason 1, as the reference's loop does (its
 * convergence test is false for NaN). On: gpuklu_newton_dc and
 * gpuklu_dc_sweep end at the first such iterate with GPUKLU_NONFINITE,
 * reason 2 and the iterations run so far. */
int gpuklu_set_stop_on_nonfinite(gpuklu_handle* h, int on);
/* Counters of NativeKluStats (native_klu.rs:584-594) plus device figures. */
int gpuklu_get_stats(gpuklu_handle* h, gpuklu_stats* out);
/* Text of the last error on this handle ("" if none). */
const char* gpuklu_last_error(const gpuklu_handle* h);
/* Refactorizations the last first factorization ran to find the pivot
 * sequence of native_klu.rs:1194-1382 (the pivot pass restated as
 * refactorizations that check the threshold rule on every column); 0 when
 * the sequential one-warp pivot pass ran instead (below 512 rows, more than 8
 * passes needed, or GPUKLU_PIVOT_PASS=sequential; GPUKLU_PIVOT_PASS=refactor
 * takes the refactorizations at every size). Both give the same pivots and
 * factor. */
int64_t gpuklu_pivot_pass_count(const gpuklu_handle* h);
/* factor/solve with values already in device memory (the device-stamp path):
 * d_ax has the cached pattern's nnz values, d_rhs has n values. */
int gpuklu_factor_device(gpuklu_handle* h, const double* d_ax);
int gpuklu_solve_device(gpuklu_handle* h, double* d_rhs);
/* Transpose solve A^T y = g with the current factors (the adjoint). No
 * counterpart in the reference: klu_l_tsolve is bound but never called
 * (crates/sim-core/src/solver.rs:1740-1747). g (length n) is overwritten
 * with y. */
int gpuklu_tsolve(gpuklu_handle* h, double* g, int64_t len);
/* Raw CUDA stream of the handle (cudaStream_t), for callers that enqueue
 * their own work around the solver. */
void* gpuklu_stream(gpuklu_handle* h);

/* Largest n gpuklu_solve_device_noalloc accepts. */
#define GPUKLU_NOALLOC_MAX_N 65536

/* Solve without allocating: for callers that cannot call cudaMalloc where
 * they solve - a simulator step run from a host callback where allocation is
 * not allowed, a real-time loop with a fixed device-memory budget, or a
 * foreign runtime that owns all device memory and only lends buffers. No
 * counterpart in the reference; it is an addition of this library. Solves
 * A x = b with the handle's current factors: d_rhs (n values, device memory)
 * is read, d_x (n values, device memory) receives x. The solve kernel's
 * scratch (about 1.5 MB, held by every GPU that loads the library until the
 * process exits) is a fixed array inside the library, not the handle's
 * buffers, so the call allocates nothing. The first call on a device looks
 * up that array's device address; make that first call before any stream
 * capture. All calls share the one array and each clears the flags it needs:
 * calls that overlap on the GPU (two handles on different streams at once)
 * race, so serialise them. n above GPUKLU_NOALLOC_MAX_N gives
 * GPUKLU_INVALID_MATRIX. The call reads the solve's status back and waits
 * for the handle's stream, so it returns after the solve has finished. */
int gpuklu_solve_device_noalloc(gpuklu_handle* h, const double* d_rhs, double* d_x);

/* ------------------------------------------------ device stamping + Newton */

/* Device types and parameter slots (p[6] per device):
 *   0 R  p0 = ohms                    1 V  p0 = volts
 *   2 I  p0 = amps                    3 D  p0 = Is, p1 = N
 *   4 M  level-1 as the reference evaluates it (bsim/evaluate.rs:285-356):
 *        p0 = is_pmos, p1 = vth0, p2 = u0, p3 = tox, p4 = W, p5 = L
 *   5 C  p0 = farads (open in DC, backward Euler in transient)
 *   6 MC level-1 with a self-consistent linearisation, same parameters.
 * nodes[4] per device: R/V/I/D/C use (a, b); M/MC use (d, g, s, b).
 * Node 0 is ground and stays in the matrix; one aux unknown per V source. */
typedef struct gpuklu_circuit gpuklu_circuit;

/* Compiles the device list into a stamp-to-slot map: the MNA pattern the
 * reference's build closure produces (crates/sim-core/src/engine.rs:262-283:
 * every instance stamped in order, ground pinned, CSC not merged), and for
 * every insert its CSC index. transient != 0 includes capacitor stamps. */
gpuklu_circuit* gpuklu_compile_devices(int64_t node_count, int64_t ndev, const int32_t* type,
                                       const int32_t* nodes, const double* p, int transient);
void gpuklu_circuit_free(gpuklu_circuit* c);
/* Matrix dimension and raw (unmerged) nonzero count of a compiled circuit. */
int gpuklu_circuit_dims(const gpuklu_circuit* c, int64_t* n, int64_t* nnz_raw);
/* CSC pattern of a compiled circuit (ap: n+1, ai: nnz_raw). */
int gpuklu_circuit_pattern(const gpuklu_circuit* c, int64_t* ap, int64_t* ai);
/* Updates device parameters in place (p has ndev*6 values). */
int gpuklu_circuit_set_params(gpuklu_circuit* c, const double* p);
/* Stamps the circuit at x on the device and copies the raw CSC values and
 * the right-hand side back (tests and callers that bring their own solver).
 * cap_v: per-device previous capacitor voltage (transient; ndev values), may
 * be NULL. */
int gpuklu_stamp(gpuklu_handle* h, gpuklu_circuit* c, const double* x, int64_t xlen,
                 double gmin, double source_scale, double dt, const double* cap_v,
                 double be_sign, double* ax_out, double* rhs_out);

typedef struct {
  int64_t max_iters;     /* itl1 */
  double abs_tol;        /* vntol */
  double rel_tol;        /* reltol */
  double gmin;
  int64_t gmin_steps;    /* GminSchedule steps (newton.rs:204-237) */
  int64_t source_steps;  /* SourceSchedule steps (newton.rs:240-265) */
  double damping, damping_min;
} gpuklu_newton_config;

/* DC operating point (engine.rs:249-311) with run_newton_with_stepping
 * (newton.rs:142-185): stamping, factor, solve and the Newton update all on
 * the device. x0 (node_count values) may be NULL for the zero start. x_out
 * receives min(x_cap, len(x)) values of the final iterate; *x_len its length
 * (n when converged, node_count otherwise). Returns a status; *reason is the
 * NewtonExitReason (0 converged, 1 max iterations, 2 solver failure) and
 * *iters the iterations of the final Newton run, *iters_total all of them. */
int gpuklu_newton_dc(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                     const double* x0, double* x_out, int64_t x_cap, int64_t* x_len,
                     int64_t* iters, int64_t* iters_total, int* reason);

/* DC sweep (the reference's .dc, crates/sim-core/src/engine.rs:684-820) of
 * one source: device src_dev's first parameter takes values[0..npts) in
 * order, one Newton solve per point on the device as gpuklu_newton_dc runs
 * it. As in the reference one solver serves the whole sweep (prepare(
 * node_count) once, engine.rs:747), so the pattern and the pivots of the
 * first point's first factorization are kept for every later point. x0 ==
 * NULL: each point starts from the previous point's final iterate (the
 * reference's continuation; after a converged point that is the full
 * solution with its aux currents, and the convergence test then covers
 * them too); else point k starts from x0 + k * x0_stride (node_count
 * values). stop_on_failure != 0 ends the sweep at the first point that does
 * not converge, as the reference does (engine.rs:785-796). Per point:
 * x_out + k * x_stride receives n values (zero beyond *x_len[k]), iters,
 * iters_total and reason as gpuklu_newton_dc gives them; points not run
 * have reason -1. The circuit keeps the last value. */
int gpuklu_dc_sweep(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                    int64_t src_dev, const double* values, int64_t npts, const double* x0,
                    int64_t x0_stride, int stop_on_failure, double* x_out, int64_t x_stride,
                    int64_t* x_len, int64_t* iters, int64_t* iters_total, int* reason);

/* AC small-signal sweep at a DC solution: the reference's .ac
 * (crates/sim-core/src/engine.rs:829-930) with its AC stamps (stamp.rs:
 * 1525-1747) and dense complex LU with partial pivoting (complex_solver.rs:
 * 28-144), every frequency point solved at once on the device. V and I
 * sources carry the AC magnitude in p[1] and the phase [deg] in p[2]. x_dc:
 * the operating point (node voltages at least); freqs: nf frequencies [Hz];
 * out_re / out_im: nf x n values (n = node_count + one aux per V source, row
 * 0 the ground); *n_out = n. Systems up to n = 118 are factored in one
 * block's shared memory per frequency; larger ones in per-block slices of a
 * global scratch (up to ~2 GB, blocks looping over the frequencies) with the
 * same arithmetic. n above GPUKLU_AC_MAX_N gives GPUKLU_INVALID_MATRIX, a
 * pivot below 1e-30 GPUKLU_SINGULAR. */
#define GPUKLU_AC_MAX_N 4096
int gpuklu_ac_sweep(gpuklu_handle* h, gpuklu_circuit* c, const double* x_dc, int64_t xlen,
                    const double* freqs, int64_t nf, double* out_re, double* out_im,
                    int64_t* n_out);

/* Adjoint of a DC operating point (no counterpart in the reference). At the
 * converged x (xlen values, node voltages first) it stamps and factors the
 * exact Jacobian A(x) on the device (the consistent level-1 model without its
 * 1e-12 S conductance floor, which cancels in the residual), solves A(x)^T lambda = dl_dx (n values) with the transpose
 * solve, and evaluates dL/dp = -lambda^T dF/dp for every device, where
 * F(x, p) = A(x) x - b(x) is the stamped KCL residual and p is the device's
 * resistance (R), value (V, I), Is (D) or VTO (M, MC). lambda_out (n) and
 * grad_out (ndev) may be NULL. */
int gpuklu_dc_backward(gpuklu_handle* h, gpuklu_circuit* c, const double* x, int64_t xlen,
                       const double* dl_dx, double gmin, double* lambda_out,
                       double* grad_out);

/* ------------------------------------------------ batched Newton */

typedef struct gpuklu_batch gpuklu_batch;

/* Many independent DC operating points in one launch. Circuits are given as
 * concatenated device lists (dev_off[ncirc+1]); instance i runs circuit
 * inst_circ[i] with the first parameter of device inst_dev[i] replaced by
 * inst_val[i] (inst_dev < 0: none) from initial iterate x0 + x0_off[i]
 * (x0_off < 0: zero start). Instances of one circuit share its analysis,
 * pivots (exact mode, found once per circuit) and device program. */
gpuklu_batch* gpuklu_batch_create(int64_t ncirc, const int64_t* dev_off,
                                  const int64_t* node_counts, const int32_t* type,
                                  const int32_t* nodes, const double* p, int64_t ninst,
                                  const int64_t* inst_circ, const int64_t* inst_dev,
                                  const double* inst_val, const double* x0,
                                  const int64_t* x0_off, int64_t x0_len);
void gpuklu_batch_destroy(gpuklu_batch* b);
/* Runs every instance's Newton loop on the device: a lane-per-instance
 * kernel for the first lane_cap iterations, then the continuation kernel (one
 * warp per instance still iterating; the warp classes when it is off); with
 * lane_cap 0 the continuation kernel starts every instance. */
int gpuklu_batch_run(gpuklu_batch* b, const gpuklu_newton_config* cfg);
/* Results: per instance iterations (final run), total iterations, exit
 * reason, and x (n of its circuit values, at x_out + x_off[i]; x_off may be
 * NULL to skip). When x_off is the batch's own layout (consecutive
 * instances, n values each) x arrives in one copy, a DMA into pinned x_out.
 * An instance whose iterate turns non-finite stops there with reason 1 and,
 * as its final run's iteration count, the cap: the count the reference
 * reports, whose loop runs on to the cap because a non-finite entry never
 * turns finite again (newton.rs:93-107). Its total counts the iterations the
 * device executed, and its x is the non-finite iterate. */
int gpuklu_batch_results(gpuklu_batch* b, int64_t* iters, int64_t* iters_total, int32_t* reason,
                         double* x_out, const int64_t* x_off);
/* Host->device copy of new per-instance values and initial iterates
 * (same layout as at creation; either pointer may be NULL). */
int gpuklu_batch_update_inputs(gpuklu_batch* b, const double* inst_val, const double* x0);
/* Last error text of the batch. */
const char* gpuklu_batch_last_error(const gpuklu_batch* b);
/* Launch geometry (out has 8 entries): out[0] grid, out[1] threads per
 * block, out[2] program groups, out[3] shared-memory bytes per warp,
 * out[4] registers per thread, out[5] resident blocks per SM (out[1], out[3..5]
 * describe the largest class), out[6] kernel launches per gpuklu_batch_run
 * (the lane kernel and one per size class), out[7] reserved (0). */
int gpuklu_batch_info(const gpuklu_batch* b, int64_t* out);
/* Work of one Newton iteration of every instance: FP64 operations and the
 * value bytes it moves through on-chip memory (arrays of ninst). */
int gpuklu_batch_work(const gpuklu_batch* b, int64_t* flops, int64_t* bytes);
void* gpuklu_batch_stream(gpuklu_batch* b);
/* Device time of the last gpuklu_batch_run (waits for it), from CUDA events
 * on the launching streams: out[0] the lane-per-instance kernel [ms], out[1]
 * the warp kernels that finish the instances it parked [ms], out[2] the
 * iterations an instance runs in the lane kernel before it is parked (0: no
 * lane phase). */
int gpuklu_batch_phase_ms(gpuklu_batch* b, double* out);
/* The batch's schedule; no counterpart in the reference. lane_cap: Newton
 * iterations an instance runs in the lane-per-instance phase before it is
 * parked for the continuation (default 6; ignored when that phase is off;
 * 0 with the continuation kernel: no lane phase, the continuation starts
 * every instance); cont_tiles: shared-program tiles per circuit program in
 * the warp classes' continuation (default 2; the continuation kernel has
 * none). Results agree across schedules to the batch's 1e-10 bar (an
 * instance's arithmetic differs between the kernels only in rounding). */
int gpuklu_batch_set_schedule(gpuklu_batch* b, int lane_cap, int cont_tiles);
/* Autotuner: times one run of the batch per candidate schedule (lane_cap in
 * {0, 1, 2, 3, 4, 5, 6, 8, 10, 12}, cont_tiles in {1, 2, 3, 4} for the warp
 * classes' continuation; two rounds of
 * coordinate descent from the current schedule, CUDA events around the
 * kernels) and keeps the fastest. out[0..2] = lane_cap, cont_tiles, runs;
 * *best_ms its device time. The batch's results afterwards are those of the
 * last trial: run it again for the tuned run's. */
int gpuklu_batch_autotune(gpuklu_batch* b, const gpuklu_newton_config* cfg, int64_t* out,
                          double* best_ms);

/* ------------------------------------------ adaptive transient */
/* The engine's transient analysis (crates/sim-core/src/engine.rs:332-602),
 * one circuit instance per warp, the whole time loop on the device: the DC
 * operating point from the instance's initial guess x_ic (its .ic values),
 * then per step a backward-Euler and a trapezoidal Newton solve from the
 * last accepted point, Milne's estimate |x_trap - x_be| / 3 over the whole
 * iterate against lte_abs + lte_rel max(|x|) (analysis.rs:147-206; the
 * engine passes vntol and reltol), the PI controller (analysis.rs:380-760),
 * breakpoints of PULSE and PWL sources with five settling steps at a tenth
 * of the step after each (waveform.rs:417-660), and ten rejections in a
 * row ending the run. Circuits as for gpuklu_tran_create (C devices take
 * p[0] as the capacitance); per device (concatenated over the circuits) an
 * optional waveform of a V or I source: wkind 0 none, 1 PULSE (7 parameters
 * v1 v2 td tr tf pw per), 2 PWL (points pwl_ptr[d]..pwl_ptr[d+1] of pwl_t,
 * pwl_v), 3 SIN (vo va freq td theta), 4 EXP (v1 v2 td1 tau1 td2 tau2), the
 * parameters in wp7[d * 7 ..]. A waveform source takes its value at tstart
 * in the DC point (the reference's DC stamp cannot parse a waveform and
 * leaves the source out). probe: the node whose voltage is recorded. */
gpuklu_batch* gpuklu_atran_create(int64_t ncirc, const int64_t* dev_off,
                                  const int64_t* node_counts, const int32_t* type,
                                  const int32_t* nodes, const double* p, const int32_t* wkind,
                                  const double* wp7, const int64_t* pwl_ptr, const double* pwl_t,
                                  const double* pwl_v, const double* x_ic,
                                  const int64_t* x_ic_off, int64_t x_ic_len,
                                  const int64_t* probe);
/* Runs the adaptive transient from tstart to tstop: min step max(1e-6 tstep,
 * 1e-15), max step min(tmax, tstop / 10), first step min(tstep, max step).
 * be_sign: -1 the reference's backward-Euler companion (rhs[a] -= (C/dt)
 * v_prev; every step with a charged capacitor is then rejected), +1 the
 * physical one. cfg: the Newton settings of every solve (the engine uses
 * the DC settings; its transient has no gmin or source stepping). Per
 * instance i: up to max_points accepted times and probe values at
 * i * max_points (the DC point first), npoints (all accepted points, also
 * those beyond max_points), accepted and rejected steps, Newton
 * iterations, status (0 completed, 1 ten rejections in a row, 2 DC point
 * not converged, 3 max_steps step attempts spent), and the last accepted
 * solution in x_out (the batch's x_out layout, n values per instance). */
int gpuklu_atran_run(gpuklu_batch* b, const gpuklu_newton_config* cfg, double tstep,
                     double tstop, double tstart, double tmax, double lte_abs, double lte_rel,
                     double be_sign, int64_t max_points, int64_t max_steps, double* times_out,
                     double* probe_out, int64_t* npoints, int64_t* accepted, int64_t* rejected,
                     int32_t* status, int64_t* iters, double* x_out);

/* ------------------------------------------ bordered block diagonal */
/* The reference's BbdSolver (crates/sim-core/src/bbd_solver.rs:86-1095,
 * bbd.rs:355-485) with a known partition (the Partitioner trait's result,
 * bbd.rs:44-72): assignment[i] = block of node i, or -1 for the border.
 * Nodes with an entry into another block are promoted to the border; a
 * trivial decomposition or a border above n/2 falls back to one solver over
 * the whole matrix (as the reference falls back to SparseLU). The diagonal
 * blocks are factored together on the device, the Schur complement
 * S = B_T - C B^-1 R is assembled and factored densely on the device (border
 * up to 16384). gpuklu_bbd_factor/solve take host arrays in the original
 * order (the LinearSolver factor/solve of solver.rs:141-166). */
typedef struct gpuklu_bbd gpuklu_bbd;
gpuklu_bbd* gpuklu_bbd_create(int64_t n, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                              int64_t ai_len, const int64_t* assignment, int64_t num_blocks);
void gpuklu_bbd_destroy(gpuklu_bbd* b);
const char* gpuklu_bbd_last_error(const gpuklu_bbd* b);
/* out[0] blocks, out[1] border start, out[2] border size, out[3] fallback,
 * out[4] Schur right-hand-side tiles, out[5] blocks the inner factorization
 * found. */
int gpuklu_bbd_info(const gpuklu_bbd* b, int64_t* out);
/* perm[new] = original index (blocks in order, then the border). */
int gpuklu_bbd_perm(const gpuklu_bbd* b, int64_t* perm);
int gpuklu_bbd_factor(gpuklu_bbd* b, const double* ax);
int gpuklu_bbd_solve(gpuklu_bbd* b, double* rhs, int64_t len);
/* DC operating point of a compiled circuit whose pattern is the solver's,
 * with the loop and outputs of gpuklu_newton_dc. */
int gpuklu_bbd_newton_dc(gpuklu_bbd* b, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                         const double* x0, double* x_out, int64_t x_cap, int64_t* x_len,
                         int64_t* iters, int64_t* iters_total, int* reason);

/* ------------------------------------------ batched transient + adjoint */
/* Fixed-step backward-Euler transient of many circuits, one instance per
 * circuit, and the discrete adjoint of the loss
 *   L_i = sum_{t=1..steps} (x_t[probe_i] - target)^2
 * by checkpointing. This is the transient the reference's engine runs with a
 * fixed step and BE (crates/sim-core/src/engine.rs:463-602,
 * stamp.rs:759-787), except that the capacitor companion current has the
 * physical sign (rhs[a] += (C/dt) v_prev; the reference subtracts it,
 * stamp.rs:777-784). No reference counterpart exists for the adjoint.
 * Circuits are given as for gpuklu_batch_create; x_init/x_init_off: each
 * instance's initial node voltages; every ckpt_every steps the forward run
 * keeps the state, and the backward run recomputes each segment from it.
 * The handle is released with gpuklu_batch_destroy. */
gpuklu_batch* gpuklu_tran_create(int64_t ncirc, const int64_t* dev_off,
                                 const int64_t* node_counts, const int32_t* type,
                                 const int32_t* nodes, const double* p, const double* x_init,
                                 const int64_t* x_init_off, int64_t x_init_len, double dt,
                                 int64_t steps, int64_t ckpt_every, const int64_t* probe,
                                 double target);
/* Forward run: per instance the loss, optionally the probe waveform
 * (ninst x steps), the Newton iterations and the reason (0 every step
 * converged, 1 a step failed; its loss is NaN). */
int gpuklu_tran_forward(gpuklu_batch* b, const gpuklu_newton_config* cfg, double* loss_out,
                        double* wave_out, int64_t* iters_out, int32_t* reason_out);
/* Backward run after a forward run with the same cfg: dL_i/dC for every
 * capacitor of instance i (0 for other devices), concatenated over the
 * instances in device order; iters_out: Newton iterations of the
 * recomputation. */
int gpuklu_tran_backward(gpuklu_batch* b, const gpuklu_newton_config* cfg, double* grad_out,
                         int64_t* iters_out);

/* Measured FP64 fused multiply-add throughput of the current device in
 * TFLOP/s (a short microbenchmark; the denominator of FP64 roofline
 * fractions). */
double gpuklu_fp64_peak_tflops(void);
/* The same for the FP64 tensor cores: mma.sync m8n8k4 f64 (DMMA), four
 * independent accumulations per warp. */
double gpuklu_fp64_mma_peak_tflops(void);
/* The BBD solver's dense Schur LU on its own (bbd_solver.rs:811-896: no
 * pivoting, pivots below 1e-14 set to +-1e-14) for a host column-major n x n
 * matrix, factored in place (L below the diagonal, unit diagonal implied; U
 * on and above). variant 0: 32-wide panel kernels, four launches per panel;
 * 1: one cooperative launch, FP64 FMA updates, pivots applied through their
 * reciprocals (agrees with variant 0 to rounding); 2: the cooperative launch
 * with DMMA updates. *ms_out: device time of the
 * factorization. No counterpart in the reference (its BbdSolver factors S
 * inside factor_bbd). */
int gpuklu_dense_lu_nopivot(double* a, int64_t n, int variant, double* ms_out);

/* ------------------------------------------------ host-only diagnostics */

/* The symbolic plan the handle would build for a pattern (host work only; no
 * device needed) in a pivot mode and for a solver kind (GPUKLU_KIND_*): BTF +
 * AMD + symbolic, and, if row_perm is not NULL, the
 * pivot sequence installed as a first factorization would (block-local
 * row_perm per position). Arrays are read back by name with
 * gpuklu_plan_array: "col_ptr", "dslot", "slot_row", "upd_ptr", "upd_dst",
 * "amap_ptr", "amap_idx", "offd_ptr", "offd_col", "offd_raw", "in_pos",
 * "out_pos", "block_ptr", "col_single", "pcol_ptr", "pcol_raw", "pcol_q",
 * "pos_block", "raw_slot", "row_perm", "lrow_ptr", "lrow_col", "lrow_slot",
 * "urow_ptr", "urow_col", "urow_slot", "info" (n, nslots, nblocks, nnz_l,
 * nnz_u, noffdiag, offd_lower, swaps). */
typedef struct gpuklu_plan gpuklu_plan;
gpuklu_plan* gpuklu_plan_build(int64_t n, const int64_t* ap, const int64_t* ai, int pivot_mode,
                               int kind, const int32_t* row_perm);
int64_t gpuklu_plan_array(const gpuklu_plan* p, const char* name, int64_t* out, int64_t cap);
void gpuklu_plan_free(gpuklu_plan* p);
/* The step program the batched warp kernels run for this plan's
 * factorization and substitutions, with the instance region's T at offset
 * nc and V at nc + n + ndv: two int32 per operation (d | a << 15 | kind
 * bits 0-1 << 30, b | c << 15 | kind bits 2-3 << 30; kinds: 0 R[d] -= R[a]
 * R[b], 4 the same unless R[b] == 0, 2 R[d] = R[a] R[b], 1 R[d] = 1 /
 * perturbed R[d] with a the singleton flag, 5 kind 4 then R[d] *= R[c], 6
 * kind 0 then R[d] *= R[c]) in step order, and the step pointers. Returns
 * nops << 32 | (nsteps + 1) (0: no program, the region exceeds 15-bit
 * offsets); copies when the capacities (in int32) suffice. */
int64_t gpuklu_plan_steps(const gpuklu_plan* p, int32_t nc, int32_t ndv, int32_t* ops,
                          int64_t ops_cap, int32_t* step_ptr, int64_t steps_cap);
/* The single-system solve's step program (k_solve_steps) for this plan: four
 * int32 per operation (destination row, source row or -1, value index, kind:
 * 0 x[d] -= lu[v] x[s], 2 x[d] -= ax[v] x[s] (block coupling), 1 x[d] /= lu[v]
 * (the pivot)) in step order, with the rows in the plan's positions, and the
 * step pointers. Returns nops << 32 | (nsteps + 1) (0: no program, the
 * solution exceeds one block's shared memory); copies when the capacities
 * (in int32) suffice. */
int64_t gpuklu_plan_solve_steps(const gpuklu_plan* p, int32_t* ops, int64_t ops_cap,
                                int32_t* step_ptr, int64_t steps_cap);
/* btf_decompose (crates/sim-core/src/btf.rs:143-550) on the host: out[0] the
 * number of blocks, out[1] the largest block's size - what
 * MatrixProperties::analyze (solver.rs:276-301) reads for the solver
 * selector. */
int gpuklu_btf_info(int64_t n, const int64_t* ap, const int64_t* ai, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif /* GPUKLU_H */
