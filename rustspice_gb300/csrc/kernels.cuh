// Kernel declarations and the device-side views of a Plan.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gk {

// Default bound on polls of a dependency flag before a waiting warp gives up,
// sets DS_TIMEOUT and returns. With the kernels' back-off this is a few
// seconds of waiting at most. A handle may lower it (gpuklu_set_spin_limit).
constexpr unsigned kSpinLimit = 1u << 22;

// Device pointers of one Plan (see analysis.h for the meaning of each array).
struct DPlan {
  int n, nslots, nblocks, ntask;
  const int *col_ptr, *dslot, *slot_row, *upd_ptr, *upd_dst, *col_single;
  const int *amap_ptr, *amap_idx;
  const int *offd_ptr, *offd_col, *offd_raw;
  const int *offdT_ptr, *offdT_row, *offdT_raw;
  const int *lrow_ptr, *lrow_col, *lrow_slot, *urow_ptr, *urow_col, *urow_slot;
  const int *in_row, *out_col;  // position -> original row / original column
  const int *pcol_ptr, *pcol_raw, *pcol_q, *pos_block, *block_ptr;
  const int *task;              // solve order: (position << 1) | is_upper
  int noffd;                    // block-coupling entries
  int cs_nchunk;                // one-block solve schedule (k_solve_cta)
  const int *cs_chunk, *cs_op;
  // The same solve with one thread block per group of consecutive BTF blocks
  // (plans without block coupling): group g covers rows [grp[4g], grp[4g+1])
  // and chunks [grp[4g+2], grp[4g+3]) of cs_gchunk / cs_gop.
  int cs_ngrp, cs_grp_rows;     // groups; rows of the largest
  const int *cs_grp, *cs_gchunk, *cs_gop;
  // The solve as a step program (k_solve_steps): ss_ptr[ss_nsteps] operations
  // (destination row, source row or -1, value index, kind: 0 lu value, 2
  // coupling ax value, 1 division by the pivot lu[value]), ss_nsteps + 1
  // step pointers; 0 steps: none.
  int ss_nsteps;
  const int4* ss_ops;
  const int* ss_ptr;
  // Polls of a dependency flag before a waiting warp gives up and reports
  // DS_TIMEOUT (kSpinLimit unless the handle sets another).
  unsigned spin_limit;
};

// Device form of a compiled circuit (device list + stamp-to-slot map).
struct DCircuit {
  int ndev, node_count, n, nnz_raw, pin_raw;
  const int* type;      // [ndev]
  const int* nodes;     // [ndev*4]; for V sources nodes[2] holds the aux row
  const double* p;      // [ndev*6]
  const int* raw;       // [ndev*8] raw CSC index of each matrix insert, -1 none
  const int* rhs_slot;  // [ndev*2] index into the rhs contribution buffer, -1 none
  const int *rhs_ptr, *rhs_src;  // per row: contributions in stamping order
};

struct NewtonCfg {
  int max_iters, gmin_steps;
  double abs_tol, rel_tol, gmin, damping, damping_min;
};

// Per-handle Newton state kept on the device between iterations.
struct NewtonState {
  double damping, prev_dx_norm, last_norm;
  int converged, iter;
};

// Batched program of one group: circuits whose device lists, analysis and
// pivots are identical share it; only parameters and inputs differ.
struct GroupHdr {
  int n, node_count, nslots, noffd, ndev, nblocks, ndv;
  int dev_off;     // program device arrays (type, nodes*4, dv)
  int col_off;     // n+1 column arrays (col_ptr, dslot, col_single, in_row, out_pos, offd_ptr)
  int slot_off;    // nslots+1 slot arrays (slot_row, upd_ptr)
  int upd_off;     // upd_dst
  int offd_off;    // offd_col
  int blk_off;     // block_ptr
  int amap_off;    // nslots+noffd+1 contribution pointers (values relative to amap_code base)
  int amap_code_off;
  int nupd;        // update-list length
  int heavy_off;   // slots/rows with long contribution lists
  int nheavy;
  int rmap_off;    // n+1 row contribution pointers
  int rmap_code_off;
  int inst_begin;  // range of the group's instances in the order array
  int inst_count;
  int cost;        // scheduling weight (FP64 operations of one Newton iteration)
  int amap4_off, rmap4_off;  // four padded codes per value slot / permuted row
  int lng_off, nlng;         // slots and rows with longer lists: (index << 1) | is_row
  int seg_off;     // factor schedule: segments (start, end, sequential) per block,
  int nseg;        //   block b's at lseg_ptr[b]..lseg_ptr[b+1] (lseg_ptr at blk_off);
                   //   the columns in schedule order sit at col_off in lvl_col
  int region;      // shared-memory doubles of one instance of this program
  int prog;        // ints of the staged program (a multiple of 4)
  // step program of the factorization and both substitutions (DC batches;
  // nsteps 0: none): nops operations at ops_off, nsteps + 1 step pointers
  // at step_off; the operations of one step are independent of each other
  int ops_off, nops, step_off, nsteps;
};

// Contribution codes of the batched stamp: (index << 3) | kind with kind
// 0 +dv[index], 1 -dv[index], 2 +1.0, 3 -1.0, 4 +0.0. A value slot (or a
// right-hand-side row) is the sum, from 0.0 and in stamping order, of its
// contributions, which is how the reference's scatter adds duplicate CSC
// entries (crates/sim-core/src/native_klu.rs:1265-1274).
struct BatchArgs {
  const GroupHdr* groups;
  int ngroups;
  const int* tile_group;   // warp work units: group of each tile
  int ntiles;
  unsigned* counter;       // next tile to hand out
  unsigned* gnext;         // per group: next instance to hand out
  const int* order;        // instances grouped by group
  const int *dev_type, *dev_nodes, *dev_dv;  // dv: offset of the device's value record
  const int *amap_ptr, *amap_code;           // per value slot (group-local ptr)
  const int *rmap_ptr, *rmap_code;           // per original row
  const int *col_ptr, *dslot, *col_single, *in_row, *out_pos, *offd_ptr, *slot_row,
      *upd_ptr, *upd_dst, *offd_col, *block_ptr;
  const int* heavy;  // (value index << 1) or (position << 1 | 1), per group
  const int *lvl_col, *lseg_ptr, *lseg;  // level-scheduled factor (see GroupHdr)
  const int *amap4, *rmap4, *lng;        // padded contribution codes (see GroupHdr)
  const int2* ops;                       // step programs (see GroupHdr)
  const int* step_ptr;
  const long long* inst_p_off;  // offset of the instance's circuit constants (4 per device)
  const double* dparams;
  const int* inst_ov_dev;
  const double* inst_ov_val;
  const long long* inst_x0_off;
  const double* x0;
  NewtonCfg cfg;
  int region;     // shared-memory doubles per instance
  int prog_ints;  // shared-memory ints of the staged program (largest group)
  int shared_bytes;  // dynamic shared memory of a launch whose warps share a program
  int *iters, *iters_total, *reason;
  const long long* inst_x_off;
  double* x_out;
  int* status;
  // transient (fixed-step backward Euler, one instance per circuit)
  int ninst;
  const int* inst_group;       // group of each instance
  double dt, inv_dt, target;
  int steps, ckpt_every;
  const int* probe;            // per instance: the node of the loss
  double* loss;                // per instance
  double* wave;                // per instance x steps values of the probe node (or null)
  double* ckpt;                // per instance: (steps / ckpt_every + 1) x node_count states
  const long long* ckpt_off;
  double* seg;                 // per instance: (ckpt_every + 1) x node_count states
  const long long* seg_off;
  double* grad;                // per instance: dL/dp[d][0] per device
  const long long* grad_off;
  // lane-per-instance phase of the batched DC run, and its continuation
  double* scratch;             // per warp: lane-interleaved state, warp_stride doubles
  long long warp_stride;
  const int* ltile_group;      // lane-phase tiles: group of each
  int nltiles;
  unsigned* lcounter;
  int cap;                     // Newton iterations per instance in the lane phase (0: all)
  int cont_mode;               // warp kernel: take the instances the lane phase left
  int* cont_list;              // per group at inst_begin: the instances left
  unsigned* cont_count;        // per group
  unsigned* gnext2;            // per group: next entry of cont_list to hand out
  int *cont_it, *cont_total, *cont_gstep;
  double *cont_damp, *cont_prev;  // the iterate itself waits in x_out
  // continuation kernel (cont.cu): one warp per parked instance, any group
  const int* cont_groups;      // the groups, most expensive first
  int cont_ngroups;
  unsigned* cont_cursor;       // first entry of cont_groups that may have parked instances
  double* dv_scratch;          // per instance slot: device records, then the iterate
  long long dv_stride;         //   at dv_x (dv_stride doubles per slot)
  long long dv_x;
  int slice;                   // shared doubles per instance slot: T and the LU values
  int cont_fresh;              // 1: no lane phase ran, the continuation starts every instance
};

// Batched adaptive transient (atran.cu): per instance its time-dependent
// sources (records wave_ptr[i]..wave_ptr[i+1]: device, kind 1 PULSE 2 PWL 3
// SIN 4 EXP, 7 parameters, PWL points at pwl_ptr) and breakpoints (bp_ptr);
// the run's controls; per instance up to max_points accepted times and
// probe-node values, counts and status (0 completed, 1 ten rejections in a
// row, 2 DC point failed, 3 max_steps attempts spent).
struct AtranArgs {
  const int *wave_ptr, *wave_dev, *wave_kind, *pwl_ptr;
  const double *wave_p, *pwl_t, *pwl_v;
  const int* bp_ptr;
  const double* bp_t;
  const int* probe;
  double tstep, tstop, tstart, tmax, lte_abs, lte_rel, be_sign;
  int max_points, max_steps;
  double *times, *probe_out;
  int *npoints, *accepted, *rejected, *status;
};

// Bordered-block-diagonal solver: the index lists its kernels read.
struct BbdArgs {
  int ntiles, bs, border_start;
  const int* tile_pos0;        // first plan position of the tile's block
  const int* tile_size;        // block size
  const long long* tile_off;   // offset of the tile's [size][32] array
  const int* tile_blk;         // plan block of the tile
  const int *init_ptr, *init_code, *init_raw;  // R entries: (row offset * 32 + lane, raw)
  // border indices below are Schur positions (the elimination order of S)
  const int *bt_ptr, *bt_row, *bt_raw;         // B_T by Schur column
  const int *yref_ptr, *yref;                  // per border column: (tile << 5 | lane)
  const int *c_ptr, *c_row, *c_pos, *c_raw;    // C by plan block: (border row, row offset of Y, raw)
  const int *crow_ptr, *crow_col, *crow_raw;   // C by border row: (block column, raw)
  const int *rrow_ptr, *rrow_col, *rrow_raw;   // R by block row: (border column, raw)
  const int* perm;                             // bordered order -> original index
  const int* bperm;                            // Schur position -> original index
};

// AC sweep: the dense cells of Y(w) = G + jwC and the per-frequency solve.
struct AcArgs {
  int n, ncell;
  const int *cell_row, *cell_col;   // cell -> (row, column); row 0 is the ground row
  const int *re_ptr, *re_idx;       // per cell: raw CSC entries of the DC stamp, in order
  const int *im_ptr, *im_code;      // per cell: (capacitor device << 1) | negated, in order
  const double* cap;                // capacitance per device
  const double* ax;                 // the DC stamp at the operating point (raw CSC)
  const double* rhs;                // 2 n: the AC sources (re, im), row 0 unused
  const double* freqs;
  double *out_re, *out_im;          // nf x n
  int* status;                      // 1: a pivot below 1e-30
  double* scratch;                  // global path: per block an n x n complex matrix
};

// --------------------------------------------------------------- launches
// maxblk: the largest diagonal block; blocks up to about 14k rows run with the
// working column in shared memory.
void launch_first_factor(const DPlan& P, int maxblk, const double* ax, double* lu,
                         double* work, int* rperm, int* rinv, double tol, int* status,
                         cudaStream_t s);
// The refactorization in its pivot-pass mode (want == nullptr: off). Before
// column k is scaled, the first factorization's threshold rule is applied to
// the column's finished values and its choice written to want[k] (the L slot
// of the row that takes the pivot, or -1 for the diagonal); then the row of
// the candidate slot cand[k] (-1: none) is swapped into the pivot. Run over
// the pivot-free pattern with the A scatter of the candidate's row order, it
// computes what the first factorization computes wherever its earlier
// choices are the candidate's, so want[] confirms the candidate up to the
// first column that disagrees.
struct PivotCheck {
  const int* cand = nullptr;
  int* want = nullptr;
  double tol = 0.0;
};
void launch_refactor(const DPlan& P, const double* ax, double* lu, unsigned* flags,
                     unsigned epoch, unsigned* counter, int* status, int grid,
                     cudaStream_t s, const PivotCheck& pc = PivotCheck());
// Slots per chunk of the one-block solve's schedule.
constexpr int kSolveChunk = 2048;
// One-block variants for small factorizations; *_cta_fits says whether the
// kernel's shared-memory working set (the whole factor, for the refactor)
// fits one block.
bool refactor_cta_fits(const DPlan& P);
void launch_refactor_cta(const DPlan& P, const double* ax, double* lu, int* status,
                         cudaStream_t s, const PivotCheck& pc = PivotCheck());
bool solve_cta_fits(const DPlan& P);
bool solve_steps_fits(const DPlan& P);
// rec: n doubles of scratch (the pivots' reciprocals)
void launch_solve_steps(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                        double* rec, double* out, cudaStream_t s);
// One block per group of uncoupled BTF blocks (cs_grp); fits when the
// largest group's rows fit one block's shared memory.
bool solve_groups_fit(const DPlan& P);
void launch_solve_groups(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                         double* out, cudaStream_t s);
void launch_solve_cta(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                      double* out, cudaStream_t s);
void launch_solve(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                  double* z, double* x, double* out, unsigned* zflag, unsigned* xflag,
                  unsigned epoch, unsigned* counter, int* status, int grid, bool transpose,
                  cudaStream_t s);
void launch_stamp(const DCircuit& C, const double* x, int xlen, double gmin, double scale,
                  double dt, const double* cap_v, double be_sign, double* ax, double* rhs_c,
                  double* rhs, cudaStream_t s, double gdev = 1e-12);
// dL/dp per device from the adjoint lambda at a DC solution x.
void launch_param_grad(const DCircuit& C, const double* x, int xlen, const double* lam,
                       double* grad, cudaStream_t s);
void launch_newton_update(int m, int n, double* x, const double* xnew, NewtonState* st,
                          NewtonCfg cfg, int* status, cudaStream_t s);
void launch_rcond(const DPlan& P, const double* lu, double* out2, cudaStream_t s);
// Pivot growth of a factorization: grow[b] = 1 for every BTF block b with a
// multiplier |l_ik| > lim (or a NaN one); grow is not cleared here.
void launch_growth(const DPlan& P, const double* lu, double lim, int* grow, cudaStream_t s);
// Measured FP64 fused multiply-add throughput of the current device [TFLOP/s].
double fp64_peak_tflops();
// m: instances per warp (1, 2 or 4); region: shared doubles per instance.
// shared: the warps of a block share one staged program (one group at a time)
void launch_batch_newton(const BatchArgs& a, int m, int grid, int warps_per_block,
                         cudaStream_t s, bool shared = false);
// Registers per thread and resident blocks per SM of the batched kernel.
// Lane-per-instance batched Newton (phase 1 of gpuklu_batch_run).
void launch_batch_cont(const BatchArgs& a, int m, int grid, int warps_per_block,
                       cudaStream_t s);
void cont_kernel_info(int m, int warps_per_block, int slice, int* regs, int* blocks_per_sm);
void launch_batch_lanes(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s);
void lanes_kernel_info(int warps_per_block, int* regs, int* blocks_per_sm);

// Bordered-block-diagonal solver pieces.
void launch_bbd_ysolve(const DPlan& P, const double* lu, const double* ax, const BbdArgs& B,
                       double* ybuf, cudaStream_t s);
void launch_bbd_schur(const double* ax, const BbdArgs& B, const double* ybuf, double* S,
                      cudaStream_t s);
void launch_dense_lu(double* S, int bs, cudaStream_t s);
// The same factorization as one cooperative launch (schur.cu): FP64 FMA
// updates (mma = false) or DMMA updates; both agree with launch_dense_lu's
// factor to rounding.
// bar: schur_lu_bar_words(bs) words of scratch (a grid barrier, block 0's
// SM and one tile counter per panel).
cudaError_t launch_schur_lu(double* S, int bs, bool mma, unsigned* bar, int* status,
                            cudaStream_t s);
inline int schur_lu_bar_words(int bs) { return 3 + (bs + 31) / 32; }
constexpr int kSchurLuDefault = 1;  // 0 panels, 1 cooperative FMA, 2 cooperative DMMA
double dmma_peak_tflops();
// The reference's DenseSolver (dense.cu).
void launch_dense_factor(int n, const int64_t* ap, const int64_t* ai, const double* ax,
                         double* A, int* piv, int* status, cudaStream_t s);
void launch_dense_solve(int n, const double* A, const int* piv, const double* rhs, double* out,
                        int* status, cudaStream_t s);
void launch_dense_lu_solve(const double* S, int bs, double* x, cudaStream_t s);
void launch_bbd_border_rhs(const double* ax, const double* rhs, const double* z,
                           const BbdArgs& B, double* bb, cudaStream_t s);
void launch_bbd_rmatvec(const double* ax, const double* xT, const BbdArgs& B, double* w,
                        cudaStream_t s);
void launch_gather(double* dst, const double* src, const int* idx, int n, cudaStream_t s);
void launch_bbd_combine(const double* z, const double* w2, const double* xT, const BbdArgs& B,
                        double* x, cudaStream_t s);

// One thread block per frequency; shared memory ac_smem_bytes(n, 256).
size_t ac_smem_bytes(int n, int threads);
void launch_ac_dense(const AcArgs& a, int nf, cudaStream_t s);
bool ac_fits_shared(int n);
void launch_ac_dense_global(const AcArgs& a, int nf, int blocks, cudaStream_t s);

// Transient forward / adjoint over a batch: one warp per instance.
void launch_atran(const BatchArgs& a, const AtranArgs& t, int grid, cudaStream_t s);
void atran_kernel_info(int region, int prog_ints, int* regs, int* blocks_per_sm);
void launch_tran_forward(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s);
void launch_tran_backward(const BatchArgs& a, int grid, int warps_per_block, cudaStream_t s);
void tran_kernel_info(bool backward, int warps_per_block, int region, int prog_ints, int* regs,
                      int* blocks_per_sm);
// shared: the warps share one program and the block holds shared_bytes.
void batch_kernel_info(int m, int warps_per_block, int region, int prog_ints, int* regs,
                       int* blocks_per_sm, bool shared = false, size_t shared_bytes = 0);

}  // namespace gk
