// Kernel declarations and the device-side views of a Plan.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gk {

// Device pointers of one Plan (see analysis.h for the meaning of each array).
struct DPlan {
  int n, nslots, nblocks, ntask;
  const int *col_ptr, *dslot, *slot_row, *upd_ptr, *upd_dst, *col_single;
  const int *amap_ptr, *amap_idx;
  const int *offd_ptr, *offd_col, *offd_raw;
  const int *lrow_ptr, *lrow_col, *lrow_slot, *urow_ptr, *urow_col, *urow_slot;
  const int *in_row, *out_col;  // position -> original row / original column
  const int *pcol_ptr, *pcol_raw, *pcol_q, *pos_block, *block_ptr;
  const int *task;              // solve order: (position << 1) | is_upper
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

// Batched program of one circuit group (all instances share it).
struct GroupHdr {
  int n, node_count, nslots, noffd, ndev, nblocks;
  int dev_off;    // device arrays (type, nodes*4, p*6, slot*8)
  int col_off;    // n+1 column arrays (col_ptr, dslot, col_single, in_row, out_col, offd_ptr)
  int slot_off;   // nslots(+1) slot arrays (slot_row, upd_ptr)
  int upd_off;    // upd_dst
  int offd_off;   // offd_col
  int blk_off;    // block_ptr
  int pin_slot;   // value slot of the ground pin
  int offd_lower; // 1: blocks in forward order
  int cost;       // scheduling weight
};

struct Tile {
  int group, first, count;
};

// --------------------------------------------------------------- launches
void launch_first_factor(const DPlan& P, const double* ax, double* lu, double* work,
                         int* rperm, int* rinv, double tol, int* status, cudaStream_t s);
void launch_refactor(const DPlan& P, const double* ax, double* lu, unsigned* flags,
                     unsigned epoch, unsigned* counter, int* status, int grid,
                     cudaStream_t s);
void launch_solve(const DPlan& P, const double* rhs, const double* ax, const double* lu,
                  double* z, double* x, double* out, unsigned* zflag, unsigned* xflag,
                  unsigned epoch, unsigned* counter, int* status, int grid, bool transpose,
                  cudaStream_t s);
void launch_stamp(const DCircuit& C, const double* x, int xlen, double gmin, double scale,
                  double dt, const double* cap_v, double be_sign, double* ax, double* rhs_c,
                  double* rhs, cudaStream_t s);
void launch_newton_update(int m, int n, double* x, const double* xnew, NewtonState* st,
                          NewtonCfg cfg, int* status, cudaStream_t s);
void launch_rcond(const DPlan& P, const double* lu, double* out2, cudaStream_t s);
void launch_batch_newton(const GroupHdr* groups, const Tile* tiles, int ntiles,
                         unsigned* tile_counter, const int* dev_type, const int* dev_nodes,
                         const double* dev_p, const int* dev_slot, const int* col_ptr,
                         const int* dslot, const int* col_single, const int* in_row,
                         const int* out_col, const int* offd_ptr, const int* slot_row,
                         const int* upd_ptr, const int* upd_dst, const int* offd_col,
                         const int* block_ptr, const int* inst_ov_dev,
                         const double* inst_ov_val, const long long* inst_x0_off,
                         const double* x0, NewtonCfg cfg, double* buf, long long buf_stride,
                         int* iters, int* iters_total, int* reason,
                         const long long* inst_x_off, double* x_out, int* status, int grid,
                         int block, cudaStream_t s);

}  // namespace gk
