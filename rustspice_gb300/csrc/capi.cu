// Host side of libgpuklu: the GpuKluSolver handle behind the LinearSolver C
// ABI, the device-stamp compiler, the device-resident Newton driver and the
// batched Newton. The numeric work is all in kernels.cu; this file owns the
// device memory, the pattern cache and the call sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gpuklu.h"
#include "analysis.h"
#include "kernels.cuh"

using gk::i32;
using gk::i64;

namespace {

std::string cuda_msg(cudaError_t e, const char* what) {
  return std::string(what) + ": " + cudaGetErrorString(e);
}

// Owning device allocation.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t resize(size_t k) {
    if (k <= n && p) return cudaSuccess;
    release();
    n = k;
    return cudaMalloc(&p, std::max<size_t>(k, 1) * sizeof(T));
  }
  cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = resize(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

int sm_count() {
  static int c = 0;
  if (!c) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    if (c <= 0) c = 1;
  }
  return c;
}

// Solve task order: blocks in the order their coupling requires, inside a
// block the L rows ascending then the U rows descending. For the transpose
// the block order reverses and U^T rows come first.
std::vector<i32> make_tasks(const gk::Plan& p, bool transpose) {
  std::vector<i32> t;
  t.reserve(2 * p.n);
  const bool fwd = transpose ? !p.offd_lower : p.offd_lower;
  for (int bb = 0; bb < p.nblocks; ++bb) {
    int b = fwd ? bb : p.nblocks - 1 - bb;
    int b0 = p.block_ptr[b], b1 = p.block_ptr[b + 1];
    for (int i = b0; i < b1; ++i) t.push_back(i << 1);
    for (int i = b1 - 1; i >= b0; --i) t.push_back((i << 1) | 1);
  }
  return t;
}

// Device copy of a Plan.
struct PlanDev {
  DBuf<i32> col_ptr, dslot, slot_row, upd_ptr, upd_dst, col_single, amap_ptr, amap_idx,
      offd_ptr, offd_col, offd_raw, lrow_ptr, lrow_col, lrow_slot, urow_ptr, urow_col,
      urow_slot, in_row, out_col, pcol_ptr, pcol_raw, pcol_q, pos_block, block_ptr, task,
      ttask;
  gk::DPlan dp{}, dpt{};

  cudaError_t upload(const gk::Plan& p, cudaStream_t s) {
    std::vector<i32> h_in_row(p.n), h_out_col(p.n), bp(p.block_ptr.begin(), p.block_ptr.end());
    for (int r = 0; r < p.n; ++r) h_in_row[p.in_pos[r]] = r;
    for (int c = 0; c < p.n; ++c) h_out_col[p.out_pos[c]] = c;
    cudaError_t e = cudaSuccess;
#define UP(name, vec) \
  if (e == cudaSuccess) e = name.upload(vec, s);
    UP(col_ptr, p.col_ptr) UP(dslot, p.dslot) UP(slot_row, p.slot_row) UP(upd_ptr, p.upd_ptr)
    UP(upd_dst, p.upd_dst) UP(col_single, p.col_single) UP(amap_ptr, p.amap_ptr)
    UP(amap_idx, p.amap_idx) UP(offd_ptr, p.offd_ptr) UP(offd_col, p.offd_col)
    UP(offd_raw, p.offd_raw) UP(lrow_ptr, p.lrow_ptr) UP(lrow_col, p.lrow_col)
    UP(lrow_slot, p.lrow_slot) UP(urow_ptr, p.urow_ptr) UP(urow_col, p.urow_col)
    UP(urow_slot, p.urow_slot) UP(in_row, h_in_row) UP(out_col, h_out_col)
    UP(pcol_ptr, p.pcol_ptr) UP(pcol_raw, p.pcol_raw) UP(pcol_q, p.pcol_q)
    UP(pos_block, p.pos_block) UP(block_ptr, bp)
#undef UP
    std::vector<i32> t = make_tasks(p, false), tt = make_tasks(p, true);
    if (e == cudaSuccess) e = task.upload(t, s);
    if (e == cudaSuccess) e = ttask.upload(tt, s);
    gk::DPlan d{};
    d.n = p.n;
    d.nslots = p.nslots();
    d.nblocks = p.nblocks;
    d.ntask = (int)t.size();
    d.col_ptr = col_ptr.p;
    d.dslot = dslot.p;
    d.slot_row = slot_row.p;
    d.upd_ptr = upd_ptr.p;
    d.upd_dst = upd_dst.p;
    d.col_single = col_single.p;
    d.amap_ptr = amap_ptr.p;
    d.amap_idx = amap_idx.p;
    d.offd_ptr = offd_ptr.p;
    d.offd_col = offd_col.p;
    d.offd_raw = offd_raw.p;
    d.lrow_ptr = lrow_ptr.p;
    d.lrow_col = lrow_col.p;
    d.lrow_slot = lrow_slot.p;
    d.urow_ptr = urow_ptr.p;
    d.urow_col = urow_col.p;
    d.urow_slot = urow_slot.p;
    d.in_row = in_row.p;
    d.out_col = out_col.p;
    d.pcol_ptr = pcol_ptr.p;
    d.pcol_raw = pcol_raw.p;
    d.pcol_q = pcol_q.p;
    d.pos_block = pos_block.p;
    d.block_ptr = block_ptr.p;
    d.task = task.p;
    dp = d;
    dpt = d;
    dpt.task = ttask.p;
    dpt.ntask = (int)tt.size();
    return e;
  }
};

}  // namespace

// ====================================================================== circuit
struct gpuklu_circuit {
  int node_count = 0, n = 0, ndev = 0, transient = 0;
  std::vector<i64> ap, ai;
  std::vector<i32> type, nodes, raw, rhs_slot, rhs_ptr, rhs_src;
  std::vector<double> p;
  int pin_raw = -1;
  int ncontrib = 0;
  cudaStream_t stream = nullptr;
  DBuf<i32> d_type, d_nodes, d_raw, d_rhs_slot, d_rhs_ptr, d_rhs_src;
  DBuf<double> d_p;
  gk::DCircuit dc{};
  std::string err;
};

namespace {

// Replays the reference's build closure symbolically: every instance's
// inserts in stamping order (crates/sim-core/src/stamp.rs:242-545, 759-787),
// one aux row per V source in device order (mna.rs:472-480), the ground pin
// last (engine.rs:280), then a stable per-column sort by row (mna.rs:320-347).
std::string compile_circuit(gpuklu_circuit& c) {
  const int nc = c.node_count;
  int naux = 0;
  for (int d = 0; d < c.ndev; ++d)
    if (c.type[d] == 1) ++naux;
  const int n = nc + naux;
  c.n = n;
  struct Ins {
    int row, col, dev, e;
  };
  std::vector<Ins> ins;
  std::vector<std::pair<int, int>> rhs;  // (row, contribution id)
  c.raw.assign((size_t)c.ndev * 8, -1);
  c.rhs_slot.assign((size_t)c.ndev * 2, -1);
  int aux = 0;
  auto add = [&](int i, int j, int d, int e) { ins.push_back({i, j, d, e}); };
  auto add_rhs = [&](int i, int d, int e) {
    int id = (int)rhs.size();
    rhs.push_back({i, id});
    c.rhs_slot[(size_t)d * 2 + e] = id;
  };
  for (int d = 0; d < c.ndev; ++d) {
    int* nd = &c.nodes[(size_t)d * 4];
    const int t = c.type[d];
    const int nn = (t == 4 || t == 6) ? 3 : 2;
    for (int q = 0; q < nn; ++q)
      if (nd[q] < 0 || nd[q] >= nc) return "device " + std::to_string(d) + ": node out of range";
    const int a = nd[0], b = nd[1];
    switch (t) {
      case 0:
      case 3:
        add(a, a, d, 0);
        add(b, b, d, 1);
        add(a, b, d, 2);
        add(b, a, d, 3);
        if (t == 3) {
          add_rhs(a, d, 0);
          add_rhs(b, d, 1);
        }
        break;
      case 1: {
        int k = nc + aux++;
        nd[2] = k;
        add(a, k, d, 0);
        add(b, k, d, 1);
        add(k, a, d, 2);
        add(k, b, d, 3);
        add_rhs(k, d, 0);
        break;
      }
      case 2:
        add_rhs(a, d, 0);
        add_rhs(b, d, 1);
        break;
      case 4:
      case 6: {
        int dr = nd[0], g = nd[1], s = nd[2];
        add(dr, dr, d, 0);
        add(s, s, d, 1);
        add(dr, s, d, 2);
        add(s, dr, d, 3);
        add(dr, g, d, 4);
        add(dr, s, d, 5);
        add(s, g, d, 6);
        add(s, s, d, 7);
        add_rhs(dr, d, 0);
        add_rhs(s, d, 1);
        break;
      }
      case 5:
        if (c.transient) {
          add(a, a, d, 0);
          add(b, b, d, 1);
          add(a, b, d, 2);
          add(b, a, d, 3);
          add_rhs(a, d, 0);
          add_rhs(b, d, 1);
        }
        break;
      default:
        return "device " + std::to_string(d) + ": unknown type " + std::to_string(t);
    }
  }
  ins.push_back({0, 0, -1, 0});  // ground pin
  std::vector<std::vector<int>> cols(n);
  for (int q = 0; q < (int)ins.size(); ++q) cols[ins[q].col].push_back(q);
  c.ap.assign(n + 1, 0);
  c.ai.clear();
  for (int j = 0; j < n; ++j) {
    std::stable_sort(cols[j].begin(), cols[j].end(),
                     [&](int x, int y) { return ins[x].row < ins[y].row; });
    for (int q : cols[j]) {
      int idx = (int)c.ai.size();
      c.ai.push_back(ins[q].row);
      if (ins[q].dev >= 0)
        c.raw[(size_t)ins[q].dev * 8 + ins[q].e] = idx;
      else
        c.pin_raw = idx;
    }
    c.ap[j + 1] = (i64)c.ai.size();
  }
  c.ncontrib = (int)rhs.size();
  c.rhs_ptr.assign(n + 1, 0);
  for (auto& r : rhs) ++c.rhs_ptr[r.first + 1];
  for (int i = 0; i < n; ++i) c.rhs_ptr[i + 1] += c.rhs_ptr[i];
  c.rhs_src.assign(rhs.size(), 0);
  std::vector<int> fill(c.rhs_ptr.begin(), c.rhs_ptr.end() - 1);
  for (auto& r : rhs) c.rhs_src[fill[r.first]++] = r.second;
  return "";
}

cudaError_t upload_circuit(gpuklu_circuit& c) {
  cudaError_t e = cudaSuccess;
  cudaStream_t s = c.stream;
  if (e == cudaSuccess) e = c.d_type.upload(c.type, s);
  if (e == cudaSuccess) e = c.d_nodes.upload(c.nodes, s);
  if (e == cudaSuccess) e = c.d_p.upload(c.p, s);
  if (e == cudaSuccess) e = c.d_raw.upload(c.raw, s);
  if (e == cudaSuccess) e = c.d_rhs_slot.upload(c.rhs_slot, s);
  if (e == cudaSuccess) e = c.d_rhs_ptr.upload(c.rhs_ptr, s);
  if (e == cudaSuccess) e = c.d_rhs_src.upload(c.rhs_src, s);
  gk::DCircuit d{};
  d.ndev = c.ndev;
  d.node_count = c.node_count;
  d.n = c.n;
  d.nnz_raw = (int)c.ai.size();
  d.pin_raw = c.pin_raw;
  d.type = c.d_type.p;
  d.nodes = c.d_nodes.p;
  d.p = c.d_p.p;
  d.raw = c.d_raw.p;
  d.rhs_slot = c.d_rhs_slot.p;
  d.rhs_ptr = c.d_rhs_ptr.p;
  d.rhs_src = c.d_rhs_src.p;
  c.dc = d;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace

// ====================================================================== handle
struct gpuklu_handle {
  enum State { EMPTY, ANALYZED, FACTORED };
  int64_t n = 0;
  int pivot_mode = GPUKLU_PIVOT_REFERENCE;
  State state = EMPTY;
  gk::Plan plan;
  PlanDev pd;
  std::vector<i64> last_ap, last_ai;
  cudaStream_t stream = nullptr;
  DBuf<double> d_ax, d_lu, d_z, d_x, d_out, d_rhs, d_work, d_rc, d_rhs_c, d_xnew, d_newx,
      d_scratch2;
  DBuf<unsigned> d_flags, d_zflag, d_xflag, d_counter;
  DBuf<int> d_rperm, d_rinv, d_status;
  DBuf<gk::NewtonState> d_nstate;
  unsigned epoch = 0, sepoch = 0;
  int64_t factor_count = 0, refactor_count = 0;
  double rcond = 0.0;
  bool rcond_valid = false;
  std::string err;
  int grid_cols = 1;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, what));
  }

  void reset() {
    state = EMPTY;
    last_ap.clear();
    last_ai.clear();
    plan = gk::Plan();
    factor_count = refactor_count = 0;
    rcond = 0.0;
    rcond_valid = false;
  }

  bool same_pattern(const int64_t* ap, int64_t ap_len, const int64_t* ai, int64_t ai_len) const {
    return (int64_t)last_ap.size() == ap_len && (int64_t)last_ai.size() == ai_len &&
           std::equal(last_ap.begin(), last_ap.end(), ap) &&
           std::equal(last_ai.begin(), last_ai.end(), ai);
  }

  int upload_plan() {
    cudaError_t e = pd.upload(plan, stream);
    if (e == cudaSuccess) e = d_lu.resize(std::max(plan.nslots(), 1));
    if (e != cudaSuccess) return cuda_fail(e, "upload plan");
    return GPUKLU_OK;
  }

  int do_analyze(const int64_t* ap, int64_t ap_len, const int64_t* ai, int64_t ai_len) {
    if (ap_len != n + 1)
      return fail(GPUKLU_INVALID_MATRIX, "Column pointer length " + std::to_string(ap_len) +
                                             " != expected " + std::to_string(n + 1));
    if (ap[n] != ai_len || ap[0] != 0)
      return fail(GPUKLU_INVALID_MATRIX, "ap[n] does not match the row index count");
    std::string m = gk::analyze((int)n, ap, ai, pivot_mode, plan);
    if (!m.empty()) return fail(GPUKLU_INVALID_MATRIX, m);
    last_ap.assign(ap, ap + ap_len);
    last_ai.assign(ai, ai + ai_len);
    int st = upload_plan();
    if (st) return st;
    cudaError_t e = cudaSuccess;
    size_t nn = (size_t)std::max<int64_t>(n, 1);
    if (e == cudaSuccess) e = d_ax.resize(std::max<int64_t>(ai_len, 1));
    for (auto* b : {&d_z, &d_x, &d_out, &d_rhs, &d_work, &d_xnew, &d_newx})
      if (e == cudaSuccess) e = b->resize(nn);
    for (auto* b : {&d_flags, &d_zflag, &d_xflag})
      if (e == cudaSuccess) e = b->resize(nn);
    if (e == cudaSuccess) e = d_counter.resize(1);
    if (e == cudaSuccess) e = d_rperm.resize(nn);
    if (e == cudaSuccess) e = d_rinv.resize(nn);
    if (e == cudaSuccess) e = d_status.resize(1);
    if (e == cudaSuccess) e = d_rc.resize(2);
    if (e == cudaSuccess) e = d_nstate.resize(1);
    if (e == cudaSuccess) {
      cudaMemsetAsync(d_flags.p, 0, nn * sizeof(unsigned), stream);
      cudaMemsetAsync(d_zflag.p, 0, nn * sizeof(unsigned), stream);
      cudaMemsetAsync(d_xflag.p, 0, nn * sizeof(unsigned), stream);
      e = cudaMemsetAsync(d_status.p, 0, sizeof(int), stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "analyze buffers");
    epoch = sepoch = 0;
    grid_cols = std::max(1, std::min<int>((int)((n + 3) / 4), sm_count() * 16));
    state = ANALYZED;
    return GPUKLU_OK;
  }

  int check_status(const char* what) {
    int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, d_status.p, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (st != 0) {
      cudaMemsetAsync(d_status.p, 0, sizeof(int), stream);
      return fail(st, std::string(what) + ": device status " + std::to_string(st));
    }
    return GPUKLU_OK;
  }

  unsigned next_epoch(unsigned& ep, DBuf<unsigned>& f) {
    if (++ep == 0) {  // wrapped: clear the flags
      cudaMemsetAsync(f.p, 0, f.n * sizeof(unsigned), stream);
      ep = 1;
    }
    return ep;
  }

  // Factor with the values already in d_ax.
  int factor_on_device(bool sync) {
    rcond_valid = false;
    if (state == FACTORED) {
      unsigned ep = next_epoch(epoch, d_flags);
      gk::launch_refactor(pd.dp, d_ax.p, d_lu.p, d_flags.p, ep, d_counter.p, d_status.p,
                          grid_cols, stream);
      ++refactor_count;
      if (!sync) return GPUKLU_OK;
      return check_status("refactor");
    }
    // First factorization: the reference's pivot pass.
    gk::launch_first_factor(pd.dp, d_ax.p, d_lu.p, d_work.p, d_rperm.p, d_rinv.p, 0.001,
                            d_status.p, stream);
    std::vector<i32> rperm(n);
    cudaError_t e = cudaMemcpyAsync(rperm.data(), d_rperm.p, n * sizeof(i32),
                                    cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "first factor");
    int st = check_status("first factor");
    if (st) return st;
    gk::set_pivots(plan, last_ap.data(), last_ai.data(), rperm);
    st = upload_plan();
    if (st) return st;
    if (pivot_mode == GPUKLU_PIVOT_EXACT) {  // refactor the exact pattern
      unsigned ep = next_epoch(epoch, d_flags);
      gk::launch_refactor(pd.dp, d_ax.p, d_lu.p, d_flags.p, ep, d_counter.p, d_status.p,
                          grid_cols, stream);
    }
    ++factor_count;
    state = FACTORED;
    return check_status("factor");
  }

  // Solve with rhs in d_rhs; result in d_out (original column order).
  int solve_on_device(bool transpose, bool sync) {
    if (transpose && plan.noffdiag > 0)
      return fail(GPUKLU_SOLVE_FAILED, "transpose solve with BTF coupling blocks");
    unsigned ep = sepoch + 1;
    if (ep == 0) ep = 1;
    sepoch = ep;
    if (ep == 1) {
      cudaMemsetAsync(d_zflag.p, 0, d_zflag.n * sizeof(unsigned), stream);
      cudaMemsetAsync(d_xflag.p, 0, d_xflag.n * sizeof(unsigned), stream);
    }
    const int grid = std::max(1, std::min<int>((int)((2 * n + 3) / 4), sm_count() * 16));
    gk::launch_solve(transpose ? pd.dpt : pd.dp, d_rhs.p, d_ax.p, d_lu.p, d_z.p, d_x.p,
                     d_out.p, d_zflag.p, d_xflag.p, ep, d_counter.p, d_status.p, grid,
                     transpose, stream);
    if (!sync) return GPUKLU_OK;
    return check_status("solve");
  }
};

// ====================================================================== C ABI
extern "C" {

gpuklu_handle* gpuklu_create(int64_t n) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    fprintf(stderr, "gpuklu: no CUDA device (%s)\n", cudaGetErrorString(e));
    return nullptr;
  }
  auto* h = new gpuklu_handle();
  h->n = n;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return nullptr;
  }
  return h;
}

void gpuklu_destroy(gpuklu_handle* h) {
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  cudaStream_t s = h->stream;
  delete h;
  cudaStreamDestroy(s);
}

void gpuklu_prepare(gpuklu_handle* h, int64_t n) {
  if (h && n != h->n) {
    h->reset();
    h->n = n;
  }
}

int gpuklu_analyze(gpuklu_handle* h, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                   int64_t ai_len) {
  if (!h) return GPUKLU_INVALID_MATRIX;
  if (h->state != gpuklu_handle::EMPTY && h->same_pattern(ap, ap_len, ai, ai_len))
    return GPUKLU_OK;
  return h->do_analyze(ap, ap_len, ai, ai_len);
}

int gpuklu_factor(gpuklu_handle* h, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                  int64_t ai_len, const double* ax) {
  if (!h) return GPUKLU_INVALID_MATRIX;
  if (h->state == gpuklu_handle::EMPTY || !h->same_pattern(ap, ap_len, ai, ai_len)) {
    int st = h->do_analyze(ap, ap_len, ai, ai_len);
    if (st) return st;
  }
  cudaError_t e = cudaMemcpyAsync(h->d_ax.p, ax, ai_len * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "factor upload");
  return h->factor_on_device(true);
}

int gpuklu_factor_device(gpuklu_handle* h, const double* d_ax) {
  if (!h || h->state == gpuklu_handle::EMPTY) return GPUKLU_FACTOR_FAILED;
  cudaError_t e = cudaMemcpyAsync(h->d_ax.p, d_ax, h->last_ai.size() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "factor_device copy");
  return h->factor_on_device(true);
}

int gpuklu_solve(gpuklu_handle* h, double* rhs, int64_t len) {
  if (!h || h->state != gpuklu_handle::FACTORED) return GPUKLU_SOLVE_FAILED;
  if (len != h->n)
    return h->fail(GPUKLU_INVALID_MATRIX, "RHS length " + std::to_string(len) +
                                              " != matrix dimension " + std::to_string(h->n));
  cudaError_t e = cudaMemcpyAsync(h->d_rhs.p, rhs, len * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "solve upload");
  int st = h->solve_on_device(false, false);
  if (st) return st;
  e = cudaMemcpyAsync(rhs, h->d_out.p, len * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "solve download");
  return h->check_status("solve");
}

int gpuklu_solve_device(gpuklu_handle* h, double* d_rhs) {
  if (!h || h->state != gpuklu_handle::FACTORED) return GPUKLU_SOLVE_FAILED;
  cudaError_t e = cudaMemcpyAsync(h->d_rhs.p, d_rhs, h->n * sizeof(double),
                                  cudaMemcpyDeviceToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "solve_device copy");
  int st = h->solve_on_device(false, false);
  if (st) return st;
  e = cudaMemcpyAsync(d_rhs, h->d_out.p, h->n * sizeof(double), cudaMemcpyDeviceToDevice,
                      h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "solve_device copy back");
  return h->check_status("solve_device");
}

int gpuklu_tsolve(gpuklu_handle* h, double* g, int64_t len) {
  if (!h || h->state != gpuklu_handle::FACTORED) return GPUKLU_SOLVE_FAILED;
  if (len != h->n) return h->fail(GPUKLU_INVALID_MATRIX, "RHS length mismatch");
  cudaError_t e = cudaMemcpyAsync(h->d_rhs.p, g, len * sizeof(double), cudaMemcpyHostToDevice,
                                  h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "tsolve upload");
  int st = h->solve_on_device(true, false);
  if (st) return st;
  e = cudaMemcpyAsync(g, h->d_out.p, len * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "tsolve download");
  return h->check_status("tsolve");
}

void gpuklu_reset_pattern(gpuklu_handle* h) {
  if (h) h->reset();
}

const char* gpuklu_name(const gpuklu_handle*) { return "GpuKLU"; }

void gpuklu_set_parallel_threads(gpuklu_handle*, size_t) {}

int gpuklu_set_pivot_mode(gpuklu_handle* h, int mode) {
  if (!h || (mode != GPUKLU_PIVOT_REFERENCE && mode != GPUKLU_PIVOT_EXACT))
    return GPUKLU_INVALID_MATRIX;
  if (mode != h->pivot_mode) {
    h->pivot_mode = mode;
    h->reset();
  }
  return GPUKLU_OK;
}

int gpuklu_get_stats(gpuklu_handle* h, gpuklu_stats* out) {
  if (!h || !out) return GPUKLU_INVALID_MATRIX;
  if (h->state == gpuklu_handle::FACTORED && !h->rcond_valid) {
    gk::launch_rcond(h->pd.dp, h->d_lu.p, h->d_rc.p, h->stream);
    double mm[2];
    cudaMemcpyAsync(mm, h->d_rc.p, sizeof(mm), cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    h->rcond = mm[1] > 0.0 ? mm[0] / mm[1] : 0.0;
    h->rcond_valid = true;
  }
  out->factor_count = h->factor_count;
  out->refactor_count = h->refactor_count;
  out->nnz_l = h->plan.nnz_l;
  out->nnz_u = h->plan.nnz_u;
  out->nblocks = h->plan.nblocks;
  out->noffdiag = h->plan.noffdiag;
  out->pivot_swaps = h->plan.swaps;
  out->refactor_flops = h->plan.flops_refactor;
  out->rcond = h->state == gpuklu_handle::FACTORED ? h->rcond : 0.0;
  return GPUKLU_OK;
}

const char* gpuklu_last_error(const gpuklu_handle* h) { return h ? h->err.c_str() : ""; }

void* gpuklu_stream(gpuklu_handle* h) { return h ? (void*)h->stream : nullptr; }

// ---------------------------------------------------------------- circuits
gpuklu_circuit* gpuklu_compile_devices(int64_t node_count, int64_t ndev, const int32_t* type,
                                       const int32_t* nodes, const double* p, int transient) {
  auto c = std::make_unique<gpuklu_circuit>();
  c->node_count = (int)node_count;
  c->ndev = (int)ndev;
  c->transient = transient;
  c->type.assign(type, type + ndev);
  c->nodes.assign(nodes, nodes + ndev * 4);
  c->p.assign(p, p + ndev * 6);
  std::string m = compile_circuit(*c);
  if (!m.empty()) {
    fprintf(stderr, "gpuklu_compile_devices: %s\n", m.c_str());
    return nullptr;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  cudaError_t e = upload_circuit(*c);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_compile_devices: %s\n", cudaGetErrorString(e));
    cudaStreamDestroy(c->stream);
    return nullptr;
  }
  return c.release();
}

void gpuklu_circuit_free(gpuklu_circuit* c) {
  if (!c) return;
  cudaStreamSynchronize(c->stream);
  cudaStream_t s = c->stream;
  delete c;
  cudaStreamDestroy(s);
}

int gpuklu_circuit_dims(const gpuklu_circuit* c, int64_t* n, int64_t* nnz) {
  if (!c) return GPUKLU_INVALID_MATRIX;
  *n = c->n;
  *nnz = (int64_t)c->ai.size();
  return GPUKLU_OK;
}

int gpuklu_circuit_pattern(const gpuklu_circuit* c, int64_t* ap, int64_t* ai) {
  if (!c) return GPUKLU_INVALID_MATRIX;
  std::copy(c->ap.begin(), c->ap.end(), ap);
  std::copy(c->ai.begin(), c->ai.end(), ai);
  return GPUKLU_OK;
}

int gpuklu_circuit_set_params(gpuklu_circuit* c, const double* p) {
  if (!c) return GPUKLU_INVALID_MATRIX;
  std::copy(p, p + (size_t)c->ndev * 6, c->p.begin());
  cudaError_t e = cudaMemcpyAsync(c->d_p.p, c->p.data(), c->p.size() * sizeof(double),
                                  cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? GPUKLU_OK : GPUKLU_CUDA_ERROR;
}

int gpuklu_stamp(gpuklu_handle* h, gpuklu_circuit* c, const double* x, int64_t xlen,
                 double gmin, double source_scale, double dt, const double* cap_v,
                 double be_sign, double* ax_out, double* rhs_out) {
  if (!h || !c) return GPUKLU_INVALID_MATRIX;
  DBuf<double> dx, dax, drc, drhs, dcap;
  cudaError_t e = dx.resize(std::max<int64_t>(xlen, 1));
  if (e == cudaSuccess) e = dax.resize(c->ai.size());
  if (e == cudaSuccess) e = drc.resize(std::max(c->ncontrib, 1));
  if (e == cudaSuccess) e = drhs.resize(c->n);
  if (e == cudaSuccess && cap_v) e = dcap.resize(c->ndev);
  if (e == cudaSuccess && xlen > 0)
    e = cudaMemcpyAsync(dx.p, x, xlen * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess && cap_v)
    e = cudaMemcpyAsync(dcap.p, cap_v, c->ndev * sizeof(double), cudaMemcpyHostToDevice,
                        h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "stamp upload");
  gk::launch_stamp(c->dc, dx.p, (int)xlen, gmin, source_scale, dt, cap_v ? dcap.p : nullptr,
                   be_sign, dax.p, drc.p, drhs.p, h->stream);
  e = cudaMemcpyAsync(ax_out, dax.p, c->ai.size() * sizeof(double), cudaMemcpyDeviceToHost,
                      h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rhs_out, drhs.p, c->n * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "stamp");
  return GPUKLU_OK;
}

int gpuklu_newton_dc(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                     const double* x0, double* x_out, int64_t x_cap, int64_t* x_len,
                     int64_t* iters, int64_t* iters_total, int* reason) {
  if (!h || !c || !cfg) return GPUKLU_INVALID_MATRIX;
  // Engine::run_dc_result: x = zeros(node_count), solver.prepare(node_count)
  gpuklu_prepare(h, c->node_count);
  // build(x) returns n = node_count + aux; run_newton calls prepare(n)
  gpuklu_prepare(h, c->n);
  int st = gpuklu_analyze(h, c->ap.data(), (int64_t)c->ap.size(), c->ai.data(),
                          (int64_t)c->ai.size());
  if (st) return st;
  const int nc = c->node_count, n = c->n;
  cudaError_t e = h->d_rhs_c.resize(std::max(c->ncontrib, 1));
  if (e != cudaSuccess) return h->cuda_fail(e, "newton buffers");
  std::vector<double> xinit(n, 0.0);
  if (x0) std::copy(x0, x0 + nc, xinit.begin());
  e = cudaMemcpyAsync(h->d_newx.p, xinit.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                      h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "newton x0");
  gk::NewtonCfg nc_{};
  nc_.max_iters = (int)cfg->max_iters;
  nc_.gmin_steps = (int)cfg->gmin_steps;
  nc_.abs_tol = cfg->abs_tol;
  nc_.rel_tol = cfg->rel_tol;
  nc_.gmin = cfg->gmin;
  nc_.damping = cfg->damping;
  nc_.damping_min = cfg->damping_min;
  const double gstart = std::max(cfg->gmin * 1e3, 1e-6);
  int64_t total = 0, last_iters = 0;
  int rsn = 1;
  bool conv = false, failed = false;
  for (int64_t gi = 0; gi <= cfg->gmin_steps && !conv && !failed; ++gi) {
    const double gmin =
        cfg->gmin_steps == 0 ? cfg->gmin
                             : gstart + (cfg->gmin - gstart) * ((double)gi / (double)cfg->gmin_steps);
    for (int64_t si = 0; si <= cfg->source_steps && !conv && !failed; ++si) {
      const double scale =
          cfg->source_steps == 0 ? 1.0 : (double)si / (double)cfg->source_steps;
      gk::NewtonState ns{cfg->damping, DBL_MAX, 0.0, 0, 0};
      e = cudaMemcpyAsync(h->d_nstate.p, &ns, sizeof(ns), cudaMemcpyHostToDevice, h->stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "newton state");
      int64_t it = 0;
      rsn = 1;
      for (; it < cfg->max_iters; ++it) {
        gk::launch_stamp(c->dc, h->d_newx.p, nc, gmin, scale, 0.0, nullptr, -1.0, h->d_ax.p,
                         h->d_rhs_c.p, h->d_rhs.p, h->stream);
        st = h->factor_on_device(h->state != gpuklu_handle::FACTORED);
        if (st == GPUKLU_OK) st = h->solve_on_device(false, false);
        if (st != GPUKLU_OK) {
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        gk::launch_newton_update(nc, n, h->d_newx.p, h->d_out.p, h->d_nstate.p, nc_,
                                 h->d_status.p, h->stream);
        gk::NewtonState hs;
        e = cudaMemcpyAsync(&hs, h->d_nstate.p, sizeof(hs), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "newton step");
        int dst = 0;
        cudaMemcpy(&dst, h->d_status.p, sizeof(int), cudaMemcpyDeviceToHost);
        if (dst == GPUKLU_DEVICE_TIMEOUT) {
          cudaMemset(h->d_status.p, 0, sizeof(int));
          h->err = "device dependency wait timed out";
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        if (dst) cudaMemset(h->d_status.p, 0, sizeof(int));
        if (hs.converged) {
          conv = true;
          rsn = 0;
          ++it;
          break;
        }
      }
      total += it;
      last_iters = it;
    }
  }
  const int64_t len = conv ? n : nc;
  std::vector<double> xh(n);
  e = cudaMemcpyAsync(xh.data(), h->d_newx.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                      h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "newton result");
  for (int64_t i = 0; i < std::min(len, x_cap); ++i) x_out[i] = xh[i];
  if (x_len) *x_len = len;
  if (iters) *iters = last_iters;
  if (iters_total) *iters_total = total;
  if (reason) *reason = rsn;
  return GPUKLU_OK;
}

}  // extern "C"

// ====================================================================== batch
struct gpuklu_batch {
  int64_t ncirc = 0, ninst = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<gk::GroupHdr> groups;
  std::vector<gk::Tile> tiles;
  std::vector<int> inst_n;
  DBuf<gk::GroupHdr> d_groups;
  DBuf<gk::Tile> d_tiles;
  DBuf<unsigned> d_counter;
  DBuf<i32> d_dev_type, d_dev_nodes, d_dev_slot, d_col_ptr, d_dslot, d_col_single, d_in_row,
      d_out_pos, d_offd_ptr, d_slot_row, d_upd_ptr, d_upd_dst, d_offd_col, d_block_ptr,
      d_ov_dev, d_iters, d_iters_total, d_reason, d_status;
  DBuf<double> d_dev_p, d_ov_val, d_x0, d_buf, d_xout;
  DBuf<long long> d_x0_off, d_x_off;
  std::vector<long long> x_off;
  int64_t x0_len = 0, xout_len = 0;
  int grid = 0, block = 128;
  long long buf_stride = 0;
  int64_t bytes_per_iter = 0;

  int fail(const std::string& m) {
    err = m;
    return GPUKLU_CUDA_ERROR;
  }
};

extern "C" {

gpuklu_batch* gpuklu_batch_create(int64_t ncirc, const int64_t* dev_off,
                                  const int64_t* node_counts, const int32_t* type,
                                  const int32_t* nodes, const double* p, int64_t ninst,
                                  const int64_t* inst_circ, const int64_t* inst_dev,
                                  const double* inst_val, const double* x0,
                                  const int64_t* x0_off, int64_t x0_len) {
  auto B = std::make_unique<gpuklu_batch>();
  B->ncirc = ncirc;
  B->ninst = ninst;
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  gpuklu_handle* H = gpuklu_create(1);
  if (!H) return nullptr;
  gpuklu_set_pivot_mode(H, GPUKLU_PIVOT_EXACT);
  // first instance of every circuit: its iterate is used for pivot discovery
  std::vector<int64_t> first(ncirc, -1);
  std::vector<std::vector<int64_t>> members(ncirc);
  for (int64_t i = 0; i < ninst; ++i) {
    if (inst_circ[i] < 0 || inst_circ[i] >= ncirc) {
      fprintf(stderr, "gpuklu_batch_create: instance %ld has no circuit\n", (long)i);
      gpuklu_destroy(H);
      return nullptr;
    }
    members[inst_circ[i]].push_back(i);
    if (first[inst_circ[i]] < 0) first[inst_circ[i]] = i;
  }
  std::vector<i32> dtype, dnodes, dslotv, col_ptr, dslot, csing, in_row, out_pos, offd_ptr,
      slot_row, upd_ptr, upd_dst, offd_col, block_ptr;
  std::vector<double> dp;
  long long maxbuf = 0;
  for (int64_t c = 0; c < ncirc; ++c) {
    const int64_t d0 = dev_off[c], nd = dev_off[c + 1] - d0;
    gpuklu_circuit* C = gpuklu_compile_devices(node_counts[c], nd, type + d0, nodes + 4 * d0,
                                               p + 6 * d0, 0);
    if (!C) {
      gpuklu_destroy(H);
      return nullptr;
    }
    const int64_t rep = first[c];
    // pivot discovery on the representative instance's first matrix
    std::vector<double> pc(C->p);
    if (rep >= 0 && inst_dev[rep] >= 0) pc[(size_t)inst_dev[rep] * 6] = inst_val[rep];
    gpuklu_circuit_set_params(C, pc.data());
    std::vector<double> xr(C->node_count, 0.0);
    if (rep >= 0 && x0 && x0_off[rep] >= 0)
      std::copy(x0 + x0_off[rep], x0 + x0_off[rep] + C->node_count, xr.begin());
    std::vector<double> ax(C->ai.size()), rhs(C->n);
    gpuklu_prepare(H, C->n);
    gpuklu_reset_pattern(H);
    int st = gpuklu_stamp(H, C, xr.data(), (int64_t)xr.size(), 1e-12, 1.0, 0.0, nullptr, -1.0,
                          ax.data(), rhs.data());
    if (st == GPUKLU_OK)
      st = gpuklu_factor(H, C->ap.data(), (int64_t)C->ap.size(), C->ai.data(),
                         (int64_t)C->ai.size(), ax.data());
    if (st != GPUKLU_OK) {
      fprintf(stderr, "gpuklu_batch_create: circuit %ld: %s\n", (long)c, H->err.c_str());
      gpuklu_circuit_free(C);
      gpuklu_destroy(H);
      return nullptr;
    }
    const gk::Plan& P = H->plan;
    std::vector<int> raw_offd(C->ai.size(), -1);
    for (size_t e = 0; e < P.offd_raw.size(); ++e) raw_offd[P.offd_raw[e]] = (int)e;
    gk::GroupHdr G{};
    G.n = P.n;
    G.node_count = C->node_count;
    G.nslots = P.nslots();
    G.noffd = (int)P.offd_raw.size();
    G.ndev = (int)nd;
    G.nblocks = P.nblocks;
    G.dev_off = (int)dtype.size();
    G.col_off = (int)col_ptr.size();
    G.slot_off = (int)slot_row.size();
    G.upd_off = (int)upd_dst.size();
    G.offd_off = (int)offd_col.size();
    G.blk_off = (int)block_ptr.size();
    G.pin_slot = C->pin_raw >= 0 ? P.raw_slot[C->pin_raw] : -1;
    G.offd_lower = P.offd_lower ? 1 : 0;
    for (int64_t d = 0; d < nd; ++d) {
      dtype.push_back(C->type[d]);
      for (int q = 0; q < 4; ++q) dnodes.push_back(C->nodes[d * 4 + q]);
      for (int q = 0; q < 6; ++q) dp.push_back(C->p[d * 6 + q]);
      for (int q = 0; q < 8; ++q) {
        int r = C->raw[d * 8 + q];
        int s = -1;
        if (r >= 0) s = P.raw_slot[r] >= 0 ? P.raw_slot[r] : (raw_offd[r] >= 0 ? G.nslots + raw_offd[r] : -1);
        dslotv.push_back(s);
      }
    }
    // column arrays: col_ptr (n+1) and the n-sized ones padded to n+1
    for (int k = 0; k <= P.n; ++k) {
      col_ptr.push_back(P.col_ptr[k]);
      dslot.push_back(k < P.n ? P.dslot[k] : 0);
      csing.push_back(k < P.n ? P.col_single[k] : 0);
      in_row.push_back(0);
      out_pos.push_back(k < P.n ? P.out_pos[k] : 0);
      offd_ptr.push_back(P.offd_ptr[k]);
    }
    for (int r = 0; r < P.n; ++r) in_row[G.col_off + P.in_pos[r]] = r;
    for (int s = 0; s <= P.nslots(); ++s) {
      slot_row.push_back(s < P.nslots() ? P.slot_row[s] : 0);
      upd_ptr.push_back(P.upd_ptr[s]);
    }
    upd_dst.insert(upd_dst.end(), P.upd_dst.begin(), P.upd_dst.end());
    offd_col.insert(offd_col.end(), P.offd_col.begin(), P.offd_col.end());
    block_ptr.insert(block_ptr.end(), P.block_ptr.begin(), P.block_ptr.end());
    G.cost = G.nslots + (int)P.upd_dst.size() + 4 * G.ndev;
    const long long need = 32LL * (G.nslots + G.noffd + 2LL * G.n + G.node_count);
    maxbuf = std::max(maxbuf, need);
    B->bytes_per_iter += 8LL * (2 * (G.nslots + G.noffd) + (long long)P.upd_dst.size() * 3 +
                                4LL * G.n + 2LL * G.node_count) +
                         4LL * ((long long)P.upd_dst.size() + G.nslots + 2LL * G.n);
    const int gid = (int)B->groups.size();
    B->groups.push_back(G);
    auto& mem = members[c];
    for (size_t t0 = 0; t0 < mem.size(); t0 += 32) {
      // instances of a tile must be consecutive: build them from the member list
      gk::Tile T{gid, (int)mem[t0], (int)std::min<size_t>(32, mem.size() - t0)};
      bool contiguous = true;
      for (int q = 1; q < T.count; ++q)
        if (mem[t0 + q] != mem[t0] + q) contiguous = false;
      if (!contiguous) {
        fprintf(stderr, "gpuklu_batch_create: instances of a circuit must be consecutive\n");
        gpuklu_circuit_free(C);
        gpuklu_destroy(H);
        return nullptr;
      }
      B->tiles.push_back(T);
    }
    gpuklu_circuit_free(C);
  }
  gpuklu_destroy(H);
  // longest programs first
  std::stable_sort(B->tiles.begin(), B->tiles.end(), [&](const gk::Tile& a, const gk::Tile& b) {
    return B->groups[a.group].cost > B->groups[b.group].cost;
  });
  // outputs: n values per instance
  B->x_off.assign(ninst, 0);
  long long off = 0;
  for (int64_t i = 0; i < ninst; ++i) {
    B->x_off[i] = off;
    off += B->groups[inst_circ[i]].n;
  }
  B->xout_len = off;
  B->x0_len = x0 ? x0_len : 0;
  // launch geometry: enough resident warps to cover the SMs several times
  int occ = 0;
  B->block = 128;
  B->grid = sm_count() * 8;
  (void)occ;
  const long long nwarps = (long long)B->grid * (B->block / 32);
  B->buf_stride = maxbuf;
  cudaStream_t s = B->stream;
  cudaError_t e = cudaSuccess;
  std::vector<i32> ov_dev(ninst);
  std::vector<double> ov_val(ninst);
  std::vector<long long> x0o(ninst, -1);
  for (int64_t i = 0; i < ninst; ++i) {
    ov_dev[i] = inst_dev[i] >= 0 ? (i32)inst_dev[i] : -1;
    ov_val[i] = inst_val ? inst_val[i] : 0.0;
    if (x0 && x0_off) x0o[i] = x0_off[i];
  }
#define UP(buf, vec) \
  if (e == cudaSuccess) e = B->buf.upload(vec, s);
  UP(d_groups, B->groups) UP(d_tiles, B->tiles) UP(d_dev_type, dtype) UP(d_dev_nodes, dnodes)
  UP(d_dev_slot, dslotv) UP(d_dev_p, dp) UP(d_col_ptr, col_ptr) UP(d_dslot, dslot)
  UP(d_col_single, csing) UP(d_in_row, in_row) UP(d_out_pos, out_pos) UP(d_offd_ptr, offd_ptr)
  UP(d_slot_row, slot_row) UP(d_upd_ptr, upd_ptr) UP(d_upd_dst, upd_dst)
  UP(d_offd_col, offd_col) UP(d_block_ptr, block_ptr) UP(d_ov_dev, ov_dev)
  UP(d_ov_val, ov_val) UP(d_x0_off, x0o) UP(d_x_off, B->x_off)
#undef UP
  if (e == cudaSuccess) {
    std::vector<double> x0v(x0 ? x0 : nullptr, x0 ? x0 + B->x0_len : nullptr);
    e = B->d_x0.upload(x0v, s);
  }
  if (e == cudaSuccess) e = B->d_buf.resize((size_t)(nwarps * B->buf_stride));
  if (e == cudaSuccess) e = B->d_xout.resize(std::max<int64_t>(B->xout_len, 1));
  if (e == cudaSuccess) e = B->d_iters.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_iters_total.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_reason.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_status.resize(1);
  if (e == cudaSuccess) e = B->d_counter.resize(1);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->d_status.p, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_batch_create: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  return B.release();
}

void gpuklu_batch_destroy(gpuklu_batch* b) {
  if (!b) return;
  cudaStreamSynchronize(b->stream);
  cudaStream_t s = b->stream;
  delete b;
  cudaStreamDestroy(s);
}

int gpuklu_batch_run(gpuklu_batch* b, const gpuklu_newton_config* cfg) {
  if (!b || !cfg) return GPUKLU_INVALID_MATRIX;
  gk::NewtonCfg c{};
  c.max_iters = (int)cfg->max_iters;
  c.gmin_steps = (int)cfg->gmin_steps;
  c.abs_tol = cfg->abs_tol;
  c.rel_tol = cfg->rel_tol;
  c.gmin = cfg->gmin;
  c.damping = cfg->damping;
  c.damping_min = cfg->damping_min;
  gk::launch_batch_newton(
      b->d_groups.p, b->d_tiles.p, (int)b->tiles.size(), b->d_counter.p, b->d_dev_type.p,
      b->d_dev_nodes.p, b->d_dev_p.p, b->d_dev_slot.p, b->d_col_ptr.p, b->d_dslot.p,
      b->d_col_single.p, b->d_in_row.p, b->d_out_pos.p, b->d_offd_ptr.p, b->d_slot_row.p,
      b->d_upd_ptr.p, b->d_upd_dst.p, b->d_offd_col.p, b->d_block_ptr.p, b->d_ov_dev.p,
      b->d_ov_val.p, b->d_x0_off.p, b->d_x0.p, c, b->d_buf.p, b->buf_stride, b->d_iters.p,
      b->d_iters_total.p, b->d_reason.p, b->d_x_off.p, b->d_xout.p, b->d_status.p, b->grid,
      b->block, b->stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch launch"));
  return GPUKLU_OK;
}

int gpuklu_batch_results(gpuklu_batch* b, int64_t* iters, int64_t* iters_total, int32_t* reason,
                         double* x_out, const int64_t* x_off) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  const int64_t ni = b->ninst;
  std::vector<i32> it(ni), itt(ni), rs(ni);
  std::vector<double> xo(b->xout_len);
  cudaStream_t s = b->stream;
  cudaError_t e = cudaMemcpyAsync(it.data(), b->d_iters.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(itt.data(), b->d_iters_total.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rs.data(), b->d_reason.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && x_out && b->xout_len)
    e = cudaMemcpyAsync(xo.data(), b->d_xout.p, b->xout_len * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch results"));
  for (int64_t i = 0; i < ni; ++i) {
    if (iters) iters[i] = it[i];
    if (iters_total) iters_total[i] = itt[i];
    if (reason) reason[i] = rs[i];
    if (x_out && x_off) {
      const int gn = b->groups[0].n;  // replaced below per instance
      (void)gn;
    }
  }
  if (x_out && x_off) {
    for (int64_t i = 0; i < ni; ++i) {
      const long long a = b->x_off[i];
      const long long len = (i + 1 < ni ? b->x_off[i + 1] : b->xout_len) - a;
      std::copy(xo.begin() + a, xo.begin() + a + len, x_out + x_off[i]);
    }
  }
  return GPUKLU_OK;
}

int gpuklu_batch_update_inputs(gpuklu_batch* b, const double* inst_val, const double* x0) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  cudaError_t e = cudaSuccess;
  if (inst_val)
    e = cudaMemcpyAsync(b->d_ov_val.p, inst_val, b->ninst * sizeof(double),
                        cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess && x0 && b->x0_len)
    e = cudaMemcpyAsync(b->d_x0.p, x0, b->x0_len * sizeof(double), cudaMemcpyHostToDevice,
                        b->stream);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch inputs"));
  return GPUKLU_OK;
}

const char* gpuklu_batch_last_error(const gpuklu_batch* b) { return b ? b->err.c_str() : ""; }

int gpuklu_batch_info(const gpuklu_batch* b, int64_t* out) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  out[0] = b->grid;
  out[1] = b->block;
  out[2] = (int64_t)b->tiles.size();
  out[3] = (int64_t)b->d_buf.n * 8;
  out[4] = b->bytes_per_iter;
  return GPUKLU_OK;
}

void* gpuklu_batch_stream(gpuklu_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"

// ====================================================================== diagnostics
struct gpuklu_plan {
  gk::Plan p;
  std::vector<int64_t> info;
};

extern "C" {

gpuklu_plan* gpuklu_plan_build(int64_t n, const int64_t* ap, const int64_t* ai, int pivot_mode,
                               const int32_t* row_perm) {
  auto P = std::make_unique<gpuklu_plan>();
  std::string m = gk::analyze((int)n, ap, ai, pivot_mode, P->p);
  if (!m.empty()) {
    fprintf(stderr, "gpuklu_plan_build: %s\n", m.c_str());
    return nullptr;
  }
  if (row_perm) gk::set_pivots(P->p, ap, ai, std::vector<i32>(row_perm, row_perm + n));
  const gk::Plan& p = P->p;
  P->info = {p.n, p.nslots(), p.nblocks, p.nnz_l, p.nnz_u, p.noffdiag, p.offd_lower ? 1 : 0,
             p.swaps};
  return P.release();
}

int64_t gpuklu_plan_array(const gpuklu_plan* P, const char* name, int64_t* out, int64_t cap) {
  if (!P || !name) return -1;
  const gk::Plan& p = P->p;
  std::string k(name);
  auto put = [&](const auto& v) -> int64_t {
    for (int64_t i = 0; i < (int64_t)v.size() && i < cap; ++i) out[i] = (int64_t)v[i];
    return (int64_t)v.size();
  };
  if (k == "info") return put(P->info);
#define ARR(nm) \
  if (k == #nm) return put(p.nm);
  ARR(col_ptr) ARR(dslot) ARR(slot_row) ARR(upd_ptr) ARR(upd_dst) ARR(amap_ptr) ARR(amap_idx)
  ARR(offd_ptr) ARR(offd_col) ARR(offd_raw) ARR(in_pos) ARR(out_pos) ARR(block_ptr)
  ARR(col_single) ARR(pcol_ptr) ARR(pcol_raw) ARR(pcol_q) ARR(pos_block) ARR(raw_slot)
  ARR(row_perm) ARR(lrow_ptr) ARR(lrow_col) ARR(lrow_slot) ARR(urow_ptr) ARR(urow_col)
  ARR(urow_slot)
#undef ARR
  return -1;
}

void gpuklu_plan_free(gpuklu_plan* p) { delete p; }

}  // extern "C"
