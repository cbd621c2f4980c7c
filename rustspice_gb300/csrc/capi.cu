// Host side of libgpuklu: the GpuKluSolver handle behind the LinearSolver C
// ABI, the device-stamp compiler, the device-resident Newton loop and the
// batched Newton. The numeric work is all in kernels.cu; this file owns the
// device memory, the pattern cache and the call sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
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
  const bool coupled = !p.offd_ptr.empty() && p.offd_ptr.back() > 0;
  if (!coupled && p.nblocks > 1) {
    // Independent blocks: their tasks interleave (row r of every block, then
    // row r+1, ...; all forward tasks before the backward ones), so the warps
    // that hold the handed-out tasks work on every block at once. Each task
    // still comes after everything it waits for.
    int longest = 0;
    for (int b = 0; b < p.nblocks; ++b)
      longest = std::max(longest, p.block_ptr[b + 1] - p.block_ptr[b]);
    for (int r = 0; r < longest; ++r)
      for (int b = 0; b < p.nblocks; ++b)
        if (p.block_ptr[b] + r < p.block_ptr[b + 1]) t.push_back((p.block_ptr[b] + r) << 1);
    for (int r = 0; r < longest; ++r)
      for (int b = 0; b < p.nblocks; ++b)
        if (p.block_ptr[b + 1] - 1 - r >= p.block_ptr[b])
          t.push_back(((p.block_ptr[b + 1] - 1 - r) << 1) | 1);
    return t;
  }
  const bool fwd = transpose ? !p.offd_lower : p.offd_lower;
  for (int bb = 0; bb < p.nblocks; ++bb) {
    int b = fwd ? bb : p.nblocks - 1 - bb;
    int b0 = p.block_ptr[b], b1 = p.block_ptr[b + 1];
    for (int i = b0; i < b1; ++i) t.push_back(i << 1);
    for (int i = b1 - 1; i >= b0; --i) t.push_back((i << 1) | 1);
  }
  return t;
}

// Chunked schedule of the one-block solve (k_solve_cta): per BTF block in
// solve order, the coupling rows, the forward sweep and the backward sweep,
// cut so that the slots each chunk needs are contiguous and at most
// gk::kSolveChunk long; consecutive pieces share a chunk while their slots fit.
// Appends the schedule of the given BTF blocks, in that order.
void cta_solve_blocks(const gk::Plan& p, const std::vector<int>& blocks, std::vector<i32>& chunk,
                      std::vector<i32>& op) {
  struct Piece {
    int code, a, b, lo, hi;  // slot range [lo, hi), empty when lo == hi
  };
  std::vector<Piece> ps;
  for (const int b : blocks) {
    const int b0 = p.block_ptr[b], b1 = p.block_ptr[b + 1];
    if (p.offd_ptr[b1] > p.offd_ptr[b0]) ps.push_back({0, b0, b1, 0, 0});
    std::vector<std::pair<int, int>> cut;  // column pieces
    for (int a = b0; a < b1;) {
      int e = a + 1;
      while (e < b1 && p.col_ptr[e + 1] - p.col_ptr[a] <= gk::kSolveChunk) ++e;
      cut.push_back({a, e});
      a = e;
    }
    for (auto& c : cut) {
      const int lo = p.col_ptr[c.first], hi = p.col_ptr[c.second];
      const bool direct = hi - lo > gk::kSolveChunk;
      ps.push_back({1 | (direct ? 4 : 0), c.first, c.second, direct ? 0 : lo, direct ? 0 : hi});
    }
    for (auto it = cut.rbegin(); it != cut.rend(); ++it) {
      const int lo = p.col_ptr[it->first], hi = p.col_ptr[it->second];
      const bool direct = hi - lo > gk::kSolveChunk;
      ps.push_back({2 | (direct ? 4 : 0), it->first, it->second, direct ? 0 : lo,
                    direct ? 0 : hi});
    }
  }
  int lo = 0, hi = 0, o0 = (int)(op.size() / 3);
  auto close = [&]() {
    const int o1 = (int)(op.size() / 3);
    if (o1 > o0) chunk.insert(chunk.end(), {lo, hi, o0, o1});
    o0 = o1;
    lo = hi = 0;
  };
  for (const Piece& q : ps) {
    if (q.lo < q.hi) {
      const bool empty = lo == hi;
      const int nlo = empty ? q.lo : std::min(lo, q.lo), nhi = empty ? q.hi : std::max(hi, q.hi);
      const bool joins = empty || (q.lo <= hi && q.hi >= lo);
      if (!joins || nhi - nlo > gk::kSolveChunk) {
        close();
        lo = q.lo;
        hi = q.hi;
      } else {
        lo = nlo;
        hi = nhi;
      }
    } else if (q.code & 4) {
      close();  // a direct piece runs alone, with nothing loaded
    }
    op.insert(op.end(), {q.code, q.a, q.b});
    if (q.code & 4) close();
  }
  close();
}

void make_cta_solve(const gk::Plan& p, std::vector<i32>& chunk, std::vector<i32>& op) {
  chunk.clear();
  op.clear();
  std::vector<int> blocks(p.nblocks);
  for (int bb = 0; bb < p.nblocks; ++bb) blocks[bb] = p.offd_lower ? bb : p.nblocks - 1 - bb;
  cta_solve_blocks(p, blocks, chunk, op);
}

// The one-block solve split over thread blocks, for plans of several BTF
// blocks without coupling (each BTF block's solve is then independent):
// consecutive BTF blocks are grouped up to max(largest block, n / SMs) rows,
// and group g gets grp[4g..4g+3] = first row, end row, first chunk, end
// chunk. Returns the largest group's rows, or 0 when the plan does not
// qualify.
int make_cta_groups(const gk::Plan& p, int sms, std::vector<i32>& grp, std::vector<i32>& chunk,
                    std::vector<i32>& op) {
  grp.clear();
  chunk.clear();
  op.clear();
  if (p.nblocks < 2 || (!p.offd_ptr.empty() && p.offd_ptr.back() > 0)) return 0;
  int maxb = 0;
  for (int b = 0; b < p.nblocks; ++b) maxb = std::max(maxb, p.block_ptr[b + 1] - p.block_ptr[b]);
  const int target = std::max(maxb, (p.n + sms - 1) / std::max(sms, 1));
  int rows = 0;
  for (int b = 0; b < p.nblocks;) {
    int e = b + 1;
    while (e < p.nblocks && p.block_ptr[e + 1] - p.block_ptr[b] <= target) ++e;
    std::vector<int> blocks;
    for (int k = b; k < e; ++k) blocks.push_back(k);
    const int c0 = (int)(chunk.size() / 4);
    cta_solve_blocks(p, blocks, chunk, op);
    grp.insert(grp.end(), {p.block_ptr[b], p.block_ptr[e], c0, (int)(chunk.size() / 4)});
    rows = std::max(rows, p.block_ptr[e] - p.block_ptr[b]);
    b = e;
  }
  return rows;
}

// The solve as a step program (k_solve_steps): every operation the column
// sweeps perform, in their order - per BTF block in solve order the
// coupling terms of its rows, the forward sweep (L columns ascending), the
// backward sweep (per column descending: the pivot division, then its U
// entries) - as (destination row, source row, value index, kind), each
// placed in the first step after the last step that writes its source or
// its destination and after the last step that reads its destination. Every
// row then sees its updates in the sweeps' order, so the results are the
// sweeps' bit for bit. Plans whose solution vector does not fit one block's
// shared memory get none.
void make_solve_steps(const gk::Plan& p, std::vector<int4>& out_ops, std::vector<i32>& out_ptr) {
  out_ops.clear();
  out_ptr.clear();
  if (p.n == 0 || (size_t)8 * p.n + 16 > (size_t)(227 * 1024)) return;
  std::vector<int4> ops;
  for (int bb = 0; bb < p.nblocks; ++bb) {
    const int b = p.offd_lower ? bb : p.nblocks - 1 - bb;
    const int b0 = p.block_ptr[b], b1 = p.block_ptr[b + 1];
    for (int i = b0; i < b1; ++i)
      for (int e = p.offd_ptr[i]; e < p.offd_ptr[i + 1]; ++e)
        ops.push_back(make_int4(i, p.offd_col[e], p.offd_raw[e], 2));
    for (int j = b0; j < b1; ++j)
      for (int q = p.dslot[j] + 1; q < p.col_ptr[j + 1]; ++q)
        ops.push_back(make_int4(p.slot_row[q], j, q, 0));
    for (int j = b1 - 1; j >= b0; --j) {
      ops.push_back(make_int4(j, -1, p.dslot[j], 1));
      for (int q = p.col_ptr[j]; q < p.dslot[j]; ++q)
        ops.push_back(make_int4(p.slot_row[q], j, q, 0));
    }
  }
  std::vector<int> lw(p.n, 0), lr(p.n, 0), step(ops.size());
  int nsteps = 0;
  for (size_t q = 0; q < ops.size(); ++q) {
    const int4 o = ops[q];
    int st = std::max(lw[o.x], lr[o.x]) + 1;
    if (o.y >= 0) st = std::max(st, lw[o.y] + 1);
    step[q] = st;
    lw[o.x] = st;
    if (o.y >= 0) lr[o.y] = std::max(lr[o.y], st);
    nsteps = std::max(nsteps, st);
  }
  std::vector<i32> cnt(nsteps + 2, 0);
  for (int st : step) ++cnt[st];
  out_ptr.assign(nsteps + 1, 0);
  for (int t = 0; t < nsteps; ++t) out_ptr[t + 1] = out_ptr[t] + cnt[t + 1];
  std::vector<i32> pos(out_ptr.begin(), out_ptr.end() - 1);
  out_ops.assign(ops.size(), make_int4(0, 0, 0, 0));
  for (size_t q = 0; q < ops.size(); ++q) out_ops[pos[step[q] - 1]++] = ops[q];
}

// Device copy of a Plan.
struct PlanDev {
  DBuf<i32> col_ptr, dslot, slot_row, upd_ptr, upd_dst, col_single, amap_ptr, amap_idx,
      offd_ptr, offd_col, offd_raw, offdT_ptr, offdT_row, offdT_raw, lrow_ptr, lrow_col,
      lrow_slot, urow_ptr, urow_col,
      urow_slot, in_row, out_col, pcol_ptr, pcol_raw, pcol_q, pos_block, block_ptr, task,
      ttask, cs_chunk, cs_op, cs_grp, cs_gchunk, cs_gop, ss_ptr;
  DBuf<int4> ss_ops;
  gk::DPlan dp{}, dpt{};
  int64_t updates = 0;  // multiply-subtract pairs of one refactorization

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
    UP(offd_raw, p.offd_raw) UP(offdT_ptr, p.offdT_ptr) UP(offdT_row, p.offdT_row)
    UP(offdT_raw, p.offdT_raw) UP(lrow_ptr, p.lrow_ptr) UP(lrow_col, p.lrow_col)
    UP(lrow_slot, p.lrow_slot) UP(urow_ptr, p.urow_ptr) UP(urow_col, p.urow_col)
    UP(urow_slot, p.urow_slot) UP(in_row, h_in_row) UP(out_col, h_out_col)
    UP(pcol_ptr, p.pcol_ptr) UP(pcol_raw, p.pcol_raw) UP(pcol_q, p.pcol_q)
    UP(pos_block, p.pos_block) UP(block_ptr, bp)
#undef UP
    std::vector<i32> t = make_tasks(p, false), tt = make_tasks(p, true);
    if (e == cudaSuccess) e = task.upload(t, s);
    if (e == cudaSuccess) e = ttask.upload(tt, s);
    std::vector<i32> hc, ho, hg, hgc, hgo;
    make_cta_solve(p, hc, ho);
    if (e == cudaSuccess) e = cs_chunk.upload(hc, s);
    if (e == cudaSuccess) e = cs_op.upload(ho, s);
    const int grp_rows = make_cta_groups(p, sm_count(), hg, hgc, hgo);
    if (e == cudaSuccess) e = cs_grp.upload(hg, s);
    if (e == cudaSuccess) e = cs_gchunk.upload(hgc, s);
    if (e == cudaSuccess) e = cs_gop.upload(hgo, s);
    std::vector<int4> sso;
    std::vector<i32> ssp;
    const char* ess = getenv("GPUKLU_SOLVE_STEPS");
    if (!(ess && ess[0] == '0')) make_solve_steps(p, sso, ssp);
    if (e == cudaSuccess) e = ss_ops.upload(sso, s);
    if (e == cudaSuccess) e = ss_ptr.upload(ssp, s);
    updates = (int64_t)p.upd_dst.size();
    gk::DPlan d{};
    d.ss_nsteps = ssp.empty() ? 0 : (int)ssp.size() - 1;
    d.ss_ops = ss_ops.p;
    d.ss_ptr = ss_ptr.p;
    d.n = p.n;
    d.noffd = p.offd_ptr.empty() ? 0 : p.offd_ptr.back();
    d.cs_nchunk = (int)(hc.size() / 4);
    d.cs_chunk = cs_chunk.p;
    d.cs_op = cs_op.p;
    d.cs_ngrp = (int)(hg.size() / 4);
    d.cs_grp_rows = grp_rows;
    d.cs_grp = cs_grp.p;
    d.cs_gchunk = cs_gchunk.p;
    d.cs_gop = cs_gop.p;
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
    d.offdT_ptr = offdT_ptr.p;
    d.offdT_row = offdT_row.p;
    d.offdT_raw = offdT_raw.p;
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
    d.spin_limit = gk::kSpinLimit;
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
  // Two plans, both resident on the device. sym_plan is what analyze()
  // builds from the pattern alone (orderings, pivot-free symbolic pattern);
  // the first factor runs on it and picks the pivots. plan is sym_plan with
  // those pivots applied; refactor and solves run on it. Both are functions
  // of (pattern, mode) and (pattern, mode, pivots) only, so they are kept
  // across reset(): a prepare(n) that changes n and comes back, as the
  // engine's DC entry does, costs a pattern compare, and a first factor that
  // picks the same pivots as last time costs a pivot compare. The first
  // factor itself always runs, as in the reference (its pivot pass checks
  // every column, even when it starts from the last pivots found).
  gk::Plan plan;
  PlanDev pd;
  gk::Plan sym_plan;
  PlanDev pd_sym;
  bool pd_sym_ok = false, piv_ok = false;
  std::vector<i32> piv_rperm;
  std::vector<i64> last_ap, last_ai;
  std::vector<i64> sym_ap, sym_ai;
  int sym_mode = -1;
  // Set by an owner that knows the matrix (the BBD solver's block-diagonal
  // part): diagonal blocks to use instead of the BTF, and no row exchanges in
  // the first factorization (the reference's SparseLU keeps the diagonal).
  std::vector<int> given_blocks;
  bool no_swap = false;
  // Which of the reference's sparse solvers this handle restates
  // (gpuklu_set_solver_kind); the SparseLU kinds never exchange rows.
  int kind = GPUKLU_KIND_NATIVEKLU;
  bool swap_off() const { return no_swap || kind != GPUKLU_KIND_NATIVEKLU; }
  // DenseSolver (GPUKLU_KIND_DENSE): the pattern on the device, the row-major
  // LU and its row order
  DBuf<int64_t> d_dap, d_dai;
  DBuf<double> d_dense;
  DBuf<int> d_dpiv;
  static constexpr int64_t kDenseMaxN = GPUKLU_DENSE_MAX_N;

  int dense_analyze(const int64_t* ap, int64_t ap_len, const int64_t* ai, int64_t ai_len) {
    if (ap_len != n + 1)  // build_dense (solver.rs:621-623)
      return fail(GPUKLU_ANALYZE_FAILED, "Column pointer length " + std::to_string(ap_len) +
                                             " != expected " + std::to_string(n + 1));
    if (n > kDenseMaxN)
      return fail(GPUKLU_INVALID_MATRIX, "dense solver: n = " + std::to_string(n) +
                                             " above GPUKLU_DENSE_MAX_N = " +
                                             std::to_string(kDenseMaxN));
    if (ap[n] != ai_len || ap[0] != 0)
      return fail(GPUKLU_INVALID_MATRIX, "ap[n] does not match the row index count");
    last_ap.assign(ap, ap + ap_len);
    last_ai.assign(ai, ai + ai_len);
    const size_t nn = (size_t)std::max<int64_t>(n, 1);
    cudaError_t e = d_dap.upload(last_ap, stream);
    if (e == cudaSuccess) e = d_dai.resize(std::max<int64_t>(ai_len, 1));
    if (e == cudaSuccess && ai_len > 0)
      e = cudaMemcpyAsync(d_dai.p, ai, ai_len * sizeof(int64_t), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = d_ax.resize(std::max<int64_t>(ai_len, 1));
    if (e == cudaSuccess) e = d_dense.resize(nn * nn);
    if (e == cudaSuccess) e = d_dpiv.resize(nn);
    for (auto* b : {&d_rhs, &d_out, &d_xnew, &d_newx})  // solve and Newton vectors
      if (e == cudaSuccess) e = b->resize(nn);
    if (e == cudaSuccess) e = d_status.resize(1);
    if (e == cudaSuccess) e = d_nstate.resize(1);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status.p, 0, sizeof(int), stream);
    if (e != cudaSuccess) return cuda_fail(e, "dense buffers");
    state = ANALYZED;
    return GPUKLU_OK;
  }
  cudaStream_t stream = nullptr;
  DBuf<double> d_ax, d_lu, d_z, d_x, d_out, d_rhs, d_work, d_rc, d_rhs_c, d_xnew, d_newx,
      d_scratch2;
  DBuf<unsigned> d_flags, d_zflag, d_xflag, d_counter;
  DBuf<int> d_rperm, d_rinv, d_status;
  DBuf<gk::NewtonState> d_nstate;
  unsigned epoch = 0, sepoch = 0;
  int64_t factor_count = 0, refactor_count = 0;
  bool cta_ref = false, cta_sol = false;  // one-block refactor / solve for this plan
  bool cta_grp = false;  // the one-block solve over groups of uncoupled BTF blocks
  bool steps_sol = false;  // the solve as a step program (k_solve_steps)
  DBuf<double> d_rec;      // its scratch: the pivots' reciprocals
  // Plans with up to this many multiply-subtract pairs refactor in one block.
  // FP64 issue on one SM (a warp instruction per 16 cycles) bounds that
  // kernel: the 32x32 diode mesh (273k pairs) already refactors faster over
  // the whole grid, despite the grid kernel's dependency hops through L2.
  static constexpr int64_t kOneBlockUpdates = 1 << 16;
  // The first factorization's pivot pass on the refactorization kernels:
  // buffers, the pass limit before the sequential kernel takes over, and the
  // passes the last first factorization ran (0: the sequential kernel).
  static constexpr int kMaxPivotPasses = 8;
  // Below this many rows the sequential pass costs about as much as one
  // refactorization plus its host round trip, so it runs directly.
  static constexpr int64_t kPivotPassMinN = 512;
  DBuf<int> d_cand, d_want, d_pamap_ptr, d_pamap_idx;
  int64_t pivot_passes = 0;
  // The candidate the last settled pass ended with (per column an L slot or
  // -1), kept with the analysis: the next first factorization of the same
  // pattern starts from it and, if the pivots did not change, settles in one
  // pass.
  std::vector<int> piv_cand;
  double rcond = 0.0;
  bool rcond_valid = false;
  std::string err;
  int grid_cols = 1;
  // Growth-triggered re-pivot (off: the reference's frozen pivots): after a
  // refactorization, a BTF block with a multiplier above 1 / kPivotTol is
  // factored afresh (see repivot_grown).
  bool repivot = false;
  int64_t repivot_count = 0;
  DBuf<int> d_grow;
  static constexpr double kPivotTol = 0.001;
  // Polls of a dependency flag before a waiting warp gives up
  // (gpuklu_set_spin_limit); applied to both resident plans.
  unsigned spin_limit = gk::kSpinLimit;
  // End the device Newton loop at the first non-finite iterate
  // (gpuklu_set_stop_on_nonfinite; off: the reference runs on to the cap).
  bool stop_nonfinite = false;

  void apply_spin_limit() {
    for (PlanDev* p : {&pd, &pd_sym}) p->dp.spin_limit = p->dpt.spin_limit = spin_limit;
  }

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
    factor_count = refactor_count = repivot_count = 0;
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
    apply_spin_limit();
    if (e == cudaSuccess) e = d_lu.resize(std::max(plan.nslots(), 1));
    if (e != cudaSuccess) return cuda_fail(e, "upload plan");
    // one-block refactor and solve for small factorizations (GPUKLU_ONE_BLOCK=0: off)
    const char* ob = getenv("GPUKLU_ONE_BLOCK");
    const bool allow = !(ob && ob[0] == '0');
    cta_ref = allow && pd.updates <= kOneBlockUpdates && gk::refactor_cta_fits(pd.dp);
    cta_sol = allow && gk::solve_cta_fits(pd.dp);
    // the step-program solve (one block) when the plan has one
    // (GPUKLU_SOLVE_STEPS=0: no step programs)
    steps_sol = allow && gk::solve_steps_fits(pd.dp);
    if (steps_sol && e == cudaSuccess) e = d_rec.resize(std::max<int64_t>(n, 1));
    if (e != cudaSuccess) return cuda_fail(e, "solve scratch");
    // the solve split over groups of uncoupled BTF blocks when one block does
    // not hold the plan (GPUKLU_SOLVE_GROUPS=1: whenever the plan has groups)
    const char* eg = getenv("GPUKLU_SOLVE_GROUPS");
    const bool prefer_grp = eg && eg[0] == '1';
    cta_grp = allow && (prefer_grp || !cta_sol) && gk::solve_groups_fit(pd.dp);
    return GPUKLU_OK;
  }

  const gk::Plan& cur_plan() const { return state == FACTORED ? plan : sym_plan; }

  int do_analyze(const int64_t* ap, int64_t ap_len, const int64_t* ai, int64_t ai_len) {
    if (kind == GPUKLU_KIND_DENSE) return dense_analyze(ap, ap_len, ai, ai_len);
    if (ap_len != n + 1)
      return fail(GPUKLU_INVALID_MATRIX, "Column pointer length " + std::to_string(ap_len) +
                                             " != expected " + std::to_string(n + 1));
    if (ap[n] != ai_len || ap[0] != 0)
      return fail(GPUKLU_INVALID_MATRIX, "ap[n] does not match the row index count");
    const int key = pivot_mode + 4 * kind;
    if (!(sym_mode == key && sym_plan.n == n && (int64_t)sym_ap.size() == ap_len &&
          (int64_t)sym_ai.size() == ai_len && std::equal(sym_ap.begin(), sym_ap.end(), ap) &&
          std::equal(sym_ai.begin(), sym_ai.end(), ai))) {
      pd_sym_ok = piv_ok = false;
      piv_cand.clear();
      sym_mode = -1;
      std::string m = gk::analyze((int)n, ap, ai, pivot_mode, sym_plan,
                                  given_blocks.empty() ? nullptr : &given_blocks, kind);
      if (!m.empty()) return fail(GPUKLU_INVALID_MATRIX, m);
      sym_ap.assign(ap, ap + ap_len);
      sym_ai.assign(ai, ai + ai_len);
      sym_mode = key;
    }
    last_ap.assign(ap, ap + ap_len);
    last_ai.assign(ai, ai + ai_len);
    cudaError_t e = cudaSuccess;
    if (!pd_sym_ok) {
      e = pd_sym.upload(sym_plan, stream);
      apply_spin_limit();
      if (e != cudaSuccess) return cuda_fail(e, "upload plan");
      pd_sym_ok = true;
    }
    e = d_lu.resize(std::max(sym_plan.nslots(), 1));
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
  void refactor_launch() {
    if (cta_ref) {
      gk::launch_refactor_cta(pd.dp, d_ax.p, d_lu.p, d_status.p, stream);
      return;
    }
    unsigned ep = next_epoch(epoch, d_flags);
    gk::launch_refactor(pd.dp, d_ax.p, d_lu.p, d_flags.p, ep, d_counter.p, d_status.p,
                        grid_cols, stream);
  }

  // The first factorization's pivot pass run as refactorizations of the
  // pivot-free pattern (PivotCheck). Each pass refactors with a candidate
  // pivot sequence - at first the last one found for this pattern, else
  // none; any start ends at the same pivots - and reads back every column's own
  // choice; from the first column that disagrees on, the choices become the
  // next candidate. The columns before that one are final (a column's values
  // depend only on earlier columns), so each pass settles at least one more
  // column, and a pass that agrees everywhere has computed exactly what the
  // sequential pass computes: its pivots, and its factor in d_lu. settled
  // stays false when kMaxPivotPasses were not enough.
  int pivot_pass(std::vector<i32>& rperm, bool& settled) {
    settled = false;
    const gk::Plan& P = sym_plan;
    const int nn = P.n;
    if (nn == 0) {
      rperm.clear();
      settled = true;
      return GPUKLU_OK;
    }
    std::vector<int> cand(nn, -1), cand_row(nn, -1), want(nn, -1);
    if ((int)piv_cand.size() == nn) cand = piv_cand;
    for (int k = 0; k < nn; ++k) {
      if (!(cand[k] > P.dslot[k] && cand[k] < P.col_ptr[k + 1])) cand[k] = -1;
      cand_row[k] = cand[k] >= 0 ? P.slot_row[cand[k]] : -1;
    }
    std::vector<i32> aptr, aidx;
    cudaError_t e = d_cand.resize(nn);
    if (e == cudaSuccess) e = d_want.resize(nn);
    if (e != cudaSuccess) return cuda_fail(e, "pivot pass buffers");
    const char* ob = getenv("GPUKLU_ONE_BLOCK");
    const bool one_block = !(ob && ob[0] == '0') && pd_sym.updates <= kOneBlockUpdates &&
                           gk::refactor_cta_fits(pd_sym.dp);
    gk::PivotCheck pc;
    pc.cand = d_cand.p;
    pc.want = d_want.p;
    pc.tol = swap_off() ? 0.0 : 0.001;
    for (int pass = 0; pass < kMaxPivotPasses; ++pass) {
      gk::pivot_pass_amap(P, cand_row, aptr, aidx, rperm);
      e = d_pamap_ptr.upload(aptr, stream);
      if (e == cudaSuccess) e = d_pamap_idx.upload(aidx, stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_cand.p, cand.data(), nn * sizeof(int), cudaMemcpyHostToDevice,
                            stream);
      if (e != cudaSuccess) return cuda_fail(e, "pivot pass upload");
      gk::DPlan dp = pd_sym.dp;
      dp.amap_ptr = d_pamap_ptr.p;
      dp.amap_idx = d_pamap_idx.p;
      if (one_block) {
        gk::launch_refactor_cta(dp, d_ax.p, d_lu.p, d_status.p, stream, pc);
      } else {
        unsigned ep = next_epoch(epoch, d_flags);
        gk::launch_refactor(dp, d_ax.p, d_lu.p, d_flags.p, ep, d_counter.p, d_status.p,
                            grid_cols, stream, pc);
      }
      e = cudaMemcpyAsync(want.data(), d_want.p, nn * sizeof(int), cudaMemcpyDeviceToHost,
                          stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
      if (e != cudaSuccess) return cuda_fail(e, "pivot pass");
      const int st = check_status("pivot pass");
      if (st) return st;
      ++pivot_passes;
      int k1 = 0;
      while (k1 < nn && want[k1] == cand[k1]) ++k1;
      if (k1 == nn) {
        settled = true;
        piv_cand.swap(cand);
        return GPUKLU_OK;
      }
      for (int k = k1; k < nn; ++k) {
        const int w = want[k];
        const bool ok = w > P.dslot[k] && w < P.col_ptr[k + 1];  // an L slot of column k
        cand[k] = ok ? w : -1;
        cand_row[k] = ok ? P.slot_row[w] : -1;
      }
    }
    return GPUKLU_OK;
  }

  // The pivots of the reference's first factorization for the values in
  // d_ax (block-local row order per position): the pivot pass as
  // refactorizations from kPivotPassMinN rows on, else (or when those do not
  // settle) the sequential one-warp kernel. GPUKLU_PIVOT_PASS=refactor /
  // sequential picks one for every size. d_lu is left with the pass's
  // values in the pivot-free pattern.
  int first_pivots(std::vector<i32>& rperm) {
    rperm.assign(n, 0);
    bool settled = false;
    pivot_passes = 0;
    const char* pp = getenv("GPUKLU_PIVOT_PASS");
    const bool seq = pp && std::strcmp(pp, "sequential") == 0;
    const bool ref = pp && std::strcmp(pp, "refactor") == 0;
    if (!seq && (ref || n >= kPivotPassMinN)) {
      const int st = pivot_pass(rperm, settled);
      if (st) return st;
    }
    if (!settled) {
      pivot_passes = 0;
      rperm.assign(n, 0);
      int maxblk = 0;
      for (int b = 0; b < sym_plan.nblocks; ++b)
        maxblk = std::max(maxblk, sym_plan.block_ptr[b + 1] - sym_plan.block_ptr[b]);
      gk::launch_first_factor(pd_sym.dp, maxblk, d_ax.p, d_lu.p, d_work.p, d_rperm.p,
                              d_rinv.p, swap_off() ? 0.0 : kPivotTol, d_status.p, stream);
      cudaError_t e = cudaMemcpyAsync(rperm.data(), d_rperm.p, n * sizeof(i32),
                                      cudaMemcpyDeviceToHost, stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
      if (e != cudaSuccess) return cuda_fail(e, "first factor");
    }
    return check_status("first factor");
  }

  // After a refactorization with the kept pivots: blocks whose multipliers
  // grew past 1 / kPivotTol get the first factorization's pivots for the
  // current values. In the exact-pattern mode only those blocks change (the
  // pass's choice for a block depends on that block's values alone, so the
  // other blocks keep theirs) and the new plan refactors; in the reference's
  // mode every block is factored afresh, as after reset_pattern.
  int repivot_grown() {
    const gk::Plan& P = plan;
    cudaError_t e = d_grow.resize(std::max(P.nblocks, 1));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_grow.p, 0, P.nblocks * sizeof(int), stream);
    if (e != cudaSuccess) return cuda_fail(e, "growth check");
    gk::launch_growth(pd.dp, d_lu.p, 1.0 / kPivotTol, d_grow.p, stream);
    std::vector<int> grow(P.nblocks, 0);
    e = cudaMemcpyAsync(grow.data(), d_grow.p, P.nblocks * sizeof(int), cudaMemcpyDeviceToHost,
                        stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "growth check");
    if (std::none_of(grow.begin(), grow.end(), [](int g) { return g != 0; })) return GPUKLU_OK;
    ++repivot_count;
    if (pivot_mode != GPUKLU_PIVOT_EXACT) {  // every block afresh
      const int64_t fc = factor_count;
      state = ANALYZED;
      const int st = factor_on_device(true);
      factor_count = fc;
      return st;
    }
    std::vector<i32> fresh;
    int st = first_pivots(fresh);
    if (st) return st;
    std::vector<i32> merged = piv_rperm;
    for (int k = 0; k < (int)n; ++k)
      if (grow[P.pos_block[k]]) merged[k] = fresh[k];
    if (merged != piv_rperm) {
      plan = sym_plan;
      gk::set_pivots(plan, last_ap.data(), last_ai.data(), merged);
      if (plan.too_large) {
        state = ANALYZED;
        return fail(GPUKLU_INVALID_MATRIX,
                    "the factorization's update lists exceed 2^31 entries "
                    "(fill too large for this solver)");
      }
      st = upload_plan();
      if (st) return st;
      piv_rperm.swap(merged);
    }
    refactor_launch();
    return GPUKLU_OK;
  }

  int factor_on_device(bool sync) {
    rcond_valid = false;
    if (kind == GPUKLU_KIND_DENSE) {  // every factorization is a full one
      gk::launch_dense_factor((int)n, d_dap.p, d_dai.p, d_ax.p, d_dense.p, d_dpiv.p, d_status.p,
                              stream);
      ++factor_count;
      state = FACTORED;
      const int st = check_status("dense factor");
      if (st) state = ANALYZED;
      return st;
    }
    if (state == FACTORED) {
      refactor_launch();
      ++refactor_count;
      if (repivot && !swap_off()) {
        const int st = repivot_grown();
        if (st) return st;
      }
      if (!sync) return GPUKLU_OK;
      return check_status("refactor");
    }
    // First factorization: the reference's pivot choice, then the plan for
    // those pivots.
    std::vector<i32> rperm;
    int st = first_pivots(rperm);
    if (st) return st;
    if (!(piv_ok && rperm == piv_rperm)) {
      piv_ok = false;
      plan = sym_plan;
      gk::set_pivots(plan, last_ap.data(), last_ai.data(), rperm);
      if (plan.too_large) {
        state = ANALYZED;
        return fail(GPUKLU_INVALID_MATRIX,
                    "the factorization's update lists exceed 2^31 entries "
                    "(fill too large for this solver)");
      }
      st = upload_plan();
      if (st) return st;
      piv_rperm.swap(rperm);
      piv_ok = true;
    }
    if (pivot_mode == GPUKLU_PIVOT_EXACT) refactor_launch();  // the exact pattern
    ++factor_count;
    state = FACTORED;
    return check_status("factor");
  }

  // Solve with rhs in d_rhs; result in d_out (original column order).
  int solve_on_device(bool transpose, bool sync) {
    if (kind == GPUKLU_KIND_DENSE) {
      if (transpose) return fail(GPUKLU_SOLVE_FAILED, "dense solver: no transpose solve");
      gk::launch_dense_solve((int)n, d_dense.p, d_dpiv.p, d_rhs.p, d_out.p, d_status.p, stream);
      if (!sync) return GPUKLU_OK;
      return check_status("dense solve");
    }
    if (steps_sol && !transpose) {
      gk::launch_solve_steps(pd.dp, d_rhs.p, d_ax.p, d_lu.p, d_rec.p, d_out.p, stream);
      if (!sync) return GPUKLU_OK;
      return check_status("solve");
    }
    if ((cta_sol || cta_grp) && !transpose) {
      if (cta_grp)
        gk::launch_solve_groups(pd.dp, d_rhs.p, d_ax.p, d_lu.p, d_out.p, stream);
      else
        gk::launch_solve_cta(pd.dp, d_rhs.p, d_ax.p, d_lu.p, d_out.p, stream);
      if (!sync) return GPUKLU_OK;
      return check_status("solve");
    }
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
  // DenseSolver::analyze accepts any pattern (solver.rs:680-682); its factor
  // reports a bad one
  if (h->kind == GPUKLU_KIND_DENSE && ap_len != h->n + 1) return GPUKLU_OK;
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
  if (len != h->n)  // DenseSolver::solve reports SolveFailed (solver.rs:689-691)
    return h->fail(h->kind == GPUKLU_KIND_DENSE ? GPUKLU_SOLVE_FAILED : GPUKLU_INVALID_MATRIX,
                   "RHS length " + std::to_string(len) + " != matrix dimension " +
                       std::to_string(h->n));
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

const char* gpuklu_name(const gpuklu_handle* h) {
  if (h && h->kind == GPUKLU_KIND_SPARSELU) return "GpuSparseLU";
  if (h && h->kind == GPUKLU_KIND_SPARSELU_BTF) return "GpuSparseLU-BTF";
  if (h && h->kind == GPUKLU_KIND_DENSE) return "GpuDense";
  return "GpuKLU";
}

void gpuklu_set_parallel_threads(gpuklu_handle*, size_t) {}

int gpuklu_set_repivot(gpuklu_handle* h, int on) {
  if (!h) return GPUKLU_INVALID_MATRIX;
  h->repivot = on != 0;
  return GPUKLU_OK;
}

int64_t gpuklu_repivot_count(const gpuklu_handle* h) { return h ? h->repivot_count : 0; }

int gpuklu_set_stop_on_nonfinite(gpuklu_handle* h, int on) {
  if (!h) return GPUKLU_INVALID_MATRIX;
  h->stop_nonfinite = on != 0;
  return GPUKLU_OK;
}

int gpuklu_set_spin_limit(gpuklu_handle* h, uint32_t polls) {
  if (!h) return GPUKLU_INVALID_MATRIX;
  h->spin_limit = polls == 0 ? gk::kSpinLimit : polls;
  h->apply_spin_limit();
  return GPUKLU_OK;
}

int gpuklu_set_solver_kind(gpuklu_handle* h, int kind) {
  if (!h || kind < GPUKLU_KIND_NATIVEKLU || kind > GPUKLU_KIND_DENSE)
    return GPUKLU_INVALID_MATRIX;
  if (kind != h->kind) {
    h->kind = kind;
    h->reset();
  }
  return GPUKLU_OK;
}

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
  if (h->state == gpuklu_handle::FACTORED && !h->rcond_valid &&
      h->kind != GPUKLU_KIND_DENSE) {
    gk::launch_rcond(h->pd.dp, h->d_lu.p, h->d_rc.p, h->stream);
    double mm[2];
    cudaMemcpyAsync(mm, h->d_rc.p, sizeof(mm), cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    h->rcond = mm[1] > 0.0 ? mm[0] / mm[1] : 0.0;
    h->rcond_valid = true;
  }
  out->factor_count = h->factor_count;
  out->refactor_count = h->refactor_count;
  const gk::Plan& P = h->cur_plan();
  out->nnz_l = P.nnz_l;
  out->nnz_u = P.nnz_u;
  out->nblocks = P.nblocks;
  out->noffdiag = P.noffdiag;
  out->pivot_swaps = P.swaps;
  out->refactor_flops = P.flops_refactor;
  out->rcond = h->state == gpuklu_handle::FACTORED ? h->rcond : 0.0;
  return GPUKLU_OK;
}

int64_t gpuklu_pivot_pass_count(const gpuklu_handle* h) { return h ? h->pivot_passes : 0; }

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

int gpuklu_ac_sweep(gpuklu_handle* h, gpuklu_circuit* c, const double* x_dc, int64_t xlen,
                    const double* freqs, int64_t nf, double* out_re, double* out_im,
                    int64_t* n_out) {
  if (!h || !c || !x_dc || !freqs || !out_re || !out_im || nf < 0) return GPUKLU_INVALID_MATRIX;
  const int n = c->n, nc = c->node_count;
  if (n_out) *n_out = n;
  if (n > GPUKLU_AC_MAX_N)
    return h->fail(GPUKLU_INVALID_MATRIX, "gpuklu_ac_sweep: n = " + std::to_string(n) +
                                              " exceeds GPUKLU_AC_MAX_N = " +
                                              std::to_string(GPUKLU_AC_MAX_N));
  if (nf == 0) return GPUKLU_OK;
  // Cells of Y(w): the DC stamp's raw entries off the ground row in CSC order
  // (duplicates add in that order), then the capacitor terms in insertion
  // order (stamp.rs:1545-1564); row 0 becomes the identity row.
  std::vector<int> cell_of((size_t)n * n, -1), crow, ccol;
  std::vector<std::vector<int>> re_l, im_l;
  auto cell = [&](int r, int col) {
    int& id = cell_of[(size_t)r * n + col];
    if (id < 0) {
      id = (int)crow.size();
      crow.push_back(r);
      ccol.push_back(col);
      re_l.emplace_back();
      im_l.emplace_back();
    }
    return id;
  };
  for (int col = 0; col < n; ++col)
    for (i64 t = c->ap[col]; t < c->ap[col + 1]; ++t)
      if (c->ai[t] != 0) re_l[cell((int)c->ai[t], col)].push_back((int)t);
  std::vector<double> cap(std::max(c->ndev, 1), 0.0);
  std::vector<double> rhs(2 * (size_t)n, 0.0);
  int aux = nc;
  for (int d = 0; d < c->ndev; ++d) {
    const int a = c->nodes[4 * d], b = c->nodes[4 * d + 1];
    const double* p = &c->p[6 * (size_t)d];
    if (c->type[d] == 5) {  // capacitor
      cap[d] = p[0];
      const int rr[4] = {a, b, a, b}, cc[4] = {a, b, b, a}, ng[4] = {0, 0, 1, 1};
      for (int q = 0; q < 4; ++q)
        if (rr[q] != 0) im_l[cell(rr[q], cc[q])].push_back((d << 1) | ng[q]);
    } else if (c->type[d] == 1 || c->type[d] == 2) {  // V (its aux row) or I: the AC phasor
      const double t = p[2] * 3.141592653589793 / 180.0;
      const double pre = p[1] * std::cos(t), pim = p[1] * std::sin(t);
      auto add = [&](int i, double re, double im) {
        if (i >= 0 && i < n) {
          rhs[2 * i] = rhs[2 * i] + re;
          rhs[2 * i + 1] = rhs[2 * i + 1] + im;
        }
      };
      if (c->type[d] == 1) {
        add(aux++, pre, pim);
      } else {
        add(a, -pre, -pim);
        add(b, pre, pim);
      }
    }
  }
  const int ncell = (int)crow.size();
  std::vector<i32> re_ptr(1, 0), re_idx, im_ptr(1, 0), im_code;
  for (int q = 0; q < ncell; ++q) {
    re_idx.insert(re_idx.end(), re_l[q].begin(), re_l[q].end());
    re_ptr.push_back((i32)re_idx.size());
    im_code.insert(im_code.end(), im_l[q].begin(), im_l[q].end());
    im_ptr.push_back((i32)im_code.size());
  }
  cudaStream_t s = h->stream;
  DBuf<i32> d_crow, d_ccol, d_re_ptr, d_re_idx, d_im_ptr, d_im_code, d_status;
  DBuf<double> d_cap, d_rhs, d_freqs, d_re, d_im, dx, dax, drc, drhs;
  cudaError_t e = cudaSuccess;
#define UP(buf, vec) \
  if (e == cudaSuccess) e = buf.upload(vec, s);
  std::vector<i32> vrow(crow.begin(), crow.end()), vcol(ccol.begin(), ccol.end());
  std::vector<double> vfreq(freqs, freqs + nf), vx(x_dc, x_dc + std::max<int64_t>(xlen, 0));
  UP(d_crow, vrow) UP(d_ccol, vcol) UP(d_re_ptr, re_ptr) UP(d_re_idx, re_idx) UP(d_im_ptr, im_ptr)
  UP(d_im_code, im_code) UP(d_cap, cap) UP(d_rhs, rhs) UP(d_freqs, vfreq)
#undef UP
  if (e == cudaSuccess) e = d_re.resize((size_t)nf * n);
  if (e == cudaSuccess) e = d_im.resize((size_t)nf * n);
  if (e == cudaSuccess) e = d_status.resize(1);
  if (e == cudaSuccess) e = dx.resize(std::max<int64_t>(xlen, 1));
  if (e == cudaSuccess) e = dax.resize(std::max<size_t>(c->ai.size(), 1));
  if (e == cudaSuccess) e = drc.resize(std::max(c->ncontrib, 1));
  if (e == cudaSuccess) e = drhs.resize(n);
  if (e == cudaSuccess && xlen > 0)
    e = cudaMemcpyAsync(dx.p, vx.data(), xlen * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status.p, 0, sizeof(int), s);
  if (e != cudaSuccess) return h->cuda_fail(e, "ac upload");
  // G: the DC stamp at the operating point (the AC stamps of R, V, D and M
  // are the DC stamp's matrix entries there, stamp.rs:1525-1747)
  gk::launch_stamp(c->dc, dx.p, (int)std::min<int64_t>(xlen, nc), 1e-12, 1.0, 0.0, nullptr, -1.0,
                   dax.p, drc.p, drhs.p, s, 1e-12);
  gk::AcArgs a{};
  a.n = n;
  a.ncell = ncell;
  a.cell_row = d_crow.p;
  a.cell_col = d_ccol.p;
  a.re_ptr = d_re_ptr.p;
  a.re_idx = d_re_idx.p;
  a.im_ptr = d_im_ptr.p;
  a.im_code = d_im_code.p;
  a.cap = d_cap.p;
  a.ax = dax.p;
  a.rhs = d_rhs.p;
  a.freqs = d_freqs.p;
  a.out_re = d_re.p;
  a.out_im = d_im.p;
  a.status = d_status.p;
  DBuf<double> d_scratch;
  if (gk::ac_fits_shared(n)) {
    gk::launch_ac_dense(a, (int)nf, s);
  } else {
    // one n x n complex matrix per block in global memory, at most ~2 GB of
    // them (and no more blocks than frequencies or two per SM)
    const size_t per = (size_t)16 * n * n;
    int blocks = (int)std::min<int64_t>(nf, std::max<size_t>(1, ((size_t)2 << 30) / per));
    blocks = std::min(blocks, 2 * sm_count());
    e = d_scratch.resize(per / 8 * blocks);
    if (e != cudaSuccess) return h->cuda_fail(e, "ac scratch");
    a.scratch = d_scratch.p;
    gk::launch_ac_dense_global(a, (int)nf, blocks, s);
  }
  int st = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_re, d_re.p, (size_t)nf * n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_im, d_im.p, (size_t)nf * n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, d_status.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return h->cuda_fail(e, "ac sweep");
  if (st) return h->fail(GPUKLU_SINGULAR, "ac sweep: a pivot below 1e-30");
  return GPUKLU_OK;
}

}  // extern "C"

namespace {
// The Newton loop of the engine's DC analyses on the device
// (run_newton_with_stepping, newton.rs:142-185, with run_newton, :65-117):
// stamping, factor, solve and the update on the device, the pattern and
// pivots kept by the handle between calls. d_newx holds the starting
// iterate: x0 (nc values, the rest zero) when x0 is given, else whatever the
// previous call left there (the sweep's continuation). m: the iterate's
// length, node_count on a fresh start (x = zeros(node_count),
// engine.rs:252), n once a converged solution with its aux currents has
// become the iterate (run_newton's x = x_new, newton.rs:97-98): the
// convergence test and the damping run over the first m entries. On return
// *m_out is the length of x afterwards and x_out receives min(x_cap, that)
// values.
int dc_newton_run(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                  const double* x0, int m, double* x_out, int64_t x_cap, int64_t* x_len,
                  int64_t* iters, int64_t* iters_total, int* reason) {
  // build(x) returns n = node_count + aux; run_newton calls prepare(n)
  gpuklu_prepare(h, c->n);
  int st = gpuklu_analyze(h, c->ap.data(), (int64_t)c->ap.size(), c->ai.data(),
                          (int64_t)c->ai.size());
  if (st) return st;
  const int nc = c->node_count, n = c->n;
  cudaError_t e = h->d_rhs_c.resize(std::max(c->ncontrib, 1));
  if (e != cudaSuccess) return h->cuda_fail(e, "newton buffers");
  if (x0) {
    std::vector<double> xinit(n, 0.0);
    std::copy(x0, x0 + nc, xinit.begin());
    m = nc;
    e = cudaMemcpyAsync(h->d_newx.p, xinit.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                        h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "newton x0");
  }
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
  int rsn = 1, ret = GPUKLU_OK;
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
          if (st == GPUKLU_DEVICE_TIMEOUT) ret = st;
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        gk::launch_newton_update(m, n, h->d_newx.p, h->d_out.p, h->d_nstate.p, nc_,
                                 h->d_status.p, h->stream);
        gk::NewtonState hs;
        int dst = 0;
        e = cudaMemcpyAsync(&hs, h->d_nstate.p, sizeof(hs), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(&dst, h->d_status.p, sizeof(int), cudaMemcpyDeviceToHost,
                              h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "newton step");
        if (dst == GPUKLU_DEVICE_TIMEOUT) {
          cudaMemset(h->d_status.p, 0, sizeof(int));
          h->err = "device dependency wait timed out";
          ret = GPUKLU_DEVICE_TIMEOUT;
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        if (dst) cudaMemset(h->d_status.p, 0, sizeof(int));
        if (dst == GPUKLU_NONFINITE && h->stop_nonfinite) {
          h->err = "non-finite Newton iterate at iteration " + std::to_string(it + 1);
          ret = GPUKLU_NONFINITE;
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
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
  const int64_t len = conv ? n : m;
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
  return ret;
}
}  // namespace

extern "C" {

int gpuklu_newton_dc(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                     const double* x0, double* x_out, int64_t x_cap, int64_t* x_len,
                     int64_t* iters, int64_t* iters_total, int* reason) {
  if (!h || !c || !cfg) return GPUKLU_INVALID_MATRIX;
  // Engine::run_dc_result: x = zeros(node_count), solver.prepare(node_count)
  // (a size other than the matrix's when there are voltage sources, so the
  // pattern and the pivots are found anew)
  gpuklu_prepare(h, c->node_count);
  std::vector<double> zero;
  if (!x0) {
    zero.assign(c->node_count, 0.0);
    x0 = zero.data();
  }
  return dc_newton_run(h, c, cfg, x0, c->node_count, x_out, x_cap, x_len, iters, iters_total,
                       reason);
}

int gpuklu_dc_sweep(gpuklu_handle* h, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                    int64_t src_dev, const double* values, int64_t npts, const double* x0,
                    int64_t x0_stride, int stop_on_failure, double* x_out, int64_t x_stride,
                    int64_t* x_len, int64_t* iters, int64_t* iters_total, int* reason) {
  if (!h || !c || !cfg || !values || npts < 0) return GPUKLU_INVALID_MATRIX;
  if (src_dev < 0 || src_dev >= c->ndev)
    return h->fail(GPUKLU_INVALID_MATRIX, "gpuklu_dc_sweep: no device " +
                                              std::to_string(src_dev) + " to sweep");
  if (x0 && x0_stride < c->node_count)
    return h->fail(GPUKLU_INVALID_MATRIX, "gpuklu_dc_sweep: x0_stride below node_count");
  if (x_out && x_stride < c->n)
    return h->fail(GPUKLU_INVALID_MATRIX, "gpuklu_dc_sweep: x_stride below n");
  for (int64_t k = 0; k < npts; ++k) {  // points not run: reason -1
    if (iters) iters[k] = 0;
    if (iters_total) iters_total[k] = 0;
    if (reason) reason[k] = -1;
    if (x_len) x_len[k] = 0;
  }
  // engine.rs:746-748: x = zeros(node_count), prepare(node_count) once
  gpuklu_prepare(h, c->node_count);
  const std::vector<double> zero(c->node_count, 0.0);
  int m = c->node_count;
  std::vector<double> xbuf(c->n);
  for (int64_t k = 0; k < npts; ++k) {
    // the swept source's value (engine.rs:758) in the device parameters
    c->p[(size_t)src_dev * 6] = values[k];
    cudaError_t e = cudaMemcpyAsync(c->d_p.p + (size_t)src_dev * 6, &c->p[(size_t)src_dev * 6],
                                    sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "dc sweep source value");
    // the start: the point's own x0, or zeros at the first point of a
    // continuation sweep, else the previous point's final iterate
    const double* start = x0 ? x0 + k * x0_stride : (k == 0 ? zero.data() : nullptr);
    int64_t len = 0, it = 0, itt = 0;
    int rsn = 1;
    const int st = dc_newton_run(h, c, cfg, start, m, xbuf.data(), c->n, &len, &it, &itt, &rsn);
    // a wait that timed out or a non-finite stop still reports its point
    if (st != GPUKLU_OK && st != GPUKLU_DEVICE_TIMEOUT && st != GPUKLU_NONFINITE) return st;
    m = (int)len;
    if (x_out)
      for (int64_t i = 0; i < c->n; ++i) x_out[k * x_stride + i] = i < len ? xbuf[i] : 0.0;
    if (x_len) x_len[k] = len;
    if (iters) iters[k] = it;
    if (iters_total) iters_total[k] = itt;
    if (reason) reason[k] = rsn;
    if (st != GPUKLU_OK) return st;
    if (rsn != 0 && stop_on_failure) break;  // engine.rs:785-796
  }
  return GPUKLU_OK;
}

int gpuklu_dc_backward(gpuklu_handle* h, gpuklu_circuit* c, const double* x, int64_t xlen,
                       const double* dl_dx, double gmin, double* lambda_out,
                       double* grad_out) {
  if (!h || !c || !x || !dl_dx) return GPUKLU_INVALID_MATRIX;
  const int n = c->n;
  gpuklu_prepare(h, n);
  int st = gpuklu_analyze(h, c->ap.data(), (int64_t)c->ap.size(), c->ai.data(),
                          (int64_t)c->ai.size());
  if (st) return st;
  DBuf<double> dx, dgrad;
  cudaError_t e = dx.resize(std::max<int64_t>(xlen, 1));
  if (e == cudaSuccess) e = dgrad.resize(std::max(c->ndev, 1));
  if (e == cudaSuccess) e = h->d_rhs_c.resize(std::max(c->ncontrib, 1));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dx.p, x, xlen * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "backward upload");
  // A at the solution: stamp and factor (refactor when the pivots are known)
  // exact Jacobian: no level-1 conductance floor (it cancels in the residual)
  gk::launch_stamp(c->dc, dx.p, (int)std::min<int64_t>(xlen, c->node_count), gmin, 1.0, 0.0,
                   nullptr, -1.0, h->d_ax.p, h->d_rhs_c.p, h->d_rhs.p, h->stream, 0.0);
  st = h->factor_on_device(true);
  if (st) return st;
  e = cudaMemcpyAsync(h->d_rhs.p, dl_dx, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "backward upload");
  st = h->solve_on_device(true, false);
  if (st) return st;
  gk::launch_param_grad(c->dc, dx.p, (int)xlen, h->d_out.p, dgrad.p, h->stream);
  if (lambda_out)
    e = cudaMemcpyAsync(lambda_out, h->d_out.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream);
  if (e == cudaSuccess && grad_out)
    e = cudaMemcpyAsync(grad_out, dgrad.p, c->ndev * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "backward download");
  return h->check_status("dc_backward");
}

}  // extern "C"

// ====================================================================== batch
struct gpuklu_batch {
  int64_t ncirc = 0, ninst = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<gk::GroupHdr> groups;
  DBuf<gk::GroupHdr> d_groups;
  DBuf<i32> d_order, d_dev_type, d_dev_nodes, d_dev_dv, d_amap_ptr, d_amap_code,
      d_rmap_ptr, d_rmap_code, d_col_ptr, d_dslot, d_col_single, d_in_row, d_out_pos,
      d_offd_ptr, d_slot_row, d_upd_ptr, d_upd_dst, d_offd_col, d_block_ptr, d_heavy, d_ov_dev,
      d_lvl_col, d_lseg_ptr, d_lseg, d_amap4, d_rmap4, d_lng, d_ops, d_step_ptr,
      d_iters,
      d_iters_total, d_reason, d_status;
  DBuf<double> d_dparams, d_ov_val, d_x0, d_xout;
  DBuf<long long> d_p_off, d_x0_off, d_x_off;
  std::vector<long long> x_off;
  int64_t x0_len = 0, xout_len = 0;
  int64_t flops_per_iter = 0, bytes_per_iter = 0;
  std::vector<int64_t> group_flops, group_bytes;
  std::vector<i32> inst_group_h;
  DBuf<unsigned> d_gnext;
  // Launch classes: groups of similar per-instance shared memory run in one
  // launch with m instances per warp; classes run concurrently on their own
  // streams.
  struct Class {
    int m = 1, region = 0, prog_ints = 0, grid = 0, warps_per_block = 1, regs = 0,
        blocks_per_sm = 0;
    // continuation phase: warps of a block share one staged program
    int grid2 = 0, wpb2 = 1, shared_bytes = 0;
    bool shared2 = false;
    // after the lane phase (parked instances): tiles2 for blocks sharing a
    // program, tiles3 for one warp per tile
    std::vector<i32> tiles, tiles2, tiles3;
    DBuf<i32> d_tiles, d_tiles2, d_tiles3;
    std::vector<int> members;  // its groups, most expensive first
    DBuf<unsigned> d_counter;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    gk::BatchArgs args{};
  };
  std::vector<std::unique_ptr<Class>> classes;
  // warps of a block that shares one program: up to this many, as the
  // group's program and instance regions fit the block's shared memory
  static constexpr int kSharedWarpsMax = 16;
  // continuation tiles per group (gpuklu_batch_set_schedule / autotune)
  static constexpr int kContTilesDefault = 2;
  int cont_tiles = kContTilesDefault;

  cudaEvent_t start_ev = nullptr;
  // timing events of the last run: before the lane kernel, after it, after
  // the warp kernels joined back
  cudaEvent_t ph_ev[3] = {nullptr, nullptr, nullptr};
  gk::BatchArgs args{};
  // lane-per-instance phase (k_batch_lanes) in front of the warp classes
  bool lanes = false;
  int lane_cap = 0, lane_grid = 0, lane_wpb = 4;
  std::vector<i32> ltiles;
  DBuf<i32> d_ltiles, d_cont_list, d_cont_it, d_cont_total, d_cont_gstep;
  DBuf<unsigned> d_lcounter, d_cont_count, d_gnext2;
  DBuf<double> d_scratch, d_cont_damp, d_cont_prev;
  // continuation kernel: one warp per parked instance from a queue over the
  // groups (cont.cu); off: the warp classes continue them
  bool cont_kernel = false;
  int cont_grid = 0, cont_wpb = 0, cont_m = 1;
  DBuf<i32> d_cont_groups;
  DBuf<unsigned> d_cont_cursor;
  DBuf<double> d_dv;
  // transient
  int transient = 0;
  double dt = 0.0;
  int64_t steps = 0, ckpt_every = 0;
  int tran_region = 0, tran_prog = 0, tran_grid_f = 0, tran_grid_b = 0;
  std::vector<long long> grad_off_h;
  int64_t grad_len = 0;
  DBuf<i32> d_inst_group, d_probe;
  DBuf<double> d_loss, d_wave, d_ckpt, d_seg, d_grad;
  DBuf<long long> d_ckpt_off, d_seg_off, d_grad_off;
  DBuf<unsigned> d_tcounter;
  bool tran_fwd_done = false;
  // adaptive transient: per instance its time-dependent sources (records
  // at_wptr[i]..at_wptr[i+1]) and the run's per-instance outputs
  bool atran = false;
  int at_grid = 0;
  std::vector<i32> at_wptr, at_wdev, at_wkind, at_pwlptr;
  std::vector<double> at_wp, at_pwlt, at_pwlv;
  DBuf<i32> d_at_wptr, d_at_wdev, d_at_wkind, d_at_pwlptr, d_at_bpptr, d_at_out;
  DBuf<double> d_at_wp, d_at_pwlt, d_at_pwlv, d_at_bpt, d_at_times, d_at_probe;

  ~gpuklu_batch() {
    for (auto& c : classes) {
      if (c->stream) cudaStreamDestroy(c->stream);
      if (c->done) cudaEventDestroy(c->done);
    }
    if (start_ev) cudaEventDestroy(start_ev);
    for (auto& ev : ph_ev)
      if (ev) cudaEventDestroy(ev);
  }

  int fail(const std::string& m) {
    err = m;
    return GPUKLU_CUDA_ERROR;
  }
};

namespace {
// Program of one circuit as flat arrays; circuits with equal programs share
// a group (only their constants and inputs differ).
struct Program {
  gk::GroupHdr h{};
  std::vector<i32> dev_type, dev_nodes, dev_dv, amap_ptr, amap_code, rmap_ptr, rmap_code,
      col_ptr, dslot, col_single, in_row, out_pos, offd_ptr, slot_row, upd_ptr, upd_dst,
      offd_col, block_ptr, heavy, lvl_col, lseg_ptr, lseg, amap4, rmap4, lng;
  std::vector<i32> ops;       // step program: two ints per operation
  std::vector<i32> step_ptr;  // nsteps + 1 (empty: no step program)
  int64_t flops = 0, bytes = 0;
  std::string key() const {
    std::string k;
    auto app = [&k](const std::vector<i32>& v) {
      int32_t sz = (int32_t)v.size();
      k.append((const char*)&sz, 4);
      k.append((const char*)v.data(), v.size() * 4);
    };
    int32_t hdr[7] = {h.n, h.node_count, h.nslots, h.noffd, h.ndev, h.nblocks, h.ndv};
    k.append((const char*)hdr, sizeof(hdr));
    for (auto* v : {&dev_type, &dev_nodes, &dev_dv, &amap_ptr, &amap_code, &rmap_ptr,
                    &rmap_code, &col_ptr, &dslot, &col_single, &in_row, &out_pos, &offd_ptr,
                    &slot_row, &upd_ptr, &upd_dst, &offd_col, &block_ptr, &heavy, &lvl_col,
                    &lseg_ptr, &lseg, &amap4, &rmap4, &lng})
      app(*v);
    return k;
  }
};

int record_size(int type, bool transient) {
  switch (type) {
    case 3: return 2;
    case 4: return 3;
    case 6: return 4;
    case 5: return transient ? 2 : 0;
    default: return 1;
  }
}

// Contribution codes of every matrix insert and rhs add of one device, in
// the reference's insert order (see compile_circuit).
void device_codes(int type, int dv, bool transient, int m[8], int r[2]) {
  auto c = [dv](int k, int kind) { return ((dv + k) << 3) | kind; };
  for (int e = 0; e < 8; ++e) m[e] = -1;
  r[0] = r[1] = -1;
  switch (type) {
    case 0:
      m[0] = c(0, 0); m[1] = c(0, 0); m[2] = c(0, 1); m[3] = c(0, 1);
      break;
    case 1:
      m[0] = 2; m[1] = 3; m[2] = 2; m[3] = 3;
      r[0] = c(0, 0);
      break;
    case 2:
      r[0] = c(0, 1); r[1] = c(0, 0);
      break;
    case 3:
      m[0] = c(0, 0); m[1] = c(0, 0); m[2] = c(0, 1); m[3] = c(0, 1);
      r[0] = c(1, 1); r[1] = c(1, 0);
      break;
    case 4:
      m[0] = c(0, 0); m[1] = c(0, 0); m[2] = c(0, 1); m[3] = c(0, 1);
      m[4] = c(1, 0); m[5] = c(1, 1); m[6] = c(1, 1); m[7] = c(1, 0);
      r[0] = c(2, 1); r[1] = c(2, 0);
      break;
    case 6:
      m[0] = c(0, 0); m[1] = c(1, 1); m[2] = c(1, 0); m[3] = c(0, 1);
      m[4] = c(2, 0); m[5] = -1; m[6] = c(2, 1); m[7] = -1;  // the +0.0 inserts add nothing
      r[0] = c(3, 1); r[1] = c(3, 0);
      break;
    case 5:  // backward-Euler companion [g, ieq], physical sign: rhs a += ieq
      if (transient) {
        m[0] = c(0, 0); m[1] = c(0, 0); m[2] = c(0, 1); m[3] = c(0, 1);
        r[0] = c(1, 0); r[1] = c(1, 1);
      }
      break;
    default:
      break;
  }
}

// The step program of the batched factorization and substitutions (see
// bt::run_steps): every operation of the column-by-column path in its order
// - per BTF block the coupling into the block's rows, per column its U
// entries' updates, the pivot's reciprocal, the L scaling and the forward
// update of the right-hand side, then the backward sweep - as offsets into
// an instance's region (X[nc], T[n], ndv unused doubles, V; the batch
// kernels keep their device records after V, so ndv is 0 there). Two pairs
// of operations are fused, each into one operation with the same two
// roundings: an L entry's last update in its column with its scaling by the
// pivot's reciprocal (nothing reads the entry in between), and a row's last
// backward update with its multiplication by its pivot's reciprocal. Each
// operation goes to the first step after the last step that writes one of
// its operands or its destination and after the last step that reads its
// destination, so a step's operations are independent and each value sees
// its operations in the original order. Regions beyond 15-bit offsets get no
// step program.
void build_steps(const gk::Plan& P, int nc, int ndv, std::vector<i32>& out_ops,
                 std::vector<i32>& out_steps) {
  out_ops.clear();
  out_steps.clear();
  const int n = P.n, nslots = P.nslots();
  const long long vbase = (long long)nc + n + ndv;
  const long long top = vbase + nslots + (long long)P.offd_raw.size();
  if (top >= 32768 || n == 0) return;
  struct Op {
    int d, a, b, c, k;
  };
  std::vector<Op> ops;
  auto T_ = [nc](int i) { return nc + i; };
  auto V_ = [vbase](long long v) { return (int)(vbase + v); };
  std::vector<int> pend_a((size_t)nslots, -1), pend_b((size_t)nslots, -1);
  std::vector<long long> last_bw((size_t)n, -1);
  for (int b = 0; b < P.nblocks; ++b) {
    const int b0 = P.block_ptr[b], b1 = P.block_ptr[b + 1];
    for (int i = b0; i < b1; ++i)
      for (int e = P.offd_ptr[i]; e < P.offd_ptr[i + 1]; ++e)
        ops.push_back({T_(i), V_(nslots + e), T_(P.offd_col[e]), 0, 0});
    for (int k = b0; k < b1; ++k) {
      const int s0 = P.col_ptr[k], ds = P.dslot[k], s1 = P.col_ptr[k + 1];
      // the column's updates in order; the last one into each L entry waits
      // for the reciprocal and is fused with the scaling
      std::vector<std::pair<int, std::pair<int, int>>> upd;  // (dst slot, (a slot, u slot))
      for (int s = s0; s < ds; ++s) {
        const int j = P.slot_row[s];
        const int q0 = P.dslot[j] + 1, q1 = P.col_ptr[j + 1];
        for (int qq = q0; qq < q1; ++qq)
          upd.push_back({P.upd_dst[P.upd_ptr[s] - q0 + qq], {qq, s}});
      }
      std::vector<char> last(upd.size(), 0);
      for (size_t u = upd.size(); u-- > 0;) {
        const int dst = upd[u].first;
        if (dst > ds && dst < s1 && pend_a[dst] < 0) {
          pend_a[dst] = upd[u].second.first;
          pend_b[dst] = upd[u].second.second;
          last[u] = 1;
        }
      }
      for (size_t u = 0; u < upd.size(); ++u)
        if (!last[u]) ops.push_back({V_(upd[u].first), V_(upd[u].second.first),
                                     V_(upd[u].second.second), 0, 4});
      ops.push_back({V_(ds), P.col_single[k] ? 1 : 0, V_(ds), 0, 1});
      for (int qq = ds + 1; qq < s1; ++qq) {
        if (pend_a[qq] >= 0) {
          ops.push_back({V_(qq), V_(pend_a[qq]), V_(pend_b[qq]), V_(ds), 5});
          pend_a[qq] = pend_b[qq] = -1;
        } else {
          ops.push_back({V_(qq), V_(qq), V_(ds), 0, 2});
        }
      }
      for (int qq = ds + 1; qq < s1; ++qq)
        ops.push_back({T_(P.slot_row[qq]), V_(qq), T_(k), 0, 0});
    }
    for (int k = b1 - 1; k >= b0; --k) {
      const int s0 = P.col_ptr[k], ds = P.dslot[k];
      if (last_bw[k] >= 0) {  // x_k fused into T[k]'s last update
        ops[(size_t)last_bw[k]].c = V_(ds);
        ops[(size_t)last_bw[k]].k = 6;
      } else {
        ops.push_back({T_(k), T_(k), V_(ds), 0, 2});
      }
      for (int s = s0; s < ds; ++s) {
        last_bw[P.slot_row[s]] = (long long)ops.size();
        ops.push_back({T_(P.slot_row[s]), V_(s), T_(k), 0, 0});
      }
    }
  }
  std::vector<int> lw((size_t)top, 0), lr((size_t)top, 0), step(ops.size());
  int nsteps = 0;
  for (size_t q = 0; q < ops.size(); ++q) {
    const Op& o = ops[q];
    int st = std::max(lw[o.d], lr[o.d]) + 1;
    if (o.k != 1) st = std::max(st, std::max(lw[o.a], lw[o.b]) + 1);
    if (o.k >= 5) st = std::max(st, lw[o.c] + 1);
    step[q] = st;
    lw[o.d] = st;
    if (o.k != 1) {
      lr[o.a] = std::max(lr[o.a], st);
      lr[o.b] = std::max(lr[o.b], st);
    }
    if (o.k >= 5) lr[o.c] = std::max(lr[o.c], st);
    nsteps = std::max(nsteps, st);
  }
  std::vector<i32> cnt(nsteps + 2, 0);
  for (int st : step) ++cnt[st];
  out_steps.assign(nsteps + 1, 0);
  for (int t = 0; t < nsteps; ++t) out_steps[t + 1] = out_steps[t] + cnt[t + 1];
  std::vector<i32> pos(out_steps.begin(), out_steps.end() - 1);
  out_ops.assign(2 * ops.size(), 0);
  for (size_t q = 0; q < ops.size(); ++q) {  // program order within a step
    const Op& o = ops[q];
    const int at = pos[step[q] - 1]++;
    out_ops[2 * at] = (i32)((unsigned)o.d | ((unsigned)o.a << 15) | (((unsigned)o.k & 3u) << 30));
    out_ops[2 * at + 1] =
        (i32)((unsigned)o.b | ((unsigned)o.c << 15) | (((unsigned)o.k >> 2) << 30));
  }
}

Program make_program(const gpuklu_circuit& C, const gk::Plan& P) {
  Program g;
  gk::GroupHdr& h = g.h;
  h.n = P.n;
  h.node_count = C.node_count;
  h.nslots = P.nslots();
  h.noffd = (int)P.offd_raw.size();
  h.ndev = C.ndev;
  h.nblocks = P.nblocks;
  std::vector<int> raw_offd(C.ai.size(), -1);
  for (size_t e = 0; e < P.offd_raw.size(); ++e) raw_offd[P.offd_raw[e]] = (int)e;
  const int nv = h.nslots + h.noffd;
  std::vector<std::vector<i32>> vlist(nv), rlist(P.n);
  int ndv = 0;
  int64_t dev_flops = 0;
  for (int d = 0; d < C.ndev; ++d) {
    const int t = C.type[d];
    g.dev_type.push_back(t);
    for (int q = 0; q < 4; ++q) g.dev_nodes.push_back(C.nodes[(size_t)d * 4 + q]);
    g.dev_dv.push_back(ndv);
    int m[8], r[2];
    device_codes(t, ndv, C.transient != 0, m, r);
    for (int e = 0; e < 8; ++e) {
      const int raw = C.raw[(size_t)d * 8 + e];
      if (raw < 0 || m[e] < 0) continue;
      const int v = P.raw_slot[raw] >= 0 ? P.raw_slot[raw]
                                         : (raw_offd[raw] >= 0 ? h.nslots + raw_offd[raw] : -1);
      if (v >= 0) vlist[v].push_back(m[e]);
    }
    const int* nd = &C.nodes[(size_t)d * 4];
    const int ra = t == 1 ? nd[2] : nd[0];
    const int rb = (t == 4 || t == 6) ? nd[2] : nd[1];
    if (r[0] >= 0) rlist[ra].push_back(r[0]);
    if (r[1] >= 0) rlist[rb].push_back(r[1]);
    ndv += record_size(t, C.transient != 0);
    dev_flops += t == 6 ? 32 : t == 4 ? 30 : t == 3 ? 30 : (t == 5 && C.transient) ? 3 : 0;
  }
  if (C.pin_raw >= 0 && P.raw_slot[C.pin_raw] >= 0) vlist[P.raw_slot[C.pin_raw]].push_back(2);
  h.ndv = std::max(ndv, h.node_count);
  int64_t nadd = 0;
  g.amap_ptr.push_back(0);
  for (int v = 0; v < nv; ++v) {
    g.amap_code.insert(g.amap_code.end(), vlist[v].begin(), vlist[v].end());
    g.amap_ptr.push_back((i32)g.amap_code.size());
    nadd += (int64_t)vlist[v].size();
  }
  g.rmap_ptr.push_back(0);
  for (int i = 0; i < P.n; ++i) {
    g.rmap_code.insert(g.rmap_code.end(), rlist[i].begin(), rlist[i].end());
    g.rmap_ptr.push_back((i32)g.rmap_code.size());
    nadd += (int64_t)rlist[i].size();
  }
  g.in_row.assign(P.n + 1, 0);
  for (int k = 0; k <= P.n; ++k) {
    g.col_ptr.push_back(P.col_ptr[k]);
    g.dslot.push_back(k < P.n ? P.dslot[k] : 0);
    g.col_single.push_back(k < P.n ? P.col_single[k] : 0);
    g.out_pos.push_back(k < P.n ? P.out_pos[k] : 0);
    g.offd_ptr.push_back(P.offd_ptr[k]);
  }
  for (int r = 0; r < P.n; ++r) g.in_row[P.in_pos[r]] = r;
  for (int s = 0; s <= P.nslots(); ++s) {
    g.slot_row.push_back(s < P.nslots() ? P.slot_row[s] : 0);
    g.upd_ptr.push_back(P.upd_ptr[s]);
  }
  // long contribution lists (must match the kernel's threshold of 12)
  for (int v = 0; v < nv; ++v)
    if (g.amap_ptr[v + 1] - g.amap_ptr[v] > 12) g.heavy.push_back(v << 1);
  for (int i = 0; i < P.n; ++i) {
    const int r = g.in_row[i];
    if (g.rmap_ptr[r + 1] - g.rmap_ptr[r] > 12) g.heavy.push_back((i << 1) | 1);
  }
  h.nheavy = (int)g.heavy.size();
  // Four codes per value slot and per permuted rhs row, padded with +0.0
  // (x + 0.0 == x); longer lists are listed in lng and summed by the loop.
  g.amap4.assign((size_t)4 * nv, 4);
  g.rmap4.assign((size_t)4 * P.n, 4);
  for (int v = 0; v < nv; ++v) {
    const int t0 = g.amap_ptr[v], t1 = g.amap_ptr[v + 1];
    if (t1 - t0 > 4) {
      g.lng.push_back(v << 1);
      continue;
    }
    for (int t = t0; t < t1; ++t) g.amap4[(size_t)4 * v + (t - t0)] = g.amap_code[t];
  }
  for (int i = 0; i < P.n; ++i) {
    const int r = g.in_row[i];
    const int t0 = g.rmap_ptr[r], t1 = g.rmap_ptr[r + 1];
    if (t1 - t0 > 4) {
      g.lng.push_back((i << 1) | 1);
      continue;
    }
    for (int t = t0; t < t1; ++t) g.rmap4[(size_t)4 * i + (t - t0)] = g.rmap_code[t];
  }
  h.nlng = (int)g.lng.size();
  g.upd_dst = P.upd_dst;
  g.offd_col = P.offd_col;
  g.block_ptr.assign(P.block_ptr.begin(), P.block_ptr.end());
  // Level schedule of the factorization: column k depends on the columns of
  // its U entries; columns of one level are independent, each writes only
  // its own slots and performs its updates in the usual order, so lanes can
  // take them in parallel with results identical to the column order.
  // Columns with many U entries (the supply and ground rails) run as
  // sequential segments, lanes spread over each update instead.
  {
    const int kHub = 16;
    std::vector<int> lvl(P.n, 0);
    g.lseg_ptr.push_back(0);
    for (int b = 0; b < P.nblocks; ++b) {
      const int b0 = P.block_ptr[b], b1 = P.block_ptr[b + 1];
      int top = 0;
      for (int k = b0; k < b1; ++k) {
        int l = 0;
        for (int s = P.col_ptr[k]; s < P.dslot[k]; ++s) l = std::max(l, lvl[P.slot_row[s]]);
        lvl[k] = l + 1;
        top = std::max(top, lvl[k]);
      }
      for (int l = 1; l <= top; ++l)
        for (int hub = 0; hub < 2; ++hub) {
          const int start = (int)g.lvl_col.size();
          for (int k = b0; k < b1; ++k)
            if (lvl[k] == l && ((P.dslot[k] - P.col_ptr[k] > kHub) == (hub == 1)))
              g.lvl_col.push_back(k);
          const int end = (int)g.lvl_col.size();
          if (end > start) {
            g.lseg.push_back(start);
            g.lseg.push_back(end);
            g.lseg.push_back(hub);
          }
        }
      g.lseg_ptr.push_back((i32)g.lseg.size() / 3);
    }
    g.lvl_col.push_back(0);  // n+1 entries, parallel to the column arrays
    // Pivoting can chain the columns (an inverter chain's threshold swaps
    // leave one column per level); then the column-by-column path with lanes
    // over each update is faster, and the schedule is dropped.
    int levels = 0;
    for (int k = 0; k < P.n; ++k) levels = std::max(levels, lvl[k]);
    if ((int64_t)levels * 4 > P.n) {
      g.lseg.clear();
      std::fill(g.lseg_ptr.begin(), g.lseg_ptr.end(), 0);
    }
  }
  const char* esp = getenv("GPUKLU_STEP_PROGRAM");
  if (!C.transient && !(esp && esp[0] == '0')) build_steps(P, C.node_count, 0, g.ops, g.step_ptr);
  // FP64 operations of one Newton iteration: device evaluation, assembly
  // additions, refactorization, both substitutions, block coupling, update
  const int64_t nl = P.nnz_l, nu = P.nnz_u - P.n;
  g.flops = dev_flops + nadd + P.flops_refactor + 2 * (nl + nu) + P.n + 2 * h.noffd +
            6LL * h.node_count;
  // value bytes a Newton iteration moves through on-chip memory
  g.bytes = 8LL * (h.ndv + 2 * nadd + 3 * (int64_t)P.upd_dst.size() + 2 * nv +
                   6 * (nl + nu) + 6LL * P.n + 4LL * h.node_count);
  h.cost = (int)std::min<int64_t>(g.flops, 0x7fffffff);
  return g;
}

// Circuit constants (4 per device) with the reference's arithmetic:
// R 1/R (stamp.rs:253); D Is, 0.02585*N, Is/vt (stamp.rs:360-370); level-1
// beff = (u0*1e-4*(EPSILON_OX/tox))*W/L (bsim/mod.rs:445, params.rs:10,
// 460-462, evaluate.rs:318).
void circuit_constants(int64_t ndev, const int32_t* type, const double* p,
                       std::vector<double>& out, double dt = 0.0) {
  const double eps_ox = 3.9 * 8.854e-12;
  for (int64_t d = 0; d < ndev; ++d) {
    const double* q = p + 6 * d;
    double c[4] = {0.0, 0.0, 0.0, 0.0};
    switch (type[d]) {
      case 0: c[0] = 1.0 / q[0]; break;
      case 1:
      case 2: c[0] = q[0]; break;
      case 3: {
        const double vt = 0.02585 * q[1];
        c[0] = q[0];
        c[1] = vt;
        c[2] = q[0] / vt;
        break;
      }
      case 4:
      case 6: {
        const double beta = q[2] * 1e-4 * (eps_ox / q[3]);
        c[0] = type[d] == 4 ? q[0] : (q[0] != 0.0 ? -1.0 : 1.0);
        c[1] = type[d] == 4 ? q[1] : std::fabs(q[1]);
        c[2] = beta * q[4] / q[5];
        break;
      }
      case 5:  // C, and C/dt for the backward-Euler companion
        c[0] = q[0];
        c[1] = dt > 0.0 ? q[0] / dt : 0.0;
        break;
      default: c[0] = q[0]; break;
    }
    out.insert(out.end(), c, c + 4);
  }
}
}  // namespace

extern "C" {

}  // extern "C"

namespace {
gk::NewtonCfg to_newton_cfg(const gpuklu_newton_config& cfg) {
  gk::NewtonCfg c{};
  c.max_iters = (int)cfg.max_iters;
  c.gmin_steps = (int)cfg.gmin_steps;
  c.abs_tol = cfg.abs_tol;
  c.rel_tol = cfg.rel_tol;
  c.gmin = cfg.gmin;
  c.damping = cfg.damping;
  c.damping_min = cfg.damping_min;
  return c;
}

// Groups, programs, constants and launch classes of a batch. transient: the
// circuits are compiled with their capacitors' backward-Euler companions
// for step dt (pivots are chosen on the matrix with those conductances).
gpuklu_batch* batch_build(int64_t ncirc, const int64_t* dev_off, const int64_t* node_counts,
                          const int32_t* type, const int32_t* nodes, const double* p,
                          int64_t ninst, const int64_t* inst_circ, const int64_t* inst_dev,
                          const double* inst_val, const double* x0, const int64_t* x0_off,
                          int64_t x0_len, int transient, double dt) {
  auto B = std::make_unique<gpuklu_batch>();
  B->ncirc = ncirc;
  B->ninst = ninst;
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  gpuklu_handle* H = gpuklu_create(1);
  if (!H) return nullptr;
  gpuklu_set_pivot_mode(H, GPUKLU_PIVOT_EXACT);
  std::vector<int64_t> first(ncirc, -1);
  for (int64_t i = 0; i < ninst; ++i) {
    if (inst_circ[i] < 0 || inst_circ[i] >= ncirc) {
      fprintf(stderr, "gpuklu_batch_create: instance %ld has no circuit\n", (long)i);
      gpuklu_destroy(H);
      return nullptr;
    }
    if (first[inst_circ[i]] < 0) first[inst_circ[i]] = i;
  }
  std::vector<Program> progs;
  std::vector<std::string> keys;
  std::vector<int> circ_group(ncirc, -1);
  std::vector<long long> circ_poff(ncirc, 0);
  std::vector<double> dparams;
  for (int64_t c = 0; c < ncirc; ++c) {
    const int64_t d0 = dev_off[c], nd = dev_off[c + 1] - d0;
    circ_poff[c] = (long long)dparams.size();
    circuit_constants(nd, type + d0, p + 6 * d0, dparams, transient ? dt : 0.0);
    if (first[c] < 0) continue;
    gpuklu_circuit* C = gpuklu_compile_devices(node_counts[c], nd, type + d0, nodes + 4 * d0,
                                               p + 6 * d0, transient);
    if (!C) {
      gpuklu_destroy(H);
      return nullptr;
    }
    // pivot discovery on the representative instance's first matrix
    const int64_t rep = first[c];
    std::vector<double> pc(C->p);
    if (inst_dev && inst_dev[rep] >= 0) pc[(size_t)inst_dev[rep] * 6] = inst_val[rep];
    gpuklu_circuit_set_params(C, pc.data());
    std::vector<double> xr(C->node_count, 0.0);
    if (x0 && x0_off && x0_off[rep] >= 0)
      std::copy(x0 + x0_off[rep], x0 + x0_off[rep] + C->node_count, xr.begin());
    std::vector<double> ax(C->ai.size()), rhs(C->n);
    gpuklu_prepare(H, C->n);
    gpuklu_reset_pattern(H);
    int st = gpuklu_stamp(H, C, xr.data(), (int64_t)xr.size(), 1e-12, 1.0, transient ? dt : 0.0,
                          nullptr, 1.0, ax.data(), rhs.data());
    if (st == GPUKLU_OK)
      st = gpuklu_factor(H, C->ap.data(), (int64_t)C->ap.size(), C->ai.data(),
                         (int64_t)C->ai.size(), ax.data());
    if (st != GPUKLU_OK) {
      fprintf(stderr, "gpuklu_batch_create: circuit %ld: %s\n", (long)c, H->err.c_str());
      gpuklu_circuit_free(C);
      gpuklu_destroy(H);
      return nullptr;
    }
    Program pr = make_program(*C, H->plan);
    std::string k = pr.key();
    int gid = -1;
    for (size_t q = 0; q < keys.size(); ++q)
      if (keys[q].size() == k.size() && keys[q] == k) {
        gid = (int)q;
        break;
      }
    if (gid < 0) {
      gid = (int)progs.size();
      progs.push_back(std::move(pr));
      keys.push_back(std::move(k));
    }
    circ_group[c] = gid;
    gpuklu_circuit_free(C);
  }
  gpuklu_destroy(H);
  const int ng = (int)progs.size();
  std::vector<i32> dev_type, dev_nodes, dev_dv, amap_ptr, amap_code, rmap_ptr, rmap_code,
      col_ptr, dslot, col_single, in_row, out_pos, offd_ptr, slot_row, upd_ptr, upd_dst,
      offd_col, block_ptr, heavy, lvl_col, lseg_ptr, lseg, amap4, rmap4, lng, ops, step_ptr;
  auto cat = [](std::vector<i32>& dst, const std::vector<i32>& src) {
    dst.insert(dst.end(), src.begin(), src.end());
  };
  int region = 0;
  for (int g = 0; g < ng; ++g) {
    Program& pr = progs[g];
    gk::GroupHdr h = pr.h;
    h.dev_off = (int)dev_type.size();
    h.col_off = (int)col_ptr.size();
    h.slot_off = (int)slot_row.size();
    h.upd_off = (int)upd_dst.size();
    h.offd_off = (int)offd_col.size();
    h.blk_off = (int)block_ptr.size();
    h.amap_off = (int)amap_ptr.size();
    h.amap_code_off = (int)amap_code.size();
    h.nupd = (int)pr.upd_dst.size();
    h.heavy_off = (int)heavy.size();
    h.rmap_off = (int)rmap_ptr.size();
    h.rmap_code_off = (int)rmap_code.size();
    h.seg_off = (int)lseg.size() / 3;
    h.nseg = (int)pr.lseg.size() / 3;
    h.amap4_off = (int)amap4.size();
    h.rmap4_off = (int)rmap4.size();
    h.lng_off = (int)lng.size();
    h.ops_off = (int)(ops.size() / 2);
    h.nops = (int)(pr.ops.size() / 2);
    h.step_off = (int)step_ptr.size();
    h.nsteps = pr.step_ptr.empty() ? 0 : (int)pr.step_ptr.size() - 1;
    cat(ops, pr.ops);
    cat(step_ptr, pr.step_ptr);
    cat(dev_type, pr.dev_type);
    cat(dev_nodes, pr.dev_nodes);
    cat(dev_dv, pr.dev_dv);
    cat(amap_ptr, pr.amap_ptr);
    cat(amap_code, pr.amap_code);
    cat(rmap_ptr, pr.rmap_ptr);
    cat(rmap_code, pr.rmap_code);
    cat(col_ptr, pr.col_ptr);
    cat(dslot, pr.dslot);
    cat(col_single, pr.col_single);
    cat(in_row, pr.in_row);
    cat(out_pos, pr.out_pos);
    cat(offd_ptr, pr.offd_ptr);
    cat(slot_row, pr.slot_row);
    cat(upd_ptr, pr.upd_ptr);
    cat(upd_dst, pr.upd_dst);
    cat(offd_col, pr.offd_col);
    cat(block_ptr, pr.block_ptr);
    cat(heavy, pr.heavy);
    cat(lvl_col, pr.lvl_col);
    cat(lseg_ptr, pr.lseg_ptr);
    cat(lseg, pr.lseg);
    cat(amap4, pr.amap4);
    cat(rmap4, pr.rmap4);
    cat(lng, pr.lng);
    B->groups.push_back(h);
    B->group_flops.push_back(pr.flops);
    B->group_bytes.push_back(pr.bytes);
    region = std::max(region, h.node_count + h.n + h.ndv + h.nslots + h.noffd);
  }
  // instances grouped by program; each group's range in the order array
  const int ngr = (int)B->groups.size();
  std::vector<std::vector<i32>> members(ngr);
  B->inst_group_h.assign(ninst, 0);
  for (int64_t i = 0; i < ninst; ++i) {
    B->inst_group_h[i] = circ_group[inst_circ[i]];
    members[B->inst_group_h[i]].push_back((i32)i);
  }
  std::vector<i32> order;
  order.reserve(ninst);
  std::vector<int> gregion(ngr);
  for (int g = 0; g < ngr; ++g) {
    B->groups[g].inst_begin = (int)order.size();
    B->groups[g].inst_count = (int)members[g].size();
    order.insert(order.end(), members[g].begin(), members[g].end());
    const gk::GroupHdr& h = B->groups[g];
    // state doubles, then the row -> slot map (n ints)
    gregion[g] = (h.node_count + h.n + h.ndv + h.nslots + h.noffd + (h.n + 1) / 2 + 2) & ~1;
  }
  (void)region;
  B->x_off.assign(ninst, 0);
  long long off = 0;
  for (int64_t i = 0; i < ninst; ++i) {
    B->x_off[i] = off;
    off += progs[circ_group[inst_circ[i]]].h.n;
  }
  B->xout_len = off;
  B->x0_len = x0 ? x0_len : 0;
  // launch classes by per-instance shared memory: small programs put four
  // instances in a warp, medium two, large one
  std::vector<int> gorder(ngr);
  for (int g = 0; g < ngr; ++g) gorder[g] = g;
  std::stable_sort(gorder.begin(), gorder.end(),
                   [&](int x, int y) { return B->groups[x].cost > B->groups[y].cost; });
  // instances per warp by per-instance shared memory: small programs put
  // four instances in a warp, medium two, large one (more resident warps
  // hide more FP64 latency than wider packing saves)
  // Behind the lane phase the warp kernels only run the instances it parked,
  // mostly long non-converging runs: there one instance per warp, with the
  // block's shared memory carved per group, beats packing (measured on the
  // inverter chains: 140 ms against 161 ms per batch). Without the lane
  // phase small programs pack four or two instances per warp.
  const char* elanes = getenv("GPUKLU_BATCH_LANES");
  const bool lanes_on = !transient && !(elanes && elanes[0] == '0');
  int t4 = lanes_on ? 0 : 1152, t2 = lanes_on ? 0 : 2304;
  if (const char* epm = getenv("GPUKLU_PICK_M")) sscanf(epm, "%d,%d", &t4, &t2);
  auto pick_m = [t4, t2](int region, int prog) {
    (void)prog;
    return region <= t4 ? 4 : (region <= t2 ? 2 : 1);
  };
  const int mclass[4] = {1, 2, 4, 8};
  for (int g = 0; g < ngr; ++g) {
    gk::GroupHdr& h = B->groups[g];
    h.region = gregion[g];
    // column records, slot rows (and the update lists for leveled programs)
    h.prog = h.nsteps > 0 ? (2 * h.nops + h.nsteps + 1 + 3) & ~3
                          : (4 * h.n + h.nslots + (h.nseg > 0 ? h.nslots + h.nupd : 0) + 3) & ~3;
  }
  for (int ci = 0; ci < 4; ++ci) {
    auto C = std::make_unique<gpuklu_batch::Class>();
    C->m = mclass[ci];
    std::vector<int> members;
    for (int g : gorder) {
      const gk::GroupHdr& h = B->groups[g];
      const int prog = h.prog;
      if (pick_m(gregion[g], prog) != C->m || h.inst_count == 0) continue;
      members.push_back(g);
      C->region = std::max(C->region, gregion[g]);
      C->prog_ints = std::max(C->prog_ints, prog);
      const int nt = (h.inst_count + C->m - 1) / C->m;
      for (int t = 0; t < nt; ++t) C->tiles.push_back(g);
      for (int t = 0; t < std::min(nt, 12); ++t) C->tiles3.push_back(g);
    }
    if (C->tiles.empty()) continue;
    // shared-program tiles of the continuation: two consecutive ones per
    // group, so two blocks share the parked instances of a large program
    // whose block holds few warps (one tile per group: 122 ms for the
    // iteration-capped instances of the inverter-chain batch against 59;
    // two were measured best against three, four, eight and round-robin
    // orders). A tile whose group has nothing parked left is skipped before
    // its program is staged.
    for (int g : members)
      for (int t = 0; t < gpuklu_batch::kContTilesDefault; ++t) C->tiles2.push_back(g);
    C->members = members;
    gk::batch_kernel_info(C->m, C->warps_per_block, C->region, C->prog_ints, &C->regs,
                          &C->blocks_per_sm);
    if (C->blocks_per_sm <= 0) {
      fprintf(stderr, "gpuklu_batch_create: a circuit needs %d KB of shared memory\n",
              (int)(C->region * 8 * C->m / 1024));
      return nullptr;
    }
    C->grid = std::min<int>(sm_count() * C->blocks_per_sm, (int)C->tiles.size());
    {  // a block of warps sharing one program: each group fills the shared
       // memory with as many instance regions as fit beside its program
      const size_t cap = 227 * 1024;
      int wmin = 1 << 30, w = 0;
      std::vector<int> fit;
      for (int g : members) {
        const gk::GroupHdr& h = B->groups[g];
        const size_t prog = (size_t)h.prog * 4, per = (size_t)h.region * 8 * C->m;
        const int f = prog < cap ? (int)((cap - prog) / per) : 0;
        fit.push_back(f);
        wmin = std::min(wmin, f);
        w = std::max(w, f);
      }
      w = std::min(w, gpuklu_batch::kSharedWarpsMax);
      size_t bytes = 0;
      for (size_t q = 0; q < members.size(); ++q) {
        const gk::GroupHdr& h = B->groups[members[q]];
        bytes = std::max(bytes, (size_t)h.prog * 4 +
                                    (size_t)std::min(w, fit[q]) * h.region * 8 * C->m);
      }
      int r2 = 0, b2 = 0;
      const char* esh = getenv("GPUKLU_SHARED_PROGRAM");
      if ((esh && esh[0] == '0') || wmin < 2) w = 0;
      if (w >= 2)
        gk::batch_kernel_info(C->m, w, C->region, C->prog_ints, &r2, &b2, true, bytes);
      C->shared_bytes = (int)bytes;
      if (w >= 2 && b2 > 0 && w * b2 > C->blocks_per_sm * C->warps_per_block) {
        C->shared2 = true;
        C->wpb2 = w;
        C->grid2 = sm_count() * b2;
      } else {
        C->grid2 = C->grid;
        C->wpb2 = C->warps_per_block;
      }
    }
    if (cudaStreamCreateWithFlags(&C->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&C->done, cudaEventDisableTiming) != cudaSuccess)
      return nullptr;
    B->classes.push_back(std::move(C));
  }
  if (cudaEventCreateWithFlags(&B->start_ev, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  for (auto& ev : B->ph_ev)
    if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
  cudaStream_t s = B->stream;
  cudaError_t e = cudaSuccess;
  std::vector<i32> ov_dev(ninst);
  std::vector<double> ov_val(ninst);
  std::vector<long long> x0o(ninst, -1), poff(ninst);
  for (int64_t i = 0; i < ninst; ++i) {
    ov_dev[i] = inst_dev ? (i32)inst_dev[i] : -1;
    ov_val[i] = inst_val ? inst_val[i] : 0.0;
    if (x0 && x0_off) x0o[i] = x0_off[i];
    poff[i] = circ_poff[inst_circ[i]];
  }
#define UP(buf, vec) \
  if (e == cudaSuccess) e = B->buf.upload(vec, s);
  UP(d_groups, B->groups) UP(d_order, order)
  UP(d_dev_type, dev_type) UP(d_dev_nodes, dev_nodes) UP(d_dev_dv, dev_dv)
  UP(d_amap_ptr, amap_ptr) UP(d_amap_code, amap_code) UP(d_rmap_ptr, rmap_ptr)
  UP(d_rmap_code, rmap_code) UP(d_col_ptr, col_ptr) UP(d_dslot, dslot)
  UP(d_col_single, col_single) UP(d_in_row, in_row) UP(d_out_pos, out_pos)
  UP(d_offd_ptr, offd_ptr) UP(d_slot_row, slot_row) UP(d_upd_ptr, upd_ptr)
  UP(d_upd_dst, upd_dst) UP(d_offd_col, offd_col) UP(d_block_ptr, block_ptr)
  UP(d_heavy, heavy) UP(d_lvl_col, lvl_col) UP(d_lseg_ptr, lseg_ptr) UP(d_lseg, lseg)
  UP(d_amap4, amap4) UP(d_rmap4, rmap4) UP(d_lng, lng) UP(d_ops, ops) UP(d_step_ptr, step_ptr)
  UP(d_dparams, dparams) UP(d_p_off, poff) UP(d_ov_dev, ov_dev) UP(d_ov_val, ov_val)
  UP(d_x0_off, x0o) UP(d_x_off, B->x_off)
#undef UP
  for (auto& C : B->classes) {
    if (e == cudaSuccess) e = C->d_tiles.upload(C->tiles, s);
    if (e == cudaSuccess) e = C->d_tiles2.upload(C->tiles2, s);
    if (e == cudaSuccess) e = C->d_tiles3.upload(C->tiles3, s);
    if (e == cudaSuccess) e = C->d_counter.resize(1);
  }
  // Lane phase: every group split into tiles of about lane_target instances,
  // most expensive programs first; a scratch of region x 32 doubles per warp.
  {
    B->lanes = lanes_on;
    const char* ecap = getenv("GPUKLU_LANE_CAP");
    B->lane_cap = ecap ? std::max(1, atoi(ecap)) : 6;
    const char* etgt = getenv("GPUKLU_LANE_TARGET");
    const int target = etgt ? std::max(32, atoi(etgt)) : 32;
    long long lregion = 0;
    for (int g : gorder) {
      const gk::GroupHdr& h = B->groups[g];
      if (h.inst_count == 0) continue;
      const int nt = std::max(1, (h.inst_count + target - 1) / target);
      for (int t = 0; t < nt; ++t) B->ltiles.push_back(g);
      lregion = std::max<long long>(lregion, (long long)h.node_count + h.n + h.ndv + h.nslots +
                                                 h.noffd + 4LL * h.ndev);
    }
    if (B->lanes && !B->ltiles.empty()) {
      int regs = 0, bps = 0;
      gk::lanes_kernel_info(B->lane_wpb, &regs, &bps);
      const long long warps_max = (long long)sm_count() * std::max(bps, 1) * B->lane_wpb;
      const long long warps = std::min<long long>(warps_max, (long long)B->ltiles.size());
      B->lane_grid = (int)((warps + B->lane_wpb - 1) / B->lane_wpb);
      const long long stride = lregion * 32;
      if (e == cudaSuccess)
        e = B->d_scratch.resize((size_t)B->lane_grid * B->lane_wpb * (size_t)stride);
      if (e == cudaSuccess) e = B->d_ltiles.upload(B->ltiles, s);
      if (e == cudaSuccess) e = B->d_lcounter.resize(1);
      if (e == cudaSuccess) e = B->d_cont_list.resize(std::max<int64_t>(ninst, 1));
      for (auto* b : {&B->d_cont_it, &B->d_cont_total, &B->d_cont_gstep})
        if (e == cudaSuccess) e = b->resize(std::max<int64_t>(ninst, 1));
      for (auto* b : {&B->d_cont_damp, &B->d_cont_prev})
        if (e == cudaSuccess) e = b->resize(std::max<int64_t>(ninst, 1));
      if (e == cudaSuccess) e = B->d_cont_count.resize(std::max(ngr, 1));
      if (e == cudaSuccess) e = B->d_gnext2.resize(std::max(ngr, 1));
      B->args.warp_stride = stride;
      // continuation kernel: a warp's shared slice holds X, T and the LU
      // values of the largest program, its global slice the device records;
      // as many warps per block as the slices fit (at most 16)
      const char* eck = getenv("GPUKLU_CONT_KERNEL");
      int slice = 0, dvs = 0, ncs = 0;
      bool steps_all = true;
      for (int g : gorder) {
        const gk::GroupHdr& h = B->groups[g];
        slice = std::max(slice, h.n + h.nslots + h.noffd);
        dvs = std::max(dvs, h.ndv);
        ncs = std::max(ncs, h.node_count);
        if (h.inst_count > 0 && h.nsteps == 0) steps_all = false;
      }
      slice = (slice + 1) & ~1;
      const int dvx = (dvs + 3) & ~3;  // the iterate after the records
      dvs = dvx + ((ncs + 3) & ~3);
      // instances per warp: one; GPUKLU_CONT_M=2 puts two of a program in a
      // warp (16 lanes each, a step's FP64 instruction serving both), which
      // measured slower: the phase waits for its longest instances, and
      // their iterations take longer with half the lanes
      const char* ecm = getenv("GPUKLU_CONT_M");
      const int cm = ecm && ecm[0] == '2' ? 2 : 1;
      int wpb = std::min(16, (int)((size_t)(227 * 1024) / ((size_t)cm * slice * 8)));
      if (const char* ecw = getenv("GPUKLU_CONT_WARPS")) wpb = std::max(1, std::min(wpb, atoi(ecw)));
      if (!(eck && eck[0] == '0') && steps_all && wpb >= 1) {
        int r3 = 0, b3 = 0;
        gk::cont_kernel_info(cm, wpb, slice, &r3, &b3);
        if (b3 > 0) {
          B->cont_kernel = true;
          B->cont_m = cm;
          B->cont_wpb = wpb;
          B->cont_grid = sm_count() * b3;
          B->args.slice = slice;
          B->args.dv_stride = dvs;
          B->args.dv_x = dvx;
          std::vector<i32> cg(gorder.begin(), gorder.end());
          if (e == cudaSuccess) e = B->d_cont_groups.upload(cg, s);
          if (e == cudaSuccess) e = B->d_cont_cursor.resize(1);
          if (e == cudaSuccess)
            e = B->d_dv.resize((size_t)B->cont_grid * wpb * cm * (size_t)dvs);
        }
      }
    } else {
      B->lanes = false;
    }
  }
  if (e == cudaSuccess) {
    std::vector<double> x0v;
    if (x0) x0v.assign(x0, x0 + B->x0_len);
    e = B->d_x0.upload(x0v, s);
  }
  if (e == cudaSuccess) e = B->d_xout.resize(std::max<int64_t>(B->xout_len, 1));
  if (e == cudaSuccess) e = B->d_iters.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_iters_total.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_reason.resize(std::max<int64_t>(ninst, 1));
  if (e == cudaSuccess) e = B->d_status.resize(1);
  if (e == cudaSuccess) e = B->d_gnext.resize(std::max(ngr, 1));
  if (e == cudaSuccess) e = cudaMemsetAsync(B->d_status.p, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_batch_create: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  gk::BatchArgs a{};
  a.groups = B->d_groups.p;
  a.ngroups = ngr;
  a.gnext = B->d_gnext.p;
  a.order = B->d_order.p;
  a.dev_type = B->d_dev_type.p;
  a.dev_nodes = B->d_dev_nodes.p;
  a.dev_dv = B->d_dev_dv.p;
  a.amap_ptr = B->d_amap_ptr.p;
  a.amap_code = B->d_amap_code.p;
  a.rmap_ptr = B->d_rmap_ptr.p;
  a.rmap_code = B->d_rmap_code.p;
  a.col_ptr = B->d_col_ptr.p;
  a.dslot = B->d_dslot.p;
  a.col_single = B->d_col_single.p;
  a.in_row = B->d_in_row.p;
  a.out_pos = B->d_out_pos.p;
  a.offd_ptr = B->d_offd_ptr.p;
  a.slot_row = B->d_slot_row.p;
  a.upd_ptr = B->d_upd_ptr.p;
  a.upd_dst = B->d_upd_dst.p;
  a.offd_col = B->d_offd_col.p;
  a.block_ptr = B->d_block_ptr.p;
  a.heavy = B->d_heavy.p;
  a.lvl_col = B->d_lvl_col.p;
  a.lseg_ptr = B->d_lseg_ptr.p;
  a.lseg = B->d_lseg.p;
  a.amap4 = B->d_amap4.p;
  a.rmap4 = B->d_rmap4.p;
  a.lng = B->d_lng.p;
  a.ops = reinterpret_cast<const int2*>(B->d_ops.p);
  a.step_ptr = B->d_step_ptr.p;
  a.inst_p_off = B->d_p_off.p;
  a.dparams = B->d_dparams.p;
  a.inst_ov_dev = B->d_ov_dev.p;
  a.inst_ov_val = B->d_ov_val.p;
  a.inst_x0_off = B->d_x0_off.p;
  a.x0 = B->d_x0.p;
  a.iters = B->d_iters.p;
  a.iters_total = B->d_iters_total.p;
  a.reason = B->d_reason.p;
  a.inst_x_off = B->d_x_off.p;
  a.x_out = B->d_xout.p;
  a.status = B->d_status.p;
  if (B->lanes) {
    a.scratch = B->d_scratch.p;
    a.warp_stride = B->args.warp_stride;
    a.ltile_group = B->d_ltiles.p;
    a.nltiles = (int)B->ltiles.size();
    a.lcounter = B->d_lcounter.p;
    a.cap = B->lane_cap;
    a.cont_list = B->d_cont_list.p;
    a.cont_count = B->d_cont_count.p;
    a.gnext2 = B->d_gnext2.p;
    a.cont_it = B->d_cont_it.p;
    a.cont_total = B->d_cont_total.p;
    a.cont_gstep = B->d_cont_gstep.p;
    a.cont_damp = B->d_cont_damp.p;
    a.cont_prev = B->d_cont_prev.p;
    if (B->cont_kernel) {
      a.cont_groups = B->d_cont_groups.p;
      a.cont_ngroups = (int)B->d_cont_groups.n;
      a.cont_cursor = B->d_cont_cursor.p;
      a.dv_scratch = B->d_dv.p;
      a.dv_stride = B->args.dv_stride;
      a.dv_x = B->args.dv_x;
      a.slice = B->args.slice;
    }
  }
  B->args = a;
  for (auto& C : B->classes) {
    C->args = a;
    C->args.tile_group = C->d_tiles.p;
    C->args.ntiles = (int)C->tiles.size();
    C->args.counter = C->d_counter.p;
    C->args.region = C->region;
    C->args.prog_ints = C->prog_ints;
    C->args.shared_bytes = C->shared_bytes;
  }
  B->transient = transient;
  B->dt = dt;
  return B.release();
}
}  // namespace

extern "C" {

gpuklu_batch* gpuklu_batch_create(int64_t ncirc, const int64_t* dev_off,
                                  const int64_t* node_counts, const int32_t* type,
                                  const int32_t* nodes, const double* p, int64_t ninst,
                                  const int64_t* inst_circ, const int64_t* inst_dev,
                                  const double* inst_val, const double* x0,
                                  const int64_t* x0_off, int64_t x0_len) {
  return batch_build(ncirc, dev_off, node_counts, type, nodes, p, ninst, inst_circ, inst_dev,
                     inst_val, x0, x0_off, x0_len, 0, 0.0);
}

gpuklu_batch* gpuklu_tran_create(int64_t ncirc, const int64_t* dev_off,
                                 const int64_t* node_counts, const int32_t* type,
                                 const int32_t* nodes, const double* p, const double* x_init,
                                 const int64_t* x_init_off, int64_t x_init_len, double dt,
                                 int64_t steps, int64_t ckpt_every, const int64_t* probe,
                                 double target) {
  if (ncirc <= 0 || !(dt > 0.0) || steps <= 0 || ckpt_every <= 0 || !x_init || !x_init_off ||
      !probe) {
    fprintf(stderr, "gpuklu_tran_create: invalid arguments\n");
    return nullptr;
  }
  for (int64_t i = 0; i < ncirc; ++i)
    if (probe[i] < 0 || probe[i] >= node_counts[i] || x_init_off[i] < 0 ||
        x_init_off[i] + node_counts[i] > x_init_len) {
      fprintf(stderr, "gpuklu_tran_create: instance %ld: probe or initial state out of range\n",
              (long)i);
      return nullptr;
    }
  std::vector<int64_t> ic(ncirc);
  for (int64_t i = 0; i < ncirc; ++i) ic[i] = i;
  std::unique_ptr<gpuklu_batch> B(batch_build(ncirc, dev_off, node_counts, type, nodes, p, ncirc,
                                              ic.data(), nullptr, nullptr, x_init, x_init_off,
                                              x_init_len, 1, dt));
  if (!B) return nullptr;
  const int64_t ninst = ncirc;
  B->steps = steps;
  B->ckpt_every = ckpt_every;
  const int64_t nck = steps / ckpt_every + 1;
  std::vector<long long> ck_off(ninst), seg_off(ninst);
  std::vector<i32> probe_h(ninst);
  B->grad_off_h.assign(ninst, 0);
  long long ck = 0, sg = 0, go = 0;
  int region = 0, prog = 0;
  for (int64_t i = 0; i < ninst; ++i) {
    const gk::GroupHdr& h = B->groups[B->inst_group_h[i]];
    region = std::max(region, 2 * h.node_count + 2 * h.n + h.ndv + h.nslots + h.noffd + h.ndev +
                                  (h.n + 1) / 2 + 1);
    prog = std::max(prog, (4 * h.n + h.nslots + (h.nseg > 0 ? h.nslots + h.nupd : 0) + 3) & ~3);
    ck_off[i] = ck;
    ck += nck * h.node_count;
    seg_off[i] = sg;
    sg += (ckpt_every + 1) * h.node_count;
    B->grad_off_h[i] = go;
    go += h.ndev;
    probe_h[i] = (i32)probe[i];
  }
  region = (region + 1) & ~1;
  B->tran_region = region;
  B->tran_prog = prog;
  B->grad_len = go;
  cudaStream_t s = B->stream;
  cudaError_t e = B->d_inst_group.upload(B->inst_group_h, s);
  if (e == cudaSuccess) e = B->d_probe.upload(probe_h, s);
  if (e == cudaSuccess) e = B->d_ckpt_off.upload(ck_off, s);
  if (e == cudaSuccess) e = B->d_seg_off.upload(seg_off, s);
  if (e == cudaSuccess) e = B->d_grad_off.upload(B->grad_off_h, s);
  if (e == cudaSuccess) e = B->d_loss.resize(ninst);
  if (e == cudaSuccess) e = B->d_ckpt.resize(std::max<long long>(ck, 1));
  if (e == cudaSuccess) e = B->d_seg.resize(std::max<long long>(sg, 1));
  if (e == cudaSuccess) e = B->d_grad.resize(std::max<long long>(go, 1));
  if (e == cudaSuccess) e = B->d_tcounter.resize(1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_tran_create: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  int regs = 0, bf = 0, bb = 0;
  gk::tran_kernel_info(false, 1, region, prog, &regs, &bf);
  gk::tran_kernel_info(true, 1, region, prog, &regs, &bb);
  if (bf <= 0 || bb <= 0) {
    fprintf(stderr, "gpuklu_tran_create: a circuit needs %d KB of shared memory\n",
            (int)((region * 8 + prog * 4) / 1024));
    return nullptr;
  }
  B->tran_grid_f = (int)std::min<int64_t>(ninst, (int64_t)sm_count() * bf);
  B->tran_grid_b = (int)std::min<int64_t>(ninst, (int64_t)sm_count() * bb);
  gk::BatchArgs& a = B->args;
  a.ninst = (int)ninst;
  a.inst_group = B->d_inst_group.p;
  a.dt = dt;
  a.inv_dt = 1.0 / dt;
  a.steps = (int)steps;
  a.ckpt_every = (int)ckpt_every;
  a.probe = B->d_probe.p;
  a.target = target;
  a.loss = B->d_loss.p;
  a.wave = nullptr;
  a.ckpt = B->d_ckpt.p;
  a.ckpt_off = B->d_ckpt_off.p;
  a.seg = B->d_seg.p;
  a.seg_off = B->d_seg_off.p;
  a.grad = B->d_grad.p;
  a.grad_off = B->d_grad_off.p;
  a.region = region;
  a.prog_ints = prog;
  a.counter = B->d_tcounter.p;
  return B.release();
}

gpuklu_batch* gpuklu_atran_create(int64_t ncirc, const int64_t* dev_off,
                                  const int64_t* node_counts, const int32_t* type,
                                  const int32_t* nodes, const double* p, const int32_t* wkind,
                                  const double* wp7, const int64_t* pwl_ptr, const double* pwl_t,
                                  const double* pwl_v, const double* x_ic,
                                  const int64_t* x_ic_off, int64_t x_ic_len,
                                  const int64_t* probe) {
  if (ncirc <= 0 || !x_ic || !x_ic_off || !probe) {
    fprintf(stderr, "gpuklu_atran_create: invalid arguments\n");
    return nullptr;
  }
  for (int64_t i = 0; i < ncirc; ++i) {
    if (probe[i] < 0 || probe[i] >= node_counts[i] || x_ic_off[i] < 0 ||
        x_ic_off[i] + node_counts[i] > x_ic_len) {
      fprintf(stderr, "gpuklu_atran_create: instance %ld: probe or initial guess out of range\n",
              (long)i);
      return nullptr;
    }
    for (int64_t d = dev_off[i]; d < dev_off[i + 1]; ++d)
      if (wkind && wkind[d] != 0 && (type[d] != 1 && type[d] != 2 || wkind[d] < 1 ||
                                     wkind[d] > 4)) {
        fprintf(stderr, "gpuklu_atran_create: device %ld: a waveform needs a V or I source "
                        "and kind 1..4\n", (long)d);
        return nullptr;
      }
  }
  std::vector<int64_t> ic(ncirc);
  for (int64_t i = 0; i < ncirc; ++i) ic[i] = i;
  std::unique_ptr<gpuklu_batch> B(batch_build(ncirc, dev_off, node_counts, type, nodes, p, ncirc,
                                              ic.data(), nullptr, nullptr, x_ic, x_ic_off,
                                              x_ic_len, 1, 1.0));
  if (!B) return nullptr;
  B->atran = true;
  const int64_t ninst = ncirc;
  int region = 0, prog = 0;
  std::vector<i32> probe_h(ninst);
  B->at_wptr.assign(1, 0);
  B->at_pwlptr.assign(1, 0);
  for (int64_t i = 0; i < ninst; ++i) {
    const gk::GroupHdr& h = B->groups[B->inst_group_h[i]];
    region = std::max(region, 4 * h.n + 2 * h.ndev + h.ndv + h.nslots + h.noffd +
                                  (h.n + 1) / 2 + 1);
    prog = std::max(prog, (4 * h.n + h.nslots + (h.nseg > 0 ? h.nslots + h.nupd : 0) + 3) & ~3);
    probe_h[i] = (i32)probe[i];
    for (int64_t d = dev_off[i]; d < dev_off[i + 1]; ++d) {
      if (!wkind || wkind[d] == 0) continue;
      B->at_wdev.push_back((i32)(d - dev_off[i]));
      B->at_wkind.push_back(wkind[d]);
      for (int k = 0; k < 7; ++k) B->at_wp.push_back(wp7 ? wp7[d * 7 + k] : 0.0);
      std::vector<std::pair<double, double>> pts;
      if (pwl_ptr)
        for (int64_t q = pwl_ptr[d]; q < pwl_ptr[d + 1]; ++q) pts.push_back({pwl_t[q], pwl_v[q]});
      std::stable_sort(pts.begin(), pts.end(),  // PwlParams::new (waveform.rs:137-143)
                       [](const std::pair<double, double>& a, const std::pair<double, double>& b) {
                         return a.first < b.first;
                       });
      for (auto& pt : pts) {
        B->at_pwlt.push_back(pt.first);
        B->at_pwlv.push_back(pt.second);
      }
      B->at_pwlptr.push_back((i32)B->at_pwlt.size());
    }
    B->at_wptr.push_back((i32)B->at_wdev.size());
  }
  region = (region + 1) & ~1;
  cudaStream_t s = B->stream;
  cudaError_t e = B->d_inst_group.upload(B->inst_group_h, s);
  if (e == cudaSuccess) e = B->d_probe.upload(probe_h, s);
  if (e == cudaSuccess) e = B->d_at_wptr.upload(B->at_wptr, s);
  if (e == cudaSuccess) e = B->d_at_wdev.upload(B->at_wdev, s);
  if (e == cudaSuccess) e = B->d_at_wkind.upload(B->at_wkind, s);
  if (e == cudaSuccess) e = B->d_at_pwlptr.upload(B->at_pwlptr, s);
  if (e == cudaSuccess) e = B->d_at_wp.upload(B->at_wp, s);
  if (e == cudaSuccess) e = B->d_at_pwlt.upload(B->at_pwlt, s);
  if (e == cudaSuccess) e = B->d_at_pwlv.upload(B->at_pwlv, s);
  if (e == cudaSuccess) e = B->d_tcounter.resize(1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_atran_create: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  int regs = 0, bps = 0;
  gk::atran_kernel_info(region, prog, &regs, &bps);
  if (bps <= 0) {
    fprintf(stderr, "gpuklu_atran_create: a circuit needs %d KB of shared memory\n",
            (int)((region * 8 + prog * 4) / 1024));
    return nullptr;
  }
  B->at_grid = (int)std::min<int64_t>(ninst, (int64_t)sm_count() * bps);
  gk::BatchArgs& a = B->args;
  a.ninst = (int)ninst;
  a.inst_group = B->d_inst_group.p;
  a.region = region;
  a.prog_ints = prog;
  a.counter = B->d_tcounter.p;
  return B.release();
}

namespace {
// Breakpoints of one instance's PULSE and PWL sources for a run to tstop
// (BreakpointManager::extract_from_sources, waveform.rs:459-530; the engine
// extracts only these two kinds, engine.rs:635-680): sorted, unique.
void instance_breakpoints(const gpuklu_batch* b, int64_t i, double tstop,
                          std::vector<double>& out) {
  out.clear();
  auto add = [&](double t) {
    if (t >= 0.0) out.push_back(t);
  };
  for (int r = b->at_wptr[i]; r < b->at_wptr[i + 1]; ++r) {
    const double* q = &b->at_wp[(size_t)r * 7];
    if (b->at_wkind[r] == 1) {
      const double td = q[2], tr = q[3], tf = q[4], pw = q[5], per = q[6];
      double t = td;
      int count = 0;
      if (td > 0.0) add(td);
      while (t <= tstop && count < 10000) {
        add(t);
        const double th = t + tr;
        if (th > tstop) break;
        add(th);
        const double tfl = th + pw;
        if (tfl > tstop) break;
        add(tfl);
        const double tl = tfl + tf;
        if (tl > tstop) break;
        add(tl);
        if (per > 0.0) {
          t = td + per * (double)(count + 1);
          count += 1;
        } else {
          break;
        }
      }
    } else if (b->at_wkind[r] == 2) {
      for (int qq = b->at_pwlptr[r]; qq < b->at_pwlptr[r + 1]; ++qq) add(b->at_pwlt[qq]);
    }
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}
}  // namespace

int gpuklu_atran_run(gpuklu_batch* b, const gpuklu_newton_config* cfg, double tstep,
                     double tstop, double tstart, double tmax, double lte_abs, double lte_rel,
                     double be_sign, int64_t max_points, int64_t max_steps, double* times_out,
                     double* probe_out, int64_t* npoints, int64_t* accepted, int64_t* rejected,
                     int32_t* status, int64_t* iters, double* x_out) {
  if (!b || !cfg || !b->atran) return GPUKLU_INVALID_MATRIX;
  if (!(tstep > 0.0) || !(tstop > tstart) || !(tmax > 0.0) || max_points < 0 || max_steps <= 0 ||
      max_steps > (int64_t)1 << 30 || (double)b->ninst * (double)max_points > 4e9) {
    b->err = "gpuklu_atran_run: tstep > 0, tstop > tstart, tmax > 0, 0 <= max_points, "
             "0 < max_steps <= 2^30";
    return GPUKLU_INVALID_MATRIX;
  }
  const int64_t ni = b->ninst;
  std::vector<i32> bp_ptr(1, 0);
  std::vector<double> bp_t, tmp;
  for (int64_t i = 0; i < ni; ++i) {
    instance_breakpoints(b, i, tstop, tmp);
    bp_t.insert(bp_t.end(), tmp.begin(), tmp.end());
    bp_ptr.push_back((i32)bp_t.size());
  }
  cudaStream_t s = b->stream;
  const size_t np = (size_t)ni * (size_t)max_points;
  cudaError_t e = b->d_at_bpptr.upload(bp_ptr, s);
  if (e == cudaSuccess) e = b->d_at_bpt.upload(bp_t, s);
  if (e == cudaSuccess) e = b->d_at_times.resize(std::max<size_t>(np, 1));
  if (e == cudaSuccess) e = b->d_at_probe.resize(std::max<size_t>(np, 1));
  if (e == cudaSuccess) e = b->d_at_out.resize((size_t)ni * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->args.counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "adaptive transient"));
  gk::BatchArgs a = b->args;
  a.cfg = to_newton_cfg(*cfg);
  gk::AtranArgs t{};
  t.wave_ptr = b->d_at_wptr.p;
  t.wave_dev = b->d_at_wdev.p;
  t.wave_kind = b->d_at_wkind.p;
  t.pwl_ptr = b->d_at_pwlptr.p;
  t.wave_p = b->d_at_wp.p;
  t.pwl_t = b->d_at_pwlt.p;
  t.pwl_v = b->d_at_pwlv.p;
  t.bp_ptr = b->d_at_bpptr.p;
  t.bp_t = b->d_at_bpt.p;
  t.probe = b->d_probe.p;
  t.tstep = tstep;
  t.tstop = tstop;
  t.tstart = tstart;
  t.tmax = tmax;
  t.lte_abs = lte_abs;
  t.lte_rel = lte_rel;
  t.be_sign = be_sign;
  t.max_points = (int)max_points;
  t.max_steps = (int)max_steps;
  t.times = b->d_at_times.p;
  t.probe_out = b->d_at_probe.p;
  t.status = b->d_at_out.p;
  t.npoints = b->d_at_out.p + ni;
  t.accepted = b->d_at_out.p + 2 * ni;
  t.rejected = b->d_at_out.p + 3 * ni;
  gk::launch_atran(a, t, b->at_grid, s);
  std::vector<i32> outs((size_t)ni * 4), it(ni);
  e = cudaGetLastError();
  if (e == cudaSuccess && times_out && np)
    e = cudaMemcpyAsync(times_out, b->d_at_times.p, np * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && probe_out && np)
    e = cudaMemcpyAsync(probe_out, b->d_at_probe.p, np * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(outs.data(), b->d_at_out.p, outs.size() * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(it.data(), b->d_iters_total.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && x_out)
    e = cudaMemcpyAsync(x_out, b->d_xout.p, b->xout_len * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "adaptive transient"));
  for (int64_t i = 0; i < ni; ++i) {
    if (status) status[i] = outs[i];
    if (npoints) npoints[i] = outs[ni + i];
    if (accepted) accepted[i] = outs[2 * ni + i];
    if (rejected) rejected[i] = outs[3 * ni + i];
    if (iters) iters[i] = it[i];
  }
  return GPUKLU_OK;
}

int gpuklu_tran_forward(gpuklu_batch* b, const gpuklu_newton_config* cfg, double* loss_out,
                        double* wave_out, int64_t* iters_out, int32_t* reason_out) {
  if (!b || !cfg || !b->transient) return GPUKLU_INVALID_MATRIX;
  gk::BatchArgs a = b->args;
  a.cfg = to_newton_cfg(*cfg);
  cudaStream_t s = b->stream;
  cudaError_t e = cudaSuccess;
  if (wave_out) {
    e = b->d_wave.resize((size_t)b->ninst * (size_t)b->steps);
    a.wave = b->d_wave.p;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "transient forward"));
  gk::launch_tran_forward(a, b->tran_grid_f, 1, s);
  const int64_t ni = b->ninst;
  std::vector<i32> it(ni), rs(ni);
  e = cudaGetLastError();
  if (e == cudaSuccess && loss_out)
    e = cudaMemcpyAsync(loss_out, b->d_loss.p, ni * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && wave_out)
    e = cudaMemcpyAsync(wave_out, b->d_wave.p, (size_t)ni * b->steps * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(it.data(), b->d_iters_total.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rs.data(), b->d_reason.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "transient forward"));
  for (int64_t i = 0; i < ni; ++i) {
    if (iters_out) iters_out[i] = it[i];
    if (reason_out) reason_out[i] = rs[i];
  }
  b->tran_fwd_done = true;
  return GPUKLU_OK;
}

int gpuklu_tran_backward(gpuklu_batch* b, const gpuklu_newton_config* cfg, double* grad_out,
                         int64_t* iters_out) {
  if (!b || !cfg || !b->transient) return GPUKLU_INVALID_MATRIX;
  if (!b->tran_fwd_done) {
    b->err = "gpuklu_tran_backward needs a completed gpuklu_tran_forward";
    return GPUKLU_SOLVE_FAILED;
  }
  gk::BatchArgs a = b->args;
  a.cfg = to_newton_cfg(*cfg);
  cudaStream_t s = b->stream;
  cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "transient backward"));
  gk::launch_tran_backward(a, b->tran_grid_b, 1, s);
  const int64_t ni = b->ninst;
  std::vector<i32> it(ni);
  e = cudaGetLastError();
  if (e == cudaSuccess && grad_out)
    e = cudaMemcpyAsync(grad_out, b->d_grad.p, b->grad_len * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(it.data(), b->d_iters.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "transient backward"));
  if (iters_out)
    for (int64_t i = 0; i < ni; ++i) iters_out[i] = it[i];
  return GPUKLU_OK;
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
  const gk::NewtonCfg c = to_newton_cfg(*cfg);
  cudaStream_t s = b->stream;
  cudaMemsetAsync(b->d_gnext.p, 0, b->d_gnext.n * sizeof(unsigned), s);
  for (auto& C : b->classes) cudaMemsetAsync(C->d_counter.p, 0, sizeof(unsigned), s);
  if (b->lanes) {  // phase 1: lane per instance, then the warp classes take the parked ones
    cudaMemsetAsync(b->d_lcounter.p, 0, sizeof(unsigned), s);
    cudaMemsetAsync(b->d_cont_count.p, 0, b->d_cont_count.n * sizeof(unsigned), s);
    cudaMemsetAsync(b->d_gnext2.p, 0, b->d_gnext2.n * sizeof(unsigned), s);
  }
  cudaEventRecord(b->ph_ev[0], s);
  const bool fresh = b->lanes && b->cont_kernel && b->lane_cap == 0;
  if (b->lanes && !fresh) {
    gk::BatchArgs la = b->args;
    la.cfg = c;
    gk::launch_batch_lanes(la, b->lane_grid, b->lane_wpb, s);
  }
  cudaEventRecord(b->ph_ev[1], s);
  if (b->lanes && b->cont_kernel) {  // phase 2: one warp per parked instance (or all)
    cudaMemsetAsync(b->d_cont_cursor.p, 0, sizeof(unsigned), s);
    gk::BatchArgs ca = b->args;
    ca.cfg = c;
    ca.cont_fresh = fresh ? 1 : 0;
    gk::launch_batch_cont(ca, b->cont_m, b->cont_grid, b->cont_wpb, s);
    cudaEventRecord(b->ph_ev[2], s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch launch"));
    return GPUKLU_OK;
  }
  cudaEventRecord(b->start_ev, s);
  for (auto& C : b->classes) {  // largest programs first, all classes concurrent
    cudaStreamWaitEvent(C->stream, b->start_ev, 0);
    C->args.cfg = c;
    gk::BatchArgs ca = C->args;
    if (b->lanes) {
      ca.cont_mode = 1;
      ca.tile_group = C->shared2 ? C->d_tiles2.p : C->d_tiles3.p;
      ca.ntiles = (int)(C->shared2 ? C->tiles2.size() : C->tiles3.size());
      gk::launch_batch_newton(ca, C->m, C->grid2, C->wpb2, C->stream, C->shared2);
    } else {
      gk::launch_batch_newton(ca, C->m, C->grid, C->warps_per_block, C->stream);
    }
    cudaEventRecord(C->done, C->stream);
    cudaStreamWaitEvent(s, C->done, 0);
  }
  cudaEventRecord(b->ph_ev[2], s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch launch"));
  return GPUKLU_OK;
}

int gpuklu_batch_set_schedule(gpuklu_batch* b, int lane_cap, int cont_tiles) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  // lane cap 0: no lane phase, the continuation kernel starts every instance
  const int cap_lo = b->cont_kernel ? 0 : 1;
  if (cont_tiles < 1 || cont_tiles > 16 ||
      (b->lanes && (lane_cap < cap_lo || lane_cap > 100))) {
    b->err = std::string("gpuklu_batch_set_schedule: lane_cap in ") + std::to_string(cap_lo) +
             "..100 and cont_tiles in 1..16";
    return GPUKLU_INVALID_MATRIX;
  }
  cudaError_t e = cudaStreamSynchronize(b->stream);  // no run may still read the tiles
  if (b->lanes) {
    b->lane_cap = lane_cap;
    b->args.cap = lane_cap;
    for (auto& C : b->classes) C->args.cap = lane_cap;
  }
  if (cont_tiles != b->cont_tiles) {
    for (auto& C : b->classes) {
      C->tiles2.clear();
      for (int g : C->members)
        for (int t = 0; t < cont_tiles; ++t) C->tiles2.push_back(g);
      if (e == cudaSuccess) e = C->d_tiles2.upload(C->tiles2, b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    b->cont_tiles = cont_tiles;
  }
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch schedule"));
  return GPUKLU_OK;
}

int gpuklu_batch_autotune(gpuklu_batch* b, const gpuklu_newton_config* cfg, int64_t* out,
                          double* best_ms) {
  if (!b || !cfg) return GPUKLU_INVALID_MATRIX;
  if (b->transient) {
    b->err = "gpuklu_batch_autotune: a transient batch has no schedule";
    return GPUKLU_INVALID_MATRIX;
  }
  // one timed run of the batch per candidate: the lane phase's iteration cap,
  // then the continuation's tiles per group, each with the other at its best
  // so far (two rounds of coordinate descent from the current schedule)
  auto timed = [&](int cap, int ct, double* ms) -> int {
    int st = gpuklu_batch_set_schedule(b, cap, ct);
    if (st == GPUKLU_OK) st = gpuklu_batch_run(b, cfg);
    double ph[3] = {0, 0, 0};
    if (st == GPUKLU_OK) st = gpuklu_batch_phase_ms(b, ph);
    *ms = ph[0] + ph[1];
    return st;
  };
  static const int caps[] = {0, 1, 2, 3, 4, 5, 6, 8, 10, 12};
  static const int cts[] = {1, 2, 3, 4};
  // the continuation kernel has no tiles: only the cap is searched then
  const bool tiles = !(b->lanes && b->cont_kernel);
  int cap = b->lanes ? b->lane_cap : 1, ct = b->cont_tiles, trials = 0;
  double best = 0.0;
  int st = timed(cap, ct, &best);  // warm-up, then the current schedule
  if (st == GPUKLU_OK) st = timed(cap, ct, &best);
  trials += 2;
  for (int round = 0; round < 2 && st == GPUKLU_OK; ++round) {
    const int cap0 = cap, ct0 = ct;
    if (b->lanes)
      for (int c : caps) {
        if (c == cap || st != GPUKLU_OK || (c == 0 && !b->cont_kernel)) continue;
        double ms = 0.0;
        st = timed(c, ct, &ms);
        ++trials;
        if (st == GPUKLU_OK && ms < best) best = ms, cap = c;
      }
    for (int c : cts) {
      if (!tiles || c == ct || st != GPUKLU_OK) continue;
      double ms = 0.0;
      st = timed(cap, c, &ms);
      ++trials;
      if (st == GPUKLU_OK && ms < best) best = ms, ct = c;
    }
    if (cap == cap0 && ct == ct0) break;
  }
  if (st == GPUKLU_OK) st = gpuklu_batch_set_schedule(b, cap, ct);
  if (out) {
    out[0] = b->lanes ? cap : 0;
    out[1] = ct;
    out[2] = trials;
  }
  if (best_ms) *best_ms = best;
  return st;
}

int gpuklu_batch_phase_ms(gpuklu_batch* b, double* out) {
  if (!b || !out) return GPUKLU_INVALID_MATRIX;
  cudaError_t e = cudaEventSynchronize(b->ph_ev[2]);
  float a = 0.f, w = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&a, b->ph_ev[0], b->ph_ev[1]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&w, b->ph_ev[1], b->ph_ev[2]);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch phase timing"));
  out[0] = a;
  out[1] = w;
  out[2] = b->lanes ? b->lane_cap : 0;
  return GPUKLU_OK;
}

int gpuklu_batch_results(gpuklu_batch* b, int64_t* iters, int64_t* iters_total, int32_t* reason,
                         double* x_out, const int64_t* x_off) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  const int64_t ni = b->ninst;
  std::vector<i32> it(ni), itt(ni), rs(ni);
  std::vector<double> xo;
  cudaStream_t s = b->stream;
  cudaError_t e = cudaMemcpyAsync(it.data(), b->d_iters.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(itt.data(), b->d_iters_total.p, ni * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rs.data(), b->d_reason.p, ni * 4, cudaMemcpyDeviceToHost, s);
  // the caller's layout is the batch's own (the usual case): one copy straight
  // into x_out, a DMA when x_out is pinned
  bool direct = x_out && x_off && b->xout_len;
  for (int64_t i = 0; direct && i < ni; ++i) direct = x_off[i] == b->x_off[i];
  if (e == cudaSuccess && direct) {
    e = cudaMemcpyAsync(x_out, b->d_xout.p, b->xout_len * 8, cudaMemcpyDeviceToHost, s);
  } else if (e == cudaSuccess && x_out && x_off && b->xout_len) {
    xo.resize(b->xout_len);
    e = cudaMemcpyAsync(xo.data(), b->d_xout.p, b->xout_len * 8, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(cuda_msg(e, "batch results"));
  for (int64_t i = 0; i < ni; ++i) {
    if (iters) iters[i] = it[i];
    if (iters_total) iters_total[i] = itt[i];
    if (reason) reason[i] = rs[i];
  }
  if (x_out && x_off && !direct) {
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
  for (int q = 0; q < 8; ++q) out[q] = 0;
  out[2] = (int64_t)b->groups.size();
  out[6] = b->lanes && b->cont_kernel ? (b->lane_cap == 0 ? 1 : 2)
                                       : (int64_t)b->classes.size() + (b->lanes ? 1 : 0);
  out[7] = b->lanes && b->cont_kernel ? 1 : 0;  // the continuation kernel runs
  for (auto& C : b->classes) {  // the largest class (first) describes the launch
    out[0] += C->grid;
    if (out[1] == 0) {
      out[1] = 32 * C->warps_per_block;
      out[3] = ((int64_t)C->region * 8 * C->m + (int64_t)C->prog_ints * 4) * C->warps_per_block;
      out[4] = C->regs;
      out[5] = C->blocks_per_sm;
    }
  }
  return GPUKLU_OK;
}

int gpuklu_batch_work(const gpuklu_batch* b, int64_t* flops, int64_t* bytes) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  for (int64_t i = 0; i < b->ninst; ++i) {
    flops[i] = b->group_flops[b->inst_group_h[i]];
    bytes[i] = b->group_bytes[b->inst_group_h[i]];
  }
  return GPUKLU_OK;
}

void* gpuklu_batch_stream(gpuklu_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"

// ====================================================================== BBD
// Bordered-block-diagonal solver (the reference's BbdSolver with a known
// partition, crates/sim-core/src/bbd_solver.rs): the diagonal blocks as one
// block-diagonal matrix M on an inner handle, the border through the Schur
// complement S = B_T - C M^-1 R, dense on the device.
struct gpuklu_bbd {
  int64_t n = 0;
  std::vector<i64> ap, ai;
  gk::BbdDecomp d;
  bool fallback = false;
  gpuklu_handle* M = nullptr;   // block-diagonal part, or the whole matrix on fallback
  std::vector<i64> m_ap, m_ai;
  std::vector<i32> m_raw;       // M raw entry -> raw entry of the full matrix
  bool tiles_ready = false;
  int ntiles = 0;
  std::vector<i32> perm32;
  DBuf<i32> d_m_raw, d_perm, d_tile_pos0, d_tile_size, d_tile_blk, d_init_ptr, d_init_code,
      d_init_raw, d_bt_ptr, d_bt_row, d_bt_raw, d_yref_ptr, d_yref, d_c_ptr, d_c_row, d_c_pos,
      d_c_raw, d_crow_ptr, d_crow_col, d_crow_raw, d_rrow_ptr, d_rrow_col, d_rrow_raw, d_bperm;
  DBuf<long long> d_tile_off;
  DBuf<double> d_ax, d_rhs, d_rhs_c, d_x, d_newx, d_y, d_S, d_xT, d_z;
  DBuf<gk::NewtonState> d_nstate;
  DBuf<int> d_status;
  DBuf<unsigned> d_bar;  // grid barrier of the cooperative Schur LU
  // Dense LU of S: 0 the 32-wide panel kernels (four launches per panel), 1
  // one cooperative launch with FP64 FMA updates, 2 the same with DMMA
  // updates (GPUKLU_SCHUR_LU=panels|fma|mma).
  int schur_lu = gk::kSchurLuDefault;
  gk::BbdArgs args{};
  std::string err;
  ~gpuklu_bbd() {
    if (M) gpuklu_destroy(M);
  }
  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  cudaStream_t stream() const { return M->stream; }

  // Tile, Schur and product index lists; they depend on M's pivots, so they
  // are built after the first factorization.
  int build_tiles() {
    const gk::Plan& P = M->plan;
    const int nm = d.border_start, bs = d.border_size;
    std::vector<int> in_pos(nm), out_pos(nm);
    for (int r = 0; r < nm; ++r) in_pos[r] = P.in_pos[r];
    for (int c = 0; c < nm; ++c) out_pos[c] = P.out_pos[c];
    const int nb = P.nblocks;
    std::vector<int> pblk(nm);  // plan block of each M index (row or column)
    for (int b = 0; b < nb; ++b)
      for (int q = P.block_ptr[b]; q < P.block_ptr[b + 1]; ++q) pblk[q] = b;
    // R entries by plan block: border column j, M row m, raw q (CSC order)
    std::vector<std::vector<int>> jcols(nb);
    std::vector<std::vector<std::pair<int, int>>> rent(nb);  // (pos offset, raw) per (j)
    std::vector<std::vector<int>> rent_j(nb);
    std::vector<std::vector<i32>> rrow(nm);  // per M row: (j, raw) pairs flattened
    std::vector<i32> bt_ptr(bs + 1, 0), bt_row, bt_raw;
    for (int j = 0; j < bs; ++j) {
      const int oc = d.perm[d.border_start + j];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const int orow = (int)ai[q];
        if (orow >= n) continue;
        const int nr = d.inv_perm[orow];
        if (nr >= d.border_start) {
          bt_row.push_back(nr - d.border_start);
          bt_raw.push_back((i32)q);
        } else {
          const int pos = in_pos[nr], b = pblk[pos];
          if (jcols[b].empty() || jcols[b].back() != j) jcols[b].push_back(j);
          rent[b].push_back({pos - P.block_ptr[b], (int)q});
          rent_j[b].push_back((int)jcols[b].size() - 1);
          rrow[nr].push_back(j);
          rrow[nr].push_back((i32)q);
        }
      }
      bt_ptr[j + 1] = (i32)bt_row.size();
    }
    // tiles of 32 border columns per plan block
    std::vector<i32> tile_pos0, tile_size, tile_blk, init_ptr(1, 0), init_code, init_raw;
    std::vector<long long> tile_off;
    std::vector<std::vector<i32>> yref(bs);
    long long off = 0;
    for (int b = 0; b < nb; ++b) {
      const int ncol = (int)jcols[b].size();
      const int sz = P.block_ptr[b + 1] - P.block_ptr[b];
      const int first_tile = (int)tile_pos0.size();
      for (int t0 = 0; t0 < ncol; t0 += 32) {
        tile_pos0.push_back(P.block_ptr[b]);
        tile_size.push_back(sz);
        tile_blk.push_back(b);
        tile_off.push_back(off);
        off += (long long)sz * 32;
        const int t = (int)tile_pos0.size() - 1;
        for (int l = 0; l < 32 && t0 + l < ncol; ++l) yref[jcols[b][t0 + l]].push_back((t << 5) | l);
      }
      (void)first_tile;
      for (int t0 = 0; t0 < ncol; t0 += 32) {  // each tile's R entries, CSC order
        for (size_t e = 0; e < rent[b].size(); ++e) {
          const int k = rent_j[b][e];
          if (k < t0 || k >= t0 + 32) continue;
          init_code.push_back(rent[b][e].first * 32 + (k - t0));
          init_raw.push_back(rent[b][e].second);
        }
        init_ptr.push_back((i32)init_code.size());
      }
    }
    ntiles = (int)tile_pos0.size();
    // C entries: block columns c with border rows, per plan block and per border row
    std::vector<std::vector<i32>> cb(nb);    // per plan block: (row, pos, raw) triples
    std::vector<std::vector<i32>> crow(bs);  // per border row: (c, raw)
    for (int c = 0; c < nm; ++c) {
      const int oc = d.perm[c];
      const int pos = out_pos[c], b = pblk[pos];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const int orow = (int)ai[q];
        if (orow >= n) continue;
        const int nr = d.inv_perm[orow];
        if (nr < d.border_start) continue;
        const int r = nr - d.border_start;
        cb[b].push_back(r);
        cb[b].push_back(pos - P.block_ptr[b]);
        cb[b].push_back((i32)q);
        crow[r].push_back(c);
        crow[r].push_back((i32)q);
      }
    }
    // Elimination order of S: AMD on its structural pattern (B_T plus, for
    // every block touching column j, the border rows of that block's C), the
    // order the reference's sparse Schur factorisation uses
    // (bbd_solver.rs:330-411 with sparse_lu.rs). It matters: the ground row
    // couples to everything, and eliminated last it keeps the final pivots
    // away from the near-singular constant mode of the conductance matrix.
    std::vector<int> spos(bs), sinv(bs);
    {
      std::vector<std::vector<int>> crows(nb);
      for (int b = 0; b < nb; ++b) {
        std::vector<char> m(bs, 0);
        for (size_t e = 0; e < cb[b].size(); e += 3)
          if (!m[cb[b][e]]) {
            m[cb[b][e]] = 1;
            crows[b].push_back(cb[b][e]);
          }
      }
      std::vector<i64> sap(bs + 1, 0), sai;
      std::vector<int> mark(bs, -1);
      for (int j = 0; j < bs; ++j) {
        std::vector<int> rows;
        for (int e = bt_ptr[j]; e < bt_ptr[j + 1]; ++e)
          if (mark[bt_row[e]] != j) {
            mark[bt_row[e]] = j;
            rows.push_back(bt_row[e]);
          }
        for (i32 code : yref[j]) {
          const int b = tile_blk[code >> 5];
          for (int r : crows[b])
            if (mark[r] != j) {
              mark[r] = j;
              rows.push_back(r);
            }
        }
        std::sort(rows.begin(), rows.end());
        for (int r : rows) sai.push_back(r);
        sap[j + 1] = (i64)sai.size();
      }
      gk::amd_order(bs, sap.data(), sai.data(), spos, sinv);
    }
    for (auto& r : bt_row) r = spos[r];
    std::vector<i32> yref_ptr(bs + 1, 0), yref_flat, bt_ptr_s(bs + 1, 0), bt_row_s, bt_raw_s;
    for (int s2 = 0; s2 < bs; ++s2) {  // S columns in elimination order
      const int j = sinv[s2];
      yref_flat.insert(yref_flat.end(), yref[j].begin(), yref[j].end());
      yref_ptr[s2 + 1] = (i32)yref_flat.size();
      for (int e = bt_ptr[j]; e < bt_ptr[j + 1]; ++e) {
        bt_row_s.push_back(bt_row[e]);
        bt_raw_s.push_back(bt_raw[e]);
      }
      bt_ptr_s[s2 + 1] = (i32)bt_row_s.size();
    }
    bt_ptr.swap(bt_ptr_s);
    bt_row.swap(bt_row_s);
    bt_raw.swap(bt_raw_s);
    std::vector<i32> bperm(bs);
    for (int s2 = 0; s2 < bs; ++s2) bperm[s2] = d.perm[d.border_start + sinv[s2]];
    std::vector<i32> c_ptr(nb + 1, 0), c_row, c_pos, c_raw;
    for (int b = 0; b < nb; ++b) {
      for (size_t e = 0; e < cb[b].size(); e += 3) {
        c_row.push_back(spos[cb[b][e]]);
        c_pos.push_back(cb[b][e + 1]);
        c_raw.push_back(cb[b][e + 2]);
      }
      c_ptr[b + 1] = (i32)c_row.size();
    }
    std::vector<i32> crow_ptr(bs + 1, 0), crow_col, crow_raw;
    for (int s2 = 0; s2 < bs; ++s2) {  // border rows in S order
      const int r = sinv[s2];
      for (size_t e = 0; e < crow[r].size(); e += 2) {
        crow_col.push_back(crow[r][e]);
        crow_raw.push_back(crow[r][e + 1]);
      }
      crow_ptr[s2 + 1] = (i32)crow_col.size();
    }
    std::vector<i32> rrow_ptr(nm + 1, 0), rrow_col, rrow_raw;
    for (int m = 0; m < nm; ++m) {
      for (size_t e = 0; e < rrow[m].size(); e += 2) {
        rrow_col.push_back(spos[rrow[m][e]]);
        rrow_raw.push_back(rrow[m][e + 1]);
      }
      rrow_ptr[m + 1] = (i32)rrow_col.size();
    }
    cudaStream_t s = stream();
    cudaError_t e = cudaSuccess;
#define UP(buf, vec) \
  if (e == cudaSuccess) e = buf.upload(vec, s);
    UP(d_tile_pos0, tile_pos0) UP(d_tile_size, tile_size) UP(d_tile_blk, tile_blk)
    UP(d_tile_off, tile_off) UP(d_init_ptr, init_ptr) UP(d_init_code, init_code)
    UP(d_init_raw, init_raw) UP(d_bt_ptr, bt_ptr) UP(d_bt_row, bt_row) UP(d_bt_raw, bt_raw)
    UP(d_yref_ptr, yref_ptr) UP(d_yref, yref_flat) UP(d_c_ptr, c_ptr) UP(d_c_row, c_row)
    UP(d_c_pos, c_pos) UP(d_c_raw, c_raw) UP(d_crow_ptr, crow_ptr) UP(d_crow_col, crow_col)
    UP(d_crow_raw, crow_raw) UP(d_rrow_ptr, rrow_ptr) UP(d_rrow_col, rrow_col)
    UP(d_rrow_raw, rrow_raw) UP(d_bperm, bperm)
#undef UP
    if (e == cudaSuccess) e = d_y.resize(std::max<long long>(off, 1));
    if (e == cudaSuccess) e = d_S.resize(std::max<size_t>((size_t)bs * bs, 1));
    if (e == cudaSuccess) e = d_xT.resize(std::max(bs, 1));
    if (e == cudaSuccess) e = d_z.resize(std::max(nm, 1));
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd tiles"));
    gk::BbdArgs& a = args;
    a.ntiles = ntiles;
    a.bs = bs;
    a.border_start = d.border_start;
    a.tile_pos0 = d_tile_pos0.p;
    a.tile_size = d_tile_size.p;
    a.tile_off = d_tile_off.p;
    a.tile_blk = d_tile_blk.p;
    a.init_ptr = d_init_ptr.p;
    a.init_code = d_init_code.p;
    a.init_raw = d_init_raw.p;
    a.bt_ptr = d_bt_ptr.p;
    a.bt_row = d_bt_row.p;
    a.bt_raw = d_bt_raw.p;
    a.yref_ptr = d_yref_ptr.p;
    a.yref = d_yref.p;
    a.c_ptr = d_c_ptr.p;
    a.c_row = d_c_row.p;
    a.c_pos = d_c_pos.p;
    a.c_raw = d_c_raw.p;
    a.crow_ptr = d_crow_ptr.p;
    a.crow_col = d_crow_col.p;
    a.crow_raw = d_crow_raw.p;
    a.rrow_ptr = d_rrow_ptr.p;
    a.rrow_col = d_rrow_col.p;
    a.rrow_raw = d_rrow_raw.p;
    a.perm = d_perm.p;
    a.bperm = d_bperm.p;
    tiles_ready = true;
    return GPUKLU_OK;
  }

  // Factor with the full matrix's values in d_ax.
  int factor_device(bool sync) {
    cudaStream_t s = stream();
    if (fallback) {
      cudaError_t e = cudaMemcpyAsync(M->d_ax.p, d_ax.p, ai.size() * 8, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd factor"));
      const bool first = M->state != gpuklu_handle::FACTORED;
      int st = M->factor_on_device(sync || first);
      if (st) return fail(st, M->err);
      return GPUKLU_OK;
    }
    gk::launch_gather(M->d_ax.p, d_ax.p, d_m_raw.p, (int)m_raw.size(), s);
    const bool first = M->state != gpuklu_handle::FACTORED;
    int st = M->factor_on_device(sync || first);
    if (st) return fail(st, M->err);
    if (!tiles_ready) {
      st = build_tiles();
      if (st) return st;
    }
    gk::launch_bbd_ysolve(M->pd.dp, M->d_lu.p, d_ax.p, args, d_y.p, s);
    gk::launch_bbd_schur(d_ax.p, args, d_y.p, d_S.p, s);
    cudaError_t e = cudaSuccess;
    if (schur_lu == 0) {
      gk::launch_dense_lu(d_S.p, d.border_size, s);
    } else {
      e = d_bar.resize(gk::schur_lu_bar_words(d.border_size));
      if (e == cudaSuccess)
        e = gk::launch_schur_lu(d_S.p, d.border_size, schur_lu == 2, d_bar.p, M->d_status.p, s);
      if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "schur lu"));
    }
    e = cudaGetLastError();
    if (e == cudaSuccess && sync) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd factor"));
    if (sync) {
      st = M->check_status("bbd factor");
      if (st) return fail(st, M->err);
    }
    return GPUKLU_OK;
  }

  // x = A^-1 rhs, both full-length device arrays (original order).
  int solve_device(const double* rhs, double* x) {
    cudaStream_t s = stream();
    if (fallback) {
      cudaError_t e = cudaMemcpyAsync(M->d_rhs.p, rhs, n * 8, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd solve"));
      int st = M->solve_on_device(false, false);
      if (st) return fail(st, M->err);
      e = cudaMemcpyAsync(x, M->d_out.p, n * 8, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd solve"));
      return GPUKLU_OK;
    }
    const int nm = d.border_start;
    gk::launch_gather(M->d_rhs.p, rhs, d_perm.p, nm, s);  // block rows
    int st = M->solve_on_device(false, false);
    if (st) return fail(st, M->err);
    cudaMemcpyAsync(d_z.p, M->d_out.p, (size_t)nm * 8, cudaMemcpyDeviceToDevice, s);
    gk::launch_bbd_border_rhs(d_ax.p, rhs, d_z.p, args, d_xT.p, s);
    gk::launch_dense_lu_solve(d_S.p, d.border_size, d_xT.p, s);
    gk::launch_bbd_rmatvec(d_ax.p, d_xT.p, args, M->d_rhs.p, s);
    st = M->solve_on_device(false, false);
    if (st) return fail(st, M->err);
    gk::launch_bbd_combine(d_z.p, M->d_out.p, d_xT.p, args, x, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd solve"));
    return GPUKLU_OK;
  }
};

extern "C" {

gpuklu_bbd* gpuklu_bbd_create(int64_t n, const int64_t* ap, int64_t ap_len, const int64_t* ai,
                              int64_t ai_len, const int64_t* assignment, int64_t num_blocks) {
  if (n <= 0 || ap_len != n + 1 || ap[n] != ai_len || !assignment) {
    fprintf(stderr, "gpuklu_bbd_create: invalid pattern\n");
    return nullptr;
  }
  auto B = std::make_unique<gpuklu_bbd>();
  B->n = n;
  B->ap.assign(ap, ap + ap_len);
  B->ai.assign(ai, ai + ai_len);
  B->d = gk::bbd_decompose((int)n, ap, ai, assignment, (int)num_blocks);
  const gk::BbdDecomp& d = B->d;
  const double ratio = (double)d.border_size / (double)n;
  B->fallback = d.num_blocks <= 1 || d.border_size == 0 || ratio > 0.5;  // bbd_solver.rs:418-431
  if (!B->fallback && d.border_size > 16384) {
    fprintf(stderr, "gpuklu_bbd_create: border of %d is above the dense limit 16384\n",
            d.border_size);
    return nullptr;
  }
  B->M = gpuklu_create(B->fallback ? n : d.border_start);
  if (!B->M) return nullptr;
  if (const char* es = getenv("GPUKLU_SCHUR_LU"))
    B->schur_lu = strcmp(es, "panels") == 0 ? 0 : strcmp(es, "mma") == 0 ? 2 : 1;
  gpuklu_set_pivot_mode(B->M, GPUKLU_PIVOT_EXACT);
  if (!B->fallback) {  // SparseLU per block (bbd_solver.rs:436-444): AMD, no row exchanges
    gpuklu_set_pivot_mode(B->M, GPUKLU_PIVOT_REFERENCE);
    B->M->given_blocks = d.block_ptr;
    B->M->no_swap = true;
  }
  int st;
  if (B->fallback) {
    st = gpuklu_analyze(B->M, ap, ap_len, ai, ai_len);
  } else {
    const int nm = d.border_start;
    B->m_ap.assign(nm + 1, 0);
    for (int c = 0; c < nm; ++c) {
      const int oc = d.perm[c];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const int orow = (int)ai[q];
        if (orow >= n) continue;
        const int nr = d.inv_perm[orow];
        if (nr < nm && d.block_of[nr] == d.block_of[c]) {
          B->m_ai.push_back(nr);
          B->m_raw.push_back((i32)q);
        }
      }
      B->m_ap[c + 1] = (i64)B->m_ai.size();
    }
    st = gpuklu_analyze(B->M, B->m_ap.data(), (int64_t)B->m_ap.size(), B->m_ai.data(),
                        (int64_t)B->m_ai.size());
  }
  if (st != GPUKLU_OK) {
    fprintf(stderr, "gpuklu_bbd_create: %s\n", B->M->err.c_str());
    return nullptr;
  }
  cudaStream_t s = B->stream();
  B->perm32.assign(d.perm.begin(), d.perm.end());
  cudaError_t e = B->d_m_raw.upload(B->m_raw, s);
  if (e == cudaSuccess) e = B->d_perm.upload(B->perm32, s);
  if (e == cudaSuccess) e = B->d_ax.resize(std::max<int64_t>(ai_len, 1));
  for (auto* b : {&B->d_rhs, &B->d_x, &B->d_newx})
    if (e == cudaSuccess) e = b->resize(n);
  if (e == cudaSuccess) e = B->d_nstate.resize(1);
  if (e == cudaSuccess) e = B->d_status.resize(1);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->d_status.p, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_bbd_create: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  return B.release();
}

void gpuklu_bbd_destroy(gpuklu_bbd* b) { delete b; }

const char* gpuklu_bbd_last_error(const gpuklu_bbd* b) { return b ? b->err.c_str() : ""; }

int gpuklu_bbd_info(const gpuklu_bbd* b, int64_t* out) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  out[0] = b->d.num_blocks;
  out[1] = b->d.border_start;
  out[2] = b->d.border_size;
  out[3] = b->fallback ? 1 : 0;
  out[4] = b->ntiles;
  out[5] = b->M ? b->M->cur_plan().nblocks : 0;
  return GPUKLU_OK;
}

int gpuklu_bbd_perm(const gpuklu_bbd* b, int64_t* perm) {
  if (!b) return GPUKLU_INVALID_MATRIX;
  for (int64_t i = 0; i < b->n; ++i) perm[i] = b->d.perm[i];
  return GPUKLU_OK;
}

int gpuklu_bbd_factor(gpuklu_bbd* b, const double* ax) {
  if (!b || !ax) return GPUKLU_INVALID_MATRIX;
  cudaError_t e = cudaMemcpyAsync(b->d_ax.p, ax, b->ai.size() * 8, cudaMemcpyHostToDevice,
                                  b->stream());
  if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd factor"));
  return b->factor_device(true);
}

int gpuklu_bbd_solve(gpuklu_bbd* b, double* rhs, int64_t len) {
  if (!b || !rhs || len != b->n) return GPUKLU_INVALID_MATRIX;
  if (!b->fallback && !b->tiles_ready) return b->fail(GPUKLU_SOLVE_FAILED, "solve before factor");
  cudaStream_t s = b->stream();
  cudaError_t e = cudaMemcpyAsync(b->d_rhs.p, rhs, len * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd solve"));
  int st = b->solve_device(b->d_rhs.p, b->d_x.p);
  if (st) return st;
  e = cudaMemcpyAsync(rhs, b->d_x.p, len * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd solve"));
  int stt = b->M->check_status("bbd solve");
  return stt ? b->fail(stt, b->M->err) : GPUKLU_OK;
}

int gpuklu_bbd_newton_dc(gpuklu_bbd* b, gpuklu_circuit* c, const gpuklu_newton_config* cfg,
                         const double* x0, double* x_out, int64_t x_cap, int64_t* x_len,
                         int64_t* iters, int64_t* iters_total, int* reason) {
  if (!b || !c || !cfg) return GPUKLU_INVALID_MATRIX;
  if (c->n != b->n || c->ap != b->ap || c->ai != b->ai)
    return b->fail(GPUKLU_INVALID_MATRIX, "the circuit's pattern differs from the solver's");
  cudaStream_t s = b->stream();
  const int nc = c->node_count, n = c->n;
  cudaError_t e = b->d_rhs_c.resize(std::max(c->ncontrib, 1));
  std::vector<double> xinit(n, 0.0);
  if (x0) std::copy(x0, x0 + nc, xinit.begin());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_newx.p, xinit.data(), n * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd newton"));
  const gk::NewtonCfg ncfg = to_newton_cfg(*cfg);
  const double gstart = std::max(cfg->gmin * 1e3, 1e-6);
  int64_t total = 0, last = 0;
  int rsn = 1;
  bool conv = false, failed = false;
  for (int64_t gi = 0; gi <= cfg->gmin_steps && !conv && !failed; ++gi) {
    const double gmin = cfg->gmin_steps == 0
                            ? cfg->gmin
                            : gstart + (cfg->gmin - gstart) * ((double)gi / (double)cfg->gmin_steps);
    for (int64_t si = 0; si <= cfg->source_steps && !conv && !failed; ++si) {
      const double scale = cfg->source_steps == 0 ? 1.0 : (double)si / (double)cfg->source_steps;
      gk::NewtonState ns{cfg->damping, DBL_MAX, 0.0, 0, 0};
      e = cudaMemcpyAsync(b->d_nstate.p, &ns, sizeof(ns), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd newton"));
      int64_t it = 0;
      rsn = 1;
      for (; it < cfg->max_iters; ++it) {
        gk::launch_stamp(c->dc, b->d_newx.p, nc, gmin, scale, 0.0, nullptr, -1.0, b->d_ax.p,
                         b->d_rhs_c.p, b->d_rhs.p, s);
        int st = b->factor_device(false);
        if (st == GPUKLU_OK) st = b->solve_device(b->d_rhs.p, b->d_x.p);
        if (st != GPUKLU_OK) {
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        gk::launch_newton_update(nc, n, b->d_newx.p, b->d_x.p, b->d_nstate.p, ncfg,
                                 b->d_status.p, s);
        gk::NewtonState hs;
        e = cudaMemcpyAsync(&hs, b->d_nstate.p, sizeof(hs), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd newton"));
        st = b->M->check_status("bbd iteration");
        if (st) {
          rsn = 2;
          failed = true;
          ++it;
          break;
        }
        if (hs.converged) {
          conv = true;
          rsn = 0;
          ++it;
          break;
        }
      }
      total += it;
      last = it;
    }
  }
  const int64_t len = conv ? n : nc;
  std::vector<double> xh(n);
  e = cudaMemcpyAsync(xh.data(), b->d_newx.p, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return b->fail(GPUKLU_CUDA_ERROR, cuda_msg(e, "bbd newton"));
  for (int64_t i = 0; i < std::min(len, x_cap); ++i) x_out[i] = xh[i];
  if (x_len) *x_len = len;
  if (iters) *iters = last;
  if (iters_total) *iters_total = total;
  if (reason) *reason = rsn;
  return GPUKLU_OK;
}

}  // extern "C"

// ====================================================================== no-allocation solve
// Some callers cannot call cudaMalloc at the point where they solve: a
// simulator step inside a host callback where allocation is not allowed, a
// real-time loop with a fixed device-memory budget, or a foreign runtime that
// owns all device memory and only lends buffers.
// gpuklu_solve_device_noalloc serves them: the caller passes device buffers
// for the right-hand side and the solution, and the solve kernel's scratch
// (the forward and backward vectors, the per-row completion flags and the
// task counter) lives in the file-scope array below instead of the handle's
// buffers. Every GPU that loads the library holds this array until the
// process exits. The call ends by reading the kernel's status back and
// synchronising the handle's stream.
namespace {
constexpr size_t kNoallocFlagBytes = 256 + 2 * (size_t)GPUKLU_NOALLOC_MAX_N * sizeof(unsigned);
constexpr size_t kNoallocBytes = kNoallocFlagBytes + 2 * (size_t)GPUKLU_NOALLOC_MAX_N * sizeof(double);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Device address of g_noalloc_scratch per device, looked up once with that
// device current. In host code the array's name is only a host-side handle.
unsigned char* g_noalloc_addr[64] = {nullptr};
std::mutex g_noalloc_mu;

cudaError_t noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}
}  // namespace

extern "C" int gpuklu_solve_device_noalloc(gpuklu_handle* h, const double* d_rhs, double* d_x) {
  if (!h || h->state != gpuklu_handle::FACTORED) return GPUKLU_SOLVE_FAILED;
  if (h->kind == GPUKLU_KIND_DENSE)
    return h->fail(GPUKLU_SOLVE_FAILED, "gpuklu_solve_device_noalloc: not for the dense solver");
  if (h->n > GPUKLU_NOALLOC_MAX_N)
    return h->fail(GPUKLU_INVALID_MATRIX,
                   "gpuklu_solve_device_noalloc: n = " + std::to_string(h->n) +
                       " exceeds GPUKLU_NOALLOC_MAX_N = " +
                       std::to_string(GPUKLU_NOALLOC_MAX_N));
  if (h->cta_sol) {  // the one-block solve keeps its vectors in shared memory
    gk::launch_solve_cta(h->pd.dp, d_rhs, h->d_ax.p, h->d_lu.p, d_x, h->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "noalloc solve launch");
    return h->check_status("solve_device_noalloc");
  }
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_scratch(&base);
  if (e != cudaSuccess) return h->cuda_fail(e, "noalloc scratch address");
  const size_t n = (size_t)h->n;
  unsigned* counter = reinterpret_cast<unsigned*>(base);
  unsigned* zflag = reinterpret_cast<unsigned*>(base + 256);
  unsigned* xflag = zflag + GPUKLU_NOALLOC_MAX_N;
  double* z = reinterpret_cast<double*>(base + kNoallocFlagBytes);
  double* x = z + GPUKLU_NOALLOC_MAX_N;
  // the array keeps the previous call's flags: clear this call's rows
  e = cudaMemsetAsync(zflag, 0, n * sizeof(unsigned), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(xflag, 0, n * sizeof(unsigned), h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "noalloc flags");
  const int grid = std::max(1, std::min<int>((int)((2 * n + 3) / 4), sm_count() * 16));
  gk::launch_solve(h->pd.dp, d_rhs, h->d_ax.p, h->d_lu.p, z, x, d_x, zflag, xflag, 1u, counter,
                   h->d_status.p, grid, false, h->stream);
  e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "noalloc solve launch");
  return h->check_status("solve_device_noalloc");
}

// ====================================================================== diagnostics
struct gpuklu_plan {
  gk::Plan p;
  std::vector<int64_t> info;
};

extern "C" {

double gpuklu_fp64_peak_tflops(void) { return gk::fp64_peak_tflops(); }

double gpuklu_fp64_mma_peak_tflops(void) { return gk::dmma_peak_tflops(); }

int gpuklu_dense_lu_nopivot(double* a, int64_t n, int variant, double* ms_out) {
  if (!a || n <= 0 || n > 16384 || variant < 0 || variant > 2) return GPUKLU_INVALID_MATRIX;
  const size_t bytes = (size_t)n * n * sizeof(double);
  DBuf<double> dS;
  DBuf<unsigned> bar;
  DBuf<int> status;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = dS.resize((size_t)n * n);
  if (e == cudaSuccess) e = bar.resize(gk::schur_lu_bar_words((int)n));
  if (e == cudaSuccess) e = status.resize(1);
  if (e == cudaSuccess) e = cudaMemsetAsync(status.p, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dS.p, a, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaEventRecord(e0, s);
  if (e == cudaSuccess) {
    if (variant == 0)
      gk::launch_dense_lu(dS.p, (int)n, s);
    else
      e = gk::launch_schur_lu(dS.p, (int)n, variant == 2, bar.p, status.p, s);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  int st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(a, dS.p, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  float ms = 0.f;
  if (e == cudaSuccess && ms_out) e = cudaEventElapsedTime(&ms, e0, e1);
  if (ms_out) *ms_out = ms;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "gpuklu_dense_lu_nopivot: %s\n", cudaGetErrorString(e));
    return GPUKLU_CUDA_ERROR;
  }
  return st == 0 ? GPUKLU_OK : st;
}

int gpuklu_btf_info(int64_t n, const int64_t* ap, const int64_t* ai, int64_t* out) {
  if (n < 0 || !out || (n > 0 && (!ap || !ai))) return GPUKLU_INVALID_MATRIX;
  if (n == 0) {
    out[0] = out[1] = 0;
    return GPUKLU_OK;
  }
  const gk::BtfResult b = gk::btf_decompose((int)n, ap, ai);
  out[0] = b.nblocks;
  out[1] = b.max_block;
  return GPUKLU_OK;
}

int64_t gpuklu_plan_steps(const gpuklu_plan* p, int32_t nc, int32_t ndv, int32_t* ops,
                          int64_t ops_cap, int32_t* step_ptr, int64_t steps_cap) {
  if (!p || nc < 0 || ndv < 0) return -1;
  std::vector<i32> o, sp;
  build_steps(p->p, nc, ndv, o, sp);
  if (ops && (int64_t)o.size() <= ops_cap) std::copy(o.begin(), o.end(), ops);
  if (step_ptr && (int64_t)sp.size() <= steps_cap) std::copy(sp.begin(), sp.end(), step_ptr);
  return (int64_t)(o.size() / 2) * ((int64_t)1 << 32) + (int64_t)sp.size();
}

int64_t gpuklu_plan_solve_steps(const gpuklu_plan* p, int32_t* ops, int64_t ops_cap,
                                int32_t* step_ptr, int64_t steps_cap) {
  if (!p) return -1;
  std::vector<int4> o;
  std::vector<i32> sp;
  make_solve_steps(p->p, o, sp);
  if (ops && (int64_t)o.size() * 4 <= ops_cap)
    for (size_t q = 0; q < o.size(); ++q) {
      ops[4 * q] = o[q].x;
      ops[4 * q + 1] = o[q].y;
      ops[4 * q + 2] = o[q].z;
      ops[4 * q + 3] = o[q].w;
    }
  if (step_ptr && (int64_t)sp.size() <= steps_cap) std::copy(sp.begin(), sp.end(), step_ptr);
  return (int64_t)o.size() * ((int64_t)1 << 32) + (int64_t)sp.size();
}

gpuklu_plan* gpuklu_plan_build(int64_t n, const int64_t* ap, const int64_t* ai, int pivot_mode,
                               int kind, const int32_t* row_perm) {
  auto P = std::make_unique<gpuklu_plan>();
  std::string m = gk::analyze((int)n, ap, ai, pivot_mode, P->p, nullptr, kind);
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
  if (k == "cs_grp" || k == "cs_gchunk" || k == "cs_gop") {  // its grouped form
    std::vector<i32> hg, hc, ho;  // grouped for 152 SMs (the device path asks the device)
    make_cta_groups(p, 152, hg, hc, ho);
    return put(k == "cs_grp" ? hg : (k == "cs_gchunk" ? hc : ho));
  }
  if (k == "cs_chunk" || k == "cs_op") {  // the one-block solve's schedule
    std::vector<i32> hc, ho;
    make_cta_solve(p, hc, ho);
    return put(k == "cs_chunk" ? hc : ho);
  }
  if (k == "task" || k == "ttask") return put(make_tasks(p, k == "ttask"));  // grid solve order
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
