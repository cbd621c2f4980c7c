// BBD decomposition and BbdSolver, restated from crates/sim-core/src/bbd.rs
// and crates/sim-core/src/bbd_solver.rs (test infrastructure; see oracle.h).
#include <algorithm>
#include <cmath>

#include "oracle.h"

namespace oracle {

BbdDecomposition bbd_decompose_known(size_t n, const i64* ap, const i64* ai,
                                     const std::vector<int64_t>& assignment,
                                     size_t num_blocks) {
  const size_t kBorder = (size_t)-1;
  std::vector<size_t> asg(n);
  for (size_t i = 0; i < n; ++i) asg[i] = assignment[i] < 0 ? kBorder : (size_t)assignment[i];
  // bbd.rs:366-385: a column touching another block's row becomes border
  for (size_t col = 0; col < n; ++col) {
    if (asg[col] == kBorder) continue;
    const size_t mine = asg[col];
    for (i64 q = ap[col]; q < ap[col + 1]; ++q) {
      const size_t row = (size_t)ai[q];
      if (row < n && row != col) {
        const size_t rb = asg[row];
        if (rb != kBorder && rb != mine) {
          asg[col] = kBorder;
          break;
        }
      }
    }
  }
  // bbd.rs:391-407: the row direction
  for (size_t col = 0; col < n; ++col)
    for (i64 q = ap[col]; q < ap[col + 1]; ++q) {
      const size_t row = (size_t)ai[q];
      if (row < n && row != col) {
        if (asg[row] == kBorder) continue;
        const size_t rb = asg[row], cb = asg[col];
        if (cb != kBorder && cb != rb) asg[row] = kBorder;
      }
    }
  std::vector<UVec> blocks(num_blocks);
  UVec border;
  for (size_t i = 0; i < n; ++i) {
    if (asg[i] == kBorder)
      border.push_back(i);
    else
      blocks[asg[i]].push_back(i);
  }
  std::vector<UVec> ne;
  for (auto& b : blocks)
    if (!b.empty()) ne.push_back(b);
  BbdDecomposition d;
  if (ne.size() <= 1) {  // bbd.rs:427-451
    UVec all;
    if (ne.size() == 1) {
      all = ne[0];
      all.insert(all.end(), border.begin(), border.end());
    } else {
      for (size_t i = 0; i < n; ++i) all.push_back(i);
    }
    d.num_blocks = 1;
    d.perm = all;
    d.inv_perm.assign(n, 0);
    for (size_t k = 0; k < n; ++k) d.inv_perm[all[k]] = k;
    d.block_ptr = {0, n};
    d.border_start = n;
    d.border_size = 0;
    return d;
  }
  for (auto& b : ne) {
    d.block_ptr.push_back(d.perm.size());
    d.perm.insert(d.perm.end(), b.begin(), b.end());
  }
  d.block_ptr.push_back(d.perm.size());
  d.border_start = d.perm.size();
  d.perm.insert(d.perm.end(), border.begin(), border.end());
  d.inv_perm.assign(n, 0);
  for (size_t k = 0; k < n; ++k) d.inv_perm[d.perm[k]] = k;
  d.num_blocks = ne.size();
  d.border_size = n - d.border_start;
  return d;
}

BbdSolver::BbdSolver(size_t n, std::vector<int64_t> assignment, size_t num_blocks)
    : n_(n), assign_(std::move(assignment)), nblk_target_(num_blocks) {}

void BbdSolver::prepare(size_t n) {
  if (n != n_) {
    n_ = n;
    reset_pattern();
  }
}

void BbdSolver::reset_pattern() {
  analyzed_ = factored_ = have_dec_ = false;
  last_ap_.clear();
  last_ai_.clear();
  fallback_.reset();
}

int BbdSolver::analyze(const IVec& ap, const IVec& ai) {
  if (analyzed_ && ap == last_ap_ && ai == last_ai_) return ST_OK;
  if (ap.size() != n_ + 1) return ST_INVALID_MATRIX;
  int st = analyze_bbd(ap, ai);
  if (st != ST_OK) return st;
  last_ap_ = ap;
  last_ai_ = ai;
  analyzed_ = true;
  factored_ = false;
  return ST_OK;
}

// bbd_solver.rs:412-500 (analyze_bbd) and :506-627 (extract_block_patterns)
int BbdSolver::analyze_bbd(const IVec& ap, const IVec& ai) {
  const size_t n = n_;
  fallback_.reset();
  if (assign_.size() != n) return ST_INVALID_MATRIX;
  dec_ = bbd_decompose_known(n, ap.data(), ai.data(), assign_, nblk_target_);
  have_dec_ = true;
  const double ratio = (double)dec_.border_size / (double)n;
  if (dec_.num_blocks <= 1 || dec_.border_size == 0 || ratio > 0.5) {
    fallback_ = std::make_unique<SparseLuSolver>(n);
    fallback_->prepare(n);
    return fallback_->analyze(ap, ai);
  }
  const BbdDecomposition& d = dec_;
  const size_t bs = d.border_size;
  blocks_.clear();
  size_t maxb = 0;
  for (size_t k = 0; k < d.num_blocks; ++k) {
    const size_t sz = d.block_ptr[k + 1] - d.block_ptr[k];
    maxb = std::max(maxb, sz);
    blocks_.emplace_back(sz);
    blocks_.back().prepare(sz);
  }
  block_work_.assign(maxb, 0.0);
  c_.assign(d.num_blocks, Sparse());
  r_.assign(d.num_blocks, Sparse());
  for (size_t k = 0; k < d.num_blocks; ++k) {
    const size_t b0 = d.block_ptr[k], b1 = d.block_ptr[k + 1], sz = b1 - b0;
    IVec bap(sz + 1, 0), bai;
    Sparse& C = c_[k];
    C.nrows = bs;
    C.ncols = sz;
    C.col_ptr.assign(sz + 1, 0);
    for (size_t lc = 0; lc < sz; ++lc) {
      const size_t oc = d.perm[b0 + lc];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= b0 && nr < b1) bai.push_back((i64)(nr - b0));
        if (nr >= d.border_start) C.row_idx.push_back(nr - d.border_start);
      }
      bap[lc + 1] = (i64)bai.size();
      C.col_ptr[lc + 1] = C.row_idx.size();
    }
    int st = blocks_[k].analyze(bap, bai);
    if (st != ST_OK) return st;
    Sparse& R = r_[k];
    R.nrows = sz;
    R.ncols = bs;
    R.col_ptr.assign(bs + 1, 0);
    for (size_t lc = 0; lc < bs; ++lc) {
      const size_t oc = d.perm[d.border_start + lc];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= b0 && nr < b1) R.row_idx.push_back(nr - b0);
      }
      R.col_ptr[lc + 1] = R.row_idx.size();
    }
  }
  dense_schur_ = bs <= 64;
  if (dense_schur_) {
    bt_dense_.assign(bs * bs, 0.0);
    schur_dense_.assign(bs * bs, 0.0);
    schur_lu_.assign(bs * bs, 0.0);
    schur_piv_.assign(bs, 0);
    schur_sparse_.reset();
  } else {  // compute_schur_pattern, bbd_solver.rs:330-411
    std::vector<std::vector<char>> crow(d.num_blocks, std::vector<char>(bs, 0)),
        rcol(d.num_blocks, std::vector<char>(bs, 0));
    for (size_t k = 0; k < d.num_blocks; ++k) {
      for (size_t r : c_[k].row_idx) crow[k][r] = 1;
      for (size_t j = 0; j < bs; ++j)
        if (r_[k].col_ptr[j] < r_[k].col_ptr[j + 1]) rcol[k][j] = 1;
    }
    schur_ap_.assign(bs + 1, 0);
    schur_ai_.clear();
    std::vector<char> mark(bs);
    for (size_t j = 0; j < bs; ++j) {
      std::fill(mark.begin(), mark.end(), 0);
      const size_t oc = d.perm[d.border_start + j];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= d.border_start) mark[nr - d.border_start] = 1;
      }
      for (size_t k = 0; k < d.num_blocks; ++k)
        if (rcol[k][j])
          for (size_t i = 0; i < bs; ++i)
            if (crow[k][i]) mark[i] = 1;
      for (size_t i = 0; i < bs; ++i)
        if (mark[i]) schur_ai_.push_back((i64)i);
      schur_ap_[j + 1] = (i64)schur_ai_.size();
    }
    schur_ax_.assign(schur_ai_.size(), 0.0);
    schur_sparse_ = std::make_unique<SparseLuSolver>(bs);
    schur_sparse_->prepare(bs);
    int st = schur_sparse_->analyze(schur_ap_, schur_ai_);
    if (st != ST_OK) return st;
  }
  return ST_OK;
}

int BbdSolver::factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  int st = analyze(ap, ai);
  if (st != ST_OK) return st;
  st = fallback_ ? fallback_->factor(ap, ai, ax) : factor_bbd(ap, ai, ax);
  factored_ = st == ST_OK;
  return st;
}

// bbd_solver.rs:633-903
int BbdSolver::factor_bbd(const IVec& ap, const IVec& ai, const Vec& ax) {
  const BbdDecomposition& d = dec_;
  const size_t n = n_, bs = d.border_size;
  for (size_t k = 0; k < d.num_blocks; ++k) {
    const size_t b0 = d.block_ptr[k], b1 = d.block_ptr[k + 1], sz = b1 - b0;
    IVec bap(sz + 1, 0), bai;
    Vec bax;
    Sparse& C = c_[k];
    C.values.clear();
    for (size_t lc = 0; lc < sz; ++lc) {
      const size_t oc = d.perm[b0 + lc];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= b0 && nr < b1) {
          bai.push_back((i64)(nr - b0));
          bax.push_back(ax[q]);
        }
        if (nr >= d.border_start) C.values.push_back(ax[q]);
      }
      bap[lc + 1] = (i64)bai.size();
    }
    int st = blocks_[k].factor(bap, bai, bax);
    if (st != ST_OK) return st;
    Sparse& R = r_[k];
    R.values.clear();
    for (size_t lc = 0; lc < bs; ++lc) {
      const size_t oc = d.perm[d.border_start + lc];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= b0 && nr < b1) R.values.push_back(ax[q]);
      }
    }
  }
  // S = B_T - sum_k C_k B_k^-1 R_k, one column of R_k at a time
  auto for_each_update = [&](auto&& sub) -> int {
    for (size_t k = 0; k < d.num_blocks; ++k) {
      const size_t sz = d.block_ptr[k + 1] - d.block_ptr[k];
      for (size_t j = 0; j < bs; ++j) {
        const size_t r0 = r_[k].col_ptr[j], r1 = r_[k].col_ptr[j + 1];
        if (r0 == r1) continue;
        Vec w(sz, 0.0);
        for (size_t q = r0; q < r1; ++q) w[r_[k].row_idx[q]] = r_[k].values[q];
        int st = blocks_[k].solve(w);
        if (st != ST_OK) return st;
        for (size_t col = 0; col < sz; ++col) {
          const double y = w[col];
          if (y == 0.0) continue;
          for (size_t q = c_[k].col_ptr[col]; q < c_[k].col_ptr[col + 1]; ++q)
            sub(c_[k].row_idx[q], j, c_[k].values[q] * y);
        }
      }
    }
    return ST_OK;
  };
  if (dense_schur_) {
    std::fill(bt_dense_.begin(), bt_dense_.end(), 0.0);
    for (size_t lc = 0; lc < bs; ++lc) {
      const size_t oc = d.perm[d.border_start + lc];
      for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
        const size_t orow = (size_t)ai[q];
        if (orow >= n) continue;
        const size_t nr = d.inv_perm[orow];
        if (nr >= d.border_start) bt_dense_[(nr - d.border_start) * bs + lc] += ax[q];
      }
    }
    schur_dense_ = bt_dense_;
    int st = for_each_update(
        [&](size_t r, size_t j, double v) { schur_dense_[r * bs + j] -= v; });
    if (st != ST_OK) return st;
    // DenseSchurSolver::factor, bbd_solver.rs:115-160
    schur_lu_ = schur_dense_;
    for (size_t k = 0; k < bs; ++k) schur_piv_[k] = k;
    for (size_t k = 0; k < bs; ++k) {
      size_t p = k;
      double mx = std::fabs(schur_lu_[k * bs + k]);
      for (size_t i = k + 1; i < bs; ++i)
        if (std::fabs(schur_lu_[i * bs + k]) > mx) {
          mx = std::fabs(schur_lu_[i * bs + k]);
          p = i;
        }
      if (mx < 1e-30) return ST_SINGULAR;
      if (p != k) {
        for (size_t j = 0; j < bs; ++j) std::swap(schur_lu_[k * bs + j], schur_lu_[p * bs + j]);
        std::swap(schur_piv_[k], schur_piv_[p]);
      }
      const double pv = schur_lu_[k * bs + k];
      for (size_t i = k + 1; i < bs; ++i) {
        const double f = schur_lu_[i * bs + k] / pv;
        schur_lu_[i * bs + k] = f;
        for (size_t j = k + 1; j < bs; ++j) schur_lu_[i * bs + j] -= f * schur_lu_[k * bs + j];
      }
    }
    return ST_OK;
  }
  std::fill(schur_ax_.begin(), schur_ax_.end(), 0.0);
  auto spos = [&](size_t r, size_t j) -> i64 {
    auto b = schur_ai_.begin() + schur_ap_[j], e = schur_ai_.begin() + schur_ap_[j + 1];
    auto it = std::lower_bound(b, e, (i64)r);
    return (it != e && *it == (i64)r) ? (i64)(it - schur_ai_.begin()) : -1;
  };
  for (size_t lc = 0; lc < bs; ++lc) {
    const size_t oc = d.perm[d.border_start + lc];
    for (i64 q = ap[oc]; q < ap[oc + 1]; ++q) {
      const size_t orow = (size_t)ai[q];
      if (orow >= n) continue;
      const size_t nr = d.inv_perm[orow];
      if (nr >= d.border_start) {
        const i64 pos = spos(nr - d.border_start, lc);
        if (pos >= 0) schur_ax_[(size_t)pos] += ax[q];
      }
    }
  }
  int st = for_each_update([&](size_t r, size_t j, double v) {
    const i64 pos = spos(r, j);
    if (pos >= 0) schur_ax_[(size_t)pos] -= v;
  });
  if (st != ST_OK) return st;
  return schur_sparse_->factor(schur_ap_, schur_ai_, schur_ax_);
}

int BbdSolver::solve(Vec& rhs) {
  if (!factored_) return ST_SOLVE_FAILED;
  if (fallback_) return fallback_->solve(rhs);
  return solve_bbd(rhs);
}

// bbd_solver.rs:906-979
int BbdSolver::solve_bbd(Vec& rhs) {
  const BbdDecomposition& d = dec_;
  const size_t n = n_, bs = d.border_size;
  if (rhs.size() != n) return ST_SOLVE_FAILED;
  Vec work(n);
  for (size_t i = 0; i < n; ++i) work[i] = rhs[d.perm[i]];
  std::vector<Vec> z(d.num_blocks);
  for (size_t k = 0; k < d.num_blocks; ++k) {
    z[k].assign(work.begin() + d.block_ptr[k], work.begin() + d.block_ptr[k + 1]);
    int st = blocks_[k].solve(z[k]);
    if (st != ST_OK) return st;
  }
  Vec bb(work.begin() + d.border_start, work.end());
  for (size_t k = 0; k < d.num_blocks; ++k)  // matvec_add_neg
    for (size_t col = 0; col < c_[k].ncols; ++col) {
      const double xc = z[k][col];
      if (xc == 0.0) continue;
      for (size_t q = c_[k].col_ptr[col]; q < c_[k].col_ptr[col + 1]; ++q)
        bb[c_[k].row_idx[q]] -= c_[k].values[q] * xc;
    }
  if (dense_schur_) {  // DenseSchurSolver::solve
    Vec b(bs);
    for (size_t i = 0; i < bs; ++i) b[i] = bb[schur_piv_[i]];
    for (size_t i = 0; i < bs; ++i)
      for (size_t j = 0; j < i; ++j) b[i] -= schur_lu_[i * bs + j] * b[j];
    for (size_t i = bs; i-- > 0;) {
      for (size_t j = i + 1; j < bs; ++j) b[i] -= schur_lu_[i * bs + j] * b[j];
      b[i] /= schur_lu_[i * bs + i];
    }
    bb = b;
  } else {
    int st = schur_sparse_->solve(bb);
    if (st != ST_OK) return st;
  }
  for (size_t k = 0; k < d.num_blocks; ++k) {
    const size_t sz = d.block_ptr[k + 1] - d.block_ptr[k];
    Vec w(sz, 0.0);
    for (size_t col = 0; col < bs; ++col) {  // matvec_add
      const double xc = bb[col];
      if (xc == 0.0) continue;
      for (size_t q = r_[k].col_ptr[col]; q < r_[k].col_ptr[col + 1]; ++q)
        w[r_[k].row_idx[q]] += r_[k].values[q] * xc;
    }
    int st = blocks_[k].solve(w);
    if (st != ST_OK) return st;
    for (size_t i = 0; i < sz; ++i) work[d.block_ptr[k] + i] = z[k][i] - w[i];
  }
  for (size_t i = 0; i < bs; ++i) work[d.border_start + i] = bb[i];
  for (size_t i = 0; i < n; ++i) rhs[i] = work[d.inv_perm[i]];
  return ST_OK;
}

}  // namespace oracle
