// Oracle (test infrastructure only): the reference's sparse and dense LU
// solvers restated. Sources:
//   DenseSolver        crates/sim-core/src/solver.rs:596-724
//   SparseLuSolver     crates/sim-core/src/sparse_lu.rs:118, 272-618, 649-745
//   SparseLuBtfSolver  crates/sim-core/src/sparse_lu_btf.rs:191-690
//   NativeKluSolver    crates/sim-core/src/native_klu.rs:605-1685
#include <algorithm>
#include <cmath>

#include "oracle.h"

namespace oracle {

// ============================================================== Dense
DenseSolver::DenseSolver(size_t n) : n_(n), lu_(n * n, 0.0), pivots_(n) {
  for (size_t i = 0; i < n; ++i) pivots_[i] = i;
}

void DenseSolver::prepare(size_t n) {  // ensure_capacity, solver.rs:612-618
  if (n_ != n) {
    n_ = n;
    lu_.assign(n * n, 0.0);
    pivots_.resize(n);
    for (size_t i = 0; i < n; ++i) pivots_[i] = i;
  }
}

int DenseSolver::factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  size_t n = n_;
  if (ap.size() != n + 1) return ST_ANALYZE_FAILED;  // build_dense :620-636
  std::fill(lu_.begin(), lu_.end(), 0.0);
  for (size_t col = 0; col < n; ++col)
    for (i64 idx = ap[col]; idx < ap[col + 1]; ++idx) {
      size_t row = (size_t)ai[idx];
      if (row < n) lu_[row * n + col] += ax[idx];
    }
  for (size_t i = 0; i < n; ++i) pivots_[i] = i;  // factorize :638-670
  for (size_t k = 0; k < n; ++k) {
    size_t piv = k;
    double mx = std::fabs(lu_[k * n + k]);
    for (size_t i = k + 1; i < n; ++i) {
      double v = std::fabs(lu_[i * n + k]);
      if (v > mx) {
        mx = v;
        piv = i;
      }
    }
    if (mx == 0.0) return ST_FACTOR_FAILED;
    if (piv != k) {
      for (size_t j = 0; j < n; ++j) std::swap(lu_[k * n + j], lu_[piv * n + j]);
      std::swap(pivots_[k], pivots_[piv]);
    }
    double pv = lu_[k * n + k];
    for (size_t i = k + 1; i < n; ++i) {
      double f = lu_[i * n + k] / pv;
      lu_[i * n + k] = f;
      for (size_t j = k + 1; j < n; ++j) lu_[i * n + j] -= f * lu_[k * n + j];
    }
  }
  return ST_OK;
}

int DenseSolver::solve(Vec& rhs) {  // solver.rs:687-715
  size_t n = n_;
  if (rhs.size() != n) return ST_SOLVE_FAILED;
  Vec b(n);
  for (size_t i = 0; i < n; ++i) b[i] = rhs[pivots_[i]];
  for (size_t i = 0; i < n; ++i) {
    double s = b[i];
    for (size_t j = 0; j < i; ++j) s -= lu_[i * n + j] * b[j];
    b[i] = s;
  }
  for (size_t ii = n; ii-- > 0;) {
    double s = b[ii];
    for (size_t j = ii + 1; j < n; ++j) s -= lu_[ii * n + j] * rhs[j];
    double d = lu_[ii * n + ii];
    if (d == 0.0) return ST_SOLVE_FAILED;
    rhs[ii] = s / d;
  }
  return ST_OK;
}

// ============================================================== SparseLU
static const double kPivotTol = 1e-14;  // sparse_lu.rs:118

SparseLuSolver::SparseLuSolver(size_t n) : n_(n), work_(n, 0.0), mark_(n, 0) {}

void SparseLuSolver::prepare(size_t n) {  // sparse_lu.rs:661-668
  if (n != n_) {
    reset_pattern();
    n_ = n;
    work_.resize(n, 0.0);
    mark_.resize(n, 0);
  }
}

void SparseLuSolver::reset_pattern() {  // sparse_lu.rs:728-741
  analyzed_ = factored_ = false;
  last_ap_.clear();
  last_ai_.clear();
  perm_.clear();
  inv_perm_.clear();
  l_ptr_.clear();
  l_idx_.clear();
  u_ptr_.clear();
  u_idx_.clear();
  l_val_.clear();
  u_val_.clear();
}

int SparseLuSolver::analyze(const IVec& ap, const IVec& ai) {  // :670-700
  if (analyzed_ && last_ap_ == ap && last_ai_ == ai) return ST_OK;
  if (ap.size() != n_ + 1) return ST_INVALID_MATRIX;
  analyzed_ = factored_ = false;
  AmdResult r = amd_order(n_, ap.data(), ai.data());
  perm_ = std::move(r.perm);
  inv_perm_ = std::move(r.inv_perm);
  symbolic(ap, ai);
  last_ap_ = ap;
  last_ai_ = ai;
  analyzed_ = true;
  return ST_OK;
}

void SparseLuSolver::symbolic(const IVec& ap, const IVec& ai) {  // :302-418
  size_t n = n_;
  std::vector<UVec> lc(n), uc(n);
  cur_mark_ = 0;
  mark_.assign(n, 0);
  UVec pat;
  for (size_t k = 0; k < n; ++k) {
    size_t oc = inv_perm_[k];
    ++cur_mark_;
    size_t mv = cur_mark_;
    pat.clear();
    for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
      size_t orow = (size_t)ai[idx];
      if (orow < n) {
        size_t pr = perm_[orow];
        if (pr != k && mark_[pr] != mv) {
          pat.push_back(pr);
          mark_[pr] = mv;
        }
      }
    }
    for (size_t i = 0; i < pat.size(); ++i) {
      size_t row = pat[i];
      if (row < k) {
        for (size_t fr : lc[row]) {
          if (mark_[fr] != mv) {
            pat.push_back(fr);
            mark_[fr] = mv;
          }
        }
      }
    }
    std::sort(pat.begin(), pat.end());
    for (size_t row : pat) {
      if (row < k)
        uc[k].push_back(row);
      else if (row > k)
        lc[k].push_back(row);
    }
  }
  l_ptr_.assign(n + 1, 0);
  u_ptr_.assign(n + 1, 0);
  size_t ln = 0, un = 0;
  for (size_t k = 0; k < n; ++k) {
    l_ptr_[k] = ln;
    ln += lc[k].size();
    u_ptr_[k] = un;
    un += uc[k].size() + 1;
  }
  l_ptr_[n] = ln;
  u_ptr_[n] = un;
  nnz_l_ = ln;
  nnz_u_ = un;
  l_idx_.assign(ln, 0);
  u_idx_.assign(un, 0);
  for (size_t k = 0; k < n; ++k) {
    std::copy(lc[k].begin(), lc[k].end(), l_idx_.begin() + l_ptr_[k]);
    std::copy(uc[k].begin(), uc[k].end(), u_idx_.begin() + u_ptr_[k]);
    u_idx_[u_ptr_[k + 1] - 1] = k;
  }
  l_val_.assign(ln, 0.0);
  u_val_.assign(un, 0.0);
}

void SparseLuSolver::numeric(const IVec& ap, const IVec& ai, const Vec& ax) {
  // sparse_lu.rs:440-537
  size_t n = n_;
  work_.assign(n, 0.0);
  for (size_t k = 0; k < n; ++k) {
    size_t oc = inv_perm_[k];
    i64 s = ap[oc], e = ap[oc + 1];
    for (i64 idx = s; idx < e; ++idx) {
      size_t orow = (size_t)ai[idx];
      if (orow < n) work_[perm_[orow]] += ax[idx];
    }
    size_t us = u_ptr_[k], ue = u_ptr_[k + 1] - 1;
    for (size_t ui = us; ui < ue; ++ui) {
      size_t j = u_idx_[ui];
      double ujk = work_[j];
      if (ujk != 0.0) {
        for (size_t li = l_ptr_[j]; li < l_ptr_[j + 1]; ++li)
          work_[l_idx_[li]] -= l_val_[li] * ujk;
      }
    }
    for (size_t ui = us; ui < ue; ++ui) u_val_[ui] = work_[u_idx_[ui]];
    double diag = work_[k];
    if (std::fabs(diag) < kPivotTol) diag = diag >= 0.0 ? kPivotTol : -kPivotTol;
    u_val_[u_ptr_[k + 1] - 1] = diag;
    size_t ls = l_ptr_[k], le = l_ptr_[k + 1];
    for (size_t li = ls; li < le; ++li) l_val_[li] = work_[l_idx_[li]] / diag;
    for (i64 idx = s; idx < e; ++idx) {
      size_t orow = (size_t)ai[idx];
      if (orow < n) work_[perm_[orow]] = 0.0;
    }
    for (size_t li = ls; li < le; ++li) work_[l_idx_[li]] = 0.0;
    for (size_t ui = us; ui < ue; ++ui) work_[u_idx_[ui]] = 0.0;
    work_[k] = 0.0;
  }
}

int SparseLuSolver::factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  // sparse_lu.rs:702-714
  if (!analyzed_ || last_ap_ != ap || last_ai_ != ai) {
    int st = analyze(ap, ai);
    if (st != ST_OK) return st;
  }
  numeric(ap, ai, ax);
  factored_ = true;
  ++factor_count;
  return ST_OK;
}

int SparseLuSolver::solve(Vec& rhs) {  // :716-726, solve_internal :564-618
  if (!factored_) return ST_SOLVE_FAILED;
  if (rhs.size() != n_) return ST_INVALID_MATRIX;
  size_t n = n_;
  Vec t(n, 0.0);
  for (size_t i = 0; i < n; ++i) t[perm_[i]] = rhs[i];
  for (size_t k = 0; k < n; ++k) {
    double z = t[k];
    for (size_t li = l_ptr_[k]; li < l_ptr_[k + 1]; ++li)
      t[l_idx_[li]] -= l_val_[li] * z;
  }
  for (size_t k = n; k-- > 0;) {
    double d = u_val_[u_ptr_[k + 1] - 1];
    t[k] /= d;
    double xk = t[k];
    for (size_t ui = u_ptr_[k]; ui < u_ptr_[k + 1] - 1; ++ui)
      t[u_idx_[ui]] -= u_val_[ui] * xk;
  }
  for (size_t i = 0; i < n; ++i) rhs[i] = t[perm_[i]];
  return ST_OK;
}

// ============================================================== SparseLU-BTF
SparseLuBtfSolver::SparseLuBtfSolver(size_t n) : n_(n), work_(n, 0.0) {}

void SparseLuBtfSolver::prepare(size_t n) {  // sparse_lu_btf.rs:575-582
  if (n != n_) {
    reset_pattern();
    n_ = n;
    work_.resize(n, 0.0);
  }
}

void SparseLuBtfSolver::reset_pattern() {  // :663-672
  analyzed_ = factored_ = false;
  last_ap_.clear();
  last_ai_.clear();
  has_btf_ = false;
  blocks_.clear();
  off_.clear();
  fallback_.clear();
  has_fallback_ = false;
}

int SparseLuBtfSolver::analyze_btf(const IVec& ap, const IVec& ai) {
  // :191-227, extract_block_patterns :230-356
  size_t n = n_;
  Btf btf = btf_decompose(n, ap.data(), ai.data());
  if (btf.num_blocks <= 1 || btf.max_block_size == n) {
    has_btf_ = false;
    fallback_.clear();
    fallback_.emplace_back(n);
    fallback_[0].prepare(n);
    has_fallback_ = true;
    return fallback_[0].analyze(ap, ai);
  }
  blocks_.clear();
  for (size_t k = 0; k < btf.num_blocks; ++k) {
    size_t bs = btf.block_size(k);
    blocks_.emplace_back(bs);
    blocks_.back().prepare(bs);
  }
  for (size_t k = 0; k < btf.num_blocks; ++k) {
    size_t b0 = btf.block_ptr[k], b1 = btf.block_ptr[k + 1];
    IVec bap(b1 - b0 + 1, 0), bai;
    for (size_t lc = 0; lc < b1 - b0; ++lc) {
      size_t oc = btf.col_perm[b0 + lc];
      for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
        size_t orow = (size_t)ai[idx];
        if (orow >= n) continue;
        size_t nr = btf.row_perm_inv[orow];
        if (nr >= b0 && nr < b1) bai.push_back((i64)(nr - b0));
      }
      bap[lc + 1] = (i64)bai.size();
    }
    int st = blocks_[k].analyze(bap, bai);
    if (st != ST_OK) return st;
  }
  off_.clear();
  for (size_t br = 0; br < btf.num_blocks; ++br) {
    size_t r0 = btf.block_ptr[br], r1 = btf.block_ptr[br + 1];
    for (size_t bc = br + 1; bc < btf.num_blocks; ++bc) {
      size_t c0 = btf.block_ptr[bc], c1 = btf.block_ptr[bc + 1];
      OffDiag od;
      od.block_row = br;
      od.block_col = bc;
      od.row_start = r0;
      od.col_start = c0;
      od.nrows = r1 - r0;
      od.ncols = c1 - c0;
      od.col_ptr.assign(od.ncols + 1, 0);
      for (size_t lc = 0; lc < od.ncols; ++lc) {
        size_t oc = btf.col_perm[c0 + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf.row_perm_inv[orow];
          if (nr >= r0 && nr < r1) od.row_idx.push_back(nr - r0);
        }
        od.col_ptr[lc + 1] = od.row_idx.size();
      }
      if (!od.row_idx.empty()) off_.push_back(std::move(od));
    }
  }
  btf_ = std::move(btf);
  has_btf_ = true;
  fallback_.clear();
  has_fallback_ = false;
  return ST_OK;
}

int SparseLuBtfSolver::analyze(const IVec& ap, const IVec& ai) {  // :584-617
  if (analyzed_ && last_ap_ == ap && last_ai_ == ai) return ST_OK;
  if (ap.size() != n_ + 1) return ST_INVALID_MATRIX;
  analyzed_ = factored_ = false;
  size_t nnz = (size_t)ap[n_];
  int st;
  if (use_btf_ && should_use_btf(n_, nnz)) {
    st = analyze_btf(ap, ai);
  } else {
    has_btf_ = false;
    fallback_.clear();
    fallback_.emplace_back(n_);
    fallback_[0].prepare(n_);
    has_fallback_ = true;
    st = fallback_[0].analyze(ap, ai);
  }
  if (st != ST_OK) return st;
  last_ap_ = ap;
  last_ai_ = ai;
  analyzed_ = true;
  return ST_OK;
}

int SparseLuBtfSolver::factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  // :619-634, factor_btf :359-438
  if (!analyzed_ || last_ap_ != ap || last_ai_ != ai) {
    int st = analyze(ap, ai);
    if (st != ST_OK) return st;
  }
  size_t n = n_;
  if (has_btf_) {
    for (size_t k = 0; k < btf_.num_blocks; ++k) {
      size_t b0 = btf_.block_ptr[k], b1 = btf_.block_ptr[k + 1];
      IVec bap(b1 - b0 + 1, 0), bai;
      Vec bax;
      for (size_t lc = 0; lc < b1 - b0; ++lc) {
        size_t oc = btf_.col_perm[b0 + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf_.row_perm_inv[orow];
          if (nr >= b0 && nr < b1) {
            bai.push_back((i64)(nr - b0));
            bax.push_back(ax[idx]);
          }
        }
        bap[lc + 1] = (i64)bai.size();
      }
      int st = blocks_[k].factor(bap, bai, bax);
      if (st != ST_OK) return st;
    }
    for (auto& od : off_) {
      size_t r1 = od.row_start + od.nrows;
      od.values.clear();
      for (size_t lc = 0; lc < od.ncols; ++lc) {
        size_t oc = btf_.col_perm[od.col_start + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf_.row_perm_inv[orow];
          if (nr >= od.row_start && nr < r1) od.values.push_back(ax[idx]);
        }
      }
    }
  } else if (has_fallback_) {
    int st = fallback_[0].factor(ap, ai, ax);
    if (st != ST_OK) return st;
  } else {
    return ST_FACTOR_FAILED;
  }
  factored_ = true;
  ++factor_count;
  return ST_OK;
}

int SparseLuBtfSolver::solve(Vec& rhs) {  // :636-651, solve_btf :441-561
  if (!factored_) return ST_SOLVE_FAILED;
  if (rhs.size() != n_) return ST_INVALID_MATRIX;
  if (!has_btf_) {
    if (has_fallback_) return fallback_[0].solve(rhs);
    return ST_SOLVE_FAILED;
  }
  size_t n = n_;
  work_.resize(n, 0.0);
  for (size_t r = 0; r < n; ++r) work_[btf_.row_perm_inv[r]] = rhs[r];
  // First pass (:461-492): block solves whose results are discarded. Kept so
  // the timed CPU baseline does the same work as the reference.
  for (size_t k = 0; k < btf_.num_blocks; ++k) {
    Vec b(work_.begin() + btf_.block_ptr[k], work_.begin() + btf_.block_ptr[k + 1]);
    int st = blocks_[k].solve(b);
    if (st != ST_OK) return st;
    for (size_t i = 0; i < b.size(); ++i) work_[btf_.block_ptr[k] + i] = b[i];
  }
  for (size_t r = 0; r < n; ++r) work_[btf_.row_perm_inv[r]] = rhs[r];
  for (size_t k = btf_.num_blocks; k-- > 0;) {
    for (auto& od : off_) {
      if (od.block_row != k) continue;
      for (size_t lc = 0; lc < od.ncols; ++lc) {
        double xj = work_[od.col_start + lc];
        for (size_t idx = od.col_ptr[lc]; idx < od.col_ptr[lc + 1]; ++idx)
          work_[od.row_start + od.row_idx[idx]] -= od.values[idx] * xj;
      }
    }
    size_t b0 = btf_.block_ptr[k], b1 = btf_.block_ptr[k + 1];
    Vec b(work_.begin() + b0, work_.begin() + b1);
    int st = blocks_[k].solve(b);
    if (st != ST_OK) return st;
    for (size_t i = 0; i < b.size(); ++i) work_[b0 + i] = b[i];
  }
  for (size_t c = 0; c < n; ++c) rhs[c] = work_[btf_.col_perm_inv[c]];
  return ST_OK;
}

// ============================================================== NativeKLU
NativeKluSolver::NativeKluSolver(size_t n, KluConfig cfg)
    : n_(n), cfg_(cfg), work_(n, 0.0) {}

void NativeKluSolver::prepare(size_t n) {  // native_klu.rs:1608-1614
  if (n != n_) {
    reset_pattern();
    n_ = n;
    work_.resize(n, 0.0);
  }
}

void NativeKluSolver::reset_pattern() {  // native_klu.rs:1657-1666
  state_ = EMPTY;
  has_btf_ = false;
  btf_ = Btf();
  sym_.clear();
  num_.clear();
  off_.clear();
  last_ap_.clear();
  last_ai_.clear();
  stats_ = KluStats();
}

int NativeKluSolver::analyze(const IVec& ap, const IVec& ai) {  // :1616-1632
  if (state_ != EMPTY && pattern_matches(ap, ai)) return ST_OK;
  if (ap.size() != n_ + 1) return ST_INVALID_MATRIX;
  return do_analyze(ap, ai);
}

int NativeKluSolver::factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  // :1634-1641
  if (state_ == EMPTY || !pattern_matches(ap, ai)) {
    int st = do_analyze(ap, ai);
    if (st != ST_OK) return st;
  }
  return do_factor(ap, ai, ax);
}

int NativeKluSolver::solve(Vec& rhs) {  // :1643-1655, do_solve :1433-1439
  if (state_ != FACTORED) return ST_SOLVE_FAILED;
  if (rhs.size() != n_) return ST_INVALID_MATRIX;
  if (!has_btf_) {
    solve_block(sym_[0], num_[0], rhs.data());  // solve_single_block :1441-1489
    return ST_OK;
  }
  // solve_btf :1491-1551
  size_t n = n_;
  work_.resize(n, 0.0);
  for (size_t r = 0; r < n; ++r) work_[btf_.row_perm_inv[r]] = rhs[r];
  // Reference: blocks last to first with the coupling above the diagonal.
  // Exact mode: BTF leaves the coupling below the diagonal blocks, so the
  // blocks are solved first to last.
  const size_t nb = btf_.num_blocks;
  for (size_t kk = 0; kk < nb; ++kk) {
    size_t k = cfg_.exact_pivots ? kk : nb - 1 - kk;
    size_t b0 = btf_.block_ptr[k], b1 = btf_.block_ptr[k + 1];
    for (auto& od : off_) {
      if (od.block_row != k) continue;
      for (size_t lc = 0; lc < od.ncols; ++lc) {
        double xj = work_[od.col_start + lc];
        for (size_t idx = od.col_ptr[lc]; idx < od.col_ptr[lc + 1]; ++idx)
          work_[od.row_start + od.row_idx[idx]] -= od.values[idx] * xj;
      }
    }
    Vec b(work_.begin() + b0, work_.begin() + b1);
    if (b1 - b0 == 1)
      b[0] /= num_[k].u_diag[0];
    else
      solve_block(sym_[k], num_[k], b.data());
    for (size_t i = 0; i < b.size(); ++i) work_[b0 + i] = b[i];
  }
  for (size_t c = 0; c < n; ++c) rhs[c] = work_[btf_.col_perm_inv[c]];
  return ST_OK;
}

void NativeKluSolver::solve_block(const Symbolic& sym, const Numeric& num,
                                  double* rhs) const {  // :1554-1600
  size_t n = sym.n;
  Vec t(n, 0.0);
  for (size_t i = 0; i < n; ++i) t[num.row_perm_inv[sym.col_perm[i]]] = rhs[i];
  for (size_t k = 0; k < n; ++k) {
    double z = t[k];
    for (size_t li = sym.l_ptr[k]; li < sym.l_ptr[k + 1]; ++li)
      t[sym.l_idx[li]] -= num.l_val[li] * z;
  }
  for (size_t k = n; k-- > 0;) {
    t[k] /= num.u_diag[k];
    double xk = t[k];
    for (size_t ui = sym.u_ptr[k]; ui < sym.u_ptr[k + 1] - 1; ++ui)
      t[sym.u_idx[ui]] -= num.u_val[ui] * xk;
  }
  for (size_t i = 0; i < n; ++i) rhs[i] = t[sym.col_perm[i]];
}

int NativeKluSolver::do_analyze(const IVec& ap, const IVec& ai) {  // :704-761
  size_t n = n_;
  size_t fc = stats_.factor_count, rc = stats_.refactor_count;
  sym_.clear();
  num_.clear();
  off_.clear();
  stats_ = KluStats();
  stats_.factor_count = fc;
  stats_.refactor_count = rc;
  bool use_btf = cfg_.use_btf && n >= 4;
  has_btf_ = false;
  if (use_btf) {
    Btf b = btf_decompose(n, ap.data(), ai.data());
    if (b.num_blocks >= cfg_.btf_min_blocks && b.max_block_size < n) {
      btf_ = std::move(b);
      has_btf_ = true;
    }
  }
  if (has_btf_) {
    stats_.nblocks = btf_.num_blocks;
    for (size_t k = 0; k < btf_.num_blocks; ++k) {  // extract_block_pattern :764-797
      size_t b0 = btf_.block_ptr[k], b1 = btf_.block_ptr[k + 1];
      IVec bap(b1 - b0 + 1, 0), bai;
      for (size_t lc = 0; lc < b1 - b0; ++lc) {
        size_t oc = btf_.col_perm[b0 + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf_.row_perm_inv[orow];
          if (nr >= b0 && nr < b1) bai.push_back((i64)(nr - b0));
        }
        bap[lc + 1] = (i64)bai.size();
      }
      sym_.push_back(symbolic_for_block(b1 - b0, bap, bai));
    }
    size_t noff = 0;  // extract_off_diag_patterns :800-857
    for (size_t br = 0; br < btf_.num_blocks; ++br) {
      size_t r0 = btf_.block_ptr[br], r1 = btf_.block_ptr[br + 1];
      // reference: blocks to the right (above); exact mode: blocks to the left
      const size_t bc_lo = cfg_.exact_pivots ? 0 : br + 1;
      const size_t bc_hi = cfg_.exact_pivots ? br : btf_.num_blocks;
      for (size_t bc = bc_lo; bc < bc_hi; ++bc) {
        size_t c0 = btf_.block_ptr[bc], c1 = btf_.block_ptr[bc + 1];
        OffDiag od;
        od.block_row = br;
        od.block_col = bc;
        od.row_start = r0;
        od.col_start = c0;
        od.nrows = r1 - r0;
        od.ncols = c1 - c0;
        od.col_ptr.assign(od.ncols + 1, 0);
        for (size_t lc = 0; lc < od.ncols; ++lc) {
          size_t oc = btf_.col_perm[c0 + lc];
          for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
            size_t orow = (size_t)ai[idx];
            if (orow >= n) continue;
            size_t nr = btf_.row_perm_inv[orow];
            if (nr >= r0 && nr < r1) od.row_idx.push_back(nr - r0);
          }
          od.col_ptr[lc + 1] = od.row_idx.size();
        }
        if (!od.row_idx.empty()) {
          noff += od.row_idx.size();
          off_.push_back(std::move(od));
        }
      }
    }
    stats_.noffdiag = noff;
  } else {
    stats_.nblocks = 1;
    sym_.push_back(symbolic_for_block(n, ap, ai));
  }
  state_ = ANALYZED;
  last_ap_ = ap;
  last_ai_ = ai;
  sym_free_ = sym_;
  for (auto& s : sym_) {
    stats_.nnz_l += s.l_idx.size();
    stats_.nnz_u += s.u_idx.size();
  }
  return ST_OK;
}

NativeKluSolver::Symbolic NativeKluSolver::symbolic_for_block(
    size_t n, const IVec& ap, const IVec& ai) const {  // :863-1014
  Symbolic s;
  s.n = n;
  if (n == 0) {
    s.l_ptr = {0};
    s.u_ptr = {0};
    return s;
  }
  if (cfg_.ordering == 3) {
    s.col_perm.resize(n);
    s.col_perm_inv.resize(n);
    for (size_t i = 0; i < n; ++i) s.col_perm[i] = s.col_perm_inv[i] = i;
  } else {
    AmdResult r = amd_order(n, ap.data(), ai.data());
    s.col_perm = std::move(r.perm);
    s.col_perm_inv = std::move(r.inv_perm);
  }
  IVec pap(n + 1, 0), pai;
  for (size_t nc = 0; nc < n; ++nc) {
    size_t oc = s.col_perm_inv[nc];
    for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
      size_t orow = (size_t)ai[idx];
      if (orow < n) pai.push_back((i64)s.col_perm[orow]);
    }
    pap[nc + 1] = (i64)pai.size();
  }
  symbolic_dfs(n, pap, pai, s);
  return s;
}

void NativeKluSolver::symbolic_dfs(size_t n, const IVec& pap, const IVec& pai,
                                   Symbolic& s) {  // native_klu.rs:915-1004
  s.l_ptr.assign(n + 1, 0);
  s.u_ptr.assign(n + 1, 0);
  UVec mark(n, 0);
  size_t cur = 0;
  std::vector<std::pair<size_t, bool>> stack;
  UVec pattern, ur, lr;
  for (size_t k = 0; k < n; ++k) {
    ++cur;
    pattern.clear();
    for (i64 idx = pap[k]; idx < pap[k + 1]; ++idx) {
      size_t row = (size_t)pai[idx];
      if (row != k && mark[row] != cur) {
        mark[row] = cur;
        if (row < k)
          stack.push_back({row, true});
        else
          pattern.push_back(row);
      }
    }
    while (!stack.empty()) {
      auto [node, first] = stack.back();
      stack.pop_back();
      if (first) {
        stack.push_back({node, false});
        for (size_t li = s.l_ptr[node]; li < s.l_ptr[node + 1]; ++li) {
          size_t child = s.l_idx[li];
          if (mark[child] != cur) {
            mark[child] = cur;
            if (child < k)
              stack.push_back({child, true});
            else
              pattern.push_back(child);
          }
        }
      }
      if (!first) pattern.push_back(node);
    }
    ur.clear();
    lr.clear();
    for (size_t row : pattern) {
      if (row < k)
        ur.push_back(row);
      else if (row > k)
        lr.push_back(row);
    }
    std::sort(ur.begin(), ur.end());
    std::sort(lr.begin(), lr.end());
    size_t us = s.u_idx.size();
    s.u_idx.insert(s.u_idx.end(), ur.begin(), ur.end());
    s.u_idx.push_back(k);
    s.u_ptr[k] = us;
    s.u_ptr[k + 1] = s.u_idx.size();
    size_t ls = s.l_idx.size();
    s.l_idx.insert(s.l_idx.end(), lr.begin(), lr.end());
    s.l_ptr[k] = ls;
    s.l_ptr[k + 1] = s.l_idx.size();
  }
}

NativeKluSolver::Symbolic NativeKluSolver::resymbolic(const Symbolic& sym,
                                                      const Numeric& num,
                                                      const IVec& ap,
                                                      const IVec& ai) const {
  // Pattern of the block as the factorization sees it after pivoting: column
  // k = col_perm[c], row w = row_perm_inv[col_perm[r]].
  size_t n = sym.n;
  Symbolic s;
  s.n = n;
  s.col_perm = sym.col_perm;
  s.col_perm_inv = sym.col_perm_inv;
  IVec pap(n + 1, 0), pai;
  for (size_t k = 0; k < n; ++k) {
    size_t oc = sym.col_perm_inv[k];
    for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
      size_t orow = (size_t)ai[idx];
      if (orow < n) pai.push_back((i64)num.row_perm_inv[sym.col_perm[orow]]);
    }
    pap[k + 1] = (i64)pai.size();
  }
  symbolic_dfs(n, pap, pai, s);
  return s;
}

thread_local size_t perturbed_pivots = 0;

NativeKluSolver::Numeric NativeKluSolver::factor_block(
    const Symbolic& sym, const IVec& ap, const IVec& ai, const Vec& ax,
    const Numeric* old, bool refactor) const {  // :1194-1382
  size_t n = sym.n;
  Numeric num;
  if (n == 0) return num;
  if (n == 1) {  // singleton fast path :1215-1237
    size_t oc = sym.col_perm_inv[0];
    double diag = 0.0;
    for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
      size_t row = (size_t)ai[idx];
      if (row < n && sym.col_perm[row] == 0) diag += ax[idx];
    }
    if (std::fabs(diag) < 1e-300) {
      diag = 1e-14;
      ++perturbed_pivots;
    }
    num.u_val = {diag};
    num.u_diag = {diag};
    num.row_perm = {0};
    num.row_perm_inv = {0};
    return num;
  }
  num.l_val.assign(sym.l_idx.size(), 0.0);
  num.u_val.assign(sym.u_idx.size(), 0.0);
  num.u_diag.assign(n, 0.0);
  bool use_old = refactor && old != nullptr;
  if (use_old) {
    num.row_perm = old->row_perm;
    num.row_perm_inv = old->row_perm_inv;
  } else {
    num.row_perm.resize(n);
    num.row_perm_inv.resize(n);
    for (size_t i = 0; i < n; ++i) num.row_perm[i] = num.row_perm_inv[i] = i;
  }
  Vec work(n, 0.0);
  for (size_t k = 0; k < n; ++k) {
    size_t oc = sym.col_perm_inv[k];
    i64 s = ap[oc], e = ap[oc + 1];
    for (i64 idx = s; idx < e; ++idx) {  // step 1: scatter
      size_t orow = (size_t)ai[idx];
      if (orow < n) work[num.row_perm_inv[sym.col_perm[orow]]] += ax[idx];
    }
    size_t us = sym.u_ptr[k], ue = sym.u_ptr[k + 1] - 1;
    for (size_t ui = us; ui < ue; ++ui) {  // step 2: left-looking update
      size_t j = sym.u_idx[ui];
      double ujk = work[j];
      if (ujk != 0.0) {
        for (size_t li = sym.l_ptr[j]; li < sym.l_ptr[j + 1]; ++li)
          work[sym.l_idx[li]] -= num.l_val[li] * ujk;
      }
    }
    size_t ls = sym.l_ptr[k], le = sym.l_ptr[k + 1];
    if (!use_old) {  // step 3: threshold pivot within the symbolic pattern
      double dabs = std::fabs(work[k]);
      double mx = dabs;
      size_t mr = k;
      for (size_t li = ls; li < le; ++li) {
        size_t row = sym.l_idx[li];
        double v = std::fabs(work[row]);
        if (v > mx) {
          mx = v;
          mr = row;
        }
      }
      if (mr != k && dabs < cfg_.pivot_tol * mx) {
        std::swap(work[k], work[mr]);
        size_t ok = num.row_perm[k], om = num.row_perm[mr];
        num.row_perm[k] = om;
        num.row_perm[mr] = ok;
        num.row_perm_inv[ok] = mr;
        num.row_perm_inv[om] = k;
      }
    }
    for (size_t ui = us; ui < ue; ++ui) num.u_val[ui] = work[sym.u_idx[ui]];
    double diag = work[k];
    if (std::fabs(diag) < 1e-14) {
      diag = diag >= 0.0 ? 1e-14 : -1e-14;
      ++perturbed_pivots;
    }
    num.u_val[sym.u_ptr[k + 1] - 1] = diag;
    num.u_diag[k] = diag;
    for (size_t li = ls; li < le; ++li) num.l_val[li] = work[sym.l_idx[li]] / diag;
    for (i64 idx = s; idx < e; ++idx) {  // step 6: clear
      size_t orow = (size_t)ai[idx];
      if (orow < n) work[num.row_perm_inv[sym.col_perm[orow]]] = 0.0;
    }
    for (size_t li = ls; li < le; ++li) work[sym.l_idx[li]] = 0.0;
    for (size_t ui = us; ui < ue; ++ui) work[sym.u_idx[ui]] = 0.0;
    work[k] = 0.0;
  }
  return num;
}

bool NativeKluSolver::growth(const Numeric& nm) const {
  const double lim = 1.0 / cfg_.pivot_tol;
  for (double l : nm.l_val)
    if (std::fabs(l) > lim || std::isnan(l)) return true;
  return false;
}

int NativeKluSolver::refactor_afresh(const IVec& ap, const IVec& ai, const Vec& ax) {
  // the reference's mode: every block's first factorization again (as after
  // reset_pattern), counted as a refactorization with one re-pivot
  KluStats keep = stats_;
  state_ = ANALYZED;
  sym_ = sym_free_;
  const int st = do_factor(ap, ai, ax);
  const double rc = stats_.rcond;
  stats_ = keep;
  stats_.rcond = rc;
  ++stats_.refactor_count;
  ++stats_.repivots;
  return st;
}

int NativeKluSolver::do_factor(const IVec& ap, const IVec& ai, const Vec& ax) {
  // :1020-1148
  bool same = state_ == FACTORED && pattern_matches(ap, ai);
  size_t n = n_;
  if (has_btf_) {
    std::vector<Numeric> nn;
    for (size_t k = 0; k < btf_.num_blocks; ++k) {
      size_t b0 = btf_.block_ptr[k], b1 = btf_.block_ptr[k + 1];
      IVec bap(b1 - b0 + 1, 0), bai;  // extract_block_values :1151-1187
      Vec bax;
      for (size_t lc = 0; lc < b1 - b0; ++lc) {
        size_t oc = btf_.col_perm[b0 + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf_.row_perm_inv[orow];
          if (nr >= b0 && nr < b1) {
            bai.push_back((i64)(nr - b0));
            bax.push_back(ax[idx]);
          }
        }
        bap[lc + 1] = (i64)bai.size();
      }
      const Numeric* old = (same && k < num_.size()) ? &num_[k] : nullptr;
      Numeric nm = factor_block(sym_[k], bap, bai, bax, old, same);
      if (cfg_.exact_pivots && !same && sym_[k].n > 1) {
        sym_[k] = resymbolic(sym_[k], nm, bap, bai);
        nm = factor_block(sym_[k], bap, bai, bax, &nm, true);
      }
      if (same && cfg_.repivot && growth(nm)) {
        if (!cfg_.exact_pivots) return refactor_afresh(ap, ai, ax);
        ++stats_.repivots;  // this block afresh: its first factorization
        nm = factor_block(sym_free_[k], bap, bai, bax, nullptr, false);
        if (sym_free_[k].n > 1) {
          sym_[k] = resymbolic(sym_free_[k], nm, bap, bai);
          nm = factor_block(sym_[k], bap, bai, bax, &nm, true);
        }
      }
      nn.push_back(std::move(nm));
    }
    num_ = std::move(nn);
    for (auto& od : off_) {
      size_t r1 = od.row_start + od.nrows;
      od.values.clear();
      for (size_t lc = 0; lc < od.ncols; ++lc) {
        size_t oc = btf_.col_perm[od.col_start + lc];
        for (i64 idx = ap[oc]; idx < ap[oc + 1]; ++idx) {
          size_t orow = (size_t)ai[idx];
          if (orow >= n) continue;
          size_t nr = btf_.row_perm_inv[orow];
          if (nr >= od.row_start && nr < r1) od.values.push_back(ax[idx]);
        }
      }
    }
  } else {
    const Numeric* old = (same && !num_.empty()) ? &num_[0] : nullptr;
    Numeric nm = factor_block(sym_[0], ap, ai, ax, old, same);
    if (cfg_.exact_pivots && !same && sym_[0].n > 1) {
      sym_[0] = resymbolic(sym_[0], nm, ap, ai);
      nm = factor_block(sym_[0], ap, ai, ax, &nm, true);
    }
    if (same && cfg_.repivot && growth(nm)) {
      if (!cfg_.exact_pivots) return refactor_afresh(ap, ai, ax);
      ++stats_.repivots;
      nm = factor_block(sym_free_[0], ap, ai, ax, nullptr, false);
      if (sym_free_[0].n > 1) {
        sym_[0] = resymbolic(sym_free_[0], nm, ap, ai);
        nm = factor_block(sym_[0], ap, ai, ax, &nm, true);
      }
    }
    num_.clear();
    num_.push_back(std::move(nm));
  }
  if (same && state_ == FACTORED)
    ++stats_.refactor_count;
  else
    ++stats_.factor_count;
  double mn = 1.7976931348623157e308, mx = 0.0;  // compute_rcond :1406-1427
  for (auto& nm : num_)
    for (double d : nm.u_diag) {
      double a = std::fabs(d);
      if (a < mn) mn = a;
      if (a > mx) mx = a;
    }
  stats_.rcond = mx > 0.0 ? mn / mx : 0.0;
  state_ = FACTORED;
  return ST_OK;
}

std::unique_ptr<LinearSolver> make_solver(const std::string& kind, size_t n) {
  if (kind == "dense") return std::make_unique<DenseSolver>(n);
  if (kind == "sparselu") return std::make_unique<SparseLuSolver>(n);
  if (kind == "sparselubtf") return std::make_unique<SparseLuBtfSolver>(n);
  if (kind == "nativeklu_exact" || kind == "nativeklu_exact_repivot" ||
      kind == "nativeklu_repivot") {
    KluConfig cfg;
    cfg.exact_pivots = kind != "nativeklu_repivot";
    cfg.repivot = kind != "nativeklu_exact";
    return std::make_unique<NativeKluSolver>(n, cfg);
  }
  return std::make_unique<NativeKluSolver>(n);
}

}  // namespace oracle
