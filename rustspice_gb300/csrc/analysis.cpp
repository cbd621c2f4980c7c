// Host-side symbolic analysis (integer work only, once per pattern).
// See analysis.h for the data model.
#include "analysis.h"

#include <algorithm>
#include <functional>
#include <queue>

namespace gk {

// ------------------------------------------------------------------ AMD
// Quotient-graph minimum degree as in crates/sim-core/src/amd.rs:172-412:
// a (degree, node) min-heap with lazy re-insertion, elements absorbed into
// the newest element, degrees recounted through elements. Ties go to the
// smaller node id, so the ordering is deterministic.
void amd_order(int n, const i64* ap, const i64* ai, std::vector<int>& perm,
               std::vector<int>& inv) {
  perm.assign(n, 0);
  inv.assign(n, 0);
  if (n == 0) return;
  std::vector<std::vector<int>> nb(n);
  auto has = [](const std::vector<int>& v, int x) {
    return std::find(v.begin(), v.end(), x) != v.end();
  };
  for (int c = 0; c < n; ++c)
    for (i64 t = ap[c]; t < ap[c + 1]; ++t) {
      int r = (int)ai[t];
      if (r >= n || r == c) continue;
      if (!has(nb[c], r)) nb[c].push_back(r);
      if (!has(nb[r], c)) nb[r].push_back(c);
    }
  std::vector<char> elem(n, 0);
  std::vector<int> deg(n);
  using Key = std::pair<int, int>;
  std::priority_queue<Key, std::vector<Key>, std::greater<Key>> pq;
  for (int i = 0; i < n; ++i) {
    deg[i] = (int)nb[i].size();
    pq.push({deg[i], i});
  }
  std::vector<unsigned> stamp(n, 0), inp(n, 0);
  unsigned tick = 0, ptick = 0;
  int done = 0;
  std::vector<int> vars, els;
  while (done < n && !pq.empty()) {
    Key k = pq.top();
    pq.pop();
    int p = k.second;
    if (elem[p]) continue;
    if (k.first != deg[p]) {
      pq.push({deg[p], p});
      continue;
    }
    perm[p] = done;
    inv[done] = p;
    ++done;
    const unsigned mk = ++tick;
    vars.clear();
    els.clear();
    for (int a : nb[p]) {
      if (elem[a])
        els.push_back(a);
      else if (stamp[a] != mk) {
        stamp[a] = mk;
        vars.push_back(a);
      }
    }
    for (int e : els)
      for (int a : nb[e])
        if (!elem[a] && a != p && stamp[a] != mk) {
          stamp[a] = mk;
          vars.push_back(a);
        }
    elem[p] = 1;
    nb[p] = vars;
    ++ptick;  // inp[v] == ptick <=> v is in nb[p]
    for (int v : vars) inp[v] = ptick;
    for (int e : els) {  // absorb e into p
      if (e == p) continue;
      std::vector<int> moved;
      moved.swap(nb[e]);
      for (int v : moved) {
        if (elem[v]) continue;
        if (inp[v] != ptick) {
          inp[v] = ptick;
          nb[p].push_back(v);
        }
        auto it = std::find(nb[v].begin(), nb[v].end(), e);
        if (it != nb[v].end()) *it = p;
      }
    }
    for (int v : vars) {  // approximate degree through elements
      if (elem[v]) continue;
      const unsigned m2 = ++tick;
      stamp[v] = m2;
      int d = 0;
      for (int a : nb[v]) {
        if (!elem[a]) {
          if (stamp[a] != m2) {
            stamp[a] = m2;
            ++d;
          }
        } else {
          for (int b : nb[a])
            if (!elem[b] && stamp[b] != m2) {
              stamp[b] = m2;
              ++d;
            }
        }
      }
      deg[v] = d;
      pq.push({d, v});
    }
  }
}

// ------------------------------------------------------------------ BTF
// Maximum transversal by augmenting paths tried row by row in row order, the
// directed graph "column i -> column j if column i has an entry in the row
// matched to j", Tarjan SCCs, blocks in reversed emission order, unmatched
// columns appended as singletons (crates/sim-core/src/btf.rs:143-550). Both
// depth-first searches use explicit stacks with the reference's visit order.
BtfResult btf_decompose(int n, const i64* ap, const i64* ai) {
  BtfResult b;
  b.block_ptr.push_back(0);
  if (n == 0) return b;
  std::vector<std::vector<int>> rows(n);
  for (int c = 0; c < n; ++c)
    for (i64 t = ap[c]; t < ap[c + 1]; ++t)
      if (ai[t] < n) rows[(int)ai[t]].push_back(c);
  std::vector<int> cmatch(n, -1), rmatch(n, -1), seen(n, -1);
  struct F {
    int row;
    size_t next;
    int via;
  };
  std::vector<F> st;
  for (int root = 0; root < n; ++root) {
    st.assign(1, F{root, 0, -1});
    while (!st.empty()) {
      F& f = st.back();
      int r = f.row;
      int go = -1;
      bool hit = false;
      while (f.next < rows[r].size()) {
        int c = rows[r][f.next++];
        if (seen[c] == root) continue;
        seen[c] = root;
        if (cmatch[c] < 0) {
          cmatch[c] = r;
          rmatch[r] = c;
          hit = true;
          break;
        }
        f.via = c;
        go = cmatch[c];
        break;
      }
      if (hit) {
        st.pop_back();
        for (auto it = st.rbegin(); it != st.rend(); ++it) {
          cmatch[it->via] = it->row;
          rmatch[it->row] = it->via;
        }
        st.clear();
        break;
      }
      if (go >= 0)
        st.push_back(F{go, 0, -1});
      else
        st.pop_back();
    }
  }
  std::vector<std::vector<int>> g(n);
  for (int j = 0; j < n; ++j) {
    if (cmatch[j] < 0) continue;
    for (int i : rows[cmatch[j]])
      if (i != j) g[i].push_back(j);
  }
  // Tarjan
  std::vector<int> idx(n, -1), low(n, -1), stk;
  std::vector<char> on(n, 0);
  int counter = 0;
  std::vector<std::vector<int>> comps;
  std::vector<std::pair<int, size_t>> fr;
  for (int v0 = 0; v0 < n; ++v0) {
    if (idx[v0] >= 0) continue;
    idx[v0] = low[v0] = counter++;
    stk.push_back(v0);
    on[v0] = 1;
    fr.assign(1, {v0, 0});
    while (!fr.empty()) {
      int v = fr.back().first;
      if (fr.back().second < g[v].size()) {
        int w = g[v][fr.back().second++];
        if (idx[w] < 0) {
          idx[w] = low[w] = counter++;
          stk.push_back(w);
          on[w] = 1;
          fr.push_back({w, 0});
        } else if (on[w]) {
          low[v] = std::min(low[v], idx[w]);
        }
        continue;
      }
      if (low[v] == idx[v]) {
        comps.emplace_back();
        int w;
        do {
          w = stk.back();
          stk.pop_back();
          on[w] = 0;
          comps.back().push_back(w);
        } while (w != v);
      }
      fr.pop_back();
      if (!fr.empty()) low[fr.back().first] = std::min(low[fr.back().first], low[v]);
    }
  }
  std::vector<char> rused(n, 0);
  for (auto it = comps.rbegin(); it != comps.rend(); ++it) {
    int cnt = 0;
    for (int c : *it)
      if (cmatch[c] >= 0) {
        b.col_perm.push_back(c);
        b.row_perm.push_back(cmatch[c]);
        rused[cmatch[c]] = 1;
        ++cnt;
      }
    if (!cnt) continue;
    b.block_ptr.push_back((int)b.col_perm.size());
    b.max_block = std::max(b.max_block, cnt);
  }
  for (int c = 0; c < n; ++c) {
    if (cmatch[c] >= 0) continue;
    b.col_perm.push_back(c);
    for (int r = 0; r < n; ++r)
      if (!rused[r]) {
        rused[r] = 1;
        b.row_perm.push_back(r);
        break;
      }
    b.block_ptr.push_back((int)b.col_perm.size());
  }
  b.nblocks = (int)b.block_ptr.size() - 1;
  b.row_inv.assign(n, 0);
  b.col_inv.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    b.row_inv[b.row_perm[i]] = i;
    b.col_inv[b.col_perm[i]] = i;
  }
  return b;
}

// True when the matrix has a perfect matching and its column graph under that
// matching is strongly connected: a single irreducible block. The block
// structure of a structurally nonsingular matrix does not depend on which
// perfect matching is used, so this answers "does the BTF keep more than one
// block" without the row-order augmenting search above, whose matching is
// only needed when there are blocks to order. The matching here uses a
// look-ahead scan of each row before descending (MC21-style).
bool structurally_irreducible(int n, const i64* ap, const i64* ai) {
  if (n <= 1) return true;
  std::vector<int> rp(n + 1, 0), rc;
  for (int c = 0; c < n; ++c)
    for (i64 t = ap[c]; t < ap[c + 1]; ++t)
      if (ai[t] < n) ++rp[(int)ai[t] + 1];
  for (int r = 0; r < n; ++r) rp[r + 1] += rp[r];
  rc.resize(rp[n]);
  {
    std::vector<int> fill(rp.begin(), rp.end() - 1);
    for (int c = 0; c < n; ++c)
      for (i64 t = ap[c]; t < ap[c + 1]; ++t)
        if (ai[t] < n) rc[fill[(int)ai[t]]++] = c;
  }
  std::vector<int> cmatch(n, -1), seen(n, -1), look(n), nxt(n);
  for (int r = 0; r < n; ++r) look[r] = rp[r];
  std::vector<int> stk;
  for (int root = 0; root < n; ++root) {
    stk.assign(1, root);
    nxt[root] = rp[root];
    bool found = false;
    while (!stk.empty() && !found) {
      int r = stk.back();
      for (; look[r] < rp[r + 1]; ++look[r]) {  // look-ahead for a free column
        int c = rc[look[r]];
        if (cmatch[c] < 0) {
          found = true;
          // augment along the stack: each row takes the column it descended through
          cmatch[c] = r;
          for (size_t k = stk.size() - 1; k-- > 0;) {
            int rr = stk[k];
            int cc = rc[nxt[rr] - 1];
            cmatch[cc] = rr;
          }
          break;
        }
      }
      if (found) break;
      int go = -1;
      while (nxt[r] < rp[r + 1]) {
        int c = rc[nxt[r]++];
        if (seen[c] == root) continue;
        seen[c] = root;
        go = cmatch[c];
        break;
      }
      if (go >= 0) {
        nxt[go] = rp[go];
        stk.push_back(go);
      } else {
        stk.pop_back();
      }
    }
    if (!found) return false;  // structurally singular
  }
  // column graph: i -> j when column i has an entry in the row matched to j
  // (edges of the reference's BTF graph); strongly connected <=> node 0
  // reaches everything forwards and backwards.
  std::vector<int> rowmatch(n);
  for (int c = 0; c < n; ++c) rowmatch[cmatch[c]] = c;
  std::vector<char> vis(n, 0);
  std::vector<int> q;
  // forward: from column i, edge to j = rowmatch[r] for every row r of column i
  q.assign(1, 0);
  vis[0] = 1;
  for (size_t h = 0; h < q.size(); ++h) {
    int i = q[h];
    for (i64 t = ap[i]; t < ap[i + 1]; ++t) {
      if (ai[t] >= n) continue;
      int j = rowmatch[(int)ai[t]];
      if (!vis[j]) {
        vis[j] = 1;
        q.push_back(j);
      }
    }
  }
  if ((int)q.size() != n) return false;
  // backward: into column j from every column i having an entry in row cmatch[j]
  std::fill(vis.begin(), vis.end(), 0);
  q.assign(1, 0);
  vis[0] = 1;
  for (size_t h = 0; h < q.size(); ++h) {
    int j = q[h];
    int r = cmatch[j];
    for (int t = rp[r]; t < rp[r + 1]; ++t) {
      int i = rc[t];
      if (!vis[i]) {
        vis[i] = 1;
        q.push_back(i);
      }
    }
  }
  return (int)q.size() == n;
}

// ------------------------------------------------------------------ symbolic
// Column k's pattern is the set of rows reachable from A(:,k) through the L
// columns of earlier columns (Gilbert-Peierls), split into U (< k, plus the
// diagonal last) and L (> k), each sorted.
void symbolic_dfs(int n, const std::vector<i64>& pap, const std::vector<i64>& pai,
                  Pattern& s) {
  s.lp.assign(n + 1, 0);
  s.up.assign(n + 1, 0);
  s.li.clear();
  s.ui.clear();
  std::vector<int> mark(n, -1), todo, lo, hi;
  for (int k = 0; k < n; ++k) {
    lo.clear();
    hi.clear();
    todo.clear();
    for (i64 t = pap[k]; t < pap[k + 1]; ++t) {
      int r = (int)pai[t];
      if (r == k || mark[r] == k) continue;
      mark[r] = k;
      (r < k ? todo : hi).push_back(r);
    }
    while (!todo.empty()) {
      int j = todo.back();
      todo.pop_back();
      lo.push_back(j);
      for (int q = s.lp[j]; q < s.lp[j + 1]; ++q) {
        int r = s.li[q];
        if (mark[r] == k) continue;
        mark[r] = k;
        if (r < k)
          todo.push_back(r);
        else if (r > k)
          hi.push_back(r);
      }
    }
    std::sort(lo.begin(), lo.end());
    std::sort(hi.begin(), hi.end());
    s.up[k] = (int)s.ui.size();
    s.ui.insert(s.ui.end(), lo.begin(), lo.end());
    s.ui.push_back(k);
    s.up[k + 1] = (int)s.ui.size();
    s.lp[k] = (int)s.li.size();
    s.li.insert(s.li.end(), hi.begin(), hi.end());
    s.lp[k + 1] = (int)s.li.size();
  }
}

// ------------------------------------------------------------------ plan
namespace {
// Block-local CSC of block b with rows remapped by `rowmap(local row)`, in
// the column order given by `colorder[k] = local column`.
void block_csc(const Plan& p, const i64* ap, const i64* ai, int b,
               const std::function<int(int)>& rowmap, const std::vector<int>& colorder,
               std::vector<i64>& bp, std::vector<i64>& bi, const std::vector<int>& btf_col_perm) {
  int b0 = p.block_ptr[b], nb = p.block_ptr[b + 1] - b0;
  bp.assign(nb + 1, 0);
  bi.clear();
  for (int k = 0; k < nb; ++k) {
    int oc = btf_col_perm[b0 + colorder[k]];
    for (i64 t = ap[oc]; t < ap[oc + 1]; ++t) {
      int r = (int)ai[t];
      if (r >= p.n) continue;
      int R = p.btf_row_inv[r];
      if (R < b0 || R >= b0 + nb) continue;
      bi.push_back(rowmap(R - b0));
    }
    bp[k + 1] = (i64)bi.size();
  }
}
}  // namespace

const char* const kTooLarge =
    "the factorization's update lists exceed 2^31 entries (fill too large for this solver)";

std::string analyze(int n, const i64* ap, const i64* ai, int pivot_mode, Plan& p,
                    const std::vector<int>* given_blocks, int kind) {
  p = Plan();
  p.n = n;
  p.nnz_raw = ap[n];
  p.pivot_mode = pivot_mode;
  p.kind = kind;
  p.no_singleton = kind != KIND_NATIVEKLU || given_blocks != nullptr;
  for (int c = 0; c < n; ++c) {
    if (ap[c + 1] < ap[c]) return "column pointers decrease";
    for (i64 t = ap[c]; t < ap[c + 1]; ++t)
      if (ai[t] < 0) return "negative row index";
  }
  BtfResult b;
  bool keep = false;
  if (given_blocks) {  // caller's blocks in index order, identity row order
    const std::vector<int>& g = *given_blocks;
    if (g.size() < 2 || g.front() != 0 || g.back() != n) return "block boundaries do not cover n";
    for (size_t k = 0; k + 1 < g.size(); ++k)
      if (g[k + 1] <= g[k]) return "empty or decreasing block";
    for (int c = 0, k = 0; c < n; ++c) {
      while (c >= g[k + 1]) ++k;
      for (i64 t = ap[c]; t < ap[c + 1]; ++t)
        if (ai[t] < n && (ai[t] < g[k] || ai[t] >= g[k + 1])) return "entry outside the given blocks";
    }
    b.block_ptr = g;
    b.nblocks = (int)g.size() - 1;
    b.col_perm.resize(n);
    b.row_inv.resize(n);
    b.col_inv.resize(n);
    for (int i = 0; i < n; ++i) b.col_perm[i] = b.row_inv[i] = b.col_inv[i] = i;
    keep = b.nblocks >= 2;
  } else if (kind == KIND_SPARSELU) {
    keep = false;
  } else if (kind == KIND_SPARSELU_BTF) {
    // should_use_btf (btf.rs:560-573) on the raw entry count, then the
    // decomposition's own test (sparse_lu_btf.rs:197-208)
    const double density = (double)ap[n] / ((double)n * (double)n);
    if (n >= 50 && !(density > 0.25)) {
      b = btf_decompose(n, ap, ai);
      keep = b.nblocks >= 2 && b.max_block < n;
    }
  } else if (n >= 4 && !structurally_irreducible(n, ap, ai)) {
    b = btf_decompose(n, ap, ai);
    keep = b.nblocks >= 2 && b.max_block < n;
  }
  std::vector<int> btf_col_perm(n);
  if (keep) {
    p.has_btf = true;
    p.block_ptr = b.block_ptr;
    p.btf_row_inv = b.row_inv;
    p.btf_col_inv = b.col_inv;
    btf_col_perm = b.col_perm;
  } else {
    p.block_ptr = {0, n};
    p.btf_row_inv.resize(n);
    p.btf_col_inv.resize(n);
    for (int i = 0; i < n; ++i) p.btf_row_inv[i] = p.btf_col_inv[i] = btf_col_perm[i] = i;
  }
  p.nblocks = (int)p.block_ptr.size() - 1;
  p.cperm.resize(p.nblocks);
  p.cperm_inv.resize(p.nblocks);
  p.pats_orig.resize(p.nblocks);
  std::vector<i64> bp, bi;
  for (int k = 0; k < p.nblocks; ++k) {
    int b0 = p.block_ptr[k], nb = p.block_ptr[k + 1] - b0;
    std::vector<int> ident(nb);
    for (int i = 0; i < nb; ++i) ident[i] = i;
    block_csc(p, ap, ai, k, [](int r) { return r; }, ident, bp, bi, btf_col_perm);
    amd_order(nb, bp.data(), bi.data(), p.cperm[k], p.cperm_inv[k]);
    const std::vector<int>& cp = p.cperm[k];
    block_csc(p, ap, ai, k, [&cp](int r) { return cp[r]; }, p.cperm_inv[k], bp, bi,
              btf_col_perm);
    symbolic_dfs(nb, bp, bi, p.pats_orig[k]);
  }
  // remember the BTF column permutation through out_pos's inverse later
  p.row_perm.resize(n);
  for (int k = 0; k < p.nblocks; ++k)
    for (int i = p.block_ptr[k]; i < p.block_ptr[k + 1]; ++i) p.row_perm[i] = i - p.block_ptr[k];
  p.row_inv = p.row_perm;
  p.pats = p.pats_orig;
  finalize_plan(p, ap, ai, p.pats);
  if (p.too_large) return kTooLarge;
  return "";
}

void set_pivots(Plan& p, const i64* ap, const i64* ai, const std::vector<i32>& row_perm) {
  p.row_perm = row_perm;
  p.row_inv.assign(p.n, 0);
  p.swaps = 0;
  for (int k = 0; k < p.nblocks; ++k) {
    int b0 = p.block_ptr[k];
    for (int i = b0; i < p.block_ptr[k + 1]; ++i) {
      p.row_inv[b0 + row_perm[i]] = i - b0;
      if (row_perm[i] != i - b0) ++p.swaps;
    }
  }
  p.pivots_known = true;
  if (p.pivot_mode == PIVOT_EXACT) {
    std::vector<int> btf_col_perm(p.n);
    for (int c = 0; c < p.n; ++c) btf_col_perm[p.btf_col_inv[c]] = c;
    std::vector<i64> bp, bi;
    for (int k = 0; k < p.nblocks; ++k) {
      int b0 = p.block_ptr[k];
      if (p.block_ptr[k + 1] - b0 <= 1) continue;
      const std::vector<int>& cp = p.cperm[k];
      const std::vector<int>& ri = p.row_inv;
      block_csc(p, ap, ai, k, [&](int r) { return ri[b0 + cp[r]]; }, p.cperm_inv[k], bp, bi,
                btf_col_perm);
      symbolic_dfs(p.block_ptr[k + 1] - b0, bp, bi, p.pats[k]);
    }
  }
  finalize_plan(p, ap, ai, p.pats);
}

void pivot_pass_amap(const Plan& p, const std::vector<int>& cand_row, std::vector<i32>& amap_ptr,
                     std::vector<i32>& amap_idx, std::vector<i32>& row_perm) {
  const int n = p.n, ns = p.nslots();
  row_perm.assign(n, 0);
  std::vector<int> rinv(n), where(n, -1), slot_of(p.pcol_raw.size(), -1);
  for (int b = 0; b < p.nblocks; ++b)
    for (int i = p.block_ptr[b]; i < p.block_ptr[b + 1]; ++i)
      row_perm[i] = rinv[i] = i - p.block_ptr[b];
  amap_ptr.assign(ns + 1, 0);
  for (int k = 0; k < n; ++k) {
    const int b0 = p.block_ptr[p.pos_block[k]];
    for (int s = p.col_ptr[k]; s < p.col_ptr[k + 1]; ++s) where[p.slot_row[s]] = s;
    for (int t = p.pcol_ptr[k]; t < p.pcol_ptr[k + 1]; ++t) {
      const int s = where[b0 + rinv[b0 + p.pcol_q[t]]];
      slot_of[t] = s;
      if (s >= 0) ++amap_ptr[s + 1];
    }
    for (int s = p.col_ptr[k]; s < p.col_ptr[k + 1]; ++s) where[p.slot_row[s]] = -1;
    const int mr = cand_row[k];
    if (mr >= 0 && mr != k) {
      const int ok = row_perm[k], om = row_perm[mr];
      row_perm[k] = om;
      row_perm[mr] = ok;
      rinv[b0 + ok] = mr - b0;
      rinv[b0 + om] = k - b0;
    }
  }
  for (int s = 0; s < ns; ++s) amap_ptr[s + 1] += amap_ptr[s];
  amap_idx.assign(amap_ptr[ns], 0);
  std::vector<int> fill(amap_ptr.begin(), amap_ptr.end() - 1);
  for (size_t t = 0; t < slot_of.size(); ++t)
    if (slot_of[t] >= 0) amap_idx[fill[slot_of[t]]++] = p.pcol_raw[t];
}

void finalize_plan(Plan& p, const i64* ap, const i64* ai, const std::vector<Pattern>& pats) {
  const int n = p.n;
  p.col_ptr.assign(n + 1, 0);
  p.dslot.assign(n, 0);
  p.slot_row.clear();
  p.col_single.assign(n, 0);
  p.pos_block.assign(n, 0);
  p.nnz_l = p.nnz_u = 0;
  for (int k = 0; k < p.nblocks; ++k) {
    int b0 = p.block_ptr[k], nb = p.block_ptr[k + 1] - b0;
    const Pattern& s = pats[k];
    for (int c = 0; c < nb; ++c) {
      int kg = b0 + c;
      p.pos_block[kg] = k;
      p.col_single[kg] = nb == 1 && !p.no_singleton;
      p.col_ptr[kg] = (int)p.slot_row.size();
      for (int q = s.up[c]; q < s.up[c + 1]; ++q) p.slot_row.push_back(b0 + s.ui[q]);
      p.dslot[kg] = (int)p.slot_row.size() - 1;
      for (int q = s.lp[c]; q < s.lp[c + 1]; ++q) p.slot_row.push_back(b0 + s.li[q]);
      p.col_ptr[kg + 1] = (int)p.slot_row.size();
      p.nnz_u += s.up[c + 1] - s.up[c];
      p.nnz_l += s.lp[c + 1] - s.lp[c];
    }
  }
  const int ns = (int)p.slot_row.size();
  // slot lookup per column through a dense row map
  std::vector<int> where(n, -1);
  auto open_col = [&](int k) {
    for (int s = p.col_ptr[k]; s < p.col_ptr[k + 1]; ++s) where[p.slot_row[s]] = s;
  };
  auto close_col = [&](int k) {
    for (int s = p.col_ptr[k]; s < p.col_ptr[k + 1]; ++s) where[p.slot_row[s]] = -1;
  };
  p.upd_ptr.assign(ns + 1, 0);
  p.upd_dst.clear();
  p.flops_refactor = 0;
  {  // one int32 destination per update: refuse fills whose list would not index
    int64_t total = 0;
    for (int k = 0; k < n; ++k)
      for (int s = p.col_ptr[k]; s < p.dslot[k]; ++s) {
        const int j = p.slot_row[s];
        total += p.col_ptr[j + 1] - p.dslot[j] - 1;
      }
    p.too_large = total > (int64_t)0x7fffffff;
  }
  for (int k = 0; k < n && !p.too_large; ++k) {
    open_col(k);
    for (int s = p.col_ptr[k]; s < p.col_ptr[k + 1]; ++s) {
      p.upd_ptr[s] = (int)p.upd_dst.size();
      if (s < p.dslot[k]) {
        int j = p.slot_row[s];
        for (int q = p.dslot[j] + 1; q < p.col_ptr[j + 1]; ++q) {
          int w = where[p.slot_row[q]];
          p.upd_dst.push_back(w);  // symbolic closure guarantees w >= 0
        }
        p.flops_refactor += 2 * (p.col_ptr[j + 1] - p.dslot[j] - 1);
      }
    }
    p.flops_refactor += p.col_ptr[k + 1] - p.dslot[k] - 1;
    close_col(k);
  }
  p.upd_ptr[ns] = (int)p.upd_dst.size();

  // block-local AMD row index and positions of every raw entry
  std::vector<int> btf_col_perm(n);
  for (int c = 0; c < n; ++c) btf_col_perm[p.btf_col_inv[c]] = c;
  p.raw_slot.assign(p.nnz_raw, -1);
  p.offd_lower = p.pivot_mode == PIVOT_EXACT;
  std::vector<std::vector<std::pair<int, int>>> offd_rows(n);  // (pos col, raw)
  p.noffdiag = 0;
  auto in_map = [&](int R) {  // BTF row position -> solve position
    int b = p.pos_block[R], b0 = p.block_ptr[b];
    return b0 + p.row_inv[b0 + p.cperm[b][R - b0]];
  };
  auto out_map = [&](int Cc) {  // BTF column position -> solve position
    int b = p.pos_block[Cc], b0 = p.block_ptr[b];
    return b0 + p.cperm[b][Cc - b0];
  };
  // slots of the diagonal blocks, column by column (CSC order within each)
  for (int kg = 0; kg < n; ++kg) {
    int b = p.pos_block[kg], b0 = p.block_ptr[b];
    int oc = btf_col_perm[b0 + p.cperm_inv[b][kg - b0]];
    open_col(kg);
    for (i64 t = ap[oc]; t < ap[oc + 1]; ++t) {
      int r = (int)ai[t];
      if (r >= n) continue;
      int R = p.btf_row_inv[r];
      if (p.pos_block[R] != b) continue;
      p.raw_slot[t] = where[in_map(R)];
    }
    close_col(kg);
  }
  // off-diagonal block entries in (block row, block column, local column,
  // CSC) order; the reference keeps only those above the diagonal blocks,
  // the exact mode keeps those below (where BTF puts them).
  // Columns in BTF position order and their entries in CSC order give every
  // row its entries ordered by (block column, local column, CSC), the order
  // the reference's block-pair loops visit them (native_klu.rs:800-857).
  for (int Cc = 0; Cc < n; ++Cc) {
    const int bc = p.pos_block[Cc];
    const int oc = btf_col_perm[Cc];
    for (i64 t = ap[oc]; t < ap[oc + 1]; ++t) {
      int r = (int)ai[t];
      if (r >= n) continue;
      int R = p.btf_row_inv[r];
      const int br = p.pos_block[R];
      if (br == bc) continue;
      if (p.offd_lower ? bc > br : bc < br) continue;
      offd_rows[in_map(R)].push_back({out_map(Cc), (int)t});
      ++p.noffdiag;
    }
  }
  p.offd_ptr.assign(n + 1, 0);
  p.offd_col.clear();
  p.offd_raw.clear();
  for (int i = 0; i < n; ++i) {
    for (auto& e : offd_rows[i]) {
      p.offd_col.push_back(e.first);
      p.offd_raw.push_back(e.second);
    }
    p.offd_ptr[i + 1] = (int)p.offd_col.size();
  }
  {
    std::vector<std::vector<std::pair<int, int>>> cols(n);
    for (int i = 0; i < n; ++i)
      for (int e = p.offd_ptr[i]; e < p.offd_ptr[i + 1]; ++e)
        cols[p.offd_col[e]].push_back({i, p.offd_raw[e]});
    p.offdT_ptr.assign(n + 1, 0);
    p.offdT_row.clear();
    p.offdT_raw.clear();
    for (int c = 0; c < n; ++c) {
      for (auto& e : cols[c]) {
        p.offdT_row.push_back(e.first);
        p.offdT_raw.push_back(e.second);
      }
      p.offdT_ptr[c + 1] = (int)p.offdT_row.size();
    }
  }
  // raw entries summed into each slot, in CSC order
  std::vector<int> cnt(ns + 1, 0);
  for (i64 t = 0; t < p.nnz_raw; ++t)
    if (p.raw_slot[t] >= 0) ++cnt[p.raw_slot[t] + 1];
  for (int s = 0; s < ns; ++s) cnt[s + 1] += cnt[s];
  p.amap_ptr = cnt;
  p.amap_idx.assign(cnt[ns], 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (i64 t = 0; t < p.nnz_raw; ++t)
    if (p.raw_slot[t] >= 0) p.amap_idx[fill[p.raw_slot[t]]++] = (int)t;
  // row views
  std::vector<std::vector<std::pair<int, int>>> lr(n), ur(n);
  for (int k = 0; k < n; ++k)
    for (int s = p.dslot[k] + 1; s < p.col_ptr[k + 1]; ++s) lr[p.slot_row[s]].push_back({k, s});
  for (int k = n - 1; k >= 0; --k)
    for (int s = p.col_ptr[k]; s < p.dslot[k]; ++s) ur[p.slot_row[s]].push_back({k, s});
  auto flat = [n](std::vector<std::vector<std::pair<int, int>>>& v, std::vector<i32>& ptr,
                  std::vector<i32>& col, std::vector<i32>& slot) {
    ptr.assign(n + 1, 0);
    col.clear();
    slot.clear();
    for (int i = 0; i < n; ++i) {
      for (auto& e : v[i]) {
        col.push_back(e.first);
        slot.push_back(e.second);
      }
      ptr[i + 1] = (int)col.size();
    }
  };
  flat(lr, p.lrow_ptr, p.lrow_col, p.lrow_slot);
  flat(ur, p.urow_ptr, p.urow_col, p.urow_slot);
  // solve permutations
  p.in_pos.assign(n, 0);
  p.out_pos.assign(n, 0);
  for (int r = 0; r < n; ++r) p.in_pos[r] = in_map(p.btf_row_inv[r]);
  for (int c = 0; c < n; ++c) p.out_pos[c] = out_map(p.btf_col_inv[c]);
  // first-factor scatter lists (pivot independent)
  p.pcol_ptr.assign(n + 1, 0);
  p.pcol_raw.clear();
  p.pcol_q.clear();
  for (int kg = 0; kg < n; ++kg) {
    int b = p.pos_block[kg], b0 = p.block_ptr[b];
    int oc = btf_col_perm[b0 + p.cperm_inv[b][kg - b0]];
    for (i64 t = ap[oc]; t < ap[oc + 1]; ++t) {
      int r = (int)ai[t];
      if (r >= n) continue;
      int R = p.btf_row_inv[r];
      if (p.pos_block[R] != b) continue;
      p.pcol_raw.push_back((int)t);
      p.pcol_q.push_back(p.cperm[b][R - b0]);
    }
    p.pcol_ptr[kg + 1] = (int)p.pcol_raw.size();
  }
}

// ------------------------------------------------------------------ BBD
BbdDecomp bbd_decompose(int n, const i64* ap, const i64* ai, const int64_t* assignment,
                        int num_blocks) {
  std::vector<int> asg(n);
  for (int i = 0; i < n; ++i)
    asg[i] = (assignment[i] < 0 || assignment[i] >= num_blocks) ? -1 : (int)assignment[i];
  for (int col = 0; col < n; ++col) {  // bbd.rs:366-385
    if (asg[col] < 0) continue;
    for (i64 q = ap[col]; q < ap[col + 1]; ++q) {
      const int row = (int)ai[q];
      if (row < n && row != col && asg[row] >= 0 && asg[row] != asg[col]) {
        asg[col] = -1;
        break;
      }
    }
  }
  for (int col = 0; col < n; ++col)  // bbd.rs:391-407
    for (i64 q = ap[col]; q < ap[col + 1]; ++q) {
      const int row = (int)ai[q];
      if (row < n && row != col && asg[row] >= 0 && asg[col] >= 0 && asg[col] != asg[row])
        asg[row] = -1;
    }
  std::vector<std::vector<int>> blocks(std::max(num_blocks, 0));
  std::vector<int> border;
  for (int i = 0; i < n; ++i) (asg[i] < 0 ? border : blocks[asg[i]]).push_back(i);
  BbdDecomp d;
  for (auto& b : blocks) {
    if (b.empty()) continue;
    d.block_ptr.push_back((int)d.perm.size());
    for (int i : b) {
      d.perm.push_back(i);
      d.block_of.push_back(d.num_blocks);
    }
    ++d.num_blocks;
  }
  d.block_ptr.push_back((int)d.perm.size());
  d.border_start = (int)d.perm.size();
  for (int i : border) {
    d.perm.push_back(i);
    d.block_of.push_back(-1);
  }
  d.border_size = n - d.border_start;
  d.inv_perm.assign(n, 0);
  for (int k = 0; k < n; ++k) d.inv_perm[d.perm[k]] = k;
  return d;
}

}  // namespace gk
