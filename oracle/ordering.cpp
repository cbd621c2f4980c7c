// Oracle (test infrastructure only): AMD and BTF orderings restated from
// crates/sim-core/src/amd.rs and crates/sim-core/src/btf.rs.
#include <algorithm>
#include <functional>
#include <queue>

#include "oracle.h"

namespace oracle {

// ============================================================== AMD
// amd.rs:143-160 (amd_order), :172-412 (AmdState).
namespace {
struct Amd {
  size_t n;
  UVec perm, inv_perm;
  std::vector<char> is_elem;   // NodeStatus::Element
  UVec degree;                 // NodeStatus::Variable(degree)
  std::vector<UVec> adj;
  // BinaryHeap<Reverse<(usize,usize)>> is a min-heap on (degree, node):
  // equal tuples are indistinguishable, so any binary heap pops the same
  // sequence (amd.rs:190, :268-288).
  std::priority_queue<std::pair<size_t, size_t>,
                      std::vector<std::pair<size_t, size_t>>,
                      std::greater<std::pair<size_t, size_t>>>
      heap;
  UVec marker;
  size_t cur = 0, num_elim = 0;

  static bool contains(const UVec& v, size_t x) {
    for (size_t y : v)
      if (y == x) return true;
    return false;
  }

  Amd(size_t n_, const i64* ap, const i64* ai) : n(n_) {  // amd.rs:207-257
    adj.assign(n, UVec());
    for (size_t col = 0; col < n; ++col) {
      for (i64 idx = ap[col]; idx < ap[col + 1]; ++idx) {
        size_t row = (size_t)ai[idx];
        if (row < n && row != col) {
          if (!contains(adj[col], row)) adj[col].push_back(row);
          if (!contains(adj[row], col)) adj[row].push_back(col);
        }
      }
    }
    is_elem.assign(n, 0);
    degree.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
      degree[i] = adj[i].size();
      heap.push({degree[i], i});
    }
    perm.assign(n, 0);
    inv_perm.assign(n, 0);
    marker.assign(n, 0);
  }

  bool find_min(size_t& out) {  // amd.rs:272-293
    while (!heap.empty()) {
      auto top = heap.top();
      heap.pop();
      size_t d = top.first, node = top.second;
      if (is_elem[node]) continue;
      if (d != degree[node]) {
        heap.push({degree[node], node});
        continue;
      }
      out = node;
      return true;
    }
    return false;
  }

  void absorb(size_t src, size_t dst) {  // amd.rs:346-369
    if (src == dst) return;
    UVec src_adj;
    src_adj.swap(adj[src]);
    for (size_t var : src_adj) {
      if (!is_elem[var]) {
        if (!contains(adj[dst], var)) adj[dst].push_back(var);
        UVec& av = adj[var];
        for (size_t q = 0; q < av.size(); ++q) {
          if (av[q] == src) {
            av[q] = dst;
            break;
          }
        }
      }
    }
  }

  void update_degree(size_t var) {  // amd.rs:372-411
    if (is_elem[var]) return;
    ++cur;
    size_t mk = cur;
    marker[var] = mk;
    size_t deg = 0;
    for (size_t a : adj[var]) {
      if (!is_elem[a]) {
        if (marker[a] != mk) {
          marker[a] = mk;
          ++deg;
        }
      } else {
        for (size_t e : adj[a]) {
          if (!is_elem[e] && marker[e] != mk) {
            marker[e] = mk;
            ++deg;
          }
        }
      }
    }
    degree[var] = deg;
    heap.push({deg, var});
  }

  void eliminate(size_t p) {  // amd.rs:296-343
    perm[p] = num_elim;
    inv_perm[num_elim] = p;
    ++num_elim;
    ++cur;
    size_t mk = cur;
    UVec nvars, nelems;
    for (size_t a : adj[p]) {
      if (!is_elem[a]) {
        if (marker[a] != mk) {
          marker[a] = mk;
          nvars.push_back(a);
        }
      } else {
        nelems.push_back(a);
      }
    }
    for (size_t e : nelems) {
      for (size_t a : adj[e]) {
        if (!is_elem[a] && a != p && marker[a] != mk) {
          marker[a] = mk;
          nvars.push_back(a);
        }
      }
    }
    is_elem[p] = 1;
    adj[p] = nvars;
    for (size_t e : nelems) absorb(e, p);
    for (size_t v : nvars) update_degree(v);
  }

  void run() {  // amd.rs:260-269
    while (num_elim < n) {
      size_t p;
      if (!find_min(p)) break;
      eliminate(p);
    }
  }
};
}  // namespace

AmdResult amd_order(size_t n, const i64* ap, const i64* ai) {
  AmdResult r;
  if (n == 0) return r;
  Amd a(n, ap, ai);
  a.run();
  r.perm = std::move(a.perm);
  r.inv_perm = std::move(a.inv_perm);
  return r;
}

// ============================================================== BTF
namespace {
std::vector<UVec> row_adjacency(size_t n, const i64* ap, const i64* ai) {
  // btf.rs:228-243
  std::vector<UVec> r(n);
  for (size_t col = 0; col < n; ++col)
    for (i64 idx = ap[col]; idx < ap[col + 1]; ++idx) {
      size_t row = (size_t)ai[idx];
      if (row < n) r[row].push_back(col);
    }
  return r;
}

// btf.rs:202-226 + augment_path :248-280. The recursion is replaced by an
// explicit stack that visits columns in the same order and applies the
// matching updates innermost-first, exactly as the recursive unwinding does.
// The per-row `visited = vec![false; n]` becomes a generation stamp, which
// marks the same set.
void maximum_transversal(size_t n, const std::vector<UVec>& r2c,
                         std::vector<long>& col_match,
                         std::vector<long>& row_match) {
  col_match.assign(n, -1);
  row_match.assign(n, -1);
  UVec visited(n, 0);
  struct Frame {
    size_t row, idx, col;
  };
  std::vector<Frame> st;
  for (size_t root = 0; root < n; ++root) {
    size_t gen = root + 1;
    st.clear();
    st.push_back({root, 0, 0});
    while (!st.empty()) {
      size_t top = st.size() - 1;
      size_t row = st[top].row;
      bool descended = false, found = false;
      while (st[top].idx < r2c[row].size()) {
        size_t col = r2c[row][st[top].idx++];
        if (visited[col] == gen) continue;
        visited[col] = gen;
        if (col_match[col] == -1) {
          col_match[col] = (long)row;
          row_match[row] = (long)col;
          found = true;
          break;
        }
        st[top].col = col;
        size_t mr = (size_t)col_match[col];
        st.push_back({mr, 0, 0});
        descended = true;
        break;
      }
      if (found) {
        st.pop_back();
        while (!st.empty()) {
          Frame& g = st.back();
          col_match[g.col] = (long)g.row;
          row_match[g.row] = (long)g.col;
          st.pop_back();
        }
        break;
      }
      if (!descended) st.pop_back();
    }
  }
}

// btf.rs:296-350 (only the second loop has an effect).
std::vector<UVec> directed_graph(size_t n, const std::vector<UVec>& r2c,
                                 const std::vector<long>& col_match) {
  std::vector<UVec> adj(n);
  for (size_t cj = 0; cj < n; ++cj) {
    if (col_match[cj] == -1) continue;
    size_t mr = (size_t)col_match[cj];
    for (size_t ci : r2c[mr])
      if (ci != cj) adj[ci].push_back(cj);
  }
  return adj;
}

// btf.rs:388-447, recursion replaced by an explicit stack with the same
// visit order; SCCs are emitted in the same (reverse topological) order.
std::vector<UVec> tarjan(size_t n, const std::vector<UVec>& adj) {
  std::vector<long> index(n, -1), low(n, -1);
  std::vector<char> on(n, 0);
  UVec stk;
  long counter = 0;
  std::vector<UVec> sccs;
  struct Frame {
    size_t v, ei;
  };
  std::vector<Frame> fr;
  for (size_t v0 = 0; v0 < n; ++v0) {
    if (index[v0] != -1) continue;
    index[v0] = low[v0] = counter++;
    stk.push_back(v0);
    on[v0] = 1;
    fr.push_back({v0, 0});
    while (!fr.empty()) {
      size_t v = fr.back().v;
      if (fr.back().ei < adj[v].size()) {
        size_t w = adj[v][fr.back().ei++];
        if (index[w] == -1) {
          index[w] = low[w] = counter++;
          stk.push_back(w);
          on[w] = 1;
          fr.push_back({w, 0});
        } else if (on[w]) {
          low[v] = std::min(low[v], index[w]);
        }
        continue;
      }
      if (low[v] == index[v]) {
        UVec scc;
        while (true) {
          size_t w = stk.back();
          stk.pop_back();
          on[w] = 0;
          scc.push_back(w);
          if (w == v) break;
        }
        sccs.push_back(std::move(scc));
      }
      fr.pop_back();
      if (!fr.empty()) {
        size_t u = fr.back().v;
        low[u] = std::min(low[u], low[v]);
      }
    }
  }
  return sccs;
}
}  // namespace

Btf btf_decompose(size_t n, const i64* ap, const i64* ai) {  // btf.rs:143-177
  Btf b;
  if (n == 0) {
    b.block_ptr = {0};
    return b;
  }
  auto r2c = row_adjacency(n, ap, ai);
  std::vector<long> cm, rm;
  maximum_transversal(n, r2c, cm, rm);
  size_t rank = 0;
  for (long c : cm)
    if (c != -1) ++rank;
  auto adj = directed_graph(n, r2c, cm);
  auto sccs = tarjan(n, adj);
  // build_permutations, btf.rs:457-550
  std::reverse(sccs.begin(), sccs.end());
  b.block_ptr.push_back(0);
  for (auto& scc : sccs) {
    size_t cnt = 0;
    for (size_t col : scc) {
      if (cm[col] != -1) {
        b.col_perm.push_back(col);
        b.row_perm.push_back((size_t)cm[col]);
        ++cnt;
      }
    }
    if (cnt == 0) continue;
    b.block_ptr.push_back(b.col_perm.size());
    if (cnt == 1) ++b.num_singletons;
    b.max_block_size = std::max(b.max_block_size, cnt);
  }
  std::vector<char> used(n, 0);
  for (size_t r : b.row_perm) used[r] = 1;
  for (size_t col = 0; col < n; ++col) {
    if (cm[col] != -1) continue;
    b.col_perm.push_back(col);
    for (size_t row = 0; row < n; ++row) {
      if (!used[row]) {
        b.row_perm.push_back(row);
        used[row] = 1;
        break;
      }
    }
    b.block_ptr.push_back(b.col_perm.size());
    ++b.num_singletons;
  }
  b.num_blocks = b.block_ptr.size() - 1;
  b.structural_rank = rank;
  b.row_perm_inv.assign(n, 0);
  b.col_perm_inv.assign(n, 0);
  for (size_t i = 0; i < b.row_perm.size(); ++i) b.row_perm_inv[b.row_perm[i]] = i;
  for (size_t i = 0; i < b.col_perm.size(); ++i) b.col_perm_inv[b.col_perm[i]] = i;
  return b;
}

bool should_use_btf(size_t n, size_t nnz) {  // btf.rs:560-573
  if (n < 50) return false;
  double density = (double)nnz / (double)(n * n);
  return !(density > 0.25);
}

}  // namespace oracle
