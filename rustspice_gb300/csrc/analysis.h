// Host-side symbolic analysis for the GPU Newton inner loop.
//
// The orderings are the reference's: BTF (maximum transversal + Tarjan SCC,
// crates/sim-core/src/btf.rs:143-550), AMD per diagonal block
// (crates/sim-core/src/amd.rs:143-412) and the Gilbert-Peierls DFS symbolic
// factor (crates/sim-core/src/native_klu.rs:863-1014). They are integer-only
// and run once per sparsity pattern. Everything numeric runs on the device.
//
// The analysis produces a Plan: one flat "position space" in which all BTF
// diagonal blocks are concatenated, the LU values of every block live in one
// array of slots (column-major, per column: U rows ascending, the diagonal,
// then L rows ascending), and every raw CSC entry of the stamped matrix knows
// the slot it accumulates into.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gk {

using i64 = int64_t;
using i32 = int32_t;

// AMD ordering of a square pattern: returns perm (old -> new) and inv
// (new -> old).
void amd_order(int n, const i64* ap, const i64* ai, std::vector<int>& perm,
               std::vector<int>& inv);

struct BtfResult {
  std::vector<int> row_perm, col_perm, row_inv, col_inv, block_ptr;
  int nblocks = 0, max_block = 0;
};
BtfResult btf_decompose(int n, const i64* ap, const i64* ai);
bool structurally_irreducible(int n, const i64* ap, const i64* ai);

// Bordered-block-diagonal decomposition of a given partition (the
// reference's bbd_decompose, crates/sim-core/src/bbd.rs:355-485): nodes with
// an entry to another block are promoted to the border (column pass, then
// row pass), empty blocks are dropped, and perm[new] = old lists the blocks
// in order, then the border. num_blocks <= 1 after dropping means trivial.
struct BbdDecomp {
  int num_blocks = 0, border_start = 0, border_size = 0;
  std::vector<int> perm, inv_perm, block_ptr, block_of;  // block_of[new]: -1 border
};
BbdDecomp bbd_decompose(int n, const i64* ap, const i64* ai, const int64_t* assignment,
                        int num_blocks);

// Symbolic L/U pattern of an already permuted block, column by column.
struct Pattern {
  std::vector<int> lp, li, up, ui;  // U columns end with the diagonal
};
void symbolic_dfs(int n, const std::vector<i64>& pap, const std::vector<i64>& pai,
                  Pattern& s);

enum PivotMode : int { PIVOT_REFERENCE = 0, PIVOT_EXACT = 1 };

// Which of the reference's sparse solvers a plan restates:
// NATIVEKLU  native_klu.rs: BTF (n >= 4, >= 2 blocks, largest < n), AMD per
//            block, threshold pivoting, singleton rule for 1x1 blocks;
// SPARSELU   sparse_lu.rs: one block, AMD, no row exchanges, every pivot
//            below 1e-14 in magnitude set to +-1e-14 (:117, :495-499);
// SPARSELU_BTF sparse_lu_btf.rs: BTF when should_use_btf (btf.rs:560-573:
//            n >= 50, density <= 0.25) finds >= 2 blocks all below n
//            (:191-226), then one SparseLU per block; else one SparseLU.
enum SolverKind : int { KIND_NATIVEKLU = 0, KIND_SPARSELU = 1, KIND_SPARSELU_BTF = 2 };

// Everything the kernels need for one matrix pattern.
struct Plan {
  int n = 0;
  i64 nnz_raw = 0;
  int nblocks = 0;
  bool has_btf = false;
  std::vector<int> block_ptr;  // positions

  // Per block, the AMD column permutation (block local).
  std::vector<std::vector<int>> cperm, cperm_inv;
  // BTF permutations (identity when BTF is not kept).
  std::vector<int> btf_row_inv, btf_col_inv;

  // LU structure in position space.
  std::vector<i32> col_ptr;   // [n+1] slot range of column k
  std::vector<i32> dslot;     // [n] slot of the diagonal of column k
  std::vector<i32> slot_row;  // [nslots] position row of each slot
  // Left-looking updates: for U slot s (row j, column k, j < k) the
  // destination slots in column k of the L entries of column j, in L order.
  std::vector<i32> upd_ptr;   // [nslots+1]
  std::vector<i32> upd_dst;
  i64 flops_refactor = 0;

  // Pivot state: position-local row permutation per position (block local
  // index), as NativeKLU's row_perm / row_perm_inv.
  std::vector<i32> row_perm, row_inv;  // [n], block-local values
  int pivot_mode = PIVOT_REFERENCE;
  int kind = KIND_NATIVEKLU;
  // 1x1 blocks take the general +-1e-14 rule instead of the singleton rule
  // (SparseLU's blocks, and the BBD solver's, which the reference factors
  // with SparseLU)
  bool no_singleton = false;
  bool too_large = false;  // update lists beyond int32 indexing: not factorable here
  bool pivots_known = false;
  i64 swaps = 0;

  // Raw CSC entry -> target. Diagonal-block entries get an LU slot (or -1 if
  // they fall outside the symbolic pattern under the reference's pivot
  // rule); off-diagonal block entries get an off-diagonal index.
  std::vector<i32> raw_slot;     // [nnz_raw]
  std::vector<i32> amap_ptr;     // [nslots+1] raw entries summed into a slot, CSC order
  std::vector<i32> amap_idx;
  // Off-diagonal block entries used by the block solve, grouped by position
  // row; each is one raw entry (duplicates kept).
  std::vector<i32> offd_ptr;     // [n+1]
  std::vector<i32> offd_col;     // position column
  std::vector<i32> offd_raw;     // raw CSC index
  // The same entries grouped by position column (for A^T solves): rows and
  // raw indices, rows ascending.
  std::vector<i32> offdT_ptr, offdT_row, offdT_raw;
  bool offd_lower = false;       // true: forward block order (exact mode)

  // Row-oriented views of L and U for the dependency-driven solve.
  std::vector<i32> lrow_ptr, lrow_col, lrow_slot;  // columns ascending
  std::vector<i32> urow_ptr, urow_col, urow_slot;  // columns descending
  // Transposed views for A^T solves (adjoint): U^T rows are U columns,
  // L^T rows are L columns, already available through col_ptr.

  // Solve permutations.
  std::vector<i32> in_pos;   // [n] original row -> position
  std::vector<i32> out_pos;  // [n] original column -> position

  // First-factor (pivot discovery) inputs: per column k the raw entries and
  // the block-local AMD row index they scatter from.
  std::vector<i32> pcol_ptr;  // [n+1]
  std::vector<i32> pcol_raw;  // raw index
  std::vector<i32> pcol_q;    // block-local AMD row index (before pivoting)
  std::vector<i32> pos_block; // [n] block of each position

  // Columns of 1x1 blocks use the singleton rule (sum, |d| < 1e-300 -> 1e-14).
  std::vector<i32> col_single;  // [n]

  // Symbolic patterns per block: as analysed (no pivoting) and current.
  std::vector<Pattern> pats_orig, pats;

  i64 nnz_l = 0, nnz_u = 0, noffdiag = 0;
  int nslots() const { return (int)slot_row.size(); }
};

// Builds the Plan for pattern (ap, ai) of dimension n: BTF kept under the
// rule of the solver kind, AMD per block, symbolic DFS. Pivots start as the
// identity.
// given_blocks: boundaries of diagonal blocks the caller guarantees (no
// entry outside them); they replace the BTF, with the identity row order.
std::string analyze(int n, const i64* ap, const i64* ai, int pivot_mode, Plan& p,
                    const std::vector<int>* given_blocks = nullptr,
                    int kind = KIND_NATIVEKLU);

// Installs a pivot sequence (block-local row_perm for every position) found
// by the first factorization and rebuilds what depends on it: in exact mode
// the symbolic pattern of the row-permuted blocks; in both modes the raw
// entry -> slot map and the solve permutations.
void set_pivots(Plan& p, const i64* ap, const i64* ai, const std::vector<i32>& row_perm);

// The A scatter of the first factorization for a candidate pivot sequence,
// as slot lists for the refactorization: column k adds its raw entries (in
// the pivot pass's order) at the row positions that the candidate's swaps of
// earlier columns give them; entries landing outside the column's pivot-free
// pattern are left out (the pass adds them at working positions it never
// reads). cand_row[k]: the row position swapped into pivot k, or -1. Also
// returns the block-local row_perm the candidate produces.
void pivot_pass_amap(const Plan& p, const std::vector<int>& cand_row, std::vector<i32>& amap_ptr,
                     std::vector<i32>& amap_idx, std::vector<i32>& row_perm);

// Rebuilds slot maps, update lists, row views and permutations from the
// current per-block patterns and pivots.
void finalize_plan(Plan& p, const i64* ap, const i64* ai,
                   const std::vector<Pattern>& pats);

}  // namespace gk
