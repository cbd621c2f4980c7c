// Kernels of the bordered-block-diagonal (BBD) solver
// (crates/sim-core/src/bbd_solver.rs:633-979, restated for the GPU).
//
// The diagonal blocks form one block-diagonal matrix M that the regular
// factor kernels handle (its BTF finds the blocks). Around them:
//  * ysolve  - Y_k = B_k^-1 R_k for the border columns that touch block k:
//              one warp per tile of 32 columns, lanes over the columns, rows
//              of L then U in order (the row-oriented views of the plan);
//              tiles live in L2-resident [block size][32] arrays.
//  * schur   - S = B_T - sum_k C_k Y_k, one warp per border column, one lane
//              summing in a fixed order (deterministic).
//  * dense LU of S without pivoting, rows and columns in the AMD order of
//              S's structural pattern (the reference factors S with its
//              no-pivot, AMD-ordered SparseLU), in 32-wide panels: panel
//              factor, row-block triangular solve, trailing update in 64x64
//              shared-memory tiles.
//  * the border right-hand side, the R x_T product and the recombination.
#include "kernels.cuh"

namespace gk {
namespace {

__device__ __forceinline__ double perturb_tiny(double d) {  // sparse_lu.rs no-pivot rule
  if (fabs(d) < 1e-14) return d >= 0.0 ? 1e-14 : -1e-14;
  return d;
}

__global__ void k_bbd_ysolve(DPlan P, const double* __restrict__ lu,
                             const double* __restrict__ ax, BbdArgs B, double* ybuf) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= B.ntiles) return;
  const int b0 = B.tile_pos0[t], sz = B.tile_size[t];
  double* const Y = ybuf + B.tile_off[t];
  for (int i = 0; i < sz; ++i) Y[(long long)i * 32 + lane] = 0.0;
  __syncwarp();
  if (lane == 0)  // R entries in CSC order (duplicates add in that order)
    for (int e = B.init_ptr[t]; e < B.init_ptr[t + 1]; ++e) Y[B.init_code[e]] += ax[B.init_raw[e]];
  __syncwarp();
  // One row's dot product over its entries [e0, e1): the indices of eight
  // entries load together, then their factor values and Y values, so a row
  // costs two memory round trips per eight entries; the next row's range is
  // read one row ahead.
  auto row_dot = [&](const int* slot, const int* col, int e0, int e1, double v) {
    double w = 0.0;
    for (int e = e0; e < e1; e += 8) {
      int sl[8], cl[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (e + u < e1) {
          sl[u] = slot[e + u];
          cl[u] = col[e + u];
        }
      double lv[8], yv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (e + u < e1) {
          lv[u] = lu[sl[u]];
          yv[u] = Y[(long long)(cl[u] - b0) * 32 + lane];
        }
#pragma unroll
      for (int u = 0; u < 8; u += 2) {
        if (e + u < e1) v = fma(-lv[u], yv[u], v);
        if (e + u + 1 < e1) w = fma(-lv[u + 1], yv[u + 1], w);
      }
    }
    return v + w;
  };
  {  // L, unit diagonal
    int e0 = P.lrow_ptr[b0], e1 = P.lrow_ptr[b0 + 1];
    for (int i = 0; i < sz; ++i) {
      const int ce0 = e0, ce1 = e1;
      if (i + 1 < sz) {
        e0 = e1;
        e1 = P.lrow_ptr[b0 + i + 2];
      }
      Y[(long long)i * 32 + lane] =
          row_dot(P.lrow_slot, P.lrow_col, ce0, ce1, Y[(long long)i * 32 + lane]);
    }
  }
  {  // U
    int e0 = P.urow_ptr[b0 + sz - 1], e1 = P.urow_ptr[b0 + sz];
    double dg = lu[P.dslot[b0 + sz - 1]];
    for (int i = sz - 1; i >= 0; --i) {
      const int ce0 = e0, ce1 = e1;
      const double cdg = dg;
      if (i > 0) {
        e1 = e0;
        e0 = P.urow_ptr[b0 + i - 1];
        dg = lu[P.dslot[b0 + i - 1]];
      }
      Y[(long long)i * 32 + lane] =
          row_dot(P.urow_slot, P.urow_col, ce0, ce1, Y[(long long)i * 32 + lane]) / cdg;
    }
  }
}

// S column j (column-major, leading dimension bs): B_T entries, then
// -C_k Y_k for every tile column that holds border column j.
__global__ void k_bbd_schur(const double* __restrict__ ax, BbdArgs B,
                            const double* __restrict__ ybuf, double* S) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= B.bs) return;
  double* const col = S + (long long)j * B.bs;
  for (int r = lane; r < B.bs; r += 32) col[r] = 0.0;
  __syncwarp();
  if (lane == 0) {
    for (int e = B.bt_ptr[j]; e < B.bt_ptr[j + 1]; ++e) col[B.bt_row[e]] += ax[B.bt_raw[e]];
    for (int q = B.yref_ptr[j]; q < B.yref_ptr[j + 1]; ++q) {
      const int code = B.yref[q];  // (tile << 5) | lane
      const int t = code >> 5, l = code & 31;
      const double* Y = ybuf + B.tile_off[t];
      const int blk = B.tile_blk[t];
      for (int e = B.c_ptr[blk]; e < B.c_ptr[blk + 1]; ++e)
        col[B.c_row[e]] = fma(-ax[B.c_raw[e]], Y[(long long)B.c_pos[e] * 32 + l], col[B.c_row[e]]);
    }
  }
}

// Panel factorisation of columns [k0, k0+nb) over rows k0..bs-1.
// Panel factorization of columns [k0, k0+nb) in two launches: k_dlu_diag
// factors the nb x nb diagonal block in place (shared memory, one lane per
// row, columns in order); k_dlu_panel then eliminates every row below it
// against that block's U, one thread per row, column by column. Every element
// sees the operations of a column-by-column panel in the same order, so the
// factor is the same bit for bit.
__global__ void k_dlu_diag(double* S, int bs, int k0, int nb) {
  __shared__ double D[32][33];  // D[r][c] = S(k0 + r, k0 + c)
  const int r = threadIdx.x;
  for (int c = 0; c < nb; ++c)
    if (r < nb) D[r][c] = S[(long long)(k0 + c) * bs + k0 + r];
  __syncwarp();
  for (int c = 0; c < nb; ++c) {
    const double d = perturb_tiny(D[c][c]);
    __syncwarp();
    if (r == c) D[c][c] = d;
    if (r > c && r < nb) {
      const double l = D[r][c] / d;
      D[r][c] = l;
      for (int c2 = c + 1; c2 < nb; ++c2) D[r][c2] = fma(-l, D[c][c2], D[r][c2]);
    }
    __syncwarp();
  }
  for (int c = 0; c < nb; ++c)
    if (r < nb) S[(long long)(k0 + c) * bs + k0 + r] = D[r][c];
}

__global__ void __launch_bounds__(256) k_dlu_panel(double* S, int bs, int k0, int nb) {
  __shared__ double D[32][33];  // the factored diagonal block
  for (int q = threadIdx.x; q < nb * nb; q += blockDim.x) {
    const int c = q / nb, r = q % nb;
    D[r][c] = S[(long long)(k0 + c) * bs + k0 + r];
  }
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= bs) return;
  double a[32];
#pragma unroll
  for (int c = 0; c < 32; ++c)
    if (c < nb) a[c] = S[(long long)(k0 + c) * bs + r];
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    if (c < nb) {
      const double l = a[c] / D[c][c];
      a[c] = l;
#pragma unroll
      for (int c2 = c + 1; c2 < 32; ++c2)
        if (c2 < nb) a[c2] = fma(-l, D[c][c2], a[c2]);
    }
  }
#pragma unroll
  for (int c = 0; c < 32; ++c)
    if (c < nb) S[(long long)(k0 + c) * bs + r] = a[c];
}

// U12 = L11^-1 A12 for the rows of the panel, one thread per column, L11 in
// shared memory.
__global__ void k_dlu_trsm(double* S, int bs, int k0, int nb) {
  __shared__ double L[32][33];  // L[i][m] = S(k0 + i, k0 + m)
  for (int q = threadIdx.x; q < nb * nb; q += blockDim.x) {
    const int m = q / nb, i = q % nb;
    L[i][m] = S[(long long)(k0 + m) * bs + k0 + i];
  }
  __syncthreads();
  const int j = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= bs) return;
  double* const col = S + (long long)j * bs;
  for (int i = 1; i < nb; ++i) {
    double v = col[k0 + i];
    for (int m = 0; m < i; ++m) v = fma(-L[i][m], col[k0 + m], v);
    col[k0 + i] = v;
  }
}

// A22 -= L21 U12 on 64x64 tiles; 256 threads, 4x4 outputs each.
__global__ void k_dlu_update(double* S, int bs, int k0, int nb) {
  __shared__ double Ls[32][65], Us[32][65];
  const int r0 = k0 + nb + blockIdx.y * 64, c0 = k0 + nb + blockIdx.x * 64;
  const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
  for (int q = tid; q < 64 * nb; q += 256) {
    const int m = q / 64, i = q % 64;
    const int r = r0 + i, c = c0 + i;
    Ls[m][i] = r < bs ? S[(long long)(k0 + m) * bs + r] : 0.0;
    Us[m][i] = c < bs ? S[(long long)c * bs + k0 + m] : 0.0;
  }
  __syncthreads();
  double acc[4][4] = {};
  for (int m = 0; m < nb; ++m) {
    double a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = Ls[m][tr * 4 + u];
      b[u] = Us[m][tc * 4 + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = r0 + tr * 4 + u, c = c0 + tc * 4 + v;
      if (r < bs && c < bs) S[(long long)c * bs + r] -= acc[u][v];
    }
}

// x <- S^-1 x with the unit-lower / upper factors, one block.
__global__ void k_dlu_solve(const double* __restrict__ S, int bs, double* x) {
  for (int c = 0; c < bs; ++c) {
    __syncthreads();
    const double xc = x[c];
    __syncthreads();
    for (int r = c + 1 + threadIdx.x; r < bs; r += blockDim.x)
      x[r] = fma(-S[(long long)c * bs + r], xc, x[r]);
  }
  for (int c = bs - 1; c >= 0; --c) {
    __syncthreads();
    if (threadIdx.x == 0) x[c] = x[c] / S[(long long)c * bs + c];
    __syncthreads();
    const double xc = x[c];
    for (int r = threadIdx.x; r < c; r += blockDim.x) x[r] = fma(-S[(long long)c * bs + r], xc, x[r]);
  }
}

// bb[j] = rhs[border row j] - sum_c C[j][c] z[c]  (row lists in CSC order)
__global__ void k_bbd_border_rhs(const double* __restrict__ ax, const double* __restrict__ rhs,
                                 const double* __restrict__ z, BbdArgs B, double* bb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B.bs) return;
  double v = rhs[B.bperm[j]];
  for (int e = B.crow_ptr[j]; e < B.crow_ptr[j + 1]; ++e)
    v = fma(-ax[B.crow_raw[e]], z[B.crow_col[e]], v);
  bb[j] = v;
}

// w[m] = sum_j R[m][j] xT[j] over the rows of M
__global__ void k_bbd_rmatvec(const double* __restrict__ ax, const double* __restrict__ xT,
                              BbdArgs B, double* w) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= B.border_start) return;
  double v = 0.0;
  for (int e = B.rrow_ptr[m]; e < B.rrow_ptr[m + 1]; ++e)
    v = fma(ax[B.rrow_raw[e]], xT[B.rrow_col[e]], v);
  w[m] = v;
}

__global__ void k_gather(double* dst, const double* __restrict__ src,
                         const int* __restrict__ idx, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

__global__ void k_bbd_combine(const double* __restrict__ z, const double* __restrict__ w2,
                              const double* __restrict__ xT, BbdArgs B, double* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < B.border_start)
    x[B.perm[i]] = z[i] - w2[i];
  else if (i < B.border_start + B.bs)
    x[B.bperm[i - B.border_start]] = xT[i - B.border_start];
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

void launch_bbd_ysolve(const DPlan& P, const double* lu, const double* ax, const BbdArgs& B,
                       double* ybuf, cudaStream_t s) {
  if (B.ntiles > 0) k_bbd_ysolve<<<cdiv(B.ntiles, 4), 128, 0, s>>>(P, lu, ax, B, ybuf);
}

void launch_bbd_schur(const double* ax, const BbdArgs& B, const double* ybuf, double* S,
                      cudaStream_t s) {
  k_bbd_schur<<<cdiv(B.bs, 4), 128, 0, s>>>(ax, B, ybuf, S);
}

void launch_dense_lu(double* S, int bs, cudaStream_t s) {
  const int nb = 32;
  for (int k0 = 0; k0 < bs; k0 += nb) {
    const int w = bs - k0 < nb ? bs - k0 : nb;
    const int rest = bs - k0 - w;
    k_dlu_diag<<<1, 32, 0, s>>>(S, bs, k0, w);
    if (rest <= 0) break;
    k_dlu_panel<<<cdiv(rest, 256), 256, 0, s>>>(S, bs, k0, w);
    k_dlu_trsm<<<cdiv(rest, 128), 128, 0, s>>>(S, bs, k0, w);
    dim3 g(cdiv(rest, 64), cdiv(rest, 64));
    k_dlu_update<<<g, 256, 0, s>>>(S, bs, k0, w);
  }
}

void launch_dense_lu_solve(const double* S, int bs, double* x, cudaStream_t s) {
  k_dlu_solve<<<1, 1024, 0, s>>>(S, bs, x);
}

void launch_bbd_border_rhs(const double* ax, const double* rhs, const double* z,
                           const BbdArgs& B, double* bb, cudaStream_t s) {
  k_bbd_border_rhs<<<cdiv(B.bs, 128), 128, 0, s>>>(ax, rhs, z, B, bb);
}

void launch_bbd_rmatvec(const double* ax, const double* xT, const BbdArgs& B, double* w,
                        cudaStream_t s) {
  if (B.border_start > 0) k_bbd_rmatvec<<<cdiv(B.border_start, 128), 128, 0, s>>>(ax, xT, B, w);
}

void launch_gather(double* dst, const double* src, const int* idx, int n, cudaStream_t s) {
  if (n > 0) k_gather<<<cdiv(n, 256), 256, 0, s>>>(dst, src, idx, n);
}

void launch_bbd_combine(const double* z, const double* w2, const double* xT, const BbdArgs& B,
                        double* x, cudaStream_t s) {
  const int n = B.border_start + B.bs;
  k_bbd_combine<<<cdiv(n, 256), 256, 0, s>>>(z, w2, xT, B, x);
}

}  // namespace gk
