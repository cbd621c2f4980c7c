// The reference's DenseSolver (crates/sim-core/src/solver.rs:596-724) on the
// device: the CSC values summed into a row-major n x n array, LU with partial
// pivoting (the first row holding the column's largest magnitude), then the
// forward and backward substitutions. The solver selector hands it the
// smallest systems (n <= 50, or n <= 200 when denser than 0.3, solver.rs:
// 215-258, 415-440), so one thread block does it all: the pivot search and
// every inner product run in the reference's order, and each trailing entry
// receives its updates k = 0, 1, ... one step at a time, which gives the
// reference's results bit for bit.
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.cuh"

namespace gk {

namespace {
constexpr unsigned FULL = 0xffffffffu;
}

// status: 2 (GPUKLU_FACTOR_FAILED) when a column has no nonzero candidate
// (solver.rs:655-657). A: n*n doubles; piv: n ints.
__global__ void __launch_bounds__(1024) k_dense_factor(int n, const int64_t* __restrict__ ap,
                                                       const int64_t* __restrict__ ai,
                                                       const double* __restrict__ ax,
                                                       double* A, int* piv, int* status) {
  __shared__ int s_piv, s_fail;
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t nn = (size_t)n * n;
  for (size_t e = tid; e < nn; e += nt) A[e] = 0.0;
  __syncthreads();
  // build_dense (:620-636): one thread per column keeps the CSC order of
  // its duplicates
  for (int col = tid; col < n; col += nt)
    for (int64_t t = ap[col]; t < ap[col + 1]; ++t) {
      const int64_t r = ai[t];
      if (r >= 0 && r < n) A[(size_t)r * n + col] = add(A[(size_t)r * n + col], ax[t]);
    }
  for (int i = tid; i < n; i += nt) piv[i] = i;
  if (tid == 0) s_fail = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {  // the first row holding the largest magnitude
      int p = k;
      double mx = fabs(A[(size_t)k * n + k]);
      for (int i = k + 1; i < n; ++i) {
        const double v = fabs(A[(size_t)i * n + k]);
        if (v > mx) {
          mx = v;
          p = i;
        }
      }
      s_piv = p;
      if (mx == 0.0) {
        s_fail = 1;
        atomicCAS(status, 0, 2);
      } else if (p != k) {
        const int t = piv[k];
        piv[k] = piv[p];
        piv[p] = t;
      }
    }
    __syncthreads();
    if (s_fail) return;  // uniform: every thread read the same flag
    const int p = s_piv;
    if (p != k)
      for (int j = tid; j < n; j += nt) {
        const double t = A[(size_t)k * n + j];
        A[(size_t)k * n + j] = A[(size_t)p * n + j];
        A[(size_t)p * n + j] = t;
      }
    __syncthreads();
    const double pv = A[(size_t)k * n + k];
    for (int i = k + 1 + tid; i < n; i += nt) A[(size_t)i * n + k] = A[(size_t)i * n + k] / pv;
    __syncthreads();
    const int m = n - k - 1;
    const size_t cells = (size_t)m * m;
    for (size_t e = tid; e < cells; e += nt) {
      const int i = k + 1 + (int)(e / m), j = k + 1 + (int)(e % m);
      A[(size_t)i * n + j] = sub(A[(size_t)i * n + j], mul(A[(size_t)i * n + k], A[(size_t)k * n + j]));
    }
    __syncthreads();
  }
}

// solve (:687-715), one warp: the lanes form 32 products at a time and lane
// 0 subtracts them in the reference's order. b lives in shared memory.
// status: 3 (GPUKLU_SOLVE_FAILED) on a zero diagonal.
__global__ void k_dense_solve(int n, const double* __restrict__ A, const int* __restrict__ piv,
                              const double* __restrict__ rhs, double* out, int* status) {
  extern __shared__ double b[];
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n; i += 32) b[i] = rhs[piv[i]];
  __syncwarp();
  for (int i = 0; i < n; ++i) {  // forward: L unit lower
    double s = b[i];
    for (int j0 = 0; j0 < i; j0 += 32) {
      const int j = j0 + lane;
      const double pr = j < i ? mul(A[(size_t)i * n + j], b[j]) : 0.0;
      const int cnt = min(32, i - j0);
      for (int t = 0; t < cnt; ++t) s = sub(s, __shfl_sync(FULL, pr, t));
    }
    if (lane == 0) b[i] = s;
    __syncwarp();
  }
  for (int i = n - 1; i >= 0; --i) {  // backward: b[j > i] already holds x[j]
    double s = b[i];
    for (int j0 = i + 1; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      const double pr = j < n ? mul(A[(size_t)i * n + j], b[j]) : 0.0;
      const int cnt = min(32, n - j0);
      for (int t = 0; t < cnt; ++t) s = sub(s, __shfl_sync(FULL, pr, t));
    }
    const double d = A[(size_t)i * n + i];
    if (d == 0.0) {
      if (lane == 0) atomicCAS(status, 0, 3);
      return;
    }
    if (lane == 0) b[i] = s / d;
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) out[i] = b[i];
}

void launch_dense_factor(int n, const int64_t* ap, const int64_t* ai, const double* ax,
                         double* A, int* piv, int* status, cudaStream_t s) {
  if (n <= 0) return;
  k_dense_factor<<<1, 1024, 0, s>>>(n, ap, ai, ax, A, piv, status);
}

void launch_dense_solve(int n, const double* A, const int* piv, const double* rhs, double* out,
                        int* status, cudaStream_t s) {
  if (n <= 0) return;
  const size_t bytes = (size_t)n * sizeof(double);
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(k_dense_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_dense_solve<<<1, 32, bytes, s>>>(n, A, piv, rhs, out, status);
}

}  // namespace gk
