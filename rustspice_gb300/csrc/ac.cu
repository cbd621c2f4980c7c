// AC small-signal sweep over many frequencies at once (the reference's .ac:
// crates/sim-core/src/engine.rs:829-930, complex_solver.rs:28-144).
//
// One thread block per frequency point keeps the dense complex system in
// shared memory (n up to 118), or, for larger systems, in its own slice of a
// global scratch (L2 / HBM; blocks loop over the frequencies): it fills
// Y(w) = G + jwC cell by cell (G from the DC stamp at the operating point,
// the capacitor terms +-w*C in insertion order), then runs the reference's
// dense LU with partial pivoting and the back substitution. Complex arithmetic is num-complex's (0.4.6): a*b = (ar br -
// ai bi, ar bi + ai br), a/b = ((ar br + ai bi)/n, (ai br - ar bi)/n) with
// n = br^2 + bi^2, |a| = hypot(ar, ai). Every element sees the reference's
// operations in the reference's order (compiled without contraction), so the
// solutions match a scalar evaluation bit for bit wherever the magnitudes
// that pick the pivots agree.
#include "kernels.cuh"

namespace gk {
namespace {

struct Cx {
  double re, im;
};
__device__ __forceinline__ Cx csub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ Cx cmul(Cx a, Cx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ Cx cdiv(Cx a, Cx b) {
  const double n = b.re * b.re + b.im * b.im;
  const double re = a.re * b.re + a.im * b.im;
  const double im = a.im * b.re - a.re * b.im;
  return {re / n, im / n};
}

// One frequency: M the n x n system (row-major; shared or global), x, pr,
// bv, bi in shared memory.
__device__ void ac_point(const AcArgs& A, long long f, Cx* M, Cx* x, Cx* pr, double* bv,
                         int* bi, int& s_fail) {
  const int n = A.n, tid = threadIdx.x, nt = blockDim.x;
  const double omega = 2.0 * 3.141592653589793 * A.freqs[f];
  for (int q = tid; q < n * n; q += nt) M[q] = Cx{0.0, 0.0};
  if (tid == 0) s_fail = 0;
  __syncthreads();
  for (int c = tid; c < A.ncell; c += nt) {  // each cell's terms in insertion order
    double re = 0.0, im = 0.0;
    for (int t = A.re_ptr[c]; t < A.re_ptr[c + 1]; ++t) re = re + A.ax[A.re_idx[t]];
    for (int t = A.im_ptr[c]; t < A.im_ptr[c + 1]; ++t) {
      const int code = A.im_code[t];
      const double y = omega * A.cap[code >> 1];
      im = im + ((code & 1) ? -y : y);
    }
    M[(size_t)A.cell_row[c] * n + A.cell_col[c]] = Cx{re, im};
  }
  if (tid == 0) M[0] = Cx{1.0, 0.0};  // ground row: 1 on the diagonal
  for (int i = tid; i < n; i += nt) x[i] = i == 0 ? Cx{0.0, 0.0} : Cx{A.rhs[2 * i], A.rhs[2 * i + 1]};
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // the first row of largest magnitude in column k, from row k down
    double best = -1.0;
    int brow = n;
    for (int i = k + tid; i < n; i += nt) {
      const Cx v = M[(size_t)i * n + k];
      const double m = hypot(v.re, v.im);
      if (m > best) {
        best = m;
        brow = i;
      }
    }
    bv[tid] = best;
    bi[tid] = brow;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) {
        const double ov = bv[tid + s];
        const int oi = bi[tid + s];
        if (ov > bv[tid] || (ov == bv[tid] && oi < bi[tid])) {
          bv[tid] = ov;
          bi[tid] = oi;
        }
      }
      __syncthreads();
    }
    const int mr = bi[0];
    __syncthreads();
    if (mr != k) {
      for (int j = tid; j < n; j += nt) {
        const Cx t = M[(size_t)k * n + j];
        M[(size_t)k * n + j] = M[(size_t)mr * n + j];
        M[(size_t)mr * n + j] = t;
      }
      if (tid == 0) {
        const Cx t = x[k];
        x[k] = x[mr];
        x[mr] = t;
      }
      __syncthreads();
    }
    const Cx piv = M[(size_t)k * n + k];
    if (hypot(piv.re, piv.im) < 1e-30) {
      if (tid == 0) s_fail = 1;
      break;
    }
    for (int i = k + 1 + tid; i < n; i += nt) M[(size_t)i * n + k] = cdiv(M[(size_t)i * n + k], piv);
    __syncthreads();
    const int w = n - k - 1;
    for (int q = tid; q < w * (w + 1); q += nt) {  // (w rows) x (w columns + the rhs)
      const int i = k + 1 + q / (w + 1), jj = q % (w + 1);
      const Cx fct = M[(size_t)i * n + k];
      if (jj < w) {
        const int j = k + 1 + jj;
        M[(size_t)i * n + j] = csub(M[(size_t)i * n + j], cmul(fct, M[(size_t)k * n + j]));
      } else {
        x[i] = csub(x[i], cmul(fct, x[k]));
      }
    }
    __syncthreads();
  }
  __syncthreads();
  if (!s_fail) {
    for (int i = n - 1; i >= 0; --i) {  // back substitution, terms in ascending order
      for (int j = i + 1 + tid; j < n; j += nt) pr[j] = cmul(M[(size_t)i * n + j], x[j]);
      __syncthreads();
      if (tid == 0) {
        Cx v = x[i];
        for (int j = i + 1; j < n; ++j) v = csub(v, pr[j]);
        const Cx piv = M[(size_t)i * n + i];
        if (hypot(piv.re, piv.im) < 1e-30)
          s_fail = 1;
        else
          x[i] = cdiv(v, piv);
      }
      __syncthreads();
      if (s_fail) break;
    }
  }
  if (s_fail) {
    if (tid == 0) atomicExch(A.status, 1);
    __syncthreads();
    return;
  }
  for (int i = tid; i < n; i += nt) {
    A.out_re[f * n + i] = x[i].re;
    A.out_im[f * n + i] = x[i].im;
  }
  __syncthreads();
}

// Systems that fit one block's shared memory.
__global__ void __launch_bounds__(256) k_ac_dense(AcArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = A.n, nt = blockDim.x;
  Cx* const M = reinterpret_cast<Cx*>(smem_raw);  // row-major n x n
  Cx* const x = M + (size_t)n * n;
  Cx* const pr = x + n;                            // products of one back-substitution row
  double* const bv = reinterpret_cast<double*>(pr + n);  // pivot search: values
  int* const bi = reinterpret_cast<int*>(bv + nt);        //               rows
  __shared__ int s_fail;
  ac_point(A, blockIdx.x, M, x, pr, bv, bi, s_fail);
}

// Larger systems: each block's matrix in its slice of the global scratch,
// the block looping over the frequencies.
__global__ void __launch_bounds__(256) k_ac_dense_global(AcArgs A, int nf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = A.n, nt = blockDim.x;
  Cx* const M = reinterpret_cast<Cx*>(A.scratch) + (size_t)blockIdx.x * n * n;
  Cx* const x = reinterpret_cast<Cx*>(smem_raw);
  Cx* const pr = x + n;
  double* const bv = reinterpret_cast<double*>(pr + n);
  int* const bi = reinterpret_cast<int*>(bv + nt);
  __shared__ int s_fail;
  for (long long f = blockIdx.x; f < nf; f += gridDim.x) ac_point(A, f, M, x, pr, bv, bi, s_fail);
}

}  // namespace

size_t ac_smem_bytes(int n, int threads) {
  return (size_t)16 * ((size_t)n * n + 2 * (size_t)n) + (size_t)12 * threads + 16;
}

bool ac_fits_shared(int n) { return ac_smem_bytes(n, 256) <= 227 * 1024; }

void launch_ac_dense(const AcArgs& a, int nf, cudaStream_t s) {
  const int threads = 256;
  const size_t bytes = ac_smem_bytes(a.n, threads);
  cudaFuncSetAttribute(k_ac_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_ac_dense<<<nf, threads, bytes, s>>>(a);
}

void launch_ac_dense_global(const AcArgs& a, int nf, int blocks, cudaStream_t s) {
  const int threads = 256;
  const size_t bytes = (size_t)32 * a.n + (size_t)12 * threads + 16;
  cudaFuncSetAttribute(k_ac_dense_global, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_ac_dense_global<<<blocks, threads, bytes, s>>>(a, nf);
}

}  // namespace gk
