// Dense LU of the BBD solver's Schur complement S (crates/sim-core/src/
// bbd_solver.rs:811-896 factors S without pivoting, in the AMD order of its
// structural pattern, with SparseLU's +-1e-14 rule for tiny pivots) as one
// cooperative kernel, and the FP64 tensor-core (DMMA) probe that decided how
// its trailing updates run.
//
// FP64 on this part issues one warp instruction per 64 cycles per SM
// sub-partition (16 per SM) whatever the active lanes, and a dependent FP64
// operation waits about 64 cycles, so the panel work - short chains of
// dependent divisions and products - sets the pace unless it is kept short
// and off the critical path:
//   - S (column-major, bs x bs, a few MB) stays in L2; two blocks per SM walk
//     the 32-wide panels with two grid barriers per panel;
//   - the 32 x 32 diagonal block is factored by four warps with the rows in
//     registers, each step's pivot row published through shared memory
//     already divided by the pivot (one reciprocal per pivot, fast_rcp: a
//     float seed and one FP64 Newton step, relative error about 1e-14), so
//     a step costs one FMA per row;
//   - it is factored ahead: block 0 updates the next panel's diagonal tile
//     first and factors it at once, while the other blocks take the other
//     tiles from a counter (except the block sharing block 0's SM, which
//     would compete with that chain for the FP64 pipes);
//   - the rows below the diagonal block (L21 = A21 U11^-1, multiplying by the
//     pivot reciprocals) and right of it (U12 = L11^-1 A12, right-looking)
//     go one per warp, lanes over the 32 entries, round robin over the
//     grid's warps;
//   - the trailing update A22 -= L21 U12 runs in 32 x 32 tiles: FP64 FMA in
//     registers (2 x 2 outputs per thread) or mma.sync m8n8k4 f64 (two 8 x 8
//     outputs per warp); the DMMA probe measured no gain over DFMA here.
// The order of operations differs from the panel kernels in bbd.cu (which
// divide, and accumulate the triangular solve row by row), so the factors
// agree to rounding, not bit for bit.
//
// Every grid-barrier wait is bounded: after kSpinLimit polls the block sets
// DS_TIMEOUT and every block leaves the panel loop. Every read of S is an
// ld.cg (L2): other SMs rewrite it between phases, and a line left in this
// SM's L1 would be stale.
#include <cuda_runtime.h>

#include "batch_common.cuh"
#include "device.cuh"
#include "kernels.cuh"

namespace gk {
namespace {

constexpr int kPanel = 32;
constexpr int kLuThreads = 256;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double tiny_pivot(double d) {  // sparse_lu.rs:495-499
  if (fabs(d) < 1e-14) return d >= 0.0 ? 1e-14 : -1e-14;
  return d;
}

// d += a * b for one m8n8k4 f64 tile: a, b one element per lane, d two.
__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
      : "+d"(d0), "+d"(d1)
      : "d"(a), "d"(b));
}

// Grid barrier over `nblocks` co-resident blocks: bar[0] counts arrivals over
// the launch, bar[1] holds the last released generation. Returns false when
// the launch has failed (this block's wait ran out, or another block's did).
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, int* status) {
  __syncthreads();
  if (threadIdx.x == 0) {
    ++gen;
    __threadfence();
    const unsigned arrived = atomicAdd(&bar[0], 1u) + 1u;
    if (arrived == gen * nblocks) {
      st_release(&bar[1], gen);
    } else {
      unsigned spins = 0;
      while (ld_acquire(&bar[1]) < gen) {
        if (++spins > kSpinLimit) {
          atomicCAS(status, DS_OK, DS_TIMEOUT);
          break;
        }
        if ((spins & 63u) == 0 && *(volatile int*)status != DS_OK) break;
        if (spins > 32) __nanosleep(64);
      }
    }
  }
  __syncthreads();
  return *(volatile int*)status == DS_OK;
}

// Warps 0-3 factor the nb x nb diagonal block at S(k0, k0) (nb <= 32; the
// rest of the 32 x 32 frame is the identity) and write it back to S if
// `store`, and to Dsh (Dsh[r][c]) if given. Warp w holds rows w, w+4, ...,
// lane j column j. At step c the warp owning row c publishes it through
// shared memory with the entries right of the pivot already divided by the
// pivot (one product per lane), so every row below updates with a single
// FMA per lane; the column of multipliers is divided by its pivot at the
// end. One FP64 instruction per row and step is what a step costs, at one
// warp instruction per 64 cycles per SM sub-partition. The published rows
// alternate between two buffers, so one barrier per step keeps a buffer
// from being rewritten while a slower warp still reads it. prow: 2 x 33 +
// 32 doubles of shared memory; named barrier 1 over the 128 threads.
__device__ __noinline__ void factor_diag(double* S, int bs, int k0, int nb, bool store,
                                         double (*Dsh)[kPanel + 1], double* prow) {
  const int w = (threadIdx.x >> 5) & 3, lane = threadIdx.x & 31;
  double* const rps = prow + 2 * (kPanel + 1);  // 1 / pivot of every step
  double v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int r = w + 4 * q;
    v[q] = (r < nb && lane < nb) ? __ldcg(&S[(size_t)(k0 + lane) * bs + k0 + r])
                                 : (r == lane ? 1.0 : 0.0);
  }
#pragma unroll
  for (int c = 0; c < kPanel; ++c) {
    if (c >= nb) break;  // the identity frame needs no steps
    double* const buf = prow + (c & 1) * (kPanel + 1);
    if (w == (c & 3)) {  // row c is final: publish it, scaled, with its pivot
      const double p = tiny_pivot(__shfl_sync(FULL, v[c >> 2], c));
      const double rp = bt::fast_rcp(p);
      if (lane == c) v[c >> 2] = p;
      buf[lane] = lane > c ? v[c >> 2] * rp : v[c >> 2];
      if (lane == 0) rps[c] = rp;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const double u = buf[lane];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (w + 4 * q > c) {
        const double lc = __shfl_sync(FULL, v[q], c);
        if (lane > c) v[q] = fma(-lc, u, v[q]);
      }
  }
  asm volatile("bar.sync 1, 128;" ::: "memory");
  const double rl = lane < nb ? rps[lane] : 1.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int r = w + 4 * q;
    if (r > lane) v[q] = v[q] * rl;  // the multipliers l(r, lane)
    if (store && r < nb && lane < nb) S[(size_t)(k0 + lane) * bs + k0 + r] = v[q];
    if (Dsh) Dsh[r][lane] = v[q];
  }
}

template <bool MMA>
__global__ void __launch_bounds__(kLuThreads, 2) k_schur_lu(double* S, int bs, unsigned* bar,
                                                            int* status) {
  __shared__ double D[kPanel][kPanel + 1];   // the factored diagonal block, D[r][c]
  __shared__ double rinv[kPanel];            // 1 / its pivots
  __shared__ double prow[3 * kPanel + 2];    // factor_diag's pivot rows and reciprocals
  __shared__ double Us1[kPanel][kPanel + 1];  // U11 rows divided by their pivots
  __shared__ double Ls[kPanel][kPanel + 1];  // trailing tile: L21 rows, Ls[m][i]
  __shared__ double Us[kPanel][kPanel + 1];  //                U12 columns, Us[m][j]
  __shared__ int s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned G = gridDim.x;
  unsigned gen = 0;
  // Block 0 runs the chain of diagonal blocks; the block sharing its SM
  // takes no trailing tiles, so no other FP64 work slows that chain.
  unsigned smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  if (blockIdx.x == 0 && tid == 0) bar[2] = smid + 1;  // read after the first barrier
  for (int k0 = 0, panel = 0; k0 < bs; k0 += kPanel, ++panel) {
    const int nb = min(kPanel, bs - k0), rest = bs - k0 - nb;
    // ---- A: the diagonal block - the first factored by every block for
    // itself (block 0 stores it), the others factored ahead in the previous
    // panel's update - then the L21 rows and U12 columns
    if (k0 == 0) {
      if (warp < 4) factor_diag(S, bs, 0, nb, blockIdx.x == 0, D, prow);
    } else {
      for (int q = tid; q < nb * nb; q += kLuThreads) {
        const int c = q / nb, r = q % nb;
        D[r][c] = __ldcg(&S[(size_t)(k0 + c) * bs + k0 + r]);
      }
    }
    __syncthreads();
    if (rest == 0) break;
    if (tid < kPanel) rinv[tid] = bt::fast_rcp(D[tid][tid]);
    __syncthreads();
    for (int q = tid; q < kPanel * kPanel; q += kLuThreads) {
      const int c = q / kPanel, j = q % kPanel;
      Us1[c][j] = D[c][j] * rinv[c];
    }
    __syncthreads();
    // (rest > 0, so nb == kPanel from here on.) One warp per row of L21 or
    // column of U12, lanes over its 32 entries, the items round robin over
    // the blocks' warps: a step is one product (or two) per lane, and FP64
    // issues one warp instruction per 64 cycles per SM sub-partition.
    for (int it = blockIdx.x + G * warp; it < 2 * rest; it += G * (kLuThreads / 32)) {
      if (it < rest) {  // row r of L21 = A21 U11^-1, the division deferred
        const int r = k0 + kPanel + it;
        double a = __ldcg(&S[(size_t)(k0 + lane) * bs + r]);
#pragma unroll
        for (int c = 0; c < kPanel - 1; ++c) {
          const double t = __shfl_sync(FULL, a, c);
          if (lane > c) a = fma(-t, Us1[c][lane], a);
        }
        S[(size_t)(k0 + lane) * bs + r] = a * rinv[lane];
      } else {  // column j of U12 = L11^-1 A12, right-looking
        double* const col = S + (size_t)(k0 + kPanel + it - rest) * bs + k0;
        double a = __ldcg(&col[lane]);
#pragma unroll
        for (int m = 0; m < kPanel - 1; ++m) {
          const double x = __shfl_sync(FULL, a, m);
          if (lane > m) a = fma(-D[lane][m], x, a);
        }
        if (lane > 0) col[lane] = a;
      }
    }
    if (!grid_barrier(bar, G, gen, status)) return;
    // ---- B: A22 -= L21 U12 in 32 x 32 tiles handed out by a counter; block
    // 0 first takes tile 0, the next panel's diagonal block, and factors it
    // as soon as it is updated (the block beside it on its SM sits out).
    const int nt = (rest + kPanel - 1) / kPanel, ntiles = nt * nt;
    const bool idle = blockIdx.x != 0 && smid + 1 == *(volatile unsigned*)&bar[2];
    for (bool first = true; !idle; first = false) {
      if (tid == 0)  // block 0 starts with tile 0; the counter hands out the rest
        s_tile = (blockIdx.x == 0 && first) ? 0 : 1 + (int)atomicAdd(&bar[3 + panel], 1u);
      __syncthreads();
      const int t = s_tile;
      if (t >= ntiles) break;
      const int r0 = k0 + kPanel + (t / nt) * kPanel, c0 = k0 + kPanel + (t % nt) * kPanel;
      for (int q = tid; q < kPanel * kPanel; q += kLuThreads) {  // lanes down a column
        const int m = q / kPanel, i = q % kPanel;
        Ls[m][i] = r0 + i < bs ? __ldcg(&S[(size_t)(k0 + m) * bs + r0 + i]) : 0.0;
        Us[i][m] = c0 + m < bs ? __ldcg(&S[(size_t)(c0 + m) * bs + k0 + i]) : 0.0;
      }
      __syncthreads();
      if (MMA) {  // warp w: the 8 x 8 tiles 2w and 2w + 1 of the 4 x 4 grid
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int s = warp * 2 + h, i0 = (s >> 2) * 8, j0 = (s & 3) * 8;
          double d0 = 0.0, d1 = 0.0;
#pragma unroll
          for (int kk = 0; kk < kPanel; kk += 4)
            dmma_8x8x4(d0, d1, Ls[kk + (lane & 3)][i0 + (lane >> 2)],
                       Us[kk + (lane & 3)][j0 + (lane >> 2)]);
          const int r = r0 + i0 + (lane >> 2), c = c0 + j0 + (lane & 3) * 2;
          if (r < bs) {
            if (c < bs) S[(size_t)c * bs + r] = __ldcg(&S[(size_t)c * bs + r]) - d0;
            if (c + 1 < bs)
              S[(size_t)(c + 1) * bs + r] = __ldcg(&S[(size_t)(c + 1) * bs + r]) - d1;
          }
        }
      } else {  // 2 x 2 outputs per thread, products accumulated in m order
        const int ty = tid >> 4, tx = tid & 15;
        double acc[2][2] = {};
#pragma unroll 8
        for (int m = 0; m < kPanel; ++m) {
          const double a0 = Ls[m][ty * 2], a1 = Ls[m][ty * 2 + 1];
          const double b0 = Us[m][tx * 2], b1 = Us[m][tx * 2 + 1];
          acc[0][0] = fma(a0, b0, acc[0][0]);
          acc[0][1] = fma(a0, b1, acc[0][1]);
          acc[1][0] = fma(a1, b0, acc[1][0]);
          acc[1][1] = fma(a1, b1, acc[1][1]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 2; ++v) {
            const int r = r0 + ty * 2 + u, c = c0 + tx * 2 + v;
            if (r < bs && c < bs)
              S[(size_t)c * bs + r] = __ldcg(&S[(size_t)c * bs + r]) - acc[u][v];
          }
      }
      __syncthreads();
      if (t == 0) {  // the next diagonal block is final: factor it ahead
        if (warp < 4) factor_diag(S, bs, k0 + kPanel, min(kPanel, rest), true, nullptr, prow);
        __syncthreads();
      }
    }
    if (!grid_barrier(bar, G, gen, status)) return;
  }
}

// FP64 tensor-core probe: every warp keeps four independent m8n8k4
// accumulations in flight; each mma is 2 x 8 x 8 x 4 = 512 flops.
__global__ void k_dmma_peak(double* out, int iters, double a, double b) {
  double d[4][2];
#pragma unroll
  for (int q = 0; q < 4; ++q) d[q][0] = d[q][1] = threadIdx.x * 1e-9 + q;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q) dmma_8x8x4(d[q][0], d[q][1], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) s += d[q][0] + d[q][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int coop_grid() {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per = 0, per2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_schur_lu<false>, kLuThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_schur_lu<true>, kLuThreads, 0);
    per = min(min(per, per2), 2);  // two blocks per SM: one loads while one computes
    grid = per > 0 ? sms * per : -1;
  }
  return grid;
}

}  // namespace

cudaError_t launch_schur_lu(double* S, int bs, bool mma, unsigned* bar, int* status,
                            cudaStream_t s) {
  if (bs <= 0) return cudaSuccess;
  const int grid = coop_grid();
  if (grid <= 0) return cudaErrorCooperativeLaunchTooLarge;
  cudaError_t e = cudaMemsetAsync(bar, 0, schur_lu_bar_words(bs) * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  void* args[] = {&S, &bs, &bar, &status};
  return cudaLaunchCooperativeKernel(mma ? (const void*)k_schur_lu<true>
                                         : (const void*)k_schur_lu<false>,
                                     dim3(grid), dim3(kLuThreads), args, 0, s);
}

double dmma_peak_tflops() {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8, block = 256, iters = 2048;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * sizeof(double)) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dmma_peak<<<grid, block>>>(out, 64, 0.999, 1e-3);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_dmma_peak<<<grid, block>>>(out, iters, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double warps = (double)grid * block / 32.0;
  const double flops = 512.0 * 4.0 * iters * warps;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace gk
