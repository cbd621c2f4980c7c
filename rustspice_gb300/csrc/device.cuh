// Device-side helpers shared by the kernels of libgpuklu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gk {

// Device status codes written into the per-handle status word. They map onto
// the C-ABI's GPUKLU_* codes.
enum DevStatus : int {
  DS_OK = 0,
  DS_TIMEOUT = 7,
  DS_NONFINITE = 8,
};

// Arithmetic without contraction: every product is rounded before it is
// added, as in the reference (Rust never fuses multiply-add), so results are
// reproducible bit for bit against the CPU restatement.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

// Waits until flag == epoch, at most `limit` polls (DPlan::spin_limit).
// Returns false on timeout or when another warp has already reported an
// error; the caller then stops its work.
__device__ __forceinline__ bool wait_flag(const unsigned* flag, unsigned epoch, int* status,
                                          unsigned limit) {
  unsigned spins = 0;
  while (ld_acquire(flag) != epoch) {
    if (++spins > limit) {
      atomicCAS(status, DS_OK, DS_TIMEOUT);
      return false;
    }
    if ((spins & 63u) == 0 && *(volatile int*)status != DS_OK) return false;
    if (spins > 16) __nanosleep(spins < 256 ? 32 : 256);  // a poll is an L2 round trip
  }
  return true;
}

// Singleton-block and general pivot perturbation rules of the reference
// (crates/sim-core/src/native_klu.rs:1229-1231 and :1345-1348).
__device__ __forceinline__ double perturb(double d, bool singleton) {
  if (singleton) return fabs(d) < 1e-300 ? 1e-14 : d;
  if (fabs(d) < 1e-14) return d >= 0.0 ? 1e-14 : -1e-14;
  return d;
}

}  // namespace gk
