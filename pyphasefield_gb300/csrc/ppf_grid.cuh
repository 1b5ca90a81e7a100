// Grid-wide barrier for persistent cooperative kernels (every CTA of the
// launch resident), with bounded waits.
#pragma once

#include <stdint.h>

#include "ppf_common.cuh"

namespace ppf {

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// sync[0] counts arrivals, sync[1] is the generation (zero both once before
// the first launch that uses them). Every thread of every CTA calls it.
// Bounded: after kBarrierPolls polls a waiting CTA ORs PPF_STATUS_TIMEOUT
// into *status, sets *flag (shared) and the call returns false for the
// whole CTA. Writes before the barrier are visible to plain (coherent) loads
// after it; loads through the read-only path (__ldg) are not.
constexpr uint32_t kBarrierPolls = 1u << 22;
__device__ __forceinline__ bool grid_barrier(unsigned* sync, unsigned nblocks, int* status,
                                             int* flag) {
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    const unsigned gen = ld_acquire(sync + 1);
    __threadfence();  // this CTA's writes before its arrival
    if (atomicAdd(sync, 1u) + 1u == nblocks) {
      atomicExch(sync, 0u);
      __threadfence();
      st_release(sync + 1, gen + 1u);
    } else {
      uint32_t i = 0;
      while (ld_acquire(sync + 1) == gen) {
        if (++i > kBarrierPolls) {
          atomicOr(status, PPF_STATUS_TIMEOUT);
          *flag = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *flag == 0;
}

}  // namespace ppf
