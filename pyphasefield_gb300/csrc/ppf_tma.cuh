// Tensor-memory-accelerator (TMA) staging helpers: mbarriers with bounded
// waits, tensor-tile loads (cp.async.bulk.tensor) and the host-side cache of
// CUtensorMap descriptors.
//
// Every wait on an mbarrier is bounded: after kWaitLimit polls the waiting
// thread reports a timeout instead of spinning forever, and the kernels turn
// that into PPF_STATUS_TIMEOUT in the library's device status word.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ppf_common.cuh"

namespace ppf {

// ------------------------------------------------------------ device side
constexpr uint32_t kWaitLimit = 1u << 22;  // polls: far above any real TMA wait

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) accesses to the same memory.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Bounded wait for phase `parity` of `bar`. Each poll lets the hardware
// suspend the thread for up to kSuspendNs until the phase completes, so
// waiting threads do not spin on issue slots; after `limit` polls (well
// under a second in total) it gives up and returns false.
constexpr uint32_t kSuspendNs = 20000;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          uint32_t limit = kWaitLimit / 128) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity), "n"(kSuspendNs)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Bounded wait by polling (mbarrier.test_wait: no suspension between polls),
// for warps that wait on their own loads and have little else to hide the
// latency with; gives up after `limit` polls.
__device__ __forceinline__ bool mbar_wait_poll(uint64_t* bar, uint32_t parity,
                                               uint32_t limit = kWaitLimit * 4) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 2-D / 3-D tensor tile load into shared memory, completing on `bar`.
// The innermost coordinate times the element size must be a multiple of 16.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y,
                                            int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// ------------------------------------------------------------ host side
// Tiled tensor map over a pitched field: dims innermost first
// (nx, ny[, nz]), byte strides of the outer dims, box innermost first.
// Descriptors are cached per (pointer, geometry, box) for the process.
int32_t tensor_map(CUtensorMap* out, const void* base, int elem_bytes, int rank,
                   const uint64_t* dims, const uint64_t* strides_bytes,
                   const uint32_t* box);
// bf16 matrix [rows][cols] (row stride row_bytes), box of box_rows x
// box_cols (box_cols * 2 <= 128 bytes) written to shared memory with the
// 128-byte swizzle that the tcgen05 K-major SW128 operand layout expects;
// out-of-range rows and columns arrive as zeros.
int32_t tensor_map_bf16_sw128(CUtensorMap* out, const void* base, uint64_t cols, uint64_t rows,
                              uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows);

}  // namespace ppf
