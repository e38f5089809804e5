// TMA (cp.async.bulk.tensor) and mbarrier helpers shared by the kernels that
// stage column groups with 2-D tensor-map copies (k_dir_fused.cu,
// k_cols_tma.cu).
//
// Every wait on a TMA completion is bounded: mbarrier.try_wait returns after a
// hardware time limit, and mbar_wait_bounded gives up after kTmaWaitLimit of
// those (seconds), records kErrTmaTimeout in the plan's device error word and
// returns false.  A kernel whose wait gave up issues no further copies and
// waits once more (bounded) for the copy in flight before it exits, so no
// copy lands in shared memory that a later CTA owns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace nsst {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// makes the initialised mbarrier visible to the async proxy (and, in a
// cluster, to the peers) before the first copy is issued against it
__device__ __forceinline__ void fence_mbarrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// 2-D tiled TMA load global -> this CTA's shared memory, completion counted
// on the mbarrier in bytes.  The tensor maps used here have 8-byte elements
// (one float2) and x is a multiple of 2, so x * 8 is a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// generic-proxy accesses of shared memory before this are ordered before
// later async-proxy (TMA) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bound on a TMA completion wait: try_wait returns after a hardware time
// limit, so this is seconds, not a spin on a value that may never come.
constexpr uint32_t kTmaWaitLimit = 1u << 22;
constexpr int kErrTmaTimeout = 1;

// waits for phase `parity` of the mbarrier; false (and the error code set)
// when the limit runs out
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int* err) {
  for (uint32_t it = 0; it < kTmaWaitLimit; it++)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(err, kErrTmaTimeout);
  return false;
}

}  // namespace nsst
