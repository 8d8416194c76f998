// hyp_tma.cuh -- tensor-memory-accelerator (TMA) bulk copies into shared memory
// with an mbarrier, as inline PTX.
//
// A tile load is one cp.async.bulk of the tile's contiguous span, issued by one
// thread, completing on an mbarrier whose transaction count the same thread set
// with arrive.expect_tx. Every wait on the barrier is bounded: a waiter that gives
// up reports it, and the kernel records HYP_CELL_TIMEOUT and returns.
// Rules kept by the callers: source and destination 16-byte aligned, the size a
// multiple of 16 bytes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hyp {

enum { HYP_CELL_TIMEOUT = 4 };  // a bounded device wait gave up (cell status bit)

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (TMA) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the completion of the barrier phase with the given parity; false
// if it has not completed after `tries` polls (each try_wait may itself block
// for a bounded, implementation-defined time).
constexpr int kWaitTries = 1 << 20;   // default poll budget of a device wait
constexpr int kDrainTries = 1 << 20;  // budget for letting an in-flight copy land after a timeout
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int tries = kWaitTries) {
  for (int k = 0; k < tries; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// `bytes` contiguous bytes of global memory at src into shared memory at dst,
// completing on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

}  // namespace hyp
