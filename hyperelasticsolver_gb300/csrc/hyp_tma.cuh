// hyp_tma.cuh -- tensor-memory-accelerator (TMA) tile loads with an mbarrier,
// as inline PTX, and the host-side tensor-map encoding.
//
// A tile load is one cp.async.bulk.tensor.2d per box, issued by one thread,
// completing on an mbarrier whose transaction count the same thread set with
// arrive.expect_tx. Every wait on the barrier is bounded: a waiter that gives
// up reports it, and the kernel records HYP_CELL_TIMEOUT and returns.
// Rules kept by the callers: the x coordinate of a box is a multiple of 4
// floats (16 bytes); the row pitch is a multiple of 16 bytes; boxes are at most
// 256 elements wide; the shared-memory destination is 128-byte aligned.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
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

// One 2D box of the tensor `map` at element coordinates (x, y) into shared memory.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// Host: a 2D FP32 tensor map over rows x cols floats (row pitch `pitch` floats)
// with boxes of box_w x box_h; out-of-range elements read as zero.
int encode_tmap_2d_f32(CUtensorMap* map, const float* base, int64_t pitch, int64_t rows, int box_w, int box_h);

}  // namespace hyp
