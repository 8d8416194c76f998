// hyp_peaks.cu -- the rates this GB300 reaches on the operations the step uses, for
// the roofline denominators beyond the HBM copy and bf16 GEMM rates: FP64 and FP32 fused
// multiply-add throughput (scalar FP32 and packed f32x2), and the host link
// (page-locked copies each way and both ways at once).
//
// FMA: every thread runs 8 independent chains of 4096 fused multiply-adds (no memory
// traffic), 8 blocks of 256 threads per SM; FLOP/s = 2 x FMAs / kernel time.
//
// Layouts (hyp_measure_layouts): the single-phase mixed step's memory traffic -- 32
// FP32 rows per cell read, the owned cells' 32 rows written -- without the physics,
// in the two block layouts the step could use: row-major (row r of cell i at
// r * pitch + i; a 256-thread block reads its 254 cells plus a halo cell each side
// from every row) and tile-major (the layout the step uses: a tile's 32 rows of 256
// floats contiguous, warp w reading the 128-byte line at 32 w of each row).
#include <cuda_runtime.h>
#include <vector>
#include "../../include/hyperelastic.h"

namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_chains(T* out, int iters, T a, T b) {
  T acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = (T)(threadIdx.x * 1e-3) + (T)j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = fma(acc[j], a, b);
  }
  T s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += acc[j];
  if (s == (T)12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

__global__ void __launch_bounds__(256) fma_chains_f32x2(float* out, int iters, float a, float b) {
  unsigned long long acc[8], av, bv;
  asm("mov.b64 %0, {%1,%2};" : "=l"(av) : "f"(a), "f"(a));
  asm("mov.b64 %0, {%1,%2};" : "=l"(bv) : "f"(b), "f"(b));
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float x = threadIdx.x * 1e-3f + j, y = x + 0.5f;
    asm("mov.b64 %0, {%1,%2};" : "=l"(acc[j]) : "f"(x), "f"(y));
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(acc[j]) : "l"(av), "l"(bv));
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float x, y;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(x), "=f"(y) : "l"(acc[j]));
    s += x + y;
  }
  if (s == 12345.678f) out[0] = s;
}

__global__ void __launch_bounds__(256, 4) copy_rows_rowmajor(const float* __restrict__ in, float* __restrict__ out,
                                                              int64_t n, int64_t pitch) {
  const int64_t first = (int64_t)blockIdx.x * 254;
  const int64_t i = first - 1 + threadIdx.x;
  const int64_t ic = i < 0 ? 0 : (i >= n ? n - 1 : i);
  float v[32];
#pragma unroll
  for (int r = 0; r < 32; ++r) v[r] = in[r * pitch + ic];
  float s = 0.f;
#pragma unroll
  for (int r = 0; r < 32; ++r) s += v[r];
  if (threadIdx.x > 0 && threadIdx.x < 255 && i < n) {
#pragma unroll
    for (int r = 0; r < 32; ++r) out[r * pitch + i] = v[r] + s * 1e-30f;  // s keeps every load live
  }
}

__global__ void __launch_bounds__(256, 4) copy_rows_tilemajor(const float* __restrict__ in, float* __restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * (32 * 256) + threadIdx.x;
  float v[32];
#pragma unroll
  for (int r = 0; r < 32; ++r) v[r] = in[base + r * 256];
  float s = 0.f;
#pragma unroll
  for (int r = 0; r < 32; ++r) s += v[r];
  // the owned cells' rows and, as the step does, the two unused floats of each row
#pragma unroll
  for (int r = 0; r < 32; ++r) out[base + r * 256] = threadIdx.x < 254 ? v[r] + s * 1e-30f : 0.0f;
}

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

}  // namespace

// out[0..5]: FP64 FMA TFLOP/s, FP32 FMA TFLOP/s, FP32x2 FMA TFLOP/s, host-to-device
// GB/s, device-to-host GB/s, and GB/s each way with both directions at once; each the
// best of `reps`; `bytes` per copy (page-locked host buffers).
extern "C" int hyp_measure_peaks(int reps, int64_t bytes, double* out) {
  if (!out || reps < 1 || bytes < (1 << 20)) return HYP_ERR_INVALID;
  int ndev = 0, sms = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return HYP_ERR_CUDA;
  for (int k = 0; k < 6; ++k) out[k] = 0.0;
  Timer t;
  cudaStream_t s[2];
  if (cudaStreamCreateWithFlags(&s[0], cudaStreamNonBlocking) != cudaSuccess) return HYP_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&s[1], cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(s[0]);
    return HYP_ERR_CUDA;
  }
  int rc = HYP_OK;
  double* sink = nullptr;
  void *h0 = nullptr, *h1 = nullptr, *d0 = nullptr, *d1 = nullptr;
  if (cudaMalloc(&sink, 64) != cudaSuccess || cudaMallocHost(&h0, bytes) != cudaSuccess ||
      cudaMallocHost(&h1, bytes) != cudaSuccess || cudaMalloc(&d0, bytes) != cudaSuccess ||
      cudaMalloc(&d1, bytes) != cudaSuccess)
    rc = HYP_ERR_CUDA;
  const unsigned grid = (unsigned)sms * 8;
  const int iters = 4096;
  const double fmas = (double)grid * 256.0 * iters * 8.0;
  float ms = 0.f;
  for (int r = 0; r < reps && rc == HYP_OK; ++r) {
    cudaEventRecord(t.a, s[0]);
    fma_chains<double><<<grid, 256, 0, s[0]>>>(sink, iters / 16, 1.0000001, 1e-9);  // 1/16: FP64 runs 1/64 the rate
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[0] = fmax(out[0], 2.0 * fmas / 16.0 / (ms * 1e-3) / 1e12);
    cudaEventRecord(t.a, s[0]);
    fma_chains<float><<<grid, 256, 0, s[0]>>>((float*)sink, iters, 1.0000001f, 1e-9f);
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[1] = fmax(out[1], 2.0 * fmas / (ms * 1e-3) / 1e12);
    cudaEventRecord(t.a, s[0]);
    fma_chains_f32x2<<<grid, 256, 0, s[0]>>>((float*)sink, iters, 1.0000001f, 1e-9f);
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[2] = fmax(out[2], 4.0 * fmas / (ms * 1e-3) / 1e12);
    if (cudaGetLastError() != cudaSuccess) rc = HYP_ERR_CUDA;
  }
  const double gb = (double)bytes / 1e9;
  for (int r = 0; r < reps && rc == HYP_OK; ++r) {
    cudaEventRecord(t.a, s[0]);
    cudaMemcpyAsync(d0, h0, bytes, cudaMemcpyHostToDevice, s[0]);
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[3] = fmax(out[3], gb / (ms * 1e-3));
    cudaEventRecord(t.a, s[0]);
    cudaMemcpyAsync(h1, d1, bytes, cudaMemcpyDeviceToHost, s[0]);
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[4] = fmax(out[4], gb / (ms * 1e-3));
    // both directions at once: the second stream waits for the first's start event
    cudaEventRecord(t.a, s[0]);
    cudaStreamWaitEvent(s[1], t.a, 0);
    cudaMemcpyAsync(d0, h0, bytes, cudaMemcpyHostToDevice, s[0]);
    cudaMemcpyAsync(h1, d1, bytes, cudaMemcpyDeviceToHost, s[1]);
    cudaEvent_t done1;
    if (cudaEventCreate(&done1) != cudaSuccess) {
      rc = HYP_ERR_CUDA;
      break;
    }
    cudaEventRecord(done1, s[1]);
    cudaStreamWaitEvent(s[0], done1, 0);
    cudaEventRecord(t.b, s[0]);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventDestroy(done1);
    cudaEventElapsedTime(&ms, t.a, t.b);
    out[5] = fmax(out[5], gb / (ms * 1e-3));
    if (cudaGetLastError() != cudaSuccess) rc = HYP_ERR_CUDA;
  }
  cudaStreamDestroy(s[0]);
  cudaStreamDestroy(s[1]);
  if (sink) cudaFree(sink);
  if (d0) cudaFree(d0);
  if (d1) cudaFree(d1);
  if (h0) cudaFreeHost(h0);
  if (h1) cudaFreeHost(h1);
  return rc;
}

// out[0..1]: GB/s (256 B per cell: 32 FP32 rows read and written) of the single-phase
// mixed step's memory traffic for n_cells cells in a row-major and in a tile-major
// block, without the physics; each the best of `reps`.
extern "C" int hyp_measure_layouts(int reps, int64_t n_cells, double* out) {
  if (!out || reps < 1 || n_cells < 256) return HYP_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  out[0] = out[1] = 0.0;
  const int64_t tiles = (n_cells + 253) / 254;
  const int64_t pitch = (n_cells + 3) & ~int64_t(3);
  const size_t floats = (size_t)32 * (size_t)(tiles * 256 > pitch ? tiles * 256 : pitch);
  float *a = nullptr, *b = nullptr;
  int rc = HYP_OK;
  if (cudaMalloc(&a, floats * sizeof(float)) != cudaSuccess || cudaMalloc(&b, floats * sizeof(float)) != cudaSuccess ||
      cudaMemset(a, 0, floats * sizeof(float)) != cudaSuccess)
    rc = HYP_ERR_CUDA;
  Timer t;
  const double gb = 256.0 * (double)n_cells / 1e9;
  float ms = 0.f;
  for (int r = 0; r < reps + 1 && rc == HYP_OK; ++r) {  // the first round warms up
    cudaEventRecord(t.a);
    copy_rows_rowmajor<<<(unsigned)tiles, 256>>>(a, b, n_cells, pitch);
    cudaEventRecord(t.b);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    if (r > 0) out[0] = fmax(out[0], gb / (ms * 1e-3));
    cudaEventRecord(t.a);
    copy_rows_tilemajor<<<(unsigned)tiles, 256>>>(a, b);
    cudaEventRecord(t.b);
    if (cudaEventSynchronize(t.b) != cudaSuccess) rc = HYP_ERR_CUDA;
    cudaEventElapsedTime(&ms, t.a, t.b);
    if (r > 0) out[1] = fmax(out[1], gb / (ms * 1e-3));
    if (cudaGetLastError() != cudaSuccess) rc = HYP_ERR_CUDA;
  }
  if (a) cudaFree(a);
  if (b) cudaFree(b);
  return rc;
}
