// hyp_noalloc.cu -- the single-phase FP64 step on caller-owned device buffers,
// without any device memory allocation.
//
// The context API (hyp_create) allocates its state and scratch buffers with
// cudaMalloc. Some callers cannot do that on the path where they step the
// solver: a host whose device memory is owned by another allocator (a
// framework's memory pool that must account for every byte), or a
// latency-critical loop that must not risk the implicit synchronisation and
// driver calls an allocation brings. hyp_step_noalloc_f64 serves them: the
// caller passes the input and output state, and everything else the step
// needs (the second state buffer of the ping-pong, per-cell fluxes and wave
// speeds, loop control) lives in one fixed, file-scope device array of
// kNoAllocDoubles doubles (65,536 cells at most; 13,631,552 bytes = 13.0 MiB that
// every GPU which loads this library keeps until the process exits).
//
// Set-up: the first call on a device looks up that array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture. Every call on a device shares the
// array, and it keeps the last call's contents: the loop-control words are
// reset at the start of every call, the other scratch is fully overwritten
// before it is read. Calls that overlap on the GPU (different streams, or
// different host threads on the same device) race on the array and must be
// serialised by the caller. Each call waits for `stream` to finish before it
// returns (it reads the final time and error word back to the host).
//
// Errors: a launch error that earlier, unrelated work left pending in the CUDA
// runtime is cleared on entry (cudaGetLastError) so that it is not reported as
// this call's; the reset kernel and the first step's two launches are checked one
// by one, so a launch that fails stops the call before the rest are queued.
#include <mutex>
#include "hyp_internal.cuh"

namespace hyp {

constexpr int64_t kNoAllocMaxCells = 65536;
constexpr size_t kNoAllocState = (size_t)14 * kNoAllocMaxCells;      // second state buffer
constexpr size_t kNoAllocFlux = (size_t)kNFlux1 * kNoAllocMaxCells;   // per-cell fluxes
constexpr size_t kNoAllocLam = (size_t)kNoAllocMaxCells;              // per-cell wave speeds
constexpr size_t kNoAllocCtl = (sizeof(DevState) + sizeof(double) - 1) / sizeof(double);
constexpr size_t kNoAllocDoubles = kNoAllocState + kNoAllocFlux + kNoAllocLam + kNoAllocCtl;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

namespace {
constexpr int kMaxDevices = 256;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

__global__ void noalloc_reset_kernel(DevState* st, double t0) {
  st->t[0] = t0;
  st->t[1] = t0;
  st->lam_bits[0] = 0ull;
  st->lam_bits[1] = 0ull;
  st->lam_query = 0ull;
  st->steps = 0;
  st->err_code = 0;
  st->pad_ = 0;
  st->err_cell = -1;
}

// Device address of the scratch array on the current device (looked up once per device).
int scratch_base(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return HYP_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return HYP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    double* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return HYP_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return HYP_OK;
}
}  // namespace

}  // namespace hyp

using namespace hyp;

extern "C" int hyp_step_noalloc_f64(const hyp_config* cfg, const double* d_Q_in, double* d_Q_out, int64_t n_cells,
                                    int n_steps, double t0, void* stream, double* t_out, int64_t* err_cell) {
  if (err_cell) *err_cell = -1;
  if (!cfg || !d_Q_in || !d_Q_out || n_steps < 0) return HYP_ERR_INVALID;
  if (n_cells < 3 || n_cells > kNoAllocMaxCells) return HYP_ERR_INVALID;  // beyond the fixed scratch
  if (cfg->n_cells != n_cells || cfg->model != HYP_MODEL_SINGLE || cfg->precision != HYP_PREC_FP64)
    return HYP_ERR_INVALID;
  if (cfg->flux != HYP_FLUX_RUSANOV && cfg->flux != HYP_FLUX_LXF) return HYP_ERR_INVALID;
  if (cfg->bc != HYP_BC_FROZEN && cfg->bc != HYP_BC_TRANSMISSIVE) return HYP_ERR_INVALID;
  if (!(cfg->cfl > 0) || !(cfg->x_length > 0) || !(cfg->eos[0].rho0 > 0) || !(cfg->eos[0].cv > 0))
    return HYP_ERR_INVALID;
  (void)cudaGetLastError();  // a pending error from the caller's earlier work is not this call's
  double* base = nullptr;
  int rc = scratch_base(&base);
  if (rc != HYP_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = n_cells;
  double* B = base;
  double* F = base + kNoAllocState;
  double* lam = F + kNoAllocFlux;
  DevState* st = (DevState*)(lam + kNoAllocLam);
  const EosC eos = make_eos(cfg->eos[0].rho0, cfg->eos[0].c0, cfg->eos[0].cv, cfg->eos[0].t0, cfg->eos[0].b0,
                            cfg->eos[0].alpha, cfg->eos[0].beta, cfg->eos[0].gamma);
  const double dx = cfg->x_length / (double)n;
  const unsigned grid = (unsigned)((n + kBlock - 1) / kBlock);
  // Ping-pong between the caller's output and the scratch state so that the last step writes the output.
  double* cur = (n_steps % 2 == 0) ? d_Q_out : B;
  if (cur != d_Q_in &&
      cudaMemcpyAsync(cur, d_Q_in, (size_t)14 * n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return HYP_ERR_CUDA;
  noalloc_reset_kernel<<<1, 1, 0, s>>>(st, t0);
  if (cudaGetLastError() != cudaSuccess) return HYP_ERR_CUDA;
  for (int k = 0; k < n_steps; ++k) {
    const int p = k & 1;
    double* nxt = (cur == d_Q_out) ? B : d_Q_out;
    cell1_f64_kernel<<<grid, kBlock, 0, s>>>(cur, n, eos, F, lam, &st->lam_bits[p], &st->t[p], INFINITY, st);
    if (k == 0 && cudaGetLastError() != cudaSuccess) return HYP_ERR_CUDA;
    update1_f64_kernel<<<grid, kBlock, 0, s>>>(cur, nxt, n, F, lam, &st->lam_bits[p], &st->lam_bits[1 - p],
                                               &st->t[p], &st->t[1 - p], &st->steps, INFINITY, cfg->cfl, dx,
                                               cfg->flux, cfg->bc);
    if (k == 0 && cudaGetLastError() != cudaSuccess) return HYP_ERR_CUDA;
    cur = nxt;
  }
  if (cudaGetLastError() != cudaSuccess) return HYP_ERR_CUDA;
  DevState h;
  if (cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess) return HYP_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return HYP_ERR_CUDA;
  if (t_out) *t_out = h.t[n_steps & 1];
  if (h.err_code) {
    if (err_cell) *err_cell = h.err_cell;
    return (h.err_code & HYP_CELL_NEG_DET) ? HYP_ERR_NEG_DET : HYP_ERR_NONFINITE;
  }
  return HYP_OK;
}
