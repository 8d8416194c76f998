// hyp_capi.cu -- context lifecycle, transfers and the step driver of the C ABI.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include "hyp_internal.cuh"
#include "hyp_relax.cuh"

using namespace hyp;

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t _e = (call);                                                               \
    if (_e != cudaSuccess) return set_err(c, HYP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

static int set_err(hyp_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

static const char* kNoCtx = "no context";

extern "C" const char* hyp_last_error(const hyp_ctx* c) { return c ? c->err.c_str() : kNoCtx; }
extern "C" int64_t hyp_error_cell(const hyp_ctx* c) { return c ? c->err_cell : -1; }

static EosC to_eos(const hyp_barton2009& b) {
  return make_eos(b.rho0, b.c0, b.cv, b.t0, b.b0, b.alpha, b.beta, b.gamma);
}

static bool valid_eos(const hyp_barton2009& b) {
  return b.rho0 > 0 && b.cv > 0 && b.t0 > 0 && b.alpha != 0 && std::isfinite(b.c0) && std::isfinite(b.b0) &&
         std::isfinite(b.beta) && std::isfinite(b.gamma);
}

static bool mixed(const hyp_ctx* c) { return c->cfg.precision == HYP_PREC_MIXED; }
static bool mixed1(const hyp_ctx* c) { return mixed(c) && c->cfg.model == HYP_MODEL_SINGLE; }

static int free_ctx(hyp_ctx* c) {
  if (!c) return HYP_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_tape(c);
  free_snap(c);
  for (auto& g : c->graph)
    if (g) cudaGraphExecDestroy(g);
  for (int p = 0; p < 2; ++p) cudaFree(c->Q[p]);
  cudaFree(c->mixed_base);
  cudaFree(c->F);
  cudaFree(c->lam);
  cudaFree(c->smin);
  cudaFree(c->smax);
  cudaFree(c->DM);
  cudaFree(c->DP);
  cudaFree(c->FF);
  cudaFree(c->F32);
  cudaFree(c->smin32);
  cudaFree(c->smax32);
  cudaFree(c->DM32);
  cudaFree(c->DP32);
  cudaFree(c->FF32);
  cudaFree(c->st);
  cudaFree(c->hist_dev);
  if (c->st_host) cudaFreeHost(c->st_host);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->prof_ev) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (auto& e : c->row_ev)
    if (e) cudaEventDestroy(e);
  delete c;
  return HYP_OK;
}

extern "C" int hyp_create(const hyp_config* cfg, hyp_ctx** out) {
  if (!cfg || !out) return HYP_ERR_INVALID;
  *out = nullptr;
  if (cfg->n_cells < 3 || cfg->x_length <= 0 || !(cfg->cfl > 0)) return HYP_ERR_INVALID;
  if (cfg->model != HYP_MODEL_SINGLE && cfg->model != HYP_MODEL_MULTI) return HYP_ERR_INVALID;
  if (cfg->flux < HYP_FLUX_RUSANOV || cfg->flux > HYP_FLUX_HLL) return HYP_ERR_INVALID;
  if (cfg->bc != HYP_BC_FROZEN && cfg->bc != HYP_BC_TRANSMISSIVE) return HYP_ERR_INVALID;
  if (cfg->precision != HYP_PREC_FP64 && cfg->precision != HYP_PREC_MIXED) return HYP_ERR_INVALID;
  if (!valid_eos(cfg->eos[0]) || (cfg->model == HYP_MODEL_MULTI && !valid_eos(cfg->eos[1]))) return HYP_ERR_INVALID;
  // single phase: Rusanov or LxF, FP64 or mixed; two phases: path-conservative HLL (the
  // reference's main.jl:225 choice) or path-conservative LxF (main.jl:223), FP64 or mixed
  if (cfg->model == HYP_MODEL_SINGLE && cfg->flux == HYP_FLUX_HLL) return HYP_ERR_UNSUPPORTED;
  if (cfg->model == HYP_MODEL_MULTI && cfg->flux == HYP_FLUX_RUSANOV) return HYP_ERR_UNSUPPORTED;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  hyp_ctx* c = new (std::nothrow) hyp_ctx();
  if (!c) return HYP_ERR_INVALID;
  for (auto& e : c->ev) e = nullptr;
  c->cfg = *cfg;
  c->eos[0] = to_eos(cfg->eos[0]);
  c->eos[1] = to_eos(cfg->model == HYP_MODEL_MULTI ? cfg->eos[1] : cfg->eos[0]);
  c->eos_mixed = make_eos_mixed(c->eos[0]);
  c->n = cfg->n_cells;
  c->nvar = cfg->model == HYP_MODEL_SINGLE ? 14 : 30;
  int rc = HYP_OK;
  auto fail = [&](cudaError_t e, const char* what) {
    rc = HYP_ERR_CUDA;
    fprintf(stderr, "hyp_create: %s: %s\n", what, cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&c->device)) != cudaSuccess) fail(e, "cudaGetDevice");
  if (rc == HYP_OK && (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
    fail(e, "cudaStreamCreate");
  if (rc == HYP_OK && (e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
    fail(e, "cudaStreamCreate");
  for (auto& ev : c->row_ev)
    if (rc == HYP_OK && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      fail(e, "cudaEventCreate");
  const size_t nq = (size_t)c->nvar * c->n * sizeof(double);
  c->eos2.e[0] = c->eos[0];
  c->eos2.e[1] = c->eos[1];
  c->quad = gauss_legendre6();
  c->lobatto = gauss_lobatto6();
  if (cfg->model == HYP_MODEL_MULTI && mixed(c)) {
    // state [2 parities][30 hi + 30 lo rows][pitch] floats; a parity's block also stages
    // FP64 uploads and downloads (30 pitch doubles >= 30 n)
    c->mpitch = mixed_pitch(c->n);
    // phases as packed FP32 pairs in the face kernels: 2.72 against 2.89 ms per HLL step
    // (1.51 against 1.58 LxF) at 2^22 cells on GB300
    c->mixed_kind = HYP_MIXED_PAIR;
    const size_t nf4 = (size_t)30 * (c->n + 1) * sizeof(float);
    if ((e = cudaMalloc(&c->mixed_base, (size_t)2 * 60 * c->mpitch * sizeof(float))) != cudaSuccess)
      fail(e, "cudaMalloc(mixed state)");
    for (int p = 0; p < 2 && rc == HYP_OK; ++p) {
      c->Qh[p] = c->mixed_base + (size_t)p * 60 * c->mpitch;
      c->Ql[p] = c->Qh[p] + (size_t)30 * c->mpitch;
    }
    if (rc == HYP_OK && (e = cudaMalloc(&c->F32, (size_t)30 * c->n * sizeof(float))) != cudaSuccess)
      fail(e, "cudaMalloc(F)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->smin32, (size_t)c->n * sizeof(float))) != cudaSuccess) fail(e, "cudaMalloc(smin)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->smax32, (size_t)c->n * sizeof(float))) != cudaSuccess) fail(e, "cudaMalloc(smax)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->DM32, nf4)) != cudaSuccess) fail(e, "cudaMalloc(DM)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->DP32, nf4)) != cudaSuccess) fail(e, "cudaMalloc(DP)");
    if (rc == HYP_OK && cfg->flux == HYP_FLUX_LXF && (e = cudaMalloc(&c->FF32, nf4)) != cudaSuccess)
      fail(e, "cudaMalloc(face fluxes)");
  } else if (cfg->model == HYP_MODEL_MULTI) {
    const size_t nfb = (size_t)30 * (c->n + 1) * sizeof(double);
    for (int p = 0; p < 2 && rc == HYP_OK; ++p)
      if ((e = cudaMalloc(&c->Q[p], nq)) != cudaSuccess) fail(e, "cudaMalloc(Q)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->F, nq)) != cudaSuccess) fail(e, "cudaMalloc(F)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->smin, (size_t)c->n * sizeof(double))) != cudaSuccess) fail(e, "cudaMalloc(smin)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->smax, (size_t)c->n * sizeof(double))) != cudaSuccess) fail(e, "cudaMalloc(smax)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->DM, nfb)) != cudaSuccess) fail(e, "cudaMalloc(DM)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->DP, nfb)) != cudaSuccess) fail(e, "cudaMalloc(DP)");
    if (rc == HYP_OK && cfg->flux == HYP_FLUX_LXF && (e = cudaMalloc(&c->FF, nfb)) != cudaSuccess)
      fail(e, "cudaMalloc(face fluxes)");
  } else if (!mixed(c)) {
    for (int p = 0; p < 2 && rc == HYP_OK; ++p)
      if ((e = cudaMalloc(&c->Q[p], nq)) != cudaSuccess) fail(e, "cudaMalloc(Q)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->F, (size_t)kNFlux1 * c->n * sizeof(double))) != cudaSuccess)
      fail(e, "cudaMalloc(F)");
    if (rc == HYP_OK && (e = cudaMalloc(&c->lam, (size_t)c->n * sizeof(double))) != cudaSuccess)
      fail(e, "cudaMalloc(lam)");
  } else {
    // per parity one tile-major block of mixed_tiles(n) tiles x 32 rows (hi, lo, lambda,
    // islands: hyp_internal.cuh); a parity's block also stages FP64 uploads and downloads
    // (32 x 254 floats per 254 cells >= 14 doubles per cell)
    const size_t block = (size_t)mixed_tiles(c->n) * kTileFloats;
    if ((e = cudaMalloc(&c->mixed_base, 2 * block * sizeof(float))) != cudaSuccess) fail(e, "cudaMalloc(mixed state)");
    for (int p = 0; p < 2 && rc == HYP_OK; ++p) c->Qh[p] = c->mixed_base + (size_t)p * block;
    if (rc == HYP_OK && setup_mixed_tma(c) != 0) c->tma_grid = 0;  // TMA kernel unavailable
  }
  if (rc == HYP_OK && (e = cudaMalloc(&c->st, sizeof(DevState))) != cudaSuccess) fail(e, "cudaMalloc(state)");
  if (rc == HYP_OK && (e = cudaMallocHost(&c->st_host, sizeof(DevState))) != cudaSuccess) fail(e, "cudaMallocHost");
  for (auto& ev : c->ev)
    if (rc == HYP_OK && (e = cudaEventCreate(&ev)) != cudaSuccess) fail(e, "cudaEventCreate");
  if (rc == HYP_OK) {
    std::memset(c->st_host, 0, sizeof(DevState));
    if ((e = cudaMemcpy(c->st, c->st_host, sizeof(DevState), cudaMemcpyHostToDevice)) != cudaSuccess)
      fail(e, "cudaMemcpy(state)");
  }
  if (rc != HYP_OK) {
    free_ctx(c);
    return rc;
  }
  *out = c;
  return HYP_OK;
}

extern "C" int hyp_destroy(hyp_ctx* c) { return free_ctx(c); }

static int sync_state(hyp_ctx* c) {
  CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return HYP_OK;
}

int ctx_set_err(hyp_ctx* c, int code, const std::string& msg) { return set_err(c, code, msg); }
int ctx_sync_state(hyp_ctx* c) { return sync_state(c); }
static int check_cell_error(hyp_ctx* c);
int ctx_check_cell_error(hyp_ctx* c) { return check_cell_error(c); }

static int check_cell_error(hyp_ctx* c) {
  int code = c->st_host->err_code;
  if (!code) return HYP_OK;
  c->err_cell = c->st_host->err_cell;
  char buf[160];
  if (code & HYP_CELL_TIMEOUT) {
    snprintf(buf, sizeof buf, "a device wait for a tile load timed out (tile starting at cell %lld)", (long long)c->err_cell);
    return set_err(c, HYP_ERR_TIMEOUT, buf);
  }
  if (code & HYP_CELL_RELAX) {
    snprintf(buf, sizeof buf, "pressure relaxation did not converge in cell %lld (left unrelaxed)",
             (long long)c->err_cell);
    return set_err(c, HYP_ERR_NONFINITE, buf);
  }
  if (code & HYP_CELL_NEG_DET) {
    snprintf(buf, sizeof buf, "det(rho A) <= 0 in cell %lld (reference: DomainError in sqrt)", (long long)c->err_cell);
    return set_err(c, HYP_ERR_NEG_DET, buf);
  }
  snprintf(buf, sizeof buf, "non-finite state or wave speed in cell %lld", (long long)c->err_cell);
  return set_err(c, HYP_ERR_NONFINITE, buf);
}

// Where an FP64 state [nvar][n] goes before ctx_finish_install makes it current:
// the FP64 buffer of parity 0, or the mixed contexts' staging block.
double* ctx_install_target(hyp_ctx* c) { return mixed(c) ? (double*)c->Qh[1] : c->Q[0]; }

// Makes the FP64 state at src (null: ctx_install_target) the current state at time
// t0 (splits it into (hi, lo) pairs for mixed precision; for the single-phase mixed
// step, in the same pass, each cell's wave speed and islands) and resets the loop
// control.
int ctx_finish_install_from(hyp_ctx* c, const double* src, double t0) {
  std::memset(c->st_host, 0, sizeof(DevState));
  c->st_host->t[0] = c->st_host->t[1] = t0;
  CK(cudaMemcpyAsync(c->st, c->st_host, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
  if (mixed(c)) {
    const double* q = src ? src : ctx_install_target(c);
    if (mixed1(c))
      CK(launch_install1_mixed(c, q, &c->st->lam_slots[0]));
    else
      CK(launch_split(c, q, c->Qh[0], c->Ql[0]));
  }
  int rc = sync_state(c);
  if (rc != HYP_OK) return rc;
  c->cur = 0;
  c->has_state = 1;
  c->t_host = t0;
  c->steps_host = 0;
  c->err_cell = -1;
  return check_cell_error(c);
}

int ctx_finish_install(hyp_ctx* c, double t0) { return ctx_finish_install_from(c, nullptr, t0); }

// Device address of page-locked host memory (cudaHostAlloc / cudaHostRegister), or
// null for memory the device does not map (pageable, or not host memory).
static const double* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? (const double*)a.devicePointer : nullptr;
}

extern "C" int hyp_upload(hyp_ctx* c, const double* Q, int64_t n_cells, int n_vars, double t0) {
  if (!c || !Q) return HYP_ERR_INVALID;
  if (n_cells != c->n || n_vars != c->nvar) return set_err(c, HYP_ERR_INVALID, "hyp_upload: size mismatch");
  CK(cudaSetDevice(c->device));
  // Mixed precision from page-locked memory: the install kernel reads the host array
  // in place (one pass over the host link, split and wave speeds included) instead of
  // a copy into the staging block followed by a pass over it.
  const double* mapped = mixed(c) ? mapped_host(Q) : nullptr;
  if (mapped) return ctx_finish_install_from(c, mapped, t0);
  const size_t bytes = (size_t)n_vars * n_cells * sizeof(double);
  CK(cudaMemcpyAsync(ctx_install_target(c), Q, bytes, cudaMemcpyHostToDevice, c->stream));
  return ctx_finish_install(c, t0);
}

extern "C" int hyp_download(hyp_ctx* c, double* Q, int64_t n_cells, int n_vars) {
  if (!c || !Q) return HYP_ERR_INVALID;
  if (n_cells != c->n || n_vars != c->nvar) return set_err(c, HYP_ERR_INVALID, "hyp_download: size mismatch");
  CK(cudaSetDevice(c->device));
  const size_t bytes = (size_t)n_vars * n_cells * sizeof(double);
  if (!mixed(c)) {
    CK(cudaMemcpyAsync(Q, c->Q[c->cur], bytes, cudaMemcpyDeviceToHost, c->stream));
  } else if (bytes < ((size_t)64 << 20)) {
    double* stage = (double*)c->Qh[1 - c->cur];  // the other parity's block is free between steps
    CK(launch_join(c, c->cur, stage));
    CK(cudaMemcpyAsync(Q, stage, bytes, cudaMemcpyDeviceToHost, c->stream));
  } else {
    // large states: join one variable row at a time on the context stream and copy each
    // row out on the copy stream as soon as it is joined, so the joins hide behind the
    // device-to-host copies
    double* stage = (double*)c->Qh[1 - c->cur];
    const size_t row = (size_t)n_cells * sizeof(double);
    for (int v = 0; v < n_vars; ++v) {
      CK(launch_join_rows(c, c->cur, stage + (size_t)v * n_cells, v, 1));
      CK(cudaEventRecord(c->row_ev[v], c->stream));
      CK(cudaStreamWaitEvent(c->copy_stream, c->row_ev[v], 0));
      CK(cudaMemcpyAsync(Q + (size_t)v * n_cells, stage + (size_t)v * n_cells, row, cudaMemcpyDeviceToHost,
                         c->copy_stream));
    }
    CK(cudaStreamSynchronize(c->copy_stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return HYP_OK;
}

// Profiling: each kernel is bracketed by events from the context's pool; the
// durations are summed when hyp_step finishes.
static int prof_event(hyp_ctx* c, cudaEvent_t* out) {
  if (c->prof_used == c->prof_ev.size()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->prof_ev.push_back(e);
  }
  *out = c->prof_ev[c->prof_used++];
  return HYP_OK;
}

// Enqueue step number k (k = steps taken since the upload + steps already
// enqueued); no host synchronisation.
static int enqueue_step(hyp_ctx* c, long long k, double t_end, bool prof) {
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  int rc;
  if (prof) {
    if ((rc = prof_event(c, &e0)) || (rc = prof_event(c, &e1)) || (rc = prof_event(c, &e2))) return rc;
    CK(cudaEventRecord(e0, c->stream));
  }
  if (c->cfg.model == HYP_MODEL_MULTI && mixed(c)) {
    const int p = (int)(k & 1);
    CK(launch_cell2_mixed(c, p, &c->st->lam_bits[p], &c->st->t[p], t_end));
    if (fused_face_update2_mixed(c)) {  // pair faces; profiled as cell, then faces + update
      if (prof) CK(cudaEventRecord(e1, c->stream));
      CK(launch_face_update2_mixed(c, p, t_end));
    } else {
      CK(launch_face2_mixed(c, p, t_end));
      if (prof) CK(cudaEventRecord(e1, c->stream));
      CK(launch_update2_mixed(c, p, t_end));
    }
    if (c->relax) CK(launch_relax2(c, p, t_end));
  } else if (c->cfg.model == HYP_MODEL_MULTI) {
    const int p = (int)(k & 1);
    CK(launch_cell2_f64(c, p, &c->st->lam_bits[p], &c->st->t[p], t_end));
    CK(launch_face2_f64(c, p, t_end));
    if (prof) CK(cudaEventRecord(e1, c->stream));
    CK(launch_update2_f64(c, p, t_end));
    if (c->relax) CK(launch_relax2(c, p, t_end));
  } else if (!mixed(c)) {
    const int p = (int)(k & 1);
    CK(launch_cell1_f64(c, p, &c->st->lam_bits[p], &c->st->t[p], t_end));
    if (prof) CK(cudaEventRecord(e1, c->stream));
    CK(launch_update1_f64(c, p, t_end));
  } else {
    CK(launch_step1_mixed(c, k, t_end));
    if (prof) CK(cudaEventRecord(e1, c->stream));
  }
  if (prof) CK(cudaEventRecord(e2, c->stream));
  return HYP_OK;
}

static int collect_profile(hyp_ctx* c) {
  for (size_t k = 0; k + 3 <= c->prof_used; k += 3) {
    float a = 0.f, b = 0.f;
    CK(cudaEventElapsedTime(&a, c->prof_ev[k], c->prof_ev[k + 1]));
    CK(cudaEventElapsedTime(&b, c->prof_ev[k + 1], c->prof_ev[k + 2]));
    c->timing.ms_cell += a;
    c->timing.n_cell += 1;
    if (!mixed1(c)) {  // the single-phase mixed step is one kernel
      c->timing.ms_update += b;
      c->timing.n_update += 1;
    }
  }
  c->prof_used = 0;
  return HYP_OK;
}

// steps per captured graph: a multiple of the launch pattern's period
static int graph_period(const hyp_ctx* c) { return mixed1(c) ? 6 : 2; }
static int graph_steps(const hyp_ctx* c) { return mixed1(c) ? 12 : 16; }

static int ensure_graph(hyp_ctx* c, long long k0, double t_end) {
  const int key = (int)(k0 % graph_period(c));
  if (c->graph_t_end != t_end || c->graph_steps != graph_steps(c)) {
    for (auto& g : c->graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    c->graph_t_end = t_end;
    c->graph_steps = graph_steps(c);
  }
  if (c->graph[key]) return HYP_OK;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = HYP_OK;
  for (int s = 0; s < c->graph_steps && rc == HYP_OK; ++s) rc = enqueue_step(c, k0 + s, t_end, false);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc != HYP_OK) return rc;
  if (e != cudaSuccess) return set_err(c, HYP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&c->graph[key], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(c, HYP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return HYP_OK;
}

// hyp_step_times: the time after a step, copied once the step's kernels are done
__global__ void log_time_kernel(const DevState* S, int parity, double* out) { *out = S->t[parity]; }

extern "C" int hyp_step(hyp_ctx* c, int max_steps, double t_end, int* steps_done, double* t_out) {
  if (!c) return HYP_ERR_INVALID;
  if (std::isnan(t_end)) return set_err(c, HYP_ERR_INVALID, "t_end is NaN");
  CK(cudaSetDevice(c->device));
  const bool unlimited = max_steps <= 0;
  if (unlimited && std::isinf(t_end)) return set_err(c, HYP_ERR_INVALID, "hyp_step: neither max_steps nor t_end bounds the run");
  if (c->slab) return set_err(c, HYP_ERR_UNSUPPORTED, "hyp_step: a slab steps with the global max (hyp_slab_step)");
  c->timing = StepTiming();
  c->prof_used = 0;
  const long long steps0 = c->steps_host;
  CK(cudaEventRecord(c->ev[0], c->stream));
  long long launched = 0;
  const bool prof = c->profiling != 0;
  // With a finite t_end, steps past t_end are no-ops on the device; launch in
  // chunks and stop once the device reports t >= t_end.
  const long long chunk = std::isinf(t_end) ? (unlimited ? 0 : max_steps) : 256;
  const int gs = graph_steps(c);
  int rc = HYP_OK;
  while (rc == HYP_OK) {
    long long todo = unlimited ? chunk : (max_steps - launched);
    if (!std::isinf(t_end) && todo > chunk) todo = chunk;
    if (todo <= 0) break;
    // Every launched step advances the pattern index. An inactive step (t >= t_end)
    // copies t across and leaves the state and its max-lambda slot alone; active
    // steps always precede inactive ones, so the state index is steps0 + active.
    long long k = steps0 + launched;
    long long s = 0;
    if (!prof && !c->hist_on) {
      while (rc == HYP_OK && todo - s >= gs) {
        rc = ensure_graph(c, k, t_end);
        if (rc == HYP_OK) {
          cudaError_t e = cudaGraphLaunch(c->graph[k % graph_period(c)], c->stream);
          if (e != cudaSuccess) rc = set_err(c, HYP_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
        }
        s += gs;
        k += gs;
      }
    }
    for (; rc == HYP_OK && s < todo; ++s, ++k) {
      rc = enqueue_step(c, k, t_end, prof);
      if (rc == HYP_OK && c->hist_on) {  // t after step k (an inactive step carries t across)
        log_time_kernel<<<1, 1, 0, c->stream>>>(c->st, (int)((k + 1) & 1), c->hist_dev + (k - steps0));
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = set_err(c, HYP_ERR_CUDA, std::string("log_time_kernel: ") + cudaGetErrorString(e));
      }
    }
    launched += todo;
    if (rc != HYP_OK) break;
    if (!std::isinf(t_end)) {
      rc = sync_state(c);
      if (rc != HYP_OK) break;
      if (c->st_host->err_code) break;
      double tl = c->st_host->t[(steps0 + launched) & 1];
      if (!(tl < t_end)) break;
    }
    if (std::isinf(t_end)) break;
  }
  CK(cudaEventRecord(c->ev[1], c->stream));
  if (rc == HYP_OK) rc = sync_state(c);
  if (rc != HYP_OK) return rc;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->timing.ms_total = ms;
  if (prof && (rc = collect_profile(c)) != HYP_OK) return rc;
  const long long active = c->st_host->steps - steps0;
  c->cur = (int)((c->cur + active) & 1);
  c->steps_host = c->st_host->steps;
  c->t_host = c->st_host->t[c->cur];
  if (steps_done) *steps_done = (int)active;
  if (t_out) *t_out = c->t_host;
  return check_cell_error(c);
}

extern "C" int hyp_step_times(hyp_ctx* c, int max_steps, double t_end, int* steps_done, double* t_out,
                              double* t_hist) {
  if (!c) return HYP_ERR_INVALID;
  if (max_steps <= 0 || !t_hist) return set_err(c, HYP_ERR_INVALID, "hyp_step_times: needs max_steps >= 1 and t_hist");
  CK(cudaSetDevice(c->device));
  if (c->hist_cap < max_steps) {
    cudaFree(c->hist_dev);
    c->hist_dev = nullptr;
    c->hist_cap = 0;
    CK(cudaMalloc(&c->hist_dev, (size_t)max_steps * sizeof(double)));
    c->hist_cap = max_steps;
  }
  // steps launched one by one (no step graphs), each followed by log_time_kernel;
  // writing the log inside the step kernels measured 0.5-1.8 % slower steps
  c->hist_on = 1;
  int done = 0;
  const int rc = hyp_step(c, max_steps, t_end, &done, t_out);
  c->hist_on = 0;
  if (steps_done) *steps_done = done;
  const bool cell_err = rc == HYP_ERR_NEG_DET || rc == HYP_ERR_NONFINITE;
  if ((rc == HYP_OK || cell_err) && done > 0) {  // the steps taken before a cell error are logged too
    CK(cudaMemcpyAsync(t_hist, c->hist_dev, (size_t)done * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return rc;
}

extern "C" int hyp_set_eos(hyp_ctx* c, int phase, const hyp_barton2009* eos) {
  if (!c || !eos) return HYP_ERR_INVALID;
  if (phase < 0 || phase > 1 || (phase == 1 && c->cfg.model != HYP_MODEL_MULTI))
    return set_err(c, HYP_ERR_INVALID, "hyp_set_eos: phase must be 0, or 1 for a two-phase context");
  if (!valid_eos(*eos)) return set_err(c, HYP_ERR_INVALID, "hyp_set_eos: invalid Barton2009 parameters");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  c->cfg.eos[phase] = *eos;
  c->eos[phase] = to_eos(*eos);
  if (c->cfg.model == HYP_MODEL_SINGLE) {  // a single-phase context keeps both slots equal (hyp_create)
    c->cfg.eos[1] = *eos;
    c->eos[1] = c->eos[0];
  }
  c->eos2.e[0] = c->eos[0];
  c->eos2.e[1] = c->eos[1];
  c->eos_mixed = make_eos_mixed(c->eos[0]);
  for (auto& g : c->graph)  // the captured steps hold the old parameters by value
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  c->graph_steps = 0;
  free_tape(c);  // a recorded run belongs to the old parameters
  if (mixed1(c) && c->has_state) {
    // the mixed step caches each cell's wave speed and float-float islands, which
    // depend on the EOS: recompute them for the current state (its slot k % 3)
    unsigned long long* slot = &c->st->lam_slots[c->steps_host % 3];
    CK(cudaMemsetAsync(slot, 0, sizeof *slot, c->stream));
    CK(launch_lam1_mixed(c, c->cur, slot));
    int rc = sync_state(c);
    if (rc != HYP_OK) return rc;
    return check_cell_error(c);
  }
  return HYP_OK;
}

extern "C" int hyp_set_wait_limit(hyp_ctx* c, int tries) {
  if (!c || tries < 0) return HYP_ERR_INVALID;
  c->wait_tries = tries;
  for (auto& g : c->graph)  // graphs hold the previous kernel arguments
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  c->graph_steps = 0;
  return HYP_OK;
}

extern "C" int hyp_set_mixed_kernel(hyp_ctx* c, int kind) {
  if (!c) return HYP_ERR_INVALID;
  if (!mixed(c)) return set_err(c, HYP_ERR_UNSUPPORTED, "hyp_set_mixed_kernel: mixed-precision contexts only");
  if (kind != HYP_MIXED_TILE && kind != HYP_MIXED_TMA && kind != HYP_MIXED_PAIR)
    return set_err(c, HYP_ERR_UNSUPPORTED, "hyp_set_mixed_kernel: unknown kernel kind");
  if (kind == HYP_MIXED_TMA && (c->cfg.model != HYP_MODEL_SINGLE || !c->tma_grid))
    return set_err(c, HYP_ERR_UNSUPPORTED, "hyp_set_mixed_kernel: TMA is not available");
  c->mixed_kind = kind;
  for (auto& g : c->graph)  // graphs hold the previous kernel
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  c->graph_steps = 0;
  return HYP_OK;
}

extern "C" int hyp_max_wavespeed(hyp_ctx* c, double* out) {
  if (!c || !out) return HYP_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  if (mixed1(c)) {  // kept by the last step (or the upload) for the current state
    int rc = sync_state(c);
    if (rc != HYP_OK) return rc;
    unsigned bits = (unsigned)c->st_host->lam_slots[c->steps_host % 3];
    float v;
    std::memcpy(&v, &bits, sizeof v);
    *out = v;
    return check_cell_error(c);
  }
  CK(cudaMemsetAsync(&c->st->lam_query, 0, sizeof(unsigned long long), c->stream));
  if (c->cfg.model == HYP_MODEL_MULTI && mixed(c))
    CK(launch_cell2_mixed(c, c->cur, &c->st->lam_query, &c->st->t[c->cur], INFINITY));
  else if (c->cfg.model == HYP_MODEL_MULTI)
    CK(launch_cell2_f64(c, c->cur, &c->st->lam_query, &c->st->t[c->cur], INFINITY));
  else
    CK(launch_cell1_f64(c, c->cur, &c->st->lam_query, &c->st->t[c->cur], INFINITY));
  int rc = sync_state(c);
  if (rc != HYP_OK) return rc;
  unsigned long long b = c->st_host->lam_query;
  double v;
  std::memcpy(&v, &b, sizeof v);
  *out = v;
  return check_cell_error(c);
}

extern "C" int hyp_get_time(const hyp_ctx* c, double* t, int64_t* steps) {
  if (!c) return HYP_ERR_INVALID;
  if (t) *t = c->t_host;
  if (steps) *steps = c->steps_host;
  return HYP_OK;
}

extern "C" int hyp_set_profiling(hyp_ctx* c, int on) {
  if (!c) return HYP_ERR_INVALID;
  c->profiling = on;
  return HYP_OK;
}

extern "C" int hyp_last_timing(const hyp_ctx* c, double* ms_total, double* ms_cell, int* n_cell, double* ms_update,
                               int* n_update) {
  if (!c) return HYP_ERR_INVALID;
  if (ms_total) *ms_total = c->timing.ms_total;
  if (ms_cell) *ms_cell = c->timing.ms_cell;
  if (n_cell) *n_cell = c->timing.n_cell;
  if (ms_update) *ms_update = c->timing.ms_update;
  if (n_update) *n_update = c->timing.n_update;
  return HYP_OK;
}

extern "C" int hyp_host_alloc(int64_t bytes, void** out) {
  if (!out || bytes <= 0) return HYP_ERR_INVALID;
  *out = nullptr;
  cudaError_t e = cudaMallocHost(out, (size_t)bytes);
  return e == cudaSuccess ? HYP_OK : HYP_ERR_CUDA;
}

extern "C" int hyp_host_free(void* p) {
  if (!p) return HYP_OK;
  return cudaFreeHost(p) == cudaSuccess ? HYP_OK : HYP_ERR_CUDA;
}
