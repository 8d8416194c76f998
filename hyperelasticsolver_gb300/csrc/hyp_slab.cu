// hyp_slab.cu -- a single-phase context as one slab of a 1D domain decomposed
// across processes (one GPU each).
//
// The reference advances one domain with a thread pool (main.jl:206, 221). Split
// into contiguous slabs, rank r holds the cells it updates plus one ghost cell at
// each inner end (a copy of the neighbour's boundary cell), and a step becomes:
//   1. the local max wave speed of the cells the rank owns (hyp_slab_local_max);
//   2. a max-allreduce of it across ranks (the caller's communicator);
//   3. the step with that global max, ghosts held (hyp_slab_step);
//   4. the exchange of boundary-cell records with the neighbours (hyp_get_cells /
//      hyp_set_cells).
// Each face sees the same two cell states as in the single-domain run and the max
// is exact, so with the global dx the slabs reproduce the single-domain run bit
// for bit. The global end cells keep the configuration's bc; a ghost end is held.
//
// Records: FP64 contexts move the 14 conservative values of a cell; mixed contexts
// the 32 floats of the tile layout (14 hi, 14 lo, the cell's wave speed and its
// three island outputs), so a ghost arrives with the speed and islands its owner
// computed and the next step's faces need nothing recomputed.
#include <cmath>
#include <cstring>
#include <string>
#include <algorithm>
#include "hyp_internal.cuh"

using namespace hyp;

#define SCK(call)                                                                                      \
  do {                                                                                                 \
    cudaError_t _e = (call);                                                                           \
    if (_e != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

double ctx_dx(const hyp_ctx* c) { return c->slab ? c->slab_dx : c->cfg.x_length / (double)c->n; }

int ctx_bc(const hyp_ctx* c) {
  if (!c->slab) return c->cfg.bc;
  const bool frozen = c->cfg.bc == HYP_BC_FROZEN;
  const bool first = frozen || c->slab_ghost[0], last = frozen || c->slab_ghost[1];
  return first && last ? HYP_BC_FROZEN : (first ? kBcHoldFirst : (last ? kBcHoldLast : HYP_BC_TRANSMISSIVE));
}

static bool slab_ok(const hyp_ctx* c) { return c->cfg.model == HYP_MODEL_SINGLE && c->cfg.flux != HYP_FLUX_HLL; }

extern "C" int hyp_set_slab(hyp_ctx* c, double dx, int left_ghost, int right_ghost) {
  if (!c) return HYP_ERR_INVALID;
  if (!slab_ok(c)) return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "hyp_set_slab: single-phase contexts only");
  if (!(dx > 0) || !std::isfinite(dx)) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_set_slab: dx must be > 0");
  c->slab = 1;
  c->slab_dx = dx;
  c->slab_ghost[0] = left_ghost != 0;
  c->slab_ghost[1] = right_ghost != 0;
  c->slab_cell_pass = -1;
  return HYP_OK;
}

extern "C" int hyp_cell_record_size(const hyp_ctx* c, int* bytes) {
  if (!c || !bytes) return HYP_ERR_INVALID;
  if (c->cfg.model != HYP_MODEL_SINGLE) return HYP_ERR_UNSUPPORTED;
  *bytes = c->cfg.precision == HYP_PREC_MIXED ? kMixedRows * (int)sizeof(float) : 14 * (int)sizeof(double);
  return HYP_OK;
}

// Copies the records of cells [first, first + count) between the current state and
// rec ([rows][count], host or device memory: cudaMemcpyDefault resolves which). FP64:
// 14 rows of the row-major [14][n] state. Mixed: the 32 rows of the tile-major block,
// one 2D copy per tile the range touches.
static int cells_copy(hyp_ctx* c, int64_t first, int64_t count, void* rec, bool to_ctx) {
  if (!c || !rec || count <= 0 || first < 0 || first + count > c->n) return HYP_ERR_INVALID;
  if (c->cfg.model != HYP_MODEL_SINGLE) return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "cell records: single phase only");
  if (!c->has_state) return ctx_set_err(c, HYP_ERR_INVALID, "cell records: no state uploaded");
  SCK(cudaSetDevice(c->device));
  const bool mixed = c->cfg.precision == HYP_PREC_MIXED;
  const size_t elem = mixed ? sizeof(float) : sizeof(double);
  const int rows = mixed ? kMixedRows : 14;
  const size_t rec_pitch = (size_t)count * elem;
  for (int64_t i = first; i < first + count;) {
    char* dev;
    size_t pitch;
    int64_t run;
    if (mixed) {  // the rest of cell i's tile
      run = std::min<int64_t>(first + count - i, kTileCells - i % kTileCells);
      dev = (char*)(c->Qh[c->cur] + tile_cell_off(i));
      pitch = (size_t)kTileRow * sizeof(float);
    } else {
      run = first + count - i;
      dev = (char*)(c->Q[c->cur] + i);
      pitch = (size_t)c->n * sizeof(double);
    }
    char* host = (char*)rec + (size_t)(i - first) * elem;
    const size_t w = (size_t)run * elem;
    if (to_ctx)
      SCK(cudaMemcpy2DAsync(dev, pitch, host, rec_pitch, w, rows, cudaMemcpyDefault, c->stream));
    else
      SCK(cudaMemcpy2DAsync(host, rec_pitch, dev, pitch, w, rows, cudaMemcpyDefault, c->stream));
    i += run;
  }
  SCK(cudaStreamSynchronize(c->stream));
  if (to_ctx) c->slab_cell_pass = -1;  // a changed cell invalidates an FP64 cell pass
  return HYP_OK;
}

extern "C" int hyp_get_cells(hyp_ctx* c, int64_t first, int64_t count, void* rec) {
  return cells_copy(c, first, count, rec, false);
}
extern "C" int hyp_set_cells(hyp_ctx* c, int64_t first, int64_t count, const void* rec) {
  return cells_copy(c, first, count, const_cast<void*>(rec), true);
}

// FP64: the cell pass (fluxes and wave speeds of every slab cell, ghosts included:
// they hold their owner's current values) of the current state, its max into
// lam_bits[p]. Mixed: the max the last step (or the upload) left in the read slot.
extern "C" int hyp_slab_local_max(hyp_ctx* c, double* lam) {
  if (!c || !lam) return HYP_ERR_INVALID;
  if (!c->slab) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_slab_local_max: not a slab (hyp_set_slab)");
  if (!c->has_state) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_slab_local_max: no state uploaded");
  SCK(cudaSetDevice(c->device));
  const long long k = c->steps_host;
  if (c->cfg.precision == HYP_PREC_MIXED) {
    unsigned long long bits = 0;
    SCK(cudaMemcpyAsync(&bits, &c->st->lam_slots[k % 3], sizeof bits, cudaMemcpyDeviceToHost, c->stream));
    SCK(cudaStreamSynchronize(c->stream));
    const unsigned u = (unsigned)bits;
    float f;
    memcpy(&f, &u, sizeof f);
    *lam = (double)f;
    return HYP_OK;
  }
  const int p = (int)(k & 1);
  SCK(cudaMemsetAsync(&c->st->lam_bits[p], 0, sizeof(unsigned long long), c->stream));
  SCK(launch_cell1_f64(c, p, &c->st->lam_bits[p], &c->st->t[p], INFINITY));
  int rc = ctx_sync_state(c);
  if (rc != HYP_OK) return rc;
  c->slab_cell_pass = k;
  if ((rc = ctx_check_cell_error(c)) != HYP_OK) return rc;
  unsigned long long bits = c->st_host->lam_bits[p];
  double v;
  memcpy(&v, &bits, sizeof v);
  *lam = v;
  return HYP_OK;
}

// One step with the global max wave speed lam_max (the max over every rank's local
// max): dt = cfl dx / lam_max as in main.jl:212, ghosts held.
extern "C" int hyp_slab_step(hyp_ctx* c, double lam_max, double* t_out) {
  if (!c) return HYP_ERR_INVALID;
  if (!c->slab) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_slab_step: not a slab (hyp_set_slab)");
  if (!c->has_state) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_slab_step: no state uploaded");
  if (!(lam_max > 0) || !std::isfinite(lam_max)) return ctx_set_err(c, HYP_ERR_NONFINITE, "hyp_slab_step: lam_max");
  SCK(cudaSetDevice(c->device));
  const long long k = c->steps_host;
  const int p = (int)(k & 1);
  if (c->cfg.precision == HYP_PREC_MIXED) {
    const float lf = (float)lam_max;  // an allreduced max of FP32 speeds: exact in FP32
    unsigned u;
    memcpy(&u, &lf, sizeof u);
    const unsigned long long bits = u;
    SCK(cudaMemcpyAsync(&c->st->lam_slots[k % 3], &bits, sizeof bits, cudaMemcpyHostToDevice, c->stream));
    SCK(launch_step1_mixed(c, k, INFINITY));
  } else {
    if (c->slab_cell_pass != k) {
      SCK(cudaMemsetAsync(&c->st->lam_bits[p], 0, sizeof(unsigned long long), c->stream));
      SCK(launch_cell1_f64(c, p, &c->st->lam_bits[p], &c->st->t[p], INFINITY));
    }
    unsigned long long bits;
    memcpy(&bits, &lam_max, sizeof bits);
    SCK(cudaMemcpyAsync(&c->st->lam_bits[p], &bits, sizeof bits, cudaMemcpyHostToDevice, c->stream));
    SCK(launch_update1_f64(c, p, INFINITY));
  }
  int rc = ctx_sync_state(c);
  if (rc != HYP_OK) return rc;
  c->slab_cell_pass = -1;
  c->cur = 1 - c->cur;
  c->steps_host = c->st_host->steps;
  c->t_host = c->st_host->t[c->cur];
  if (t_out) *t_out = c->t_host;
  return ctx_check_cell_error(c);
}
