// hyp_batch.cu -- many independent single-phase problems of uneven size advanced
// together (the reference runs one problem per main.jl invocation).
//
// All problems' cells sit back to back in one structure-of-arrays state
// ([var][total]); problem p owns cells [offsets[p], offsets[p+1]) with its own
// dx = X / N_p, CFL time step, time and step count (main.jl:202-227 per
// problem). A tile table assigns each work item to one problem (tiles never
// span two problems; halos clamp at the problem's ends). The step kernels are
// persistent (grid = SMs x resident blocks, a loop over tiles), one launch per
// step, and a whole run of steps is captured as one CUDA graph.
//
// Mixed precision: the tile body of hyp_mixed_tile.cuh on a tile-major state block
// (hyp_internal.cuh): every problem is cut into tiles of kTileCells cells, and tile
// t of the tile table (problems in order) owns span t of the block, so that a
// problem's tiles are consecutive spans and a tile's halo cells are the edge cells
// of its neighbouring spans (at a problem's ends the clamped ghost is in the tile
// itself). The autotuner times the grid variants (persistent at 4 or 3 resident
// blocks per SM, or one block per tile) on the batch itself and keeps the fastest.
// FP64: per-cell flux / wave speed then update, on row-major [var][cell] states.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include "hyp_internal.cuh"
#include "hyp_mixed_tile.cuh"

namespace hyp {

struct TileDesc {
  int64_t first;  // first owned cell
  int64_t lo, hi; // the problem's cells [lo, hi)
  int problem;
  int lead;       // 1 for the problem's first tile: it advances the problem's time
};

// A tile's step control, written each step by batch_mixed_ctl_kernel so that the
// tile kernel reads it alongside the tile descriptor (no dependent load).
struct TileCtl {
  float dtdx;
  int active;
};

// Per-problem loop control on the device.
struct BatchDev {
  double* t;                   // [2][P] time before the step of parity p
  unsigned long long* slots;   // mixed: [3][P] FP32 max-lambda bits; FP64: [2][P] FP64 max-lambda bits
  long long* steps;            // [P]
  double* dx;                  // [P]
  int P;
};


// ---- mixed precision ---------------------------------------------------------
// Step control of every tile: dt/dx and whether its problem is still running;
// the problem's lead tile advances the problem's time and step count and
// rotates its max-lambda slots (read rd, write wr, clear clr; a finished
// problem carries its max lambda from rd to wr).
__global__ void batch_mixed_ctl_kernel(const TileDesc* __restrict__ tiles, int ntiles, BatchDev b, int par, int rd,
                                       int wr, int clr, double t_end, double cfl, TileCtl* __restrict__ ctl) {
  const int tix = blockIdx.x * blockDim.x + threadIdx.x;
  if (tix >= ntiles) return;
  const int P = b.P;
  const TileDesc d = tiles[tix];
  const int p = d.problem;
  const double tn = b.t[par * P + p];
  const bool active = tn < t_end;
  const float lmax = __uint_as_float((unsigned)b.slots[rd * P + p]);
  ctl[tix] = TileCtl{(float)cfl / lmax, active ? 1 : 0};
  if (d.lead) {
    const double dt = (cfl * b.dx[p]) / (double)lmax;
    b.t[(1 - par) * P + p] = active ? tn + dt : tn;
    b.slots[clr * P + p] = 0ull;
    if (active) b.steps[p] += 1;
    else b.slots[wr * P + p] = b.slots[rd * P + p];  // a finished problem keeps its max lambda
  }
}

// One tile of the batch: its problem's step (or, for a finished problem, its cells
// carried to the other buffer), the block max of the new wave speeds into the
// problem's slot.
template <int BLOCK, bool kOwnRegs>
__device__ __forceinline__ void batch_tile(const MixedArrays& a, const EosMixed& em, const TileDesc& d,
                                           const TileCtl& k, int tix, unsigned long long* slots_wr, int flux, int bc,
                                           DevState* S) {
  const TileOrigin org{(int64_t)tix * kTileFloats, d.first};
  const MixedGlobalLoader<BLOCK, true> ld{a, org};
  MixedCellIn c;
  mixed_tile_load<BLOCK>(d.first, d.lo, d.hi, ld, c);
  if (!k.active) {  // uniform over the block: carry the problem's cells to the other buffer unchanged
    const int j = tile_local<BLOCK>();
    const int64_t i = d.first - 1 + j;
    if (j > 0 && j < BLOCK - 1 && i < d.hi) mixed_store_cell(a.out + org.base + (j - 1), kTileRow, c.qh, c.ql, c.li, c.I0);
    return;
  }
  const float l = mixed_tile_run<BLOCK, kOwnRegs, true>(a, em, d.first, d.lo, d.hi, k.dtdx, flux, bc, S, ld, c);
  const float m = mixed_block_max<BLOCK>(l);
  if (threadIdx.x == 0) atomicMax(&slots_wr[d.problem], (unsigned long long)__float_as_uint(m));
}

// Persistent grid: each block strides over the tile table. Faces from shared memory:
// at 64 registers the loop's state leaves no room for the own-register faces.
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
    batch_mixed_kernel(MixedArrays a, EosMixed em, const TileDesc* __restrict__ tiles,
                       const TileCtl* __restrict__ ctl, int ntiles, unsigned long long* __restrict__ slots_wr,
                       int flux, int bc, DevState* S) {
  for (int tix = blockIdx.x; tix < ntiles; tix += gridDim.x) {
    const TileDesc d = tiles[tix];
    const TileCtl k = ctl[tix];
    batch_tile<BLOCK, false>(a, em, d, k, tix, slots_wr, flux, bc, S);
    __syncthreads();  // the shared scratch is reused by the next tile
  }
}

// One block per tile.
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
    batch_tile_kernel(MixedArrays a, EosMixed em, const TileDesc* __restrict__ tiles, const TileCtl* __restrict__ ctl,
                      unsigned long long* __restrict__ slots_wr, int flux, int bc, DevState* S) {
  const int tix = blockIdx.x;
  const TileDesc d = tiles[tix];
  const TileCtl k = ctl[tix];
  batch_tile<BLOCK, true>(a, em, d, k, tix, slots_wr, flux, bc, S);
}

// An uploaded batch installed in one pass, one block per tile: thread j reads cell
// first + j's 14 FP64 values from the staged [14][total] array, splits them into
// (hi, lo) pairs into slot j of the tile's span, and computes the cell's wave speed
// and island outputs there (mixed_cell_lambda_of); the problem's max lambda into its
// slot 0.
__global__ void __launch_bounds__(kBlock) batch_install_kernel(const double* __restrict__ q, int64_t total,
                                                               float* __restrict__ out, EosMixed em,
                                                               const TileDesc* __restrict__ tiles, int ntiles,
                                                               BatchDev b, DevState* S) {
  for (int tix = blockIdx.x; tix < ntiles; tix += gridDim.x) {
    const TileDesc d = tiles[tix];
    const int64_t i = d.first + threadIdx.x;
    float l = 0.0f;
    if (threadIdx.x < kTileCells && i < d.hi) {
      float qh[14], ql[14];
      float* o = out + (int64_t)tix * kTileFloats + threadIdx.x;
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        const double x = q[v * total + i];
        qh[v] = (float)x;
        ql[v] = (float)(x - (double)qh[v]);
        o[v * kTileRow] = qh[v];
        o[(kRowLo + v) * kTileRow] = ql[v];
      }
      l = mixed_cell_lambda_of(em, qh, ql, i, S, o, kTileRow);
    }
    l = mixed_block_max<kBlock>(l);
    if (threadIdx.x == 0) atomicMax(&b.slots[d.problem], (unsigned long long)__float_as_uint(l));
    __syncthreads();
  }
}

// The batch's FP64 state [14][total] from a tile-major block, one block per tile.
__global__ void __launch_bounds__(kBlock) batch_join_kernel(const float* __restrict__ in, int64_t total,
                                                            double* __restrict__ q, const TileDesc* __restrict__ tiles,
                                                            int ntiles) {
  for (int tix = blockIdx.x; tix < ntiles; tix += gridDim.x) {
    const TileDesc d = tiles[tix];
    const int64_t i = d.first + threadIdx.x;
    if (threadIdx.x < kTileCells && i < d.hi) {
      const float* c = in + (int64_t)tix * kTileFloats + threadIdx.x;
#pragma unroll
      for (int v = 0; v < 14; ++v) q[v * total + i] = (double)c[v * kTileRow] + (double)c[(kRowLo + v) * kTileRow];
    }
  }
}

// ---- FP64 ----------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) batch_f64_cell_kernel(const double* __restrict__ Q, int64_t n, EosC e,
                                                                double* __restrict__ F, double* __restrict__ lam,
                                                                const TileDesc* __restrict__ tiles, int ntiles,
                                                                int tile_cells, BatchDev b, int par, double t_end,
                                                                unsigned long long* slot_base, DevState* S) {
  const int P = b.P;
  for (int tix = blockIdx.x; tix < ntiles; tix += gridDim.x) {
    const TileDesc d = tiles[tix];
    if (!(b.t[par * P + d.problem] < t_end)) continue;
    double l = 0.0;
    for (int64_t i = d.first + threadIdx.x; i < d.first + tile_cells && i < d.hi; i += kBlock) {
      double q[14];
#pragma unroll
      for (int v = 0; v < 14; ++v) q[v] = Q[v * n + i];
      Prim Pm;
      int st = cons_to_prim(e, 1.0, q + 1, q[4], q + 5, Pm);
      StressC c = stress_coeffs(e, Pm.k, Pm.w, Pm.xm1);
      double f[14], s0[3];
      phase_flux(e, 1.0, Pm, c, f, s0);
      const double li = fabs(Pm.u[0]) + phase_cmax(e, Pm, c);
      if (!(li <= 1.79e308)) st |= HYP_CELL_NONFINITE;
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        const int sl = flux_slot1(v);
        if (sl >= 0) F[sl * n + i] = f[v];
      }
      lam[i] = li;
      if (st) mixed_record_err(S, st, i);
      l = fmax(l, li);
    }
    __shared__ double red[kBlock / 32];
    for (int o = 16; o > 0; o >>= 1) l = fmax(l, __shfl_xor_sync(0xffffffffu, l, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = red[0];
      for (int w = 1; w < kBlock / 32; ++w) m = fmax(m, red[w]);
      atomicMax(&slot_base[d.problem], (unsigned long long)__double_as_longlong(m));
    }
    __syncthreads();
  }
}

// One tile of kBlock cells per block iteration (tile_cells == kBlock for the FP64
// batch); each face of the tile once into shared memory, as update1_f64_kernel.
__global__ void __launch_bounds__(kBlock) batch_f64_update_kernel(const double* __restrict__ Q, double* __restrict__ Qn,
                                                                  int64_t n, const double* __restrict__ F,
                                                                  const double* __restrict__ lam,
                                                                  const TileDesc* __restrict__ tiles, int ntiles,
                                                                  int tile_cells, BatchDev b, int par, double t_end,
                                                                  double cfl, int flux, int bc) {
  __shared__ double sF[14][kBlock + 1];  // face k of the tile = left face of cell first + k
  const int P = b.P;
  const bool lxf = flux == HYP_FLUX_LXF;
  for (int tix = blockIdx.x; tix < ntiles; tix += gridDim.x) {
    const TileDesc d = tiles[tix];
    const int p = d.problem;
    const double tn = b.t[par * P + p];
    const bool active = tn < t_end;
    const double lmax = __longlong_as_double((long long)b.slots[par * P + p]);
    const double dx = b.dx[p];
    const StepScalars sc = step_scalars(cfl, dx, lmax, lxf);
    const double dt = sc.dt, lam_lxf = sc.lam_lxf, dtdx = sc.dtdx;
    if (d.lead && threadIdx.x == 0) {
      b.t[(1 - par) * P + p] = active ? tn + dt : tn;
      b.slots[(1 - par) * P + p] = 0ull;
      if (active) b.steps[p] += 1;
    }
    const int64_t i = d.first + threadIdx.x;
    const bool own = (int)threadIdx.x < tile_cells && i < d.hi;
    if (!active) {  // a finished problem's cells go to the other buffer unchanged (uniform per tile)
      if (own)
        for (int v = 0; v < 14; ++v) Qn[v * n + i] = Q[v * n + i];
      continue;
    }
    if (own) {
      rusanov_face<kBlock + 1>(Q, F, lam, n, d.lo, d.hi, i, lxf, lam_lxf, sF, threadIdx.x);
      if ((int)threadIdx.x == tile_cells - 1 || i == d.hi - 1)
        rusanov_face<kBlock + 1>(Q, F, lam, n, d.lo, d.hi, i + 1, lxf, lam_lxf, sF, threadIdx.x + 1);
    }
    __syncthreads();
    if (own) {
      const bool frozen = bc == HYP_BC_FROZEN && (i == d.lo || i == d.hi - 1);
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        const double qc = Q[v * n + i];
        Qn[v * n + i] = frozen ? qc : __fma_rn(-dtdx, __dsub_rn(sF[v][threadIdx.x + 1], sF[v][threadIdx.x]), qc);
      }
    }
    __syncthreads();  // the next tile rewrites the face table
  }
}

// ---- mixed kernel variants (autotuned) -------------------------------------------
// A variant: block size, resident blocks per SM the registers are budgeted for,
// and whether the grid is persistent (one wave of blocks striding over the tile
// table) or one block per tile.
struct Variant {
  int block, minb, persist;
};
constexpr Variant kVariants[] = {{256, 4, 1}, {256, 3, 1}, {256, 4, 0}};
constexpr int kNumVariants = HYP_BATCH_NUM_VARIANTS;
static_assert(sizeof(kVariants) / sizeof(kVariants[0]) == kNumVariants, "variant table");

template <int BLOCK, int MINB>
cudaError_t launch_batch_mixed_t(cudaStream_t s, int grid, bool persist, const MixedArrays& a, const EosMixed& em,
                                 const TileDesc* tiles, const TileCtl* ctl, int ntiles, unsigned long long* slots_wr,
                                 int flux, int bc, DevState* S) {
  if (persist)
    batch_mixed_kernel<BLOCK, MINB><<<grid, BLOCK, 0, s>>>(a, em, tiles, ctl, ntiles, slots_wr, flux, bc, S);
  else
    batch_tile_kernel<BLOCK, MINB><<<ntiles, BLOCK, 0, s>>>(a, em, tiles, ctl, slots_wr, flux, bc, S);
  return cudaGetLastError();
}

template <int BLOCK, int MINB>
int resident_blocks() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<BLOCK, MINB>, BLOCK, 0);
  return nb;
}

}  // namespace hyp

using namespace hyp;

struct hyp_batch {
  hyp_config cfg;
  int P = 0;
  int64_t total = 0;
  bool mixed = false;
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  EosC eos;
  EosMixed eos_mixed;
  // mixed state: per parity one tile-major block of the tile table's spans; a parity's
  // block also stages FP64 uploads and downloads
  float* mixed_base = nullptr;
  float* Qh[2] = {nullptr, nullptr};
  // FP64 state
  double* Q[2] = {nullptr, nullptr};
  double* F = nullptr;
  double* lam = nullptr;
  // per-problem control
  BatchDev b{};
  DevState* st = nullptr;
  // tile table of the current variant
  TileDesc* tiles = nullptr;
  TileCtl* ctl = nullptr;  // mixed: per-tile step control
  int ntiles = 0;
  int tile_cells = 0;
  int variant = 2;
  int grid = 0;
  std::vector<int64_t> offsets;
  long long k = 0;  // steps taken by every problem since the upload (the batch steps in lockstep)
  int cur = 0;
  cudaGraphExec_t graph = nullptr;
  long long graph_key[4] = {-1, -1, -1, -1};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  float last_ms = 0.f;
  std::string err;
};

static int berr(hyp_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}
#define BCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t _e = (call);                                                                            \
    if (_e != cudaSuccess) return berr(b, HYP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

static int build_tiles(hyp_batch* b, int cells_per_tile) {
  std::vector<TileDesc> t;
  for (int p = 0; p < b->P; ++p) {
    const int64_t lo = b->offsets[p], hi = b->offsets[p + 1];
    for (int64_t f = lo; f < hi; f += cells_per_tile)
      t.push_back(TileDesc{f, lo, hi, p, f == lo ? 1 : 0});
  }
  if (b->tiles) cudaFree(b->tiles);
  if (b->ctl) cudaFree(b->ctl);
  b->tiles = nullptr;
  b->ctl = nullptr;
  BCK(cudaMalloc(&b->tiles, t.size() * sizeof(TileDesc)));
  if (b->mixed) BCK(cudaMalloc(&b->ctl, t.size() * sizeof(TileCtl)));
  BCK(cudaMemcpy(b->tiles, t.data(), t.size() * sizeof(TileDesc), cudaMemcpyHostToDevice));
  b->ntiles = (int)t.size();
  b->tile_cells = cells_per_tile;
  return HYP_OK;
}

static int select_variant(hyp_batch* b, int v) {
  if (!b->mixed) {
    b->variant = 0;
    int rc = build_tiles(b, kBlock);
    b->grid = b->sms * 8;
    return rc;
  }
  if (v < 0 || v >= kNumVariants) return berr(b, HYP_ERR_INVALID, "no such kernel variant");
  const int res = kVariants[v].minb == 4 ? resident_blocks<256, 4>() : resident_blocks<256, 3>();
  b->variant = v;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  const int rc = b->tiles ? HYP_OK : build_tiles(b, kTileCells);  // the block's spans follow this table
  b->grid = kVariants[v].persist ? b->sms * (res > 0 ? res : 1) : b->ntiles;
  return rc;
}

static MixedArrays batch_arrays(hyp_batch* b, int p) {
  MixedArrays a;
  a.in = b->Qh[p];
  a.out = b->Qh[1 - p];
  a.rstride = kTileRow;
  a.n = b->total;
  a.own_lo = 0;
  a.own_hi = b->total;
  return a;
}

static int enqueue_batch_step(hyp_batch* b, long long k, double t_end) {
  const int par = (int)(k & 1);
  if (b->mixed) {
    const MixedArrays a = batch_arrays(b, par);
    const int rd = (int)(k % 3), wr = (int)((k + 1) % 3), clr = (int)((k + 2) % 3);
    batch_mixed_ctl_kernel<<<(b->ntiles + 255) / 256, 256, 0, b->stream>>>(b->tiles, b->ntiles, b->b, par, rd, wr, clr,
                                                                          t_end, b->cfg.cfl, b->ctl);
    BCK(cudaGetLastError());
    unsigned long long* sw = b->b.slots + (size_t)wr * b->P;
    const int fl = b->cfg.flux, bc = b->cfg.bc;
    cudaError_t e;
    const bool persist = kVariants[b->variant].persist != 0;
    if (kVariants[b->variant].minb == 4)
      e = launch_batch_mixed_t<256, 4>(b->stream, b->grid, persist, a, b->eos_mixed, b->tiles, b->ctl, b->ntiles, sw,
                                       fl, bc, b->st);
    else
      e = launch_batch_mixed_t<256, 3>(b->stream, b->grid, persist, a, b->eos_mixed, b->tiles, b->ctl, b->ntiles, sw,
                                       fl, bc, b->st);
    BCK(e);
  } else {
    batch_f64_cell_kernel<<<b->grid, kBlock, 0, b->stream>>>(b->Q[par], b->total, b->eos, b->F, b->lam, b->tiles,
                                                             b->ntiles, b->tile_cells, b->b, par, t_end,
                                                             b->b.slots + (size_t)par * b->P, b->st);
    BCK(cudaGetLastError());
    batch_f64_update_kernel<<<b->grid, kBlock, 0, b->stream>>>(b->Q[par], b->Q[1 - par], b->total, b->F, b->lam,
                                                               b->tiles, b->ntiles, b->tile_cells, b->b, par, t_end,
                                                               b->cfg.cfl, b->cfg.flux, b->cfg.bc);
    BCK(cudaGetLastError());
  }
  return HYP_OK;
}

static void free_batch(hyp_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (int p = 0; p < 2; ++p) cudaFree(b->Q[p]);
  cudaFree(b->mixed_base);
  cudaFree(b->F);
  cudaFree(b->lam);
  cudaFree(b->b.t);
  cudaFree(b->b.slots);
  cudaFree(b->b.steps);
  cudaFree(b->b.dx);
  cudaFree(b->st);
  cudaFree(b->tiles);
  cudaFree(b->ctl);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" int hyp_batch_create(const hyp_config* cfg, const int64_t* offsets, int n_problems, hyp_batch** out) {
  if (!cfg || !offsets || !out || n_problems < 1) return HYP_ERR_INVALID;
  *out = nullptr;
  if (cfg->model != HYP_MODEL_SINGLE || (cfg->flux != HYP_FLUX_RUSANOV && cfg->flux != HYP_FLUX_LXF))
    return HYP_ERR_UNSUPPORTED;
  if (cfg->precision != HYP_PREC_FP64 && cfg->precision != HYP_PREC_MIXED) return HYP_ERR_INVALID;
  if (cfg->bc != HYP_BC_FROZEN && cfg->bc != HYP_BC_TRANSMISSIVE) return HYP_ERR_INVALID;
  if (!(cfg->cfl > 0) || !(cfg->x_length > 0) || offsets[0] != 0) return HYP_ERR_INVALID;
  for (int p = 0; p < n_problems; ++p)
    if (offsets[p + 1] - offsets[p] < 3) return HYP_ERR_INVALID;
  if (cfg->n_cells != offsets[n_problems]) return HYP_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  hyp_batch* b = new (std::nothrow) hyp_batch();
  if (!b) return HYP_ERR_INVALID;
  b->cfg = *cfg;
  b->P = n_problems;
  b->total = offsets[n_problems];
  b->mixed = cfg->precision == HYP_PREC_MIXED;
  b->offsets.assign(offsets, offsets + n_problems + 1);
  b->eos = make_eos(cfg->eos[0].rho0, cfg->eos[0].c0, cfg->eos[0].cv, cfg->eos[0].t0, cfg->eos[0].b0,
                    cfg->eos[0].alpha, cfg->eos[0].beta, cfg->eos[0].gamma);
  b->eos_mixed = make_eos_mixed(b->eos);
  b->b.P = n_problems;
  int rc = HYP_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == HYP_OK) rc = HYP_ERR_CUDA;
  };
  ck(cudaGetDevice(&b->device));
  ck(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
  ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  const size_t nq = (size_t)14 * b->total;
  if (b->mixed) {
    // one span per tile of kTileCells cells of each problem (the tile table's order);
    // 32,768 bytes per 254 cells also hold the 14 FP64 values per cell of a staged upload
    int64_t nt = 0;
    for (int p = 0; p < n_problems; ++p) nt += mixed_tiles(offsets[p + 1] - offsets[p]);
    const size_t block = (size_t)nt * kTileFloats;
    ck(cudaMalloc(&b->mixed_base, 2 * block * sizeof(float)));
    for (int p = 0; p < 2 && rc == HYP_OK; ++p) b->Qh[p] = b->mixed_base + (size_t)p * block;
  } else {
    for (int p = 0; p < 2 && rc == HYP_OK; ++p) ck(cudaMalloc(&b->Q[p], nq * sizeof(double)));
  }
  if (!b->mixed) {
    ck(cudaMalloc(&b->F, (size_t)kNFlux1 * b->total * sizeof(double)));
    ck(cudaMalloc(&b->lam, (size_t)b->total * sizeof(double)));
  }
  ck(cudaMalloc(&b->b.t, (size_t)2 * n_problems * sizeof(double)));
  ck(cudaMalloc(&b->b.slots, (size_t)3 * n_problems * sizeof(unsigned long long)));
  ck(cudaMalloc(&b->b.steps, (size_t)n_problems * sizeof(long long)));
  ck(cudaMalloc(&b->b.dx, (size_t)n_problems * sizeof(double)));
  ck(cudaMalloc(&b->st, sizeof(DevState)));
  for (auto& e : b->ev) ck(cudaEventCreate(&e));
  if (rc == HYP_OK) {
    std::vector<double> dx(n_problems);
    for (int p = 0; p < n_problems; ++p) dx[p] = cfg->x_length / (double)(offsets[p + 1] - offsets[p]);
    ck(cudaMemcpy(b->b.dx, dx.data(), dx.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (rc == HYP_OK) rc = select_variant(b, b->mixed ? 2 : 0);
  }
  if (rc != HYP_OK) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return HYP_OK;
}

extern "C" int hyp_batch_destroy(hyp_batch* b) {
  free_batch(b);
  return HYP_OK;
}

extern "C" const char* hyp_batch_last_error(const hyp_batch* b) { return b ? b->err.c_str() : "no batch"; }

static int batch_check_error(hyp_batch* b) {
  DevState h;
  BCK(cudaMemcpyAsync(&h, b->st, sizeof h, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (!h.err_code) return HYP_OK;
  char buf[128];
  snprintf(buf, sizeof buf, "cell %lld (global index)", (long long)h.err_cell);
  const int code = (h.err_code & HYP_CELL_TIMEOUT)   ? HYP_ERR_TIMEOUT
                   : (h.err_code & HYP_CELL_NEG_DET) ? HYP_ERR_NEG_DET
                                                     : HYP_ERR_NONFINITE;
  return berr(b, code, buf);
}

extern "C" int hyp_batch_upload(hyp_batch* b, const double* Q, double t0) {
  if (!b || !Q) return HYP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  const size_t bytes = (size_t)14 * b->total * sizeof(double);
  std::vector<double> t(2 * (size_t)b->P, t0);
  BCK(cudaMemcpyAsync(b->b.t, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemsetAsync(b->b.slots, 0, (size_t)3 * b->P * sizeof(unsigned long long), b->stream));
  BCK(cudaMemsetAsync(b->b.steps, 0, (size_t)b->P * sizeof(long long), b->stream));
  BCK(cudaMemsetAsync(b->st, 0, sizeof(DevState), b->stream));
  if (b->mixed) {
    double* stage = (double*)b->Qh[1];
    BCK(cudaMemcpyAsync(stage, Q, bytes, cudaMemcpyHostToDevice, b->stream));
    batch_install_kernel<<<b->sms * 8, kBlock, 0, b->stream>>>(stage, b->total, b->Qh[0], b->eos_mixed, b->tiles,
                                                                b->ntiles, b->b, b->st);
    BCK(cudaGetLastError());
  } else {
    BCK(cudaMemcpyAsync(b->Q[0], Q, bytes, cudaMemcpyHostToDevice, b->stream));
  }
  b->k = 0;
  b->cur = 0;
  return batch_check_error(b);
}

extern "C" int hyp_batch_download(hyp_batch* b, double* Q) {
  if (!b || !Q) return HYP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  const size_t bytes = (size_t)14 * b->total * sizeof(double);
  if (b->mixed) {
    double* stage = (double*)b->Qh[1 - b->cur];
    batch_join_kernel<<<b->sms * 8, kBlock, 0, b->stream>>>(b->Qh[b->cur], b->total, stage, b->tiles, b->ntiles);
    BCK(cudaGetLastError());
    BCK(cudaMemcpyAsync(Q, stage, bytes, cudaMemcpyDeviceToHost, b->stream));
  } else {
    BCK(cudaMemcpyAsync(Q, b->Q[b->cur], bytes, cudaMemcpyDeviceToHost, b->stream));
  }
  BCK(cudaStreamSynchronize(b->stream));
  return HYP_OK;
}

// Advance every problem n_steps steps (a problem whose time reaches t_end stops
// there). The n_steps launches are captured once as a CUDA graph and replayed.
extern "C" int hyp_batch_step(hyp_batch* b, int n_steps, double t_end) {
  if (!b || n_steps < 0 || std::isnan(t_end)) return HYP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  if (n_steps == 0) return HYP_OK;
  const long long key0 = n_steps, key1 = b->k % 6, key2 = b->variant;
  long long key3;
  std::memcpy(&key3, &t_end, sizeof key3);
  if (!b->graph || b->graph_key[0] != key0 || b->graph_key[1] != key1 || b->graph_key[2] != key2 ||
      b->graph_key[3] != key3) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = HYP_OK;
    for (int s = 0; s < n_steps && rc == HYP_OK; ++s) rc = enqueue_batch_step(b, b->k + s, t_end);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != HYP_OK) return rc;
    BCK(e);
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    BCK(e);
    b->graph_key[0] = key0;
    b->graph_key[1] = key1;
    b->graph_key[2] = key2;
    b->graph_key[3] = key3;
  }
  BCK(cudaEventRecord(b->ev[0], b->stream));
  BCK(cudaGraphLaunch(b->graph, b->stream));
  BCK(cudaEventRecord(b->ev[1], b->stream));
  BCK(cudaEventSynchronize(b->ev[1]));
  BCK(cudaEventElapsedTime(&b->last_ms, b->ev[0], b->ev[1]));
  b->k += n_steps;
  b->cur = (int)(b->k & 1);
  return batch_check_error(b);
}

// Per-problem time and step count.
extern "C" int hyp_batch_status(hyp_batch* b, double* t, int64_t* steps) {
  if (!b) return HYP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  std::vector<double> tt(2 * (size_t)b->P);
  std::vector<long long> ss(b->P);
  BCK(cudaMemcpyAsync(tt.data(), b->b.t, tt.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaMemcpyAsync(ss.data(), b->b.steps, ss.size() * sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  for (int p = 0; p < b->P; ++p) {  // every problem changes parity each launched step
    if (t) t[p] = tt[(size_t)(b->k & 1) * b->P + p];
    if (steps) steps[p] = ss[p];
  }
  return HYP_OK;
}

extern "C" int hyp_batch_last_ms(const hyp_batch* b, double* ms) {
  if (!b || !ms) return HYP_ERR_INVALID;
  *ms = b->last_ms;
  return HYP_OK;
}

// Time every mixed kernel variant for trial_steps steps on the batch's current
// state (the state is advanced and restored from a device copy) and keep the
// fastest. ms_per_step (optional, kNumVariants entries) receives the timings.
extern "C" int hyp_batch_autotune(hyp_batch* b, int trial_steps, int* chosen, double* ms_per_step) {
  if (!b || trial_steps < 1) return HYP_ERR_INVALID;
  if (!b->mixed) {
    if (chosen) *chosen = 0;
    return HYP_OK;
  }
  BCK(cudaSetDevice(b->device));
  // save the state of the current parity (hi/lo, lambda, islands) and the per-problem
  // control in one device buffer; every trial starts from it
  const int p0 = b->cur;
  const long long k0 = b->k;
  // the parity block holds hi, lo, lambda and islands
  const size_t bq = (size_t)b->ntiles * kTileFloats * sizeof(float), bt = (size_t)2 * b->P * sizeof(double),
               bs = (size_t)3 * b->P * sizeof(unsigned long long), bk = (size_t)b->P * sizeof(long long);
  char* save = nullptr;
  BCK(cudaMalloc(&save, bq + bt + bs + bk));
  struct Seg {
    void* dev;
    size_t off, bytes;
  } segs[] = {{b->Qh[p0], 0, bq},
              {b->b.t, bq, bt},
              {b->b.slots, bq + bt, bs},
              {b->b.steps, bq + bt + bs, bk}};
  // The copies go on the batch's own (non-blocking) stream: a device-to-device
  // cudaMemcpy would run on the legacy stream, which that stream does not wait for.
  for (auto& s : segs)
    if (cudaMemcpyAsync(save + s.off, s.dev, s.bytes, cudaMemcpyDeviceToDevice, b->stream) != cudaSuccess) {
      cudaFree(save);
      return berr(b, HYP_ERR_CUDA, "autotune: saving the state failed");
    }
  auto restore = [&]() -> int {
    for (auto& s : segs)
      if (cudaMemcpyAsync(s.dev, save + s.off, s.bytes, cudaMemcpyDeviceToDevice, b->stream) != cudaSuccess)
        return berr(b, HYP_ERR_CUDA, "autotune: restoring the state failed");
    BCK(cudaStreamSynchronize(b->stream));
    b->k = k0;
    b->cur = p0;
    return HYP_OK;
  };
  struct Freer {
    char* p;
    ~Freer() { cudaFree(p); }
  } freer{save};
  int best = b->variant;
  double best_ms = 1e300;
  for (int v = 0; v < kNumVariants; ++v) {
    int rc = select_variant(b, v);
    if (rc != HYP_OK) return rc;
    if ((rc = hyp_batch_step(b, trial_steps, INFINITY)) != HYP_OK) return rc;  // includes graph capture
    if ((rc = restore()) != HYP_OK) return rc;
    if ((rc = hyp_batch_step(b, trial_steps, INFINITY)) != HYP_OK) return rc;  // timed replay
    const double ms = b->last_ms / trial_steps;
    if (ms_per_step) ms_per_step[v] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
    if ((rc = restore()) != HYP_OK) return rc;
  }
  int rc = select_variant(b, best);
  if (chosen) *chosen = best;
  return rc;
}

extern "C" int hyp_batch_set_variant(hyp_batch* b, int v) {
  if (!b) return HYP_ERR_INVALID;
  return select_variant(b, v);
}
