// hyp_step1_mixed.cu -- single-phase step in mixed precision: FP32 fluxes and
// wave speeds, a compensated (hi, lo) FP32 state, float-float islands in
// cons2prim (hyp_physics_mixed.cuh).
//
// One fused kernel per step; each tile of hyp_mixed_tile.cuh (block - 2 owned
// cells plus a halo cell each side) runs the flux phase, the Rusanov faces, the
// compensated update, then the wave speed of the NEW state, stored per cell and
// max-reduced (warp shuffles, one shared-memory pass, one atomicMax per block)
// for the next step's dt = cfl dx / max lambda (main.jl:204-212).
// HBM traffic per cell-update: the state read and written (14 x 2 x 4 B each
// way) plus, each way, the cell's FP32 lambda and the three outputs of its
// float-float islands (1/rho, e_int, rho/rho0 - 1), so that the flux phase needs
// no float-float work: 256 B, against 224 B for the state alone.
// The three max-lambda slots rotate (read k%3, write (k+1)%3, clear (k+2)%3)
// so one launch per step needs no separate reset.
//
// Three kernels run the same tile arithmetic:
//   step1_mixed_kernel      one block per tile, each thread loading its cell;
//   step1_mixed_pair_kernel one block per two adjacent tiles of 126 cells, thread j
//                           holding local cell j of both in the lanes of packed
//                           FP32 pairs (hyp_mixed_pair.cuh), so one instruction
//                           advances two cells;
//   step1_mixed_tma_kernel  a persistent grid; thread 0 of a block prefetches
//                           the block's next tile (the tile's contiguous span of
//                           the tile-major block) with one TMA bulk copy into
//                           shared memory while the block computes the current
//                           tile from its copy, so loads overlap compute.
// The state blocks are tile-major (hyp_internal.cuh): a tile's 32 rows are one
// contiguous 32,512-byte span, which the block reads and writes whole (the halo
// cells come from the neighbouring spans). Against row-major blocks (each row a
// separate 1 KB piece 64 MB from the next at 2^24 cells) this measured 0.771
// against 0.845 ms per step at 2^24 cells; a copy of the same bytes in the two
// patterns, without the physics: 0.60 against 0.68 ms.
#include "hyp_internal.cuh"
#include "hyp_mixed_pair.cuh"
#include "hyp_mixed_tile.cuh"

namespace hyp {

constexpr int kTileM = kBlock - 2;

struct MixedSlots {
  int p;              // state / time parity
  int rd, wr, clr;    // max-lambda slots: read (this step), write (next step), clear
};

// t, the step count and the max-lambda slots (block 0, thread 0); returns
// whether the step is active and dt/dx. Every thread reads the control itself: a
// lane-0 read broadcast by shuffles measured 0.939 against 0.847 ms per step at
// 2^24 cells (the cell loads issued ahead of it no longer overlap it).
__device__ __forceinline__ bool mixed_step_prologue(const MixedSlots& sl, DevState* S, double t_end, double cfl,
                                                    double dx, float& dtdx) {
  const double tn = S->t[sl.p];
  const bool active = tn < t_end;
  const float lmax = __uint_as_float((unsigned)S->lam_slots[sl.rd]);
  dtdx = (float)cfl / lmax;  // dt/dx = cfl / max lambda
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double dt = (cfl * dx) / (double)lmax;
    S->t[1 - sl.p] = active ? tn + dt : tn;
    if (active) {  // an inactive step must keep the slot that holds the current state's max lambda
      S->lam_slots[sl.clr] = 0ull;
      S->steps += 1;
    }
  }
  return active;
}

__global__ void __launch_bounds__(kBlock, 4)
    step1_mixed_kernel(MixedArrays a, EosMixed em, MixedSlots sl, DevState* S, double t_end, double cfl, double dx,
                       int flux, int bc) {
  const int64_t first = (int64_t)blockIdx.x * kTileM;
  const MixedGlobalLoader<kBlock, true> ld{a, {(int64_t)blockIdx.x * kTileFloats, first}};
  MixedCellIn c;
  mixed_tile_load<kBlock>(first, 0, a.n, ld, c);  // issued before the control reads below
  float dtdx;
  if (!mixed_step_prologue(sl, S, t_end, cfl, dx, dtdx)) return;
  float l = mixed_tile_run<kBlock, true, true>(a, em, first, 0, a.n, dtdx, flux, bc, S, ld, c);
  const int64_t i = first - 1 + tile_local<kBlock>();
  if (i < a.own_lo || i >= a.own_hi) l = 0.0f;  // a slab's ghost cells: their owner reports them
  const float m = mixed_block_max<kBlock>(l);
  if (threadIdx.x == 0) atomicMax(&S->lam_slots[sl.wr], (unsigned long long)__float_as_uint(m));
}

// ---- two tiles per block in packed FP32 pairs ----------------------------------

constexpr int kPairBlock = 128;

// Tiles 2b (lane x) and 2b + 1 (lane y) of BLOCK - 2 cells each: the phases of
// mixed_tile_run (cell fluxes from the cached islands, faces, compensated update,
// islands and wave speed of the new state) with every value a pair. A lane whose
// cell is held (frozen end, slab ghost) keeps its state, lambda and islands.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 4)
    step1_mixed_pair_kernel(MixedArrays a, EosMixed em, MixedSlots sl, DevState* S, double t_end, double cfl,
                            double dx, int flux, int bc) {
  constexpr int M = BLOCK - 2;
  __shared__ float2 sFF[14][BLOCK];  // cell fluxes (11 slots), then the face fluxes (14)
  __shared__ float2 sQ[14][BLOCK];
  __shared__ float2 sL[BLOCK];
  constexpr int64_t r = kTileRow;
  const int64_t hi = a.n;
  const int j = threadIdx.x;
  const int64_t firstA = (int64_t)blockIdx.x * (2 * M);
  const int64_t iA = firstA - 1 + j, iB = iA + M;  // this thread's cells (halo at j = 0, BLOCK - 1)
  const int64_t cA = iA < 0 ? 0 : (iA >= hi ? hi - 1 : iA), cB = iB >= hi ? hi - 1 : iB;
  const float* qA = a.in + tile_cell_off(cA);
  const float* qB = a.in + tile_cell_off(cB);
  float2 qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = make_float2(qA[v * r], qB[v * r]);
    ql[v] = make_float2(qA[(kRowLo + v) * r], qB[(kRowLo + v) * r]);
  }
  const float2 li = make_float2(qA[kRowLam * r], qB[kRowLam * r]);
  IslandsP I0;
  I0.ir = make_float2(qA[kRowIsl * r], qB[kRowIsl * r]);
  I0.e_int = make_float2(qA[(kRowIsl + 1) * r], qB[(kRowIsl + 1) * r]);
  I0.sm1 = make_float2(qA[(kRowIsl + 2) * r], qB[(kRowIsl + 2) * r]);
  float dtdx;
  if (!mixed_step_prologue(sl, S, t_end, cfl, dx, dtdx)) return;
  const bool inner = j > 0 && j < BLOCK - 1;
  float2 f11[kNFlux1];
  {
    PrimP P;
    const int st = prim_from_islands_pair(em, qh, ql, I0, P);
    const CoefP sc = stress_coeffs_pair(em.f, P);
    flux_pair(qh, P, sc, f11);
#pragma unroll
    for (int s = 0; s < kNFlux1; ++s) sFF[s][j] = f11[s];
#pragma unroll
    for (int v = 0; v < 14; ++v) sQ[v][j] = qh[v];
    sL[j] = li;
    if (inner && (st & 0xff) && iA == cA) mixed_record_err(S, st & 0xff, iA);
    if (inner && (st >> 8) && iB == cB) mixed_record_err(S, st >> 8, iB);
  }
  __syncthreads();
  // face j + 1/2 between local cells j (registers) and j + 1 (shared memory)
  float2 fv[14];
  if (j < BLOCK - 1) {
    const float2 lr = sL[j + 1];
    const float2 lf = flux == HYP_FLUX_LXF ? f2s(1.0f / dtdx) : f2max(li, lr);
    const float2 nhl = f2mul(f2s(-0.5f), lf);
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const int s = flux_slot1(v);
      const float2 sum = s >= 0 ? f2add(f11[s], sFF[s][j + 1]) : f2s(0.0f);
      fv[v] = f2fma(nhl, f2sub(sQ[v][j + 1], qh[v]), f2mul(f2s(0.5f), sum));
    }
  }
  __syncthreads();
  if (j < BLOCK - 1) {
#pragma unroll
    for (int v = 0; v < 14; ++v) sFF[v][j] = fv[v];
  }
  __syncthreads();
  float lA = 0.0f, lB = 0.0f;
  const bool ownA = inner && iA < hi, ownB = inner && iB < hi;
  if (ownA || ownB) {
    const bool holdA = bc_holds(bc, iA == 0, iA == hi - 1), holdB = !ownB || bc_holds(bc, false, iB == hi - 1);
    const float2 ndt = f2s(-dtdx);
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const float2 delta = f2mul(ndt, f2sub(fv[v], sFF[v][j - 1]));  // F_{j+1/2} - F_{j-1/2}
      const ff2 q = ff2_add_f(ff2{qh[v], ql[v]}, delta);
      if (!holdA) {
        qh[v].x = q.hi.x;
        ql[v].x = q.lo.x;
      }
      if (!holdB) {
        qh[v].y = q.hi.y;
        ql[v].y = q.lo.y;
      }
    }
    IslandsP I;
    int st = islands_pair(em, qh, ql, I);
    PrimP P;
    st |= prim_from_islands_pair(em, qh, ql, I, P);
    const CoefP sc = stress_coeffs_pair(em.f, P);
    const float2 lnew = lambda_pair(em, P, sc);
    st |= lane_status(!(lnew.x <= 3.0e38f), !(lnew.y <= 3.0e38f), HYP_CELL_NONFINITE);
    if (holdA) {
      lA = li.x;
      I.ir.x = I0.ir.x;
      I.e_int.x = I0.e_int.x;
      I.sm1.x = I0.sm1.x;
    } else {
      lA = lnew.x;
      if (ownA && (st & 0xff)) mixed_record_err(S, st & 0xff, iA);
    }
    if (holdB) {
      lB = li.y;
      I.ir.y = I0.ir.y;
      I.e_int.y = I0.e_int.y;
      I.sm1.y = I0.sm1.y;
    } else {
      lB = lnew.y;
      if (st >> 8) mixed_record_err(S, st >> 8, iB);
    }
    if (ownA) {
      float* q = a.out + tile_cell_off(iA);
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        q[v * r] = qh[v].x;
        q[(kRowLo + v) * r] = ql[v].x;
      }
      q[kRowLam * r] = lA;
      q[kRowIsl * r] = I.ir.x;
      q[(kRowIsl + 1) * r] = I.e_int.x;
      q[(kRowIsl + 2) * r] = I.sm1.x;
    }
    if (ownB) {
      float* q = a.out + tile_cell_off(iB);
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        q[v * r] = qh[v].y;
        q[(kRowLo + v) * r] = ql[v].y;
      }
      q[kRowLam * r] = lB;
      q[kRowIsl * r] = I.ir.y;
      q[(kRowIsl + 1) * r] = I.e_int.y;
      q[(kRowIsl + 2) * r] = I.sm1.y;
    }
  }
  // a slab's ghost cells: their owner reports them
  if (!ownA || iA < a.own_lo || iA >= a.own_hi) lA = 0.0f;
  if (!ownB || iB < a.own_lo || iB >= a.own_hi) lB = 0.0f;
  const float m = mixed_block_max<BLOCK>(fmaxf(lA, lB));
  if (threadIdx.x == 0) atomicMax(&S->lam_slots[sl.wr], (unsigned long long)__float_as_uint(m));
}

// ---- TMA-prefetched persistent kernel ----------------------------------------

// A tile's span of the tile-major block (32 rows x kTileRow floats) staged in
// shared memory by one bulk copy.
constexpr unsigned kTmaTileBytes = kTileFloats * 4u;  // 32 KB, a multiple of 16
constexpr unsigned kTmaSmem = kTmaTileBytes + 128u;   // dynamic shared memory (alignment slack)

// Loads a cell's inputs from the staged tile (its owned cells; o its origin) or,
// for a halo cell in a neighbouring tile, from global memory; the halo
// cells' hi parts are kept in shared memory for the face phase. The next tile is
// copied in (release) once the faces have read the stage.
template <int BLOCK>
struct MixedStageLoader {
  const float* stage;   // [32][kTileRow]
  const MixedArrays& a;
  float2 (*halo)[7];    // [2][7]: the left / right halo cell's hi parts
  TileOrigin o;
  uint64_t* bar;
  const float* next;    // the next tile's span in global memory (null: none)
  __device__ __forceinline__ bool staged(int64_t ic) const { return ic >= o.first && ic < o.first + kTileCells; }
  __device__ __forceinline__ const TileOrigin& origin() const { return o; }
  __device__ __forceinline__ void operator()(int, int64_t ic, MixedCellIn& c) const {
    const float* q = staged(ic) ? stage + (ic - o.first) : a.in + tile_rel_off(o, ic);
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      c.qh[v] = q[v * kTileRow];
      c.ql[v] = q[(kRowLo + v) * kTileRow];
    }
    c.li = q[kRowLam * kTileRow];
    c.I0.ir = q[kRowIsl * kTileRow];
    c.I0.e_int = q[(kRowIsl + 1) * kTileRow];
    c.I0.sm1 = q[(kRowIsl + 2) * kTileRow];
  }
  __device__ __forceinline__ void keep(int j, const MixedCellIn& c) const {
    const int64_t i = o.first - 1 + j;
    if ((j == 0 || j == BLOCK - 1) && !staged(i < 0 ? 0 : (i >= a.n ? a.n - 1 : i)))
#pragma unroll
      for (int k = 0; k < 7; ++k) halo[j == 0 ? 0 : 1][k] = pair_of(c.qh, k);
  }
  __device__ __forceinline__ float2 face_q2(int k, int j, int64_t ic) const {
    if (!staged(ic)) return halo[j == 0 ? 0 : 1][k];
    const float* s = stage + (ic - o.first);
    return make_float2(s[2 * k * kTileRow], s[(2 * k + 1) * kTileRow]);
  }
  // called after a barrier that follows the block's last read of the stage
  __device__ __forceinline__ void release() const {
    if (threadIdx.x == 0 && next) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(bar, kTmaTileBytes);
      bulk_load(const_cast<float*>(stage), next, kTmaTileBytes, bar);
    }
  }
};

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
    step1_mixed_tma_kernel(MixedArrays a, EosMixed em, MixedSlots sl, DevState* S, double t_end, double cfl, double dx,
                           int flux, int bc, int ntiles, int wait_tries) {
  static_assert(BLOCK == kTileCells + 2, "a block steps one tile of the tile-major block");
  extern __shared__ __align__(128) float stage_raw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ float2 halo[2][7];
  float dtdx;
  if (!mixed_step_prologue(sl, S, t_end, cfl, dx, dtdx)) return;
  // bulk-copy destinations are 16-byte aligned (128 here; the launch adds 128 bytes of slack)
  float* stage = stage_raw + ((128u - (smem_addr(stage_raw) & 127u)) & 127u) / 4u;
  int tile = blockIdx.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    if (tile < ntiles) {
      mbar_arrive_expect_tx(&bar, kTmaTileBytes);
      bulk_load(stage, a.in + (int64_t)tile * kTileFloats, kTmaTileBytes, &bar);
    }
  }
  __syncthreads();
  unsigned phase = 0;
  float m = 0.0f;
  for (; tile < ntiles; tile += gridDim.x) {
    const bool ok = mbar_wait_bounded(&bar, phase, wait_tries);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) mixed_record_err(S, HYP_CELL_TIMEOUT, (long long)tile * kTileCells);
      // the awaited copy is the block's only one in flight: let it land (again a
      // bounded wait) before the block's shared memory goes away
      mbar_wait_bounded(&bar, phase, kDrainTries);
      return;
    }
    phase ^= 1u;
    const int64_t first = (int64_t)tile * kTileCells;
    const int next = tile + gridDim.x;
    MixedStageLoader<BLOCK> ld{stage, a, halo, {(int64_t)tile * kTileFloats, first}, &bar,
                               next < ntiles ? a.in + (int64_t)next * kTileFloats : nullptr};
    m = fmaxf(m, mixed_tile<BLOCK, true>(a, em, first, 0, a.n, dtdx, flux, bc, S, ld));
  }
  m = mixed_block_max<BLOCK>(m);
  if (threadIdx.x == 0) atomicMax(&S->lam_slots[sl.wr], (unsigned long long)__float_as_uint(m));
}

constexpr int kTmaBlock = 256, kTmaMinB = 3;

// lambda of every cell of the state (after an upload) and its max into a slot.
__global__ void __launch_bounds__(kBlock) lam1_mixed_kernel(MixedArrays a, EosMixed em, unsigned long long* slot,
                                                            DevState* S) {
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  float l = 0.0f;
  if (i < a.n) l = mixed_cell_lambda<true>(a, em, i, S);
  const float m = mixed_block_max<kBlock>(l);
  if (threadIdx.x == 0) atomicMax(slot, (unsigned long long)__float_as_uint(m));
}

// An uploaded single-phase state installed in one pass: each thread reads its
// cell's 14 FP64 values (from device memory, or straight from page-locked host
// memory that the device maps, so that the host link is the only transfer), splits
// them into (hi, lo) pairs exactly as split_kernel does, and computes the cell's
// wave speed and island outputs from those pairs exactly as lam1_mixed_kernel does
// (max into `slot`). a.out: the parity-0 block.
__global__ void __launch_bounds__(kBlock) install1_mixed_kernel(const double* __restrict__ q, MixedArrays a,
                                                                EosMixed em, unsigned long long* slot, DevState* S) {
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  float l = 0.0f;
  if (i < a.n) {
    float qh[14], ql[14];
    float* o = a.out + tile_cell_off(i);
    constexpr int64_t r = kTileRow;
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const double x = q[v * a.n + i];
      qh[v] = (float)x;
      ql[v] = (float)(x - (double)qh[v]);
      o[v * r] = qh[v];
      o[(kRowLo + v) * r] = ql[v];
    }
    l = mixed_cell_lambda_of(em, qh, ql, i, S, o, r);
  }
  const float m = mixed_block_max<kBlock>(l);
  if (threadIdx.x == 0) atomicMax(slot, (unsigned long long)__float_as_uint(m));
}

// FP64 [14][n] -> (hi, lo) rows of pitch `pitch`, and back.
__global__ void split_kernel(const double* __restrict__ q, float* __restrict__ hi, float* __restrict__ lo, int64_t n,
                             int64_t pitch, int64_t m) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    const double x = q[k];
    const float h = (float)x;
    const int64_t d = (k / n) * pitch + k % n;
    hi[d] = h;
    lo[d] = (float)(x - (double)h);
  }
}
__global__ void join_kernel(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ q,
                            int64_t n, int64_t pitch, int64_t m) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = (k / n) * pitch + k % n;
    q[k] = (double)hi[d] + (double)lo[d];
  }
}

// Tile-major single-phase block -> FP64 rows v0 .. v0 + rows - 1 of [14][n] (q points
// at row v0): hi + lo of each variable.
__global__ void join1_tiled_kernel(const float* __restrict__ base, double* __restrict__ q, int64_t n, int v0,
                                   int64_t m) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    const int v = v0 + (int)(k / n);
    const float* c = base + tile_cell_off(k % n) + (int64_t)v * kTileRow;
    q[k] = (double)c[0] + (double)c[kRowLo * kTileRow];
  }
}

unsigned elementwise_grid(int64_t m) {
  int64_t g = (m + kBlock - 1) / kBlock;
  return (unsigned)(g > 152 * 64 ? 152 * 64 : (g < 1 ? 1 : g));
}

cudaError_t launch_split_n(cudaStream_t s, const double* q, float* hi, float* lo, int rows, int64_t n,
                           int64_t pitch) {
  split_kernel<<<elementwise_grid(rows * n), kBlock, 0, s>>>(q, hi, lo, n, pitch, rows * n);
  return cudaGetLastError();
}
cudaError_t launch_join_n(cudaStream_t s, const float* hi, const float* lo, double* q, int rows, int64_t n,
                          int64_t pitch) {
  join_kernel<<<elementwise_grid(rows * n), kBlock, 0, s>>>(hi, lo, q, n, pitch, rows * n);
  return cudaGetLastError();
}
cudaError_t launch_split(hyp_ctx* c, const double* q, float* hi, float* lo) {
  return launch_split_n(c->stream, q, hi, lo, c->nvar, c->n, c->mpitch);
}
// The FP64 state [nvar][n] of parity p: rows v0 .. v0 + rows - 1 into q (row v0 first).
cudaError_t launch_join_rows(hyp_ctx* c, int p, double* q, int v0, int rows) {
  if (c->cfg.model == HYP_MODEL_SINGLE) {
    const int64_t m = (int64_t)rows * c->n;
    join1_tiled_kernel<<<elementwise_grid(m), kBlock, 0, c->stream>>>(c->Qh[p], q, c->n, v0, m);
    return cudaGetLastError();
  }
  return launch_join_n(c->stream, c->Qh[p] + (size_t)v0 * c->mpitch, c->Ql[p] + (size_t)v0 * c->mpitch, q, rows, c->n,
                       c->mpitch);
}
cudaError_t launch_join(hyp_ctx* c, int p, double* q) { return launch_join_rows(c, p, q, 0, c->nvar); }

static MixedArrays arrays_of(hyp_ctx* c, int p) {
  MixedArrays a;
  a.in = c->Qh[p];
  a.out = c->Qh[1 - p];
  a.rstride = kTileRow;
  a.n = c->n;
  a.own_lo = c->slab && c->slab_ghost[0] ? 1 : 0;
  a.own_hi = c->slab && c->slab_ghost[1] ? c->n - 1 : c->n;
  return a;
}

cudaError_t launch_install1_mixed(hyp_ctx* c, const double* q, unsigned long long* slot) {
  const unsigned grid = (unsigned)((c->n + kBlock - 1) / kBlock);
  MixedArrays a = arrays_of(c, 1);  // outputs: parity 0
  install1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(q, a, c->eos_mixed, slot, c->st);
  return cudaGetLastError();
}

cudaError_t launch_lam1_mixed(hyp_ctx* c, int p, unsigned long long* slot) {
  const unsigned grid = (unsigned)((c->n + kBlock - 1) / kBlock);
  MixedArrays a = arrays_of(c, p);  // the uploaded state's own lambda and islands, into its own block
  lam1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(a, c->eos_mixed, slot, c->st);
  return cudaGetLastError();
}

// Prepares the TMA kernel for a context: its shared memory and persistent grid.
int setup_mixed_tma(hyp_ctx* c) {
  auto kern = step1_mixed_tma_kernel<kTmaBlock, kTmaMinB>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTmaSmem) != cudaSuccess) return 1;
  int nb = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kTmaBlock, kTmaSmem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nb < 1)
    return 1;
  c->tma_grid = (int)std::min<int64_t>(mixed_tiles(c->n), (int64_t)sms * nb);
  return 0;
}

cudaError_t launch_step1_mixed(hyp_ctx* c, long long k, double t_end) {
  const int p = (int)(k & 1);
  MixedSlots sl;
  sl.p = p;
  sl.rd = (int)(k % 3);
  sl.wr = (int)((k + 1) % 3);
  sl.clr = (int)((k + 2) % 3);
  const double dx = ctx_dx(c);
  if (c->mixed_kind == HYP_MIXED_TMA && !c->slab) {
    step1_mixed_tma_kernel<kTmaBlock, kTmaMinB><<<c->tma_grid, kTmaBlock, kTmaSmem, c->stream>>>(
        arrays_of(c, p), c->eos_mixed, sl, c->st, t_end, c->cfg.cfl, dx, c->cfg.flux, c->cfg.bc,
        (int)mixed_tiles(c->n), c->wait_tries);
  } else if (c->mixed_kind == HYP_MIXED_PAIR) {
    const int64_t ntiles = (c->n + (kPairBlock - 2) - 1) / (kPairBlock - 2);
    step1_mixed_pair_kernel<kPairBlock><<<(unsigned)((ntiles + 1) / 2), kPairBlock, 0, c->stream>>>(
        arrays_of(c, p), c->eos_mixed, sl, c->st, t_end, c->cfg.cfl, dx, c->cfg.flux, ctx_bc(c));
  } else {
    const unsigned grid = (unsigned)((c->n + kTileM - 1) / kTileM);
    step1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(arrays_of(c, p), c->eos_mixed, sl, c->st, t_end, c->cfg.cfl,
                                                       dx, c->cfg.flux, ctx_bc(c));
  }
  return cudaGetLastError();
}

}  // namespace hyp
