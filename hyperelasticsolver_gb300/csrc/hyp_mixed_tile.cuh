// hyp_mixed_tile.cuh -- one tile of the mixed-precision single-phase step,
// shared by the single-problem kernel (hyp_step1_mixed.cu) and the batched
// kernel (hyp_batch.cu).
//
// A block of BLOCK threads owns BLOCK - 2 consecutive cells of one problem and
// loads them plus one halo cell on each side (clamped to the problem's cells
// [lo, hi): a ghost cell copies the end cell, i.e. a zero-gradient boundary);
// threads 0 .. BLOCK - 3 take the owned cells and the last two the halos
// (tile_local), and the state blocks are row-major or tile-major (MixedArrays):
//   1. flux of every loaded cell from its (hi, lo) state and the float-float
//      island outputs cached by the step that produced it -> shared memory;
//   2. Rusanov face fluxes 0.5 (f_L + f_R) - 0.5 lambda_face (Q_R - Q_L)
//      (NumFluxes.jl:25-33; main.jl:45-48), lambda_face = max(lambda_L, lambda_R);
//   3. Q += -dt/dx (F_{i+1/2} - F_{i-1/2}) accumulated into (hi, lo) (main.jl:43-60);
//   4. islands, cons2prim and wave speed of the NEW state, stored per cell.
// Returns the thread's new wave speed; the caller reduces the block max.
// Phases 2 and 3 treat the 14 variables as 7 pairs (2k, 2k+1) in packed FP32
// instructions (hyp_pair.cuh) and keep them in shared memory as float2: the same
// operations in the same order, half the instructions and shared-memory accesses.
#pragma once
#include "hyp_internal.cuh"
#include "hyp_pair.cuh"

namespace hyp {

// A step's input and output state blocks (32 rows per cell: kRowLo, kRowLam,
// kRowIsl), row-major (row r of cell i at r * rstride + i) or tile-major (at
// tile_cell_off(i) + r * kTileRow).
struct MixedArrays {
  const float* in;
  float* out;
  int64_t rstride;  // row-major blocks: the pitch
  int64_t n;        // cells
  int64_t own_lo, own_hi;  // cells whose new wave speed enters the step's max (a slab's ghosts do not)
};
// A tile of a tile-major block: where its span starts and its first cell. Its halo
// cells are the last cell of the span before and the first of the span after (a
// problem's tiles are consecutive spans).
struct TileOrigin {
  int64_t base;   // offset of the tile's span in the block (a multiple of kTileFloats)
  int64_t first;  // the tile's first cell
};
// Offset of cell ic (first - 1 <= ic <= first + kTileCells) relative to a tile.
__device__ __forceinline__ int64_t tile_rel_off(const TileOrigin& o, int64_t ic) {
  const int64_t rel = ic - o.first;
  return o.base + (rel < 0 ? (int64_t)(kTileCells - 1) - kTileFloats : (rel >= kTileCells ? (int64_t)kTileFloats : rel));
}
// kTiled: tile-major blocks, whose row stride is known at compile time, so that a
// cell's 32 rows are immediate offsets from one address; else row-major.
template <bool kTiled>
__device__ __forceinline__ int64_t rows_apart(const MixedArrays& a) {
  return kTiled ? (int64_t)kTileRow : a.rstride;
}
template <bool kTiled>
__device__ __forceinline__ int64_t cell_at(int64_t i) {
  return kTiled ? tile_cell_off(i) : i;
}

// One cell's inputs to a tile.
struct MixedCellIn {
  float qh[14], ql[14];
  float li;
  Islands I0;
};

__device__ __forceinline__ float2 pair_of(const float* v, int k) { return make_float2(v[2 * k], v[2 * k + 1]); }

// Loads the cell's inputs straight from the state arrays and keeps the hi parts
// the face phase reads in shared memory.
// Loader interface used by mixed_tile: operator()(j, ic, c) fills cell ic's
// inputs for local index j; keep(j, c) stores what face_q2 needs; face_q2(k, j, ic)
// returns the hi parts of variables 2k, 2k+1 of local cell j (cell ic); release()
// runs once the face phase has read its inputs.
template <int BLOCK, bool kTiled = false>
struct MixedGlobalLoader {
  const MixedArrays& a;
  TileOrigin o;  // tile-major: the tile being stepped
  __device__ __forceinline__ static float2 (&sQ())[7][BLOCK] {
    __shared__ float2 q[7][BLOCK];
    return q;
  }
  __device__ __forceinline__ void operator()(int, int64_t ic, MixedCellIn& c) const {
    const int64_t r = rows_apart<kTiled>(a);
    const float* q = a.in + (kTiled ? tile_rel_off(o, ic) : ic);
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      c.qh[v] = q[v * r];
      c.ql[v] = q[(kRowLo + v) * r];
    }
    c.li = q[kRowLam * r];
    c.I0.ir = q[kRowIsl * r];
    c.I0.e_int = q[(kRowIsl + 1) * r];
    c.I0.sm1 = q[(kRowIsl + 2) * r];
  }
  __device__ __forceinline__ void keep(int j, const MixedCellIn& c) const {
#pragma unroll
    for (int k = 0; k < 7; ++k) sQ()[k][j] = pair_of(c.qh, k);
  }
  __device__ __forceinline__ float2 face_q2(int k, int j, int64_t) const { return sQ()[k][j]; }
  __device__ __forceinline__ void release() const {}
  __device__ __forceinline__ const TileOrigin& origin() const { return o; }
};

// A cell's 11 flux components (flux_slot1 order) as 7 pairs of variables, zero
// where a variable of rho A has no x-flux (row 1 of rho A: variables 5, 8, 11).
__device__ __forceinline__ void flux_pairs(const float* f11, float2* f2) {
  f2[0] = make_float2(f11[0], f11[1]);
  f2[1] = make_float2(f11[2], f11[3]);
  f2[2] = make_float2(f11[4], 0.0f);
  f2[3] = make_float2(f11[5], f11[6]);
  f2[4] = make_float2(0.0f, f11[7]);
  f2[5] = make_float2(f11[8], 0.0f);
  f2[6] = make_float2(f11[9], f11[10]);
}

// A cell's 32 rows into a state block (q: the cell's row 0, rows rstride apart).
__device__ __forceinline__ void mixed_store_cell(float* q, int64_t rstride, const float* qh, const float* ql,
                                                 float lam, const Islands& I) {
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    q[v * rstride] = qh[v];
    q[(kRowLo + v) * rstride] = ql[v];
  }
  q[kRowLam * rstride] = lam;
  q[kRowIsl * rstride] = I.ir;
  q[(kRowIsl + 1) * rstride] = I.e_int;
  q[(kRowIsl + 2) * rstride] = I.sm1;
}

__device__ __forceinline__ void mixed_record_err(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

template <int BLOCK>
__device__ __forceinline__ float mixed_block_max(float v) {
  __shared__ float red[BLOCK / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < BLOCK / 32 ? red[l] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

// first: first owned cell (global index); [lo, hi): the problem's cells.
// mixed_tile_load fills this thread's cell inputs; kernels call it before they
// read the step's control data (time, max lambda), so that the cell loads do not
// wait behind those. mixed_tile_run then takes the step and returns this
// thread's new wave speed (0 if it owns no cell).
// Position in the tile (0 = left halo, 1 .. BLOCK-2 the owned cells, BLOCK-1 the
// right halo) of this thread's cell: threads 0 .. BLOCK-3 take the owned cells, so
// that warp w's 32 cells are the 128-byte line at 32 w of each tile-major row;
// thread BLOCK-2 the right halo, thread BLOCK-1 the left.
template <int BLOCK>
__device__ __forceinline__ int tile_local() {
  const int t = threadIdx.x;
  return t == BLOCK - 1 ? 0 : t + 1;
}
__device__ __forceinline__ int64_t tile_cell(int64_t first, int64_t lo, int64_t hi, int j) {
  const int64_t i = first - 1 + j;               // cell at position j
  return i < lo ? lo : (i >= hi ? hi - 1 : i);  // ghost cells copy the end cells
}
template <int BLOCK, class Loader>
__device__ __forceinline__ void mixed_tile_load(int64_t first, int64_t lo, int64_t hi, const Loader& load,
                                                MixedCellIn& c) {
  const int j = tile_local<BLOCK>();
  load(j, tile_cell(first, lo, hi, j), c);
}
// kOwnRegs: a face reads its left cell (this thread's) and an update its right face
// (this thread's) from registers instead of shared memory -- 21 fewer shared loads
// per cell (the 7 pairs of flux, state and face), at 11 more registers live across a
// barrier (the same values either way).
template <int BLOCK, bool kOwnRegs = true, bool kTiled = false, class Loader>
__device__ __forceinline__ float mixed_tile_run(const MixedArrays& a, const EosMixed& em, int64_t first, int64_t lo,
                                                int64_t hi, float dtdx, int flux, int bc, DevState* S,
                                                const Loader& load, MixedCellIn& c) {
  __shared__ float2 sF[7][BLOCK];  // per variable pair: cell fluxes, then the face fluxes
  __shared__ float sL[BLOCK];
  const int j = tile_local<BLOCK>();  // position of this thread's cell in the tile
  const int64_t i = first - 1 + j;
  const int64_t ic = tile_cell(first, lo, hi, j);
  float2 fc[7];  // this cell's flux: its own face reads it from registers
  {
    PrimM P;
    int st = prim_from_islands(em, c.qh, c.ql, c.I0, P);
    StressCT<float> sc = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
    float f11[kNFlux1];
    flux_mixed(em, c.qh, P, sc, f11);
    flux_pairs(f11, fc);
#pragma unroll
    for (int k = 0; k < 7; ++k) sF[k][j] = fc[k];
    load.keep(j, c);
    sL[j] = c.li;
    if (st && i == ic && j > 0 && j < BLOCK - 1) mixed_record_err(S, st, i);
  }
  __syncthreads();
  // face j + 1/2 between local cells j (this thread: registers) and j + 1 (shared memory)
  float2 fv[7];
  if (j < BLOCK - 1) {
    const float lf = flux == HYP_FLUX_LXF ? 1.0f / dtdx : fmaxf(kOwnRegs ? c.li : sL[j], sL[j + 1]);
    const float2 nhl = f2s(-0.5f * lf), half = f2s(0.5f);
    const int64_t i1 = i + 1, ic1 = i1 < lo ? lo : (i1 >= hi ? hi - 1 : i1);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const float2 fl = kOwnRegs ? fc[k] : sF[k][j], fr = sF[k][j + 1];
      const float2 ql = kOwnRegs ? pair_of(c.qh, k) : load.face_q2(k, j, ic);
      fv[k] = f2fma(nhl, f2sub(load.face_q2(k, j + 1, ic1), ql), f2mul(half, f2add(fl, fr)));
    }
  }
  __syncthreads();
  load.release();
  if (j < BLOCK - 1) {
#pragma unroll
    for (int k = 0; k < 7; ++k) sF[k][j] = fv[k];
  }
  __syncthreads();
  float lnew = 0.0f;
  const bool own = j > 0 && j < BLOCK - 1 && i < hi;
  if (own) {
    const bool frozen = bc_holds(bc, i == lo, i == hi - 1);
    Islands I = c.I0;
    if (frozen) {
      lnew = c.li;
    } else {
      const float2 ndt = f2s(-dtdx);
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        const float2 delta = f2mul(ndt, f2sub(kOwnRegs ? fv[k] : sF[k][j], sF[k][j - 1]));  // F_{j+1/2} - F_{j-1/2}
        const ff2 q = ff2_add_f(ff2{pair_of(c.qh, k), pair_of(c.ql, k)}, delta);
        c.qh[2 * k] = q.hi.x;
        c.qh[2 * k + 1] = q.hi.y;
        c.ql[2 * k] = q.lo.x;
        c.ql[2 * k + 1] = q.lo.y;
      }
      PrimM P;
      int st = prim_mixed(em, c.qh, c.ql, P, I);
      StressCT<float> sc = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
      lnew = lambda_mixed(em, P, sc);
      if (!(lnew <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
      if (st) mixed_record_err(S, st, i);
    }
    int64_t off = i;
    if constexpr (kTiled) off = load.origin().base + (i - first);  // an owned cell: in the tile's span
    mixed_store_cell(a.out + off, rows_apart<kTiled>(a), c.qh, c.ql, lnew, I);
  } else if constexpr (kTiled && BLOCK == kTileCells + 2) {
    if (j == 0 || j == BLOCK - 1) {
      // the halo threads fill the two unused floats of each row of the output tile, so
      // that the last warp writes whole 128-byte lines (no partial sectors for L2 to merge)
      float* q = a.out + load.origin().base + (j == 0 ? kTileRow - 1 : kTileRow - 2);
#pragma unroll
      for (int r = 0; r < kMixedRows; ++r) q[r * kTileRow] = 0.0f;
    }
  }
  __syncthreads();  // the shared arrays are reused by the block's next tile
  return lnew;
}
template <int BLOCK, bool kTiled = false, class Loader>
__device__ __forceinline__ float mixed_tile(const MixedArrays& a, const EosMixed& em, int64_t first, int64_t lo,
                                            int64_t hi, float dtdx, int flux, int bc, DevState* S,
                                            const Loader& load) {
  MixedCellIn c;
  mixed_tile_load<BLOCK>(first, lo, hi, load, c);
  return mixed_tile_run<BLOCK, true, kTiled>(a, em, first, lo, hi, dtdx, flux, bc, S, load, c);
}

// Wave speed and island outputs of one cell of a freshly uploaded state, into rows
// kRowLam.. of the cell at q (rows rstride apart).
__device__ __forceinline__ float mixed_cell_lambda_of(const EosMixed& em, const float* qh, const float* ql, int64_t i,
                                                      DevState* S, float* q, int64_t rstride) {
  PrimM P;
  Islands I;
  int st = prim_mixed(em, qh, ql, P, I);
  StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
  const float l = lambda_mixed(em, P, c);
  if (!(l <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
  if (st) mixed_record_err(S, st, i);
  q[kRowLam * rstride] = l;
  q[kRowIsl * rstride] = I.ir;
  q[(kRowIsl + 1) * rstride] = I.e_int;
  q[(kRowIsl + 2) * rstride] = I.sm1;
  return l;
}
// The same for cell i of a.in, written into a.in's own block (an upload's state).
template <bool kTiled>
__device__ __forceinline__ float mixed_cell_lambda(const MixedArrays& a, const EosMixed& em, int64_t i, DevState* S) {
  const int64_t r = rows_apart<kTiled>(a);
  float* q = const_cast<float*>(a.in) + cell_at<kTiled>(i);
  float qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = q[v * r];
    ql[v] = q[(kRowLo + v) * r];
  }
  return mixed_cell_lambda_of(em, qh, ql, i, S, q, r);
}

}  // namespace hyp
