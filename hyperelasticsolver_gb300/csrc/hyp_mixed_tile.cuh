// hyp_mixed_tile.cuh -- one tile of the mixed-precision single-phase step,
// shared by the single-problem kernel (hyp_step1_mixed.cu) and the batched
// kernel (hyp_batch.cu).
//
// A block of BLOCK threads owns BLOCK - 2 consecutive cells of one problem and
// loads them plus one halo cell on each side (clamped to the problem's cells
// [lo, hi): a ghost cell copies the end cell, i.e. a zero-gradient boundary):
//   1. flux of every loaded cell from its (hi, lo) state and the float-float
//      island outputs cached by the step that produced it -> shared memory;
//   2. Rusanov face fluxes 0.5 (f_L + f_R) - 0.5 lambda_face (Q_R - Q_L)
//      (NumFluxes.jl:25-33; main.jl:45-48), lambda_face = max(lambda_L, lambda_R);
//   3. Q += -dt/dx (F_{i+1/2} - F_{i-1/2}) accumulated into (hi, lo) (main.jl:43-60);
//   4. islands, cons2prim and wave speed of the NEW state, stored per cell.
// Returns the thread's new wave speed; the caller reduces the block max.
#pragma once
#include "hyp_internal.cuh"

namespace hyp {

struct MixedArrays {
  const float* Qh;  // [14][stride] hi parts
  const float* Ql;  // [14][stride] lo parts
  const float* lam; // [stride] wave speed of the state
  const float* isl; // [3][stride] island outputs of the state
  float* Qh_out;
  float* Ql_out;
  float* lam_out;
  float* isl_out;
  int64_t stride;   // floats between rows (a multiple of 4)
  int64_t n;        // cells
  int64_t own_lo, own_hi;  // cells whose new wave speed enters the step's max (a slab's ghosts do not)
};

// One cell's inputs to a tile.
struct MixedCellIn {
  float qh[14], ql[14];
  float li;
  Islands I0;
};

// Loads the cell's inputs straight from the state arrays and keeps the hi parts
// the face phase reads in shared memory.
// Loader interface used by mixed_tile: operator()(j, ic, c) fills cell ic's
// inputs for local index j; keep(j, c) stores what face_q needs; face_q(v, j, ic)
// returns the hi part of variable v of local cell j (cell ic); release() runs
// once the face phase has read its inputs.
template <int BLOCK>
struct MixedGlobalLoader {
  const MixedArrays& a;
  __device__ __forceinline__ static float (&sQ())[14][BLOCK] {
    __shared__ float q[14][BLOCK];
    return q;
  }
  __device__ __forceinline__ void operator()(int, int64_t ic, MixedCellIn& c) const {
    const int64_t n = a.stride;
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      c.qh[v] = a.Qh[v * n + ic];
      c.ql[v] = a.Ql[v * n + ic];
    }
    c.li = a.lam[ic];
    c.I0.ir = a.isl[ic];
    c.I0.e_int = a.isl[n + ic];
    c.I0.sm1 = a.isl[2 * n + ic];
  }
  __device__ __forceinline__ void keep(int j, const MixedCellIn& c) const {
#pragma unroll
    for (int v = 0; v < 14; ++v) sQ()[v][j] = c.qh[v];
  }
  __device__ __forceinline__ float face_q(int v, int j, int64_t) const { return sQ()[v][j]; }
  __device__ __forceinline__ void release() const {}
};

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
__device__ __forceinline__ int64_t tile_cell(int64_t first, int64_t lo, int64_t hi) {
  const int64_t i = first - 1 + threadIdx.x;     // cell of this thread (halo at j = 0, BLOCK - 1)
  return i < lo ? lo : (i >= hi ? hi - 1 : i);  // ghost cells copy the end cells
}
template <class Loader>
__device__ __forceinline__ void mixed_tile_load(int64_t first, int64_t lo, int64_t hi, const Loader& load,
                                                MixedCellIn& c) {
  load((int)threadIdx.x, tile_cell(first, lo, hi), c);
}
// kOwnRegs: a face reads its left cell (this thread's) and an update its right face
// (this thread's) from registers instead of shared memory -- 39 fewer shared loads
// per cell, at 11 more registers live across a barrier (the same values either way).
template <int BLOCK, bool kOwnRegs = true, class Loader>
__device__ __forceinline__ float mixed_tile_run(const MixedArrays& a, const EosMixed& em, int64_t first, int64_t lo,
                                                int64_t hi, float dtdx, int flux, int bc, DevState* S,
                                                const Loader& load, MixedCellIn& c) {
  __shared__ float sFF[14][BLOCK];  // cell fluxes (11 slots), then the face fluxes (14)
  __shared__ float sL[BLOCK];
  const int64_t n = a.stride;
  const int j = threadIdx.x;
  const int64_t i = first - 1 + j;
  const int64_t ic = tile_cell(first, lo, hi);
  float f11[kNFlux1];  // this cell's flux: its own face reads it from registers
  {
    PrimM P;
    int st = prim_from_islands(em, c.qh, c.ql, c.I0, P);
    StressCT<float> sc = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
    flux_mixed(em, c.qh, P, sc, f11);
#pragma unroll
    for (int s = 0; s < kNFlux1; ++s) sFF[s][j] = f11[s];
    load.keep(j, c);
    sL[j] = c.li;
    if (st && i == ic && j > 0 && j < BLOCK - 1) mixed_record_err(S, st, i);
  }
  __syncthreads();
  // face j + 1/2 between local cells j (this thread: registers) and j + 1 (shared memory)
  float fv[14];
  if (j < BLOCK - 1) {
    const float lf = flux == HYP_FLUX_LXF ? 1.0f / dtdx : fmaxf(kOwnRegs ? c.li : sL[j], sL[j + 1]);
    const float hl = 0.5f * lf;
    const int64_t i1 = i + 1, ic1 = i1 < lo ? lo : (i1 >= hi ? hi - 1 : i1);
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const int s = flux_slot1(v);
      const float fl = s >= 0 ? (kOwnRegs ? f11[s] : sFF[s][j]) : 0.0f, fr = s >= 0 ? sFF[s][j + 1] : 0.0f;
      fv[v] = 0.5f * (fl + fr) - hl * (load.face_q(v, j + 1, ic1) - (kOwnRegs ? c.qh[v] : load.face_q(v, j, ic)));
    }
  }
  __syncthreads();
  load.release();
  if (j < BLOCK - 1) {
#pragma unroll
    for (int v = 0; v < 14; ++v) sFF[v][j] = fv[v];
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
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        const float delta = -dtdx * ((kOwnRegs ? fv[v] : sFF[v][j]) - sFF[v][j - 1]);  // F_{j+1/2} - F_{j-1/2}
        ff q = ff_add_f(ff{c.qh[v], c.ql[v]}, delta);
        c.qh[v] = q.hi;
        c.ql[v] = q.lo;
      }
      PrimM P;
      int st = prim_mixed(em, c.qh, c.ql, P, I);
      StressCT<float> sc = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
      lnew = lambda_mixed(em, P, sc);
      if (!(lnew <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
      if (st) mixed_record_err(S, st, i);
    }
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      a.Qh_out[v * n + i] = c.qh[v];
      a.Ql_out[v * n + i] = c.ql[v];
    }
    a.lam_out[i] = lnew;
    a.isl_out[i] = I.ir;
    a.isl_out[n + i] = I.e_int;
    a.isl_out[2 * n + i] = I.sm1;
  }
  __syncthreads();  // the shared arrays are reused by the block's next tile
  return lnew;
}
template <int BLOCK, class Loader>
__device__ __forceinline__ float mixed_tile(const MixedArrays& a, const EosMixed& em, int64_t first, int64_t lo,
                                            int64_t hi, float dtdx, int flux, int bc, DevState* S,
                                            const Loader& load) {
  MixedCellIn c;
  mixed_tile_load(first, lo, hi, load, c);
  return mixed_tile_run<BLOCK>(a, em, first, lo, hi, dtdx, flux, bc, S, load, c);
}

// Wave speed and island outputs of one cell of a freshly uploaded state.
__device__ __forceinline__ float mixed_cell_lambda_of(const EosMixed& em, const float* qh, const float* ql, int64_t i,
                                                      int64_t n, DevState* S, float* lam_out, float* isl_out) {
  PrimM P;
  Islands I;
  int st = prim_mixed(em, qh, ql, P, I);
  StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
  const float l = lambda_mixed(em, P, c);
  if (!(l <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
  if (st) mixed_record_err(S, st, i);
  lam_out[i] = l;
  isl_out[i] = I.ir;
  isl_out[n + i] = I.e_int;
  isl_out[2 * n + i] = I.sm1;
  return l;
}
__device__ __forceinline__ float mixed_cell_lambda(const MixedArrays& a, const EosMixed& em, int64_t i, DevState* S,
                                                   float* lam_out, float* isl_out) {
  const int64_t n = a.stride;
  float qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = a.Qh[v * n + i];
    ql[v] = a.Ql[v * n + i];
  }
  return mixed_cell_lambda_of(em, qh, ql, i, n, S, lam_out, isl_out);
}

}  // namespace hyp
