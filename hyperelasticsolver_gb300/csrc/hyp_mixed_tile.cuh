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
// Returns the block max of the new wave speeds (valid in thread 0).
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
  int64_t stride;   // cells per variable row
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
template <int BLOCK>
__device__ __forceinline__ float mixed_tile(const MixedArrays& a, const EosMixed& em, int64_t first, int64_t lo,
                                            int64_t hi, float dtdx, int flux, int bc, DevState* S) {
  __shared__ float sF[kNFlux1][BLOCK];
  __shared__ float sQ[14][BLOCK];
  __shared__ float sFace[14][BLOCK];
  __shared__ float sL[BLOCK];
  const int64_t n = a.stride;
  const int j = threadIdx.x;
  const int64_t i = first - 1 + j;                         // cell of this thread (halo at j = 0, BLOCK - 1)
  const int64_t ic = i < lo ? lo : (i >= hi ? hi - 1 : i);  // ghost cells copy the end cells
  float qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = a.Qh[v * n + ic];
    ql[v] = a.Ql[v * n + ic];
  }
  const float li = a.lam[ic];
  Islands I0;  // this state's island outputs, cached by the step that produced it
  I0.ir = a.isl[ic];
  I0.e_int = a.isl[n + ic];
  I0.sm1 = a.isl[2 * n + ic];
  {
    PrimM P;
    int st = prim_from_islands(em, qh, ql, I0, P);
    StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
    float f11[kNFlux1];
    flux_mixed(em, qh, P, c, f11);
#pragma unroll
    for (int s = 0; s < kNFlux1; ++s) sF[s][j] = f11[s];
#pragma unroll
    for (int v = 0; v < 14; ++v) sQ[v][j] = qh[v];
    sL[j] = li;
    if (st && i == ic && j > 0 && j < BLOCK - 1) mixed_record_err(S, st, i);
  }
  __syncthreads();
  // face j + 1/2 between local cells j and j + 1
  if (j < BLOCK - 1) {
    const float lf = flux == HYP_FLUX_LXF ? 1.0f / dtdx : fmaxf(sL[j], sL[j + 1]);
    const float hl = 0.5f * lf;
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const int s = flux_slot1(v);
      const float fl = s >= 0 ? sF[s][j] : 0.0f, fr = s >= 0 ? sF[s][j + 1] : 0.0f;
      sFace[v][j] = 0.5f * (fl + fr) - hl * (sQ[v][j + 1] - sQ[v][j]);
    }
  }
  __syncthreads();
  float lnew = 0.0f;
  const bool own = j > 0 && j < BLOCK - 1 && i < hi;
  if (own) {
    const bool frozen = bc == HYP_BC_FROZEN && (i == lo || i == hi - 1);
    Islands I = I0;
    if (frozen) {
      lnew = li;
    } else {
#pragma unroll
      for (int v = 0; v < 14; ++v) {
        const float delta = -dtdx * (sFace[v][j] - sFace[v][j - 1]);
        ff q = ff_add_f(ff{qh[v], ql[v]}, delta);
        qh[v] = q.hi;
        ql[v] = q.lo;
      }
      PrimM P;
      int st = prim_mixed(em, qh, ql, P, I);
      StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
      lnew = lambda_mixed(em, P, c);
      if (!(lnew <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
      if (st) mixed_record_err(S, st, i);
    }
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      a.Qh_out[v * n + i] = qh[v];
      a.Ql_out[v * n + i] = ql[v];
    }
    a.lam_out[i] = lnew;
    a.isl_out[i] = I.ir;
    a.isl_out[n + i] = I.e_int;
    a.isl_out[2 * n + i] = I.sm1;
  }
  return mixed_block_max<BLOCK>(own ? lnew : 0.0f);
}

// Wave speed and island outputs of one cell of a freshly uploaded state.
__device__ __forceinline__ float mixed_cell_lambda(const MixedArrays& a, const EosMixed& em, int64_t i, DevState* S,
                                                   float* lam_out, float* isl_out) {
  const int64_t n = a.stride;
  float qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = a.Qh[v * n + i];
    ql[v] = a.Ql[v * n + i];
  }
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

}  // namespace hyp
