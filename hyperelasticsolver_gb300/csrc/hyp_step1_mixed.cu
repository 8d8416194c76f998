// hyp_step1_mixed.cu -- single-phase step in mixed precision: FP32 fluxes and
// wave speeds, a compensated (hi, lo) FP32 state, float-float islands in
// cons2prim (hyp_physics_mixed.cuh).
//
// One fused kernel per step. A block owns kTile = 254 cells and loads
// kTile + 2 (one halo cell each side) with one thread per cell:
//   1. cons2prim and flux of every loaded cell into shared memory, with the
//      cell's wave speed lambda_i computed by the previous step;
//   2. Rusanov face fluxes 0.5 (f_L + f_R) - 0.5 max(lambda_L, lambda_R) (Q_R - Q_L)
//      (NumFluxes.jl:25-33; main.jl:45-48) for the kTile + 1 faces;
//   3. Q += -dt/dx (F_{i+1/2} - F_{i-1/2}) accumulated into (hi, lo) (main.jl:43-60);
//   4. epilogue: lambda of the NEW state (cons2prim, acoustic tensor,
//      spectral radius), stored per cell and max-reduced (warp shuffles, one
//      shared-memory pass, one atomicMax per block) for the next step's
//      dt = cfl dx / max lambda (main.jl:204-212).
// HBM traffic per cell-update: the state read and written (14 x 2 x 4 B each
// way) plus, each way, the cell's FP32 lambda and the three outputs of its
// float-float islands (1/rho, e_int, rho/rho0 - 1), so that step 1 needs no
// float-float work: 256 B, against 224 B for the state alone.
// The three max-lambda slots rotate (read k%3, write (k+1)%3, clear (k+2)%3)
// so one launch per step needs no separate reset.
#include "hyp_internal.cuh"
#include "hyp_physics_mixed.cuh"

namespace hyp {

constexpr int kTileM = kBlock - 2;

__device__ __forceinline__ float block_max_f(float v) {
  __shared__ float red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < kBlock / 32 ? red[l] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

__device__ __forceinline__ void record_err(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

struct MixedSlots {
  int p;              // state / time parity
  int rd, wr, clr;    // max-lambda slots: read (this step), write (next step), clear
};

__global__ void __launch_bounds__(kBlock, 4)
    step1_mixed_kernel(const float* __restrict__ Qh, const float* __restrict__ Ql, const float* __restrict__ lam,
                       const float* __restrict__ isl, float* __restrict__ Qh_out, float* __restrict__ Ql_out,
                       float* __restrict__ lam_out, float* __restrict__ isl_out, int64_t n, EosMixed em,
                       MixedSlots sl, DevState* S, double t_end, double cfl, double dx, int flux, int bc) {
  __shared__ float sF[kNFlux1][kBlock];
  __shared__ float sQ[14][kBlock];
  __shared__ float sFace[14][kBlock];
  __shared__ float sL[kBlock];

  const double tn = S->t[sl.p];
  const bool active = tn < t_end;
  const float lmax = __uint_as_float((unsigned)S->lam_slots[sl.rd]);
  const float dtdx = (float)cfl / lmax;  // dt/dx = cfl / max lambda
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double dt = (cfl * dx) / (double)lmax;
    S->t[1 - sl.p] = active ? tn + dt : tn;
    if (active) {  // an inactive step must keep the slot that holds the current state's max lambda
      S->lam_slots[sl.clr] = 0ull;
      S->steps += 1;
    }
  }
  if (!active) return;

  const int j = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * kTileM - 1 + j;  // cell of this thread (halo at j = 0, kBlock-1)
  const int64_t ic = i < 0 ? 0 : (i >= n ? n - 1 : i);    // ghost cells copy the end cells
  float qh[14], ql[14];
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    qh[v] = Qh[v * n + ic];
    ql[v] = Ql[v * n + ic];
  }
  const float li = lam[ic];
  Islands I0;  // this state's island outputs, cached by the step that produced it
  I0.ir = isl[ic];
  I0.e_int = isl[n + ic];
  I0.sm1 = isl[2 * n + ic];
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
    if (st && i == ic && j > 0 && j < kBlock - 1) record_err(S, st, i);
  }
  __syncthreads();
  // face j + 1/2 between local cells j and j + 1
  if (j < kBlock - 1) {
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
  const bool own = j > 0 && j < kBlock - 1 && i < n;
  if (own) {
    const bool frozen = bc == HYP_BC_FROZEN && (i == 0 || i == n - 1);
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
      if (st) record_err(S, st, i);
    }
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      Qh_out[v * n + i] = qh[v];
      Ql_out[v * n + i] = ql[v];
    }
    lam_out[i] = lnew;
    isl_out[i] = I.ir;
    isl_out[n + i] = I.e_int;
    isl_out[2 * n + i] = I.sm1;
  }
  const float m = block_max_f(own ? lnew : 0.0f);
  if (threadIdx.x == 0) atomicMax(&S->lam_slots[sl.wr], (unsigned long long)__float_as_uint(m));
}

// lambda of every cell of the state (after an upload) and its max into a slot.
__global__ void __launch_bounds__(kBlock) lam1_mixed_kernel(const float* __restrict__ Qh, const float* __restrict__ Ql,
                                                            float* __restrict__ lam, float* __restrict__ isl,
                                                            int64_t n, EosMixed em, unsigned long long* slot,
                                                            DevState* S) {
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  float l = 0.0f;
  if (i < n) {
    float qh[14], ql[14];
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      qh[v] = Qh[v * n + i];
      ql[v] = Ql[v * n + i];
    }
    PrimM P;
    Islands I;
    int st = prim_mixed(em, qh, ql, P, I);
    StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
    l = lambda_mixed(em, P, c);
    if (!(l <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
    if (st) record_err(S, st, i);
    lam[i] = l;
    isl[i] = I.ir;
    isl[n + i] = I.e_int;
    isl[2 * n + i] = I.sm1;
  }
  const float m = block_max_f(l);
  if (threadIdx.x == 0) atomicMax(slot, (unsigned long long)__float_as_uint(m));
}

// FP64 -> (hi, lo) and back.
__global__ void split_kernel(const double* __restrict__ q, float* __restrict__ hi, float* __restrict__ lo, int64_t m) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    const double x = q[k];
    const float h = (float)x;
    hi[k] = h;
    lo[k] = (float)(x - (double)h);
  }
}
__global__ void join_kernel(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ q, int64_t m) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x)
    q[k] = (double)hi[k] + (double)lo[k];
}

static unsigned elementwise_grid(int64_t m) {
  int64_t g = (m + kBlock - 1) / kBlock;
  return (unsigned)(g > 152 * 64 ? 152 * 64 : (g < 1 ? 1 : g));
}

cudaError_t launch_split(hyp_ctx* c, const double* q, float* hi, float* lo) {
  const int64_t m = (int64_t)14 * c->n;
  split_kernel<<<elementwise_grid(m), kBlock, 0, c->stream>>>(q, hi, lo, m);
  return cudaGetLastError();
}
cudaError_t launch_join(hyp_ctx* c, const float* hi, const float* lo, double* q) {
  const int64_t m = (int64_t)14 * c->n;
  join_kernel<<<elementwise_grid(m), kBlock, 0, c->stream>>>(hi, lo, q, m);
  return cudaGetLastError();
}
cudaError_t launch_lam1_mixed(hyp_ctx* c, int p, unsigned long long* slot) {
  const unsigned grid = (unsigned)((c->n + kBlock - 1) / kBlock);
  lam1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(c->Qh[p], c->Ql[p], c->lamf[p], c->isl[p], c->n, c->eos_mixed,
                                                    slot, c->st);
  return cudaGetLastError();
}
cudaError_t launch_step1_mixed(hyp_ctx* c, long long k, double t_end) {
  const int p = (int)(k & 1);
  MixedSlots sl;
  sl.p = p;
  sl.rd = (int)(k % 3);
  sl.wr = (int)((k + 1) % 3);
  sl.clr = (int)((k + 2) % 3);
  const unsigned grid = (unsigned)((c->n + kTileM - 1) / kTileM);
  const double dx = c->cfg.x_length / (double)c->n;
  step1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(c->Qh[p], c->Ql[p], c->lamf[p], c->isl[p], c->Qh[1 - p],
                                                     c->Ql[1 - p], c->lamf[1 - p], c->isl[1 - p], c->n, c->eos_mixed,
                                                     sl, c->st, t_end, c->cfg.cfl, dx, c->cfg.flux, c->cfg.bc);
  return cudaGetLastError();
}

}  // namespace hyp
