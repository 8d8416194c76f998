// hyp_step1_mixed.cu -- single-phase step in mixed precision: FP32 fluxes and
// wave speeds, a compensated (hi, lo) FP32 state, float-float islands in
// cons2prim (hyp_physics_mixed.cuh).
//
// One fused kernel per step; each block runs one tile of hyp_mixed_tile.cuh
// (kBlock - 2 owned cells plus a halo cell each side): flux phase, Rusanov
// faces, compensated update, then the wave speed of the NEW state, stored per
// cell and max-reduced (warp shuffles, one shared-memory pass, one atomicMax
// per block) for the next step's dt = cfl dx / max lambda (main.jl:204-212).
// HBM traffic per cell-update: the state read and written (14 x 2 x 4 B each
// way) plus, each way, the cell's FP32 lambda and the three outputs of its
// float-float islands (1/rho, e_int, rho/rho0 - 1), so that the flux phase needs
// no float-float work: 256 B, against 224 B for the state alone.
// The three max-lambda slots rotate (read k%3, write (k+1)%3, clear (k+2)%3)
// so one launch per step needs no separate reset.
#include "hyp_internal.cuh"
#include "hyp_mixed_tile.cuh"

namespace hyp {

constexpr int kTileM = kBlock - 2;

struct MixedSlots {
  int p;              // state / time parity
  int rd, wr, clr;    // max-lambda slots: read (this step), write (next step), clear
};

__global__ void __launch_bounds__(kBlock, 4)
    step1_mixed_kernel(MixedArrays a, EosMixed em, MixedSlots sl, DevState* S, double t_end, double cfl, double dx,
                       int flux, int bc) {
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
  const float m = mixed_tile<kBlock>(a, em, (int64_t)blockIdx.x * kTileM, 0, a.stride, dtdx, flux, bc, S);
  if (threadIdx.x == 0) atomicMax(&S->lam_slots[sl.wr], (unsigned long long)__float_as_uint(m));
}

// lambda of every cell of the state (after an upload) and its max into a slot.
__global__ void __launch_bounds__(kBlock) lam1_mixed_kernel(MixedArrays a, EosMixed em, unsigned long long* slot,
                                                            DevState* S) {
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  float l = 0.0f;
  if (i < a.stride) l = mixed_cell_lambda(a, em, i, S, a.lam_out, a.isl_out);
  const float m = mixed_block_max<kBlock>(l);
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

unsigned elementwise_grid(int64_t m) {
  int64_t g = (m + kBlock - 1) / kBlock;
  return (unsigned)(g > 152 * 64 ? 152 * 64 : (g < 1 ? 1 : g));
}

cudaError_t launch_split_n(cudaStream_t s, const double* q, float* hi, float* lo, int64_t m) {
  split_kernel<<<elementwise_grid(m), kBlock, 0, s>>>(q, hi, lo, m);
  return cudaGetLastError();
}
cudaError_t launch_join_n(cudaStream_t s, const float* hi, const float* lo, double* q, int64_t m) {
  join_kernel<<<elementwise_grid(m), kBlock, 0, s>>>(hi, lo, q, m);
  return cudaGetLastError();
}
cudaError_t launch_split(hyp_ctx* c, const double* q, float* hi, float* lo) {
  return launch_split_n(c->stream, q, hi, lo, (int64_t)14 * c->n);
}
cudaError_t launch_join(hyp_ctx* c, const float* hi, const float* lo, double* q) {
  return launch_join_n(c->stream, hi, lo, q, (int64_t)14 * c->n);
}

static MixedArrays arrays_of(hyp_ctx* c, int p) {
  MixedArrays a;
  a.Qh = c->Qh[p];
  a.Ql = c->Ql[p];
  a.lam = c->lamf[p];
  a.isl = c->isl[p];
  a.Qh_out = c->Qh[1 - p];
  a.Ql_out = c->Ql[1 - p];
  a.lam_out = c->lamf[1 - p];
  a.isl_out = c->isl[1 - p];
  a.stride = c->n;
  return a;
}

cudaError_t launch_lam1_mixed(hyp_ctx* c, int p, unsigned long long* slot) {
  const unsigned grid = (unsigned)((c->n + kBlock - 1) / kBlock);
  MixedArrays a = arrays_of(c, p);
  a.lam_out = c->lamf[p];  // the uploaded state's own lambda and islands
  a.isl_out = c->isl[p];
  lam1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(a, c->eos_mixed, slot, c->st);
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
  step1_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(arrays_of(c, p), c->eos_mixed, sl, c->st, t_end, c->cfg.cfl, dx,
                                                     c->cfg.flux, c->cfg.bc);
  return cudaGetLastError();
}

}  // namespace hyp
