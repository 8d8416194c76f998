// hyp_step1.cu -- single-phase FP64 step: Rusanov / LxF first-order update of
// main.jl:202-227 with the per-phase model of HyperelasticityMPh.jl at alpha == 1.
//
// One step = two kernels on the context stream:
//   cell   : per cell cons2prim -> stress -> flux (11 non-zero components) and
//            lambda_i = |u1| + sqrt(max|eig(acoustic)|); block max of lambda by
//            warp shuffles and one shared-memory pass, one atomicMax per block.
//            (main.jl:204-211; HyperelasticityMPh.jl:106-175, 252-266)
//   update : dt = cfl*dx / max lambda, t += dt, and per interior cell
//            Q - dt/dx (F_{i+1/2} - F_{i-1/2}) with the Rusanov face flux
//            0.5 (f_L + f_R) - 0.5 max(lambda_L, lambda_R) (Q_R - Q_L)
//            (NumFluxes.jl:25-33; main.jl:45-48, 43-60); end cells frozen
//            (main.jl:219-220) or transmissive.
// The flux/wave-speed work is done once per cell; the update kernel streams
// state, fluxes and speeds (SoA, coalesced 8-byte loads along the cell index).
#include "hyp_internal.cuh"

namespace hyp {

__device__ __forceinline__ void record_error(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < kBlock / 32 ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

__global__ void __launch_bounds__(kBlock) cell1_f64_kernel(const double* __restrict__ Q, int64_t n, EosC e,
                                                           double* __restrict__ F, double* __restrict__ lam,
                                                           unsigned long long* lam_slot, const double* t_now,
                                                           double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;  // uniform across the grid
  int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    double q[14];
#pragma unroll
    for (int v = 0; v < 14; ++v) q[v] = Q[v * n + i];
    Prim P;
    int st = cons_to_prim(e, 1.0, q + 1, q[4], q + 5, P);
    StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
    double f[14], s0[3];
    phase_flux(e, 1.0, P, c, f, s0);
    l = fabs(P.u[0]) + phase_cmax(e, P, c);
    if (!(l <= 1.79e308)) st |= HYP_CELL_NONFINITE;
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      int sl = flux_slot1(v);
      if (sl >= 0) F[sl * n + i] = f[v];
    }
    lam[i] = l;
    if (st) record_error(S, st, i);
  }
  double m = block_max(l);
  if (threadIdx.x == 0) atomicMax(lam_slot, (unsigned long long)__double_as_longlong(m));
}

// Each face is evaluated once, by the block that owns the cell on its right (the
// block's last cell also evaluates its right face), into shared memory; both cells
// of a face read the same value, so the update conserves exactly.
__global__ void __launch_bounds__(kBlock) update1_f64_kernel(const double* __restrict__ Q, double* __restrict__ Qn,
                                                             int64_t n, const double* __restrict__ F,
                                                             const double* __restrict__ lam,
                                                             const unsigned long long* lam_in,
                                                             unsigned long long* lam_next, const double* t_in,
                                                             double* t_out, long long* steps, double t_end,
                                                             double cfl, double dx, int flux, int bc) {
  __shared__ double sF[14][kBlock + 1];  // face k of the block = left face of cell i0 + k
  const double tn = *t_in;
  const bool active = tn < t_end;
  const double lmax = __longlong_as_double((long long)*lam_in);
  // Rusanov / HLL: dt/dx (main.jl:225); LxF: 1/lambda with lambda = dx/dt (main.jl:223, :40)
  const StepScalars sc = step_scalars(cfl, dx, lmax, flux == HYP_FLUX_LXF);
  const double dt = sc.dt, lam_lxf = sc.lam_lxf, dtdx = sc.dtdx;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *t_out = active ? tn + dt : tn;
    *lam_next = 0ull;
    if (active) *steps += 1;
  }
  if (!active) return;  // the same for every block
  const int64_t i0 = (int64_t)blockIdx.x * kBlock;
  const int64_t i = i0 + threadIdx.x;
  const bool lxf = flux == HYP_FLUX_LXF;
  if (i < n) {
    rusanov_face<kBlock + 1>(Q, F, lam, n, 0, n, i, lxf, lam_lxf, sF, threadIdx.x);
    if (threadIdx.x == kBlock - 1 || i == n - 1)
      rusanov_face<kBlock + 1>(Q, F, lam, n, 0, n, i + 1, lxf, lam_lxf, sF, threadIdx.x + 1);
  }
  __syncthreads();
  if (i >= n) return;
  const bool frozen = bc_holds(bc, i == 0, i == n - 1);
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    const double qc = Q[v * n + i];
    Qn[v * n + i] = frozen ? qc : __fma_rn(-dtdx, __dsub_rn(sF[v][threadIdx.x + 1], sF[v][threadIdx.x]), qc);
  }
}

static inline unsigned grid_for(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

cudaError_t launch_cell1_f64(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end) {
  cell1_f64_kernel<<<grid_for(c->n), kBlock, 0, c->stream>>>(c->Q[p], c->n, c->eos[0], c->F, c->lam, lam_slot, t_now,
                                                             t_end, c->st);
  return cudaGetLastError();
}

cudaError_t launch_update1_f64(hyp_ctx* c, int p, double t_end) {
  update1_f64_kernel<<<grid_for(c->n), kBlock, 0, c->stream>>>(
      c->Q[p], c->Q[1 - p], c->n, c->F, c->lam, &c->st->lam_bits[p], &c->st->lam_bits[1 - p], &c->st->t[p],
      &c->st->t[1 - p], &c->st->steps, t_end, c->cfg.cfl, ctx_dx(c), c->cfg.flux, ctx_bc(c));
  return cudaGetLastError();
}

}  // namespace hyp
