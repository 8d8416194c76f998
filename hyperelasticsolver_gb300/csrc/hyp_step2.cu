// hyp_step2.cu -- two-phase FP64 step with the path-conservative HLL flux
// (main.jl:202-241 with update_cell :43-60 and NumFluxes.hll :70-132) or the
// path-conservative Lax-Friedrichs flux (update_cell :30-41, NumFluxes.lxf :25-60).
//
// Three kernels per step on the context stream:
//   cell   : per cell, both phases' flux (HyperelasticityMPh.jl:140-175) and
//            wave-speed bounds (:252-266); lambda_i = max |speed|, block max ->
//            one atomicMax (main.jl:204-212);
//   face   : per face, the HLL fluctuations D-, D+ (hll_face2: midpoint speeds,
//            three 6-point Gauss-Legendre path integrals of B, Q_hll), one
//            thread per face -- 18 evaluations of B per face instead of the 30
//            the reference makes, since the integrals repeated in D- and D+ are
//            the same;
//   update : dt = cfl dx / max lambda, t += dt, Q_i - dt/dx ((F_r - F_l) + (D-_{i+1/2} + D+_{i-1/2}))
//            with frozen or transmissive ends; F = 0 for HLL (it folds the conservative
//            part into D+-), the LxF face flux otherwise.
// The LxF face kernel takes lambda = dx/dt of this step (main.jl:223) from the
// max wave speed the cell kernel has just reduced, and integrates B with the
// 6-point Gauss-Lobatto rule.
#include "hyp_internal.cuh"
#include "hyp_physics_mph.cuh"

namespace hyp {

__device__ __forceinline__ void record_err2(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

__device__ __forceinline__ double block_max2(double v) {
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

__global__ void __launch_bounds__(kBlock) cell2_f64_kernel(const double* __restrict__ Q, int64_t n, Eos2 E,
                                                           double* __restrict__ F, double* __restrict__ smin,
                                                           double* __restrict__ smax, unsigned long long* lam_slot,
                                                           const double* t_now, double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    double q[30], f[30];
    for (int v = 0; v < 30; ++v) q[v] = Q[v * n + i];
    int st = flux2(E.e, q, f);
    double lo = 0.0, hi = 0.0;
    st |= speeds2(E.e, q, lo, hi);
    for (int v = 0; v < 30; ++v) F[v * n + i] = f[v];
    smin[i] = lo;
    smax[i] = hi;
    l = fmax(fabs(lo), fabs(hi));
    if (!(l <= 1.79e308)) st |= HYP_CELL_NONFINITE;
    if (st) record_err2(S, st, i);
  }
  const double m = block_max2(l);
  if (threadIdx.x == 0) atomicMax(lam_slot, (unsigned long long)__double_as_longlong(m));
}

constexpr int kFaceBlock = 64;

__global__ void __launch_bounds__(kFaceBlock) face2_f64_kernel(const double* __restrict__ Q, int64_t n, Eos2 E,
                                                               Quad6D qd, const double* __restrict__ F,
                                                               const double* __restrict__ smin,
                                                               const double* __restrict__ smax, double* __restrict__ DM,
                                                               double* __restrict__ DP, const double* t_now,
                                                               double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const int64_t f = (int64_t)blockIdx.x * kFaceBlock + threadIdx.x;  // face between cells f-1 and f
  if (f > n) return;
  const int64_t nf = n + 1;
  const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
  double dm[30], dp[30];
  if (L == R) {  // boundary face with a zero-gradient ghost: no jump, no fluctuation
    for (int v = 0; v < 30; ++v) dm[v] = dp[v] = 0.0;
  } else {
    double QL[30], QR[30], fl[30], fr[30];
    for (int v = 0; v < 30; ++v) {
      QL[v] = Q[v * n + L];
      QR[v] = Q[v * n + R];
      fl[v] = F[v * n + L];
      fr[v] = F[v * n + R];
    }
    int st = hll_face2(E.e, qd, QL, QR, fl, fr, smin[L], smax[R], dm, dp);
    if (st) record_err2(S, st, R);
  }
  for (int v = 0; v < 30; ++v) {
    DM[v * nf + f] = dm[v];
    DP[v * nf + f] = dp[v];
  }
}

__global__ void __launch_bounds__(kFaceBlock) face2_lxf_f64_kernel(
    const double* __restrict__ Q, int64_t n, Eos2 E, Quad6D lobatto, const double* __restrict__ F,
    const unsigned long long* lam_now, double cfl, double dx, double* __restrict__ FF, double* __restrict__ DM,
    double* __restrict__ DP, const double* t_now, double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const double lmax = __longlong_as_double((long long)*lam_now);
  const double lam = step_scalars(cfl, dx, lmax, true).lam_lxf;  // lambda = dx/dt (main.jl:223)
  const int64_t f = (int64_t)blockIdx.x * kFaceBlock + threadIdx.x;  // face between cells f-1 and f
  if (f > n) return;
  const int64_t nf = n + 1;
  const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
  double QL[30], QR[30], fl[30], fr[30], ff[30], dm[30], dp[30];
  for (int v = 0; v < 30; ++v) {
    QL[v] = Q[v * n + L];
    QR[v] = Q[v * n + R];
    fl[v] = F[v * n + L];
    fr[v] = F[v * n + R];
  }
  const int st = lxf_face2(E.e, lobatto, QL, QR, fl, fr, lam, ff, dm, dp);
  if (st) record_err2(S, st, R);
  for (int v = 0; v < 30; ++v) {
    FF[v * nf + f] = ff[v];
    DM[v * nf + f] = dm[v];
    DP[v * nf + f] = dp[v];
  }
}

__global__ void __launch_bounds__(kBlock) update2_f64_kernel(const double* __restrict__ Q, double* __restrict__ Qn,
                                                             int64_t n, const double* __restrict__ FF,
                                                             const double* __restrict__ DM,
                                                             const double* __restrict__ DP,
                                                             const unsigned long long* lam_in,
                                                             unsigned long long* lam_next, const double* t_in,
                                                             double* t_out, long long* steps, double t_end,
                                                             double cfl, double dx, int bc) {
  const double tn = *t_in;
  const bool active = tn < t_end;
  const double lmax = __longlong_as_double((long long)*lam_in);
  const StepScalars sc = step_scalars(cfl, dx, lmax, false);
  const double dt = sc.dt, dtdx = sc.dtdx;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *t_out = active ? tn + dt : tn;
    *lam_next = 0ull;
    if (active) *steps += 1;
  }
  if (!active) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  const int64_t nf = n + 1;
  if (bc == HYP_BC_FROZEN && (i == 0 || i == n - 1)) {
    for (int v = 0; v < 30; ++v) Qn[v * n + i] = Q[v * n + i];
    return;
  }
  for (int v = 0; v < 30; ++v) {
    // F_r = F_l = zeros(30) for hll (NumFluxes.jl:82), NF_r = D- of face i+1/2, NF_l = D+ of face i-1/2
    const double fr = FF ? FF[v * nf + i + 1] : 0.0, fl = FF ? FF[v * nf + i] : 0.0;
    const double nfr = DM[v * nf + i + 1], nfl = DP[v * nf + i];
    Qn[v * n + i] = Q[v * n + i] - dtdx * ((fr - fl) + (nfr + nfl));
  }
}

static inline unsigned grid_n(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

cudaError_t launch_cell2_f64(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end) {
  cell2_f64_kernel<<<grid_n(c->n, kBlock), kBlock, 0, c->stream>>>(c->Q[p], c->n, c->eos2, c->F, c->smin, c->smax,
                                                                    lam_slot, t_now, t_end, c->st);
  return cudaGetLastError();
}
cudaError_t launch_face2_f64(hyp_ctx* c, int p, double t_end) {
  if (c->cfg.flux == HYP_FLUX_LXF) {
    const double dx = c->cfg.x_length / (double)c->n;
    face2_lxf_f64_kernel<<<grid_n(c->n + 1, kFaceBlock), kFaceBlock, 0, c->stream>>>(
        c->Q[p], c->n, c->eos2, c->lobatto, c->F, &c->st->lam_bits[p], c->cfg.cfl, dx, c->FF, c->DM, c->DP,
        &c->st->t[p], t_end, c->st);
  } else {
    face2_f64_kernel<<<grid_n(c->n + 1, kFaceBlock), kFaceBlock, 0, c->stream>>>(
        c->Q[p], c->n, c->eos2, c->quad, c->F, c->smin, c->smax, c->DM, c->DP, &c->st->t[p], t_end, c->st);
  }
  return cudaGetLastError();
}
cudaError_t launch_update2_f64(hyp_ctx* c, int p, double t_end) {
  const double dx = c->cfg.x_length / (double)c->n;
  update2_f64_kernel<<<grid_n(c->n, kBlock), kBlock, 0, c->stream>>>(
      c->Q[p], c->Q[1 - p], c->n, c->FF, c->DM, c->DP, &c->st->lam_bits[p], &c->st->lam_bits[1 - p], &c->st->t[p],
      &c->st->t[1 - p], &c->st->steps, t_end, c->cfg.cfl, dx, c->cfg.bc);
  return cudaGetLastError();
}

// Gauss-Legendre 6 on [0,1]: Newton on P6 from Chebyshev-like guesses in long
// double, mapped (x + 1)/2, w/2, ascending (FastGaussQuadrature.gausslegendre(6)).
Quad6D gauss_legendre6() {
  long double xs[6], ws[6];
  for (int i = 0; i < 6; ++i) {
    long double x = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / 6.5L);
    long double dp = 1.0L;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1.0L, p1 = x;
      for (int k = 2; k <= 6; ++k) {
        long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = 6.0L * (x * p1 - p0) / (x * x - 1.0L);
      long double dx = p1 / dp;
      x -= dx;
      if (fabsl(dx) < 1e-30L) break;
    }
    {
      long double p0 = 1.0L, p1 = x;
      for (int k = 2; k <= 6; ++k) {
        long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = 6.0L * (x * p1 - p0) / (x * x - 1.0L);
    }
    xs[i] = x;
    ws[i] = 2.0L / ((1.0L - x * x) * dp * dp);
  }
  Quad6D q;
  for (int i = 0; i < 6; ++i) {
    const double nx = (double)xs[5 - i], nw = (double)ws[5 - i];
    q.x[i] = (nx + 1.0) / 2.0;
    q.w[i] = nw / 2.0;
  }
  return q;
}

// Gauss-Lobatto 6 on [0,1] (FastGaussQuadrature.gausslobatto(6), NumFluxes.jl:36):
// nodes -1, -a, -b, b, a, 1 with a, b = sqrt(1/3 +- 2 sqrt(7)/21), weights 1/15 at the
// ends and (14 -+ sqrt 7)/30 inside, mapped (x + 1)/2, w/2; evaluated in long double.
Quad6D gauss_lobatto6() {
  const long double s7 = sqrtl(7.0L);
  const long double a = sqrtl(1.0L / 3.0L + 2.0L * s7 / 21.0L), b = sqrtl(1.0L / 3.0L - 2.0L * s7 / 21.0L);
  const long double xs[6] = {-1.0L, -a, -b, b, a, 1.0L};
  const long double ws[6] = {1.0L / 15.0L, (14.0L - s7) / 30.0L, (14.0L + s7) / 30.0L,
                             (14.0L + s7) / 30.0L, (14.0L - s7) / 30.0L, 1.0L / 15.0L};
  Quad6D q;
  for (int i = 0; i < 6; ++i) {
    q.x[i] = ((double)xs[i] + 1.0) / 2.0;
    q.w[i] = (double)ws[i] / 2.0;
  }
  return q;
}

}  // namespace hyp
