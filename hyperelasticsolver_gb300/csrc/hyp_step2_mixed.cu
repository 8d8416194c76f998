// hyp_step2_mixed.cu -- two-phase step in mixed precision: the kernels of
// hyp_step2.cu with FP32 physics (hyp_physics_mph_mixed.cuh) and the state held
// as compensated (hi, lo) FP32 pairs of its 30 variables.
//
//   cell   : per cell, both phases' flux and wave-speed bounds from the (hi, lo)
//            state (float-float islands in cons2prim); block max of the wave speed
//            -> one atomicMax on the step's max-lambda slot (main.jl:204-212);
//   face   : per face, the path-conservative HLL fluctuations (NumFluxes.jl:85-132)
//            or the LxF face with D+- from the Gauss-Lobatto path integral
//            (NumFluxes.jl:25-60), in FP32;
//   update : dt = cfl dx / max lambda (FP64, for the time), t += dt, and per
//            updated cell the increment -dt/dx ((F_r - F_l) + (D-_{i+1/2} +
//            D+_{i-1/2})), dt/dx = cfl / max lambda in FP32, added to the (hi, lo)
//            pair with a two-sum (main.jl:30-60).
#include "hyp_internal.cuh"
#include "hyp_mixed_tile.cuh"
#include "hyp_physics_mph_mixed.cuh"
#include "hyp_physics_mph_pair.cuh"

namespace hyp {

__device__ __forceinline__ void record_err2m(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

// at most 85 registers: 3 blocks of 256 per SM (0.02-0.03 ms per step better at 2^22
// cells than 2 blocks at its natural 99)
template <int kDef>
__global__ void __launch_bounds__(kBlock, 3) cell2_mixed_kernel(const float* __restrict__ Qh,
                                                             const float* __restrict__ Ql, int64_t pitch, int64_t n,
                                                             Eos2M E, float* __restrict__ F, int64_t fpitch,
                                                             float* __restrict__ smin, float* __restrict__ smax,
                                                             unsigned long long* lam_slot, const double* t_now,
                                                             double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  float l = 0.0f;
  if (i < n) {
    float qh[30], ql[30], f[30];
    for (int v = 0; v < 30; ++v) {
      qh[v] = Qh[v * pitch + i];
      ql[v] = Ql[v * pitch + i];
    }
    float lo = 0.0f, hi = 0.0f;
    int st = cell2_mixed<kDef>(E, qh, ql, f, lo, hi);
    for (int v = 0; v < 30; ++v) F[v * fpitch + i] = f[v];
    smin[i] = lo;
    smax[i] = hi;
    l = fmaxf(fabsf(lo), fabsf(hi));
    if (!(l <= 3.0e38f)) st |= HYP_CELL_NONFINITE;
    if (st) record_err2m(S, st, i);
  }
  const float m = mixed_block_max<kBlock>(l);
  if (threadIdx.x == 0) atomicMax(lam_slot, (unsigned long long)__double_as_longlong((double)m));
}

constexpr int kFaceBlockM = 64;

__device__ __forceinline__ void load_face_states(const float* Qh, int64_t pitch, const float* F, int64_t fpitch,
                                                 int64_t L, int64_t R, float* QL, float* QR, float* fl, float* fr) {
  for (int v = 0; v < 30; ++v) {
    QL[v] = Qh[v * pitch + L];
    QR[v] = Qh[v * pitch + R];
    fl[v] = F[v * fpitch + L];
    fr[v] = F[v * fpitch + R];
  }
}

template <int kDef>
__global__ void __launch_bounds__(kFaceBlockM) face2_hll_mixed_kernel(
    const float* __restrict__ Qh, int64_t pitch, int64_t n, Eos2M E, Quad6F qd, const float* __restrict__ F,
    int64_t fpitch, const float* __restrict__ smin, const float* __restrict__ smax, float* __restrict__ DM,
    float* __restrict__ DP, const double* t_now, double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const int64_t f = (int64_t)blockIdx.x * kFaceBlockM + threadIdx.x;  // face between cells f-1 and f
  if (f > n) return;
  const int64_t nf = n + 1;
  const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
  float dm[30], dp[30];
  if (L == R) {  // boundary face with a zero-gradient ghost: no jump, no fluctuation
    for (int v = 0; v < 30; ++v) dm[v] = dp[v] = 0.0f;
  } else {
    float QL[30], QR[30], fl[30], fr[30];
    load_face_states(Qh, pitch, F, fpitch, L, R, QL, QR, fl, fr);
    for (int v = 0; v < 30; ++v) fr[v] -= fl[v];  // f(Q_r) - f(Q_l)
    const int st = hll_face2_m<kDef>(E, qd, QL, QR, fr, smin[L], smax[R], dm, dp);
    if (st) record_err2m(S, st, R);
  }
  for (int v = 0; v < 30; ++v) {
    DM[v * nf + f] = dm[v];
    DP[v * nf + f] = dp[v];
  }
}

// 128 registers (8 blocks of 64 per SM) with a small spill: 2.00 ms per step at 2^22
// cells against 2.36 ms at its natural 197 registers. The HLL face kernel, with three
// path integrals live, spills heavily under the same cap and stays uncapped (200
// registers for 10 warps per SM: 3.23 against 3.05 ms per step). At 168 registers
// (12 warps, no spills) this kernel takes 1.96 against 1.79 ms per step.
template <int kDef>
__global__ void __launch_bounds__(kFaceBlockM, 8) face2_lxf_mixed_kernel(
    const float* __restrict__ Qh, int64_t pitch, int64_t n, Eos2M E, Quad6F lobatto, const float* __restrict__ F,
    int64_t fpitch, const unsigned long long* lam_now, double cfl, float* __restrict__ FF,
    float* __restrict__ DM, float* __restrict__ DP, const double* t_now, double t_end, DevState* S) {
  if (!(*t_now < t_end)) return;
  const int64_t f = (int64_t)blockIdx.x * kFaceBlockM + threadIdx.x;
  if (f > n) return;
  const int64_t nf = n + 1;
  const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
  const double lmax = __longlong_as_double((long long)*lam_now);
  const float lam = (float)lmax / (float)cfl;  // lambda = dx/dt = lmax/cfl (main.jl:223), in FP32
  float QL[30], QR[30], fl[30], fr[30], ff_[30], dm[30], dp[30];
  load_face_states(Qh, pitch, F, fpitch, L, R, QL, QR, fl, fr);
  const int st = lxf_face2_m<kDef>(E, lobatto, QL, QR, fl, fr, lam, ff_, dm, dp);
  if (st) record_err2m(S, st, R);
  for (int v = 0; v < 30; ++v) {
    FF[v * nf + f] = ff_[v];
    DM[v * nf + f] = dm[v];
    DP[v * nf + f] = dp[v];
  }
}

// The face kernels with the phases as the lanes of packed FP32 pairs
// (hyp_physics_mph_pair.cuh): pair k holds variable k of phase 1 and phase 2.
__device__ __forceinline__ void load_face_pairs(const float* Qh, int64_t pitch, const float* F, int64_t fpitch,
                                                int64_t L, int64_t R, float2* QL, float2* QR, float2* fl,
                                                float2* fr) {
  for (int k = 0; k < 15; ++k) {
    QL[k] = make_float2(Qh[k * pitch + L], Qh[(15 + k) * pitch + L]);
    QR[k] = make_float2(Qh[k * pitch + R], Qh[(15 + k) * pitch + R]);
    fl[k] = make_float2(F[k * fpitch + L], F[(15 + k) * fpitch + L]);
    fr[k] = make_float2(F[k * fpitch + R], F[(15 + k) * fpitch + R]);
  }
}

__device__ __forceinline__ void store_face_pairs(float* D, int64_t nf, int64_t f, const float2* d) {
  for (int k = 0; k < 15; ++k) {
    D[k * nf + f] = d[k].x;
    D[(15 + k) * nf + f] = d[k].y;
  }
}

// The HLL faces on packed pairs (hll_face2_pair) with the update fused in: the
// default two-phase mixed HLL step (HYP_MIXED_PAIR). Block b computes faces
// 63 b .. 63 b + 63 (one per thread; the last is computed again by block b + 1 as its
// first) and updates cells 63 b .. 63 b + 62: cell i from the D+ of its left face i
// (this thread's) and the D- of its right face i + 1 (the next thread's, through shared
// memory), with update2_mixed_kernel's dt/dx, FP32 expression and two-sum. D+- never
// go to memory; the face work is bound by FP32 issue, and the update's loads and
// stores of the (hi, lo) state run under it instead of in a kernel of their own.
constexpr int kFusedCells = kFaceBlockM - 1;

template <int kDef>
__global__ void __launch_bounds__(kFaceBlockM) face_update2_hll_pair_kernel(
    const float* __restrict__ Qh, const float* __restrict__ Ql, float* __restrict__ Qh_out,
    float* __restrict__ Ql_out, int64_t pitch, int64_t n, Eos2M E, EosPair ep, Quad6F qd,
    const float* __restrict__ F, int64_t fpitch, const float* __restrict__ smin, const float* __restrict__ smax,
    const unsigned long long* lam_in, unsigned long long* lam_next, const double* t_in, double* t_out,
    long long* steps, double t_end, double cfl, float cfl_f, double dx, int bc, DevState* S) {
  __shared__ float2 sDM[15][kFaceBlockM];  // D- of face 63 b + t, column t
  double tn = 0.0, lmax = 0.0;
  int act = 0;
  float dtdx_0 = 0.0f;
  if ((threadIdx.x & 31) == 0) {
    tn = *t_in;
    act = tn < t_end;
    lmax = __longlong_as_double((long long)*lam_in);
    dtdx_0 = cfl_f / (float)lmax;
  }
  const bool active = __shfl_sync(0xffffffffu, act, 0) != 0;  // the same in every warp
  const float dtdx = __shfl_sync(0xffffffffu, dtdx_0, 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double dt = (cfl * dx) / lmax;
    *t_out = active ? tn + dt : tn;
    *lam_next = 0ull;
    if (active) *steps += 1;
  }
  if (!active) return;  // the whole grid
  const int64_t f = (int64_t)blockIdx.x * kFusedCells + threadIdx.x;  // face between cells f-1 and f
  float2 dm[15], dp[15];
  if (f <= n) {
    const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
    if (L == R) {  // boundary face with a zero-gradient ghost: no jump, no fluctuation
      for (int k = 0; k < 15; ++k) dm[k] = dp[k] = f2s(0.0f);
    } else {
      float2 QL[15], QR[15], fl[15], fr[15];
      load_face_pairs(Qh, pitch, F, fpitch, L, R, QL, QR, fl, fr);
      for (int k = 0; k < 15; ++k) fr[k] = f2sub(fr[k], fl[k]);  // f(Q_r) - f(Q_l)
      const int st = hll_face2_pair<kDef>(E, ep, qd, QL, QR, fr, smin[L], smax[R], dm, dp);
      if (st) record_err2m(S, st, R);
    }
    for (int k = 0; k < 15; ++k) sDM[k][threadIdx.x] = dm[k];
  }
  __syncthreads();
  const int64_t i = f;  // the cell right of this thread's face
  if (threadIdx.x >= kFusedCells || i >= n) return;
  const bool frozen = bc == HYP_BC_FROZEN && (i == 0 || i == n - 1);
#pragma unroll
  for (int k = 0; k < 15; ++k) {  // variables k and 15 + k: the pair's lanes
    const float2 m2 = sDM[k][threadIdx.x + 1];
#pragma unroll
    for (int ph = 0; ph < 2; ++ph) {
      const int64_t o = (int64_t)(15 * ph + k) * pitch + i;
      float h = Qh[o], l = Ql[o];
      if (!frozen) {
        const float dmv = ph ? m2.y : m2.x, dpv = ph ? dp[k].y : dp[k].x;
        const float delta = -dtdx * (0.0f + (dmv + dpv));  // update2_mixed_kernel's form, F_r - F_l = 0
        const ff q = ff_add_f(ff{h, l}, delta);
        h = q.hi;
        l = q.lo;
      }
      Qh_out[o] = h;
      Ql_out[o] = l;
    }
  }
}

// The LxF pair faces (lxf_face2_pair) with the update fused in, as
// face_update2_hll_pair_kernel: cell i from F_{i+1/2} - F_{i-1/2} and D-_{i+1/2} +
// D+_{i-1/2}, the right face's F and D (D- = D+ for LxF) through shared memory; at most
// 168 registers (6 blocks of 64 per SM): 1.00 against 1.36 ms per LxF step at 2^22
// cells with the face and update kernels apart.
template <int kDef>
__global__ void __launch_bounds__(kFaceBlockM, 6) face_update2_lxf_pair_kernel(
    const float* __restrict__ Qh, const float* __restrict__ Ql, float* __restrict__ Qh_out,
    float* __restrict__ Ql_out, int64_t pitch, int64_t n, EosPair ep, Quad6F lobatto, const float* __restrict__ F,
    int64_t fpitch, const unsigned long long* lam_in, unsigned long long* lam_next, const double* t_in,
    double* t_out, long long* steps, double t_end, double cfl, float cfl_f, double dx, int bc, DevState* S) {
  __shared__ float2 sFF[15][kFaceBlockM], sD[15][kFaceBlockM];
  double tn = 0.0, lmax = 0.0;
  int act = 0;
  float dtdx_0 = 0.0f;
  if ((threadIdx.x & 31) == 0) {
    tn = *t_in;
    act = tn < t_end;
    lmax = __longlong_as_double((long long)*lam_in);
    dtdx_0 = cfl_f / (float)lmax;
  }
  const bool active = __shfl_sync(0xffffffffu, act, 0) != 0;
  const float dtdx = __shfl_sync(0xffffffffu, dtdx_0, 0);
  lmax = __shfl_sync(0xffffffffu, lmax, 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double dt = (cfl * dx) / lmax;
    *t_out = active ? tn + dt : tn;
    *lam_next = 0ull;
    if (active) *steps += 1;
  }
  if (!active) return;
  const int64_t f = (int64_t)blockIdx.x * kFusedCells + threadIdx.x;
  float2 ff_[15], dm[15], dp[15];
  if (f <= n) {
    const int64_t L = f > 0 ? f - 1 : 0, R = f < n ? f : n - 1;
    const float lam = (float)lmax / (float)cfl;  // lambda = dx/dt = lmax/cfl (main.jl:223), in FP32
    float2 QL[15], QR[15], fl[15], fr[15];
    load_face_pairs(Qh, pitch, F, fpitch, L, R, QL, QR, fl, fr);
    const int st = lxf_face2_pair<kDef>(ep, lobatto, QL, QR, fl, fr, lam, ff_, dm, dp);
    if (st) record_err2m(S, st, R);
    for (int k = 0; k < 15; ++k) {
      sFF[k][threadIdx.x] = ff_[k];
      sD[k][threadIdx.x] = dm[k];
    }
  }
  __syncthreads();
  const int64_t i = f;
  if (threadIdx.x >= kFusedCells || i >= n) return;
  const bool frozen = bc == HYP_BC_FROZEN && (i == 0 || i == n - 1);
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    const float2 fr2 = sFF[k][threadIdx.x + 1], dm2 = sD[k][threadIdx.x + 1];
#pragma unroll
    for (int ph = 0; ph < 2; ++ph) {
      const int64_t o = (int64_t)(15 * ph + k) * pitch + i;
      float h = Qh[o], l = Ql[o];
      if (!frozen) {
        const float frv = ph ? fr2.y : fr2.x, flv = ph ? ff_[k].y : ff_[k].x;
        const float dmv = ph ? dm2.y : dm2.x, dpv = ph ? dp[k].y : dp[k].x;
        const float delta = -dtdx * ((frv - flv) + (dmv + dpv));  // update2_mixed_kernel's form
        const ff q = ff_add_f(ff{h, l}, delta);
        h = q.hi;
        l = q.lo;
      }
      Qh_out[o] = h;
      Ql_out[o] = l;
    }
  }
}

__global__ void __launch_bounds__(kBlock) update2_mixed_kernel(
    const float* __restrict__ Qh, const float* __restrict__ Ql, float* __restrict__ Qh_out, float* __restrict__ Ql_out,
    int64_t pitch, int64_t n, const float* __restrict__ FF, const float* __restrict__ DM, const float* __restrict__ DP,
    const unsigned long long* lam_in, unsigned long long* lam_next, const double* t_in, double* t_out,
    long long* steps, double t_end, double cfl, float cfl_f, double dx, int bc) {
  // lane 0 reads the control and broadcasts: dt/dx = cfl / lmax in FP32, cfl_f = cfl
  // rounded on the host (two FP64 divisions in every thread cost this memory-bound
  // kernel a quarter of its time: 0.65 -> 0.49 ms at 2^22 cells; the broadcast of
  // the FP64 compare, 0.49 -> 0.48 ms)
  double tn = 0.0, lmax = 0.0;
  int act = 0;
  float dtdx_0 = 0.0f;
  if ((threadIdx.x & 31) == 0) {
    tn = *t_in;
    act = tn < t_end;
    lmax = __longlong_as_double((long long)*lam_in);
    dtdx_0 = cfl_f / (float)lmax;
  }
  const bool active = __shfl_sync(0xffffffffu, act, 0) != 0;
  const float dtdx = __shfl_sync(0xffffffffu, dtdx_0, 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double dt = (cfl * dx) / lmax;
    *t_out = active ? tn + dt : tn;
    *lam_next = 0ull;
    if (active) *steps += 1;
  }
  if (!active) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  const int64_t nf = n + 1;
  const bool frozen = bc == HYP_BC_FROZEN && (i == 0 || i == n - 1);
  // one variable at a time: unrolled by 5 or 10 the kernel measured 0.66 / 0.81
  // against 0.49 ms at 2^22 cells (more row streams in flight at once)
#pragma unroll 1
  for (int v = 0; v < 30; ++v) {
    float h = Qh[v * pitch + i], l = Ql[v * pitch + i];
    if (!frozen) {
      const float fr = FF ? FF[v * nf + i + 1] : 0.0f, fl = FF ? FF[v * nf + i] : 0.0f;
      const float delta = -dtdx * ((fr - fl) + (DM[v * nf + i + 1] + DP[v * nf + i]));
      const ff q = ff_add_f(ff{h, l}, delta);
      h = q.hi;
      l = q.lo;
    }
    Qh_out[v * pitch + i] = h;
    Ql_out[v * pitch + i] = l;
  }
}

static inline unsigned grid_m(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

static Quad6F to_f(const Quad6D& q) {
  Quad6F r;
  for (int i = 0; i < 6; ++i) {
    r.x[i] = (float)q.x[i];
    r.w[i] = (float)q.w[i];
  }
  return r;
}

static Eos2M eos2m(const hyp_ctx* c) {
  Eos2M E;
  E.m[0] = make_eos_mixed(c->eos[0]);
  E.m[1] = make_eos_mixed(c->eos[1]);
  return E;
}

// Both phases with the reference's default exponents: the kernels compiled with the
// integer powers only (kDef = 1), whose smaller code the face kernel's instruction
// fetch feels (3.26 -> 3.05 ms per two-phase HLL step at 2^22 cells); else the
// general form (kDef = -1).
static bool default_exps(const hyp_ctx* c) { return c->eos[0].default_exp && c->eos[1].default_exp; }

cudaError_t launch_cell2_mixed(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end) {
  auto kern = default_exps(c) ? cell2_mixed_kernel<1> : cell2_mixed_kernel<-1>;
  kern<<<grid_m(c->n, kBlock), kBlock, 0, c->stream>>>(c->Qh[p], c->Ql[p], c->mpitch, c->n, eos2m(c), c->F32, c->n,
                                                        c->smin32, c->smax32, lam_slot, t_now, t_end, c->st);
  return cudaGetLastError();
}

cudaError_t launch_face2_mixed(hyp_ctx* c, int p, double t_end) {
  const bool def = default_exps(c), pair = c->mixed_kind == HYP_MIXED_PAIR;
  const unsigned grid = grid_m(c->n + 1, kFaceBlockM);
  if (pair) return cudaErrorInvalidValue;  // the pair faces run with the update (launch_face_update2_mixed)
  if (c->cfg.flux == HYP_FLUX_LXF) {
    auto kern = def ? face2_lxf_mixed_kernel<1> : face2_lxf_mixed_kernel<-1>;
    kern<<<grid, kFaceBlockM, 0, c->stream>>>(c->Qh[p], c->mpitch, c->n, eos2m(c), to_f(c->lobatto), c->F32, c->n,
                                              &c->st->lam_bits[p], c->cfg.cfl, c->FF32, c->DM32, c->DP32,
                                              &c->st->t[p], t_end, c->st);
  } else {
    auto kern = def ? face2_hll_mixed_kernel<1> : face2_hll_mixed_kernel<-1>;
    kern<<<grid, kFaceBlockM, 0, c->stream>>>(c->Qh[p], c->mpitch, c->n, eos2m(c), to_f(c->quad), c->F32, c->n,
                                              c->smin32, c->smax32, c->DM32, c->DP32, &c->st->t[p], t_end, c->st);
  }
  return cudaGetLastError();
}

// Both fluxes' pair faces run with the update; the scalar faces (HYP_MIXED_TILE) apart.
bool fused_face_update2_mixed(const hyp_ctx* c) { return c->mixed_kind == HYP_MIXED_PAIR; }

cudaError_t launch_face_update2_mixed(hyp_ctx* c, int p, double t_end) {
  const double dx = c->cfg.x_length / (double)c->n;
  if (c->cfg.flux == HYP_FLUX_LXF) {
    auto kern = default_exps(c) ? face_update2_lxf_pair_kernel<1> : face_update2_lxf_pair_kernel<-1>;
    kern<<<grid_m(c->n, kFusedCells), kFaceBlockM, 0, c->stream>>>(
        c->Qh[p], c->Ql[p], c->Qh[1 - p], c->Ql[1 - p], c->mpitch, c->n, make_eos_pair(eos2m(c)), to_f(c->lobatto),
        c->F32, c->n, &c->st->lam_bits[p], &c->st->lam_bits[1 - p], &c->st->t[p], &c->st->t[1 - p], &c->st->steps,
        t_end, c->cfg.cfl, (float)c->cfg.cfl, dx, c->cfg.bc, c->st);
    return cudaGetLastError();
  }
  auto kern = default_exps(c) ? face_update2_hll_pair_kernel<1> : face_update2_hll_pair_kernel<-1>;
  const Eos2M E = eos2m(c);
  kern<<<grid_m(c->n, kFusedCells), kFaceBlockM, 0, c->stream>>>(
      c->Qh[p], c->Ql[p], c->Qh[1 - p], c->Ql[1 - p], c->mpitch, c->n, E, make_eos_pair(E), to_f(c->quad), c->F32,
      c->n, c->smin32, c->smax32, &c->st->lam_bits[p], &c->st->lam_bits[1 - p], &c->st->t[p], &c->st->t[1 - p],
      &c->st->steps, t_end, c->cfg.cfl, (float)c->cfg.cfl, dx, c->cfg.bc, c->st);
  return cudaGetLastError();
}

cudaError_t launch_update2_mixed(hyp_ctx* c, int p, double t_end) {
  const double dx = c->cfg.x_length / (double)c->n;
  update2_mixed_kernel<<<grid_m(c->n, kBlock), kBlock, 0, c->stream>>>(
      c->Qh[p], c->Ql[p], c->Qh[1 - p], c->Ql[1 - p], c->mpitch, c->n, c->FF32, c->DM32, c->DP32,
      &c->st->lam_bits[p], &c->st->lam_bits[1 - p], &c->st->t[p], &c->st->t[1 - p], &c->st->steps, t_end,
      c->cfg.cfl, (float)c->cfg.cfl, dx, c->cfg.bc);
  return cudaGetLastError();
}

}  // namespace hyp
