// hyp_adjoint.cu -- discrete adjoint of the single-phase FP64 Rusanov step
// (main.jl:202-227 with the Rusanov face rule of main.jl:45-48) with
// checkpointing, and a density-misfit loss.
//
// Forward step n (as hyp_step1.cu computes it):
//   r_n = dt/dx = (cfl dx / max_i lambda_i) / dx,
//   F_{i+1/2} = (f_i + f_{i+1})/2 - lambda_{i+1/2} (Q_{i+1} - Q_i)/2,
//               lambda_{i+1/2} = lambda_i if lambda_i > lambda_{i+1} else lambda_{i+1},
//   Q'_i = Q_i - r_n (F_{i+1/2} - F_{i-1/2})   for updated cells (all cells with
//          transmissive ends; frozen ends copy, main.jl:219-220).
// Its adjoint, given Qb' = dL/dQ_{n+1}:
//   Fb_{i+1/2} = r_n (Qb'_{i+1} [i+1 updated] - Qb'_i [i updated]),
//   fb_i       = (Fb_{i-1/2} + Fb_{i+1/2}) / 2      (a ghost face counts fully),
//   lambdab    = -(Fb . (Q_R - Q_L)) / 2 for the cell whose lambda the face took,
//   Qb_i       = Qb'_i + lambda_{i+1/2} Fb_{i+1/2}/2 - lambda_{i-1/2} Fb_{i-1/2}/2
//                + (df/dq)^T fb_i + (dlambda/dq) lambdab_i          (cell_vjp),
//   rb_n       = -sum_{updated i} Qb'_i . (F_{i+1/2} - F_{i-1/2}),
//   lambdab of the arg-max cell (smallest index among equal maxima) += -rb_n r_n / max lambda.
// Two kernels per adjoint step: adj_dtdx (streaming: the partial sums of rb_n and the
// arg-max cell) and adj_cell (face terms + cell_vjp; every block first sums the
// partials of rb_n in a fixed order, so the result does not depend on scheduling).
// The EOS-modulus adjoints are summed per block into a per-block accumulator that
// the same block owns in every step; the host adds the blocks in index order.
//
// Checkpointing: hyp_adjoint_record runs the forward steps with the FP64 step
// kernels of hyp_step1.cu and keeps the state every K steps. hyp_adjoint walks the
// segments backwards: it reruns a segment from its checkpoint with the same
// kernels (bit-identical states, fluxes and wave speeds), keeping its K states,
// fluxes and wave speeds, then takes the K adjoint steps.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>
#include "hyp_internal.cuh"
#include "hyp_adjoint.cuh"

namespace hyp {

constexpr int kAdjBlock = 128;
constexpr int kPartBlocks = 1024;  // upper bound of the adj_dtdx grid (partial sums of rb)

struct AdjTape {
  int K = 0;            // checkpoint interval
  int n_steps = 0;      // recorded steps
  long long steps_at_end = -1;  // context step count the recording ended at
  int n_ckpt = 0;
  double* ckpt = nullptr;     // [n_ckpt][14][n]
  double* seg_Q = nullptr;    // [K][14][n]
  double* seg_F = nullptr;    // [K][11][n]
  double* seg_lam = nullptr;  // [K][n]
  unsigned long long* seg_lmax = nullptr;  // [K + 1]
  double* seg_t = nullptr;    // [K + 1]
  long long* seg_steps = nullptr;
  double* Qb[2] = {nullptr, nullptr};
  double* rpart = nullptr;    // [kPartBlocks]
  int* amax = nullptr;        // [2]
  double* eacc = nullptr;     // [2][adj_cell grid]
  double* misfit = nullptr;   // [n] target density / scratch
  double* mpart = nullptr;    // [kPartBlocks] loss partial sums
  int part_grid = 0, cell_grid = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float ms_record = 0.f, ms_recompute = 0.f, ms_adjoint = 0.f;
};

void free_tape(hyp_ctx* c) {
  AdjTape* t = c->tape;
  if (!t) return;
  cudaFree(t->ckpt);
  cudaFree(t->seg_Q);
  cudaFree(t->seg_F);
  cudaFree(t->seg_lam);
  cudaFree(t->seg_lmax);
  cudaFree(t->seg_t);
  cudaFree(t->seg_steps);
  cudaFree(t->Qb[0]);
  cudaFree(t->Qb[1]);
  cudaFree(t->rpart);
  cudaFree(t->amax);
  cudaFree(t->eacc);
  cudaFree(t->misfit);
  cudaFree(t->mpart);
  for (auto& e : t->ev)
    if (e) cudaEventDestroy(e);
  delete t;
  c->tape = nullptr;
}

template <int B>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < B / 32; ++k) r += sh[k];
  return r;  // valid in thread 0
}

struct AdjArgs {
  const double* Q;     // Q_n [14][n]
  const double* Qn;    // Q_{n+1} [14][n] (the step's result, kept by the recompute)
  const double* F;     // fluxes of Q_n [11][n]
  const double* lam;   // wave speeds of Q_n [n]
  const unsigned long long* lmax;  // max wave speed of Q_n (bits)
  const double* Qb1;   // dL/dQ_{n+1}
  double* Qb0;         // dL/dQ_n
  double* rpart;
  int* amax_rd;        // arg-max cell of this step
  int* amax_clr;       // the slot the next (earlier) step uses, reset here
  double* eacc;
  int64_t n;
  double cfl, dx;
  int trans;
  int part_grid;
};

__device__ __forceinline__ bool updated(int64_t i, int64_t n, int trans) { return trans || (i > 0 && i < n - 1); }

__device__ __forceinline__ double face_lambda(double la, double lb) { return la > lb ? la : lb; }


// Partial sums of r * rb_n, where rb_n = -sum_{updated i} Qb'_i . (F_{i+1/2} - F_{i-1/2})
// and, for an updated cell, F_{i+1/2} - F_{i-1/2} = (Q_i - Q'_i) / r with Q' the step's
// result: r rb_n = sum Qb'_i . (Q'_i - Q_i), a 14-term dot product per cell. Also the
// arg-max cell (smallest index whose wave speed equals the step's max), one atomicMin
// per block.
__global__ void __launch_bounds__(256) adj_dtdx_kernel(AdjArgs g) {
  __shared__ double sh[8];
  __shared__ int shi[8];
  const int64_t n = g.n;
  const double lmax = __longlong_as_double((long long)*g.lmax);
  double acc = 0.0;
  int imin = INT_MAX;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (g.lam[i] == lmax && (int)i < imin) imin = (int)i;
    if (!updated(i, n, g.trans)) continue;
    double s = 0.0;
    for (int v = 0; v < 14; ++v) s += g.Qb1[v * n + i] * (g.Qn[v * n + i] - g.Q[v * n + i]);
    acc += s;
  }
  for (int o = 16; o > 0; o >>= 1) imin = min(imin, __shfl_xor_sync(0xffffffffu, imin, o));
  if ((threadIdx.x & 31) == 0) shi[threadIdx.x >> 5] = imin;
  const double b = block_sum<256>(acc, sh);  // its barriers also publish shi
  if (threadIdx.x == 0) {
    g.rpart[blockIdx.x] = b;
    int m = INT_MAX;
    for (int w = 0; w < 8; ++w) m = min(m, shi[w]);
    if (m != INT_MAX) atomicMin(g.amax_rd, m);
  }
}

__global__ void __launch_bounds__(kAdjBlock) adj_cell_kernel(AdjArgs g, EosC e) {
  __shared__ double sh[kAdjBlock / 32];
  __shared__ double s_lamb_max;
  const int64_t n = g.n;
  const double lmax = __longlong_as_double((long long)*g.lmax);
  const double r = step_scalars(g.cfl, g.dx, lmax, false).dtdx;  // dt/dx of the forward step
  if (threadIdx.x < 32) {  // rb_n: the partial sums in a fixed order
    double s = 0.0;
    for (int k = threadIdx.x; k < g.part_grid; k += 32) s += g.rpart[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    // the partials sum to r rb_n; d r / d lmax = -r / lmax, so dL/d lmax = -(r rb_n) / lmax
    if (threadIdx.x == 0) s_lamb_max = -s / lmax;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *g.amax_clr = INT_MAX;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kAdjBlock + threadIdx.x;
  EosBar eb{0.0, 0.0};
  if (i < n) {
    const int64_t il = i > 0 ? i - 1 : 0, ir = i < n - 1 ? i + 1 : n - 1;
    const bool ui = updated(i, n, g.trans);
    const bool ul = il != i && updated(il, n, g.trans), ur = ir != i && updated(ir, n, g.trans);
    const double li = g.lam[i], ll = g.lam[il], lr = g.lam[ir];
    const double lL = face_lambda(ll, li), lR = face_lambda(li, lr);
    const bool takeL = !(ll > li);  // the left face took lambda_i
    const bool takeR = li > lr;     // the right face took lambda_i
    double q[14], qb[14], fb[14];
    double lamb = (int)i == *g.amax_rd ? s_lamb_max : 0.0;
    double dL = 0.0, dR = 0.0;
#pragma unroll
    for (int v = 0; v < 14; ++v) {
      const double qc = g.Q[v * n + i];
      q[v] = qc;
      const double bc = g.Qb1[v * n + i];
      const double FbL = r * ((ui ? bc : 0.0) - (ul ? g.Qb1[v * n + il] : 0.0));
      const double FbR = r * ((ur ? g.Qb1[v * n + ir] : 0.0) - (ui ? bc : 0.0));
      double acc = bc, f = 0.0;
      if (il != i) {
        f += 0.5 * FbL;
        acc -= 0.5 * lL * FbL;
        dL += FbL * (qc - g.Q[v * n + il]);
      } else {
        f += FbL;  // ghost face (Q, Q): flux f(Q), no dissipation
      }
      if (ir != i) {
        f += 0.5 * FbR;
        acc += 0.5 * lR * FbR;
        dR += FbR * (g.Q[v * n + ir] - qc);
      } else {
        f += FbR;
      }
      qb[v] = acc;
      fb[v] = f;
    }
    if (il != i && takeL) lamb -= 0.5 * dL;
    if (ir != i && takeR) lamb -= 0.5 * dR;
    bool any = lamb != 0.0;
#pragma unroll
    for (int v = 0; v < 14; ++v) any |= fb[v] != 0.0;
    // where the face adjoints vanish (a region where the adjoint field is constant) the
    // VJP adds exact zeros: skip it
    if (any) cell_vjp(e, q, fb, lamb, qb, eb);
#pragma unroll
    for (int v = 0; v < 14; ++v) g.Qb0[v * n + i] = qb[v];
  }
  const double b0 = block_sum<kAdjBlock>(eb.b0sq, sh);
  const double k0 = block_sum<kAdjBlock>(eb.k0, sh);
  if (threadIdx.x == 0) {
    g.eacc[2 * blockIdx.x] += b0;
    g.eacc[2 * blockIdx.x + 1] += k0;
  }
}

// L = 1/2 sum (rho_i - target_i)^2 with rho_i = sqrt(det(rho A)_i / rho0)
// (HyperelasticityMPh.jl:114, the density save_data writes, main.jl:71), and dL/dQ.
__global__ void __launch_bounds__(256) misfit_kernel(const double* __restrict__ Q, const double* __restrict__ target,
                                                     int64_t n, double inv_rho0, double* __restrict__ Qb,
                                                     double* __restrict__ part) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double m[9];
    for (int t = 0; t < 9; ++t) m[t] = Q[(5 + t) * n + i];
    const double d = det3(m);
    const double rho = sqrt(d * inv_rho0);
    const double res = rho - target[i];
    acc += 0.5 * res * res;
    if (Qb) {
      const double db = res * inv_rho0 / (2.0 * rho);
      for (int v = 0; v < 5; ++v) Qb[v * n + i] = 0.0;
      Qb[5 * n + i] = db * (m[4] * m[8] - m[5] * m[7]);
      Qb[6 * n + i] = db * (m[5] * m[6] - m[3] * m[8]);
      Qb[7 * n + i] = db * (m[3] * m[7] - m[4] * m[6]);
      Qb[8 * n + i] = db * (m[2] * m[7] - m[1] * m[8]);
      Qb[9 * n + i] = db * (m[0] * m[8] - m[2] * m[6]);
      Qb[10 * n + i] = db * (m[1] * m[6] - m[0] * m[7]);
      Qb[11 * n + i] = db * (m[1] * m[5] - m[2] * m[4]);
      Qb[12 * n + i] = db * (m[2] * m[3] - m[0] * m[5]);
      Qb[13 * n + i] = db * (m[0] * m[4] - m[1] * m[3]);
    }
  }
  const double b = block_sum<256>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = b;
}

__global__ void prim2cons_vjp_kernel(EosC e, const double* P, const double* Qb, double* Pb, double* ebar, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[14], qb[14], pb[14];
  for (int v = 0; v < 14; ++v) {
    p[v] = P[v * n + i];
    qb[v] = Qb[v * n + i];
    pb[v] = 0.0;
  }
  EosBar b{0.0, 0.0};
  prim2cons_vjp(e, p, qb, pb, b);
  for (int v = 0; v < 14; ++v) Pb[v * n + i] = pb[v];
  ebar[2 * i] = b.b0sq;
  ebar[2 * i + 1] = b.k0;
}

}  // namespace hyp

using namespace hyp;

#define ACK(call)                                                                            \
  do {                                                                                       \
    cudaError_t _e = (call);                                                                 \
    if (_e != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

static int adjoint_supported(hyp_ctx* c) {
  if (c->cfg.model != HYP_MODEL_SINGLE || c->cfg.precision != HYP_PREC_FP64 || c->cfg.flux != HYP_FLUX_RUSANOV)
    return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "the adjoint covers the single-phase FP64 Rusanov step");
  return HYP_OK;
}

static int ensure_tape(hyp_ctx* c, int n_steps, int K) {
  AdjTape* t = c->tape;
  const int n_ckpt = (n_steps + K - 1) / K;
  if (t && t->K == K && t->n_ckpt >= n_ckpt) return HYP_OK;
  free_tape(c);
  t = c->tape = new AdjTape();
  const size_t n = (size_t)c->n;
  t->K = K;
  t->n_ckpt = n_ckpt;
  t->part_grid = (int)std::min<int64_t>(kPartBlocks, (c->n + 255) / 256);
  t->cell_grid = (int)((c->n + kAdjBlock - 1) / kAdjBlock);
  ACK(cudaMalloc(&t->ckpt, (size_t)n_ckpt * 14 * n * sizeof(double)));
  ACK(cudaMalloc(&t->seg_Q, (size_t)K * 14 * n * sizeof(double)));
  ACK(cudaMalloc(&t->seg_F, (size_t)K * kNFlux1 * n * sizeof(double)));
  ACK(cudaMalloc(&t->seg_lam, (size_t)K * n * sizeof(double)));
  ACK(cudaMalloc(&t->seg_lmax, (size_t)(K + 1) * sizeof(unsigned long long)));
  ACK(cudaMalloc(&t->seg_t, (size_t)(K + 1) * sizeof(double)));
  ACK(cudaMalloc(&t->seg_steps, sizeof(long long)));
  for (int p = 0; p < 2; ++p) ACK(cudaMalloc(&t->Qb[p], 14 * n * sizeof(double)));
  ACK(cudaMalloc(&t->rpart, kPartBlocks * sizeof(double)));
  ACK(cudaMalloc(&t->amax, 2 * sizeof(int)));
  ACK(cudaMalloc(&t->eacc, (size_t)2 * t->cell_grid * sizeof(double)));
  for (auto& e : t->ev) ACK(cudaEventCreate(&e));
  return HYP_OK;
}

extern "C" int hyp_adjoint_record(hyp_ctx* c, int n_steps, int ckpt_every, double* t_out) {
  if (!c) return HYP_ERR_INVALID;
  int rc = adjoint_supported(c);
  if (rc != HYP_OK) return rc;
  if (n_steps <= 0 || ckpt_every <= 0) return ctx_set_err(c, HYP_ERR_INVALID, "hyp_adjoint_record: n_steps and ckpt_every must be positive");
  ACK(cudaSetDevice(c->device));
  if ((rc = ensure_tape(c, n_steps, ckpt_every)) != HYP_OK) return rc;
  AdjTape* t = c->tape;
  t->n_steps = n_steps;
  t->steps_at_end = -1;
  const size_t bytes = (size_t)14 * c->n * sizeof(double);
  const double inf = INFINITY;
  ACK(cudaEventRecord(t->ev[0], c->stream));
  for (int s = 0; s < n_steps; ++s) {
    const long long k = c->steps_host + s;
    const int p = (int)(k & 1);
    if (s % ckpt_every == 0)
      ACK(cudaMemcpyAsync(t->ckpt + (size_t)(s / ckpt_every) * 14 * c->n, c->Q[p], bytes, cudaMemcpyDeviceToDevice,
                          c->stream));
    ACK(launch_cell1_f64(c, p, &c->st->lam_bits[p], &c->st->t[p], inf));
    ACK(launch_update1_f64(c, p, inf));
  }
  ACK(cudaEventRecord(t->ev[1], c->stream));
  if ((rc = ctx_sync_state(c)) != HYP_OK) return rc;
  ACK(cudaEventElapsedTime(&t->ms_record, t->ev[0], t->ev[1]));
  const long long active = c->st_host->steps - c->steps_host;
  c->cur = (int)((c->cur + active) & 1);
  c->steps_host = c->st_host->steps;
  c->t_host = c->st_host->t[c->cur];
  if (t_out) *t_out = c->t_host;
  if ((rc = ctx_check_cell_error(c)) != HYP_OK) return rc;
  t->steps_at_end = c->steps_host;
  return HYP_OK;
}

extern "C" int hyp_adjoint(hyp_ctx* c, const double* dL_dQ_final, double* dL_dQ0, double* dL_deos) {
  if (!c || !dL_dQ_final) return HYP_ERR_INVALID;
  int rc = adjoint_supported(c);
  if (rc != HYP_OK) return rc;
  AdjTape* t = c->tape;
  if (!t || t->steps_at_end < 0 || t->steps_at_end != c->steps_host)
    return ctx_set_err(c, HYP_ERR_INVALID, "hyp_adjoint: no recorded run ends at the current state");
  ACK(cudaSetDevice(c->device));
  const int64_t n = c->n;
  const size_t bytes = (size_t)14 * n * sizeof(double);
  ACK(cudaMemcpyAsync(t->Qb[0], dL_dQ_final, bytes, cudaMemcpyHostToDevice, c->stream));
  ACK(cudaMemsetAsync(t->eacc, 0, (size_t)2 * t->cell_grid * sizeof(double), c->stream));
  const int big[2] = {INT_MAX, INT_MAX};
  ACK(cudaMemcpyAsync(t->amax, big, sizeof big, cudaMemcpyHostToDevice, c->stream));
  ACK(cudaMemsetAsync(t->seg_t, 0, (size_t)(t->K + 1) * sizeof(double), c->stream));
  const double dx = c->cfg.x_length / (double)n;
  const double inf = INFINITY;
  const unsigned egrid = (unsigned)((n + kBlock - 1) / kBlock);
  int cur = 0;
  t->ms_recompute = t->ms_adjoint = 0.f;
  const int n_seg = (t->n_steps + t->K - 1) / t->K;
  for (int s = n_seg - 1; s >= 0; --s) {
    const int a = s * t->K;
    const int L = std::min(t->K, t->n_steps - a);
    ACK(cudaEventRecord(t->ev[0], c->stream));
    // rerun the segment from its checkpoint with the step kernels
    ACK(cudaMemcpyAsync(t->seg_Q, t->ckpt + (size_t)s * 14 * n, bytes, cudaMemcpyDeviceToDevice, c->stream));
    ACK(cudaMemsetAsync(t->seg_lmax, 0, sizeof(unsigned long long), c->stream));
    for (int k = 0; k < L; ++k) {
      double* Qk = t->seg_Q + (size_t)k * 14 * n;
      double* Fk = t->seg_F + (size_t)k * kNFlux1 * n;
      double* lk = t->seg_lam + (size_t)k * n;
      cell1_f64_kernel<<<egrid, kBlock, 0, c->stream>>>(Qk, n, c->eos[0], Fk, lk, &t->seg_lmax[k], &t->seg_t[k], inf,
                                                        c->st);
      ACK(cudaGetLastError());
      if (k + 1 < L) {
        update1_f64_kernel<<<egrid, kBlock, 0, c->stream>>>(Qk, Qk + 14 * n, n, Fk, lk, &t->seg_lmax[k],
                                                            &t->seg_lmax[k + 1], &t->seg_t[k], &t->seg_t[k + 1],
                                                            t->seg_steps, inf, c->cfg.cfl, dx, c->cfg.flux,
                                                            c->cfg.bc);
        ACK(cudaGetLastError());
      }
    }
    ACK(cudaEventRecord(t->ev[1], c->stream));
    // adjoint steps a + L - 1 .. a
    for (int k = L - 1; k >= 0; --k) {
      const int step = a + k;
      AdjArgs g;
      g.Q = t->seg_Q + (size_t)k * 14 * n;
      // the step's result: the next segment state, the next checkpoint, or the final state
      g.Qn = k + 1 < L ? t->seg_Q + (size_t)(k + 1) * 14 * n
                       : (s + 1 < n_seg ? t->ckpt + (size_t)(s + 1) * 14 * n : c->Q[c->cur]);
      g.F = t->seg_F + (size_t)k * kNFlux1 * n;
      g.lam = t->seg_lam + (size_t)k * n;
      g.lmax = &t->seg_lmax[k];
      g.Qb1 = t->Qb[cur];
      g.Qb0 = t->Qb[1 - cur];
      g.rpart = t->rpart;
      g.amax_rd = &t->amax[step & 1];
      g.amax_clr = &t->amax[(step + 1) & 1];
      g.eacc = t->eacc;
      g.n = n;
      g.cfl = c->cfg.cfl;
      g.dx = dx;
      g.trans = c->cfg.bc == HYP_BC_TRANSMISSIVE;
      g.part_grid = t->part_grid;
      adj_dtdx_kernel<<<t->part_grid, 256, 0, c->stream>>>(g);
      ACK(cudaGetLastError());
      adj_cell_kernel<<<t->cell_grid, kAdjBlock, 0, c->stream>>>(g, c->eos[0]);
      ACK(cudaGetLastError());
      cur = 1 - cur;
    }
    ACK(cudaEventRecord(t->ev[2], c->stream));
    ACK(cudaEventSynchronize(t->ev[2]));
    float m1 = 0.f, m2 = 0.f;
    ACK(cudaEventElapsedTime(&m1, t->ev[0], t->ev[1]));
    ACK(cudaEventElapsedTime(&m2, t->ev[1], t->ev[2]));
    t->ms_recompute += m1;
    t->ms_adjoint += m2;
  }
  if (dL_dQ0) ACK(cudaMemcpyAsync(dL_dQ0, t->Qb[cur], bytes, cudaMemcpyDeviceToHost, c->stream));
  std::vector<double> eacc((size_t)2 * t->cell_grid);
  ACK(cudaMemcpyAsync(eacc.data(), t->eacc, eacc.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = ctx_sync_state(c)) != HYP_OK) return rc;
  if (dL_deos) {
    double b = 0.0, k = 0.0;
    for (int j = 0; j < t->cell_grid; ++j) {
      b += eacc[2 * j];
      k += eacc[2 * j + 1];
    }
    dL_deos[0] = b;
    dL_deos[1] = k;
  }
  return ctx_check_cell_error(c);
}

extern "C" int hyp_adjoint_timing(const hyp_ctx* c, double* ms_record, double* ms_recompute, double* ms_adjoint) {
  if (!c || !c->tape) return HYP_ERR_INVALID;
  if (ms_record) *ms_record = c->tape->ms_record;
  if (ms_recompute) *ms_recompute = c->tape->ms_recompute;
  if (ms_adjoint) *ms_adjoint = c->tape->ms_adjoint;
  return HYP_OK;
}

extern "C" int hyp_density_misfit(hyp_ctx* c, const double* rho_target, double* loss, double* dL_dQ) {
  if (!c || !rho_target) return HYP_ERR_INVALID;
  if (c->cfg.model != HYP_MODEL_SINGLE || c->cfg.precision != HYP_PREC_FP64)
    return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "hyp_density_misfit: single-phase FP64 context");
  ACK(cudaSetDevice(c->device));
  AdjTape* t = c->tape;
  if (!t) t = c->tape = new AdjTape();
  const int64_t n = c->n;
  if (!t->misfit) ACK(cudaMalloc(&t->misfit, (size_t)n * sizeof(double)));
  if (!t->mpart) ACK(cudaMalloc(&t->mpart, kPartBlocks * sizeof(double)));
  if (dL_dQ && !t->Qb[0]) ACK(cudaMalloc(&t->Qb[0], (size_t)14 * n * sizeof(double)));
  ACK(cudaMemcpyAsync(t->misfit, rho_target, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const int grid = (int)std::min<int64_t>(kPartBlocks, (n + 255) / 256);
  misfit_kernel<<<grid, 256, 0, c->stream>>>(c->Q[c->cur], t->misfit, n, c->eos[0].inv_rho0, dL_dQ ? t->Qb[0] : nullptr,
                                            t->mpart);
  ACK(cudaGetLastError());
  std::vector<double> part(grid);
  ACK(cudaMemcpyAsync(part.data(), t->mpart, grid * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (dL_dQ)
    ACK(cudaMemcpyAsync(dL_dQ, t->Qb[0], (size_t)14 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ACK(cudaStreamSynchronize(c->stream));
  double s = 0.0;
  for (double v : part) s += v;
  if (loss) *loss = s;
  return HYP_OK;
}

extern "C" int hyp_eval_prim2cons_vjp(const hyp_config* cfg, const double* P, const double* Qbar, double* Pbar,
                                      double* eos_bar, int64_t n) {
  if (!cfg || !P || !Qbar || !Pbar || !eos_bar || n <= 0) return HYP_ERR_INVALID;
  if (cfg->model != HYP_MODEL_SINGLE) return HYP_ERR_UNSUPPORTED;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  const hyp_barton2009& b = cfg->eos[0];
  const EosC e = make_eos(b.rho0, b.c0, b.cv, b.t0, b.b0, b.alpha, b.beta, b.gamma);
  double *dP = nullptr, *dQ = nullptr, *dR = nullptr, *dE = nullptr;
  const size_t bytes = (size_t)14 * n * sizeof(double);
  int rc = HYP_OK;
  if (cudaMalloc(&dP, bytes) != cudaSuccess || cudaMalloc(&dQ, bytes) != cudaSuccess ||
      cudaMalloc(&dR, bytes) != cudaSuccess || cudaMalloc(&dE, (size_t)2 * n * sizeof(double)) != cudaSuccess)
    rc = HYP_ERR_CUDA;
  if (rc == HYP_OK && (cudaMemcpy(dP, P, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(dQ, Qbar, bytes, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = HYP_ERR_CUDA;
  std::vector<double> eb((size_t)2 * n);
  if (rc == HYP_OK) {
    prim2cons_vjp_kernel<<<(unsigned)((n + 127) / 128), 128>>>(e, dP, dQ, dR, dE, n);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(Pbar, dR, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(eb.data(), dE, eb.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = HYP_ERR_CUDA;
  }
  cudaFree(dP);
  cudaFree(dQ);
  cudaFree(dR);
  cudaFree(dE);
  if (rc == HYP_OK) {
    double s0 = 0.0, s1 = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      s0 += eb[2 * i];
      s1 += eb[2 * i + 1];
    }
    eos_bar[0] = s0;
    eos_bar[1] = s1;
  }
  return rc;
}
