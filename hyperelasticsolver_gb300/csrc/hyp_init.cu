// hyp_init.cu -- initial conditions built on the device.
//
//   hyp_initial_states : the two-phase Riemann test cases of
//                        HyperelasticityMPh.jl:275-426 (cases 1-7 and 10, the ones
//                        the reference defines), returned as conservative
//                        30-vectors after prim2cons on the device;
//   hyp_init_riemann   : the two-state fill of main.jl:99-106 (cells with
//                        (i - 1) < nx/2 left, 1-based), written straight into the
//                        context's state;
//   hyp_init_tanh      : initial_condition_tanh of main.jl:110-123: per cell
//                        x = (i - 1/2)/nx, the primitive state of the side x falls
//                        on, alpha1 = 0.2/2 (tanh(4 (x - 1/2)/eps) + 1) + 0.4,
//                        alpha2 = 1 - alpha1, then prim2cons.
// The test-case values are the reference's data (they have to match).
#include <cmath>
#include "hyp_internal.cuh"

namespace hyp {

struct InitArg {
  EosC e[2];
  int model;  // HYP_MODEL_SINGLE: 14 variables, else 30
  double ql[30], qr[30];
};

__global__ void init_riemann_kernel(InitArg a, double* __restrict__ Q, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nv = a.model == HYP_MODEL_SINGLE ? 14 : 30;
  const bool left = (double)i < (double)n / 2.0;  // (i - 1) < nx / 2 with 1-based i
  for (int v = 0; v < nv; ++v) Q[v * n + i] = left ? a.ql[v] : a.qr[v];
}

__global__ void init_tanh_kernel(InitArg a, double eps, double* __restrict__ Q, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = ((double)i + 0.5) / (double)n;  // (i - 0.5)/nx with 1-based i
  const double* q = x < 0.5 ? a.ql : a.qr;
  double p[30], r[30];
  phase_cons2prim(a.e[0], q, p);
  phase_cons2prim(a.e[1], q + 15, p + 15);
  p[0] = 0.2 / 2 * (tanh(4 * (x - 0.5) / eps) + 1) + 0.4;
  p[15] = 1 - p[0];
  phase_prim2cons(a.e[0], p, r);
  phase_prim2cons(a.e[1], p + 15, r + 15);
  for (int v = 0; v < 30; ++v) Q[v * n + i] = r[v];
}

__global__ void prim2cons2_kernel(EosC e0, EosC e1, const double* p, double* q) {
  if (threadIdx.x == 0) phase_prim2cons(e0, p, q);
  if (threadIdx.x == 1) phase_prim2cons(e1, p + 15, q + 15);
}

// Primitive 30-vectors of a test case of HyperelasticityMPh.jl:275-426; false if
// the reference does not define it.
static bool testcase_prims(int tc, double* Pl, double* Pr) {
  struct Side {
    double a1, a2, u[3], S;
    double F[9];  // row-major as written in the reference
  };
  const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const double F3[9] = {1.0, 0.0, 0.0, -0.01, 0.95, 0.02, -0.015, 0.0, 0.9};
  const double F5r[9] = {1.0, 0.0, 0.0, 0.015, 0.95, 0.0, -0.01, 0.0, 0.9};
  const double F4l[9] = {0.98, 0.0, 0.0, 0.02, 1.0, 0.1, 0.0, 0.0, 1.0};
  const double F4r[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.1, 0.0, 0.0, 1.0};
  Side L{}, R{};
  double den = 8.9;
  auto set = [](Side& s, double a1, double a2, double u0, double u1, double u2, double S, const double* F) {
    s.a1 = a1;
    s.a2 = a2;
    s.u[0] = u0;
    s.u[1] = u1;
    s.u[2] = u2;
    s.S = S;
    for (int k = 0; k < 9; ++k) s.F[k] = F[k];
  };
  switch (tc) {
    case 1:
      den = 5.0;
      set(L, 0.5, 0.5, 0, 0, 0, 0, I);
      set(R, 0.5, 0.5, 0, 0, 0, 0, I);
      break;
    case 2:
      den = 5.0;
      set(L, 0.5, 0.5, 1.0, 0, 0, 0, I);
      set(R, 0.5, 0.5, 1.0, 0, 0, 0, I);
      break;
    case 3:
      set(L, 0.5, 0.5, 2.0, 0.0, 0.1, 0, F3);
      set(R, 0.5, 0.5, 2.0, 0.0, 0.1, 0, F3);
      break;
    case 4:
      set(L, 0.5, 0.5, 0.0, 0.5, 1.0, 1e-3, F4l);
      set(R, 0.5, 0.5, 0, 0, 0, 0, F4r);
      break;
    case 5:
      set(L, 0.5, 0.5, 2.0, 0.0, 0.1, 0, F3);
      set(R, 0.5, 0.5, 0.0, -0.03, -0.01, 0, F5r);
      break;
    case 6:
      set(L, 0.1, 0.9, 0.0, 0.5, 1.0, 1e-3, F4l);
      set(R, 0.9, 0.1, 0, 0, 0, 0, F4r);
      break;
    case 7:
      set(L, 0.1, 0.9, 2.0, 0.0, 0.1, 0, F3);
      set(R, 0.9, 0.1, 0.0, -0.03, -0.01, 0, F5r);
      break;
    case 10:
      set(L, 0.4, 0.6, 2.0, 0.0, 0.1, 0, F3);
      set(R, 0.6, 0.4, 2.0, 0.0, 0.1, 0, F3);
      break;
    default:
      return false;
  }
  auto fill = [den](const Side& s, double* P) {
    // det(F) of the row-major matrix; den_p = den / det(F_p) (HyperelasticityMPh.jl:412-415)
    const double* f = s.F;
    const double d = f[0] * (f[4] * f[8] - f[5] * f[7]) - f[1] * (f[3] * f[8] - f[5] * f[6]) +
                     f[2] * (f[3] * f[7] - f[4] * f[6]);
    for (int ph = 0; ph < 2; ++ph) {
      double* p = P + 15 * ph;
      p[0] = ph == 0 ? s.a1 : s.a2;
      p[1] = den / d;
      for (int c = 0; c < 3; ++c) p[2 + c] = s.u[c];
      p[5] = s.S;
      for (int c = 0; c < 3; ++c)  // column-major splat of F
        for (int r = 0; r < 3; ++r) p[6 + r + 3 * c] = f[3 * r + c];
    }
  };
  fill(L, Pl);
  fill(R, Pr);
  return true;
}

static EosC eos_c(const hyp_barton2009& b) { return make_eos(b.rho0, b.c0, b.cv, b.t0, b.b0, b.alpha, b.beta, b.gamma); }

}  // namespace hyp

using namespace hyp;

extern "C" int hyp_initial_states(const hyp_config* cfg, int testcase, double* Ql, double* Qr) {
  if (!cfg || !Ql || !Qr) return HYP_ERR_INVALID;
  if (cfg->model != HYP_MODEL_MULTI) return HYP_ERR_UNSUPPORTED;
  double P[60];
  if (!testcase_prims(testcase, P, P + 30)) return HYP_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  double *dP = nullptr, *dQ = nullptr;
  int rc = HYP_OK;
  if (cudaMalloc(&dP, sizeof P) != cudaSuccess || cudaMalloc(&dQ, sizeof P) != cudaSuccess ||
      cudaMemcpy(dP, P, sizeof P, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = HYP_ERR_CUDA;
  if (rc == HYP_OK) {
    const EosC e0 = eos_c(cfg->eos[0]), e1 = eos_c(cfg->eos[1]);
    prim2cons2_kernel<<<1, 32>>>(e0, e1, dP, dQ);
    prim2cons2_kernel<<<1, 32>>>(e0, e1, dP + 30, dQ + 30);
    double Q[60];
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(Q, dQ, sizeof Q, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = HYP_ERR_CUDA;
    } else {
      for (int k = 0; k < 30; ++k) {
        Ql[k] = Q[k];
        Qr[k] = Q[30 + k];
      }
    }
  }
  cudaFree(dP);
  cudaFree(dQ);
  return rc;
}

static InitArg init_arg(const hyp_ctx* c, const double* Ql, const double* Qr) {
  InitArg a;
  a.e[0] = c->eos[0];
  a.e[1] = c->eos[1];
  a.model = c->cfg.model;
  for (int v = 0; v < c->nvar; ++v) {
    a.ql[v] = Ql[v];
    a.qr[v] = Qr[v];
  }
  return a;
}

extern "C" int hyp_init_riemann(hyp_ctx* c, const double* Ql, const double* Qr) {
  if (!c || !Ql || !Qr) return HYP_ERR_INVALID;
  if (cudaSetDevice(c->device) != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, "cudaSetDevice");
  init_riemann_kernel<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(init_arg(c, Ql, Qr),
                                                                           ctx_install_target(c), c->n);
  if (cudaGetLastError() != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, "hyp_init_riemann: launch");
  return ctx_finish_install(c, 0.0);
}

extern "C" int hyp_init_tanh(hyp_ctx* c, const double* Ql, const double* Qr, double eps) {
  if (!c || !Ql || !Qr || !(eps > 0.0)) return HYP_ERR_INVALID;
  if (c->cfg.model != HYP_MODEL_MULTI)
    return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "hyp_init_tanh: the tanh volume-fraction profile needs two phases");
  if (cudaSetDevice(c->device) != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, "cudaSetDevice");
  init_tanh_kernel<<<(unsigned)((c->n + 127) / 128), 128, 0, c->stream>>>(init_arg(c, Ql, Qr), eps,
                                                                         ctx_install_target(c), c->n);
  if (cudaGetLastError() != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, "hyp_init_tanh: launch");
  return ctx_finish_install(c, 0.0);
}
