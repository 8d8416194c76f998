// hyp_eval.cu -- function-level evaluators of the C ABI: the reference's pure
// per-cell functions (Strains, EquationsOfState, HyperelasticityMPh, NumFluxes)
// applied to n independent inputs on the GPU with the same device code as the
// step. Host arrays in and out (SoA [k][n]).
#include <cmath>
#include <vector>
#include "hyp_internal.cuh"
#include "hyp_hank.cuh"
#include "hyp_relax.cuh"

using namespace hyp;

namespace {

struct Buf {
  const double* host_in = nullptr;
  double* host_out = nullptr;
  int k = 0;
  double* dev = nullptr;
};

int run(int64_t n, std::vector<Buf> bufs, void (*launch)(int64_t, double**, const void*), const void* arg) {
  if (n <= 0) return n == 0 ? HYP_OK : HYP_ERR_INVALID;
  for (auto& b : bufs)
    if (!b.host_in && !b.host_out) return HYP_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYP_ERR_NO_DEVICE;
  int rc = HYP_OK;
  std::vector<double*> ptrs;
  for (auto& b : bufs) {
    if (cudaMalloc(&b.dev, (size_t)b.k * n * sizeof(double)) != cudaSuccess) { rc = HYP_ERR_CUDA; break; }
    if (b.host_in && cudaMemcpy(b.dev, b.host_in, (size_t)b.k * n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      rc = HYP_ERR_CUDA;
      break;
    }
    ptrs.push_back(b.dev);
  }
  if (rc == HYP_OK) {
    launch(n, ptrs.data(), arg);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = HYP_ERR_CUDA;
  }
  for (auto& b : bufs) {
    if (rc == HYP_OK && b.host_out &&
        cudaMemcpy(b.host_out, b.dev, (size_t)b.k * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = HYP_ERR_CUDA;
    if (b.dev) cudaFree(b.dev);
  }
  return rc;
}

inline unsigned grid(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }
#define IDX int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x; if (i >= n) return;
#define LD(dst, src, k) for (int _c = 0; _c < (k); ++_c) (dst)[_c] = (src)[_c * n + i]
#define ST(dst, src, k) for (int _c = 0; _c < (k); ++_c) (dst)[_c * n + i] = (src)[_c]

__global__ void k_finger(const double* A, double* G, int64_t n) {
  IDX double a[9], g[9];
  LD(a, A, 9);
  finger_A(a, g);
  ST(G, g, 9);
}
__global__ void k_invariants(const double* G, double* I, int64_t n) {
  IDX double g[9], v[3];
  LD(g, G, 9);
  invariants_general(g, v);
  ST(I, v, 3);
}
__global__ void k_energy(EosC e, const double* S, const double* G, double* out, int64_t n) {
  IDX double g[9];
  LD(g, G, 9);
  out[i] = energy_SG(e, S[i], g);
}
__global__ void k_entropy(EosC e, const double* E, const double* G, double* out, int64_t n) {
  IDX double g[9];
  LD(g, G, 9);
  out[i] = entropy_eG(e, E[i], g);
}
__global__ void k_stress(EosC e, const double* S, const double* F, double* out, int64_t n) {
  IDX double f[9], s[9];
  LD(f, F, 9);
  stress_SF(e, S[i], f, s);
  ST(out, s, 9);
}
__global__ void k_acoustic(EosC e, const double* S, const double* F, double* out, int64_t n) {
  IDX double f[9], s[9];
  LD(f, F, 9);
  acoustic_SF(e, S[i], f, s);
  ST(out, s, 9);
}
__global__ void k_acoustic_dir(EosC e, const double* S, const double* F, const double* D, double* out, int64_t n) {
  IDX double f[9], s[9], dir[3];
  LD(f, F, 9);
  LD(dir, D, 3);
  acoustic_SFn(e, S[i], f, dir, s);
  ST(out, s, 9);
}
__global__ void k_stress_den(EosC e, const double* den, const double* E, const double* F, double* out, int64_t n) {
  IDX double f[9], s[9];
  LD(f, F, 9);
  stress_den_eF(e, den[i], E[i], f, s);
  ST(out, s, 9);
}
__global__ void k_acoustic_prim(EosC e, const double* P, const double* D, double* out, int64_t n) {
  IDX double p[15], s[9], dir[3];
  LD(p, P, 15);
  LD(dir, D, 3);
  acoustic_Pn(e, p, dir, s);
  ST(out, s, 9);
}

__device__ void phase_flux15(const EosC& e, const double* q, double* f) {
  Prim P;
  cons_to_prim(e, q[0], q + 2, q[5], q + 6, P);
  StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
  double s0[3];
  f[0] = 0.0;
  phase_flux(e, q[0], P, c, f + 1, s0);
}
// get_eigvals for one phase (HyperelasticityMPh.jl:258-266) along direction n:
// u.n + c_k then u.n - c_k, c_k = sqrt|mu_k| in the order of eig_sorted3 (the
// order Julia's eigvals gives the reference).
__device__ void phase_eigvals(const EosC& e, const double* q, const double* n, double* out6) {
  Prim P;
  cons_to_prim(e, q[0], q + 2, q[5], q + 6, P);
  StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
  const double rho_s = e.rho0 * P.k.s;
  double sig[9], sn[3], om[9], m[3];
  stress_full(rho_s, P.k, c, sig);
  for (int k = 0; k < 3; ++k) sn[k] = (sig[k] * n[0] + sig[k + 3] * n[1] + sig[k + 6] * n[2]) / rho_s;
  acoustic_omega_dir(e, P.k, P.w, c, P.xm1, false, false, sn, n, om);
  eig_sorted3(om, m);
  const double un = (P.u[0] * n[0] + P.u[1] * n[1]) + P.u[2] * n[2];  // dot(P[3:5], n)
  for (int k = 0; k < 3; ++k) {
    const double cs = sqrt(m[k]);
    out6[k] = un + cs;
    out6[3 + k] = un - cs;
  }
}

struct ModelArg {
  EosC e[2];
  int model;
};

// Model-level kernels: expand a single-phase 14-vector to alpha = 1.
__device__ int load_cell(const ModelArg& m, const double* Q, int64_t n, int64_t i, double* q30) {
  if (m.model == HYP_MODEL_SINGLE) {
    q30[0] = 1.0;
    for (int c = 0; c < 14; ++c) q30[1 + c] = Q[c * n + i];
    return 1;
  }
  for (int c = 0; c < 30; ++c) q30[c] = Q[c * n + i];
  return 2;
}
__device__ void store_cell(const ModelArg& m, double* Q, int64_t n, int64_t i, const double* q30) {
  if (m.model == HYP_MODEL_SINGLE) {
    for (int c = 0; c < 14; ++c) Q[c * n + i] = q30[1 + c];
  } else {
    for (int c = 0; c < 30; ++c) Q[c * n + i] = q30[c];
  }
}
__global__ void k_cons2prim(ModelArg m, const double* Q, double* P, int64_t n) {
  IDX double q[30], p[30];
  int np = load_cell(m, Q, n, i, q);
  for (int ph = 0; ph < np; ++ph) phase_cons2prim(m.e[ph], q + 15 * ph, p + 15 * ph);
  store_cell(m, P, n, i, p);
}
__global__ void k_prim2cons(ModelArg m, const double* P, double* Q, int64_t n) {
  IDX double p[30], q[30];
  int np = load_cell(m, P, n, i, p);
  for (int ph = 0; ph < np; ++ph) phase_prim2cons(m.e[ph], p + 15 * ph, q + 15 * ph);
  store_cell(m, Q, n, i, q);
}
__global__ void k_flux(ModelArg m, const double* Q, double* F, int64_t n) {
  IDX double q[30], f[30];
  int np = load_cell(m, Q, n, i, q);
  for (int ph = 0; ph < np; ++ph) phase_flux15(m.e[ph], q + 15 * ph, f + 15 * ph);
  store_cell(m, F, n, i, f);
}
// D: directions [3][n], or null for n = e1 (the direction main.jl's step uses).
__global__ void k_eigvals(ModelArg m, const double* Q, const double* D, double* out, int64_t n) {
  IDX double q[30], s[12], dir[3] = {1.0, 0.0, 0.0};
  if (D) LD(dir, D, 3);
  int np = load_cell(m, Q, n, i, q);
  for (int ph = 0; ph < np; ++ph) phase_eigvals(m.e[ph], q + 15 * ph, dir, s + 6 * ph);
  ST(out, s, 6 * np);
}
__global__ void k_lxf1(ModelArg m, const double* Ql, const double* Qr, const double* lam, double* cons, double* dm,
                       double* dp, int64_t n) {
  IDX double ql[30], qr[30], fl[30], fr[30];
  load_cell(m, Ql, n, i, ql);
  load_cell(m, Qr, n, i, qr);
  phase_flux15(m.e[0], ql, fl);
  phase_flux15(m.e[0], qr, fr);
  double hl = lam[i] * 0.5;
  for (int c = 0; c < 14; ++c) {
    cons[c * n + i] = 0.5 * (fl[1 + c] + fr[1 + c]) - hl * (qr[1 + c] - ql[1 + c]);
    dm[c * n + i] = 0.0;
    dp[c * n + i] = 0.0;
  }
}

ModelArg model_arg(const hyp_config* cfg) {
  ModelArg m;
  m.model = cfg->model;
  m.e[0] = make_eos(cfg->eos[0].rho0, cfg->eos[0].c0, cfg->eos[0].cv, cfg->eos[0].t0, cfg->eos[0].b0,
                    cfg->eos[0].alpha, cfg->eos[0].beta, cfg->eos[0].gamma);
  const hyp_barton2009& b = cfg->model == HYP_MODEL_MULTI ? cfg->eos[1] : cfg->eos[0];
  m.e[1] = make_eos(b.rho0, b.c0, b.cv, b.t0, b.b0, b.alpha, b.beta, b.gamma);
  return m;
}
EosC eos_of(const hyp_barton2009* b) {
  return make_eos(b->rho0, b->c0, b->cv, b->t0, b->b0, b->alpha, b->beta, b->gamma);
}
int nvar_of(const hyp_config* c) { return c->model == HYP_MODEL_SINGLE ? 14 : 30; }
bool model_ok(const hyp_config* c) { return c && (c->model == HYP_MODEL_SINGLE || c->model == HYP_MODEL_MULTI); }

}  // namespace

extern "C" int hyp_eval_finger(const double* A, double* G, int64_t n) {
  return run(n, {{A, nullptr, 9}, {nullptr, G, 9}},
             [](int64_t n, double** d, const void*) { k_finger<<<grid(n), kBlock>>>(d[0], d[1], n); }, nullptr);
}
extern "C" int hyp_eval_invariants(const double* G, double* out, int64_t n) {
  return run(n, {{G, nullptr, 9}, {nullptr, out, 3}},
             [](int64_t n, double** d, const void*) { k_invariants<<<grid(n), kBlock>>>(d[0], d[1], n); }, nullptr);
}
extern "C" int hyp_eval_energy(const hyp_barton2009* eos, const double* S, const double* G, double* e, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{S, nullptr, 1}, {G, nullptr, 9}, {nullptr, e, 1}},
             [](int64_t n, double** d, const void* a) {
               k_energy<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], n);
             },
             &ec);
}
extern "C" int hyp_eval_entropy(const hyp_barton2009* eos, const double* e, const double* G, double* S, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{e, nullptr, 1}, {G, nullptr, 9}, {nullptr, S, 1}},
             [](int64_t n, double** d, const void* a) {
               k_entropy<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], n);
             },
             &ec);
}
extern "C" int hyp_eval_stress(const hyp_barton2009* eos, const double* S, const double* F, double* sigma, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{S, nullptr, 1}, {F, nullptr, 9}, {nullptr, sigma, 9}},
             [](int64_t n, double** d, const void* a) {
               k_stress<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], n);
             },
             &ec);
}
extern "C" int hyp_eval_acoustic(const hyp_barton2009* eos, const double* S, const double* F, double* ac, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{S, nullptr, 1}, {F, nullptr, 9}, {nullptr, ac, 9}},
             [](int64_t n, double** d, const void* a) {
               k_acoustic<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], n);
             },
             &ec);
}
extern "C" int hyp_eval_acoustic_dir(const hyp_barton2009* eos, const double* S, const double* F, const double* dir,
                                     double* ac, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{S, nullptr, 1}, {F, nullptr, 9}, {dir, nullptr, 3}, {nullptr, ac, 9}},
             [](int64_t n, double** d, const void* a) {
               k_acoustic_dir<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], d[3], n);
             },
             &ec);
}
extern "C" int hyp_eval_stress_den(const hyp_barton2009* eos, const double* den, const double* e_int, const double* F,
                                   double* sigma, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{den, nullptr, 1}, {e_int, nullptr, 1}, {F, nullptr, 9}, {nullptr, sigma, 9}},
             [](int64_t n, double** d, const void* a) {
               k_stress_den<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], d[3], n);
             },
             &ec);
}
extern "C" int hyp_eval_acoustic_prim(const hyp_barton2009* eos, const double* P, const double* dir, double* ac,
                                      int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  EosC ec = eos_of(eos);
  return run(n, {{P, nullptr, 15}, {dir, nullptr, 3}, {nullptr, ac, 9}},
             [](int64_t n, double** d, const void* a) {
               k_acoustic_prim<<<grid(n), kBlock>>>(*(const EosC*)a, d[0], d[1], d[2], n);
             },
             &ec);
}
// ---- Hank2016 (EquationsOfState.jl:305-366) ----------------------------------
namespace {
__global__ void k_hank_energy(Hank h, const double* den, const double* pres, const double* G, double* out,
                              int64_t n) {
  IDX double g[9];
  LD(g, G, 9);
  out[i] = hank_energy(h, den[i], pres[i], g);
}
__global__ void k_hank_pressure(Hank h, const double* den, const double* e, const double* I3, double* out,
                                int64_t n) {
  IDX double v[3];
  LD(v, I3, 3);
  out[i] = hank_pressure(h, den[i], e[i], v);
}
__global__ void k_hank_stress(Hank h, const double* den, const double* pres, const double* F, double* out,
                              int64_t n) {
  IDX double f[9], s[9];
  LD(f, F, 9);
  hank_stress(h, den[i], pres[i], f, s);
  ST(out, s, 9);
}
Hank hank_of(const hyp_hank2016* e) { return Hank{e->rho0, e->mu, e->gamma, e->pres_inf, e->a}; }
}  // namespace

extern "C" int hyp_eval_hank2016_energy(const hyp_hank2016* eos, const double* den, const double* pres,
                                        const double* G, double* e, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  const Hank h = hank_of(eos);
  return run(n, {{den, nullptr, 1}, {pres, nullptr, 1}, {G, nullptr, 9}, {nullptr, e, 1}},
             [](int64_t n, double** d, const void* a) {
               k_hank_energy<<<grid(n), kBlock>>>(*(const Hank*)a, d[0], d[1], d[2], d[3], n);
             },
             &h);
}
extern "C" int hyp_eval_hank2016_pressure(const hyp_hank2016* eos, const double* den, const double* e_int,
                                          const double* inv, double* pres, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  const Hank h = hank_of(eos);
  return run(n, {{den, nullptr, 1}, {e_int, nullptr, 1}, {inv, nullptr, 3}, {nullptr, pres, 1}},
             [](int64_t n, double** d, const void* a) {
               k_hank_pressure<<<grid(n), kBlock>>>(*(const Hank*)a, d[0], d[1], d[2], d[3], n);
             },
             &h);
}
extern "C" int hyp_eval_hank2016_stress(const hyp_hank2016* eos, const double* den, const double* pres,
                                        const double* F, double* sigma, int64_t n) {
  if (!eos) return HYP_ERR_INVALID;
  const Hank h = hank_of(eos);
  return run(n, {{den, nullptr, 1}, {pres, nullptr, 1}, {F, nullptr, 9}, {nullptr, sigma, 9}},
             [](int64_t n, double** d, const void* a) {
               k_hank_stress<<<grid(n), kBlock>>>(*(const Hank*)a, d[0], d[1], d[2], d[3], n);
             },
             &h);
}

extern "C" int hyp_eval_cons2prim(const hyp_config* cfg, const double* Q, double* P, int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  int k = nvar_of(cfg);
  return run(n, {{Q, nullptr, k}, {nullptr, P, k}},
             [](int64_t n, double** d, const void* a) {
               k_cons2prim<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], n);
             },
             &m);
}
extern "C" int hyp_eval_prim2cons(const hyp_config* cfg, const double* P, double* Q, int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  int k = nvar_of(cfg);
  return run(n, {{P, nullptr, k}, {nullptr, Q, k}},
             [](int64_t n, double** d, const void* a) {
               k_prim2cons<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], n);
             },
             &m);
}
extern "C" int hyp_eval_flux(const hyp_config* cfg, const double* Q, double* F, int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  int k = nvar_of(cfg);
  return run(n, {{Q, nullptr, k}, {nullptr, F, k}},
             [](int64_t n, double** d, const void* a) {
               k_flux<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], n);
             },
             &m);
}
extern "C" int hyp_eval_eigvals(const hyp_config* cfg, const double* Q, double* out, int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  int k = nvar_of(cfg);
  int ns = cfg->model == HYP_MODEL_SINGLE ? 6 : 12;
  return run(n, {{Q, nullptr, k}, {nullptr, out, ns}},
             [](int64_t n, double** d, const void* a) {
               k_eigvals<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], nullptr, d[1], n);
             },
             &m);
}
extern "C" int hyp_eval_eigvals_dir(const hyp_config* cfg, const double* Q, const double* dir, double* out,
                                    int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  int k = nvar_of(cfg);
  int ns = cfg->model == HYP_MODEL_SINGLE ? 6 : 12;
  return run(n, {{Q, nullptr, k}, {dir, nullptr, 3}, {nullptr, out, ns}},
             [](int64_t n, double** d, const void* a) {
               k_eigvals<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], d[2], n);
             },
             &m);
}
namespace {
struct LxfArg2 {
  ModelArg m;
  Quad6D qd;
};
__global__ void k_lxf2(LxfArg2 a, const double* Ql, const double* Qr, const double* lam, double* cons, double* DMo,
                       double* DPo, int64_t n) {
  IDX double ql[30], qr[30], fl[30], fr[30], ff[30], dm[30], dp[30];
  LD(ql, Ql, 30);
  LD(qr, Qr, 30);
  flux2(a.m.e, ql, fl);
  flux2(a.m.e, qr, fr);
  lxf_face2(a.m.e, a.qd, ql, qr, fl, fr, lam[i], ff, dm, dp);
  ST(cons, ff, 30);
  ST(DMo, dm, 30);
  ST(DPo, dp, 30);
}
}  // namespace

extern "C" int hyp_eval_lxf(const hyp_config* cfg, const double* Ql, const double* Qr, const double* lambda,
                            double* cons, double* dm, double* dp, int64_t n) {
  if (!model_ok(cfg)) return HYP_ERR_INVALID;
  if (cfg->model == HYP_MODEL_MULTI) {
    LxfArg2 a2{model_arg(cfg), gauss_lobatto6()};
    return run(n,
               {{Ql, nullptr, 30}, {Qr, nullptr, 30}, {lambda, nullptr, 1}, {nullptr, cons, 30}, {nullptr, dm, 30},
                {nullptr, dp, 30}},
               [](int64_t n, double** d, const void* a) {
                 k_lxf2<<<grid(n), kBlock>>>(*(const LxfArg2*)a, d[0], d[1], d[2], d[3], d[4], d[5], n);
               },
               &a2);
  }
  ModelArg m = model_arg(cfg);
  return run(n,
             {{Ql, nullptr, 14}, {Qr, nullptr, 14}, {lambda, nullptr, 1}, {nullptr, cons, 14}, {nullptr, dm, 14},
              {nullptr, dp, 14}},
             [](int64_t n, double** d, const void* a) {
               k_lxf1<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], d[2], d[3], d[4], d[5], n);
             },
             &m);
}

// ---- two-phase evaluators ----------------------------------------------------
namespace {
__global__ void k_noncons(ModelArg m, const double* Q, double* B, int64_t n) {
  IDX double q[30], b[30];
  LD(q, Q, 30);
  noncons_bcol(m.e, q, b);
  ST(B, b, 30);
}
struct HllArg {
  ModelArg m;
  Quad6D qd;
};
// EL, ER: the caller's wave speeds of the left and right cell ([12][n] each, the
// eigvals[1], eigvals[2] of NumFluxes.jl:90-91), or null for the cells' own.
__global__ void k_hll(HllArg a, const double* Ql, const double* Qr, const double* EL, const double* ER, double* DMo,
                      double* DPo, int64_t n) {
  IDX double ql[30], qr[30], fl[30], fr[30], dm[30], dp[30];
  LD(ql, Ql, 30);
  LD(qr, Qr, 30);
  flux2(a.m.e, ql, fl);
  flux2(a.m.e, qr, fr);
  double lo_l, hi_l, lo_r, hi_r;
  if (EL) {  // minimum(eigvals[1]), maximum(eigvals[2])
    lo_l = EL[i];
    hi_r = ER[i];
    for (int k = 1; k < 12; ++k) {
      const double a_ = EL[(int64_t)k * n + i], b_ = ER[(int64_t)k * n + i];
      lo_l = a_ < lo_l ? a_ : lo_l;
      hi_r = b_ > hi_r ? b_ : hi_r;
    }
  } else {
    speeds2(a.m.e, ql, lo_l, hi_l);
    speeds2(a.m.e, qr, lo_r, hi_r);
  }
  hll_face2(a.m.e, a.qd, ql, qr, fl, fr, lo_l, hi_r, dm, dp);
  ST(DMo, dm, 30);
  ST(DPo, dp, 30);
}
}  // namespace

extern "C" int hyp_eval_noncons(const hyp_config* cfg, const double* Q, double* bcol, int64_t n) {
  if (!model_ok(cfg) || cfg->model != HYP_MODEL_MULTI) return HYP_ERR_INVALID;
  ModelArg m = model_arg(cfg);
  return run(n, {{Q, nullptr, 30}, {nullptr, bcol, 30}},
             [](int64_t n, double** d, const void* a) {
               k_noncons<<<grid(n), kBlock>>>(*(const ModelArg*)a, d[0], d[1], n);
             },
             &m);
}

extern "C" int hyp_eval_hll(const hyp_config* cfg, const double* Ql, const double* Qr, double* dm, double* dp,
                            int64_t n) {
  if (!model_ok(cfg) || cfg->model != HYP_MODEL_MULTI) return HYP_ERR_INVALID;
  HllArg a{model_arg(cfg), gauss_legendre6()};
  return run(n, {{Ql, nullptr, 30}, {Qr, nullptr, 30}, {nullptr, dm, 30}, {nullptr, dp, 30}},
             [](int64_t n, double** d, const void* p) {
               k_hll<<<(unsigned)((n + 63) / 64), 64>>>(*(const HllArg*)p, d[0], d[1], nullptr, nullptr, d[2], d[3],
                                                        n);
             },
             &a);
}
extern "C" int hyp_eval_hll_eigvals(const hyp_config* cfg, const double* Ql, const double* Qr, const double* eig_l,
                                    const double* eig_r, double* dm, double* dp, int64_t n) {
  if (!model_ok(cfg) || cfg->model != HYP_MODEL_MULTI) return HYP_ERR_INVALID;
  HllArg a{model_arg(cfg), gauss_legendre6()};
  return run(n,
             {{Ql, nullptr, 30}, {Qr, nullptr, 30}, {eig_l, nullptr, 12}, {eig_r, nullptr, 12}, {nullptr, dm, 30},
              {nullptr, dp, 30}},
             [](int64_t n, double** d, const void* p) {
               k_hll<<<(unsigned)((n + 63) / 64), 64>>>(*(const HllArg*)p, d[0], d[1], d[2], d[3], d[4], d[5], n);
             },
             &a);
}

// ---- two-phase pressure relaxation (hyp_relax.cuh) --------------------------
namespace {
struct RelaxArg {
  ModelArg m;
  int mode;
};
__global__ void k_relax(RelaxArg a, const double* Q, double* R, int64_t n) {
  IDX double q[30];
  LD(q, Q, 30);
  if (relax_cell2(a.m.e, a.mode, q)) {
    for (int c = 0; c < 30; ++c) q[c] = NAN;  // not converged
  }
  ST(R, q, 30);
}
}  // namespace

extern "C" int hyp_eval_relax(const hyp_config* cfg, int mode, const double* Q, double* Q_out, int64_t n) {
  if (!model_ok(cfg) || cfg->model != HYP_MODEL_MULTI) return HYP_ERR_INVALID;
  if (mode != HYP_RELAX_PRESSURE && mode != HYP_RELAX_MECHANICAL) return HYP_ERR_INVALID;
  RelaxArg a{model_arg(cfg), mode};
  return run(n, {{Q, nullptr, 30}, {nullptr, Q_out, 30}},
             [](int64_t n, double** d, const void* p) {
               k_relax<<<grid(n), kBlock>>>(*(const RelaxArg*)p, d[0], d[1], n);
             },
             &a);
}
