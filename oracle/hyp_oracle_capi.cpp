// oracle/hyp_oracle_capi.cpp -- extern "C" entry points of the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY (the oracle): loaded by tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference arm through ctypes. Never part of the
// product path. Arrays are structure-of-arrays: x[k*n + i] is component k of item i.
#include <cstdint>
#include <cstdlib>
#include <vector>
#include "hyp_oracle.hpp"

using namespace hyp_oracle;

extern "C" {

typedef struct { double rho0, c0, cv, t0, b0, alpha, beta, gamma; } hyo_eos;
typedef struct {
  int model, flux, bc, nx;
  double X, cfl;
  hyo_eos eos[2];
  int relax;
} hyo_problem;

static Barton to_barton(const hyo_eos* p) {
  return make_barton(p->rho0, p->c0, p->cv, p->t0, p->b0, p->alpha, p->beta, p->gamma);
}
static Problem to_problem(const hyo_problem* p) {
  Problem pb;
  pb.model = p->model;
  pb.eos[0] = to_barton(&p->eos[0]);
  pb.eos[1] = to_barton(&p->eos[1]);
  pb.flux = p->flux;
  pb.bc = p->bc;
  pb.nx = p->nx;
  pb.X = p->X;
  pb.cfl = p->cfl;
  pb.relax = p->relax;
  return pb;
}

#define GATHER(dst, src, k, n, i) for (int _c = 0; _c < (k); ++_c) (dst)[_c] = (src)[(size_t)_c * (n) + (i)]
#define SCATTER(dst, src, k, n, i) for (int _c = 0; _c < (k); ++_c) (dst)[(size_t)_c * (n) + (i)] = (src)[_c]

int hyo_finger(const double* A, double* G, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double a[9], g[9];
    GATHER(a, A, 9, n, i);
    finger(a, g);
    SCATTER(G, g, 9, n, i);
  }
  return 0;
}
int hyo_invariants(const double* G, double* I, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double g[9], v[3];
    GATHER(g, G, 9, n, i);
    invariants(g, v);
    SCATTER(I, v, 3, n, i);
  }
  return 0;
}
int hyo_energy(const hyo_eos* eos, const double* S, const double* G, double* e, int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double g[9];
    GATHER(g, G, 9, n, i);
    e[i] = energy(b, S[i], g);
  }
  return 0;
}
int hyo_entropy(const hyo_eos* eos, const double* e, const double* G, double* S, int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double g[9];
    GATHER(g, G, 9, n, i);
    S[i] = entropy(b, e[i], g);
  }
  return 0;
}
int hyo_stress(const hyo_eos* eos, const double* S, const double* F, double* sig, int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double f[9], s[9];
    GATHER(f, F, 9, n, i);
    stress(b, S[i], f, s);
    SCATTER(sig, s, 9, n, i);
  }
  return 0;
}
int hyo_acoustic(const hyo_eos* eos, const double* S, const double* F, double* ac, int64_t n) {
  Barton b = to_barton(eos);
  const double nv[3] = {1.0, 0.0, 0.0};
  for (int64_t i = 0; i < n; ++i) {
    double f[9], a[9];
    GATHER(f, F, 9, n, i);
    acoustic(b, S[i], f, nv, a);
    SCATTER(ac, a, 9, n, i);
  }
  return 0;
}
// acoustic(eos, ent, F, n) with a direction per item (dir: [3][n]).
int hyo_acoustic_dir(const hyo_eos* eos, const double* S, const double* F, const double* dir, double* ac, int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double f[9], a[9], d[3];
    GATHER(f, F, 9, n, i);
    GATHER(d, dir, 3, n, i);
    acoustic(b, S[i], f, d, a);
    SCATTER(ac, a, 9, n, i);
  }
  return 0;
}
// stress(eos, den, e_int, F) (EquationsOfState.jl:162-176).
int hyo_stress_den(const hyo_eos* eos, const double* den, const double* e_int, const double* F, double* sig,
                   int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double f[9], s[9];
    GATHER(f, F, 9, n, i);
    stress_den(b, den[i], e_int[i], f, s);
    SCATTER(sig, s, 9, n, i);
  }
  return 0;
}
// acoustic(eos, P, n) (EquationsOfState.jl:192-221); P: [15][n].
int hyo_acoustic_prim(const hyo_eos* eos, const double* P, const double* dir, double* ac, int64_t n) {
  Barton b = to_barton(eos);
  for (int64_t i = 0; i < n; ++i) {
    double pp[15], a[9], d[3];
    GATHER(pp, P, 15, n, i);
    GATHER(d, dir, 3, n, i);
    acoustic_prim(b, pp, d, a);
    SCATTER(ac, a, 9, n, i);
  }
  return 0;
}
// Eigenvalue moduli in Julia's eigvals order (ascending real part).
int hyo_eig3_sorted(const double* a, double* mods, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double m[9], r[3];
    GATHER(m, a, 9, n, i);
    eig3_sorted(m, r);
    SCATTER(mods, r, 3, n, i);
  }
  return 0;
}
typedef struct { double rho0, mu, gamma, pres_inf, a; } hyo_hank;
int hyo_hank_energy(const hyo_hank* p, const double* den, const double* pres, const double* G, double* e, int64_t n) {
  Hank2016 h{p->rho0, p->mu, p->gamma, p->pres_inf, p->a};
  for (int64_t i = 0; i < n; ++i) {
    double g[9];
    GATHER(g, G, 9, n, i);
    e[i] = hank_energy(h, den[i], pres[i], g);
  }
  return 0;
}
int hyo_hank_pressure(const hyo_hank* p, const double* den, const double* e, const double* I, double* pr, int64_t n) {
  Hank2016 h{p->rho0, p->mu, p->gamma, p->pres_inf, p->a};
  for (int64_t i = 0; i < n; ++i) {
    double v[3];
    GATHER(v, I, 3, n, i);
    pr[i] = hank_pressure(h, den[i], e[i], v);
  }
  return 0;
}
int hyo_hank_stress(const hyo_hank* p, const double* den, const double* pres, const double* F, double* sig, int64_t n) {
  Hank2016 h{p->rho0, p->mu, p->gamma, p->pres_inf, p->a};
  for (int64_t i = 0; i < n; ++i) {
    double f[9], s[9];
    GATHER(f, F, 9, n, i);
    hank_stress(h, den[i], pres[i], f, s);
    SCATTER(sig, s, 9, n, i);
  }
  return 0;
}
int hyo_eig3_moduli(const double* a, double* mods, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double m[9], r[3];
    GATHER(m, a, 9, n, i);
    eig3_moduli(m, r);
    SCATTER(mods, r, 3, n, i);
  }
  return 0;
}
int hyo_cons2prim(const hyo_problem* p, const double* Q, double* P, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double q[30], r[30];
    GATHER(q, Q, nv, n, i);
    if (pb.model == MODEL_SINGLE) {
      double q15[15], p15[15];
      expand1(q, q15);
      cons2prim(pb.eos[0], q15, p15);
      for (int k = 0; k < 14; ++k) r[k] = p15[1 + k];
    } else {
      cons2prim(pb.eos[0], q, r);
      cons2prim(pb.eos[1], q + 15, r + 15);
    }
    SCATTER(P, r, nv, n, i);
  }
  return 0;
}
int hyo_prim2cons(const hyo_problem* p, const double* P, double* Q, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double q[30], r[30];
    GATHER(r, P, nv, n, i);
    if (pb.model == MODEL_SINGLE) {
      double q15[15], p15[15];
      expand1(r, p15);
      prim2cons(pb.eos[0], p15, q15);
      for (int k = 0; k < 14; ++k) q[k] = q15[1 + k];
    } else {
      prim2cons(pb.eos[0], r, q);
      prim2cons(pb.eos[1], r + 15, q + 15);
    }
    SCATTER(Q, q, nv, n, i);
  }
  return 0;
}
int hyo_flux(const hyo_problem* p, const double* Q, double* F, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double q[30], f[30];
    GATHER(q, Q, nv, n, i);
    cell_flux(pb, q, f);
    SCATTER(F, f, nv, n, i);
  }
  return 0;
}
int hyo_speeds(const hyo_problem* p, const double* Q, double* spd, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model), ns = nspd_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double q[30], s[12];
    GATHER(q, Q, nv, n, i);
    cell_speeds(pb, q, s);
    SCATTER(spd, s, ns, n, i);
  }
  return 0;
}
// get_eigvals(eos, Q, n) with a direction per item (dir: [3][n]).
int hyo_speeds_dir(const hyo_problem* p, const double* Q, const double* dir, double* spd, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model), ns = nspd_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double q[30], s[12], d[3];
    GATHER(q, Q, nv, n, i);
    GATHER(d, dir, 3, n, i);
    cell_speeds(pb, q, s, d);
    SCATTER(spd, s, ns, n, i);
  }
  return 0;
}
// The two-phase relaxation of n cells: pressure, after the velocities when
// p->relax == 2 (status per cell in st: 0 or 8).
int hyo_relax(const hyo_problem* p, const double* Q, double* R, int* st, int64_t n) {
  Problem pb = to_problem(p);
  for (int64_t i = 0; i < n; ++i) {
    double q[30];
    GATHER(q, Q, 30, n, i);
    if (pb.relax == 2 && q[0] >= 1e-5 && q[15] >= 1e-5) relax_velocity2(pb.eos, q);
    st[i] = relax_pressure2(pb.eos, q);
    SCATTER(R, q, 30, n, i);
  }
  return 0;
}
int hyo_noncons(const hyo_problem* p, const double* Q, double* bcol, int64_t n) {
  Problem pb = to_problem(p);
  if (pb.model != MODEL_MULTI) return 1;
  for (int64_t i = 0; i < n; ++i) {
    double q[30], b[30];
    GATHER(q, Q, 30, n, i);
    noncons_cols(pb.eos, q, b);
    SCATTER(bcol, b, 30, n, i);
  }
  return 0;
}
int hyo_lxf(const hyo_problem* p, const double* Ql, const double* Qr, const double* lam, double* cons, double* dm,
            double* dp, int64_t n) {
  Problem pb = to_problem(p);
  int nv = nvar_of(pb.model);
  for (int64_t i = 0; i < n; ++i) {
    double l[30], r[30], c[30], m[30], pp[30];
    GATHER(l, Ql, nv, n, i);
    GATHER(r, Qr, nv, n, i);
    lxf_face(pb, l, r, lam[i], c, m, pp);
    SCATTER(cons, c, nv, n, i);
    SCATTER(dm, m, nv, n, i);
    SCATTER(dp, pp, nv, n, i);
  }
  return 0;
}
int hyo_hll(const hyo_problem* p, const double* Ql, const double* Qr, const double* spdL, const double* spdR,
            double* dm, double* dp, int64_t n) {
  Problem pb = to_problem(p);
  if (pb.model != MODEL_MULTI) return 1;
  for (int64_t i = 0; i < n; ++i) {
    double l[30], r[30], sl[12], sr[12], m[30], pp[30];
    GATHER(l, Ql, 30, n, i);
    GATHER(r, Qr, 30, n, i);
    GATHER(sl, spdL, 12, n, i);
    GATHER(sr, spdR, 12, n, i);
    hll_face(pb, l, r, sl, sr, m, pp);
    SCATTER(dm, m, 30, n, i);
    SCATTER(dp, pp, 30, n, i);
  }
  return 0;
}
void hyo_quadrature(int kind, double* x, double* w) {
  Quad6 q = kind == 0 ? gauss_legendre6_01() : gauss_lobatto6_01();
  for (int i = 0; i < 6; ++i) { x[i] = q.x[i]; w[i] = q.w[i]; }
}

// max_i max|speeds(Q_i)|, the CFL wave speed of main.jl:204-212.
double hyo_max_speed(const hyo_problem* p, const double* Q, int nthreads) {
  Problem pb = to_problem(p);
  int nx = pb.nx, nv = nvar_of(pb.model), ns = nspd_of(pb.model);
  std::vector<double> lam(nx);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int i = 0; i < nx; ++i) {
    double q[30], s[12];
    GATHER(q, Q, nv, nx, i);
    cell_speeds(pb, q, s);
    lam[i] = max_abs(s, ns);
  }
  double m = lam[0];
  for (int i = 1; i < nx; ++i) if (lam[i] > m) m = lam[i];
  return m;
}

// main.jl:202-227: advance Q (SoA [nvar][nx], in/out) while steps < max_steps
// (max_steps <= 0: no limit) and t < t_end. *t_io holds t on entry and exit.
int hyo_run(const hyo_problem* p, double* Q, int max_steps, double t_end, int nthreads, int literal,
            int* steps_done, double* t_io, double* dt_last) {
  Problem pb = to_problem(p);
  int nx = pb.nx, nv = nvar_of(pb.model);
  if (nx < 3) return 1;
  std::vector<double> q((size_t)nx * nv);
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < nv; ++k) q[(size_t)i * nv + k] = Q[(size_t)k * nx + i];
  double t = *t_io, dt = 0.0;
  int s = 0;
  while (t < t_end && (max_steps <= 0 || s < max_steps)) {
    dt = step(pb, q, literal, nthreads);
    t += dt;
    ++s;
  }
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < nv; ++k) Q[(size_t)k * nx + i] = q[(size_t)i * nv + k];
  *steps_done = s;
  *t_io = t;
  if (dt_last) *dt_last = dt;
  return 0;
}

// Advance n_steps with prescribed time steps dts[k] (Q SoA [nvar][nx], in/out).
int hyo_run_dts(const hyo_problem* p, double* Q, int n_steps, const double* dts, int nthreads) {
  Problem pb = to_problem(p);
  int nx = pb.nx, nv = nvar_of(pb.model);
  if (nx < 3) return 1;
  std::vector<double> q((size_t)nx * nv);
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < nv; ++k) q[(size_t)i * nv + k] = Q[(size_t)k * nx + i];
  for (int s = 0; s < n_steps; ++s) step(pb, q, 0, nthreads, (double*)nullptr, &dts[s]);
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < nv; ++k) Q[(size_t)k * nx + i] = q[(size_t)i * nv + k];
  return 0;
}

}  // extern "C"
