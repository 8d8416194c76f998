// Host build of the product's closed-form physics (hyp_physics.cuh) for the
// CPU unit tests: lets tests compare the GPU math against the oracle without a
// GPU. Compiled by tests/test_physics_host.py into a temporary shared library.
#include "../hyperelasticsolver_gb300/csrc/hyp_physics.cuh"
#include "../hyperelasticsolver_gb300/csrc/hyp_adjoint.cuh"
#include "../hyperelasticsolver_gb300/csrc/hyp_hank.cuh"
#include "../hyperelasticsolver_gb300/csrc/hyp_relax.cuh"

using namespace hyp;

extern "C" {

static EosC mk(const double* p) { return make_eos(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7]); }

void hs_finger(const double* A, double* G) { finger_A(A, G); }
void hs_invariants(const double* G, double* I) { invariants_general(G, I); }
double hs_energy(const double* ep, double S, const double* G) { return energy_SG(mk(ep), S, G); }
double hs_entropy(const double* ep, double e, const double* G) { return entropy_eG(mk(ep), e, G); }
void hs_stress(const double* ep, double S, const double* F, double* sig) { stress_SF(mk(ep), S, F, sig); }
void hs_acoustic(const double* ep, double S, const double* F, double* om) { acoustic_SF(mk(ep), S, F, om); }
double hs_spectral_radius(const double* a) { return spectral_radius(a); }
void hs_eig_moduli3(const double* a, double* m) { eig_moduli3(a, m); }
void hs_eig_sorted3(const double* a, double* m) { eig_sorted3(a, m); }
// two-phase pressure relaxation of one cell in place (30 values); returns its status
int hs_relax2(const double* ep1, const double* ep2, double* Q) {
  EosC e[2] = {mk(ep1), mk(ep2)};
  return relax_pressure2(e, Q);
}
// mean-stress pressure of one phase at e_int and distortion lam * A, and dp/de
void hs_relax_pressure(const double* ep, const double* A, double lam, double eint, double* out) {
  PhaseP r = relax_phase_pressure(mk(ep), A, lam, eint);
  out[0] = r.p;
  out[1] = r.dpde;
}

// one phase of a cell: q = [alpha, alpha*rho, alpha*rho*u(3), alpha*rho*E, alpha*rho*A(9)]
// out: [flux(14 after alpha), u1, cmax, S, status]
void hs_cell(const double* ep, const double* q, double* out) {
  EosC e = mk(ep);
  Prim P;
  int st = cons_to_prim(e, q[0], q + 2, q[5], q + 6, P);
  StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
  double s0[3];
  phase_flux(e, q[0], P, c, out, s0);
  out[14] = P.u[0];
  out[15] = phase_cmax(e, P, c);
  out[16] = e.cv * log(P.xm1 + 1.0);
  out[17] = st;
}

// single-phase cell at alpha = 1: q (14) -> out = [flux (14), lambda]
void hs_cell1(const double* ep, const double* q, double* out) {
  EosC e = mk(ep);
  CellFwd F = cell_forward(e, q);
  double s0[3];
  phase_flux(e, 1.0, F.P, F.c, out, s0);
  out[14] = fabs(F.P.u[0]) + phase_cmax(e, F.P, F.c);
}
// qb (14) += (df/dq)^T fb + (dlambda/dq) lb; eb = (dL/db0sq, dL/dk0)
int hs_cell1_vjp(const double* ep, const double* q, const double* fb, double lb, double* qb, double* eb) {
  EosC e = mk(ep);
  EosBar b{0.0, 0.0};
  int st = cell_vjp(e, q, fb, lb, qb, b);
  eb[0] = b.b0sq;
  eb[1] = b.k0;
  return st;
}
void hs_prim2cons1(const double* ep, const double* p, double* q) {
  EosC e = mk(ep);
  double p15[15], q15[15];
  p15[0] = 1.0;
  for (int t = 0; t < 14; ++t) p15[1 + t] = p[t];
  double den = p15[1];
  Kin k = kinematics(p15 + 6, det3(p15 + 6));
  Pows w = powers(e, k);
  double eint = e_cold(e, w) + e.cvt0 * w.Pg * (exp(p15[5] / e.cv) - 1.0) + e_shear(e, k, w);
  double ek = 0.5 * (p15[2] * p15[2] + p15[3] * p15[3] + p15[4] * p15[4]);
  q[0] = den;
  for (int c = 0; c < 3; ++c) q[1 + c] = den * p15[2 + c];
  q[4] = den * (eint + ek);
  for (int c = 0; c < 9; ++c) q[5 + c] = den * p15[6 + c];
  (void)q15;
}
void hs_prim2cons1_vjp(const double* ep, const double* p, const double* qb, double* pb, double* eb) {
  EosC e = mk(ep);
  EosBar b{0.0, 0.0};
  prim2cons_vjp(e, p, qb, pb, b);
  eb[0] = b.b0sq;
  eb[1] = b.k0;
}

// Hank2016: h = [rho0, mu, gamma, pres_inf, a]
double hs_hank_energy(const double* h, double den, double pres, const double* G) {
  return hank_energy(Hank{h[0], h[1], h[2], h[3], h[4]}, den, pres, G);
}
void hs_hank_stress(const double* h, double den, double pres, const double* F, double* sig) {
  hank_stress(Hank{h[0], h[1], h[2], h[3], h[4]}, den, pres, F, sig);
}
}
