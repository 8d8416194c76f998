// Host build of the product's closed-form physics (hyp_physics.cuh) for the
// CPU unit tests: lets tests compare the GPU math against the oracle without a
// GPU. Compiled by tests/test_physics_host.py into a temporary shared library.
#include "../hyperelasticsolver_gb300/csrc/hyp_physics.cuh"

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
}
