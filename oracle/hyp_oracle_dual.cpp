// oracle/hyp_oracle_dual.cpp -- forward-mode derivative of a single-phase run.
//
// TEST INFRASTRUCTURE ONLY (the oracle): checks the device adjoint. The whole
// restatement of the reference run (prim2cons, main.jl:202-227 steps with the
// reference's own nested-dual stress and acoustic tensor, cons2prim) is
// instantiated with a dual number carrying 15 partials: the 13 left-state
// parameters (rho, u(3), A(9) column-major) and the Barton2009 moduli b0sq, k0
// (EquationsOfState.jl:111-112, each with the other held fixed). One run gives
// the value and the gradient of L = 1/2 sum_i (rho_i - target_i)^2.
#include <cstdint>
#include <vector>
#include "hyp_oracle.hpp"

using namespace hyp_oracle;

namespace {
using O = Dual<double, 15>;
const int kPrimIndex[13] = {0, 1, 2, 3, 5, 6, 7, 8, 9, 10, 11, 12, 13};  // theta -> (rho, u, S, A)
}

extern "C" {

typedef struct { double rho0, c0, cv, t0, b0, alpha, beta, gamma; } hyo_eos_d;
typedef struct {
  int model, flux, bc, nx;
  double X, cfl;
  hyo_eos_d eos[2];
} hyo_problem_d;

// prim_left / prim_right: (rho, u(3), S, A(9)); cells i < nx/2 hold the left state
// (main.jl:99-106). Returns 0 on success.
int hyo_misfit_grad_dual(const hyo_problem_d* p, const double* prim_left, const double* prim_right, int n_steps,
                         const double* target, int nthreads, double* loss, double* grad) {
  if (p->model != MODEL_SINGLE || p->nx < 3) return 1;
  ProblemT<O> pb;
  pb.model = p->model;
  pb.flux = p->flux;
  pb.bc = p->bc;
  pb.nx = p->nx;
  pb.X = p->X;
  pb.cfl = p->cfl;
  for (int ph = 0; ph < 2; ++ph) {
    const hyo_eos_d& s = p->eos[ph];
    Barton b = make_barton(s.rho0, s.c0, s.cv, s.t0, s.b0, s.alpha, s.beta, s.gamma);
    BartonT<O>& e = pb.eos[ph];
    e.rho0 = b.rho0; e.c0 = b.c0; e.cv = b.cv; e.t0 = b.t0; e.b0 = b.b0;
    e.alpha = b.alpha; e.beta = b.beta; e.gamma = b.gamma;
    e.b0sq = O(b.b0sq);
    e.k0 = O(b.k0);
  }
  pb.eos[0].b0sq.d[13] = 1.0;
  pb.eos[0].k0.d[14] = 1.0;
  O pl[15], pr[15], ql[15], qr[15];
  pl[0] = O(1.0);
  pr[0] = O(1.0);
  for (int k = 0; k < 14; ++k) {
    pl[1 + k] = O(prim_left[k]);
    pr[1 + k] = O(prim_right[k]);
  }
  for (int j = 0; j < 13; ++j) pl[1 + kPrimIndex[j]].d[j] = 1.0;
  prim2cons(pb.eos[0], pl, ql);
  prim2cons(pb.eos[0], pr, qr);
  const int nx = p->nx;
  std::vector<O> q((size_t)nx * 14);
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < 14; ++k) q[(size_t)i * 14 + k] = (i < nx / 2.0) ? ql[1 + k] : qr[1 + k];
  for (int s = 0; s < n_steps; ++s) step(pb, q, 0, nthreads);
  O L(0.0);
  for (int i = 0; i < nx; ++i) {
    O q15[15], p15[15];
    expand1(&q[(size_t)i * 14], q15);
    cons2prim(pb.eos[0], q15, p15);
    O r = p15[1] - target[i];
    L = L + 0.5 * (r * r);
  }
  *loss = L.v;
  for (int j = 0; j < 15; ++j) grad[j] = L.d[j];
  return 0;
}

}  // extern "C"
