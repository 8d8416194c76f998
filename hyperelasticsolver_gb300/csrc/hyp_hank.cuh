// hyp_hank.cuh -- the Hank2016 equation of state (EquationsOfState.jl:305-366).
//
// The reference defines it at function level only:
//   energy(eos, den, pres, G)  = e_el(G) + (pres + gamma p_inf) / (den (gamma - 1)),
//   e_el = mu / (4 rho0) ((1 - 2a)/3 j1^2 + a j2 + 3 (a - 1)),
//   j1 = i1 / i3^(1/3),  j2 = (i1^2 - 2 i2) / i3^(2/3)   (invariants of G, Strains.jl:46-52);
//   pressure(eos, den, e_int, i) = (e_int - e_el) (gamma - 1) den - gamma p_inf;
//   stress(eos, den, pres, F) = -2 den G dE/dG with G = finger(inv(F)) = F^T F and
//     den, pres held fixed, so only e_el contributes.
// The gradient the reference takes with ForwardDiff is written in closed form:
//   d i1 = I, d i2 = i1 I - G^T, d i3 = cof(G),
//   d j1 = i3^(-1/3) d i1 - (1/3) i1 i3^(-4/3) d i3,
//   d j2 = i3^(-2/3) (2 i1 d i1 - 2 d i2) - (2/3) (i1^2 - 2 i2) i3^(-5/3) d i3.
#pragma once
#include "hyp_physics.cuh"

namespace hyp {

struct Hank {
  double rho0, mu, gamma, pres_inf, a;
};

HYP_HD double hank_e_el(const Hank& h, const double* inv3) {
  const double i1 = inv3[0], i2 = inv3[1], i3 = inv3[2];
  const double j1 = i1 / pow(i3, 1.0 / 3.0);
  const double j2 = (i1 * i1 - 2.0 * i2) / pow(i3, 2.0 / 3.0);
  return h.mu / (4.0 * h.rho0) * ((1.0 - 2.0 * h.a) / 3.0 * (j1 * j1) + h.a * j2 + 3.0 * (h.a - 1.0));
}

// energy(eos, den, pres, G) (EquationsOfState.jl:321-336), G column-major
HYP_HD double hank_energy(const Hank& h, double den, double pres, const double* G) {
  double inv3[3];
  invariants_general(G, inv3);
  const double e_h = (pres + h.gamma * h.pres_inf) / (den * (h.gamma - 1.0));
  return hank_e_el(h, inv3) + e_h;
}

// pressure(eos, den, e_int, i) (EquationsOfState.jl:338-352)
HYP_HD double hank_pressure(const Hank& h, double den, double e_int, const double* inv3) {
  return (e_int - hank_e_el(h, inv3)) * (h.gamma - 1.0) * den - h.gamma * h.pres_inf;
}

// stress(eos, den, pres, distortion) (EquationsOfState.jl:354-361), F and sigma column-major
HYP_HD void hank_stress(const Hank& h, double den, double /*pres*/, const double* F, double* sig) {
  double G[9];  // F^T F
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) G[i + 3 * j] = F[3 * i] * F[3 * j] + F[1 + 3 * i] * F[1 + 3 * j] + F[2 + 3 * i] * F[2 + 3 * j];
  double inv3[3];
  invariants_general(G, inv3);
  const double i1 = inv3[0], i2 = inv3[1], i3 = inv3[2];
  const double c13 = pow(i3, -1.0 / 3.0), c23 = pow(i3, -2.0 / 3.0);
  const double k = h.mu / (4.0 * h.rho0);
  const double j1 = i1 * c13;
  // de/dG = A1 d i1 + A2 d i2 + A3 d i3
  const double dj1_di1 = c13, dj1_di3 = -(1.0 / 3.0) * i1 * c13 / i3;
  const double dj2_di1 = 2.0 * i1 * c23, dj2_di2 = -2.0 * c23, dj2_di3 = -(2.0 / 3.0) * (i1 * i1 - 2.0 * i2) * c23 / i3;
  const double b = (1.0 - 2.0 * h.a) / 3.0 * 2.0 * j1;
  const double A1 = k * (b * dj1_di1 + h.a * dj2_di1);
  const double A2 = k * (h.a * dj2_di2);
  const double A3 = k * (b * dj1_di3 + h.a * dj2_di3);
  double D[9];  // column-major dE/dG
  for (int q = 0; q < 3; ++q)
    for (int p = 0; p < 3; ++p) {
      const int p1 = (p + 1) % 3, p2 = (p + 2) % 3, q1 = (q + 1) % 3, q2 = (q + 2) % 3;
      const double cof = G[p1 + 3 * q1] * G[p2 + 3 * q2] - G[p1 + 3 * q2] * G[p2 + 3 * q1];
      const double di2 = (p == q ? i1 : 0.0) - G[q + 3 * p];
      D[p + 3 * q] = A1 * (p == q ? 1.0 : 0.0) + A2 * di2 + A3 * cof;
    }
  for (int q = 0; q < 3; ++q)
    for (int p = 0; p < 3; ++p) {
      double s = 0.0;
      for (int m = 0; m < 3; ++m) s += G[p + 3 * m] * D[m + 3 * q];
      sig[p + 3 * q] = -2.0 * den * s;
    }
}

}  // namespace hyp
