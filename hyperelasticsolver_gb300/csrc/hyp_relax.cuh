// hyp_relax.cuh -- instantaneous pressure (and velocity) relaxation of a two-phase
// cell (FP64).
//
// The reference's two-phase model (HyperelasticityMPh.jl) carries two volume
// fractions, velocities and distortions per cell and has no relaxation terms; this
// is an extension, off by default (hyp_set_relaxation), with no reference to match.
// It follows the instantaneous pressure relaxation of Saurel, Petitpas & Berry
// (2009, J. Comput. Phys.), applied to hyperelastic phases as Favrie, Gavrilyuk &
// Saurel (2009, J. Comput. Phys.) do: the volume fractions move until both phases
// have one pressure p*, each phase's internal energy follows de_k = -p* dv_k, and a
// phase's distortion changes only in its volumetric part (A_k -> (v_k'/v_k)^(1/3) A_k,
// the unimodular shape kept). Per phase the pressure is the mean stress
// p = -tr(sigma)/3, sigma the Barton2009 Cauchy stress (EquationsOfState.jl:179-190)
// at the entropy that the internal energy and distortion give (:139-156); along an
// isotropic scaling of A at fixed entropy de = -p dv, so p is the phase's
// thermodynamic pressure.
//
// Unknowns alpha_1' (alpha_2' = 1 - alpha_1') and p*, with m_k = alpha_k rho_k and
// the velocities held:
//   v_k' = alpha_k' / m_k,   e_k' = e_k - p* (v_k' - v_k),
//   p_k(e_k', v_k') = p*     (k = 1, 2),
// solved by Newton's method (dp/de in closed form, dp/dv at fixed e by a central
// difference), with the step halved while it would leave 0 < alpha_1' < 1.
// Conserved: each phase's mass and momentum, the mixture's total energy
// (sum_k m_k (e_k' - e_k) = -p* sum_k (alpha_k' - alpha_k) = 0), alpha_1 + alpha_2.
// A cell with a phase below kRelaxMinAlpha is left as it is (a vanishing phase has no
// weight in the mixture and its relaxation is ill-conditioned). HYP_RELAX_MECHANICAL
// relaxes the velocities first (relax_velocity2): at a diffuse interface pressure
// relaxation alone let the two velocities drift apart and the minority phase's
// density collapse within 100 steps of the 8-cell smoothed interface.
#pragma once
#include "hyp_physics.cuh"

namespace hyp {

constexpr double kRelaxMinAlpha = 1e-5;
constexpr int kRelaxMaxIter = 40;
enum { HYP_CELL_RELAX = 8 };  // relaxation did not converge (cell left unrelaxed)

// Mean-stress pressure p = -tr(sigma)/3 of one phase at internal energy eint and
// distortion lam * A, and dp/de at that distortion.
struct PhaseP {
  double p, dpde;
};
HYP_HD PhaseP relax_phase_pressure(const EosC& e, const double* A, double lam, double eint) {
  double As[9];
  for (int c = 0; c < 9; ++c) As[c] = lam * A[c];
  Kin k = kinematics(As, det3(As));
  Pows w = powers(e, k);
  double xm1 = (eint - e_shear(e, k, w) - e_cold(e, w)) * e.inv_cvt0 * w.inv_Pg;
  const bool clamped = xm1 + 1.0 < 1e-6;
  if (clamped) xm1 = 1e-6 - 1.0;  // EquationsOfState.jl:152-154
  StressC c = stress_coeffs(e, k, w, xm1);
  const double rho_s = e.rho0 * k.s;
  const double trH = k.H.a00 + k.H.a11 + k.H.a22;
  PhaseP r;
  // tr sigma = -2 rho (cG i1 + cGG tr G^2 + 3 cI)
  r.p = (2.0 / 3.0) * rho_s * (c.cG * k.i1 + c.cGG * trH + 3.0 * c.cI);
  // only cI depends on e (through xm1): d cI / de = kE3g Pg1 p_det / (cv t0 Pg)
  r.dpde = clamped ? 0.0 : 2.0 * rho_s * e.kE3g * w.Pg1 * k.p * e.inv_cvt0 * w.inv_Pg;
  return r;
}

// Instantaneous velocity relaxation of one two-phase cell in place: both phases take
// the mixture velocity u* = sum m_k u_k / sum m_k (m_k = alpha_k rho_k); a phase's
// momentum becomes m_k u* and its total energy changes by m_k u* . (u* - u_k), which
// keeps the mixture's momentum and total energy and adds |u_k - u*|^2 / 2 to each
// phase's internal energy (the drag's dissipation). Applied before the pressure
// relaxation, it brings the cell to mechanical equilibrium (one velocity, one
// pressure), which the two-velocity model needs at a diffuse interface: pressure
// relaxation alone lets the phases' velocities drift apart there.
HYP_HD int relax_velocity2(const EosC* eos, double* Q) {
  Prim P[2];
  int st = 0;
  for (int k = 0; k < 2; ++k) st |= cons_to_prim(eos[k], Q[15 * k], Q + 15 * k + 2, Q[15 * k + 5], Q + 15 * k + 6, P[k]);
  if (st) return st;
  if (!(Q[0] >= kRelaxMinAlpha && Q[15] >= kRelaxMinAlpha)) return 0;
  const double m0 = P[0].den, m1 = P[1].den, im = 1.0 / (m0 + m1);
  double us[3];
  for (int c = 0; c < 3; ++c) us[c] = (m0 * P[0].u[c] + m1 * P[1].u[c]) * im;
  for (int k = 0; k < 2; ++k) {
    double* q = Q + 15 * k;
    const double m = P[k].den;
    const double w = us[0] * (us[0] - P[k].u[0]) + us[1] * (us[1] - P[k].u[1]) + us[2] * (us[2] - P[k].u[2]);
    q[5] = q[5] + m * w;
    for (int c = 0; c < 3; ++c) q[2 + c] = m * us[c];
  }
  return 0;
}

// Relax one two-phase cell in place (30 conservative values, HyperelasticityMPh.jl:80-84).
// Returns HYP_CELL_* bits; 0 also when the cell is left as it is.
HYP_HD int relax_pressure2(const EosC* eos, double* Q);
// The relaxation of a hyp_set_relaxation mode: 1 pressure, 2 velocity then pressure.
HYP_HD int relax_cell2(const EosC* eos, int mode, double* Q) {
  if (mode == 2) {
    const int st = relax_velocity2(eos, Q);
    if (st) return st;
  }
  return relax_pressure2(eos, Q);
}
HYP_HD int relax_pressure2(const EosC* eos, double* Q) {
  Prim P[2];
  int st = 0;
  for (int k = 0; k < 2; ++k) st |= cons_to_prim(eos[k], Q[15 * k], Q + 15 * k + 2, Q[15 * k + 5], Q + 15 * k + 6, P[k]);
  if (st) return st;
  const double a0[2] = {Q[0], Q[15]};
  if (!(a0[0] >= kRelaxMinAlpha && a0[1] >= kRelaxMinAlpha)) return 0;
  double m[2], v[2];
  for (int k = 0; k < 2; ++k) {
    m[k] = P[k].den;  // alpha_k rho_k (rho from det(alpha rho A / alpha), as cons2prim)
    v[k] = a0[k] / m[k];
  }
  const double dvdx[2] = {1.0 / m[0], -1.0 / m[1]};
  double x = a0[0];
  double ps = 0.0;
  for (int k = 0; k < 2; ++k) ps += a0[k] * relax_phase_pressure(eos[k], P[k].A, 1.0, P[k].e_int).p;
  double pscale = fabs(ps);
  for (int k = 0; k < 2; ++k) pscale = fmax(pscale, eos[k].k0 * eos[k].rho0);
  bool done = false;
  for (int it = 0; it < kRelaxMaxIter && !done; ++it) {
    double F[2], Jx[2], Jp[2];
    for (int k = 0; k < 2; ++k) {
      const double ak = k == 0 ? x : 1.0 - x;
      const double vk = ak / m[k];
      const double ek = P[k].e_int - ps * (vk - v[k]);
      const PhaseP r = relax_phase_pressure(eos[k], P[k].A, cbrt(vk / v[k]), ek);
      const double h = 1e-7 * vk;
      const double pp = relax_phase_pressure(eos[k], P[k].A, cbrt((vk + h) / v[k]), ek).p;
      const double pm = relax_phase_pressure(eos[k], P[k].A, cbrt((vk - h) / v[k]), ek).p;
      const double dpdv = (pp - pm) / (2.0 * h);
      F[k] = r.p - ps;
      Jx[k] = (dpdv - r.dpde * ps) * dvdx[k];
      Jp[k] = -r.dpde * (vk - v[k]) - 1.0;
    }
    const double det = Jx[0] * Jp[1] - Jx[1] * Jp[0];
    if (!(fabs(det) > 0.0) || !isfinite(det)) break;
    double dx = (-F[0] * Jp[1] + F[1] * Jp[0]) / det;
    double dp = (-Jx[0] * F[1] + Jx[1] * F[0]) / det;
    for (int h = 0; h < 60 && !(x + dx > 0.0 && x + dx < 1.0); ++h) {
      dx *= 0.5;
      dp *= 0.5;
    }
    x += dx;
    ps += dp;
    done = fabs(dx) <= 1e-14 && fabs(dp) <= 1e-13 * pscale;
  }
  if (!done || !(x > 0.0 && x < 1.0) || !isfinite(ps)) return HYP_CELL_RELAX;
  for (int k = 0; k < 2; ++k) {
    const double ak = k == 0 ? x : 1.0 - x;
    const double vk = ak / m[k];
    const double ek = P[k].e_int - ps * (vk - v[k]);
    const double lam = cbrt(vk / v[k]);
    double* q = Q + 15 * k;
    const double ke = 0.5 * (P[k].u[0] * P[k].u[0] + P[k].u[1] * P[k].u[1] + P[k].u[2] * P[k].u[2]);
    q[0] = ak;
    q[5] = m[k] * (ek + ke);
    for (int c = 0; c < 9; ++c) q[6 + c] *= lam;  // alpha rho A: mass held, A scaled
  }
  return 0;
}

}  // namespace hyp
