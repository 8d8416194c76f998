// hyp_physics_mph.cuh -- two-phase pieces of the step (FP64): the
// non-conservative matrix B of HyperelasticityMPh.jl:178-250 and the
// path-conservative HLL fluctuations of NumFluxes.jl:85-132.
//
// A two-phase cell is the reference's 30-vector: for p = 1, 2 the phase state
// [alpha_p, alpha_p rho_p, alpha_p rho_p u_p(3), alpha_p rho_p E_p, alpha_p rho_p A_p(9)].
// Only column 1 of each 15x15 phase block of B is non-zero, so B is carried as
// the 30-vector bcol (bcol[r] = B[r,1] for phase-1 rows, B[r,16] for phase-2
// rows) and B dQ = bcol * dalpha_p.
#pragma once
#include "hyp_physics.cuh"

namespace hyp {

// 6-point Gauss-Legendre nodes and weights on [0, 1], ascending (NumFluxes.jl:94-95).
struct Quad6D {
  double x[6], w[6];
};

// What B needs from one phase (HyperelasticityMPh.jl:186-217).
struct PhaseB {
  double true_den;
  double u[3];
  double A[9];
  double K0[3];  // column 1 of K_p = strs_p / frac_p = sigma_p  (sigma symmetric: = row 1)
  double T;      // temperature dE/dS = t0 p^(gamma/2) exp(S/cv)  (:212)
};

HYP_HD int phase_b(const EosC& e, const double* q, PhaseB& b) {
  Prim P;
  int st = cons_to_prim(e, q[0], q + 2, q[5], q + 6, P);
  StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
  stress_row0(e.rho0 * P.k.s, P.k, c, b.K0);
  b.T = e.t0 * P.w.Pg * (P.xm1 + 1.0);
  b.true_den = P.true_den;
  for (int a = 0; a < 3; ++a) b.u[a] = P.u[a];
  for (int k = 0; k < 9; ++k) b.A[k] = P.A[k];
  return st;
}

// bcol of B(Q) (HyperelasticityMPh.jl:178-250) with omega = 0, k = (1/2, 1/2), beta = 0.
HYP_HD int noncons_bcol(const EosC* eos, const double* Q, double* bcol) {
  PhaseB b[2];
  int st = phase_b(eos[0], Q, b[0]) | phase_b(eos[1], Q + 15, b[1]);
  double uI[3], sI[3];
  for (int a = 0; a < 3; ++a) uI[a] = 0.5 * b[0].u[a] + 0.5 * b[1].u[a];
  const double iden = 1.0 / (0.5 * b[0].T + 0.5 * b[1].T);
  for (int a = 0; a < 3; ++a) sI[a] = ((0.5 * b[1].T) * b[0].K0[a] + (0.5 * b[0].T) * b[1].K0[a]) * iden;
  for (int p = 0; p < 2; ++p) {
    double* r = bcol + 15 * p;
    const PhaseB& B = b[p];
    r[0] = uI[0];
    r[1] = 0.0;
    r[2] = sI[0];
    r[3] = sI[1];
    r[4] = sI[2];
    r[5] = (sI[0] * uI[0] + sI[1] * uI[1]) + sI[2] * uI[2];
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) r[6 + a + 3 * c] = (B.true_den * B.A[3 * c]) * B.u[a];
    double dv[3] = {uI[0] - B.u[0], uI[1] - B.u[1], uI[2] - B.u[2]};
    for (int c = 0; c < 3; ++c)
      r[6 + 3 * c] += B.true_den * ((B.A[3 * c] * dv[0] + B.A[1 + 3 * c] * dv[1]) + B.A[2 + 3 * c] * dv[2]);
  }
  return st;
}

// Wave-speed bounds of a two-phase state: min and max over both phases of
// u1 -+ c_max (HyperelasticityMPh.jl:252-266).
HYP_HD int speeds2(const EosC* eos, const double* Q, double& smin, double& smax) {
  int st = 0;
  for (int p = 0; p < 2; ++p) {
    const double* q = Q + 15 * p;
    Prim P;
    st |= cons_to_prim(eos[p], q[0], q + 2, q[5], q + 6, P);
    StressC c = stress_coeffs(eos[p], P.k, P.w, P.xm1);
    const double cm = phase_cmax(eos[p], P, c);
    const double lo = P.u[0] - cm, hi = P.u[0] + cm;
    if (p == 0 || lo < smin) smin = lo;
    if (p == 0 || hi > smax) smax = hi;
  }
  return st;
}

// Physical flux of both phases (HyperelasticityMPh.jl:140-175), 30 components.
HYP_HD int flux2(const EosC* eos, const double* Q, double* F) {
  int st = 0;
  for (int p = 0; p < 2; ++p) {
    const double* q = Q + 15 * p;
    Prim P;
    st |= cons_to_prim(eos[p], q[0], q + 2, q[5], q + 6, P);
    StressC c = stress_coeffs(eos[p], P.k, P.w, P.xm1);
    double s0[3];
    F[15 * p] = 0.0;
    phase_flux(eos[p], q[0], P, c, F + 15 * p + 1, s0);
  }
  return st;
}

// acc[k] += sum_i (w_i * B_i[k]) * (Qb - Qa)[alpha_p(k)] along psi(s) = Qa (1 - s) + Qb s
// (NumFluxes.jl:97-107), starting from acc as given.
HYP_HD int path_integral_add(const EosC* eos, const Quad6D& qd, const double* Qa, const double* Qb, double* acc) {
  const double da0 = Qb[0] - Qa[0], da1 = Qb[15] - Qa[15];
  int st = 0;
  double u[30], bc[30];
  for (int i = 0; i < 6; ++i) {
    const double s = qd.x[i], oms = 1.0 - s;
    for (int k = 0; k < 30; ++k) u[k] = Qa[k] * oms + Qb[k] * s;
    st |= noncons_bcol(eos, u, bc);
    // w B dQ = bcol (w d alpha): one multiply-add per row; rows 1 and 16 of B are 0
    const double wd0 = qd.w[i] * da0, wd1 = qd.w[i] * da1;
    for (int k = 0; k < 30; ++k)
      if (k != 1 && k != 16) acc[k] = fma(bc[k], k < 15 ? wd0 : wd1, acc[k]);
  }
  return st;
}

// Path-conservative HLL fluctuations D-, D+ of one face (NumFluxes.jl:85-132).
// fl, fr: physical fluxes of QL, QR; sminL = min speed of QL, smaxR = max speed of QR.
HYP_HD int hll_face2(const EosC* eos, const Quad6D& qd, const double* QL, const double* QR, const double* fl,
                     const double* fr, double sminL, double smaxR, double* dm, double* dp) {
  double Qm[30];
  for (int k = 0; k < 30; ++k) Qm[k] = 0.5 * (QL[k] + QR[k]);
  double mmin, mmax;
  int st = speeds2(eos, Qm, mmin, mmax);
  double sl = 0.0;
  if (mmin < sl) sl = mmin;
  if (sminL < sl) sl = sminL;
  double sr = 0.0;
  if (mmax > sr) sr = mmax;
  if (smaxR > sr) sr = smaxR;
  const double idsr = 1.0 / (sr - sl);
  double acc[30], Qh[30];
  for (int k = 0; k < 30; ++k) acc[k] = 0.0;
  st |= path_integral_add(eos, qd, QL, QR, acc);  // B_int(Q_l, Q_r)
  for (int k = 0; k < 30; ++k) {
    const double pint = (acc[k] + fr[k]) - fl[k];
    Qh[k] = ((QR[k] * sr - QL[k] * sl) - pint) * idsr;
  }
  // inner = ((f_r - f_l) + B_int(Q_l, Q_hll)) + B_int(Q_hll, Q_r), each integral summed first
  double b2[30];
  for (int k = 0; k < 30; ++k) {
    acc[k] = 0.0;
    b2[k] = 0.0;
  }
  st |= path_integral_add(eos, qd, QL, Qh, acc);
  st |= path_integral_add(eos, qd, Qh, QR, b2);
  const double cm = (-sl) * idsr, cp = sr * idsr, cq = (sl * sr) * idsr;
  for (int k = 0; k < 30; ++k) {
    const double inner = ((fr[k] - fl[k]) + acc[k]) + b2[k];
    const double jump = QR[k] - QL[k];
    dm[k] = cm * inner + cq * jump;
    dp[k] = cp * inner - cq * jump;
  }
  return st;
}

// Path-conservative Lax-Friedrichs face of the two-phase model (NumFluxes.jl:25-60):
// conservative part F = (f_l + f_r)/2 - lambda (Q_r - Q_l)/2 and D- = D+ = half the
// path integral of B with the 6-point Gauss-Lobatto rule (NumFluxes.jl:36-47).
HYP_HD int lxf_face2(const EosC* eos, const Quad6D& lobatto, const double* QL, const double* QR, const double* fl,
                     const double* fr, double lambda, double* F, double* dm, double* dp) {
  const double hl = lambda * 0.5;
  for (int k = 0; k < 30; ++k) F[k] = 0.5 * (fl[k] + fr[k]) - hl * (QR[k] - QL[k]);
  double acc[30];
  for (int k = 0; k < 30; ++k) acc[k] = 0.0;
  const int st = path_integral_add(eos, lobatto, QL, QR, acc);
  for (int k = 0; k < 30; ++k) dm[k] = dp[k] = 0.5 * acc[k];
  return st;
}

}  // namespace hyp
