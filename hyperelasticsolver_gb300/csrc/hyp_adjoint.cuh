// hyp_adjoint.cuh -- reverse-mode derivatives (vector-Jacobian products) of the
// single-phase FP64 cell functions of hyp_physics.cuh, written by hand.
//
// For one cell with state q (14) the step consumes the physical flux f(q)
// (HyperelasticityMPh.jl:146-175 at alpha = 1) and the wave-speed bound
// lambda(q) = |u1| + sqrt(max |eig(Omega)|) (HyperelasticityMPh.jl:252-266,
// Omega = acoustic(eos, S, A, e1), EquationsOfState.jl:223-246).  cell_vjp
// returns
//     qb += (df/dq)^T fb + (dlambda/dq) lb,      eb += (df/deos)^T fb + (dlambda/deos) lb
// for the two Barton2009 moduli b0sq (shear, b0^2) and k0 (bulk, c0^2 - 4/3 b0^2),
// each held fixed while the other varies (EquationsOfState.jl:111-112).
//
// Each function below reverses one forward function of hyp_physics.cuh,
// statement by statement, in the opposite order: the primal is recomputed
// first, then the adjoints flow back through
//   eigenvalue -> acoustic tensor -> stress row 1 -> stress coefficients ->
//   entropy argument -> powers of det G -> kinematics (G, G^2, invariants) ->
//   cons2prim (det, sqrt, divisions).
// The derivative of the top eigenvalue nu of the (non-symmetric) 3x3 Omega is
// d nu / d Omega_ij = Cof(nu I - Omega)_ij / p'(nu), p(x) = det(x I - Omega),
// p'(nu) = tr adj(nu I - Omega): the implicit-function form, so the Newton
// iterations of the eigen-solve need no reverse pass.
// Non-smooth points follow the derivative convention of a central difference:
// d|u1|/du1 = 0 at u1 = 0, and no derivative flows through the clamped entropy
// argument (EquationsOfState.jl:153).
#pragma once
#include "hyp_physics.cuh"

namespace hyp {

// Adjoints of the two moduli differentiated.
struct EosBar {
  double b0sq, k0;
};

HYP_HD double& sym_ref(Sym& s, int i, int j) {
  if (i == j) return i == 0 ? s.a00 : (i == 1 ? s.a11 : s.a22);
  int k = i + j;
  return k == 1 ? s.a01 : (k == 2 ? s.a02 : s.a12);
}
HYP_HD Sym sym_zero() { return Sym{0.0, 0.0, 0.0, 0.0, 0.0, 0.0}; }

struct PowsBar {
  double Pa, Pa1, Pa2, Pb, Pb1, Pb2, Pg, Pg1, Pg2, inv_Pg, Pam1;
};
HYP_HD PowsBar pows_zero() { return PowsBar{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}; }

struct StressBar {
  double cG, cGG, cI, E3;
};

// Adjoint of p from the adjoints of every power p^x (powers(), both branches):
// d p^x / dp = x p^x / p.  Pam1 = Pa - 1.
HYP_HD double powers_vjp(const EosC& e, const Kin& k, const Pows& w, const PowsBar& b) {
  const double ha = 0.5 * e.alpha, hb = 0.5 * e.beta, hg = 0.5 * e.gamma;
  double acc = (b.Pa + b.Pam1) * ha * w.Pa + b.Pa1 * (ha - 1.0) * w.Pa1 + b.Pa2 * (ha - 2.0) * w.Pa2;
  acc += b.Pb * hb * w.Pb + b.Pb1 * (hb - 1.0) * w.Pb1 + b.Pb2 * (hb - 2.0) * w.Pb2;
  acc += b.Pg * hg * w.Pg + b.Pg1 * (hg - 1.0) * w.Pg1 + b.Pg2 * (hg - 2.0) * w.Pg2;
  acc -= b.inv_Pg * hg * w.inv_Pg;
  return acc / k.p;
}

// Reverse of kinematics_s(A, s, 1/s) (FP64 branch): adjoints of the stored G, H
// entries, of i1, psi and p -> adjoint of A (accumulated) and of s (returned).
HYP_HD double kinematics_vjp(const double* A, const Kin& k, Sym Gb, Sym Hb, double i1b, double psib, double pb,
                             double* Ab) {
  // psi = i1^2/3 - i2, i2 = (i1^2 - tr H)/2  ->  psi = -i1^2/6 + tr H / 2
  i1b -= psib * k.i1 * (1.0 / 3.0);
  Hb.a00 += 0.5 * psib;
  Hb.a11 += 0.5 * psib;
  Hb.a22 += 0.5 * psib;
  Gb.a00 += i1b;
  Gb.a11 += i1b;
  Gb.a22 += i1b;
  // H = G G. With the full (symmetric) adjoint Hf (off-diagonal stored adjoints
  // split in half), Gf = Hf G + G Hf, and the stored off-diagonal adjoint is 2 Gf_ab.
  {
    double g[3][3], h[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        g[i][j] = sym_at(k.G, i, j);
        h[i][j] = (i == j ? 1.0 : 0.5) * sym_at(Hb, i, j);
      }
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        double s = 0.0;
        for (int m = 0; m < 3; ++m) s += h[i][m] * g[m][j] + g[i][m] * h[m][j];
        sym_ref(Gb, i, j) += (i == j ? 1.0 : 2.0) * s;
      }
  }
  // M = A A^T; G = adj(M) p (stored entries as in kinematics_s)
  const double m00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  const double m11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  const double m22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  const double m01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  const double m02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  const double m12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  const double j00 = m11 * m22 - m12 * m12, j11 = m00 * m22 - m02 * m02, j22 = m00 * m11 - m01 * m01;
  const double j01 = m02 * m12 - m01 * m22, j02 = m01 * m12 - m02 * m11, j12 = m01 * m02 - m00 * m12;
  pb += Gb.a00 * j00 + Gb.a11 * j11 + Gb.a22 * j22 + Gb.a01 * j01 + Gb.a02 * j02 + Gb.a12 * j12;
  const double p = k.p;
  const double b00 = Gb.a00 * p, b11 = Gb.a11 * p, b22 = Gb.a22 * p;
  const double b01 = Gb.a01 * p, b02 = Gb.a02 * p, b12 = Gb.a12 * p;
  double M00 = b11 * m22 + b22 * m11 - b12 * m12;
  double M11 = b00 * m22 + b22 * m00 - b02 * m02;
  double M22 = b00 * m11 + b11 * m00 - b01 * m01;
  double M01 = -2.0 * b22 * m01 - b01 * m22 + b02 * m12 + b12 * m02;
  double M02 = -2.0 * b11 * m02 + b01 * m12 - b02 * m11 + b12 * m01;
  double M12 = -2.0 * b00 * m12 + b01 * m02 + b02 * m01 - b12 * m00;
  // M = A A^T (column-major A[a + 3c])
  for (int c = 0; c < 3; ++c) {
    const double a0 = A[3 * c], a1 = A[1 + 3 * c], a2 = A[2 + 3 * c];
    Ab[3 * c] += 2.0 * M00 * a0 + M01 * a1 + M02 * a2;
    Ab[1 + 3 * c] += 2.0 * M11 * a1 + M01 * a0 + M12 * a2;
    Ab[2 + 3 * c] += 2.0 * M22 * a2 + M02 * a0 + M12 * a1;
  }
  // p = s^2
  return 2.0 * k.s * pb;
}

// Reverse of entropy_xm1 (no derivative through the clamp).
HYP_HD void entropy_xm1_vjp(const EosC& e, double e_int, const Kin& k, const Pows& w, double xm1b, double& eintb,
                            PowsBar& wb, double& psib, EosBar& eb) {
  const double z = e_int - e_shear(e, k, w) - e_cold(e, w);
  if (z * e.inv_cvt0 * w.inv_Pg + 1.0 < 1e-6) return;
  const double zb = xm1b * e.inv_cvt0 * w.inv_Pg;
  wb.inv_Pg += xm1b * z * e.inv_cvt0;
  eintb += zb;
  // e_shear = 0.5 b0sq Pb psi
  eb.b0sq -= zb * 0.5 * w.Pb * k.psi;
  wb.Pb -= zb * 0.5 * e.b0sq * k.psi;
  psib -= zb * 0.5 * e.b0sq * w.Pb;
  // e_cold = kU Pam1^2, kU = k0 / (2 alpha^2)
  eb.k0 -= zb * w.Pam1 * w.Pam1 * 0.5 / (e.alpha * e.alpha);
  wb.Pam1 -= zb * 2.0 * e.kU * w.Pam1;
}

// Reverse of stress_coeffs.
HYP_HD void stress_coeffs_vjp(const EosC& e, const Kin& k, const Pows& w, double xm1, const StressC& c, StressBar cb,
                              PowsBar& wb, double& i1b, double& pb, double& psib, double& xm1b, EosBar& eb) {
  // cI = E3 p
  cb.E3 += cb.cI * k.p;
  pb += cb.cI * c.E3;
  // cGG = -E2, cG = E1 + E2 i1, E1 = b0sq/3 Pb i1, E2 = -b0sq/2 Pb
  const double E2 = -0.5 * e.b0sq * w.Pb;
  const double E1b = cb.cG;
  const double E2b = -cb.cGG + cb.cG * k.i1;
  i1b += cb.cG * E2;
  eb.b0sq += E1b * w.Pb * k.i1 * (1.0 / 3.0);
  wb.Pb += E1b * e.b0sq_3 * k.i1;
  i1b += E1b * e.b0sq_3 * w.Pb;
  eb.b0sq -= 0.5 * E2b * w.Pb;
  wb.Pb -= 0.5 * e.b0sq * E2b;
  // E3 = kE3a Pam1 Pa1 + kE3g Pg1 xm1 + kE3b Pb1 psi; kE3a = k0/(2 alpha), kE3b = b0sq beta/4
  eb.k0 += cb.E3 * w.Pam1 * w.Pa1 / (2.0 * e.alpha);
  wb.Pam1 += cb.E3 * e.kE3a * w.Pa1;
  wb.Pa1 += cb.E3 * e.kE3a * w.Pam1;
  wb.Pg1 += cb.E3 * e.kE3g * xm1;
  xm1b += cb.E3 * e.kE3g * w.Pg1;
  eb.b0sq += cb.E3 * w.Pb1 * k.psi * e.beta / 4.0;
  wb.Pb1 += cb.E3 * e.kE3b * k.psi;
  psib += cb.E3 * e.kE3b * w.Pb1;
}

// Reverse of acoustic_omega: om_b (column-major 3x3) -> adjoints of its inputs.
HYP_HD void acoustic_omega_vjp(const EosC& e, const Kin& k, const Pows& w, const StressC& c, double xm1,
                               const double* omb, Sym& Gb, Sym& Hb, double& i1b, double& pb, double& psib,
                               PowsBar& wb, StressBar& cb, double& xm1b, double* s0rb, EosBar& eb) {
  const double bs6 = e.b0sq_6;
  for (int j = 0; j < 3; ++j) {
    const double G0j = sym_at(k.G, 0, j), H0j = sym_at(k.H, 0, j);
    const double di1 = -2.0 * G0j;
    const double dpsi = (2.0 / 3.0) * k.i1 * G0j - 2.0 * H0j;
    double dp = 0.0, dPb = 0.0, dPa = 0.0, dPa1 = 0.0, dPg1 = 0.0, dPb1 = 0.0, dcG, dcGG, dE3;
    if (j == 0) {
      dp = -2.0 * k.p;
      dPb = 0.5 * e.beta * w.Pb1 * dp;
      dPa = 0.5 * e.alpha * w.Pa1 * dp;
      dPa1 = (0.5 * e.alpha - 1.0) * w.Pa2 * dp;
      dPg1 = (0.5 * e.gamma - 1.0) * w.Pg2 * dp;
      dPb1 = (0.5 * e.beta - 1.0) * w.Pb2 * dp;
      dcG = -bs6 * (dPb * k.i1 + w.Pb * di1);
      dcGG = 0.5 * e.b0sq * dPb;
      dE3 = e.kE3a * (dPa * w.Pa1 + w.Pam1 * dPa1) + e.kE3g * dPg1 * xm1 + e.kE3b * (dPb1 * k.psi + w.Pb1 * dpsi);
    } else {
      dcG = -bs6 * w.Pb * di1;
      dcGG = 0.0;
      dE3 = e.kE3b * w.Pb1 * dpsi;
    }
    double dcGb = 0.0, dcGGb = 0.0, dcIb = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double ob = omb[i + 3 * j];
      if (j == 0) s0rb[i] -= ob;
      const double vb = -2.0 * ob;
      const double G0i = sym_at(k.G, 0, i), H0i = sym_at(k.H, 0, i), Gij = sym_at(k.G, i, j);
      const double dG0i = -((i == 0 ? G0j : 0.0) + Gij);
      const double dH0i = -(G0j * G0i + sym_at(k.H, i, j) + (i == 0 ? H0j : 0.0) + k.G.a00 * Gij);
      // v = dcG G0i + cG dG0i + dcGG H0i + cGG dH0i + [i==0] dcI
      dcGb += vb * G0i;
      sym_ref(Gb, 0, i) += vb * dcG;
      cb.cG += vb * dG0i;
      const double dG0ib = vb * c.cG;
      dcGGb += vb * H0i;
      sym_ref(Hb, 0, i) += vb * dcGG;
      cb.cGG += vb * dH0i;
      const double dH0ib = vb * c.cGG;
      if (i == 0) dcIb += vb;
      if (i == 0) sym_ref(Gb, 0, j) -= dG0ib;
      sym_ref(Gb, i, j) -= dG0ib;
      sym_ref(Gb, 0, j) -= dH0ib * G0i;
      sym_ref(Gb, 0, i) -= dH0ib * G0j;
      sym_ref(Hb, i, j) -= dH0ib;
      if (i == 0) sym_ref(Hb, 0, j) -= dH0ib;
      Gb.a00 -= dH0ib * Gij;
      sym_ref(Gb, i, j) -= dH0ib * k.G.a00;
    }
    double dpsib = 0.0, di1b = 0.0;
    if (j == 0) {
      // dcI = dE3 p + E3 dp
      const double dE3b = dcIb * k.p;
      pb += dcIb * dE3;
      cb.E3 += dcIb * dp;
      double dpb = dcIb * c.E3;
      // dE3
      eb.k0 += dE3b * (dPa * w.Pa1 + w.Pam1 * dPa1) / (2.0 * e.alpha);
      const double dPab = dE3b * e.kE3a * w.Pa1;
      wb.Pa1 += dE3b * e.kE3a * dPa;
      wb.Pam1 += dE3b * e.kE3a * dPa1;
      const double dPa1b = dE3b * e.kE3a * w.Pam1;
      const double dPg1b = dE3b * e.kE3g * xm1;
      xm1b += dE3b * e.kE3g * dPg1;
      eb.b0sq += dE3b * (dPb1 * k.psi + w.Pb1 * dpsi) * e.beta / 4.0;
      const double dPb1b = dE3b * e.kE3b * k.psi;
      psib += dE3b * e.kE3b * dPb1;
      wb.Pb1 += dE3b * e.kE3b * dpsi;
      dpsib += dE3b * e.kE3b * w.Pb1;
      // dcGG = b0sq/2 dPb
      eb.b0sq += 0.5 * dcGGb * dPb;
      double dPbb = 0.5 * e.b0sq * dcGGb;
      // dcG = -b0sq/6 (dPb i1 + Pb di1)
      eb.b0sq -= dcGb * (dPb * k.i1 + w.Pb * di1) * (1.0 / 6.0);
      dPbb -= bs6 * dcGb * k.i1;
      i1b -= bs6 * dcGb * dPb;
      wb.Pb -= bs6 * dcGb * di1;
      di1b -= bs6 * dcGb * w.Pb;
      // dPx = coefficient * Px' * dp
      wb.Pb1 += dPbb * 0.5 * e.beta * dp;
      dpb += dPbb * 0.5 * e.beta * w.Pb1;
      wb.Pa1 += dPab * 0.5 * e.alpha * dp;
      dpb += dPab * 0.5 * e.alpha * w.Pa1;
      wb.Pa2 += dPa1b * (0.5 * e.alpha - 1.0) * dp;
      dpb += dPa1b * (0.5 * e.alpha - 1.0) * w.Pa2;
      wb.Pg2 += dPg1b * (0.5 * e.gamma - 1.0) * dp;
      dpb += dPg1b * (0.5 * e.gamma - 1.0) * w.Pg2;
      wb.Pb2 += dPb1b * (0.5 * e.beta - 1.0) * dp;
      dpb += dPb1b * (0.5 * e.beta - 1.0) * w.Pb2;
      // dp = -2 p
      pb -= 2.0 * dpb;
    } else {
      // dcI = dE3 p, dE3 = kE3b Pb1 dpsi, dcG = -b0sq/6 Pb di1
      const double dE3b = dcIb * k.p;
      pb += dcIb * dE3;
      eb.b0sq += dE3b * w.Pb1 * dpsi * e.beta / 4.0;
      wb.Pb1 += dE3b * e.kE3b * dpsi;
      dpsib += dE3b * e.kE3b * w.Pb1;
      eb.b0sq -= dcGb * w.Pb * di1 * (1.0 / 6.0);
      wb.Pb -= bs6 * dcGb * di1;
      di1b -= bs6 * dcGb * w.Pb;
    }
    // dpsi = (2/3) i1 G0j - 2 H0j, di1 = -2 G0j
    i1b += (2.0 / 3.0) * dpsib * G0j;
    sym_ref(Gb, 0, j) += (2.0 / 3.0) * dpsib * k.i1 - 2.0 * di1b;
    sym_ref(Hb, 0, j) -= 2.0 * dpsib;
  }
}

// Adjoint of mu = spectral_radius(a) (column-major 3x3) for a simple real top
// eigenvalue: ab = mub * sign(nu) Cof(nu I - a) / p'(nu).
HYP_HD void eig_top_vjp(const double* a, double mu, double mub, double* ab) {
  const double c2 = a[0] + a[4] + a[8];
  const double c1 = (a[0] * a[4] - a[3] * a[1]) + (a[0] * a[8] - a[6] * a[2]) + (a[4] * a[8] - a[7] * a[5]);
  const double c0 = det3(a);
  const double pp = ((mu - c2) * mu + c1) * mu - c0, pm = ((-mu - c2) * -mu + c1) * -mu - c0;
  const double nu = fabs(pp) <= fabs(pm) ? mu : -mu;
  double B[9];
  for (int t = 0; t < 9; ++t) B[t] = -a[t];
  B[0] += nu;
  B[4] += nu;
  B[8] += nu;
  double C[9];  // cofactors, column-major: C(i,j) = B(i+1,j+1) B(i+2,j+2) - B(i+1,j+2) B(i+2,j+1)
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      C[i + 3 * j] = B[i1 + 3 * j1] * B[i2 + 3 * j2] - B[i1 + 3 * j2] * B[i2 + 3 * j1];
    }
  const double dp = C[0] + C[4] + C[8];
  const double g = dp != 0.0 ? (nu >= 0.0 ? mub : -mub) / dp : 0.0;
  for (int t = 0; t < 9; ++t) ab[t] = g * C[t];
}

// The cell's forward quantities the reverse pass reads.
struct CellFwd {
  Prim P;
  StressC c;
  double rho_s;
  double s0[3];
  int st;
};

HYP_HD CellFwd cell_forward(const EosC& e, const double* q) {
  CellFwd F;
  F.st = cons_to_prim(e, 1.0, q + 1, q[4], q + 5, F.P);
  F.c = stress_coeffs(e, F.P.k, F.P.w, F.P.xm1);
  F.rho_s = e.rho0 * F.P.k.s;
  stress_row0(F.rho_s, F.P.k, F.c, F.s0);
  return F;
}

// qb += (df/dq)^T fb + (dlambda/dq) lb; eb likewise. fb is indexed like the
// state (14; entries whose flux is identically zero are ignored). Returns the
// cons2prim status of the cell.
HYP_HD int cell_vjp(const EosC& e, const double* q, const double* fb, double lb, double* qb, EosBar& eb) {
  const CellFwd F = cell_forward(e, q);
  const Prim& P = F.P;
  const Kin& k = P.k;
  const Pows& w = P.w;
  const double rho = P.den;
  double rhob = 0.0, ub[3] = {0.0, 0.0, 0.0}, Eb = 0.0, Ab[9];
  for (int t = 0; t < 9; ++t) Ab[t] = 0.0;
  double s0b[3] = {0.0, 0.0, 0.0}, rhosb = 0.0;
  // ---- flux (phase_flux at alpha = 1) ----
  {
    const double du = rho * P.u[0];
    double dub = fb[0] + fb[4] * P.E;
    for (int a = 0; a < 3; ++a) {
      dub += fb[1 + a] * P.u[a];
      ub[a] += fb[1 + a] * du - fb[4] * F.s0[a];
      s0b[a] -= fb[1 + a] + fb[4] * P.u[a];
    }
    Eb += fb[4] * du;
    for (int b = 0; b < 3; ++b)
      for (int a = 1; a < 3; ++a) {  // a = 0 rows are identically zero
        const double g = fb[5 + a + 3 * b];
        rhob += g * (P.u[0] * P.A[a + 3 * b] - P.u[a] * P.A[3 * b]);
        ub[0] += g * rho * P.A[a + 3 * b];
        Ab[a + 3 * b] += g * rho * P.u[0];
        ub[a] -= g * rho * P.A[3 * b];
        Ab[3 * b] -= g * rho * P.u[a];
      }
    rhob += dub * P.u[0];
    ub[0] += dub * rho;
  }
  Sym Gb = sym_zero(), Hb = sym_zero();
  double i1b = 0.0, pb = 0.0, psib = 0.0, xm1b = 0.0;
  PowsBar wb = pows_zero();
  StressBar cb{0.0, 0.0, 0.0, 0.0};
  // ---- wave speed lambda = |u1| + sqrt(mu) ----
  if (lb != 0.0) {
    ub[0] += P.u[0] > 0.0 ? lb : (P.u[0] < 0.0 ? -lb : 0.0);
    double s0r[3], om[9], omb[9], s0rb[3] = {0.0, 0.0, 0.0};
    const double irs = k.inv_s * e.inv_rho0;  // 1/rho_s = det A / rho0
    for (int i = 0; i < 3; ++i) s0r[i] = F.s0[i] * irs;
    acoustic_omega(e, k, w, F.c, P.xm1, s0r, om);
    const double mu = spectral_radius(om);
    eig_top_vjp(om, mu, lb * 0.5 / sqrt(mu), omb);
    acoustic_omega_vjp(e, k, w, F.c, P.xm1, omb, Gb, Hb, i1b, pb, psib, wb, cb, xm1b, s0rb, eb);
    for (int i = 0; i < 3; ++i) {
      s0b[i] += s0rb[i] * irs;
      rhosb -= s0rb[i] * s0r[i] * irs;
    }
  }
  // ---- stress row 1: s0 = -2 rho_s (cG G0. + cGG H0. + cI e0) ----
  {
    const double m = -2.0 * F.rho_s;
    const double t0 = F.c.cG * k.G.a00 + F.c.cGG * k.H.a00 + F.c.cI;
    const double t1 = F.c.cG * k.G.a01 + F.c.cGG * k.H.a01;
    const double t2 = F.c.cG * k.G.a02 + F.c.cGG * k.H.a02;
    rhosb += -2.0 * (s0b[0] * t0 + s0b[1] * t1 + s0b[2] * t2);
    const double tb0 = m * s0b[0], tb1 = m * s0b[1], tb2 = m * s0b[2];
    cb.cG += tb0 * k.G.a00 + tb1 * k.G.a01 + tb2 * k.G.a02;
    cb.cGG += tb0 * k.H.a00 + tb1 * k.H.a01 + tb2 * k.H.a02;
    cb.cI += tb0;
    Gb.a00 += tb0 * F.c.cG;
    Gb.a01 += tb1 * F.c.cG;
    Gb.a02 += tb2 * F.c.cG;
    Hb.a00 += tb0 * F.c.cGG;
    Hb.a01 += tb1 * F.c.cGG;
    Hb.a02 += tb2 * F.c.cGG;
  }
  stress_coeffs_vjp(e, k, w, P.xm1, F.c, cb, wb, i1b, pb, psib, xm1b, eb);
  double eintb = 0.0;
  entropy_xm1_vjp(e, P.e_int, k, w, xm1b, eintb, wb, psib, eb);
  pb += powers_vjp(e, k, w, wb);
  double sb = kinematics_vjp(P.A, k, Gb, Hb, i1b, psib, pb, Ab);
  sb += e.rho0 * rhosb;  // rho_s = rho0 s
  // ---- cons2prim (alpha = 1): s = rho/rho0 (through det A = rho0/rho) ----
  rhob += sb * e.inv_rho0;
  Eb += eintb;  // e_int = E - |u|^2/2
  for (int a = 0; a < 3; ++a) ub[a] -= eintb * P.u[a];
  const double irho = P.inv_den;
  double irhob = Eb * q[4];
  qb[4] += Eb * irho;
  for (int a = 0; a < 3; ++a) {
    irhob += ub[a] * q[1 + a];
    qb[1 + a] += ub[a] * irho;
  }
  for (int t = 0; t < 9; ++t) {
    irhob += Ab[t] * q[5 + t];
    qb[5 + t] += Ab[t] * irho;
  }
  rhob -= irhob * irho * irho;
  // rho = sqrt(det(rho A) / rho0)
  const double db = rhob * e.inv_rho0 * (0.5 * P.inv_den);
  const double* m = q + 5;
  qb[5] += db * (m[4] * m[8] - m[5] * m[7]);
  qb[6] += db * (m[5] * m[6] - m[3] * m[8]);
  qb[7] += db * (m[3] * m[7] - m[4] * m[6]);
  qb[8] += db * (m[2] * m[7] - m[1] * m[8]);
  qb[9] += db * (m[0] * m[8] - m[2] * m[6]);
  qb[10] += db * (m[1] * m[6] - m[0] * m[7]);
  qb[11] += db * (m[1] * m[5] - m[2] * m[4]);
  qb[12] += db * (m[2] * m[3] - m[0] * m[5]);
  qb[13] += db * (m[0] * m[4] - m[1] * m[3]);
  return F.st;
}

// Adjoint of prim2cons at alpha = 1 (HyperelasticityMPh.jl:66-87): prim
// p = (rho, u(3), S, A(9)) -> q = (rho, rho u, rho E, rho A); pb += (dq/dp)^T qb.
HYP_HD void prim2cons_vjp(const EosC& e, const double* p, const double* qb, double* pb, EosBar& eb) {
  const double rho = p[0];
  const double* A = p + 5;
  const double detA = det3(A);
  const Kin k = kinematics(A, detA);
  const Pows w = powers(e, k);
  const double xS = exp(p[4] / e.cv) - 1.0;
  const double eint = e_cold(e, w) + e.cvt0 * w.Pg * xS + e_shear(e, k, w);
  const double ek = 0.5 * (p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
  double rhob = qb[0] + qb[4] * (eint + ek);
  for (int a = 0; a < 3; ++a) {
    rhob += qb[1 + a] * p[1 + a];
    pb[1 + a] += qb[1 + a] * rho + qb[4] * rho * p[1 + a];
  }
  double Ab[9];
  for (int t = 0; t < 9; ++t) {
    rhob += qb[5 + t] * A[t];
    Ab[t] = qb[5 + t] * rho;
  }
  pb[0] += rhob;
  const double eb_ = qb[4] * rho;
  PowsBar wb = pows_zero();
  eb.k0 += eb_ * w.Pam1 * w.Pam1 * 0.5 / (e.alpha * e.alpha);
  wb.Pam1 += eb_ * 2.0 * e.kU * w.Pam1;
  wb.Pg += eb_ * e.cvt0 * xS;
  pb[4] += eb_ * e.cvt0 * w.Pg * (xS + 1.0) / e.cv;
  eb.b0sq += eb_ * 0.5 * w.Pb * k.psi;
  wb.Pb += eb_ * 0.5 * e.b0sq * k.psi;
  const double psib = eb_ * 0.5 * e.b0sq * w.Pb;
  const double pbar = powers_vjp(e, k, w, wb);
  const double sb = kinematics_vjp(A, k, sym_zero(), sym_zero(), 0.0, psib, pbar, Ab);
  // s = 1 / det A
  const double dAb = -sb * k.s * k.s;
  Ab[0] += dAb * (A[4] * A[8] - A[5] * A[7]);
  Ab[1] += dAb * (A[5] * A[6] - A[3] * A[8]);
  Ab[2] += dAb * (A[3] * A[7] - A[4] * A[6]);
  Ab[3] += dAb * (A[2] * A[7] - A[1] * A[8]);
  Ab[4] += dAb * (A[0] * A[8] - A[2] * A[6]);
  Ab[5] += dAb * (A[1] * A[6] - A[0] * A[7]);
  Ab[6] += dAb * (A[1] * A[5] - A[2] * A[4]);
  Ab[7] += dAb * (A[2] * A[3] - A[0] * A[5]);
  Ab[8] += dAb * (A[0] * A[4] - A[1] * A[3]);
  for (int t = 0; t < 9; ++t) pb[5 + t] += Ab[t];
}

}  // namespace hyp
