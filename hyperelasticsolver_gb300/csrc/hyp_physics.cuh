// hyp_physics.cuh -- per-cell hyperelastic physics in closed form (FP64).
//
// Restates, for one phase of one cell, the chain the reference evaluates with
// ForwardDiff and LAPACK:
//   cons2prim            HyperelasticityMPh.jl:106-133
//   finger, invariants   Strains.jl:26-32, 46-52
//   energy, entropy      EquationsOfState.jl:118-137, 139-156   (Barton2009)
//   stress               EquationsOfState.jl:179-190  sigma = -2 rho G dE/dG
//   acoustic (n = e1)    EquationsOfState.jl:223-246
//   get_eigvals          HyperelasticityMPh.jl:258-266  u1 +- sqrt|eig(acoustic)|
//   flux                 HyperelasticityMPh.jl:146-175
// The reference differentiates the energy numerically-exactly with dual
// numbers; here the same derivatives are written in closed form:
//   dE/dG = E1 I + E2 (i1 I - G) + E3 p M,   M = A A^T = G^-1, p = det G,
//   G dE/dG = cG G + cGG G^2 + cI I,  cG = E1 + E2 i1, cGG = -E2, cI = E3 p,
// and the acoustic tensor needs only the three directional derivatives of
// row 1 of sigma along dA = e_j A[0,:]:  dG = -(G e_j e_0^T + e_0 e_j^T G),
// d i1 = -2 G0j, d i2 = -2 i1 G0j + 2 (G^2)0j, d p = -2 p [j==0],
// d rho_s = -rho_s [j==0].  Only the spectral radius of that tensor is used
// (max |u1 +- c| = |u1| + c_max, and the HLL bounds u1 -+ c_max), so the
// eigen-solve returns max |mu| of the 3x3 matrix.
//
// Written as __host__ __device__ code with no CUDA intrinsics so that the
// same source can be compiled on the host by the unit tests.
#pragma once
#include <math.h>
#include <stdint.h>

#ifndef HYP_HD
#ifdef __CUDACC__
#define HYP_HD __host__ __device__ __forceinline__
#else
#define HYP_HD inline
#endif
#endif

namespace hyp {

// Barton2009 parameters with the derived constants the closed forms use. The
// templates below take the arithmetic type R: double for the FP64 step, float
// for the mixed-precision step (every constant goes through R(...) so that no
// FP32 expression is promoted to the slow FP64 pipe).
template <class R> struct EosT {
  R rho0, inv_rho0, cv, t0, cvt0, inv_cvt0;
  R alpha, beta, gamma;
  R b0sq, k0;
  R kU;            // 0.5 k0 / alpha^2          (cold energy prefactor)
  R kE3a;          // k0 / (2 alpha)            (dUcold/dp prefactor)
  R kE3b;          // b0sq * beta / 4           (dW/dp prefactor)
  R kE3g;          // cv t0 gamma / 2           (d thermal / dp prefactor)
  R b0sq_3, b0sq_6;  // b0sq / 3, b0sq / 6
  int default_exp; // alpha == 1, beta == 3, gamma == 2 (integer-power fast path)
};
using EosC = EosT<double>;

HYP_HD EosC make_eos(double rho0, double c0, double cv, double t0, double b0, double alpha, double beta,
                     double gamma) {
  EosC e;
  e.rho0 = rho0;
  e.inv_rho0 = 1.0 / rho0;
  e.cv = cv;
  e.t0 = t0;
  e.cvt0 = cv * t0;
  e.inv_cvt0 = 1.0 / e.cvt0;
  e.alpha = alpha;
  e.beta = beta;
  e.gamma = gamma;
  e.b0sq = b0 * b0;                          // EquationsOfState.jl:111
  e.k0 = c0 * c0 - (4.0 / 3.0) * (b0 * b0);  // EquationsOfState.jl:112
  e.kU = 0.5 * e.k0 / (alpha * alpha);
  e.kE3a = e.k0 / (2.0 * alpha);
  e.kE3b = e.b0sq * beta / 4.0;
  e.kE3g = e.cvt0 * gamma / 2.0;
  e.b0sq_3 = e.b0sq / 3.0;
  e.b0sq_6 = e.b0sq / 6.0;
  e.default_exp = (alpha == 1.0 && beta == 3.0 && gamma == 2.0) ? 1 : 0;
  return e;
}
template <class R> HYP_HD EosT<R> eos_as(const EosC& e) {
  EosT<R> r;
  r.rho0 = (R)e.rho0; r.inv_rho0 = (R)e.inv_rho0; r.cv = (R)e.cv; r.t0 = (R)e.t0;
  r.cvt0 = (R)e.cvt0; r.inv_cvt0 = (R)e.inv_cvt0;
  r.alpha = (R)e.alpha; r.beta = (R)e.beta; r.gamma = (R)e.gamma;
  r.b0sq = (R)e.b0sq; r.k0 = (R)e.k0;
  r.kU = (R)e.kU; r.kE3a = (R)e.kE3a; r.kE3b = (R)e.kE3b; r.kE3g = (R)e.kE3g;
  r.b0sq_3 = (R)e.b0sq_3; r.b0sq_6 = (R)e.b0sq_6;
  r.default_exp = e.default_exp;
  return r;
}

// Symmetric 3x3 stored as (00, 11, 22, 01, 02, 12).
template <class R> struct SymT {
  R a00, a11, a22, a01, a02, a12;
};
using Sym = SymT<double>;
template <class R> HYP_HD R sym_at(const SymT<R>& s, int i, int j) {
  if (i == j) return i == 0 ? s.a00 : (i == 1 ? s.a11 : s.a22);
  int k = i + j;  // 1: (0,1), 2: (0,2), 3: (1,2)
  return k == 1 ? s.a01 : (k == 2 ? s.a02 : s.a12);
}

// Powers of p = i3 = det G needed by the energy and its first two p-derivatives.
template <class R> struct PowsT {
  R Pa, Pa1, Pa2;  // p^(a/2), p^(a/2-1), p^(a/2-2)   a = alpha
  R Pb, Pb1, Pb2;  // beta
  R Pg, Pg1, Pg2;  // gamma
  R inv_Pg;
  R Pam1;          // p^(a/2) - 1 (the cold-energy strain; set accurately by the mixed path)
};
using Pows = PowsT<double>;

// Kinematic quantities of the distortion A (column-major 9-vector).
template <class R> struct KinT {
  SymT<R> G;         // Finger tensor G = (A A^T)^-1   (Strains.jl:26-32)
  SymT<R> H;         // G^2
  R i1, i2, p;       // invariants (Strains.jl:46-52); p = i3 = det G
  R s, inv_s;        // sqrt(p) = 1/det A and det A
  R psi;             // i1^2/3 - i2
};
using Kin = KinT<double>;

// A -> G, G^2, invariants, given s = 1/det A (> 0 for admissible states).
template <class R> HYP_HD KinT<R> kinematics_s(const R* A, R s, R inv_s) {
  KinT<R> k;
  // M = A A^T (symmetric)
  R m00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  R m11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  R m22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  R m01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  R m02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  R m12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  k.inv_s = inv_s;
  k.s = s;
  k.p = k.s * k.s;  // det G = 1/det(M) = 1/det(A)^2
  // G = adj(M) / det(M) = adj(M) * p
  k.G.a00 = (m11 * m22 - m12 * m12) * k.p;
  k.G.a11 = (m00 * m22 - m02 * m02) * k.p;
  k.G.a22 = (m00 * m11 - m01 * m01) * k.p;
  k.G.a01 = (m02 * m12 - m01 * m22) * k.p;
  k.G.a02 = (m01 * m12 - m02 * m11) * k.p;
  k.G.a12 = (m01 * m02 - m00 * m12) * k.p;
  const SymT<R>& g = k.G;
  k.H.a00 = g.a00 * g.a00 + g.a01 * g.a01 + g.a02 * g.a02;
  k.H.a11 = g.a01 * g.a01 + g.a11 * g.a11 + g.a12 * g.a12;
  k.H.a22 = g.a02 * g.a02 + g.a12 * g.a12 + g.a22 * g.a22;
  k.H.a01 = g.a00 * g.a01 + g.a01 * g.a11 + g.a02 * g.a12;
  k.H.a02 = g.a00 * g.a02 + g.a01 * g.a12 + g.a02 * g.a22;
  k.H.a12 = g.a01 * g.a02 + g.a11 * g.a12 + g.a12 * g.a22;
  k.i1 = g.a00 + g.a11 + g.a22;
  R trH = k.H.a00 + k.H.a11 + k.H.a22;
  k.i2 = R(0.5) * (k.i1 * k.i1 - trH);
  if (sizeof(R) == sizeof(double)) {
    k.psi = k.i1 * k.i1 / R(3) - k.i2;
  } else {
    // i1^2/3 - i2 = |dev G|^2 / 2 without the cancellation near G = I (FP32)
    R d01 = g.a00 - g.a11, d12 = g.a11 - g.a22, d20 = g.a22 - g.a00;
    k.psi = (d01 * d01 + d12 * d12 + d20 * d20) * R(1.0 / 6.0) + (g.a01 * g.a01 + g.a02 * g.a02 + g.a12 * g.a12);
  }
  return k;
}
template <class R> HYP_HD KinT<R> kinematics(const R* A, R detA) { return kinematics_s(A, R(1) / detA, detA); }

template <class R> HYP_HD R det3(const R* m) {  // column-major, cofactor expansion (SimpleLA.jl:84-89)
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
         m[6] * (m[1] * m[5] - m[4] * m[2]);
}

// kDef: 1 = the reference's default exponents (alpha 1, beta 3, gamma 2) known at
// compile time, so the general powers' code drops out of a kernel; -1 = decided by
// e.default_exp at run time.
template <int kDef, class E> HYP_HD bool default_exponents(const E& e) { return kDef == 1 || (kDef < 0 && e.default_exp); }

template <class R, int kDef = -1> HYP_HD PowsT<R> powers(const EosT<R>& e, const KinT<R>& k) {
  PowsT<R> w;
  if (default_exponents<kDef>(e)) {  // alpha = 1, beta = 3, gamma = 2: p^(n/2) = s^n
    R s = k.s, is = k.inv_s, ip = is * is;
    w.Pa = s;         w.Pa1 = is;  w.Pa2 = is * ip;
    w.Pb = s * k.p;   w.Pb1 = s;   w.Pb2 = is;
    w.Pg = k.p;       w.Pg1 = R(1); w.Pg2 = ip;
    w.inv_Pg = ip;
  } else {
    R lp = log(k.p), ip = R(1) / k.p;
    w.Pa = exp(R(0.5) * e.alpha * lp); w.Pa1 = w.Pa * ip; w.Pa2 = w.Pa1 * ip;
    w.Pb = exp(R(0.5) * e.beta * lp);  w.Pb1 = w.Pb * ip; w.Pb2 = w.Pb1 * ip;
    w.Pg = exp(R(0.5) * e.gamma * lp); w.Pg1 = w.Pg * ip; w.Pg2 = w.Pg1 * ip;
    w.inv_Pg = R(1) / w.Pg;
  }
  w.Pam1 = w.Pa - R(1);
  return w;
}

// Cold (Ucold) and shear (W) parts of the Barton2009 energy (EquationsOfState.jl:129-134).
template <class R> HYP_HD R e_cold(const EosT<R>& e, const PowsT<R>& w) { return e.kU * w.Pam1 * w.Pam1; }
template <class R> HYP_HD R e_shear(const EosT<R>& e, const KinT<R>& k, const PowsT<R>& w) {
  return R(0.5) * e.b0sq * w.Pb * k.psi;
}

// x - 1 with x the entropy argument of EquationsOfState.jl:150-154 (clamped at
// 1e-6); exp(S/cv) - 1 of the energy equals it because S = cv log x.
template <class R> HYP_HD R entropy_xm1(const EosT<R>& e, R e_int, const KinT<R>& k, const PowsT<R>& w) {
  R xm1 = (e_int - e_shear(e, k, w) - e_cold(e, w)) * e.inv_cvt0 * w.inv_Pg;
  if (xm1 + R(1) < R(1e-6)) xm1 = R(1e-6) - R(1);
  return xm1;
}

// Stress coefficients: G dE/dG = cG G + cGG G^2 + cI I (with S fixed).
template <class R> struct StressCT {
  R cG, cGG, cI, E3;
};
using StressC = StressCT<double>;
template <class R>
HYP_HD StressCT<R> stress_coeffs(const EosT<R>& e, const KinT<R>& k, const PowsT<R>& w, R xm1) {
  StressCT<R> c;
  R E1 = e.b0sq_3 * w.Pb * k.i1;
  R E2 = R(-0.5) * e.b0sq * w.Pb;
  c.E3 = e.kE3a * w.Pam1 * w.Pa1 + e.kE3g * w.Pg1 * xm1 + e.kE3b * w.Pb1 * k.psi;
  c.cG = E1 + E2 * k.i1;
  c.cGG = -E2;
  c.cI = c.E3 * k.p;
  return c;
}

// Row 1 of sigma = -2 rho_s (cG G + cGG G^2 + cI I).
template <class R> HYP_HD void stress_row0(R rho_s, const KinT<R>& k, const StressCT<R>& c, R* s0) {
  R m = R(-2) * rho_s;
  s0[0] = m * (c.cG * k.G.a00 + c.cGG * k.H.a00 + c.cI);
  s0[1] = m * (c.cG * k.G.a01 + c.cGG * k.H.a01);
  s0[2] = m * (c.cG * k.G.a02 + c.cGG * k.H.a02);
}
template <class R> HYP_HD void stress_full(R rho_s, const KinT<R>& k, const StressCT<R>& c, R* sig) {
  R m = R(-2) * rho_s;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i)
      sig[i + 3 * j] = m * (c.cG * sym_at(k.G, i, j) + c.cGG * sym_at(k.H, i, j) + (i == j ? c.cI : R(0)));
}

// Acoustic tensor Omega[i][j] = (1/rho_s) d_j sigma[0,i] (EquationsOfState.jl:223-246, n = e1),
// written column-major: om[i + 3 j].
template <class R>
HYP_HD void acoustic_omega(const EosT<R>& e, const KinT<R>& k, const PowsT<R>& w, const StressCT<R>& c, R xm1,
                           const R* s0_over_rho, R* om) {
  const R bs6 = e.b0sq_6;
  for (int j = 0; j < 3; ++j) {
    R G0j = sym_at(k.G, 0, j), H0j = sym_at(k.H, 0, j);
    R di1 = R(-2) * G0j;
    R dpsi = (R(2) / R(3)) * k.i1 * G0j - R(2) * H0j;
    R dcG, dcGG, dE3, dcI;
    if (j == 0) {
      R dp = R(-2) * k.p;
      R dPb = R(0.5) * e.beta * w.Pb1 * dp;
      R dPa = R(0.5) * e.alpha * w.Pa1 * dp;
      R dPa1 = (R(0.5) * e.alpha - R(1)) * w.Pa2 * dp;
      R dPg1 = (R(0.5) * e.gamma - R(1)) * w.Pg2 * dp;
      R dPb1 = (R(0.5) * e.beta - R(1)) * w.Pb2 * dp;
      dcG = -bs6 * (dPb * k.i1 + w.Pb * di1);
      dcGG = R(0.5) * e.b0sq * dPb;
      dE3 = e.kE3a * (dPa * w.Pa1 + w.Pam1 * dPa1) + e.kE3g * dPg1 * xm1 +
            e.kE3b * (dPb1 * k.psi + w.Pb1 * dpsi);
      dcI = dE3 * k.p + c.E3 * dp;
    } else {
      dcG = -bs6 * w.Pb * di1;
      dcGG = R(0);
      dE3 = e.kE3b * w.Pb1 * dpsi;
      dcI = dE3 * k.p;
    }
    for (int i = 0; i < 3; ++i) {
      R G0i = sym_at(k.G, 0, i), H0i = sym_at(k.H, 0, i);
      R Gij = sym_at(k.G, i, j), Hij = sym_at(k.H, i, j);
      R Gi0 = G0i;
      R dG0i = -(G0j * (i == 0 ? R(1) : R(0)) + Gij);
      R dH0i = -(G0j * Gi0 + Hij + H0j * (i == 0 ? R(1) : R(0)) + k.G.a00 * Gij);
      R v = dcG * G0i + c.cG * dG0i + dcGG * H0i + c.cGG * dH0i + (i == 0 ? dcI : R(0));
      om[i + 3 * j] = R(-2) * v - (j == 0 ? s0_over_rho[i] : R(0));
    }
  }
}

// Acoustic tensor along a general direction n (EquationsOfState.jl:192-246),
// column-major: Omega[i][j] = (1/rho_s) sum_m n_m d_j sigma[m,i], d_j the
// derivative along dA = e_j (A^T n)^T, for which dG = -(g_j n^T + n g_j^T)
// (g_j = G e_j), d i1 = -2 (Gn)_j, d i2 = -2 i1 (Gn)_j + 2 (Hn)_j,
// d p = -2 p n_j and d rho_s = -rho_s n_j; n = e1 gives acoustic_omega.
// hold_energy = false: the entropy is held (acoustic(eos, ent, F, n), :223-246)
// and sn_over_rho = (sigma n)/rho_s carries the density's derivative.
// hold_energy = true: the density and the internal energy are held and the
// entropy follows G through entropy(e_int, G) (acoustic(eos, P, n), :192-221,
// over stress(eos, den, e_int, F), :162-176); sn_over_rho is not read, and an
// entropy argument at its 1e-6 clamp (xm1_clamped) does not move.
template <class R>
HYP_HD void acoustic_omega_dir(const EosT<R>& e, const KinT<R>& k, const PowsT<R>& w, const StressCT<R>& c, R xm1,
                               bool hold_energy, bool xm1_clamped, const R* sn_over_rho, const R* n, R* om) {
  R Gn[3], Hn[3];
  for (int i = 0; i < 3; ++i) {
    Gn[i] = sym_at(k.G, i, 0) * n[0] + sym_at(k.G, i, 1) * n[1] + sym_at(k.G, i, 2) * n[2];
    Hn[i] = sym_at(k.H, i, 0) * n[0] + sym_at(k.H, i, 1) * n[1] + sym_at(k.H, i, 2) * n[2];
  }
  const R nGn = n[0] * Gn[0] + n[1] * Gn[1] + n[2] * Gn[2];
  const R nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
  const R bs6 = e.b0sq_6;
  for (int j = 0; j < 3; ++j) {
    const R dp = R(-2) * k.p * n[j];
    const R di1 = R(-2) * Gn[j];
    const R dpsi = (R(2) / R(3)) * k.i1 * Gn[j] - R(2) * Hn[j];
    const R dPb = R(0.5) * e.beta * w.Pb1 * dp;
    const R dPa = R(0.5) * e.alpha * w.Pa1 * dp;
    const R dPa1 = (R(0.5) * e.alpha - R(1)) * w.Pa2 * dp;
    const R dPg1 = (R(0.5) * e.gamma - R(1)) * w.Pg2 * dp;
    const R dPb1 = (R(0.5) * e.beta - R(1)) * w.Pb2 * dp;
    const R dcG = -bs6 * (dPb * k.i1 + w.Pb * di1);
    const R dcGG = R(0.5) * e.b0sq * dPb;
    R dxm1 = R(0);
    if (hold_energy && !xm1_clamped) {
      const R dPg = R(0.5) * e.gamma * w.Pg1 * dp;
      const R dW = R(0.5) * e.b0sq * (dPb * k.psi + w.Pb * dpsi);
      const R dUc = R(2) * e.kU * w.Pam1 * dPa;
      dxm1 = -(dW + dUc) * e.inv_cvt0 * w.inv_Pg - xm1 * dPg * w.inv_Pg;
    }
    const R dE3 = e.kE3a * (dPa * w.Pa1 + w.Pam1 * dPa1) + e.kE3g * (dPg1 * xm1 + w.Pg1 * dxm1) +
                  e.kE3b * (dPb1 * k.psi + w.Pb1 * dpsi);
    const R dcI = dE3 * k.p + c.E3 * dp;
    for (int i = 0; i < 3; ++i) {
      const R Gij = sym_at(k.G, i, j), Hij = sym_at(k.H, i, j);
      const R ndG = -(Gn[j] * n[i] + nn * Gij);
      const R ndH = -(Gn[j] * Gn[i] + nn * Hij + Hn[j] * n[i] + nGn * Gij);
      const R v = dcG * Gn[i] + c.cG * ndG + dcGG * Hn[i] + c.cGG * ndH + dcI * n[i];
      om[i + 3 * j] = R(-2) * v - (hold_energy ? R(0) : n[j] * sn_over_rho[i]);
    }
  }
}

// Eigenvalue moduli of a real 3x3 (column-major). Characteristic polynomial
// mu^3 - c2 mu^2 + c1 mu - c0; single-precision closed-form seeds
// (trigonometric for three real roots, Cardano otherwise), three Newton steps
// in R on the seed of largest modulus (a real root r), and deflation to the
// quadratic mu^2 - (c2 - r) mu + c0/r for the other two (a complex pair has
// modulus sqrt(c0/r)).
template <class R> struct CubicTop {
  R c2, c1, c0;
  R r;          // Newton-refined real root of largest seed modulus
  float other;  // single-precision estimate of the larger other modulus (-1: unknown)
};

// FP32 reciprocal of a Newton step's slope: the step's own error is then ~1e-7 of
// the (shrinking) correction, so three steps still reach the root to the last bit.
template <class R> HYP_HD R newton_recip(R fp) {
  const float f = (float)fp;
#ifdef __CUDA_ARCH__
  const float inv = __frcp_rn(f);
#else
  const float inv = 1.0f / f;
#endif
  return (fabsf(f) > 1e-30f && fabsf(f) < 1e30f) ? R(inv) : R(1) / fp;
}

template <class R> HYP_HD CubicTop<R> cubic_top(const R* a) {
  CubicTop<R> t;
  const R c2 = a[0] + a[4] + a[8];
  const R c1 = (a[0] * a[4] - a[3] * a[1]) + (a[0] * a[8] - a[6] * a[2]) + (a[4] * a[8] - a[7] * a[5]);
  const R c0 = det3(a);
  float C2 = (float)c2, C1 = (float)c1, C0 = (float)c0;
  float p = C1 - C2 * C2 * (1.0f / 3.0f);
  float q = -2.0f / 27.0f * C2 * C2 * C2 + C2 * C1 * (1.0f / 3.0f) - C0;
  float disc = 0.25f * q * q + p * p * p * (1.0f / 27.0f);
  float seed, other = -1.0f;
  if (disc < 0.0f && p < 0.0f) {
    float m = 2.0f * sqrtf(-p * (1.0f / 3.0f));
    float cc = fminf(1.0f, fmaxf(-1.0f, 3.0f * q / (p * m)));
    float th = acosf(cc) * (1.0f / 3.0f);
    float y0 = m * cosf(th) + C2 * (1.0f / 3.0f);
    float y1 = m * cosf(th - 2.0943951f) + C2 * (1.0f / 3.0f);
    float y2 = m * cosf(th - 4.1887902f) + C2 * (1.0f / 3.0f);
    seed = y0;
    float o1 = y1, o2 = y2;
    if (fabsf(y1) > fabsf(seed)) { o1 = seed; seed = y1; }
    if (fabsf(y2) > fabsf(seed)) { o2 = seed; seed = y2; }
    other = fmaxf(fabsf(o1), fabsf(o2));
  } else {
    float sd = sqrtf(fmaxf(disc, 0.0f));
    seed = cbrtf(-0.5f * q + sd) + cbrtf(-0.5f * q - sd) + C2 * (1.0f / 3.0f);
    if (seed != 0.0f) other = sqrtf(fabsf(C0 / seed));  // modulus of the complex pair
  }
  R r = (R)seed;
  for (int it = 0; it < 3; ++it) {
    R f = ((r - c2) * r + c1) * r - c0;
    R fp = (R(3) * r - R(2) * c2) * r + c1;
    r = (fp != R(0)) ? r - f * newton_recip(fp) : r;
  }
  t.c2 = c2;
  t.c1 = c1;
  t.c0 = c0;
  t.r = r;
  t.other = (other == other && seed == seed) ? other : -1.0f;
  return t;
}

// Moduli of the two roots other than t.r (deflation).
template <class R> HYP_HD void cubic_rest(const CubicTop<R>& t, R* m1, R* m2) {
  R s, qq;
  if (t.r != R(0)) {
    s = t.c2 - t.r;
    qq = t.c0 / t.r;
  } else {  // singular: the other roots solve mu^2 - c2 mu + c1
    s = t.c2;
    qq = t.c1;
  }
  R dsc = s * s - R(4) * qq;
  if (dsc < R(0)) {
    *m1 = *m2 = sqrt(fabs(qq));
  } else {
    R sq = sqrt(dsc);
    R ra = s >= R(0) ? R(0.5) * (s + sq) : R(0.5) * (s - sq);
    *m1 = fabs(ra);
    *m2 = ra != R(0) ? fabs(qq / ra) : fabs(s - ra);
  }
}

// Eigenvalues of the symmetric part of a 3x3 (column-major) by cyclic Jacobi
// rotations (Jacobi 1846, with Rutishauser's rotation formulas): accurate to a few
// ulps of the largest modulus whatever the gaps between eigenvalues, where the
// characteristic polynomial loses half the digits of a repeated root. At theta = 0
// the rotation's sign follows a_pq, so a matrix and its mirror S A S (S a signature
// matrix) give the same diagonal bit for bit.
template <class R> HYP_HD void sym_eig_jacobi(const R* a, R* d) {
  R m[3][3];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) m[i][j] = R(0.5) * (a[i + 3 * j] + a[j + 3 * i]);
  for (int sweep = 0; sweep < 12; ++sweep) {
    const R off = fabs(m[0][1]) + fabs(m[0][2]) + fabs(m[1][2]);
    const R dg = fabs(m[0][0]) + fabs(m[1][1]) + fabs(m[2][2]);
    if (!(off > R(1e-20) * dg)) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const R apq = m[p][q];
        if (apq == R(0)) continue;
        const R theta = (m[q][q] - m[p][p]) / (R(2) * apq);
        const R sg = theta > R(0) ? R(1) : (theta < R(0) ? R(-1) : (apq > R(0) ? R(1) : R(-1)));
        const R at = fabs(theta);
        const R t = sg / (at < R(1e150) ? at + sqrt(R(1) + at * at) : R(2) * at);
        const R c = R(1) / sqrt(R(1) + t * t), sn = t * c;
        m[p][p] -= t * apq;
        m[q][q] += t * apq;
        m[p][q] = m[q][p] = R(0);
        const int r = 3 - p - q;
        const R arp = m[r][p], arq = m[r][q];
        m[r][p] = m[p][r] = c * arp - sn * arq;
        m[r][q] = m[q][r] = sn * arp + c * arq;
      }
  }
  d[0] = m[0][0];
  d[1] = m[1][1];
  d[2] = m[2][2];
}

// True when a (column-major 3x3) is symmetric to rounding, as the acoustic tensor
// of a hyperelastic material is.
template <class R> HYP_HD bool symmetric_to_rounding(const R* a) {
  R mx = R(0);
  for (int k = 0; k < 9; ++k) mx = fmax(mx, fabs(a[k]));
  const R tol = R(64) * R(sizeof(R) == 8 ? 1.1102230246251565e-16 : 5.9604645e-8) * mx;
  return fabs(a[3] - a[1]) <= tol && fabs(a[6] - a[2]) <= tol && fabs(a[7] - a[5]) <= tol;
}

// All three moduli: Jacobi for a symmetric matrix, else |r| and the deflated pair.
template <class R> HYP_HD void eig_core(const R* a, R* mods) {
  if (symmetric_to_rounding(a)) {
    sym_eig_jacobi(a, mods);
    for (int k = 0; k < 3; ++k) mods[k] = fabs(mods[k]);
    return;
  }
  const CubicTop<R> t = cubic_top(a);
  mods[0] = fabs(t.r);
  cubic_rest(t, mods + 1, mods + 2);
}

// Largest eigenvalue modulus (what the step consumes). When the single-precision
// roots put the other two moduli below 0.9 |r|, the maximum is |r| itself (seed
// errors are ~1e-6 relative, far inside that margin): the Newton root, accurate to
// the last bits for a root that separated. Otherwise a symmetric matrix goes to
// Jacobi and a general one compares |r| with the deflated pair.
template <class R> HYP_HD R spectral_radius(const R* a) {
  const CubicTop<R> t = cubic_top(a);
  const R top = fabs(t.r);
  if (t.other >= 0.0f && R(t.other) < R(0.9) * top) return top;
  R m1, m2;
  if (symmetric_to_rounding(a)) {
    R d[3];
    sym_eig_jacobi(a, d);
    return fmax(fabs(d[0]), fmax(fabs(d[1]), fabs(d[2])));
  }
  cubic_rest(t, &m1, &m2);
  return fmax(top, fmax(m1, m2));
}
// All three moduli, descending (the function-level get_eigvals).
HYP_HD void eig_moduli3(const double* a, double* mods) {
  double v[3];
  eig_core(a, v);
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j)
      if (v[j] > v[i]) { double t = v[i]; v[i] = v[j]; v[j] = t; }
  mods[0] = v[0]; mods[1] = v[1]; mods[2] = v[2];
}

// Moduli |mu_k| of the eigenvalues of a real 3x3 in the order Julia's `eigvals`
// returns them (HyperelasticityMPh.jl:263): ascending real part, LinearAlgebra's
// default lexicographic (real, imag) sort; the two members of a complex pair share
// a modulus, so their order does not show. Jacobi rotations for a matrix symmetric
// to rounding (accurate to a few ulps for every root), else the Newton-polished
// real root and the deflated quadratic.
HYP_HD void eig_sorted3(const double* a, double* mods) {
  double re[3], md[3];
  if (symmetric_to_rounding(a)) {
    sym_eig_jacobi(a, re);
    for (int k = 0; k < 3; ++k) md[k] = fabs(re[k]);
  } else {
    const CubicTop<double> t = cubic_top(a);
    double s, qq;
    if (t.r != 0.0) {
      s = t.c2 - t.r;
      qq = t.c0 / t.r;
    } else {
      s = t.c2;
      qq = t.c1;
    }
    re[0] = t.r;
    md[0] = fabs(t.r);
    const double dsc = s * s - 4.0 * qq;
    if (dsc < 0.0) {  // complex pair: real part s/2, modulus sqrt(qq)
      re[1] = re[2] = 0.5 * s;
      md[1] = md[2] = sqrt(fabs(qq));
    } else {
      const double sq = sqrt(dsc);
      const double ra = s >= 0.0 ? 0.5 * (s + sq) : 0.5 * (s - sq);
      const double rb = ra != 0.0 ? qq / ra : s - ra;
      re[1] = ra;
      re[2] = rb;
      md[1] = fabs(ra);
      md[2] = fabs(rb);
    }
  }
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && re[j] < re[j - 1]; --j) {
      double t = re[j]; re[j] = re[j - 1]; re[j - 1] = t;
      t = md[j]; md[j] = md[j - 1]; md[j - 1] = t;
    }
  mods[0] = md[0]; mods[1] = md[1]; mods[2] = md[2];
}

// ---- per-cell, per-phase evaluation ---------------------------------------

// Status bits a cell can raise (reported through the context's error word).
enum { HYP_CELL_OK = 0, HYP_CELL_NEG_DET = 1, HYP_CELL_NONFINITE = 2 };

// Primitive quantities of one phase: alpha, stored alpha*rho (unused, as in the
// reference), alpha*rho*u, alpha*rho*E, alpha*rho*A.
struct Prim {
  double den, true_den, inv_den;  // alpha*rho_true, rho_true, 1/(alpha*rho_true)
  double u[3], E, e_int;
  double A[9];
  double xm1;                     // exp(S/cv) - 1 (clamped entropy argument minus one)
  Kin k;
  Pows w;
};

// 1/sqrt(x): CUDA's rsqrt on the device (1 ulp), the quotient on the host.
HYP_HD double rsqrt_d(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

// HyperelasticityMPh.jl:106-133. Returns HYP_CELL_* status.
HYP_HD int cons_to_prim(const EosC& e, double alpha, const double* m, double rhoE, const double* rA, Prim& P) {
  double FQ[9];
  double ia = 1.0 / alpha;
  for (int c = 0; c < 9; ++c) FQ[c] = rA[c] * ia;
  double d = det3(FQ);
  int st = d > 0.0 ? HYP_CELL_OK : HYP_CELL_NEG_DET;
  // rho_true = sqrt(x) and 1/(alpha rho_true) from one reciprocal square root
  // (within an ulp or two of the sqrt and the division it replaces)
  const double x = d * e.inv_rho0, r = rsqrt_d(x);
  P.true_den = x * r;
  P.den = alpha * P.true_den;
  P.inv_den = r * ia;
  for (int c = 0; c < 3; ++c) P.u[c] = m[c] * P.inv_den;
  P.E = rhoE * P.inv_den;
  P.e_int = P.E - 0.5 * (P.u[0] * P.u[0] + P.u[1] * P.u[1] + P.u[2] * P.u[2]);
  for (int c = 0; c < 9; ++c) P.A[c] = rA[c] * P.inv_den;
  // det A = det(rA/den) = d alpha^3 / den^3 = rho0 / true_den = rho0 alpha / den,
  // 1/det A = true_den / rho0
  const double detA = (e.rho0 * alpha) * P.inv_den;
  P.k = kinematics_s(P.A, P.true_den * e.inv_rho0, detA);
  P.w = powers(e, P.k);
  P.xm1 = entropy_xm1(e, P.e_int, P.k, P.w);
  if (!(P.e_int == P.e_int) || !(P.xm1 == P.xm1) || !isfinite(P.k.p)) st |= HYP_CELL_NONFINITE;
  return st;
}

// Physical x-flux of one phase, the 14 entries after alpha (HyperelasticityMPh.jl:146-175):
// [alpha*rho u1, momentum(3), energy, alpha*rho*A(9)], plus row 1 of sigma.
HYP_HD void phase_flux(const EosC& e, double alpha, const Prim& P, const StressC& c, double* f, double* s0) {
  double rho_s = e.rho0 * P.k.s;  // rho0 / det A (EquationsOfState.jl:180)
  stress_row0(rho_s, P.k, c, s0);
  s0[0] *= alpha; s0[1] *= alpha; s0[2] *= alpha;
  double du = P.den * P.u[0];
  f[0] = du;
  f[1] = du * P.u[0] - s0[0];
  f[2] = du * P.u[1] - s0[1];
  f[3] = du * P.u[2] - s0[2];
  f[4] = du * P.E - (P.u[0] * s0[0] + P.u[1] * s0[1] + P.u[2] * s0[2]);
  for (int b = 0; b < 3; ++b)
    for (int a = 0; a < 3; ++a) f[5 + a + 3 * b] = P.den * (P.u[0] * P.A[a + 3 * b] - P.u[a] * P.A[3 * b]);
}

// Largest acoustic wave speed sqrt(max |eig(acoustic)|) of one phase.
HYP_HD double phase_cmax(const EosC& e, const Prim& P, const StressC& c) {
  double rho_s = e.rho0 * P.k.s;
  double s0[3], s0r[3], om[9];
  stress_row0(rho_s, P.k, c, s0);
  const double irs = P.k.inv_s * e.inv_rho0;  // 1/rho_s = det A / rho0
  for (int i = 0; i < 3; ++i) s0r[i] = s0[i] * irs;
  acoustic_omega(e, P.k, P.w, c, P.xm1, s0r, om);
  return sqrt(spectral_radius(om));
}

// cons2prim / prim2cons of one phase (HyperelasticityMPh.jl:106-133, 63-90):
// q[15] = [alpha, alpha rho, alpha rho u(3), alpha rho E, alpha rho A(9)],
// p[15] = [alpha, rho_true, u(3), S, A(9)].
HYP_HD void phase_cons2prim(const EosC& e, const double* q, double* p) {
  Prim P;
  cons_to_prim(e, q[0], q + 2, q[5], q + 6, P);
  p[0] = q[0];
  p[1] = P.true_den;
  for (int c = 0; c < 3; ++c) p[2 + c] = P.u[c];
  p[5] = e.cv * log(P.xm1 + 1.0);  // S = cv log x (EquationsOfState.jl:155)
  for (int c = 0; c < 9; ++c) p[6 + c] = P.A[c];
}
HYP_HD void phase_prim2cons(const EosC& e, const double* p, double* q) {
  double den = p[0] * p[1];
  Kin k = kinematics(p + 6, det3(p + 6));
  Pows w = powers(e, k);
  double eint = e_cold(e, w) + e.cvt0 * w.Pg * (exp(p[5] / e.cv) - 1.0) + e_shear(e, k, w);
  double ek = 0.5 * (p[2] * p[2] + p[3] * p[3] + p[4] * p[4]);
  q[0] = p[0];
  q[1] = den;
  for (int c = 0; c < 3; ++c) q[2 + c] = den * p[2 + c];
  q[5] = den * (eint + ek);
  for (int c = 0; c < 9; ++c) q[6 + c] = den * p[6 + c];
}

// ---- function-level forms with the reference's signatures -----------------

// stress(eos, ent, F) (EquationsOfState.jl:179-190): full 3x3, column-major.
HYP_HD void stress_SF(const EosC& e, double S, const double* F, double* sig) {
  Kin k = kinematics(F, det3(F));
  Pows w = powers(e, k);
  StressC c = stress_coeffs(e, k, w, exp(S / e.cv) - 1.0);
  stress_full(e.rho0 * k.s, k, c, sig);
}
// acoustic(eos, ent, F, [1,0,0]) (EquationsOfState.jl:223-246), column-major.
HYP_HD void acoustic_SF(const EosC& e, double S, const double* F, double* om) {
  Kin k = kinematics(F, det3(F));
  Pows w = powers(e, k);
  double xm1 = exp(S / e.cv) - 1.0;
  StressC c = stress_coeffs(e, k, w, xm1);
  double rho_s = e.rho0 * k.s, s0[3], s0r[3];
  stress_row0(rho_s, k, c, s0);
  for (int i = 0; i < 3; ++i) s0r[i] = s0[i] / rho_s;
  acoustic_omega(e, k, w, c, xm1, s0r, om);
}
// acoustic(eos, ent, F, n) (EquationsOfState.jl:223-246) for any direction n.
HYP_HD void acoustic_SFn(const EosC& e, double S, const double* F, const double* n, double* om) {
  Kin k = kinematics(F, det3(F));
  Pows w = powers(e, k);
  const double xm1 = exp(S / e.cv) - 1.0;
  StressC c = stress_coeffs(e, k, w, xm1);
  const double rho_s = e.rho0 * k.s;
  double sig[9], sn[3];
  stress_full(rho_s, k, c, sig);
  for (int i = 0; i < 3; ++i) sn[i] = (sig[i] * n[0] + sig[i + 3] * n[1] + sig[i + 6] * n[2]) / rho_s;
  acoustic_omega_dir(e, k, w, c, xm1, false, false, sn, n, om);
}
// stress(eos, den, e_int, F) (EquationsOfState.jl:162-176): the entropy from the
// internal energy (entropy(e_int, finger(F)), clamped), sigma = -2 den G dE/dG at
// that entropy, with den given rather than rho0 / det F.
HYP_HD void stress_den_eF(const EosC& e, double den, double eint, const double* F, double* sig) {
  Kin k = kinematics(F, det3(F));
  Pows w = powers(e, k);
  StressC c = stress_coeffs(e, k, w, entropy_xm1(e, eint, k, w));
  stress_full(den, k, c, sig);
}
// acoustic(eos, P, n) (EquationsOfState.jl:192-221), P = [alpha, rho, u(3), S, A(9)]:
// e_int = energy(eos, S, finger(A)), then the Jacobian of stress(eos, den, e_int, F)
// over F at F = A with den = alpha rho held, divided by den.
HYP_HD void acoustic_Pn(const EosC& e, const double* P, const double* n, double* om) {
  const double* F = P + 6;
  Kin k = kinematics(F, det3(F));
  Pows w = powers(e, k);
  const double eint = e_cold(e, w) + e.cvt0 * w.Pg * (exp(P[5] / e.cv) - 1.0) + e_shear(e, k, w);
  const double raw = (eint - e_shear(e, k, w) - e_cold(e, w)) * e.inv_cvt0 * w.inv_Pg;
  const bool clamped = raw + 1.0 < 1e-6;
  const double xm1 = clamped ? 1e-6 - 1.0 : raw;
  StressC c = stress_coeffs(e, k, w, xm1);
  acoustic_omega_dir(e, k, w, c, xm1, true, clamped, (const double*)nullptr, n, om);
}
// Invariants of a general (not necessarily symmetric) G (Strains.jl:46-52).
HYP_HD void invariants_general(const double* g, double* out) {
  double i1 = g[0] + g[4] + g[8];
  double trg2 = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) trg2 += g[i + 3 * k] * g[k + 3 * i];
  out[0] = i1;
  out[1] = 0.5 * (i1 * i1 - trg2);
  out[2] = det3(g);
}
HYP_HD double pow_half(const EosC& e, double p, double a) { return e.default_exp ? pow(p, 0.5 * a) : exp(0.5 * a * log(p)); }
// energy(eos, S, G) (EquationsOfState.jl:118-137)
HYP_HD double energy_SG(const EosC& e, double S, const double* G) {
  double i[3];
  invariants_general(G, i);
  double pa = pow_half(e, i[2], e.alpha) - 1.0;
  return e.kU * pa * pa + e.cvt0 * pow_half(e, i[2], e.gamma) * (exp(S / e.cv) - 1.0) +
         0.5 * e.b0sq * pow_half(e, i[2], e.beta) * (i[0] * i[0] / 3.0 - i[1]);
}
// entropy(eos, e, G) (EquationsOfState.jl:139-156)
HYP_HD double entropy_eG(const EosC& e, double eint, const double* G) {
  double i[3];
  invariants_general(G, i);
  double pa = pow_half(e, i[2], e.alpha) - 1.0;
  double x = eint - 0.5 * e.b0sq * pow_half(e, i[2], e.beta) * (i[0] * i[0] / 3.0 - i[1]) - e.kU * pa * pa;
  x = x / (e.cvt0 * pow_half(e, i[2], e.gamma)) + 1.0;
  if (x < 1e-6) x = 1e-6;
  return log(x) * e.cv;
}
// finger(A) = (A A^T)^-1, column-major 9-vector (Strains.jl:26-32)
HYP_HD void finger_A(const double* A, double* g) {
  Kin k = kinematics(A, det3(A));
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) g[i + 3 * j] = sym_at(k.G, i, j);
}

}  // namespace hyp
