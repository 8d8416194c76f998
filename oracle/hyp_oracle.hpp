// oracle/hyp_oracle.hpp -- CPU restatement of BlackSiberian/HyperelasticSolver's
// explicit first-order finite-volume step (single-phase and two-phase
// hyperelasticity, Barton2009 EOS, Rusanov / LxF / path-conservative HLL).
//
// TEST INFRASTRUCTURE ONLY: this is the oracle. Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference arm load it, and only as the checker
// (or, for the reference arm, as the timed CPU restatement of the reference).
// The GPU product never links, calls or falls back to it.
//
// PARITY STATUS: unpinned against the reference's own execution. The reference is
// Julia; Julia is absent here and on the GPU host, and the reference ships no tests,
// golden vectors or fixtures. This restatement follows the reference's expression
// graphs operation by operation (same association order, LU determinant where the
// reference calls LinearAlgebra.det, cofactor formulas where it calls SimpleLA,
// forward-mode duals where it calls ForwardDiff). It is checked against physics
// known-answer tests, against LAPACK eigenvalues (numpy) and against an
// independent pure-Python transliteration (oracle/literal.py).
//
// Conventions: every 9-vector is a column-major 3x3 matrix, m(i,j) = m[i + 3*j]
// (0-based), as the reference's reshape(x, (3,3)). A phase state is the
// reference's 15-vector [alpha, alpha*rho, alpha*rho*u(3), alpha*rho*E,
// alpha*rho*A(9)] (HyperelasticityMPh.jl:80-84). The single-phase model is the
// same per-phase math with alpha == 1 (14 stored values, alpha dropped).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <type_traits>
#include "dual.hpp"

namespace hyp_oracle {

// ---------------------------------------------------------------------------
// EquationsOfState.jl:71-116  Barton2009 parameters and the derived b0sq, k0.
// The moduli b0sq and k0 have the type PM: double, or a dual number when the
// oracle differentiates a run with respect to them (forward mode).
template <class PM> struct BartonT {
  double rho0, c0, cv, t0, b0, alpha, beta, gamma;
  PM b0sq, k0;
};
using Barton = BartonT<double>;
inline Barton make_barton(double rho0 = 8.93, double c0 = 4.6, double cv = 3.9e-4, double t0 = 300,
                          double b0 = 2.1, double alpha = 1, double beta = 3, double gamma = 2) {
  Barton e{rho0, c0, cv, t0, b0, alpha, beta, gamma, 0, 0};
  e.b0sq = b0 * b0;                               // b0^2            (:111)
  e.k0 = c0 * c0 - (4.0 / 3.0) * (b0 * b0);       // c0^2 - 4/3 b0^2 (:112)
  return e;
}

#define M3(m, i, j) (m)[(i) + 3 * (j)]

// ---------------------------------------------------------------------------
// SimpleLA.jl:84-89  det_ by cofactor expansion along row 1.
template <class T> T det_(const T* m) {
  return M3(m, 0, 0) * (M3(m, 1, 1) * M3(m, 2, 2) - M3(m, 2, 1) * M3(m, 1, 2)) -
         M3(m, 0, 1) * (M3(m, 1, 0) * M3(m, 2, 2) - M3(m, 1, 2) * M3(m, 2, 0)) +
         M3(m, 0, 2) * (M3(m, 1, 0) * M3(m, 2, 1) - M3(m, 1, 1) * M3(m, 2, 0));
}
// SimpleLA.jl:94-96
template <class T> T tr_(const T* m) { return (M3(m, 0, 0) + M3(m, 1, 1)) + M3(m, 2, 2); }
// SimpleLA.jl:51-79  inverse by adjugate, multiplied by 1/det.
template <class T> void inv_(const T* m, T* r) {
  T dt = det_(m);
  T invdet = 1.0 / dt;
  M3(r, 0, 0) = (M3(m, 1, 1) * M3(m, 2, 2) - M3(m, 2, 1) * M3(m, 1, 2)) * invdet;
  M3(r, 0, 1) = (M3(m, 0, 2) * M3(m, 2, 1) - M3(m, 0, 1) * M3(m, 2, 2)) * invdet;
  M3(r, 0, 2) = (M3(m, 0, 1) * M3(m, 1, 2) - M3(m, 0, 2) * M3(m, 1, 1)) * invdet;
  M3(r, 1, 0) = (M3(m, 1, 2) * M3(m, 2, 0) - M3(m, 1, 0) * M3(m, 2, 2)) * invdet;
  M3(r, 1, 1) = (M3(m, 0, 0) * M3(m, 2, 2) - M3(m, 0, 2) * M3(m, 2, 0)) * invdet;
  M3(r, 1, 2) = (M3(m, 1, 0) * M3(m, 0, 2) - M3(m, 0, 0) * M3(m, 1, 2)) * invdet;
  M3(r, 2, 0) = (M3(m, 1, 0) * M3(m, 2, 1) - M3(m, 2, 0) * M3(m, 1, 1)) * invdet;
  M3(r, 2, 1) = (M3(m, 2, 0) * M3(m, 0, 1) - M3(m, 0, 0) * M3(m, 2, 1)) * invdet;
  M3(r, 2, 2) = (M3(m, 0, 0) * M3(m, 1, 1) - M3(m, 1, 0) * M3(m, 0, 1)) * invdet;
}
// Julia's 3x3 matrix product (LinearAlgebra matmul3x3): left-to-right sums.
template <class T> void matmul3(const T* a, const T* b, T* c) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i)
      M3(c, i, j) = (M3(a, i, 0) * M3(b, 0, j) + M3(a, i, 1) * M3(b, 1, j)) + M3(a, i, 2) * M3(b, 2, j);
}
// LinearAlgebra.det on a 3x3 matrix: LU with partial (row-maximum) pivoting,
// scaling by the pivot's inverse, det = prod(diag(U)) * (-1)^(#swaps).
// (HyperelasticityMPh.jl:114,152,187; EquationsOfState.jl:180,228.)
template <class T> T det_lu(const T* m_in) {
  T a[9];
  for (int i = 0; i < 9; ++i) a[i] = m_in[i];
  int swaps = 0;
  for (int k = 0; k < 3; ++k) {
    int kp = k;
    double amax = std::fabs(value_of(M3(a, k, k)));
    for (int i = k + 1; i < 3; ++i) {
      double absi = std::fabs(value_of(M3(a, i, k)));
      if (absi > amax) { kp = i; amax = absi; }
    }
    if (value_of(M3(a, kp, k)) != 0.0) {
      if (kp != k) {
        ++swaps;
        for (int j = 0; j < 3; ++j) std::swap(M3(a, k, j), M3(a, kp, j));
      }
      T akkinv = inv(M3(a, k, k));
      for (int i = k + 1; i < 3; ++i) M3(a, i, k) = M3(a, i, k) * akkinv;
    }
    for (int j = k + 1; j < 3; ++j)
      for (int i = k + 1; i < 3; ++i) M3(a, i, j) = M3(a, i, j) - M3(a, i, k) * M3(a, k, j);
  }
  T p = T(1.0);
  for (int i = 0; i < 3; ++i) p = p * M3(a, i, i);
  return (swaps & 1) ? p * -1.0 : p;
}

// ---------------------------------------------------------------------------
// Strains.jl:26-32  finger(a) = inv_(a * transpose(a))[:]
template <class T> void finger(const T* a, T* g) {
  T at[9], aat[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M3(at, i, j) = M3(a, j, i);
  matmul3(a, at, aat);
  inv_(aat, g);
}
// Strains.jl:46-52  (tr g, 0.5*(tr(g)^2 - tr(g^2)), det_ g)
template <class T> void invariants(const T* g, T* out) {
  T g2[9];
  matmul3(g, g, g2);
  T i1 = tr_(g);
  out[0] = i1;
  out[1] = 0.5 * (ipow2(tr_(g)) - tr_(g2));
  out[2] = det_(g);
}

// ---------------------------------------------------------------------------
// EquationsOfState.jl:118-137  Barton2009 internal energy e(S, G).
template <class T, class S, class PM> T energy(const BartonT<PM>& e, const S& ent, const T* G) {
  T i[3];
  invariants(G, i);
  T U = ((0.5 * e.k0) / (e.alpha * e.alpha)) * ipow2(pow(i[2], 0.5 * e.alpha) - 1.0) +
        ((e.cv * e.t0) * pow(i[2], 0.5 * e.gamma)) * (exp(ent / e.cv) - 1.0);
  T W = ((0.5 * e.b0sq) * pow(i[2], 0.5 * e.beta)) * (ipow2(i[0]) / 3.0 - i[1]);
  return U + W;
}
// EquationsOfState.jl:139-156  entropy from internal energy, argument clamped at 1e-6.
template <class T, class PM> T entropy(const BartonT<PM>& e, const T& e_int, const T* G) {
  T i[3];
  invariants(G, i);
  T S = (e_int - ((0.5 * e.b0sq) * pow(i[2], 0.5 * e.beta)) * (ipow2(i[0]) / 3.0 - i[1])) -
        ((0.5 * e.k0) / (e.alpha * e.alpha)) * ipow2(pow(i[2], 0.5 * e.alpha) - 1.0);
  S = S / ((e.cv * e.t0) * pow(i[2], 0.5 * e.gamma)) + 1.0;
  if (S < 1e-6) S = T(1e-6);
  return log(S) * e.cv;
}

// ForwardDiff.gradient(G -> energy(eos, ent, G), G) with one chunk of 9.
template <class T, class S, class PM> void denergy_dG(const BartonT<PM>& e, const S& ent, const T* G, T* dedG) {
  using D = Dual<T, 9>;
  D g[9];
  for (int k = 0; k < 9; ++k) {
    g[k] = D(G[k]);
    g[k].d[k] = T(1.0);
  }
  D en = energy(e, ent, g);
  for (int k = 0; k < 9; ++k) dedG[k] = en.d[k];
}

// EquationsOfState.jl:179-190  Cauchy stress sigma = -2 rho G dE/dG,
// rho = rho0/det(F) (LU), G = finger(F).
template <class T, class S, class PM> void stress(const BartonT<PM>& e, const S& ent, const T* F, T* sig) {
  T den = e.rho0 / det_lu(F);
  T G[9], dedG[9], a[9];
  finger(F, G);
  denergy_dG(e, ent, G, dedG);
  T m2den = den * -2.0;
  for (int k = 0; k < 9; ++k) a[k] = m2den * G[k];
  matmul3(a, dedG, sig);
}

// EquationsOfState.jl:223-246  acoustic tensor for direction n:
// dTdF = jacobian(F -> stress(eos, ent, F), F) reshaped (3,3,3,3),
// A = (1/den) * dTdF, acoustic[i,j] = sum_{k,l,m} A[m,i,j,l] F[k,l] n[m] n[k].
template <class T, class S, class PM> void acoustic(const BartonT<PM>& e, const S& ent, const T* F, const double* n, T* ac) {
  using D = Dual<T, 9>;
  D f[9], sd[9];
  for (int k = 0; k < 9; ++k) {
    f[k] = D(F[k]);
    f[k].d[k] = T(1.0);
  }
  stress(e, ent, f, sd);  // sd[p].d[q] = d sigma_p / d F_q
  T den = e.rho0 / det_lu(F);
  T rden = 1.0 / den;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T acc = T(0.0);
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
          for (int m = 0; m < 3; ++m) {
            // A[m,i,j,l] = rden * J[p][q], p = m + 3i, q = j + 3l
            T A = rden * sd[m + 3 * i].d[j + 3 * l];
            acc = acc + ((A * M3(F, k, l)) * n[m]) * n[k];
          }
      M3(ac, i, j) = acc;
    }
}

// EquationsOfState.jl:162-176  stress(eos, den, e_int, F): S = entropy(eos, e_int,
// finger(F)), then -2 den G dE/dG at that entropy (the gradient over G with S held).
template <class T, class U, class PM>
void stress_den(const BartonT<PM>& e, const U& den, const U& e_int, const T* F, T* sig) {
  T G[9], dedG[9], a[9];
  finger(F, G);
  T S = entropy(e, T(e_int), G);
  denergy_dG(e, S, G, dedG);
  for (int k = 0; k < 9; ++k) a[k] = (den * -2.0) * G[k];
  matmul3(a, dedG, sig);
}

// EquationsOfState.jl:192-221  acoustic(eos, P, n), P = [alpha, rho, u(3), S, A(9)]:
// den = P[1] P[2], e_int = energy(eos, S, finger(F)), the jacobian over F of
// stress(eos, den, e_int, F) (den and e_int held, the entropy following F),
// A = (1/den) dTdF, then the contraction of :207-218.
inline void acoustic_prim(const Barton& e, const double* P, const double* n, double* ac) {
  const double den = P[0] * P[1];
  const double ent = P[5];
  const double* F = P + 6;
  double G0[9];
  finger(F, G0);
  const double e_int = energy(e, ent, G0);
  using D = Dual<double, 9>;
  D f[9], sd[9];
  for (int k = 0; k < 9; ++k) {
    f[k] = D(F[k]);
    f[k].d[k] = 1.0;
  }
  stress_den(e, den, e_int, f, sd);
  const double rden = 1.0 / den;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
          for (int m = 0; m < 3; ++m) {
            double A = rden * sd[m + 3 * i].d[j + 3 * l];
            acc = acc + ((A * M3(F, k, l)) * n[m]) * n[k];
          }
      M3(ac, i, j) = acc;
    }
}

// ---------------------------------------------------------------------------
// EquationsOfState.jl:305-366  Hank2016: energy(eos, den, pres, G), pressure(eos,
// den, e_int, i), stress(eos, den, pres, distortion) = -2 den G dE/dG with
// G = finger(inv(F)) and the gradient by forward-mode duals (ForwardDiff.gradient).
struct Hank2016 {
  double rho0, mu, gamma, pres_inf, a;
};
template <class T> T hank_e_el(const Hank2016& h, const T* i) {
  T j1 = i[0] / pow(i[2], 1.0 / 3.0);
  T j2 = (ipow2(i[0]) - 2.0 * i[1]) / pow(i[2], 2.0 / 3.0);
  return h.mu / (4.0 * h.rho0) * (((1.0 - 2.0 * h.a) / 3.0 * ipow2(j1) + h.a * j2) + 3.0 * (h.a - 1.0));
}
template <class T> T hank_energy(const Hank2016& h, double den, double pres, const T* G) {
  T i[3];
  invariants(G, i);
  T e_el = hank_e_el(h, i);
  double e_h = (pres + h.gamma * h.pres_inf) / (den * (h.gamma - 1.0));
  return e_el + e_h;
}
inline double hank_pressure(const Hank2016& h, double den, double e_int, const double* i) {
  double e_h = e_int - hank_e_el(h, i);
  return e_h * (h.gamma - 1.0) * den - h.gamma * h.pres_inf;
}
inline void hank_stress(const Hank2016& h, double den, double pres, const double* F, double* sig) {
  double Fi[9], G[9];
  inv_(F, Fi);
  finger(Fi, G);
  using D = Dual<double, 9>;
  D g[9];
  for (int k = 0; k < 9; ++k) {
    g[k] = D(G[k]);
    g[k].d[k] = 1.0;
  }
  D e = hank_energy(h, den, pres, g);
  double dedG[9], a[9];
  for (int k = 0; k < 9; ++k) dedG[k] = e.d[k];
  for (int k = 0; k < 9; ++k) a[k] = (-2.0 * den) * G[k];
  matmul3(a, dedG, sig);
}

// ---------------------------------------------------------------------------
// Eigenvalue moduli of a real 3x3 matrix (the reference calls LAPACK
// `eigvals`, HyperelasticityMPh.jl:263, and consumes only sqrt(abs(.))).
// Characteristic polynomial mu^3 - c2 mu^2 + c1 mu - c0; closed-form
// (trigonometric / Cardano) seeds, Newton polishing of the real root of
// largest modulus, and deflation to a quadratic for the other two.
// A symmetric matrix (the acoustic tensor of a hyperelastic material is one, to
// rounding) takes classical Jacobi rotations instead, in plain double: LAPACK's
// eigenvalues of such a matrix are accurate to a few ulps even for a repeated pair
// (the rest state's b0^2, b0^2), which a deflated quadratic resolves only to about
// the square root of the rounding.
inline bool eig3_symmetric(const double* a) {
  double mx = 0.0;
  for (int k = 0; k < 9; ++k) mx = std::max(mx, std::fabs(a[k]));
  const double tol = 64.0 * 2.220446049250313e-16 * 0.5 * mx;
  return std::fabs(M3(a, 0, 1) - M3(a, 1, 0)) <= tol && std::fabs(M3(a, 0, 2) - M3(a, 2, 0)) <= tol &&
         std::fabs(M3(a, 1, 2) - M3(a, 2, 1)) <= tol;
}

// Classical Jacobi (largest off-diagonal entry first) on the symmetric part.
inline void eig3_jacobi(const double* a, double* ev) {
  double m[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m[i][j] = 0.5 * (M3(a, i, j) + M3(a, j, i));
  for (int it = 0; it < 100; ++it) {
    int p = 0, q = 1;
    if (std::fabs(m[0][2]) > std::fabs(m[p][q])) { p = 0; q = 2; }
    if (std::fabs(m[1][2]) > std::fabs(m[p][q])) { p = 1; q = 2; }
    const double apq = m[p][q];
    const double scale = std::fabs(m[0][0]) + std::fabs(m[1][1]) + std::fabs(m[2][2]);
    if (apq == 0.0 || std::fabs(apq) <= 1e-22 * scale) break;
    const double phi = 0.5 * std::atan2(2.0 * apq, m[q][q] - m[p][p]);
    const double c = std::cos(phi), sn = std::sin(phi);
    // rows/columns p, q of R^T m R with R the rotation in the (p, q) plane
    double np[3], nq[3];
    for (int k = 0; k < 3; ++k) {
      np[k] = c * m[p][k] - sn * m[q][k];
      nq[k] = sn * m[p][k] + c * m[q][k];
    }
    for (int k = 0; k < 3; ++k) {
      m[p][k] = np[k];
      m[q][k] = nq[k];
    }
    for (int k = 0; k < 3; ++k) {
      const double kp = c * m[k][p] - sn * m[k][q], kq = sn * m[k][p] + c * m[k][q];
      m[k][p] = kp;
      m[k][q] = kq;
    }
    m[p][q] = m[q][p] = 0.0;
  }
  for (int k = 0; k < 3; ++k) ev[k] = m[k][k];
}

template <class T> void eig3_moduli(const T* a, T* mods) {
  if constexpr (std::is_same<T, double>::value) {
    if (eig3_symmetric(a)) {
      eig3_jacobi(a, mods);
      for (int k = 0; k < 3; ++k) mods[k] = std::fabs(mods[k]);
      return;
    }
  }
  T c2 = (M3(a, 0, 0) + M3(a, 1, 1)) + M3(a, 2, 2);
  T c1 = ((M3(a, 0, 0) * M3(a, 1, 1) - M3(a, 0, 1) * M3(a, 1, 0)) +
          (M3(a, 0, 0) * M3(a, 2, 2) - M3(a, 0, 2) * M3(a, 2, 0))) +
         (M3(a, 1, 1) * M3(a, 2, 2) - M3(a, 1, 2) * M3(a, 2, 1));
  T c0 = det_(a);
  double C2 = value_of(c2), C1 = value_of(c1), C0 = value_of(c0);
  // seed in double
  double p = C1 - C2 * C2 / 3.0;
  double q = -2.0 * C2 * C2 * C2 / 27.0 + C2 * C1 / 3.0 - C0;
  double disc = (q * 0.5) * (q * 0.5) + (p / 3.0) * (p / 3.0) * (p / 3.0);
  double seed;
  if (disc < 0.0 && p < 0.0) {
    double m = 2.0 * std::sqrt(-p / 3.0);
    double c = 3.0 * q / (p * m);
    c = std::max(-1.0, std::min(1.0, c));
    double th = std::acos(c) / 3.0;
    seed = 0.0;
    for (int k = 0; k < 3; ++k) {
      double y = m * std::cos(th - 2.0 * M_PI * k / 3.0) + C2 / 3.0;
      if (std::fabs(y) > std::fabs(seed)) seed = y;
    }
  } else {
    double sd = std::sqrt(std::max(disc, 0.0));
    seed = std::cbrt(-q * 0.5 + sd) + std::cbrt(-q * 0.5 - sd) + C2 / 3.0;
  }
  // Newton polishing in double, then two steps in T (converges the partials).
  double r = seed;
  for (int it = 0; it < 50; ++it) {
    double f = ((r - C2) * r + C1) * r - C0;
    double fp = (3.0 * r - 2.0 * C2) * r + C1;
    if (fp == 0.0) break;
    double dr = f / fp;
    r -= dr;
    if (std::fabs(dr) <= 1e-16 * std::fabs(r)) break;
  }
  T rt = T(r);
  for (int it = 0; it < 2; ++it) {
    T f = ((rt - c2) * rt + c1) * rt - c0;
    T fp = (3.0 * rt - 2.0 * c2) * rt + c1;
    if (value_of(fp) == 0.0) break;
    rt = rt - f / fp;
  }
  mods[0] = abs(rt);
  T s = c2 - rt;
  if (value_of(rt) == 0.0) {  // singular matrix: remaining roots of mu^2 - c2 mu + c1
    s = c2;
    T qq = c1;
    T dsc = s * s - 4.0 * qq;
    if (value_of(dsc) < 0.0) {
      mods[1] = mods[2] = sqrt(abs(qq));
    } else {
      T sq = sqrt(dsc);
      mods[1] = abs((s + sq) * 0.5);
      mods[2] = abs((s - sq) * 0.5);
    }
    return;
  }
  T qq = c0 / rt;  // product of the other two roots
  T dsc = s * s - 4.0 * qq;
  if (value_of(dsc) < 0.0) {
    T m = sqrt(qq);
    mods[1] = m;
    mods[2] = m;
  } else {
    T sq = sqrt(dsc);
    T ra = value_of(s) >= 0.0 ? (s + sq) * 0.5 : (s - sq) * 0.5;
    mods[1] = abs(ra);
    mods[2] = value_of(ra) == 0.0 ? abs(s - ra) : abs(qq / ra);
  }
}

// The eigenvalues of a real 3x3 in the order Julia's `eigvals` returns them
// (HyperelasticityMPh.jl:263): LinearAlgebra sorts them by default
// lexicographically by (real, imag). Returned as moduli |mu| (what
// sqrt.(abs.(eigvals(ac))) consumes). Roots: Jacobi for a matrix symmetric to
// rounding (the symmetric path Julia's eigvals takes for an exactly symmetric
// matrix), else the Newton-polished real root of the characteristic polynomial
// and the two roots of the deflated quadratic (complex when its discriminant is
// negative).
inline void eig3_sorted(const double* a, double* mods) {
  double re[3], im[3], md[3];
  if (eig3_symmetric(a)) {
    eig3_jacobi(a, re);
    for (int k = 0; k < 3; ++k) {
      im[k] = 0.0;
      md[k] = std::fabs(re[k]);
    }
  } else {
    const double c2 = (M3(a, 0, 0) + M3(a, 1, 1)) + M3(a, 2, 2);
    const double c1 = ((M3(a, 0, 0) * M3(a, 1, 1) - M3(a, 0, 1) * M3(a, 1, 0)) +
                       (M3(a, 0, 0) * M3(a, 2, 2) - M3(a, 0, 2) * M3(a, 2, 0))) +
                      (M3(a, 1, 1) * M3(a, 2, 2) - M3(a, 1, 2) * M3(a, 2, 1));
    const double c0 = det_(a);
    const double p = c1 - c2 * c2 / 3.0;
    const double q = -2.0 * c2 * c2 * c2 / 27.0 + c2 * c1 / 3.0 - c0;
    const double disc = (q * 0.5) * (q * 0.5) + (p / 3.0) * (p / 3.0) * (p / 3.0);
    double r;
    if (disc < 0.0 && p < 0.0) {
      const double m = 2.0 * std::sqrt(-p / 3.0);
      const double th = std::acos(std::max(-1.0, std::min(1.0, 3.0 * q / (p * m)))) / 3.0;
      r = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double y = m * std::cos(th - 2.0 * M_PI * k / 3.0) + c2 / 3.0;
        if (std::fabs(y) > std::fabs(r)) r = y;
      }
    } else {
      const double sd = std::sqrt(std::max(disc, 0.0));
      r = std::cbrt(-q * 0.5 + sd) + std::cbrt(-q * 0.5 - sd) + c2 / 3.0;
    }
    for (int it = 0; it < 50; ++it) {
      const double f = ((r - c2) * r + c1) * r - c0;
      const double fp = (3.0 * r - 2.0 * c2) * r + c1;
      if (fp == 0.0) break;
      const double dr = f / fp;
      r -= dr;
      if (std::fabs(dr) <= 1e-16 * std::fabs(r)) break;
    }
    const double sm = r != 0.0 ? c2 - r : c2, pr = r != 0.0 ? c0 / r : c1;
    const double dsc = sm * sm - 4.0 * pr;
    re[0] = r;
    im[0] = 0.0;
    md[0] = std::fabs(r);
    if (dsc < 0.0) {
      re[1] = re[2] = 0.5 * sm;
      im[1] = -0.5 * std::sqrt(-dsc);
      im[2] = -im[1];
      md[1] = md[2] = std::sqrt(std::fabs(pr));
    } else {
      const double sq = std::sqrt(dsc);
      const double ra = sm >= 0.0 ? 0.5 * (sm + sq) : 0.5 * (sm - sq);
      const double rb = ra != 0.0 ? pr / ra : sm - ra;
      re[1] = ra;
      re[2] = rb;
      im[1] = im[2] = 0.0;
      md[1] = std::fabs(ra);
      md[2] = std::fabs(rb);
    }
  }
  int ord[3] = {0, 1, 2};
  std::sort(ord, ord + 3, [&](int x, int y) { return re[x] < re[y] || (re[x] == re[y] && im[x] < im[y]); });
  for (int k = 0; k < 3; ++k) mods[k] = md[ord[k]];
}

// ---------------------------------------------------------------------------
// HyperelasticityMPh.jl:106-133  cons2prim for one phase.
// Q[1] (alpha*rho) is never read: density comes from det(Q[7:15]/alpha).
template <class T, class PM> void cons2prim(const BartonT<PM>& e, const T* Q, T* P) {
  T frac = Q[0];
  T FQ[9];
  for (int k = 0; k < 9; ++k) FQ[k] = Q[6 + k] / frac;
  T true_den = sqrt(det_lu(FQ) / e.rho0);
  T den = frac * true_den;
  T vel[3];
  for (int k = 0; k < 3; ++k) vel[k] = Q[2 + k] / den;
  T e_total = Q[5] / den;
  T e_kin = ((ipow2(vel[0]) + ipow2(vel[1])) + ipow2(vel[2])) / 2.0;
  T e_int = e_total - e_kin;
  T A[9], G[9];
  for (int k = 0; k < 9; ++k) A[k] = Q[6 + k] / den;
  finger(A, G);
  T ent = entropy(e, e_int, G);
  P[0] = frac;
  P[1] = true_den;
  for (int k = 0; k < 3; ++k) P[2 + k] = vel[k];
  P[5] = ent;
  for (int k = 0; k < 9; ++k) P[6 + k] = A[k];
}
// HyperelasticityMPh.jl:66-87  prim2cons for one phase.
template <class T, class PM> void prim2cons(const BartonT<PM>& e, const T* P, T* Q) {
  T frac = P[0], true_den = P[1];
  T den = frac * true_den;
  T G[9];
  finger(P + 6, G);
  T e_int = energy(e, P[5], G);
  T e_kin = ((ipow2(P[2]) + ipow2(P[3])) + ipow2(P[4])) / 2.0;
  T e_total = e_int + e_kin;
  Q[0] = frac;
  Q[1] = den;
  for (int k = 0; k < 3; ++k) Q[2 + k] = den * P[2 + k];
  Q[5] = den * e_total;
  for (int k = 0; k < 9; ++k) Q[6 + k] = den * P[6 + k];
}

// HyperelasticityMPh.jl:146-175  physical x-flux for one phase.
template <class T, class PM> void flux(const BartonT<PM>& e, const T* Q, T* Fx) {
  T frac = Q[0];
  T FQ[9];
  for (int k = 0; k < 9; ++k) FQ[k] = Q[6 + k] / frac;
  T true_den = sqrt(det_lu(FQ) / e.rho0);
  T den = frac * true_den;
  T vel[3];
  for (int k = 0; k < 3; ++k) vel[k] = Q[2 + k] / den;
  T e_total = Q[5] / den;
  T e_kin = ((ipow2(vel[0]) + ipow2(vel[1])) + ipow2(vel[2])) / 2.0;
  T e_int = e_total - e_kin;
  T A[9], G[9], s1[9], strs[9];
  for (int k = 0; k < 9; ++k) A[k] = Q[6 + k] / den;
  finger(A, G);
  T ent = entropy(e, e_int, G);
  stress(e, ent, A, s1);
  for (int k = 0; k < 9; ++k) strs[k] = frac * s1[k];
  // strs[begin:3:end] = elements 1,4,7 = row 1 of sigma
  T r0 = strs[0], r1 = strs[3], r2 = strs[6];
  T du = den * vel[0];
  Fx[0] = T(0.0);
  Fx[1] = du;
  Fx[2] = du * vel[0] - r0;
  Fx[3] = du * vel[1] - r1;
  Fx[4] = du * vel[2] - r2;
  Fx[5] = du * e_total - ((vel[0] * r0 + vel[1] * r1) + vel[2] * r2);
  T arow[3] = {A[0], A[3], A[6]};
  for (int b = 0; b < 3; ++b)
    for (int a = 0; a < 3; ++a)
      Fx[6 + a + 3 * b] = den * (vel[0] * M3(A, a, b) - vel[a] * arow[b]);
}

// HyperelasticityMPh.jl:258-266  wave speeds u.n +- sqrt|eig(acoustic)| for one phase
// (n = e1 on the step's path). In plain double the moduli come in Julia's eigvals
// order (eig3_sorted); the dual-number runs consume only their min and max.
template <class T, class PM> void eigvals_phase(const BartonT<PM>& e, const T* Q, T* spd6, const double* n = nullptr) {
  static const double e1[3] = {1.0, 0.0, 0.0};
  if (!n) n = e1;
  T P[15];
  cons2prim(e, Q, P);
  T ac[9], mods[3];
  acoustic(e, P[5], P + 6, n, ac);
  if constexpr (std::is_same<T, double>::value) {
    eig3_sorted(ac, mods);
  } else {
    eig3_moduli(ac, mods);
  }
  T spd = ((T(0.0) + P[2] * n[0]) + P[3] * n[1]) + P[4] * n[2];  // dot(P[3:5], n)
  for (int k = 0; k < 3; ++k) {
    T c = sqrt(mods[k]);
    spd6[k] = spd + c;
    spd6[3 + k] = spd - c;
  }
}

// HyperelasticityMPh.jl:178-250  non-conservative matrix B of the two-phase
// model. Only column 1 of each 15x15 phase block is non-zero, so it is returned
// as bcol[30]: bcol[r] = B[r, 1] for r in phase 1 and B[r, 16] for phase 2.
template <class T, class PM> void noncons_cols(const BartonT<PM>* eos, const T* Q, T* bcol) {
  T frac[2], true_den[2], den[2], vel[2][3], e_total[2], e_int[2], A[2][9], G[2][9], ent[2], strs[2][9], temp[2];
  for (int p = 0; p < 2; ++p) {
    const T* q = Q + 15 * p;
    frac[p] = q[0];
    T FQ[9];
    for (int k = 0; k < 9; ++k) FQ[k] = q[6 + k] / frac[p];
    true_den[p] = sqrt(det_lu(FQ) / eos[p].rho0);
    den[p] = frac[p] * true_den[p];
    for (int k = 0; k < 3; ++k) vel[p][k] = q[2 + k] / den[p];
    e_total[p] = q[5] / den[p];
    T e_kin = ((ipow2(vel[p][0]) + ipow2(vel[p][1])) + ipow2(vel[p][2])) / 2.0;
    e_int[p] = e_total[p] - e_kin;
    for (int k = 0; k < 9; ++k) A[p][k] = q[6 + k] / den[p];
  }
  for (int p = 0; p < 2; ++p) finger(A[p], G[p]);
  for (int p = 0; p < 2; ++p) ent[p] = entropy(eos[p], e_int[p], G[p]);
  for (int p = 0; p < 2; ++p) {
    T s1[9];
    stress(eos[p], ent[p], A[p], s1);
    for (int k = 0; k < 9; ++k) strs[p][k] = frac[p] * s1[k];
  }
  // temp_p = derivative(S -> energy(eos_p, S, G_p), ent_p)  (:212)
  for (int p = 0; p < 2; ++p) {
    Dual<T, 1> s(ent[p]);
    s.d[0] = T(1.0);
    Dual<T, 1> gg[9];
    for (int k = 0; k < 9; ++k) gg[k] = Dual<T, 1>(G[p][k]);
    temp[p] = energy(eos[p], s, gg).d[0];
  }
  const double k1 = 0.5, k2 = 1.0 - 0.5;  // k = [1/2, 1 - 1/2]; omega = 0; beta = 0
  T vel_i[3];
  for (int a = 0; a < 3; ++a) vel_i[a] = k1 * vel[0][a] + k2 * vel[1][a];
  // K_p = 1/frac_p .* strs_p  (omega = 0, beta = 0 make the other terms exact zeros)
  T K[2][9];
  for (int p = 0; p < 2; ++p) {
    T rf = 1.0 / frac[p];
    for (int k = 0; k < 9; ++k) K[p][k] = rf * strs[p][k];
  }
  T den_i = k1 * temp[0] + k2 * temp[1];
  T si[9];
  for (int k = 0; k < 9; ++k) si[k] = ((k2 * temp[1]) * K[0][k] + (k1 * temp[0]) * K[1][k]) / den_i;
  for (int p = 0; p < 2; ++p) {
    T* b = bcol + 15 * p;
    b[0] = vel_i[0];
    b[1] = T(0.0);
    for (int a = 0; a < 3; ++a) b[2 + a] = M3(si, a, 0);
    b[5] = (M3(si, 0, 0) * vel_i[0] + M3(si, 1, 0) * vel_i[1]) + M3(si, 2, 0) * vel_i[2];
    // rows 7..15: true_den * A[1, c] * vel[a]  at entry (a, c)
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) b[6 + a + 3 * c] = (true_den[p] * M3(A[p], 0, c)) * vel[p][a];
    // rows 7, 10, 13 += true_den * transpose(A) * (vel_i - vel)
    T dv[3];
    for (int a = 0; a < 3; ++a) dv[a] = vel_i[a] - vel[p][a];
    T At[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M3(At, i, j) = true_den[p] * M3(A[p], j, i);
    for (int c = 0; c < 3; ++c) {
      T mv = (M3(At, c, 0) * dv[0] + M3(At, c, 1) * dv[1]) + M3(At, c, 2) * dv[2];
      b[6 + 3 * c] = b[6 + 3 * c] + mv;
    }
  }
}

// ---------------------------------------------------------------------------
// Quadrature on [0,1]: FastGaussQuadrature gausslegendre(6) / gausslobatto(6)
// (NumFluxes.jl:94-95, 36-37), mapped (x+1)/2, w/2. Nodes ascending.
struct Quad6 { double x[6], w[6]; };
inline long double legendre_p(int n, long double x, long double* dp) {
  long double p0 = 1.0L, p1 = x;
  for (int k = 2; k <= n; ++k) {
    long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    p0 = p1; p1 = p2;
  }
  *dp = n * (x * p1 - p0) / (x * x - 1.0L);
  return p1;
}
inline Quad6 gauss_legendre6_01() {
  Quad6 q;
  long double xs[6], ws[6];
  for (int i = 0; i < 6; ++i) {
    long double x = std::cos(M_PI * (i + 0.75L) / (6 + 0.5L));
    for (int it = 0; it < 100; ++it) {
      long double dp, p = legendre_p(6, x, &dp);
      long double dx = p / dp;
      x -= dx;
      if (std::fabs((double)dx) < 1e-30) break;
    }
    long double dp;
    legendre_p(6, x, &dp);
    xs[i] = x;
    ws[i] = 2.0L / ((1.0L - x * x) * dp * dp);
  }
  for (int i = 0; i < 6; ++i) {  // ascending
    double nx = (double)xs[5 - i], nw = (double)ws[5 - i];
    q.x[i] = (nx + 1.0) / 2.0;
    q.w[i] = nw / 2.0;
  }
  return q;
}
inline Quad6 gauss_lobatto6_01() {
  // nodes +-1, +-sqrt(1/3 -+ 2 sqrt(7)/21); weights 1/15, (14 +- sqrt 7)/30
  long double s7 = std::sqrt(7.0L);
  long double a = std::sqrt(1.0L / 3.0L + 2.0L * s7 / 21.0L);
  long double b = std::sqrt(1.0L / 3.0L - 2.0L * s7 / 21.0L);
  long double xs[6] = {-1.0L, -a, -b, b, a, 1.0L};
  long double ws[6] = {1.0L / 15.0L, (14.0L - s7) / 30.0L, (14.0L + s7) / 30.0L,
                       (14.0L + s7) / 30.0L, (14.0L - s7) / 30.0L, 1.0L / 15.0L};
  Quad6 q;
  for (int i = 0; i < 6; ++i) {
    double nx = (double)xs[i], nw = (double)ws[i];
    q.x[i] = (nx + 1.0) / 2.0;
    q.w[i] = nw / 2.0;
  }
  return q;
}

// ---------------------------------------------------------------------------
// Model-level wrappers. nvar = 14 (single phase, alpha == 1) or 30 (two phases).
enum { MODEL_SINGLE = 1, MODEL_MULTI = 2 };
enum { FLUX_RUSANOV = 0, FLUX_LXF = 1, FLUX_HLL = 2 };
enum { BC_FROZEN = 0, BC_TRANSMISSIVE = 1 };

// ---------------------------------------------------------------------------
// Instantaneous pressure relaxation of a two-phase cell (an extension: the reference
// has no relaxation terms, so nothing here is pinned to it). The procedure of Saurel,
// Petitpas & Berry (2009) with hyperelastic phases as Favrie, Gavrilyuk & Saurel (2009)
// treat them: unknowns alpha_1' and p*; per phase v' = alpha'/m, e' = e - p* (v' - v),
// the distortion scaled by (v'/v)^(1/3), and p(e', v') = p* where p = -tr(sigma)/3 of
// stress(eos, S, A') (the dual-number stress above) at S = entropy(eos, e', finger(A')).
// Newton's method on the 2x2 system, its derivatives by central differences.
inline double relax_pressure_of(const Barton& e, const double* A, double lam, double eint) {
  double As[9], G[9], sig[9];
  for (int c = 0; c < 9; ++c) As[c] = lam * A[c];
  finger(As, G);
  const double S = entropy(e, eint, G);
  stress(e, S, As, sig);
  return -(M3(sig, 0, 0) + M3(sig, 1, 1) + M3(sig, 2, 2)) / 3.0;
}
// Instantaneous velocity relaxation: both phases take the mixture velocity
// u* = sum m_k u_k / sum m_k; each phase's momentum becomes m_k u*, its total energy
// changes by m_k u* . (u* - u_k), so the mixture's momentum and energy are kept and
// each phase's internal energy grows by |u_k - u*|^2 / 2.
inline void relax_velocity2(const Barton* eos, double* Q) {
  double P[2][15], m[2];
  for (int k = 0; k < 2; ++k) {
    cons2prim(eos[k], Q + 15 * k, P[k]);
    m[k] = P[k][0] * P[k][1];
  }
  double us[3];
  for (int c = 0; c < 3; ++c) us[c] = (m[0] * P[0][2 + c] + m[1] * P[1][2 + c]) / (m[0] + m[1]);
  for (int k = 0; k < 2; ++k) {
    double* q = Q + 15 * k;
    double w = 0.0;
    for (int c = 0; c < 3; ++c) w += us[c] * (us[c] - P[k][2 + c]);
    q[5] = q[5] + m[k] * w;
    for (int c = 0; c < 3; ++c) q[2 + c] = m[k] * us[c];
  }
}
inline int relax_pressure2(const Barton* eos, double* Q) {
  constexpr double kMinAlpha = 1e-5;
  double P[2][15], m[2], v[2], a0[2] = {Q[0], Q[15]};
  if (!(a0[0] >= kMinAlpha && a0[1] >= kMinAlpha)) return 0;
  for (int k = 0; k < 2; ++k) {
    cons2prim(eos[k], Q + 15 * k, P[k]);
    m[k] = P[k][0] * P[k][1];
    v[k] = 1.0 / P[k][1];
  }
  double e0[2], A[2][9], ke[2];
  for (int k = 0; k < 2; ++k) {
    for (int c = 0; c < 9; ++c) A[k][c] = P[k][6 + c];
    ke[k] = 0.5 * (P[k][2] * P[k][2] + P[k][3] * P[k][3] + P[k][4] * P[k][4]);
    e0[k] = Q[15 * k + 5] / m[k] - ke[k];
  }
  auto pres = [&](int k, double vk, double ek) { return relax_pressure_of(eos[k], A[k], std::cbrt(vk / v[k]), ek); };
  double x = a0[0], ps = a0[0] * pres(0, v[0], e0[0]) + a0[1] * pres(1, v[1], e0[1]);
  double pscale = std::fabs(ps);
  for (int k = 0; k < 2; ++k) pscale = std::max(pscale, eos[k].k0 * eos[k].rho0);
  bool done = false;
  for (int it = 0; it < 40 && !done; ++it) {
    double F[2], Jx[2], Jp[2];
    for (int k = 0; k < 2; ++k) {
      const double ak = k == 0 ? x : 1.0 - x, vk = ak / m[k], ek = e0[k] - ps * (vk - v[k]);
      const double hv = 1e-7 * vk, he = 1e-7 * (std::fabs(ek) + std::fabs(ps * vk)) + 1e-12;
      const double p0 = pres(k, vk, ek);
      const double dpdv = (pres(k, vk + hv, ek) - pres(k, vk - hv, ek)) / (2.0 * hv);
      const double dpde = (pres(k, vk, ek + he) - pres(k, vk, ek - he)) / (2.0 * he);
      const double dvdx = k == 0 ? 1.0 / m[0] : -1.0 / m[1];
      F[k] = p0 - ps;
      Jx[k] = (dpdv - dpde * ps) * dvdx;
      Jp[k] = -dpde * (vk - v[k]) - 1.0;
    }
    const double det = Jx[0] * Jp[1] - Jx[1] * Jp[0];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) break;
    double dx = (-F[0] * Jp[1] + F[1] * Jp[0]) / det, dp = (-Jx[0] * F[1] + Jx[1] * F[0]) / det;
    for (int h = 0; h < 60 && !(x + dx > 0.0 && x + dx < 1.0); ++h) {
      dx *= 0.5;
      dp *= 0.5;
    }
    x += dx;
    ps += dp;
    done = std::fabs(dx) <= 1e-14 && std::fabs(dp) <= 1e-13 * pscale;
  }
  if (!done || !(x > 0.0 && x < 1.0) || !std::isfinite(ps)) return 8;  // not converged: left as it is
  for (int k = 0; k < 2; ++k) {
    const double ak = k == 0 ? x : 1.0 - x, vk = ak / m[k], ek = e0[k] - ps * (vk - v[k]);
    const double lam = std::cbrt(vk / v[k]);
    double* q = Q + 15 * k;
    q[0] = ak;
    q[5] = m[k] * (ek + ke[k]);
    for (int c = 0; c < 9; ++c) q[6 + c] = q[6 + c] * lam;
  }
  return 0;
}

template <class PM> struct ProblemT {
  int model;
  BartonT<PM> eos[2];
  int flux;
  int bc;
  int nx;
  double X;
  double cfl;
  int relax = 0;  // two-phase pressure relaxation after each step (an extension: relax_pressure2)
};
using Problem = ProblemT<double>;
inline int nvar_of(int model) { return model == MODEL_SINGLE ? 14 : 30; }
inline int nspd_of(int model) { return model == MODEL_SINGLE ? 6 : 12; }

template <class T> void expand1(const T* q14, T* q15) {
  q15[0] = T(1.0);
  for (int k = 0; k < 14; ++k) q15[1 + k] = q14[k];
}
// flux_mph (HyperelasticityMPh.jl:140-144) / single-phase flux at alpha == 1.
template <class T, class PM> void cell_flux(const ProblemT<PM>& pb, const T* Q, T* Fx) {
  if (pb.model == MODEL_SINGLE) {
    T q15[15], f15[15];
    expand1(Q, q15);
    flux(pb.eos[0], q15, f15);
    for (int k = 0; k < 14; ++k) Fx[k] = f15[1 + k];
  } else {
    flux(pb.eos[0], Q, Fx);
    flux(pb.eos[1], Q + 15, Fx + 15);
  }
}
// get_eigvals (HyperelasticityMPh.jl:252-256): all phases' speeds.
template <class T, class PM> void cell_speeds(const ProblemT<PM>& pb, const T* Q, T* spd, const double* n = nullptr) {
  if (pb.model == MODEL_SINGLE) {
    T q15[15];
    expand1(Q, q15);
    eigvals_phase(pb.eos[0], q15, spd, n);
  } else {
    eigvals_phase(pb.eos[0], Q, spd, n);
    eigvals_phase(pb.eos[1], Q + 15, spd + 6, n);
  }
}
template <class T> T max_abs(const T* v, int n) {
  T m = abs(v[0]);
  for (int i = 1; i < n; ++i) { T a = abs(v[i]); if (a > m) m = a; }
  return m;
}
template <class T> T min_of(const T* v, int n) {
  T m = v[0];
  for (int i = 1; i < n; ++i) if (v[i] < m) m = v[i];
  return m;
}
template <class T> T max_of(const T* v, int n) {
  T m = v[0];
  for (int i = 1; i < n; ++i) if (v[i] > m) m = v[i];
  return m;
}

// Path integral int_0^1 B(psi(s)) psi'(s) ds with psi(s) = Qa (1-s) + Qb s
// (NumFluxes.jl:97-107 / :39-47): sum_i (w_i * B_i) * (Qb - Qa).
template <class T, class PM> void path_integral(const ProblemT<PM>& pb, const Quad6& qd, const T* Qa, const T* Qb, T* out) {
  T dv[30], u[30], bcol[30], acc[30];
  for (int k = 0; k < 30; ++k) dv[k] = Qb[k] - Qa[k];
  for (int i = 0; i < 6; ++i) {
    double s = qd.x[i];
    for (int k = 0; k < 30; ++k) u[k] = Qa[k] * (1.0 - s) + Qb[k] * s;
    noncons_cols(pb.eos, u, bcol);
    for (int k = 0; k < 30; ++k) {
      T term = (qd.w[i] * bcol[k]) * dv[k < 15 ? 0 : 15];
      if (i == 0) acc[k] = term;
      else acc[k] = acc[k] + term;
    }
  }
  for (int k = 0; k < 30; ++k) out[k] = acc[k];
}

// NumFluxes.jl:25-60  lxf: cons = 0.5 (f_l + f_r) - 0.5 lambda (Q_r - Q_l),
// noncons D- = D+ = 0.5 * Gauss-Lobatto path integral (two-phase only).
template <class T, class PM> void lxf_face(const ProblemT<PM>& pb, const T* Ql, const T* Qr, const T& lambda, T* cons, T* dm, T* dp,
                                 const T* fl = nullptr, const T* fr = nullptr) {
  int nv = nvar_of(pb.model);
  T fl_[30], fr_[30];
  if (!fl) { cell_flux(pb, Ql, fl_); fl = fl_; }
  if (!fr) { cell_flux(pb, Qr, fr_); fr = fr_; }
  T hl = lambda * 0.5;
  for (int k = 0; k < nv; ++k) cons[k] = 0.5 * (fl[k] + fr[k]) - hl * (Qr[k] - Ql[k]);
  if (pb.model == MODEL_SINGLE) {
    for (int k = 0; k < nv; ++k) dm[k] = dp[k] = T(0.0);
  } else {
    static const Quad6 glo = gauss_lobatto6_01();
    T fp[30];
    path_integral(pb, glo, Ql, Qr, fp);
    for (int k = 0; k < 30; ++k) dm[k] = dp[k] = 0.5 * fp[k];
  }
}

// NumFluxes.jl:70-132  hll / hll_pathcons (two-phase). Returns D-, D+.
// literal = 1 repeats the evaluations the reference repeats (get_eigvals(Q_m)
// twice, flux_mph six times, B_int(Q_l,Q_hll) and B_int(Q_hll,Q_r) twice each);
// the results are identical, only the cost differs.
template <class T, class PM> void hll_face(const ProblemT<PM>& pb, const T* Ql, const T* Qr, const T* spdL, const T* spdR, T* dm, T* dp,
                                 int literal = 0) {
  const int reps = literal ? 2 : 1;
  T Qm[30], spdM[12];
  for (int k = 0; k < 30; ++k) Qm[k] = 0.5 * (Ql[k] + Qr[k]);
  for (int r = 0; r < reps; ++r) cell_speeds(pb, Qm, spdM);
  T mnm = min_of(spdM, 12), mnl = min_of(spdL, 12);
  T mxm = max_of(spdM, 12), mxr = max_of(spdR, 12);
  T sl = T(0.0); if (mnm < sl) sl = mnm; if (mnl < sl) sl = mnl;
  T sr = T(0.0); if (mxm > sr) sr = mxm; if (mxr > sr) sr = mxr;
  static const Quad6 gle = gauss_legendre6_01();
  T fl[30], fr[30];
  for (int r = 0; r < (literal ? 3 : 1); ++r) {  // one pair, or three as the reference evaluates
    cell_flux(pb, Ql, fl);
    cell_flux(pb, Qr, fr);
  }
  T b0[30], b1[30], b2[30], path_int[30], Qh[30];
  path_integral(pb, gle, Ql, Qr, b0);
  for (int k = 0; k < 30; ++k) path_int[k] = (b0[k] + fr[k]) - fl[k];
  T dsr = sr - sl;
  for (int k = 0; k < 30; ++k) Qh[k] = ((Qr[k] * sr - Ql[k] * sl) - path_int[k]) / dsr;
  for (int r = 0; r < reps; ++r) {
    path_integral(pb, gle, Ql, Qh, b1);
    path_integral(pb, gle, Qh, Qr, b2);
  }
  T cm = (-sl) / dsr, cp = sr / dsr, cq = (sl * sr) / dsr;
  for (int k = 0; k < 30; ++k) {
    T inner = ((fr[k] - fl[k]) + b1[k]) + b2[k];
    T jump = Qr[k] - Ql[k];
    dm[k] = cm * inner + cq * jump;
    dp[k] = cp * inner - cq * jump;
  }
}

// ---------------------------------------------------------------------------
// main.jl:202-227  one time step. Q is AoS [cell][nvar]. Returns dt.
// literal = 1: each interior cell calls the face flux twice, as update_cell does
// (main.jl:30-60); literal = 0: each face once. Both give identical results.
// dt_given (optional): use this time step instead of cfl*dx/max lambda (for checking a
// window of a larger run whose dt came from cells outside the window).
template <class T, class PM> T step(const ProblemT<PM>& pb, std::vector<T>& Q, int literal, int nthreads, T* lam_max_out = nullptr,
                          const T* dt_given = nullptr) {
  const int nx = pb.nx, nv = nvar_of(pb.model), ns = nspd_of(pb.model);
  const bool trans = pb.bc == BC_TRANSMISSIVE;
  std::vector<T> spd((size_t)nx * ns), lam(nx);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int i = 0; i < nx; ++i) {
    cell_speeds(pb, &Q[(size_t)i * nv], &spd[(size_t)i * ns]);
    lam[i] = max_abs(&spd[(size_t)i * ns], ns);
  }
  T lmax = lam[0];
  for (int i = 1; i < nx; ++i) if (lam[i] > lmax) lmax = lam[i];
  if (lam_max_out) *lam_max_out = lmax;
  const double dx = pb.X / nx;
  T dt = dt_given ? *dt_given : (pb.cfl * dx) / lmax;
  // Rusanov / HLL: update_cell(..., dt / dx, eos) (main.jl:224-225, 43-60).
  // LxF: update_cell(..., dx / dt, eos) with lambda = dx/dt (main.jl:223, 30-41).
  T lam_lxf = dx / dt;
  T dtdx = pb.flux == FLUX_LXF ? 1.0 / lam_lxf : dt / dx;
  std::vector<T> Q1(Q.size());
  const int i0 = trans ? 0 : 1, i1 = trans ? nx - 1 : nx - 2;
  if (!trans) {
    for (int k = 0; k < nv; ++k) {
      Q1[k] = Q[k];
      Q1[(size_t)(nx - 1) * nv + k] = Q[(size_t)(nx - 1) * nv + k];
    }
  }
  auto cellQ = [&](int j) { j = std::max(0, std::min(nx - 1, j)); return &Q[(size_t)j * nv]; };
  auto cellS = [&](int j) { j = std::max(0, std::min(nx - 1, j)); return &spd[(size_t)j * ns]; };
  auto cellL = [&](int j) { j = std::max(0, std::min(nx - 1, j)); return lam[j]; };
  // face fluxes: face f sits between cells f-1 and f (f = 0 .. nx)
  // returns (F, NF_minus, NF_plus) for the face
  auto face = [&](int f, T* F, T* dm, T* dp) {
    const T* Ql = cellQ(f - 1);
    const T* Qr = cellQ(f);
    if (pb.flux == FLUX_HLL) {
      for (int k = 0; k < nv; ++k) F[k] = T(0.0);  // hll returns zeros(30) as its first output
      hll_face(pb, Ql, Qr, cellS(f - 1), cellS(f), dm, dp, literal);
    } else {
      T lf = pb.flux == FLUX_RUSANOV ? (cellL(f - 1) > cellL(f) ? cellL(f - 1) : cellL(f)) : lam_lxf;
      lxf_face(pb, Ql, Qr, lf, F, dm, dp);
    }
  };
  if (literal) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
    for (int i = i0; i <= i1; ++i) {
      T Fl[30], dml[30], dpl[30], Fr[30], dmr[30], dpr[30];
      face(i, Fl, dml, dpl);      // flux_num(eos, Q_l, Q, ...)  -> F_l, _, NF_l (= D+)
      face(i + 1, Fr, dmr, dpr);  // flux_num(eos, Q, Q_r, ...)  -> F_r, NF_r (= D-), _
      const T* q = &Q[(size_t)i * nv];
      for (int k = 0; k < nv; ++k) Q1[(size_t)i * nv + k] = q[k] - dtdx * ((Fr[k] - Fl[k]) + (dmr[k] + dpl[k]));
    }
  } else {
    const int nf = nx + 1;
    std::vector<T> F((size_t)nf * nv), DM((size_t)nf * nv), DP((size_t)nf * nv);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
    for (int f = i0; f <= i1 + 1; ++f) face(f, &F[(size_t)f * nv], &DM[(size_t)f * nv], &DP[(size_t)f * nv]);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int i = i0; i <= i1; ++i) {
      const T* q = &Q[(size_t)i * nv];
      const T* Fl = &F[(size_t)i * nv];
      const T* Fr = &F[(size_t)(i + 1) * nv];
      const T* dmr = &DM[(size_t)(i + 1) * nv];
      const T* dpl = &DP[(size_t)i * nv];
      for (int k = 0; k < nv; ++k) Q1[(size_t)i * nv + k] = q[k] - dtdx * ((Fr[k] - Fl[k]) + (dmr[k] + dpl[k]));
    }
  }
  if constexpr (std::is_same<T, double>::value) {
    if (pb.model == MODEL_MULTI && pb.relax) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
      for (int i = i0; i <= i1; ++i) {
        double* q = &Q1[(size_t)i * nv];
        if (pb.relax == 2 && q[0] >= 1e-5 && q[15] >= 1e-5) relax_velocity2(pb.eos, q);
        relax_pressure2(pb.eos, q);
      }
    }
  }
  Q.swap(Q1);
  return dt;
}

}  // namespace hyp_oracle
