// hyp_physics_mph_mixed.cuh -- the two-phase physics of hyp_physics_mph.cuh in
// FP32 for the mixed-precision two-phase step.
//
// Per phase, cons2prim (HyperelasticityMPh.jl:106-133) of a cell's state keeps
// its cancellation-prone steps in float-float, as the single-phase mixed step does:
// det(alpha rho A) (with the lo parts of a compensated state through the
// cofactors), rho_true = sqrt(det(rho A / alpha) / rho0), 1/(alpha rho_true),
// alpha rho e = alpha rho E - |alpha rho u|^2 / (2 alpha rho_true), and
// s - 1 = rho_true/rho0 - 1. The states a face evaluates between its cells
// (midpoint, Gauss nodes, Q_hll) are FP32 interpolants and go through a plain FP32
// cons2prim. Everything else -- the Finger tensor, stress,
// temperature, the non-conservative columns of B (HyperelasticityMPh.jl:178-250),
// wave speeds, fluxes and the path-conservative HLL / LxF faces
// (NumFluxes.jl:25-132) -- is FP32, statement for statement as in the FP64 forms,
// with the hardware's approximate reciprocal and square root (about one ulp) where
// the FP64 forms divide or take a root.
#pragma once
#include "hyp_pair.cuh"
#include "hyp_physics_mixed.cuh"
#include "hyp_physics_mph.cuh"

namespace hyp {

struct Eos2M {
  EosMixed m[2];
};

struct Quad6F {
  float x[6], w[6];
};

// One phase of a two-phase cell in FP32.
struct PrimM2 {
  float den, true_den;  // alpha rho_true, rho_true
  float u[3], E, e_int;
  float A[9];
  float xm1;
  float sm1, rho_s;     // rho_true/rho0 - 1, rho0 s
  KinT<float> k;
  PowsT<float> w;
};

// q: [alpha, alpha rho (unused), alpha rho u(3), alpha rho E, alpha rho A(9)]; ql: the lo
// parts (or nullptr). Returns HYP_CELL_* status.
template <int kDef = -1>
__device__ __forceinline__ int cons_to_prim_m2(const EosMixed& em, const float* q, const float* ql, PrimM2& P) {
  const EosT<float>& e = em.f;
  const float* m = q + 6;
  // det(alpha rho A) in float-float, lo parts through the cofactors
  ff C00 = ff_diff_prod(m[4], m[8], m[7], m[5]);
  ff C01 = ff_neg(ff_diff_prod(m[1], m[8], m[7], m[2]));
  ff C02 = ff_diff_prod(m[1], m[5], m[4], m[2]);
  ff d = ff_add(ff_add(ff_mul_f(C00, m[0]), ff_mul_f(C01, m[3])), ff_mul_f(C02, m[6]));
  if (ql) {
    const float* l = ql + 6;
    float dlo = C00.hi * l[0] + C01.hi * l[3] + C02.hi * l[6];
    dlo += -(m[3] * m[8] - m[6] * m[5]) * l[1] + (m[0] * m[8] - m[6] * m[2]) * l[4] -
           (m[0] * m[5] - m[3] * m[2]) * l[7];
    dlo += (m[3] * m[7] - m[6] * m[4]) * l[2] - (m[0] * m[7] - m[6] * m[1]) * l[5] +
           (m[0] * m[4] - m[3] * m[1]) * l[8];
    d = ff_add_f(d, dlo);
  }
  int st = d.hi > 0.0f ? HYP_CELL_OK : HYP_CELL_NEG_DET;
  const ff alpha{q[0], ql ? ql[0] : 0.0f};
  const ff ia = ff_recip(alpha);
  // det(rho A / alpha) = det(alpha rho A) / alpha^3
  const ff dq = ff_mul(ff_mul(ff_mul(d, ia), ia), ia);
  const ff rho = ff_sqrt(ff_mul(dq, em.inv_rho0));  // rho_true
  const ff den = ff_mul(alpha, rho);
  const ff inv_den = ff_recip(den);
  ff m0{q[2], ql ? ql[2] : 0.0f}, m1{q[3], ql ? ql[3] : 0.0f}, m2{q[4], ql ? ql[4] : 0.0f};
  const ff k2 = ff_add(ff_add(ff_mul(m0, m0), ff_mul(m1, m1)), ff_mul(m2, m2));
  const ff rhoe = ff_sub(ff{q[5], ql ? ql[5] : 0.0f}, ff_mul(k2, ff_mul_f(inv_den, 0.5f)));
  P.e_int = ff_val(ff_mul(rhoe, inv_den));
  const ff s = ff_mul(rho, em.inv_rho0);  // 1/det A
  P.sm1 = ff_val(ff_add_f(s, -1.0f));
  P.true_den = ff_val(rho);
  P.den = ff_val(den);
  const float idn = ff_val(inv_den);
  for (int c = 0; c < 3; ++c) P.u[c] = q[2 + c] * idn;
  P.E = q[5] * idn;
  for (int c = 0; c < 9; ++c) P.A[c] = m[c] * idn;
  const float sf = 1.0f + P.sm1;
  P.k = kinematics_s<float>(P.A, sf, __frcp_rn(sf));
  P.w = powers<float, kDef>(e, P.k);
  P.w.Pam1 = default_exponents<kDef>(e) ? P.sm1 : expm1f(e.alpha * log1pf(P.sm1));
  P.xm1 = entropy_xm1<float>(e, P.e_int, P.k, P.w);
  P.rho_s = e.rho0 * sf;
  if (!(P.e_int == P.e_int) || !(P.xm1 == P.xm1) || !isfinite(P.k.p)) st |= HYP_CELL_NONFINITE;
  return st;
}

// Flux of one phase after alpha (HyperelasticityMPh.jl:146-175), 14 components.
__device__ __forceinline__ void phase_flux_m2(const EosT<float>& e, float alpha, const PrimM2& P,
                                              const StressCT<float>& c, float* f) {
  float s0[3];
  stress_row0<float>(P.rho_s, P.k, c, s0);
  s0[0] *= alpha;
  s0[1] *= alpha;
  s0[2] *= alpha;
  const float du = P.den * P.u[0];
  f[0] = du;
  f[1] = du * P.u[0] - s0[0];
  f[2] = du * P.u[1] - s0[1];
  f[3] = du * P.u[2] - s0[2];
  f[4] = du * P.E - (P.u[0] * s0[0] + P.u[1] * s0[1] + P.u[2] * s0[2]);
  for (int b = 0; b < 3; ++b)
    for (int a = 0; a < 3; ++a) f[5 + a + 3 * b] = P.den * (P.u[0] * P.A[a + 3 * b] - P.u[a] * P.A[3 * b]);
}

__device__ __forceinline__ float phase_cmax_m2(const EosT<float>& e, const PrimM2& P, const StressCT<float>& c) {
  float s0[3], s0r[3], om[9];
  stress_row0<float>(P.rho_s, P.k, c, s0);
  const float irs = rcp_approx(P.rho_s);
  for (int i = 0; i < 3; ++i) s0r[i] = s0[i] * irs;
  acoustic_omega<float>(e, P.k, P.w, c, P.xm1, s0r, om);
  return sqrt_approx(spectral_radius_fast(om));
}

// Both phases' flux (30) and wave-speed bounds of a cell from its compensated state.
template <int kDef = -1>
__device__ __forceinline__ int cell2_mixed(const Eos2M& E, const float* qh, const float* ql, float* F, float& smin,
                                           float& smax) {
  int st = 0;
#pragma unroll  // static indices keep the 90-float arrays in registers, not local memory
  for (int p = 0; p < 2; ++p) {
    const float* q = qh + 15 * p;
    PrimM2 P;
    st |= cons_to_prim_m2<kDef>(E.m[p], q, ql + 15 * p, P);
    const StressCT<float> c = stress_coeffs<float>(E.m[p].f, P.k, P.w, P.xm1);
    F[15 * p] = 0.0f;
    phase_flux_m2(E.m[p].f, q[0], P, c, F + 15 * p + 1);
    const float cm = phase_cmax_m2(E.m[p].f, P, c);
    const float lo = P.u[0] - cm, hi = P.u[0] + cm;
    if (p == 0 || lo < smin) smin = lo;
    if (p == 0 || hi > smax) smax = hi;
  }
  return st;
}

// cons2prim of one phase in plain FP32, for the states a face evaluates between
// its two cells (midpoint, path nodes, Q_hll): these are FP32 interpolants, whose
// own rounding the float-float islands could not undo.
template <int kDef = -1>
__device__ __forceinline__ int cons_to_prim_f2(const EosMixed& em, const float* q, PrimM2& P) {
  const EosT<float>& e = em.f;
  const float* m = q + 6;
  const float ia = rcp_approx(q[0]);
  const float d = det3(m) * (ia * ia * ia);  // det(alpha rho A / alpha)
  int st = d > 0.0f ? HYP_CELL_OK : HYP_CELL_NEG_DET;
  const float rho = sqrt_approx(d * e.inv_rho0);
  P.true_den = rho;
  P.den = q[0] * rho;
  const float idn = rcp_approx(P.den);
  for (int c = 0; c < 3; ++c) P.u[c] = q[2 + c] * idn;
  P.E = q[5] * idn;
  P.e_int = P.E - 0.5f * (P.u[0] * P.u[0] + P.u[1] * P.u[1] + P.u[2] * P.u[2]);
  for (int c = 0; c < 9; ++c) P.A[c] = m[c] * idn;
  const float sf = rho * e.inv_rho0;
  P.sm1 = sf - 1.0f;
  P.k = kinematics_s<float>(P.A, sf, rcp_approx(sf));
  P.w = powers<float, kDef>(e, P.k);
  P.w.Pam1 = default_exponents<kDef>(e) ? P.sm1 : expm1f(e.alpha * log1pf(P.sm1));
  P.xm1 = entropy_xm1<float>(e, P.e_int, P.k, P.w);
  P.rho_s = e.rho0 * sf;
  if (!(P.e_int == P.e_int) || !(P.xm1 == P.xm1) || !isfinite(P.k.p)) st |= HYP_CELL_NONFINITE;
  return st;
}

template <int kDef = -1>
__device__ __forceinline__ int speeds2_m(const Eos2M& E, const float* Q, float& smin, float& smax) {
  int st = 0;
  // phase loop kept rolled: unrolled, the face kernels' code grows and the HLL step
  // measured 3.08 against 2.72 ms at 2^22 cells (the local copy of the EOS pair it
  // avoids costs less)
  for (int p = 0; p < 2; ++p) {
    PrimM2 P;
    st |= cons_to_prim_f2<kDef>(E.m[p], Q + 15 * p, P);
    const StressCT<float> c = stress_coeffs<float>(E.m[p].f, P.k, P.w, P.xm1);
    const float cm = phase_cmax_m2(E.m[p].f, P, c);
    const float lo = P.u[0] - cm, hi = P.u[0] + cm;
    if (p == 0 || lo < smin) smin = lo;
    if (p == 0 || hi > smax) smax = hi;
  }
  return st;
}

// What B needs from one phase (as phase_b).
struct PhaseBM {
  float true_den, u[3], A[9], K0[3], T;
};

template <int kDef = -1>
__device__ __forceinline__ int phase_b_m(const EosMixed& em, const float* q, PhaseBM& b) {
  PrimM2 P;
  const int st = cons_to_prim_f2<kDef>(em, q, P);
  const StressCT<float> c = stress_coeffs<float>(em.f, P.k, P.w, P.xm1);
  stress_row0<float>(P.rho_s, P.k, c, b.K0);
  b.T = em.f.t0 * P.w.Pg * (P.xm1 + 1.0f);
  b.true_den = P.true_den;
  for (int a = 0; a < 3; ++a) b.u[a] = P.u[a];
  for (int k = 0; k < 9; ++k) b.A[k] = P.A[k];
  return st;
}

// bcol of B(Q) (noncons_bcol in FP32).
template <int kDef = -1>
__device__ __forceinline__ int noncons_bcol_m(const Eos2M& E, const float* Q, float* bcol) {
  PhaseBM b[2];
  const int st = phase_b_m<kDef>(E.m[0], Q, b[0]) | phase_b_m<kDef>(E.m[1], Q + 15, b[1]);
  float uI[3], sI[3];
  for (int a = 0; a < 3; ++a) uI[a] = 0.5f * b[0].u[a] + 0.5f * b[1].u[a];
  const float iden = rcp_approx(0.5f * b[0].T + 0.5f * b[1].T);
  for (int a = 0; a < 3; ++a) sI[a] = ((0.5f * b[1].T) * b[0].K0[a] + (0.5f * b[0].T) * b[1].K0[a]) * iden;
  for (int p = 0; p < 2; ++p) {
    float* r = bcol + 15 * p;
    const PhaseBM& B = b[p];
    r[0] = uI[0];
    r[1] = 0.0f;
    r[2] = sI[0];
    r[3] = sI[1];
    r[4] = sI[2];
    r[5] = (sI[0] * uI[0] + sI[1] * uI[1]) + sI[2] * uI[2];
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) r[6 + a + 3 * c] = (B.true_den * B.A[3 * c]) * B.u[a];
    const float dv[3] = {uI[0] - B.u[0], uI[1] - B.u[1], uI[2] - B.u[2]};
    for (int c = 0; c < 3; ++c)
      r[6 + 3 * c] += B.true_den * ((B.A[3 * c] * dv[0] + B.A[1 + 3 * c] * dv[1]) + B.A[2 + 3 * c] * dv[2]);
  }
  return st;
}

template <int kDef = -1>
__device__ __forceinline__ int path_integral_add_m(const Eos2M& E, const Quad6F& qd, const float* Qa, const float* Qb,
                                                   float* acc) {
  const float da0 = Qb[0] - Qa[0], da1 = Qb[15] - Qa[15];
  int st = 0;
  float u[30], bc[30];
  for (int i = 0; i < 6; ++i) {
    const float s = qd.x[i];
    for (int k = 0; k < 30; ++k) u[k] = fmaf(s, Qb[k] - Qa[k], Qa[k]);  // Qa + s (Qb - Qa)
    st |= noncons_bcol_m<kDef>(E, u, bc);
    const float wd0 = qd.w[i] * da0, wd1 = qd.w[i] * da1;
    for (int k = 0; k < 30; ++k)
      if (k != 1 && k != 16) acc[k] = fmaf(bc[k], k < 15 ? wd0 : wd1, acc[k]);  // rows 1 and 16 of B are 0
  }
  return st;
}

// Path-conservative HLL fluctuations of one face (hll_face2 in FP32).
template <int kDef = -1>
__device__ __forceinline__ int hll_face2_m(const Eos2M& E, const Quad6F& qd, const float* QL, const float* QR,
                                           const float* dF, float sminL, float smaxR, float* dm, float* dp) {
  float Qm[30];
  for (int k = 0; k < 30; ++k) Qm[k] = 0.5f * (QL[k] + QR[k]);
  float mmin = 0.0f, mmax = 0.0f;
  int st = speeds2_m<kDef>(E, Qm, mmin, mmax);
  float sl = 0.0f;
  if (mmin < sl) sl = mmin;
  if (sminL < sl) sl = sminL;
  float sr = 0.0f;
  if (mmax > sr) sr = mmax;
  if (smaxR > sr) sr = smaxR;
  const float idsr = 1.0f / (sr - sl);
  float acc[30], Qh[30];
  for (int k = 0; k < 30; ++k) acc[k] = 0.0f;
  st |= path_integral_add_m<kDef>(E, qd, QL, QR, acc);
  for (int k = 0; k < 30; ++k) {
    Qh[k] = ((QR[k] * sr - QL[k] * sl) - (acc[k] + dF[k])) * idsr;
    acc[k] = 0.0f;
  }
  // B_int(Q_l, Q_hll) + B_int(Q_hll, Q_r) in one accumulator
  st |= path_integral_add_m<kDef>(E, qd, QL, Qh, acc);
  st |= path_integral_add_m<kDef>(E, qd, Qh, QR, acc);
  const float cm = (-sl) * idsr, cp = sr * idsr, cq = (sl * sr) * idsr;
  for (int k = 0; k < 30; ++k) {
    const float inner = dF[k] + acc[k];
    const float jump = QR[k] - QL[k];
    dm[k] = cm * inner + cq * jump;
    dp[k] = cp * inner - cq * jump;
  }
  return st;
}

// Path-conservative LxF face (lxf_face2 in FP32).
template <int kDef = -1>
__device__ __forceinline__ int lxf_face2_m(const Eos2M& E, const Quad6F& lobatto, const float* QL, const float* QR,
                                           const float* fl, const float* fr, float lambda, float* F, float* dm,
                                           float* dp) {
  const float hl = lambda * 0.5f;
  for (int k = 0; k < 30; ++k) F[k] = 0.5f * (fl[k] + fr[k]) - hl * (QR[k] - QL[k]);
  float acc[30];
  for (int k = 0; k < 30; ++k) acc[k] = 0.0f;
  const int st = path_integral_add_m<kDef>(E, lobatto, QL, QR, acc);
  for (int k = 0; k < 30; ++k) dm[k] = dp[k] = 0.5f * acc[k];
  return st;
}

}  // namespace hyp
