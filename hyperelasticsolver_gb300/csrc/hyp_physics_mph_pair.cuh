// hyp_physics_mph_pair.cuh -- the two-phase face physics of hyp_physics_mph_mixed.cuh
// with the two phases as the two lanes of packed FP32 pairs (hyp_pair.cuh).
//
// Both phases of a two-phase state run the same chain -- cons2prim, the Finger tensor,
// the stress row, the temperature -- with their own EOS constants
// (HyperelasticityMPh.jl:178-250 evaluates B per phase). Held as float2 values whose
// .x is phase 1 and .y phase 2 (a 30-value state is 15 pairs: pair k = (Q[k], Q[15+k])),
// each step of the chain is one packed instruction for both phases instead of two,
// and the path integrals accumulate both phases' rows the same way. What mixes the
// phases -- the interface velocity u_I and stress sigma_I of B (:213-217), the speed
// bounds -- is scalar. The arithmetic is the FP32 of the scalar forms, with the
// multiply-adds written out as fused pairs (so results differ from the scalar forms
// in the last bits, as two FP32 evaluations of different contraction do).
#pragma once
#include "hyp_pair.cuh"
#include "hyp_physics_mph_mixed.cuh"

namespace hyp {

// The EOS constants the face chain reads, lane p = phase p.
struct EosPair {
  float2 rho0, inv_rho0, t0, inv_cvt0;
  float2 alpha, beta, gamma;
  float2 b0sq, b0sq_6, kU, kE3a, kE3b, kE3g;
  int default_exp;  // both phases have the reference's default exponents
};
inline EosPair make_eos_pair(const Eos2M& E) {
  const EosT<float>&a = E.m[0].f, &b = E.m[1].f;
  EosPair p;
  p.rho0 = make_float2(a.rho0, b.rho0);
  p.inv_rho0 = make_float2(a.inv_rho0, b.inv_rho0);
  p.t0 = make_float2(a.t0, b.t0);
  p.inv_cvt0 = make_float2(a.inv_cvt0, b.inv_cvt0);
  p.alpha = make_float2(a.alpha, b.alpha);
  p.beta = make_float2(a.beta, b.beta);
  p.gamma = make_float2(a.gamma, b.gamma);
  p.b0sq = make_float2(a.b0sq, b.b0sq);
  p.b0sq_6 = make_float2(a.b0sq_6, b.b0sq_6);
  p.kU = make_float2(a.kU, b.kU);
  p.kE3a = make_float2(a.kE3a, b.kE3a);
  p.kE3b = make_float2(a.kE3b, b.kE3b);
  p.kE3g = make_float2(a.kE3g, b.kE3g);
  p.default_exp = a.default_exp && b.default_exp;
  return p;
}

// p^(n/2) factors for the three exponents; the reference's default exponents
// (kDef = 1) are products of s = sqrt(p).
struct PowPair {
  float2 Pa1, Pb, Pb1, Pg, Pg1, inv_Pg;
};

// What B needs from both phases (phase_b_m, paired): rho_true, u, A, row 1 of sigma
// and the temperature T = dE/dS (HyperelasticityMPh.jl:212).
struct PhaseBPair {
  float2 true_den, u[3], A[9], K0[3], T;
};

// q: the 15 pairs of a two-phase state (an FP32 interpolant). Returns HYP_CELL_* bits.
template <int kDef = -1>
__device__ __forceinline__ int phase_b_pair(const EosPair& e, const float2* q, PhaseBPair& b) {
  const float2* m = q + 6;
  const float2 ia = f2rcp_approx(q[0]);
  // det3 (cofactor expansion, SimpleLA.jl:84-89) / alpha^3
  const float2 c0 = f2fma(m[4], m[8], f2neg(f2mul(m[5], m[7])));
  const float2 c1 = f2fma(m[1], m[8], f2neg(f2mul(m[7], m[2])));
  const float2 c2 = f2fma(m[1], m[5], f2neg(f2mul(m[4], m[2])));
  const float2 det = f2fma(m[6], c2, f2fma(f2neg(m[3]), c1, f2mul(m[0], c0)));
  const float2 d = f2mul(det, f2mul(f2mul(ia, ia), ia));
  int st = (d.x > 0.0f && d.y > 0.0f) ? HYP_CELL_OK : HYP_CELL_NEG_DET;
  const float2 rho = f2sqrt_approx(f2mul(d, e.inv_rho0));
  const float2 den = f2mul(q[0], rho);
  const float2 idn = f2rcp_approx(den);
  float2 u[3];
  for (int c = 0; c < 3; ++c) u[c] = f2mul(q[2 + c], idn);
  const float2 E = f2mul(q[5], idn);
  const float2 uu = f2fma(u[2], u[2], f2fma(u[1], u[1], f2mul(u[0], u[0])));
  const float2 e_int = f2fma(f2s(-0.5f), uu, E);
  float2 A[9];
  for (int c = 0; c < 9; ++c) A[c] = f2mul(m[c], idn);
  const float2 sf = f2mul(rho, e.inv_rho0);  // 1/det A
  const float2 sm1 = f2add(sf, f2s(-1.0f));
  const float2 isf = f2rcp_approx(sf);
  // Finger tensor G = adj(A A^T) p, p = s^2 (Strains.jl:26-32), and row 1 of H = G^2
  const float2 m00 = f2fma(A[6], A[6], f2fma(A[3], A[3], f2mul(A[0], A[0])));
  const float2 m11 = f2fma(A[7], A[7], f2fma(A[4], A[4], f2mul(A[1], A[1])));
  const float2 m22 = f2fma(A[8], A[8], f2fma(A[5], A[5], f2mul(A[2], A[2])));
  const float2 m01 = f2fma(A[6], A[7], f2fma(A[3], A[4], f2mul(A[0], A[1])));
  const float2 m02 = f2fma(A[6], A[8], f2fma(A[3], A[5], f2mul(A[0], A[2])));
  const float2 m12 = f2fma(A[7], A[8], f2fma(A[4], A[5], f2mul(A[1], A[2])));
  const float2 p = f2mul(sf, sf);
  const float2 g00 = f2mul(f2fma(m11, m22, f2neg(f2mul(m12, m12))), p);
  const float2 g11 = f2mul(f2fma(m00, m22, f2neg(f2mul(m02, m02))), p);
  const float2 g22 = f2mul(f2fma(m00, m11, f2neg(f2mul(m01, m01))), p);
  const float2 g01 = f2mul(f2fma(m02, m12, f2neg(f2mul(m01, m22))), p);
  const float2 g02 = f2mul(f2fma(m01, m12, f2neg(f2mul(m02, m11))), p);
  const float2 g12 = f2mul(f2fma(m01, m02, f2neg(f2mul(m00, m12))), p);
  const float2 h00 = f2fma(g02, g02, f2fma(g01, g01, f2mul(g00, g00)));
  const float2 h01 = f2fma(g02, g12, f2fma(g01, g11, f2mul(g00, g01)));
  const float2 h02 = f2fma(g02, g22, f2fma(g01, g12, f2mul(g00, g02)));
  const float2 i1 = f2add(f2add(g00, g11), g22);
  // psi = i1^2/3 - i2 = |dev G|^2 / 2, without the cancellation near G = I
  const float2 d01 = f2sub(g00, g11), d12 = f2sub(g11, g22), d20 = f2sub(g22, g00);
  const float2 dd = f2fma(d20, d20, f2fma(d12, d12, f2mul(d01, d01)));
  const float2 oo = f2fma(g12, g12, f2fma(g02, g02, f2mul(g01, g01)));
  const float2 psi = f2fma(dd, f2s(1.0f / 6.0f), oo);
  // powers of p (EquationsOfState.jl:118-137)
  PowPair w;
  float2 Pam1;
  if (default_exponents<kDef>(e)) {  // alpha 1, beta 3, gamma 2: p^(n/2) = s^n
    const float2 ip = f2mul(isf, isf);
    w.Pa1 = isf;
    w.Pb = f2mul(sf, p);
    w.Pb1 = sf;
    w.Pg = p;
    w.Pg1 = f2s(1.0f);
    w.inv_Pg = ip;
    Pam1 = sm1;
  } else {
    const float2 ip = f2rcp(p);
    const float2 lp = make_float2(logf(p.x), logf(p.y));
    const float2 ha = f2mul(f2s(0.5f), e.alpha), hb = f2mul(f2s(0.5f), e.beta), hg = f2mul(f2s(0.5f), e.gamma);
    const float2 Pa = make_float2(expf(ha.x * lp.x), expf(ha.y * lp.y));
    w.Pa1 = f2mul(Pa, ip);
    w.Pb = make_float2(expf(hb.x * lp.x), expf(hb.y * lp.y));
    w.Pb1 = f2mul(w.Pb, ip);
    w.Pg = make_float2(expf(hg.x * lp.x), expf(hg.y * lp.y));
    w.Pg1 = f2mul(w.Pg, ip);
    w.inv_Pg = f2rcp(w.Pg);
    Pam1 = make_float2(expm1f(e.alpha.x * log1pf(sm1.x)), expm1f(e.alpha.y * log1pf(sm1.y)));
  }
  // entropy argument minus one, clamped at 1e-6 (EquationsOfState.jl:150-154)
  const float2 w_sh = f2mul(f2mul(f2mul(f2s(0.5f), e.b0sq), w.Pb), psi);
  const float2 u_c = f2mul(f2mul(e.kU, Pam1), Pam1);
  float2 xm1 = f2mul(f2mul(f2sub(f2sub(e_int, w_sh), u_c), e.inv_cvt0), w.inv_Pg);
  if (xm1.x + 1.0f < 1e-6f) xm1.x = 1e-6f - 1.0f;
  if (xm1.y + 1.0f < 1e-6f) xm1.y = 1e-6f - 1.0f;
  // stress coefficients: G dE/dG = cG G + cGG G^2 + cI I
  const float2 cG = f2mul(f2mul(f2neg(e.b0sq_6), w.Pb), i1);  // E1 + E2 i1 = -b0sq Pb i1 / 6
  const float2 cGG = f2mul(f2mul(f2s(0.5f), e.b0sq), w.Pb);   // -E2
  const float2 E3 = f2fma(f2mul(e.kE3b, w.Pb1), psi, f2fma(f2mul(e.kE3g, w.Pg1), xm1, f2mul(f2mul(e.kE3a, Pam1), w.Pa1)));
  const float2 cI = f2mul(E3, p);
  // row 1 of sigma = -2 rho_s (cG G + cGG G^2 + cI I)
  const float2 m2r = f2mul(f2s(-2.0f), f2mul(e.rho0, sf));
  b.K0[0] = f2mul(m2r, f2fma(cG, g00, f2fma(cGG, h00, cI)));
  b.K0[1] = f2mul(m2r, f2fma(cG, g01, f2mul(cGG, h01)));
  b.K0[2] = f2mul(m2r, f2fma(cG, g02, f2mul(cGG, h02)));
  b.T = f2mul(f2mul(e.t0, w.Pg), f2add(xm1, f2s(1.0f)));
  b.true_den = rho;
  for (int a = 0; a < 3; ++a) b.u[a] = u[a];
  for (int k = 0; k < 9; ++k) b.A[k] = A[k];
  const bool bad = !(e_int.x == e_int.x) || !(e_int.y == e_int.y) || !(xm1.x == xm1.x) || !(xm1.y == xm1.y) ||
                   !isfinite(p.x) || !isfinite(p.y);
  if (bad) st |= HYP_CELL_NONFINITE;
  return st;
}

// The non-zero columns of B(Q) (noncons_bcol_m) as 15 pairs: pair k = (B[k, 1], B[15 + k, 16]).
template <int kDef = -1>
__device__ __forceinline__ int noncons_bcol_pair(const EosPair& e, const float2* Q, float2* bc) {
  PhaseBPair b;
  const int st = phase_b_pair<kDef>(e, Q, b);
  // interface velocity and stress (HyperelasticityMPh.jl:213-217, k = (1/2, 1/2))
  float uI[3], sI[3];
  for (int a = 0; a < 3; ++a) uI[a] = 0.5f * b.u[a].x + 0.5f * b.u[a].y;
  const float iden = rcp_approx(0.5f * b.T.x + 0.5f * b.T.y);
  for (int a = 0; a < 3; ++a) sI[a] = ((0.5f * b.T.y) * b.K0[a].x + (0.5f * b.T.x) * b.K0[a].y) * iden;
  bc[0] = f2s(uI[0]);
  bc[1] = f2s(0.0f);
  bc[2] = f2s(sI[0]);
  bc[3] = f2s(sI[1]);
  bc[4] = f2s(sI[2]);
  bc[5] = f2s((sI[0] * uI[0] + sI[1] * uI[1]) + sI[2] * uI[2]);
  const float2 dv[3] = {f2sub(f2s(uI[0]), b.u[0]), f2sub(f2s(uI[1]), b.u[1]), f2sub(f2s(uI[2]), b.u[2])};
  for (int c = 0; c < 3; ++c) {
    const float2 ra = f2mul(b.true_den, b.A[3 * c]);
    for (int a = 0; a < 3; ++a) bc[6 + a + 3 * c] = f2mul(ra, b.u[a]);
    const float2 t = f2fma(b.A[2 + 3 * c], dv[2], f2fma(b.A[1 + 3 * c], dv[1], f2mul(b.A[3 * c], dv[0])));
    bc[6 + 3 * c] = f2fma(b.true_den, t, bc[6 + 3 * c]);
  }
  return st;
}

// acc += sum_i (w_i B_i) (Qb - Qa)[alpha] along psi(s) = Qa + s (Qb - Qa)
// (NumFluxes.jl:97-107); pair k of acc holds rows k and 15 + k.
template <int kDef = -1>
__device__ __forceinline__ int path_integral_add_pair(const EosPair& e, const Quad6F& qd, const float2* Qa,
                                                      const float2* Qb, float2* acc) {
  float2 dq[15];
  for (int k = 0; k < 15; ++k) dq[k] = f2sub(Qb[k], Qa[k]);
  const float2 da = dq[0];  // (d alpha_1, d alpha_2)
  int st = 0;
  float2 u[15], bc[15];
  for (int i = 0; i < 6; ++i) {
    const float2 s = f2s(qd.x[i]);
    for (int k = 0; k < 15; ++k) u[k] = f2fma(s, dq[k], Qa[k]);
    st |= noncons_bcol_pair<kDef>(e, u, bc);
    const float2 wd = f2mul(f2s(qd.w[i]), da);
    for (int k = 0; k < 15; ++k)
      if (k != 1) acc[k] = f2fma(bc[k], wd, acc[k]);  // rows 1 and 16 of B are 0
  }
  return st;
}

// Path-conservative HLL fluctuations of one face (hll_face2_m with paired phases).
// QL, QR, dF (f(Q_r) - f(Q_l)), dm, dp: 15 pairs each.
template <int kDef = -1>
__device__ __forceinline__ int hll_face2_pair(const Eos2M& E, const EosPair& e, const Quad6F& qd, const float2* QL,
                                              const float2* QR, const float2* dF, float sminL, float smaxR,
                                              float2* dm, float2* dp) {
  float Qm[30];
  for (int k = 0; k < 15; ++k) {
    const float2 m = f2mul(f2s(0.5f), f2add(QL[k], QR[k]));
    Qm[k] = m.x;
    Qm[15 + k] = m.y;
  }
  float mmin = 0.0f, mmax = 0.0f;
  int st = speeds2_m<kDef>(E, Qm, mmin, mmax);
  float sl = 0.0f;
  if (mmin < sl) sl = mmin;
  if (sminL < sl) sl = sminL;
  float sr = 0.0f;
  if (mmax > sr) sr = mmax;
  if (smaxR > sr) sr = smaxR;
  const float idsr = 1.0f / (sr - sl);
  float2 acc[15], Qh[15];
  for (int k = 0; k < 15; ++k) acc[k] = f2s(0.0f);
  st |= path_integral_add_pair<kDef>(e, qd, QL, QR, acc);
  const float2 s_r = f2s(sr), s_l = f2s(sl), id = f2s(idsr);
  for (int k = 0; k < 15; ++k) {
    Qh[k] = f2mul(f2sub(f2fma(QR[k], s_r, f2neg(f2mul(QL[k], s_l))), f2add(acc[k], dF[k])), id);
    acc[k] = dF[k];  // the two integrals through Q_hll add onto f_R - f_L: dF is not live across them
  }
  st |= path_integral_add_pair<kDef>(e, qd, QL, Qh, acc);
  st |= path_integral_add_pair<kDef>(e, qd, Qh, QR, acc);
  const float2 cm = f2s((-sl) * idsr), cp = f2s(sr * idsr), cq = f2s((sl * sr) * idsr);
  for (int k = 0; k < 15; ++k) {
    const float2 inner = acc[k];
    const float2 jump = f2sub(QR[k], QL[k]);
    dm[k] = f2fma(cm, inner, f2mul(cq, jump));
    dp[k] = f2fma(cp, inner, f2neg(f2mul(cq, jump)));
  }
  return st;
}

// Path-conservative LxF face (lxf_face2_m with paired phases).
template <int kDef = -1>
__device__ __forceinline__ int lxf_face2_pair(const EosPair& e, const Quad6F& lobatto, const float2* QL,
                                              const float2* QR, const float2* fl, const float2* fr, float lambda,
                                              float2* F, float2* dm, float2* dp) {
  const float2 hl = f2s(lambda * 0.5f), half = f2s(0.5f);
  for (int k = 0; k < 15; ++k) F[k] = f2fma(f2neg(hl), f2sub(QR[k], QL[k]), f2mul(half, f2add(fl[k], fr[k])));
  float2 acc[15];
  for (int k = 0; k < 15; ++k) acc[k] = f2s(0.0f);
  const int st = path_integral_add_pair<kDef>(e, lobatto, QL, QR, acc);
  for (int k = 0; k < 15; ++k) dm[k] = dp[k] = f2mul(half, acc[k]);
  return st;
}

}  // namespace hyp
