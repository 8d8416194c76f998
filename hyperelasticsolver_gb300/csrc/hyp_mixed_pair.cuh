// hyp_mixed_pair.cuh -- the single-phase mixed-precision cell physics of
// hyp_physics_mixed.cuh for two cells at once, as the lanes of packed FP32 pairs
// (hyp_pair.cuh): lane x is one cell, lane y another, with the same EOS.
//
// Each statement of the scalar chain -- the float-float islands of cons2prim, the
// Finger tensor and its invariants, the energy's powers and entropy argument, the
// stress coefficients, the x-flux, the acoustic tensor along e1 and its spectral
// radius -- becomes one packed instruction for both cells. What has no packed form
// runs per lane: reciprocals, square roots, transcendental powers, and the branchy
// closed-form seed and deflation of the spectral radius. Multiply-adds are written
// as fused pairs, so results differ from the scalar forms (whose contraction the
// compiler chooses) in the last bits of FP32.
//
// Status words carry lane x's HYP_CELL_* bits in bits 0-7 and lane y's in 8-15.
#pragma once
#include "hyp_pair.cuh"
#include "hyp_physics_mixed.cuh"

namespace hyp {

__device__ __forceinline__ int lane_status(bool bad_x, bool bad_y, int code) {
  return (bad_x ? code : 0) | (bad_y ? code << 8 : 0);
}

struct IslandsP {
  float2 ir, e_int, sm1;  // 1 / rho_true, specific internal energy, rho_true / rho0 - 1
};

// G = (A A^T)^-1, H = G^2 as (00, 11, 22, 01, 02, 12), invariants (kinematics_s).
struct KinP {
  float2 g[6], h[6];
  float2 i1, p, s, inv_s, psi;
};
__device__ __forceinline__ constexpr int sym_idx(int i, int j) {
  return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5));
}

struct PowP {
  float2 Pa1, Pa2, Pb, Pb1, Pb2, Pg, Pg1, Pg2, inv_Pg, Pam1;
};

struct PrimP {
  float2 rho_u1, u[3], E, e_int, A[9], xm1, rho_s, inv_rho_s;
  KinP k;
  PowP w;
};

struct CoefP {
  float2 cG, cGG, cI, E3;
};

// islands_mixed for two cells (float-float det(rho A) with the lo parts through the
// cofactors, rho_true, rho e = rho E - |rho u|^2 / (2 rho), s - 1).
__device__ __forceinline__ int islands_pair(const EosMixed& em, const float2* qh, const float2* ql, IslandsP& I) {
  const float2* m = qh + 5;
  const float2* l = ql + 5;
  const ff2 C00 = ff2_diff_prod(m[4], m[8], m[7], m[5]);
  const ff2 C01 = ff2_neg(ff2_diff_prod(m[1], m[8], m[7], m[2]));
  const ff2 C02 = ff2_diff_prod(m[1], m[5], m[4], m[2]);
  ff2 d = ff2_add(ff2_add(ff2_mul_f(C00, m[0]), ff2_mul_f(C01, m[3])), ff2_mul_f(C02, m[6]));
  // first-order contribution of the lo parts through the nine cofactors
  float2 dlo = f2fma(C02.hi, l[6], f2fma(C01.hi, l[3], f2mul(C00.hi, l[0])));
  const float2 c10 = f2fma(m[3], m[8], f2neg(f2mul(m[6], m[5])));
  const float2 c11 = f2fma(m[0], m[8], f2neg(f2mul(m[6], m[2])));
  const float2 c12 = f2fma(m[0], m[5], f2neg(f2mul(m[3], m[2])));
  const float2 c20 = f2fma(m[3], m[7], f2neg(f2mul(m[6], m[4])));
  const float2 c21 = f2fma(m[0], m[7], f2neg(f2mul(m[6], m[1])));
  const float2 c22 = f2fma(m[0], m[4], f2neg(f2mul(m[3], m[1])));
  dlo = f2add(dlo, f2fma(f2neg(c12), l[7], f2fma(c11, l[4], f2mul(f2neg(c10), l[1]))));
  dlo = f2add(dlo, f2fma(c22, l[8], f2fma(f2neg(c21), l[5], f2mul(c20, l[2]))));
  d = ff2_add_f(d, dlo);
  int st = lane_status(!(d.hi.x > 0.0f), !(d.hi.y > 0.0f), HYP_CELL_NEG_DET);
  const ff2 inv_rho0{f2s(em.inv_rho0.hi), f2s(em.inv_rho0.lo)};
  const ff2 rho = ff2_sqrt(ff2_mul(d, inv_rho0));
  const ff2 inv_rho = ff2_recip(rho);
  const ff2 m0{qh[1], ql[1]}, m1{qh[2], ql[2]}, m2{qh[3], ql[3]};
  const ff2 k2 = ff2_add(ff2_add(ff2_mul(m0, m0), ff2_mul(m1, m1)), ff2_mul(m2, m2));
  const ff2 ke = ff2_mul(k2, ff2_mul_f(inv_rho, f2s(0.5f)));
  const ff2 rhoe = ff2_sub(ff2{qh[4], ql[4]}, ke);
  I.e_int = ff2_val(ff2_mul(rhoe, inv_rho));
  const ff2 s = ff2_mul(rho, inv_rho0);
  I.sm1 = ff2_val(ff2_add_f(s, f2s(-1.0f)));
  I.ir = ff2_val(inv_rho);
  st |= lane_status(!(I.e_int.x == I.e_int.x) || !(I.sm1.x == I.sm1.x),
                    !(I.e_int.y == I.e_int.y) || !(I.sm1.y == I.sm1.y), HYP_CELL_NONFINITE);
  return st;
}

__device__ __forceinline__ void kinematics_pair(const float2* A, float2 s, float2 inv_s, KinP& k) {
  const float2 m00 = f2fma(A[6], A[6], f2fma(A[3], A[3], f2mul(A[0], A[0])));
  const float2 m11 = f2fma(A[7], A[7], f2fma(A[4], A[4], f2mul(A[1], A[1])));
  const float2 m22 = f2fma(A[8], A[8], f2fma(A[5], A[5], f2mul(A[2], A[2])));
  const float2 m01 = f2fma(A[6], A[7], f2fma(A[3], A[4], f2mul(A[0], A[1])));
  const float2 m02 = f2fma(A[6], A[8], f2fma(A[3], A[5], f2mul(A[0], A[2])));
  const float2 m12 = f2fma(A[7], A[8], f2fma(A[4], A[5], f2mul(A[1], A[2])));
  k.s = s;
  k.inv_s = inv_s;
  k.p = f2mul(s, s);
  float2* g = k.g;
  g[0] = f2mul(f2fma(m11, m22, f2neg(f2mul(m12, m12))), k.p);
  g[1] = f2mul(f2fma(m00, m22, f2neg(f2mul(m02, m02))), k.p);
  g[2] = f2mul(f2fma(m00, m11, f2neg(f2mul(m01, m01))), k.p);
  g[3] = f2mul(f2fma(m02, m12, f2neg(f2mul(m01, m22))), k.p);
  g[4] = f2mul(f2fma(m01, m12, f2neg(f2mul(m02, m11))), k.p);
  g[5] = f2mul(f2fma(m01, m02, f2neg(f2mul(m00, m12))), k.p);
  float2* h = k.h;
  h[0] = f2fma(g[4], g[4], f2fma(g[3], g[3], f2mul(g[0], g[0])));
  h[1] = f2fma(g[5], g[5], f2fma(g[1], g[1], f2mul(g[3], g[3])));
  h[2] = f2fma(g[2], g[2], f2fma(g[5], g[5], f2mul(g[4], g[4])));
  h[3] = f2fma(g[4], g[5], f2fma(g[3], g[1], f2mul(g[0], g[3])));
  h[4] = f2fma(g[4], g[2], f2fma(g[3], g[5], f2mul(g[0], g[4])));
  h[5] = f2fma(g[5], g[2], f2fma(g[1], g[5], f2mul(g[3], g[4])));
  k.i1 = f2add(f2add(g[0], g[1]), g[2]);
  // i1^2/3 - i2 = |dev G|^2 / 2 (no cancellation near G = I)
  const float2 d01 = f2sub(g[0], g[1]), d12 = f2sub(g[1], g[2]), d20 = f2sub(g[2], g[0]);
  const float2 dd = f2fma(d20, d20, f2fma(d12, d12, f2mul(d01, d01)));
  const float2 oo = f2fma(g[5], g[5], f2fma(g[4], g[4], f2mul(g[3], g[3])));
  k.psi = f2fma(dd, f2s(1.0f / 6.0f), oo);
}

__device__ __forceinline__ float2 f2pow_half(float2 lp, float ex) {  // p^(ex/2) from log p
  const float h = 0.5f * ex;
  return make_float2(expf(h * lp.x), expf(h * lp.y));
}

__device__ __forceinline__ void powers_pair(const EosT<float>& e, const KinP& k, float2 sm1, PowP& w) {
  if (e.default_exp) {  // alpha 1, beta 3, gamma 2: p^(n/2) = s^n
    const float2 is = k.inv_s, ip = f2mul(is, is);
    w.Pa1 = is;
    w.Pa2 = f2mul(is, ip);
    w.Pb = f2mul(k.s, k.p);
    w.Pb1 = k.s;
    w.Pb2 = is;
    w.Pg = k.p;
    w.Pg1 = f2s(1.0f);
    w.Pg2 = ip;
    w.inv_Pg = ip;
    w.Pam1 = sm1;
  } else {
    const float2 lp = make_float2(logf(k.p.x), logf(k.p.y)), ip = f2rcp(k.p);
    const float2 Pa = f2pow_half(lp, e.alpha);
    w.Pa1 = f2mul(Pa, ip);
    w.Pa2 = f2mul(w.Pa1, ip);
    w.Pb = f2pow_half(lp, e.beta);
    w.Pb1 = f2mul(w.Pb, ip);
    w.Pb2 = f2mul(w.Pb1, ip);
    w.Pg = f2pow_half(lp, e.gamma);
    w.Pg1 = f2mul(w.Pg, ip);
    w.Pg2 = f2mul(w.Pg1, ip);
    w.inv_Pg = f2rcp(w.Pg);
    w.Pam1 = make_float2(expm1f(e.alpha * log1pf(sm1.x)), expm1f(e.alpha * log1pf(sm1.y)));
  }
}

// prim_from_islands for two cells.
__device__ __forceinline__ int prim_from_islands_pair(const EosMixed& em, const float2* qh, const float2* ql,
                                                      const IslandsP& I, PrimP& P) {
  const EosT<float>& e = em.f;
  const float2 ir = I.ir, sf = f2add(f2s(1.0f), I.sm1);
  P.e_int = I.e_int;
  P.rho_u1 = f2add(qh[1], ql[1]);
  for (int c = 0; c < 3; ++c) P.u[c] = f2mul(qh[1 + c], ir);
  P.E = f2mul(qh[4], ir);
  for (int c = 0; c < 9; ++c) P.A[c] = f2mul(qh[5 + c], ir);
  kinematics_pair(P.A, sf, f2rcp_approx(sf), P.k);
  powers_pair(e, P.k, I.sm1, P.w);
  // entropy argument minus one, clamped at 1e-6 (EquationsOfState.jl:150-154)
  const float2 w_sh = f2mul(f2mul(f2s(0.5f * e.b0sq), P.w.Pb), P.k.psi);
  const float2 u_c = f2mul(f2mul(f2s(e.kU), P.w.Pam1), P.w.Pam1);
  float2 xm1 = f2mul(f2mul(f2sub(f2sub(P.e_int, w_sh), u_c), f2s(e.inv_cvt0)), P.w.inv_Pg);
  if (xm1.x + 1.0f < 1e-6f) xm1.x = 1e-6f - 1.0f;
  if (xm1.y + 1.0f < 1e-6f) xm1.y = 1e-6f - 1.0f;
  P.xm1 = xm1;
  P.rho_s = f2mul(f2s(e.rho0), sf);
  P.inv_rho_s = f2mul(P.k.inv_s, f2s(e.inv_rho0));
  return lane_status(!(xm1.x == xm1.x) || !isfinite(P.k.p.x), !(xm1.y == xm1.y) || !isfinite(P.k.p.y),
                     HYP_CELL_NONFINITE);
}

__device__ __forceinline__ CoefP stress_coeffs_pair(const EosT<float>& e, const PrimP& P) {
  CoefP c;
  const PowP& w = P.w;
  c.E3 = f2fma(f2mul(f2s(e.kE3b), w.Pb1), P.k.psi,
               f2fma(f2mul(f2s(e.kE3g), w.Pg1), P.xm1, f2mul(f2mul(f2s(e.kE3a), w.Pam1), w.Pa1)));
  c.cG = f2mul(f2mul(f2s(-e.b0sq_6), w.Pb), P.k.i1);  // E1 + E2 i1 = -b0sq Pb i1 / 6
  c.cGG = f2mul(f2s(0.5f * e.b0sq), w.Pb);            // -E2
  c.cI = f2mul(c.E3, P.k.p);
  return c;
}

// Row 1 of sigma = -2 rho_s (cG G + cGG G^2 + cI I).
__device__ __forceinline__ void stress_row0_pair(const PrimP& P, const CoefP& c, float2* s0) {
  const float2 m = f2mul(f2s(-2.0f), P.rho_s);
  s0[0] = f2mul(m, f2fma(c.cG, P.k.g[0], f2fma(c.cGG, P.k.h[0], c.cI)));
  s0[1] = f2mul(m, f2fma(c.cG, P.k.g[3], f2mul(c.cGG, P.k.h[3])));
  s0[2] = f2mul(m, f2fma(c.cG, P.k.g[4], f2mul(c.cGG, P.k.h[4])));
}

// flux_mixed for two cells: the 11 non-zero components in flux_slot1 order.
__device__ __forceinline__ void flux_pair(const float2* qh, const PrimP& P, const CoefP& c, float2* f11) {
  float2 s0[3];
  stress_row0_pair(P, c, s0);
  const float2 mu = P.rho_u1;
  f11[0] = mu;
  f11[1] = f2fma(mu, P.u[0], f2neg(s0[0]));
  f11[2] = f2fma(mu, P.u[1], f2neg(s0[1]));
  f11[3] = f2fma(mu, P.u[2], f2neg(s0[2]));
  f11[4] = f2fma(mu, P.E, f2neg(f2fma(P.u[2], s0[2], f2fma(P.u[1], s0[1], f2mul(P.u[0], s0[0])))));
  const float2* rA = qh + 5;
  for (int b = 0; b < 3; ++b)
    for (int a = 1; a < 3; ++a)
      f11[5 + 2 * b + (a - 1)] = f2fma(P.u[0], rA[a + 3 * b], f2neg(f2mul(P.u[a], rA[3 * b])));
}

// acoustic_omega (n = e1) for two cells, column-major om[i + 3 j].
__device__ __forceinline__ void acoustic_pair(const EosT<float>& e, const PrimP& P, const CoefP& c, const float2* s0r,
                                              float2* om) {
  const KinP& k = P.k;
  const PowP& w = P.w;
  const float2 bs6n = f2s(-e.b0sq_6), hb = f2s(0.5f * e.b0sq);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float2 G0j = k.g[sym_idx(0, j)], H0j = k.h[sym_idx(0, j)];
    const float2 di1 = f2mul(f2s(-2.0f), G0j);
    const float2 dpsi = f2fma(f2mul(f2s(2.0f / 3.0f), k.i1), G0j, f2mul(f2s(-2.0f), H0j));
    float2 dcG, dcGG, dcI;
    if (j == 0) {
      const float2 dp = f2mul(f2s(-2.0f), k.p);
      const float2 dPb = f2mul(f2mul(f2s(0.5f * e.beta), w.Pb1), dp);
      const float2 dPa = f2mul(f2mul(f2s(0.5f * e.alpha), w.Pa1), dp);
      const float2 dPa1 = f2mul(f2mul(f2s(0.5f * e.alpha - 1.0f), w.Pa2), dp);
      const float2 dPg1 = f2mul(f2mul(f2s(0.5f * e.gamma - 1.0f), w.Pg2), dp);
      const float2 dPb1 = f2mul(f2mul(f2s(0.5f * e.beta - 1.0f), w.Pb2), dp);
      dcG = f2mul(bs6n, f2fma(dPb, k.i1, f2mul(w.Pb, di1)));
      dcGG = f2mul(hb, dPb);
      const float2 dE3 = f2fma(f2s(e.kE3b), f2fma(dPb1, k.psi, f2mul(w.Pb1, dpsi)),
                               f2fma(f2mul(f2s(e.kE3g), dPg1), P.xm1,
                                     f2mul(f2s(e.kE3a), f2fma(dPa, w.Pa1, f2mul(w.Pam1, dPa1)))));
      dcI = f2fma(dE3, k.p, f2mul(c.E3, dp));
    } else {
      dcG = f2mul(f2mul(bs6n, w.Pb), di1);
      dcGG = f2s(0.0f);
      dcI = f2mul(f2mul(f2mul(f2s(e.kE3b), w.Pb1), dpsi), k.p);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 G0i = k.g[sym_idx(0, i)], H0i = k.h[sym_idx(0, i)];
      const float2 Gij = k.g[sym_idx(i, j)], Hij = k.h[sym_idx(i, j)];
      const float2 dG0i = f2neg(i == 0 ? f2add(G0j, Gij) : Gij);
      float2 t = f2fma(G0j, G0i, Hij);
      if (i == 0) t = f2add(t, H0j);
      const float2 dH0i = f2neg(f2fma(k.g[0], Gij, t));
      float2 v = f2fma(c.cGG, dH0i, f2fma(dcGG, H0i, f2fma(c.cG, dG0i, f2mul(dcG, G0i))));
      if (i == 0) v = f2add(v, dcI);
      om[i + 3 * j] = j == 0 ? f2fma(f2s(-2.0f), v, f2neg(s0r[i])) : f2mul(f2s(-2.0f), v);
    }
  }
}

// Closed-form seed of spectral_radius_fast for one lane: the root of largest modulus
// and the largest modulus of the other two.
__device__ __forceinline__ void seed_lane(float c0, float c2, float t, float p, float q, float disc, float& seed,
                                          float& other) {
  if (disc < 0.0f && p < 0.0f) {
    const float m = 2.0f * sqrt_approx(-p * (1.0f / 3.0f));
    const float cc = fminf(1.0f, fmaxf(-1.0f, __fdividef(3.0f * q, p * m)));
    const float th = acos_seed(cc) * (1.0f / 3.0f);
    const float y0 = m * __cosf(th) + t, y1 = m * __cosf(th - 2.0943951f) + t, y2 = m * __cosf(th - 4.1887902f) + t;
    const float a0 = fabsf(y0), a1 = fabsf(y1), a2 = fabsf(y2);
    if (a0 >= a1 && a0 >= a2) {
      seed = y0;
      other = fmaxf(a1, a2);
    } else if (a1 >= a2) {
      seed = y1;
      other = fmaxf(a0, a2);
    } else {
      seed = y2;
      other = fmaxf(a0, a1);
    }
  } else {
    const float sd = sqrt_approx(fmaxf(disc, 0.0f));
    seed = cbrt_seed(-0.5f * q + sd) + cbrt_seed(-0.5f * q - sd) + t;
    other = seed != 0.0f ? sqrt_approx(fabsf(__fdividef(c0, seed))) : fabsf(c2);
  }
}

// The other two roots' largest modulus after deflating root r (spectral_radius_fast).
__device__ __forceinline__ float deflate_lane(float c0, float c1, float c2, float r) {
  float s, qq;
  if (r != 0.0f) {
    s = c2 - r;
    qq = c0 / r;
  } else {
    s = c2;
    qq = c1;
  }
  const float dsc = s * s - 4.0f * qq;
  return dsc < 0.0f ? sqrt_approx(fabsf(qq)) : 0.5f * (fabsf(s) + sqrt_approx(dsc));
}

// spectral_radius_fast for two 3x3 matrices: the characteristic polynomial and the
// Newton steps packed, the seed and the deflation per lane.
__device__ __forceinline__ float2 spectral_radius_pair(const float2* a) {
  const float2 c2 = f2add(f2add(a[0], a[4]), a[8]);
  const float2 c1 = f2add(f2add(f2fma(a[0], a[4], f2neg(f2mul(a[3], a[1]))), f2fma(a[0], a[8], f2neg(f2mul(a[6], a[2])))),
                          f2fma(a[4], a[8], f2neg(f2mul(a[7], a[5]))));
  const float2 k0 = f2fma(a[4], a[8], f2neg(f2mul(a[5], a[7])));
  const float2 k1 = f2fma(a[1], a[8], f2neg(f2mul(a[7], a[2])));
  const float2 k2 = f2fma(a[1], a[5], f2neg(f2mul(a[4], a[2])));
  const float2 c0 = f2fma(a[6], k2, f2fma(f2neg(a[3]), k1, f2mul(a[0], k0)));
  const float2 t = f2mul(c2, f2s(1.0f / 3.0f));
  const float2 p = f2fma(f2neg(c2), t, c1);
  const float2 c2sq = f2mul(c2, c2);
  const float2 q = f2sub(f2fma(f2mul(c2, c1), f2s(1.0f / 3.0f), f2mul(f2mul(f2s(-2.0f / 27.0f), c2sq), c2)), c0);
  const float2 disc = f2fma(f2mul(f2s(0.25f), q), q, f2mul(f2mul(f2mul(p, p), p), f2s(1.0f / 27.0f)));
  float2 seed, other;
  seed_lane(c0.x, c2.x, t.x, p.x, q.x, disc.x, seed.x, other.x);
  seed_lane(c0.y, c2.y, t.y, p.y, q.y, disc.y, seed.y, other.y);
  float2 r = seed;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const float2 f = f2sub(f2mul(f2fma(f2sub(r, c2), r, c1), r), c0);
    const float2 fp = f2fma(f2fma(f2s(3.0f), r, f2mul(f2s(-2.0f), c2)), r, c1);
    r.x = fp.x != 0.0f ? r.x - __fdividef(f.x, fp.x) : r.x;
    r.y = fp.y != 0.0f ? r.y - __fdividef(f.y, fp.y) : r.y;
  }
  float2 rad = f2abs(r);
  if (!(other.x < 0.9f * fabsf(seed.x))) rad.x = fmaxf(rad.x, deflate_lane(c0.x, c1.x, c2.x, r.x));
  if (!(other.y < 0.9f * fabsf(seed.y))) rad.y = fmaxf(rad.y, deflate_lane(c0.y, c1.y, c2.y, r.y));
  return rad;
}

// lambda_mixed for two cells: |u1| + sqrt(spectral radius of the acoustic tensor).
__device__ __forceinline__ float2 lambda_pair(const EosMixed& em, const PrimP& P, const CoefP& c) {
  float2 s0[3], s0r[3], om[9];
  stress_row0_pair(P, c, s0);
  for (int i = 0; i < 3; ++i) s0r[i] = f2mul(s0[i], P.inv_rho_s);
  acoustic_pair(em.f, P, c, s0r, om);
  return f2add(f2abs(P.u[0]), f2sqrt_approx(spectral_radius_pair(om)));
}

}  // namespace hyp
