// hyp_physics_mixed.cuh -- per-cell physics of the mixed-precision step.
//
// The state arrives as compensated pairs (hi, lo) of FP32 per conservative
// variable. The steps whose cancellation would spoil FP32 are evaluated in
// float-float (about 48 bits, on the FP32 pipe):
//   - det(rho A) and rho_true = sqrt(det / rho0)  (HyperelasticityMPh.jl:113-114),
//     with the lo parts entering through the cofactors;
//   - the internal-energy subtraction e = E - |u|^2/2   (HyperelasticityMPh.jl:117-120),
//     as rho e = rho E - |rho u|^2 / (2 rho);
//   - the volumetric strain s - 1 = rho/rho0 - 1 of the cold energy;
// and the near-identity shear invariant i1^2/3 - i2 is formed from differences
// of G's entries (no cancellation). Everything else (finger tensor, stress,
// acoustic tensor, eigen-solve, flux) is FP32, shared with the FP64 step
// through the templates of hyp_physics.cuh.
#pragma once
#include "hyp_ff.cuh"
#include "hyp_pair.cuh"
#include "hyp_physics.cuh"

namespace hyp {

struct EosMixed {
  EosT<float> f;
  ff inv_rho0;  // 1/rho0 as a float-float
};

inline EosMixed make_eos_mixed(const EosC& e) {
  EosMixed m;
  m.f = eos_as<float>(e);
  float h = (float)e.inv_rho0;
  m.inv_rho0 = ff{h, (float)(e.inv_rho0 - (double)h)};
  return m;
}

struct PrimM {
  float rho_u1;          // alpha*rho*u1 of the state (the mass flux)
  float u[3], E, e_int;  // velocity, specific total and internal energy
  float A[9];            // distortion
  float xm1;             // exp(S/cv) - 1
  float rho_s, inv_rho_s;
  KinT<float> k;
  PowsT<float> w;
};

// Outputs of the float-float islands of one cell, cached per cell between steps.
struct Islands {
  float ir;     // 1 / rho_true
  float e_int;  // specific internal energy
  float sm1;    // rho_true / rho0 - 1
};

// The float-float islands of cons2prim for one single-phase cell from (hi, lo)
// pairs; returns HYP_CELL_* status.
__device__ __forceinline__ int islands_mixed(const EosMixed& em, const float* qh, const float* ql, Islands& I) {
  const float* m = qh + 5;  // rho*A (hi), column-major
  const float* l = ql + 5;  // rho*A (lo)
  // det(rho A) in float-float: first-row expansion with exact products, plus the
  // first-order contribution of the lo parts through all nine cofactors.
  ff C00 = ff_diff_prod(m[4], m[8], m[7], m[5]);
  ff C01 = ff_neg(ff_diff_prod(m[1], m[8], m[7], m[2]));
  ff C02 = ff_diff_prod(m[1], m[5], m[4], m[2]);
  ff d = ff_add(ff_add(ff_mul_f(C00, m[0]), ff_mul_f(C01, m[3])), ff_mul_f(C02, m[6]));
  float dlo = C00.hi * l[0] + C01.hi * l[3] + C02.hi * l[6];
  dlo += -(m[3] * m[8] - m[6] * m[5]) * l[1] + (m[0] * m[8] - m[6] * m[2]) * l[4] - (m[0] * m[5] - m[3] * m[2]) * l[7];
  dlo += (m[3] * m[7] - m[6] * m[4]) * l[2] - (m[0] * m[7] - m[6] * m[1]) * l[5] + (m[0] * m[4] - m[3] * m[1]) * l[8];
  d = ff_add_f(d, dlo);
  int st = d.hi > 0.0f ? HYP_CELL_OK : HYP_CELL_NEG_DET;
  ff rho = ff_sqrt(ff_mul(d, em.inv_rho0));  // rho_true = sqrt(det(rho A) / rho0)
  ff inv_rho = ff_recip(rho);
  // rho e = rho E - |rho u|^2 / (2 rho)
  ff m0{qh[1], ql[1]}, m1{qh[2], ql[2]}, m2{qh[3], ql[3]};
  ff k2 = ff_add(ff_add(ff_mul(m0, m0), ff_mul(m1, m1)), ff_mul(m2, m2));
  ff ke = ff_mul(k2, ff_mul_f(inv_rho, 0.5f));
  ff rhoe = ff_sub(ff{qh[4], ql[4]}, ke);
  I.e_int = ff_val(ff_mul(rhoe, inv_rho));
  // s = rho / rho0 = 1/det A, and s - 1
  ff s = ff_mul(rho, em.inv_rho0);
  I.sm1 = ff_val(ff_add_f(s, -1.0f));
  I.ir = ff_val(inv_rho);
  if (!(I.e_int == I.e_int) || !(I.sm1 == I.sm1)) st |= HYP_CELL_NONFINITE;
  return st;
}

// The FP32 rest of cons2prim given the island outputs; returns HYP_CELL_* status.
__device__ __forceinline__ int prim_from_islands(const EosMixed& em, const float* qh, const float* ql, const Islands& I,
                                                 PrimM& P) {
  const EosT<float>& e = em.f;
  const float ir = I.ir, sm1 = I.sm1;
  const float sf = 1.0f + sm1;
  P.e_int = I.e_int;
  P.rho_u1 = __fadd_rn(qh[1], ql[1]);
  for (int c = 0; c < 3; ++c) P.u[c] = qh[1 + c] * ir;
  P.E = qh[4] * ir;
  for (int c = 0; c < 9; ++c) P.A[c] = qh[5 + c] * ir;
  P.k = kinematics_s<float>(P.A, sf, rcp_approx(sf));
  P.w = powers<float>(e, P.k);
  P.w.Pam1 = e.default_exp ? sm1 : expm1f(e.alpha * log1pf(sm1));
  P.xm1 = entropy_xm1<float>(e, P.e_int, P.k, P.w);
  P.rho_s = e.rho0 * sf;
  P.inv_rho_s = P.k.inv_s * e.inv_rho0;
  return (P.xm1 == P.xm1 && isfinite(P.k.p)) ? HYP_CELL_OK : HYP_CELL_NONFINITE;
}

__device__ __forceinline__ int prim_mixed(const EosMixed& em, const float* qh, const float* ql, PrimM& P,
                                          Islands& I) {
  int st = islands_mixed(em, qh, ql, I);
  return st | prim_from_islands(em, qh, ql, I, P);
}

// Physical x-flux of a single-phase cell (HyperelasticityMPh.jl:146-175 at alpha = 1):
// the 11 components that are not identically zero, in the order of flux_slot1.
__device__ __forceinline__ void flux_mixed(const EosMixed& em, const float* qh, const PrimM& P,
                                           const StressCT<float>& c, float* f11) {
  float s0[3];
  stress_row0<float>(P.rho_s, P.k, c, s0);
  const float mu = P.rho_u1;
  f11[0] = mu;
  f11[1] = mu * P.u[0] - s0[0];
  f11[2] = mu * P.u[1] - s0[1];
  f11[3] = mu * P.u[2] - s0[2];
  f11[4] = mu * P.E - (P.u[0] * s0[0] + P.u[1] * s0[1] + P.u[2] * s0[2]);
  const float* rA = qh + 5;
  // rho A flux [a,b] = u1 rhoA[a,b] - u_a rhoA[0,b]  for a = 1, 2
  for (int b = 0; b < 3; ++b)
    for (int a = 1; a < 3; ++a) f11[5 + 2 * b + (a - 1)] = P.u[0] * rA[a + 3 * b] - P.u[a] * rA[3 * b];
}

// acos on [-1, 1] to ~7e-5 (Abramowitz & Stegun 4.4.45): enough for a Newton seed.
__device__ __forceinline__ float acos_seed(float x) {
  const float ax = fabsf(x);
  const float r = sqrt_approx(1.0f - ax) * (1.5707288f + ax * (-0.2121144f + ax * (0.0742610f - 0.0187293f * ax)));
  return x >= 0.0f ? r : 3.14159265f - r;
}
__device__ __forceinline__ float cbrt_seed(float x) {
  return x == 0.0f ? 0.0f : copysignf(exp2f(__log2f(fabsf(x)) * (1.0f / 3.0f)), x);
}

// Spectral radius of a real 3x3 (column-major) in FP32 for the mixed step: the
// same characteristic-polynomial method as eig_core (closed-form seed of the
// root of largest modulus, Newton polishing, deflation), with a seed from fast
// approximations, two Newton steps, and the deflation evaluated only when the
// seeds do not already show that root to dominate the other two by 10 %.
__device__ __forceinline__ float spectral_radius_fast(const float* a) {
  const float c2 = a[0] + a[4] + a[8];
  const float c1 = (a[0] * a[4] - a[3] * a[1]) + (a[0] * a[8] - a[6] * a[2]) + (a[4] * a[8] - a[7] * a[5]);
  const float c0 = det3(a);
  const float t = c2 * (1.0f / 3.0f);
  const float p = c1 - c2 * t;
  const float q = -2.0f / 27.0f * c2 * c2 * c2 + c2 * c1 * (1.0f / 3.0f) - c0;
  const float disc = 0.25f * q * q + p * p * p * (1.0f / 27.0f);
  float seed, other;  // seed: root of largest modulus; other: largest modulus of the rest
  if (disc < 0.0f && p < 0.0f) {
    const float m = 2.0f * sqrt_approx(-p * (1.0f / 3.0f));
    const float cc = fminf(1.0f, fmaxf(-1.0f, __fdividef(3.0f * q, p * m)));
    const float th = acos_seed(cc) * (1.0f / 3.0f);
    const float y0 = m * __cosf(th) + t, y1 = m * __cosf(th - 2.0943951f) + t, y2 = m * __cosf(th - 4.1887902f) + t;
    const float a0 = fabsf(y0), a1 = fabsf(y1), a2 = fabsf(y2);
    if (a0 >= a1 && a0 >= a2) { seed = y0; other = fmaxf(a1, a2); }
    else if (a1 >= a2) { seed = y1; other = fmaxf(a0, a2); }
    else { seed = y2; other = fmaxf(a0, a1); }
  } else {
    const float sd = sqrt_approx(fmaxf(disc, 0.0f));
    seed = cbrt_seed(-0.5f * q + sd) + cbrt_seed(-0.5f * q - sd) + t;
    other = seed != 0.0f ? sqrt_approx(fabsf(__fdividef(c0, seed))) : fabsf(c2);  // |complex pair| = sqrt(c0 / r)
  }
  float r = seed;
  for (int it = 0; it < 2; ++it) {
    const float f = ((r - c2) * r + c1) * r - c0;
    const float fp = (3.0f * r - 2.0f * c2) * r + c1;
    r = fp != 0.0f ? r - __fdividef(f, fp) : r;
  }
  float rad = fabsf(r);
  if (!(other < 0.9f * fabsf(seed))) {  // close moduli: resolve the other two exactly
    float s, qq;
    if (r != 0.0f) { s = c2 - r; qq = c0 / r; } else { s = c2; qq = c1; }
    const float dsc = s * s - 4.0f * qq;
    const float m2 = dsc < 0.0f ? sqrt_approx(fabsf(qq)) : 0.5f * (fabsf(s) + sqrt_approx(dsc));
    rad = fmaxf(rad, m2);
  }
  return rad;
}

// acoustic_omega<float> with columns 1 and 2 (the same formulas, dcGG = 0 and no
// density or p term) as the two lanes of packed FP32 pairs; column 0 scalar.
__device__ __forceinline__ void acoustic_omega_f32(const EosT<float>& e, const KinT<float>& k, const PowsT<float>& w,
                                                   const StressCT<float>& c, float xm1, const float* s0r, float* om) {
  const SymT<float>& G = k.G;
  const SymT<float>& H = k.H;
  const float G0[3] = {G.a00, G.a01, G.a02}, H0[3] = {H.a00, H.a01, H.a02};
  float o0[3];
  {  // column 0 (acoustic_omega's j = 0 statements)
    const float di1 = -2.0f * G.a00;
    const float dpsi = (2.0f / 3.0f) * k.i1 * G.a00 - 2.0f * H.a00;
    const float dp = -2.0f * k.p;
    const float dPb = 0.5f * e.beta * w.Pb1 * dp;
    const float dPa = 0.5f * e.alpha * w.Pa1 * dp;
    const float dPa1 = (0.5f * e.alpha - 1.0f) * w.Pa2 * dp;
    const float dPg1 = (0.5f * e.gamma - 1.0f) * w.Pg2 * dp;
    const float dPb1 = (0.5f * e.beta - 1.0f) * w.Pb2 * dp;
    const float dcG = -e.b0sq_6 * (dPb * k.i1 + w.Pb * di1);
    const float dcGG = 0.5f * e.b0sq * dPb;
    const float dE3 = e.kE3a * (dPa * w.Pa1 + w.Pam1 * dPa1) + e.kE3g * dPg1 * xm1 + e.kE3b * (dPb1 * k.psi + w.Pb1 * dpsi);
    const float dcI = dE3 * k.p + c.E3 * dp;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float dG0i = -((i == 0 ? G.a00 : 0.0f) + G0[i]);
      const float dH0i = -(G.a00 * G0[i] + H0[i] + (i == 0 ? H.a00 : 0.0f) + G.a00 * G0[i]);
      const float v = dcG * G0[i] + c.cG * dG0i + dcGG * H0[i] + c.cGG * dH0i + (i == 0 ? dcI : 0.0f);
      o0[i] = -2.0f * v - s0r[i];
    }
  }
  const float2 G0j = make_float2(G.a01, G.a02), H0j = make_float2(H.a01, H.a02);
  const float2 di1 = f2mul(f2s(-2.0f), G0j);
  const float2 dpsi = f2fma(f2s((2.0f / 3.0f) * k.i1), G0j, f2mul(f2s(-2.0f), H0j));
  const float2 dcG = f2mul(f2s(-e.b0sq_6 * w.Pb), di1);
  const float2 dcI = f2mul(f2mul(f2s(e.kE3b * w.Pb1), dpsi), f2s(k.p));
  const float2 cG = f2s(c.cG), cGG = f2s(c.cGG);
  // rows i of columns 1, 2: G(i,1), G(i,2) and H(i,1), H(i,2)
  const float2 Gi[3] = {make_float2(G.a01, G.a02), make_float2(G.a11, G.a12), make_float2(G.a12, G.a22)};
  const float2 Hi[3] = {make_float2(H.a01, H.a02), make_float2(H.a11, H.a12), make_float2(H.a12, H.a22)};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float2 dG0i = f2neg(i == 0 ? f2add(G0j, Gi[i]) : Gi[i]);
    float2 t = f2fma(G0j, f2s(G0[i]), Hi[i]);
    if (i == 0) t = f2add(t, H0j);
    const float2 dH0i = f2neg(f2fma(f2s(G.a00), Gi[i], t));
    float2 v = f2fma(cGG, dH0i, f2fma(cG, dG0i, f2mul(dcG, f2s(G0[i]))));
    if (i == 0) v = f2add(v, dcI);
    const float2 o = f2mul(f2s(-2.0f), v);
    om[i] = o0[i];
    om[i + 3] = o.x;
    om[i + 6] = o.y;
  }
}

// max |u1 +- c_k| = |u1| + sqrt(spectral radius of the acoustic tensor)
__device__ __forceinline__ float lambda_mixed(const EosMixed& em, const PrimM& P, const StressCT<float>& c) {
  float s0[3], s0r[3], om[9];
  stress_row0<float>(P.rho_s, P.k, c, s0);
  for (int i = 0; i < 3; ++i) s0r[i] = s0[i] * P.inv_rho_s;
  acoustic_omega_f32(em.f, P.k, P.w, c, P.xm1, s0r, om);
  return fabsf(P.u[0]) + sqrt_approx(spectral_radius_fast(om));
}

}  // namespace hyp
