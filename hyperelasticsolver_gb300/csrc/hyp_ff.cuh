// hyp_ff.cuh -- float-float ("double-FP32") arithmetic for the mixed-precision step.
//
// A value is hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits, computed
// on the FP32 pipe (64x the FP64 rate of GB300). Error-free transformations:
// two_sum (Knuth 1969), fast_two_sum and two_prod via fused multiply-add
// (Dekker 1971); products, quotients and square roots after Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic" (ACM TOMS 2017). The _rn intrinsics keep the compiler
// from contracting or reassociating the error terms. A quotient's and a square
// root's first FP32 approximation comes from the hardware's approximate reciprocal
// and square root (about one ulp): the correction step that follows takes its error
// to the square of it (~2^-46 relative), as it does for a rounded first value.
#pragma once
#include <cuda_runtime.h>

namespace hyp {

// PTX rcp.approx.f32 / sqrt.approx.f32: one special-function instruction each.
__device__ __forceinline__ float rcp_approx(float a) {
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ float sqrt_approx(float a) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

struct ff {
  float hi, lo;
};

__device__ __forceinline__ float ff_val(ff a) { return __fadd_rn(a.hi, a.lo); }

// s + e == a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return ff{s, e};
}
// p + e == a * b exactly
__device__ __forceinline__ ff two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return ff{p, e};
}
// Sum with one two_sum of the high parts and the low parts added in FP32: the
// error is of order u^2 (|a| + |b|), u = 2^-24, i.e. ~1e-14 of the operands even
// under cancellation (rho E - |rho u|^2 / 2 rho), which is all the islands need.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  ff s = two_sum(a.hi, b);
  float v = __fadd_rn(a.lo, s.lo);
  return fast_two_sum(s.hi, v);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  float t = __fmul_rn(a.hi, b.lo);
  t = __fmaf_rn(a.lo, b.hi, t);
  return fast_two_sum(p.hi, __fadd_rn(p.lo, t));
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a / b: a first quotient from the correctly rounded reciprocal, its exact
// remainder in float-float, and one correction (the remainder step removes the
// first quotient's error, so IEEE division is not needed).
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float rb = rcp_approx(b.hi);
  float q1 = __fmul_rn(a.hi, rb);
  ff r = ff_sub(a, ff_mul(b, ff{q1, 0.0f}));
  float q2 = __fmul_rn(r.hi, rb);
  return fast_two_sum(q1, q2);
}
__device__ __forceinline__ ff ff_recip(ff b) { return ff_div(ff{1.0f, 0.0f}, b); }
// sqrt(a), a > 0: one Newton correction of the FP32 root in float-float
__device__ __forceinline__ ff ff_sqrt(ff a) {
  float s = sqrt_approx(a.hi);
  ff p = two_prod(s, s);
  float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo);
  float c = __fmul_rn(r, __fmul_rn(0.5f, rcp_approx(s)));
  return fast_two_sum(s, c);
}
// a*b - c*d with one rounding of the final sum (cofactors of the determinant)
__device__ __forceinline__ ff ff_diff_prod(float a, float b, float c, float d) {
  ff p = two_prod(a, b);
  ff q = two_prod(c, d);
  return ff_sub(p, q);
}

}  // namespace hyp
