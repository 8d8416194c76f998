// hyp_pair.cuh -- packed FP32 pairs (sm_100+ f32x2 arithmetic) and float-float pairs.
//
// A float2 here holds one value of two independent evaluations (two cells, or two
// phases of a cell): .x of the first, .y of the second. Each helper is one packed
// instruction (__fadd2_rn, __fmul2_rn, __ffma2_rn) or, where no packed form exists
// (reciprocal, square root, comparisons), two scalar ones. Fused multiply-adds are
// written out, so results differ from contracted scalar code in the last bits.
//
// ff2 is the float-float type of hyp_ff.cuh for two lanes at once: the same
// error-free transformations (Knuth's two_sum, Dekker's fast_two_sum and FMA-based
// two_prod) and the same double-word products, quotients and square roots (Joldes,
// Muller and Popescu, ACM TOMS 2017), lane by lane.
#pragma once
#include <cuda_runtime.h>
#include "hyp_ff.cuh"

namespace hyp {

__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __fadd2_rn(a, f2neg(b)); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2rcp(float2 a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
__device__ __forceinline__ float2 f2sqrt(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ float2 f2abs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
// The hardware's approximate reciprocal and square root (hyp_ff.cuh; about one ulp
// from the rounded results) for FP32 states whose own rounding already exceeds that.
__device__ __forceinline__ float2 f2rcp_approx(float2 a) { return make_float2(rcp_approx(a.x), rcp_approx(a.y)); }
__device__ __forceinline__ float2 f2sqrt_approx(float2 a) { return make_float2(sqrt_approx(a.x), sqrt_approx(a.y)); }
__device__ __forceinline__ float2 f2max(float2 a, float2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }

struct ff2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 ff2_val(ff2 a) { return f2add(a.hi, a.lo); }
__device__ __forceinline__ ff2 two_sum2(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  const float2 bb = f2sub(s, a);
  const float2 e = f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
  return ff2{s, e};
}
__device__ __forceinline__ ff2 fast_two_sum2(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  return ff2{s, f2sub(b, f2sub(s, a))};
}
__device__ __forceinline__ ff2 two_prod2(float2 a, float2 b) {
  const float2 p = f2mul(a, b);
  return ff2{p, f2fma(a, b, f2neg(p))};
}
__device__ __forceinline__ ff2 ff2_add(ff2 a, ff2 b) {
  const ff2 s = two_sum2(a.hi, b.hi);
  return fast_two_sum2(s.hi, f2add(s.lo, f2add(a.lo, b.lo)));
}
__device__ __forceinline__ ff2 ff2_neg(ff2 a) { return ff2{f2neg(a.hi), f2neg(a.lo)}; }
__device__ __forceinline__ ff2 ff2_sub(ff2 a, ff2 b) { return ff2_add(a, ff2_neg(b)); }
__device__ __forceinline__ ff2 ff2_add_f(ff2 a, float2 b) {
  const ff2 s = two_sum2(a.hi, b);
  return fast_two_sum2(s.hi, f2add(a.lo, s.lo));
}
__device__ __forceinline__ ff2 ff2_mul(ff2 a, ff2 b) {
  const ff2 p = two_prod2(a.hi, b.hi);
  const float2 t = f2fma(a.lo, b.hi, f2mul(a.hi, b.lo));
  return fast_two_sum2(p.hi, f2add(p.lo, t));
}
__device__ __forceinline__ ff2 ff2_mul_f(ff2 a, float2 b) {
  const ff2 p = two_prod2(a.hi, b);
  return fast_two_sum2(p.hi, f2fma(a.lo, b, p.lo));
}
__device__ __forceinline__ ff2 ff2_div(ff2 a, ff2 b) {
  const float2 rb = f2rcp_approx(b.hi);
  const float2 q1 = f2mul(a.hi, rb);
  const ff2 r = ff2_sub(a, ff2_mul(b, ff2{q1, f2s(0.0f)}));
  return fast_two_sum2(q1, f2mul(r.hi, rb));
}
__device__ __forceinline__ ff2 ff2_recip(ff2 b) { return ff2_div(ff2{f2s(1.0f), f2s(0.0f)}, b); }
__device__ __forceinline__ ff2 ff2_sqrt(ff2 a) {
  const float2 s = f2sqrt_approx(a.hi);
  const ff2 p = two_prod2(s, s);
  const float2 r = f2add(f2sub(f2sub(a.hi, p.hi), p.lo), a.lo);
  const float2 c = f2mul(r, f2mul(f2s(0.5f), f2rcp_approx(s)));
  return fast_two_sum2(s, c);
}
__device__ __forceinline__ ff2 ff2_diff_prod(float2 a, float2 b, float2 c, float2 d) {
  return ff2_sub(two_prod2(a, b), two_prod2(c, d));
}

}  // namespace hyp
