// cgb_pair.cuh — FP32-pair ("double-float") arithmetic for the mixed-precision shape stage.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about
// 48 significant bits. Everything here runs on the FP32 pipe, which on GB300 issues 62x
// the FP64 rate, so per-neighbour work in pairs costs a fraction of the same work in FP64.
//
// Published methods, restated:
//  - TwoSum (Knuth, TAOCP vol. 2, sec. 4.2.2; Moller 1965): s = fl(a + b) and the exact
//    rounding error e, a + b = s + e, in six additions, any magnitudes.
//  - FastTwoSum (Dekker 1971): the same in three additions when |a| >= |b|.
//  - TwoProd with a fused multiply-add: p = fl(a b), e = fma(a, b, -p) is exact.
//  - Pair addition and multiplication as in Dekker (1971), "A floating-point technique for
//    extending the available precision", and the double-double library of Hida, Li and
//    Bailey (2001), with float in place of double ("sloppy" addition where operands do not
//    cancel, the two-TwoSum addition where they may).
//  - Reciprocal and square root by one Newton step on the pair (Karp and Markstein 1997,
//    "High-precision division and square root"), seeded by the single-precision result.
//  - Dot products accumulated as in Ogita, Rump and Oishi (2005), "Accurate sum and dot
//    product" (Dot2): the high parts by TwoSum, all rounding errors in a second float.
// All operations use explicitly rounded intrinsics, so the compiler neither contracts nor
// reorders the error-free transforms.
#pragma once

#include <cuda_runtime.h>

namespace cgb {

struct fp2 {
  float hi, lo;
};

__device__ __forceinline__ fp2 fp2_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ fp2 fp2_fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ fp2 fp2_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ fp2 fp2_of(float a) { return {a, 0.0f}; }

// Split of a double into a pair (per point or per node only: uses the FP64 pipe).
__device__ __forceinline__ fp2 fp2_from_double(double d) {
  const float hi = __double2float_rn(d);
  return {hi, __double2float_rn(d - static_cast<double>(hi))};
}

__device__ __forceinline__ double fp2_to_double(fp2 a) {
  return static_cast<double>(a.hi) + static_cast<double>(a.lo);
}

__device__ __forceinline__ fp2 operator-(fp2 a) { return {-a.hi, -a.lo}; }

// a + b, for operands that do not nearly cancel.
__device__ __forceinline__ fp2 operator+(fp2 a, fp2 b) {
  const fp2 s = fp2_two_sum(a.hi, b.hi);
  return fp2_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ fp2 operator-(fp2 a, fp2 b) { return a + (-b); }

// a + b with full relative accuracy also under cancellation.
__device__ __forceinline__ fp2 fp2_add_exact(fp2 a, fp2 b) {
  fp2 s = fp2_two_sum(a.hi, b.hi);
  const fp2 t = fp2_two_sum(a.lo, b.lo);
  s = fp2_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fp2_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ __forceinline__ fp2 operator*(fp2 a, fp2 b) {
  const fp2 p = fp2_two_prod(a.hi, b.hi);
  return fp2_fast_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}
// By a float that is exact (small integers, powers of two, sides +-1).
__device__ __forceinline__ fp2 operator*(fp2 a, float b) {
  const fp2 p = fp2_two_prod(a.hi, b);
  return fp2_fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ fp2 operator*(float b, fp2 a) { return a * b; }
__device__ __forceinline__ fp2 operator+(fp2 a, float b) {
  const fp2 s = fp2_two_sum(a.hi, b);
  return fp2_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ fp2 operator+(float b, fp2 a) { return a + b; }
__device__ __forceinline__ fp2 operator-(float b, fp2 a) { return (-a) + b; }
__device__ __forceinline__ fp2 operator-(fp2 a, float b) { return a + (-b); }

__device__ __forceinline__ fp2 fp2_sqr(fp2 a) {
  const fp2 p = fp2_two_prod(a.hi, a.hi);
  return fp2_fast_two_sum(p.hi, __fmaf_rn(2.0f * a.hi, a.lo, p.lo));
}

// 1 / b: x = 1 / b.hi, then x + x (1 - b x) with the residual formed in pairs.
__device__ __forceinline__ fp2 fp2_recip(fp2 b) {
  const float x = __frcp_rn(b.hi);
  // r = 1 - b x, exactly enough: 1 - b.hi x is exact by one FMA, then the b.lo term.
  const float r = __fmaf_rn(-b.lo, x, __fmaf_rn(-b.hi, x, 1.0f));
  return fp2_fast_two_sum(x, __fmul_rn(x, r));
}

// sqrt(a) for a >= 0: y = sqrt(a.hi), then y + (a - y^2) / (2 y).
__device__ __forceinline__ fp2 fp2_sqrt(fp2 a) {
  if (a.hi <= 0.0f) return {0.0f, 0.0f};
  const float y = __fsqrt_rn(a.hi);
  const fp2 y2 = fp2_two_prod(y, y);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, y2.hi), y2.lo), a.lo);
  return fp2_fast_two_sum(y, __fmul_rn(r, __fdividef(0.5f, y)));
}

// Dot-product accumulator (Dot2): acc.hi carries the running sum by TwoSum, acc.lo the
// sum of every rounding error; normalise with fp2_norm once the sum is complete.
__device__ __forceinline__ void fp2_fma_acc(fp2& acc, fp2 a, fp2 b) {
  const fp2 p = fp2_two_prod(a.hi, b.hi);
  const float cross = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
  const fp2 s = fp2_two_sum(acc.hi, p.hi);
  acc.hi = s.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, __fadd_rn(p.lo, cross)));
}

__device__ __forceinline__ fp2 fp2_norm(fp2 a) { return fp2_two_sum(a.hi, a.lo); }

// Comparisons with float constants (exact in float: 0, 0.5, 1).
__device__ __forceinline__ bool fp2_ge(fp2 a, float c) { return a.hi > c || (a.hi == c && a.lo >= 0.0f); }
__device__ __forceinline__ bool fp2_le(fp2 a, float c) { return a.hi < c || (a.hi == c && a.lo <= 0.0f); }
__device__ __forceinline__ bool fp2_is_zero(fp2 a) { return a.hi == 0.0f && a.lo == 0.0f; }

}  // namespace cgb
