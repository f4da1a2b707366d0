// fec_df64.cuh -- double-float ("df64") arithmetic on the FP32 pipes.
//
// A value is carried as an unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi)/2, about 48 significant bits.  Products use the exact
// error of the high product from one fused multiply-add (Dekker's two-product
// with FMA), sums use Knuth's error-free TwoSum, and every result is
// renormalised with Fast2Sum.  All operations go through the _rn intrinsics so
// that the compiler cannot contract a multiply and an add into an FMA and break
// the error-free transformations.
//
// Why: the GB300 executes FP64 at 1/62 of its FP32 rate (1.26 vs 78 TFLOP/s
// measured), so the FP64 variant of the element-tangent contraction is bound by
// the FP64 pipe.  Running that contraction in df64 moves it to the FP32 pipes at
// ~2^-48 relative error per operation, far inside the 1e-12 relative bar on the
// assembled values.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fec {

// Split by conversion: three FP64-pipe operations (two conversions, one
// subtraction).  Used for zero, subnormal-range, huge and non-finite values.
static __device__ __noinline__ float2 df64_split_fp64(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - double(hi));
  return make_float2(hi, lo);
}

// Split of a double into hi + lo on the integer and FP32 pipes.  For binary
// exponents E in [949, 1149] (|x| in about [2^-74, 2^126)):
//   hi: the mantissa rounded to 24 bits by adding half of the discarded field
//       (2^28) to the bit pattern -- a carry into the exponent is the correct
//       rounding -- then the exponent rebiased 1023 -> 127 by one subtraction
//       on the funnel-shifted word;
//   lo: x - hi is the difference of the two bit patterns in units of
//       2^(E-1075) (the bit pattern is linear in the value within a binade and
//       across the boundary the carry crosses), |diff| <= 2^28, converted to
//       float (rounded to 24 bits) and scaled by the signed power of two.
// |lo| <= ulp(hi)/2 (ties round away from zero), |hi + lo - x| <= 2^-48 |x|: the
// same representation __double2float_rn gives up to the tie rule.  Signed
// zeros are selected in place; everything else takes the conversion path.
__device__ __forceinline__ float2 df64_split(double x) {
  const uint64_t b = uint64_t(__double_as_longlong(x));
  const uint32_t bh = uint32_t(b >> 32), bl = uint32_t(b);
  const uint32_t E = (bh >> 20) & 0x7FFu;
  const bool zero = ((bh & 0x7FFFFFFFu) | bl) == 0u;
  if (E - 949u > 200u && !zero) return df64_split_fp64(x);
  const uint64_t r = b + (uint64_t(1) << 28);
  const uint32_t rh = uint32_t(r >> 32), rl = uint32_t(r);
  const uint32_t fs = __funnelshift_l(rl, rh, 3);  // exponent (low 9 bits) | top 23 mantissa bits
  const float hi = __uint_as_float(((fs - 0xC0000000u) & 0x7FFFFFFFu) | (rh & 0x80000000u));
  const int32_t diff = int32_t(bl - (rl & 0xE0000000u));
  const float scale = __uint_as_float(((E - 948u) << 23) | (bh & 0x80000000u));
  const float lo = __fmul_rn(__int2float_rn(diff), scale);
  return zero ? make_float2(__uint_as_float(bh & 0x80000000u), 0.f) : make_float2(hi, lo);
}

__device__ __forceinline__ float2 df64_fast2sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// a * b
__device__ __forceinline__ float2 df64_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return df64_fast2sum(p, e);
}

// a + b
__device__ __forceinline__ float2 df64_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float v = __fsub_rn(s, a.x);
  const float t = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, v)), __fsub_rn(b.x, v));
  return df64_fast2sum(s, __fadd_rn(t, __fadd_rn(a.y, b.y)));
}

// c + a * b
__device__ __forceinline__ float2 df64_fma(float2 a, float2 b, float2 c) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float s = __fadd_rn(c.x, p);
  const float v = __fsub_rn(s, c.x);
  const float t = __fadd_rn(__fsub_rn(c.x, __fsub_rn(s, v)), __fsub_rn(p, v));
  return df64_fast2sum(s, __fadd_rn(t, __fadd_rn(c.y, e)));
}

__device__ __forceinline__ float2 df64_neg(float2 a) { return make_float2(-a.x, -a.y); }

// c + a0 b0 + a1 b1 + a2 b2 with one renormalisation: each product's high part
// and exact error come from one FMA (two-product), the three high parts are
// added to c.x with TwoSum, and all low-order terms (product errors, cross
// terms, TwoSum errors, c.y) are summed in FP32 before the final Fast2Sum.
// 38 FP32 operations against 45 for three chained df64_fma, same ~2^-48
// relative accuracy for these short sums.
__device__ __forceinline__ float2 df64_dot3_acc(float2 c, float2 a0, float2 b0, float2 a1, float2 b1, float2 a2,
                                                float2 b2) {
  const float p0 = __fmul_rn(a0.x, b0.x), p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
  float e = __fmaf_rn(a0.x, b0.x, -p0);
  e = __fmaf_rn(a0.x, b0.y, e);
  e = __fmaf_rn(a0.y, b0.x, e);
  e = __fadd_rn(__fmaf_rn(a1.x, b1.x, -p1), e);
  e = __fmaf_rn(a1.x, b1.y, e);
  e = __fmaf_rn(a1.y, b1.x, e);
  e = __fadd_rn(__fmaf_rn(a2.x, b2.x, -p2), e);
  e = __fmaf_rn(a2.x, b2.y, e);
  e = __fmaf_rn(a2.y, b2.x, e);
  float s = c.x, lo = __fadd_rn(c.y, e);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float p = k == 0 ? p0 : (k == 1 ? p1 : p2);
    const float t = __fadd_rn(s, p);
    const float v = __fsub_rn(t, s);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v)));
    s = t;
  }
  return df64_fast2sum(s, lo);
}

// df64_dot3_acc without the final renormalization, for long accumulation chains:
// c and the result are (s, lo) with s the FP32 running sum and lo the sum of its
// exact rounding errors (TwoSum) and of the products' low parts, |lo| not held
// below ulp(s)/2; the chain ends with df64_renorm.  Over n calls lo carries about
// n ulps of s, so its own rounding stays near n 2^-48 |s|, the bound of the
// renormalized chain; it saves three of the ~36 operations per call.
__device__ __forceinline__ float2 df64_dot3_acc_lazy(float2 c, float2 a0, float2 b0, float2 a1, float2 b1, float2 a2,
                                                     float2 b2) {
  const float p0 = __fmul_rn(a0.x, b0.x), p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
  float e = __fmaf_rn(a0.x, b0.x, -p0);
  e = __fmaf_rn(a0.x, b0.y, e);
  e = __fmaf_rn(a0.y, b0.x, e);
  e = __fadd_rn(__fmaf_rn(a1.x, b1.x, -p1), e);
  e = __fmaf_rn(a1.x, b1.y, e);
  e = __fmaf_rn(a1.y, b1.x, e);
  e = __fadd_rn(__fmaf_rn(a2.x, b2.x, -p2), e);
  e = __fmaf_rn(a2.x, b2.y, e);
  e = __fmaf_rn(a2.y, b2.x, e);
  float s = c.x, lo = __fadd_rn(c.y, e);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float p = k == 0 ? p0 : (k == 1 ? p1 : p2);
    const float t = __fadd_rn(s, p);
    const float v = __fsub_rn(t, s);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v)));
    s = t;
  }
  return make_float2(s, lo);
}
// (s, lo) -> the double-float s + lo, with no ordering precondition (TwoSum)
__device__ __forceinline__ float2 df64_renorm(float2 v) {
  const float s = __fadd_rn(v.x, v.y), bb = __fsub_rn(s, v.x);
  return make_float2(s, __fadd_rn(__fsub_rn(v.x, __fsub_rn(s, bb)), __fsub_rn(v.y, bb)));
}

// a0 b0 + a1 b1 + a2 b2 (the same without an accumulator: the first high part
// starts the sum).
__device__ __forceinline__ float2 df64_dot3(float2 a0, float2 b0, float2 a1, float2 b1, float2 a2, float2 b2) {
  const float p0 = __fmul_rn(a0.x, b0.x), p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
  float e = __fmaf_rn(a0.x, b0.x, -p0);
  e = __fmaf_rn(a0.x, b0.y, e);
  e = __fmaf_rn(a0.y, b0.x, e);
  e = __fadd_rn(__fmaf_rn(a1.x, b1.x, -p1), e);
  e = __fmaf_rn(a1.x, b1.y, e);
  e = __fmaf_rn(a1.y, b1.x, e);
  e = __fadd_rn(__fmaf_rn(a2.x, b2.x, -p2), e);
  e = __fmaf_rn(a2.x, b2.y, e);
  e = __fmaf_rn(a2.y, b2.x, e);
  float s = p0, lo = e;
#pragma unroll
  for (int k = 1; k < 3; ++k) {
    const float p = k == 1 ? p1 : p2;
    const float t = __fadd_rn(s, p);
    const float v = __fsub_rn(t, s);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v)));
    s = t;
  }
  return df64_fast2sum(s, lo);
}

}  // namespace fec
