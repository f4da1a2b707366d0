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

__device__ __forceinline__ float2 df64_split(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - double(hi));
  return make_float2(hi, lo);
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

}  // namespace fec
