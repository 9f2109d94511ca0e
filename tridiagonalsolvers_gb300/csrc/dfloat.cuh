// Double-float arithmetic (an unevaluated sum hi + lo of two FP32 values,
// 48-bit significand) and exact FP32 -> FP64 assembly without the FP64
// pipe, for the residuals and updates of the refinement kernels: GB300's FP64
// rate is 1/64 of its FP32 rate.
#pragma once
#include "tridi_device.cuh"

namespace tridi {

// Exact float -> double by assembling the IEEE-754 fields (normal numbers and
// zeros; subnormals, infinities and NaNs take the conversion instruction).
// Keeps the residual's conversions off the FP64 pipe.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return (double)f;
}

// The double nearest hi + lo for a normalised double-float pair
// (|lo| <= ulp_float(hi) / 2), mostly without the FP64 pipe: when lo is a
// whole number K of hi's double ulps (its lowest set bit no finer than that
// ulp, i.e. float exponent of lo >= exponent of hi - 29), hi + lo is exactly
// representable and its bit pattern is hi's plus or minus K (the sum stays in
// hi's binade, except when hi is a power of two and lo pulls it below: that
// case, lo finer than the ulp, and non-normal inputs take one FP64 add).
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  const unsigned uh = __float_as_uint(hi), ul = __float_as_uint(lo);
  const int eh = (int)((uh >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu);
  if ((ul & 0x7fffffffu) == 0u) return f2d_exact(hi);
  const int sh = el - eh + 29;  // lo = +-Ml * 2^sh ulps of hi's double
  const bool opposite = ((uh ^ ul) >> 31) != 0u;
  if (eh >= 1 && eh <= 254 && el >= 1 && sh >= 0 && !(opposite && (uh & 0x7fffffu) == 0u)) {
    const long long H = __double_as_longlong(f2d_exact(hi));
    const long long K = (long long)((ul & 0x7fffffu) | 0x800000u) << sh;
    return __longlong_as_double(opposite ? H - K : H + K);
  }
  return f2d_exact(hi) + f2d_exact(lo);
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}
// Dekker's FastTwoSum (|a| >= |b| or a == 0).
__device__ __forceinline__ float fast_two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
  return s;
}

// (hi, lo) + v for a normalised pair and an FP32 v: TwoSum of the high
// words, the low word added to the error, renormalised by FastTwoSum.
__device__ __forceinline__ float2 df_add(float2 x, float v) {
  float e;
  const float s = two_sum(x.x, v, e);
  float lo;
  const float hi = fast_two_sum(s, __fadd_rn(e, x.y), lo);
  return make_float2(hi, lo);
}

// d - a xm - b x0 - c xp for double-float x, rounded to FP32: products of
// the high words exactly (TwoProd by FMA), summed with TwoSum; the low
// words' products and all rounding errors gathered in one FP32 term.
__device__ __forceinline__ float df_residual(float a, float b, float c, float d, float2 xm, float2 x0, float2 xp) {
  const float pb = __fmul_rn(b, x0.x), pa = __fmul_rn(a, xm.x), pc = __fmul_rn(c, xp.x);
  float t = -(fmaf(b, x0.x, -pb) + fmaf(a, xm.x, -pa) + fmaf(c, xp.x, -pc));
  float e;
  float s = two_sum(d, -pb, e);
  t += e;
  s = two_sum(s, -pa, e);
  t += e;
  s = two_sum(s, -pc, e);
  t += e;
  t = fmaf(-b, x0.y, t);
  t = fmaf(-a, xm.y, t);
  t = fmaf(-c, xp.y, t);
  return __fadd_rn(s, t);
}

}  // namespace tridi
