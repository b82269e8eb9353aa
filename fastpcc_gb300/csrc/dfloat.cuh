// Double-float complex arithmetic on the FP32 pipes.
//
// A value is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), which
// carries about 44-48 bits of significand.  The GB300 issues FP32 operations at
// tens of times its FP64 rate, so transforms that need more than FP32 precision
// (analytic signals of windows with gaps) run faster this way than in FP64.
// The building blocks are Knuth's two-sum, the fast two-sum of Dekker, and the
// product error term from a fused multiply-add (the exact a*b - round(a*b));
// every step uses the _rn intrinsics so the compiler neither contracts nor
// reorders them.  Complex values are float4 {re.hi, im.hi, re.lo, im.lo}.
#pragma once

#include <cuda_runtime.h>

namespace fpcc {

struct df {
  float hi, lo;
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// s + e = a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ df df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// Dekker's addition: the high parts' two-sum, the low parts added to its
// error, one fast two-sum (11 operations instead of the 20 of the form that
// also two-sums the low parts).  Its error is bounded relative to the operands'
// magnitudes rather than to the sum, which is the bound a transform's error
// analysis uses: in a float32 emulation of 4096-point transforms against FP64
// both forms gave 6e-15 of the norm, and 2e-12 relative on analytic-signal
// samples inside a run of zeros.
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = df_two_sum(a.hi, b.hi);
  const float e = __fadd_rn(__fadd_rn(s.lo, a.lo), b.lo);
  return df_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

// scaling by a power of two is exact
__device__ __forceinline__ df df_scale2(df a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }

__device__ __forceinline__ df df_from_double(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ float df_to_float(df a) { return __fadd_rn(a.hi, a.lo); }

// complex
__device__ __forceinline__ df df_re(float4 z) { return {z.x, z.z}; }
__device__ __forceinline__ df df_im(float4 z) { return {z.y, z.w}; }
__device__ __forceinline__ float4 dfc(df re, df im) { return make_float4(re.hi, im.hi, re.lo, im.lo); }

__device__ __forceinline__ float4 dfc_add(float4 a, float4 b) {
  return dfc(df_add(df_re(a), df_re(b)), df_add(df_im(a), df_im(b)));
}
__device__ __forceinline__ float4 dfc_sub(float4 a, float4 b) {
  return dfc(df_sub(df_re(a), df_re(b)), df_sub(df_im(a), df_im(b)));
}
__device__ __forceinline__ float4 dfc_mul(float4 a, float4 b) {
  const df ar = df_re(a), ai = df_im(a), br = df_re(b), bi = df_im(b);
  return dfc(df_sub(df_mul(ar, br), df_mul(ai, bi)), df_add(df_mul(ar, bi), df_mul(ai, br)));
}
// a * conj(b) when conj, else a * b
__device__ __forceinline__ float4 dfc_mul_c(float4 a, float4 b, bool conj) {
  if (conj) b = make_float4(b.x, -b.y, b.z, -b.w);
  return dfc_mul(a, b);
}
// a * s for a real double-float s
__device__ __forceinline__ float4 dfc_mul_r(float4 a, df s) { return dfc(df_mul(df_re(a), s), df_mul(df_im(a), s)); }
// i * a
__device__ __forceinline__ float4 dfc_muli(float4 a) { return make_float4(-a.y, a.x, -a.w, a.z); }
__device__ __forceinline__ float4 dfc_scale2(float4 a, float p2) {
  return make_float4(__fmul_rn(a.x, p2), __fmul_rn(a.y, p2), __fmul_rn(a.z, p2), __fmul_rn(a.w, p2));
}

}  // namespace fpcc
