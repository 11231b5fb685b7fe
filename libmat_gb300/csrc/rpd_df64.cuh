// rpd_df64.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// about 48 significant bits.  GB300's FP64 rate is a small fraction of its
// FP32 rate, so the FP64-accurate vertex reconstruction runs in double-float
// on the FP32 pipe.  The building blocks are the published error-free
// transformations -- Knuth's TwoSum, Dekker's Fast2Sum, and TwoProd with a
// fused multiply-add -- and the double-word sum / product algorithms of
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic" (ACM TOMS 44(2), 2017):
// AccurateDWPlusDW (relative error <= 3u^2 + 13u^3) and DWTimesDW with FMA
// (<= 5u^2), u = 2^-24.  The translation unit must not contract a*b+c into
// FMA behind the code's back (compiled with -fmad=false).
#pragma once

namespace rpd {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float h, float l) {
  df r;
  r.hi = h;
  r.lo = l;
  return r;
}

__device__ __forceinline__ df df_from_double(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return df_make(h, l);
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return df_make(s, e);
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return df_make(s, e);
}

__device__ __forceinline__ df two_prod(float a, float b) {
  float p = a * b;
  float e = __fmaf_rn(a, b, -p);
  return df_make(p, e);
}

__device__ __forceinline__ df df_add(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  df t = two_sum(x.lo, y.lo);
  float c = s.lo + t.hi;
  df v = fast_two_sum(s.hi, c);
  float w = t.lo + v.lo;
  return fast_two_sum(v.hi, w);
}

__device__ __forceinline__ df df_neg(df x) { return df_make(-x.hi, -x.lo); }

__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

// SloppyDWPlusDW (Joldes, Muller, Popescu, Alg. 5): one TwoSum instead of
// two.  Its relative error is bounded only for operands of one sign, but its
// absolute error stays below about 3u^2 (|x| + |y|) -- which is what the
// forward error analysis of a determinant or a dot product needs (errors
// relative to the magnitudes of the summed products).  Used by the geometry.
__device__ __forceinline__ df df_add_s(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  float v = x.lo + y.lo;
  float w = s.lo + v;
  return fast_two_sum(s.hi, w);
}
__device__ __forceinline__ df df_sub_s(df x, df y) { return df_add_s(x, df_neg(y)); }

__device__ __forceinline__ df df_mul(df x, df y) {
  df c = two_prod(x.hi, y.hi);
  float t = x.hi * y.lo;
  t = __fmaf_rn(x.lo, y.hi, t);
  float l = c.lo + t;
  return fast_two_sum(c.hi, l);
}

// reciprocal: q = 1/y.hi refined by one Newton step on the double-word
// residual 1 - y*q (relative error about u^2)
__device__ __forceinline__ df df_recip(df y) {
  float q = 1.0f / y.hi;
  df p = df_mul(y, df_make(q, 0.f));
  df r = df_sub(df_make(1.0f, 0.f), p);
  float q2 = r.hi * q;
  return fast_two_sum(q, q2);
}

}  // namespace rpd
