// Double-float arithmetic shared by the mixed-precision kernels.
#pragma once
#include "eif_internal.cuh"

namespace eifdf {

// Double-float arithmetic for the mixed-precision form: a value is the
// unevaluated sum hi + lo of two floats (about 48 significant bits), combined
// with the error-free transformations of Knuth (TwoSum), Dekker (Fast2Sum) and
// an FMA-based product (Ogita, Rump and Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26, 2005). Only the FP32 pipe is used.
struct DF { float hi, lo; };

__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF fast_sum(float a, float b) {  // requires |a| >= |b| or a == 0
  const float s = a + b;
  return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = two_sum(x.hi, y.hi);
  const DF t = two_sum(x.lo, y.lo);
  s = fast_sum(s.hi, s.lo + t.hi);
  return fast_sum(s.hi, s.lo + t.lo);
}
__device__ __forceinline__ DF df_neg(DF x) { return DF{-x.hi, -x.lo}; }
__device__ __forceinline__ DF df_sub(DF x, DF y) { return df_add(x, df_neg(y)); }
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  return fast_sum(p, e);
}
__device__ __forceinline__ DF df_scale(DF x, float pow2) { return DF{x.hi * pow2, x.lo * pow2}; }
__device__ __forceinline__ DF df_of(double v) {
  const float2 t = eifd::split(v);
  return fast_sum(t.x, t.y);
}
__device__ __forceinline__ double df_to_double(DF x) { return eifd::f2d(x.hi) + eifd::f2d(x.lo); }

// Transforms use the "sloppy" double-float sum (exact sum of the leading parts,
// the trailing parts added in single precision): its error is below about
// 2^-47 (|x| + |y|), the norm-wise bound that an FFT's error analysis needs, at
// about half the operations of df_add.
__device__ __forceinline__ DF df_add_nw(DF x, DF y) {
  const DF s = two_sum(x.hi, y.hi);
  return fast_sum(s.hi, s.lo + (x.lo + y.lo));
}

}  // namespace eifdf
