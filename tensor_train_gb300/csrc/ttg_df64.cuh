// Double-float ("df64") arithmetic on the FP32 pipes, for the mixed path.
//
// A value is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// ~48 significant bits.  On GB300 the FP32 pipes are ~62x faster than the
// FP64 pipe, so the O(h c^2) Householder and contraction work of a sweep
// step runs in df64 and is rounded to FP64 once per step.  The algorithms are
// the classical error-free transformations: TwoSum (Knuth 1969), TwoProd via
// FMA, and the double-word arithmetic of Joldes, Muller & Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic"
// (ACM TOMS 2017), algorithms 6 (DWPlusDW) and 10 (DWTimesDW, FMA variant).
//
// Range: every matrix handed to these routines is first scaled by a power
// of two so that its largest entry is ~1 (exact in binary), which keeps all
// intermediate values far inside the FP32 exponent range.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ttg
{

struct df64
{
  float hi, lo;
};

__device__ __forceinline__ df64 df_from(double x)
{
  const float h = static_cast<float>(x);
  return df64{h, static_cast<float>(x - static_cast<double>(h))};
}

__device__ __forceinline__ double df_to(df64 a)
{
  return static_cast<double>(a.hi) + static_cast<double>(a.lo);
}

// s + e = a + b exactly (TwoSum).
__device__ __forceinline__ df64 two_sum(float a, float b)
{
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64{s, e};
}

__device__ __forceinline__ df64 fast_two_sum(float a, float b)
{
  const float s = a + b;
  return df64{s, b - (s - a)};
}

// DWPlusDW (accurate version).
__device__ __forceinline__ df64 df_add(df64 a, df64 b)
{
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  float c = s.lo + t.hi;
  df64 v = fast_two_sum(s.hi, c);
  float w = t.lo + v.lo;
  return fast_two_sum(v.hi, w);
}

__device__ __forceinline__ df64 df_neg(df64 a) { return df64{-a.hi, -a.lo}; }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

// DWTimesDW with FMA.
__device__ __forceinline__ df64 df_mul(df64 a, df64 b)
{
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// c + a*b in one pass: the product's error terms are folded into the sum.
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c)
{
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  df64 s = two_sum(c.hi, p);
  const float t = s.lo + (c.lo + e);
  return fast_two_sum(s.hi, t);
}

__device__ __forceinline__ df64 df_shfl_xor(df64 a, int o)
{
  return df64{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

__device__ __forceinline__ df64 df_warp_sum(df64 v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = df_add(v, df_shfl_xor(v, o));
  return v;
}

}  // namespace ttg
