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

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace ttg
{

// IEEE bit patterns, on the device by intrinsic and on the host by memcpy
// (the conversions below are also compiled into a host test).
__host__ __device__ __forceinline__ unsigned long long dbits(double x)
{
#ifdef __CUDA_ARCH__
  return static_cast<unsigned long long>(__double_as_longlong(x));
#else
  unsigned long long u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}
__host__ __device__ __forceinline__ double dfrom_bits(unsigned long long u)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}
__host__ __device__ __forceinline__ unsigned fbits(float x)
{
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}
__host__ __device__ __forceinline__ float ffrom_bits(unsigned u)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

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
__host__ __device__ __forceinline__ df64 two_sum(float a, float b)
{
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64{s, e};
}

__host__ __device__ __forceinline__ df64 fast_two_sum(float a, float b)
{
  const float s = a + b;
  return df64{s, b - (s - a)};
}

// DWPlusDW (accurate version).
__host__ __device__ __forceinline__ df64 df_add(df64 a, df64 b)
{
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  float c = s.lo + t.hi;
  df64 v = fast_two_sum(s.hi, c);
  float w = t.lo + v.lo;
  return fast_two_sum(v.hi, w);
}

__host__ __device__ __forceinline__ df64 df_neg(df64 a) { return df64{-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

// DWTimesDW with FMA.
__host__ __device__ __forceinline__ df64 df_mul(df64 a, df64 b)
{
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// c + a*b in one pass: the product's error terms are folded into the sum.
__host__ __device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c)
{
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  df64 s = two_sum(c.hi, p);
  const float t = s.lo + (c.lo + e);
  return fast_two_sum(s.hi, t);
}

// ---------------------------------------------------------------------------
// FP64 <-> df64 conversions with a power-of-two scale, from the IEEE bit
// patterns on the integer and FP32 pipes.  df_from / df_to above take four
// and three instructions of the FP64 pipe per element (conversions and an
// add), and GB300's FP64 pipe retires 2 lanes per clock per SM against the
// FP32 pipes' 128: in the mixed path those conversions, not the df64
// arithmetic, would bound the step.
// ---------------------------------------------------------------------------

// Unbiased exponent of a power of two held in a double.
__host__ __device__ __forceinline__ int pow2_exponent(double s)
{
  return static_cast<int>((dbits(s) >> 52) & 0x7ff) - 1023;
}

// (hi, lo) with hi + lo = x * 2^k to 2^-48 relative: hi = x * 2^k rounded
// to 24 significand bits (nearest), lo = the remaining 29-bit signed
// remainder rounded to a float.  |x * 2^k| below 2^-126 flushes to a signed
// zero, and lo to zero below 2^-74 (both far under 2^-44 of the largest
// entry in every use, which scales that entry to [1, 2)); a non-finite x
// gives a non-finite hi.
__host__ __device__ __forceinline__ df64 df_split_pow2(double x, int k)
{
  const unsigned long long u = dbits(x);
  const unsigned sign = static_cast<unsigned>(u >> 32) & 0x80000000u;
  const int ex = static_cast<int>((u >> 52) & 0x7ff);
  const unsigned mhi = static_cast<unsigned>(u >> 29) & 0x7fffffu;  // leading 23 stored bits
  const unsigned rem = static_cast<unsigned>(u) & 0x1fffffffu;      // trailing 29 bits
  if (ex == 0x7ff)
    return df64{ffrom_bits(sign | 0x7f800000u | (((u << 12) != 0ull) ? 0x400000u : 0u)), 0.0f};
  const int e = ex - 1023 + k;
  if (ex == 0 || e < -126)
    return df64{ffrom_bits(sign), 0.0f};
  if (e > 127)
    return df64{ffrom_bits(sign | 0x7f800000u), 0.0f};
  // Round hi to nearest: a remainder of at least half an ulp carries into
  // hi (a carry out of the significand steps the exponent, as it should)
  // and leaves lo = remainder - 2^29 with the opposite sign.
  const unsigned up = rem >> 28;
  const float hi = ffrom_bits(sign | ((static_cast<unsigned>(e + 127) << 23) + mhi + up));
  const unsigned mag = up ? (0x20000000u - rem) : rem;  // |lo| / 2^(e-52), <= 2^28
  // mag as a float: two exact 15-bit halves (2^23 + n - 2^23), one rounding.
  const float m1 = ffrom_bits(0x4b000000u | (mag >> 15)) - 8388608.0f;
  const float m0 = ffrom_bits(0x4b000000u | (mag & 0x7fffu)) - 8388608.0f;
  const float mf = fmaf(m1, 32768.0f, m0);
  const float lo = (e >= -74) ? mf * ffrom_bits(static_cast<unsigned>(e - 52 + 127) << 23) : 0.0f;
  return df64{hi, ffrom_bits(fbits(lo) | (sign ^ (up << 31)))};
}

// f * 2^k as a double, exactly, for a normal float f (zero and subnormal f
// give a signed zero; inf and NaN stay so).
__host__ __device__ __forceinline__ double f32_to_f64_pow2(float f, int k)
{
  const unsigned b = fbits(f);
  const unsigned long long sign = static_cast<unsigned long long>(b & 0x80000000u) << 32;
  const int ex = static_cast<int>((b >> 23) & 0xffu);
  if (ex == 0xff)
    return dfrom_bits(sign | 0x7ff0000000000000ull | ((b & 0x7fffffu) ? 0x8000000000000ull : 0ull));
  const int e = ex - 127 + k;
  if (ex == 0 || e < -1022)
    return dfrom_bits(sign);
  if (e > 1023)
    return dfrom_bits(sign | 0x7ff0000000000000ull);
  return dfrom_bits(sign | (static_cast<unsigned long long>(e + 1023) << 52) |
                    (static_cast<unsigned long long>(b & 0x7fffffu) << 29));
}

// (hi + lo) * 2^k rounded to FP64: one add on the FP64 pipe.
__host__ __device__ __forceinline__ double df_join_pow2(df64 a, int k)
{
  return f32_to_f64_pow2(a.hi, k) + f32_to_f64_pow2(a.lo, k);
}

// 1 / b: the FP32 reciprocal of b.hi refined by one Newton step in df64,
// r = x + x (1 - b x) (Karp & Markstein, "High-precision division and square
// root", ACM TOMS 23(4), 1997): relative error ~2^-46.
__host__ __device__ __forceinline__ df64 df_recip(df64 b)
{
  const float x = 1.0f / b.hi;
  float e = fmaf(-b.hi, x, 1.0f);  // exact: b.hi x is within an ulp of 1
  e = fmaf(-b.lo, x, e);
  const float p = x * e;
  return fast_two_sum(x, p);
}

// sqrt(a), a > 0: y = sqrt(a.hi) (correctly rounded FP32) refined by one
// Newton step, s = y + (a - y^2) / (2 y) with the residual in double-float
// (Karp & Markstein, 1997): relative error ~2^-46.  a.hi <= 0 gives 0.
__host__ __device__ __forceinline__ df64 df_sqrt(df64 a)
{
  if (a.hi <= 0.0f)
    return df64{0.0f, 0.0f};
  const float y = sqrtf(a.hi);
  const float p = y * y;
  const float pe = fmaf(y, y, -p);
  const float d = ((a.hi - p) - pe) + a.lo;  // a.hi - p is exact (Sterbenz)
  return fast_two_sum(y, d / (y + y));
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
