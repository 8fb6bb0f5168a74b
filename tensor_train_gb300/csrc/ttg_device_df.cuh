// CTA-level df64 counterparts of the Householder QR, Q formation/application
// and GEMM in ttg_device.cuh, used by the mixed path.  Same algorithms, same
// reflector convention; arithmetic on the FP32 pipes (ttg_df64.cuh).  Inputs
// and outputs stay FP64 in memory; a matrix is split into (hi, lo) pairs
// once, after scaling by a power of two (exact) so that its largest entry is
// in [1, 2).
#pragma once

#include "ttg_device.cuh"
#include "ttg_df64.cuh"

namespace ttg
{

// Sum over the CTA in df64; every thread gets the same value.
__device__ df64 cta_sum_df(df64 v, CtaShared& sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = df_warp_sum(v);
  __syncthreads();
  if (lane == 0)
    reinterpret_cast<df64*>(sh.red)[w] = v;
  __syncthreads();
  df64 t{0.0f, 0.0f};
#pragma unroll
  for (int i = 0; i < kWarps; ++i)
    t = df_add(t, reinterpret_cast<const df64*>(sh.red)[i]);
  return t;
}

// Largest |x| over an (m x n) view, exactly, via the bit patterns (integer
// max on the absolute value's bits orders like the value).  Returns the
// power of two 2^e with 2^e <= max < 2^(e+1) (1.0 for an all-zero block).
__device__ double cta_pow2_of_max(View X, int64_t m, int64_t n, CtaShared& sh)
{
  unsigned long long mx = 0ull;
  const int64_t total = m * n;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const unsigned long long b =
      static_cast<unsigned long long>(__double_as_longlong(X(t % m, t / m))) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = y > mx ? y : mx;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0)
    reinterpret_cast<unsigned long long*>(sh.red)[threadIdx.x >> 5] = mx;
  __syncthreads();
  unsigned long long all = 0ull;
#pragma unroll
  for (int i = 0; i < kWarps; ++i)
  {
    const unsigned long long y = reinterpret_cast<const unsigned long long*>(sh.red)[i];
    all = y > all ? y : all;
  }
  __syncthreads();
  const int ex = static_cast<int>((all >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff)
    return 1.0;  // zero/subnormal block, or non-finite (caught by the NaN checks)
  return __longlong_as_double(static_cast<long long>(ex) << 52);
}

// W (df64, column-major m x n, ld) = split(X / scale).
__device__ void cta_split_to_df(df64* W, int64_t ld, View X, int64_t m, int64_t n, double inv_scale)
{
  const int64_t total = m * n;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int64_t i = t % m, j = t / m;
    W[i + j * ld] = df_from(X(i, j) * inv_scale);
  }
}

// Householder QR in df64, in place (see cta_householder_qr for the layout
// and convention).  tau is kept in df64.
__device__ void cta_householder_qr_df(df64* A, int m, int c, int64_t ld, df64* tau, CtaShared& sh)
{
  const int k = m < c ? m : c;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < k; ++j)
  {
    df64* x = A + j * ld + j;
    const int len = m - j;
    df64 part{0.0f, 0.0f};
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      part = df_fma(x[i], x[i], part);
    const double tail2 = df_to(cta_sum_df(part, sh));
    const df64 x0d = x[0];
    const double x0 = df_to(x0d);
    double beta, t, inv;
    if (tail2 <= 1.0e-36)
    {
      t = 0.0;
      beta = x0;
      inv = 0.0;
    }
    else
    {
      beta = sqrt(x0 * x0 + tail2);
      if (x0 >= 0.0)
        beta = -beta;
      inv = 1.0 / (x0 - beta);
      t = (beta - x0) / beta;
    }
    const df64 invd = df_from(inv);
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      x[i] = (t == 0.0) ? df64{0.0f, 0.0f} : df_mul(x[i], invd);
    __syncthreads();
    const df64 td = df_from(t);
    if (threadIdx.x == 0)
    {
      x[0] = df_from(beta);
      tau[j] = td;
    }
    if (t != 0.0)
    {
      for (int col = j + 1 + w; col < c; col += kWarps)
      {
        df64* y = A + col * ld + j;
        df64 dot = (lane == 0) ? y[0] : df64{0.0f, 0.0f};
        for (int i = 1 + lane; i < len; i += 32)
          dot = df_fma(x[i], y[i], dot);
        dot = df_mul(df_warp_sum(dot), td);
        const df64 nd = df_neg(dot);
        if (lane == 0)
          y[0] = df_add(y[0], nd);
        for (int i = 1 + lane; i < len; i += 32)
          y[i] = df_fma(nd, x[i], y[i]);
      }
    }
    __syncthreads();
  }
}

// R (k x c, column-major, FP64, ld k) = upper triangle of A, times scale.
__device__ void cta_extract_r_df(double* R, const df64* A, int k, int c, int64_t ld, double scale)
{
  const int64_t total = static_cast<int64_t>(k) * c;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int i = static_cast<int>(t % k), j = static_cast<int>(t / k);
    R[t] = (i <= j) ? df_to(A[i + j * ld]) * scale : 0.0;
  }
  __syncthreads();
}

// Thin Q (m x k) in place, df64 (dorg2r order, as cta_form_q).
__device__ void cta_form_q_df(df64* A, int m, int k, int64_t ld, const df64* tau)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = k - 1; j >= 0; --j)
  {
    df64* v = A + j * ld + j;
    const df64 t = tau[j];
    const int len = m - j;
    if (t.hi != 0.0f)
    {
      for (int col = j + 1 + w; col < k; col += kWarps)
      {
        df64* y = A + col * ld + j;
        df64 dot = (lane == 0) ? y[0] : df64{0.0f, 0.0f};
        for (int i = 1 + lane; i < len; i += 32)
          dot = df_fma(v[i], y[i], dot);
        dot = df_mul(df_warp_sum(dot), t);
        const df64 nd = df_neg(dot);
        if (lane == 0)
          y[0] = df_add(y[0], nd);
        for (int i = 1 + lane; i < len; i += 32)
          y[i] = df_fma(nd, v[i], y[i]);
      }
    }
    __syncthreads();
    const df64 nt = df_neg(t);
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      v[i] = df_mul(v[i], nt);
    if (threadIdx.x == 0)
      v[0] = df_add(df64{1.0f, 0.0f}, nt);
    for (int i = threadIdx.x; i < j; i += blockDim.x)
      A[j * ld + i] = df64{0.0f, 0.0f};
    __syncthreads();
  }
}

// B (m x p, column-major df64, ldb) <- H_0 ... H_{kref-1} B.
__device__ void cta_apply_q_df(const df64* A, int m, int kref, int64_t lda, const df64* tau,
                               df64* B, int p, int64_t ldb)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = kref - 1; j >= 0; --j)
  {
    const df64 t = tau[j];
    if (t.hi == 0.0f)
      continue;
    const df64* v = A + j * lda + j;
    const int len = m - j;
    for (int col = w; col < p; col += kWarps)
    {
      df64* y = B + col * ldb + j;
      df64 dot = (lane == 0) ? y[0] : df64{0.0f, 0.0f};
      for (int i = 1 + lane; i < len; i += 32)
        dot = df_fma(v[i], y[i], dot);
      dot = df_mul(df_warp_sum(dot), t);
      const df64 nd = df_neg(dot);
      if (lane == 0)
        y[0] = df_add(y[0], nd);
      for (int i = 1 + lane; i < len; i += 32)
        y[i] = df_fma(nd, v[i], y[i]);
    }
    __syncthreads();
  }
}

// C(i, j) = sum_p A(i, p) B(p, j) in df64 (FP64 in, FP64 out).  A and B are
// scaled by powers of two (exact) so the split never leaves FP32 range.
// 64x64 output tiles, 16-deep k slabs in shared memory (the df64 slabs reuse
// the CtaShared GEMM buffers, one df64 per double slot), 4x4 per thread.
__device__ void cta_gemm_df(int M, int N, int K, View A, View B, double* C, int64_t c_rs,
                            int64_t c_cs, CtaShared& sh)
{
  const double sa = cta_pow2_of_max(A, M, K, sh);
  const double sb = cta_pow2_of_max(B, K, N, sh);
  const double isa = 1.0 / sa, isb = 1.0 / sb, scale = sa * sb;
  df64(*as)[64 + 1] = reinterpret_cast<df64(*)[64 + 1]>(sh.gemm_a);
  df64(*bs)[64 + 1] = reinterpret_cast<df64(*)[64 + 1]>(sh.gemm_b);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int i0 = 0; i0 < M; i0 += 64)
    for (int j0 = 0; j0 < N; j0 += 64)
    {
      df64 acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          acc[a][b] = df64{0.0f, 0.0f};
      for (int p0 = 0; p0 < K; p0 += 16)
      {
        __syncthreads();
        for (int t = threadIdx.x; t < 16 * 64; t += blockDim.x)
        {
          const int kk = t / 64, ii = t % 64;
          const int gi = i0 + ii, gp = p0 + kk, gj = j0 + ii;
          as[kk][ii] = (gi < M && gp < K) ? df_from(A(gi, gp) * isa) : df64{0.0f, 0.0f};
          bs[kk][ii] = (gp < K && gj < N) ? df_from(B(gp, gj) * isb) : df64{0.0f, 0.0f};
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; ++kk)
        {
          df64 av[4], bv[4];
#pragma unroll
          for (int a = 0; a < 4; ++a)
            av[a] = as[kk][ty + 16 * a];
#pragma unroll
          for (int b = 0; b < 4; ++b)
            bv[b] = bs[kk][tx + 16 * b];
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
              acc[a][b] = df_fma(av[a], bv[b], acc[a][b]);
        }
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
        {
          const int gi = i0 + ty + 16 * a, gj = j0 + tx + 16 * b;
          if (gi < M && gj < N)
            C[gi * c_rs + gj * c_cs] = df_to(acc[a][b]) * scale;
        }
    }
  __syncthreads();
}

}  // namespace ttg
