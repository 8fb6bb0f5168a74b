// Blocked Householder (compact WY) building blocks for the per-TT sweep, in
// FP64 or df64 (E = double or df64), executed by all threads of one CTA.
//
// The reflectors are those of cta_householder_qr[_df]: H_j = I - tau_j v_j
// v_j^T with v_j(j) = 1 implicit and v_j(j+1:m) stored below the diagonal of
// column j.  A block of b consecutive reflectors j0 .. j0+b-1 is applied as
//   H_j0 ... H_{j0+b-1} = I - V T V^T            (LAPACK dlarft, forward,
//                                                  columnwise; Schreiber &
//                                                  Van Loan, SISC 1989)
// with V the m x b unit lower-trapezoidal block and T upper triangular, so
// a pass over the matrix handles b reflectors: W = V^T B, W = T' W,
// B -= V W.  The arithmetic is the same as one reflector at a time (the
// same products, summed in another order); the matrix is streamed 3 times
// per block instead of 3 times per reflector and the CTA meets a barrier a
// few times per block instead of twice per reflector.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "ttg_device.cuh"
#include "ttg_device_df.cuh"

namespace ttg
{
namespace
{

constexpr int kWyB = 8;             // reflectors per block
constexpr int kWyColChunk = 128;    // columns of B per pass (workspace kWyB x kWyColChunk)

template <class E>
struct WyOps;
template <>
struct WyOps<double>
{
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double one() { return 1.0; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double neg(double a) { return -a; }
  static __device__ __forceinline__ double warp_sum(double v) { return ttg::warp_sum(v); }
  static __device__ __forceinline__ double from(double x) { return x; }
  static __device__ __forceinline__ double to(double x) { return x; }
  static __device__ __forceinline__ double tiny() { return DBL_MIN; }
  static __device__ __forceinline__ double sum(double v, CtaShared& sh) { return cta_sum(v, sh); }
};
template <>
struct WyOps<df64>
{
  static __device__ __forceinline__ df64 zero() { return df64{0.0f, 0.0f}; }
  static __device__ __forceinline__ df64 one() { return df64{1.0f, 0.0f}; }
  static __device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) { return df_fma(a, b, c); }
  static __device__ __forceinline__ df64 mul(df64 a, df64 b) { return df_mul(a, b); }
  static __device__ __forceinline__ df64 add(df64 a, df64 b) { return df_add(a, b); }
  static __device__ __forceinline__ df64 neg(df64 a) { return df_neg(a); }
  static __device__ __forceinline__ df64 warp_sum(df64 v) { return df_warp_sum(v); }
  static __device__ __forceinline__ df64 from(double x) { return df_from(x); }
  static __device__ __forceinline__ double to(df64 x) { return df_to(x); }
  static __device__ __forceinline__ double tiny() { return 1.0e-36; }
  static __device__ __forceinline__ double sum(df64 v, CtaShared& sh) { return df_to(cta_sum_df(v, sh)); }
};

// V(r, i) of the block starting at reflector j0 (column j0 + i of A).
template <class E>
__device__ __forceinline__ E wy_v(const E* A, int64_t lda, int j0, int r, int i)
{
  const int d = j0 + i;
  if (r < d)
    return WyOps<E>::zero();
  if (r == d)
    return WyOps<E>::one();
  return A[r + static_cast<int64_t>(d) * lda];
}

// T (nb x nb, column-major, ld kWyB) of reflectors j0 .. j0+nb-1 over rows
// j0 .. m-1.  Ends with a barrier.
template <class E>
__device__ void wy_build_t(const E* A, int m, int j0, int nb, int64_t lda, const E* tau, E* T)
{
  using O = WyOps<E>;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // G(l, i) = v_l^T v_i for l < i, over rows from j0 + i (v_i is zero
  // above), kept above the diagonal of T until column i is formed.
  for (int pr = w; pr < nb * nb; pr += kWarps)
  {
    const int l = pr % nb, i = pr / nb;
    if (l >= i)
      continue;
    E acc = O::zero();
    for (int r = j0 + i + lane; r < m; r += 32)
      acc = O::fma(wy_v(A, lda, j0, r, l), wy_v(A, lda, j0, r, i), acc);
    acc = O::warp_sum(acc);
    if (lane == 0)
      T[l + i * kWyB] = acc;
  }
  __syncthreads();
  // T(i, i) = tau_i; T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i), column by
  // column (one thread: nb^3/6 products).
  if (threadIdx.x == 0)
  {
    for (int i = 0; i < nb; ++i)
    {
      const E t = tau[j0 + i];
      const E nt = O::neg(t);
      E z[kWyB];
      for (int l = 0; l < i; ++l)
        z[l] = O::mul(nt, T[l + i * kWyB]);
      for (int l = 0; l < i; ++l)
      {
        E acc = O::zero();
        for (int q = l; q < i; ++q)
          acc = O::fma(T[l + q * kWyB], z[q], acc);
        T[l + i * kWyB] = acc;
      }
      T[i + i * kWyB] = t;
      for (int l = i + 1; l < nb; ++l)
        T[l + i * kWyB] = O::zero();
    }
  }
  __syncthreads();
}

// B(j0:m, c0:c0+p) <- (I - V T' V^T) B(j0:m, c0:c0+p), T' = T (trans = false:
// the product H_j0 ... H_{j0+nb-1}) or T^T (trans = true: its transpose,
// H_{j0+nb-1} ... H_j0, as the factorisation applies them).  Wk: kWyB x
// kWyColChunk workspace.  Ends with a barrier.
template <class E>
__device__ void wy_apply(const E* A, int m, int j0, int nb, int64_t lda, const E* T, bool trans,
                         E* B, int64_t ldb, int c0, int p, E* Wk)
{
  using O = WyOps<E>;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int cb = 0; cb < p; cb += kWyColChunk)
  {
    const int pc = p - cb < kWyColChunk ? p - cb : kWyColChunk;
    // W = V^T B: one warp per column, lanes over rows, nb sums per lane.
    for (int q = w; q < pc; q += kWarps)
    {
      const E* y = B + static_cast<int64_t>(c0 + cb + q) * ldb;
      E acc[kWyB];
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
        acc[i] = O::zero();
      for (int r = j0 + lane; r < m; r += 32)
      {
        const E yr = y[r];
#pragma unroll
        for (int i = 0; i < kWyB; ++i)
          if (i < nb)
            acc[i] = O::fma(wy_v(A, lda, j0, r, i), yr, acc[i]);
      }
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
        if (i < nb)
        {
          const E s = O::warp_sum(acc[i]);
          if (lane == 0)
            Wk[i + q * kWyB] = s;
        }
    }
    __syncthreads();
    // W = T' W, one thread per column.
    for (int q = threadIdx.x; q < pc; q += blockDim.x)
    {
      E wv[kWyB], nv[kWyB];
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
        wv[i] = i < nb ? Wk[i + q * kWyB] : O::zero();
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
      {
        E acc = O::zero();
        if (i < nb)
        {
          if (!trans)
            for (int l = i; l < nb; ++l)  // (T w)_i = sum_{l >= i} T(i, l) w_l
              acc = O::fma(T[i + l * kWyB], wv[l], acc);
          else
            for (int l = 0; l <= i; ++l)  // (T^T w)_i = sum_{l <= i} T(l, i) w_l
              acc = O::fma(T[l + i * kWyB], wv[l], acc);
        }
        nv[i] = acc;
      }
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
        if (i < nb)
          Wk[i + q * kWyB] = nv[i];
    }
    __syncthreads();
    // B -= V W: lanes over rows; each lane keeps its row of V in registers
    // and runs over the chunk's columns.
    for (int r0 = j0 + w * 32; r0 < m; r0 += kWarps * 32)
    {
      const int r = r0 + lane;
      if (r >= m)
        continue;
      E v[kWyB];
#pragma unroll
      for (int i = 0; i < kWyB; ++i)
        v[i] = i < nb ? wy_v(A, lda, j0, r, i) : O::zero();
      for (int q = 0; q < pc; ++q)
      {
        E* yp = B + static_cast<int64_t>(c0 + cb + q) * ldb + r;
        E acc = O::zero();
#pragma unroll
        for (int i = 0; i < kWyB; ++i)
          if (i < nb)
            acc = O::fma(v[i], Wk[i + q * kWyB], acc);
        *yp = O::add(*yp, O::neg(acc));
      }
    }
    __syncthreads();
  }
}

// Columns j0 .. j0+nb-1 factored one reflector at a time (the arithmetic of
// cta_householder_qr[_df], with the update restricted to the panel).
template <class E>
__device__ void wy_panel(E* A, int m, int j0, int nb, int64_t lda, E* tau, CtaShared& sh)
{
  using O = WyOps<E>;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = j0; j < j0 + nb; ++j)
  {
    E* x = A + static_cast<int64_t>(j) * lda + j;
    const int len = m - j;
    E part = O::zero();
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      part = O::fma(x[i], x[i], part);
    const double tail2 = O::sum(part, sh);
    const double x0 = O::to(x[0]);
    double beta, t, inv;
    if (tail2 <= O::tiny())
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
    const E invd = O::from(inv);
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      x[i] = (t == 0.0) ? O::zero() : O::mul(x[i], invd);
    __syncthreads();
    const E td = O::from(t);
    if (threadIdx.x == 0)
    {
      x[0] = O::from(beta);
      tau[j] = td;
    }
    if (t != 0.0)
      for (int col = j + 1 + w; col < j0 + nb; col += kWarps)
      {
        E* y = A + static_cast<int64_t>(col) * lda + j;
        E dot = (lane == 0) ? y[0] : O::zero();
        for (int i = 1 + lane; i < len; i += 32)
          dot = O::fma(x[i], y[i], dot);
        dot = O::mul(O::warp_sum(dot), td);
        const E nd = O::neg(dot);
        if (lane == 0)
          y[0] = O::add(y[0], nd);
        for (int i = 1 + lane; i < len; i += 32)
          y[i] = O::fma(nd, x[i], y[i]);
      }
    __syncthreads();
  }
}

// Householder QR of A (m x c, column-major, lda), in place, blocked: the
// layout and conventions of cta_householder_qr (R in the upper triangle,
// reflector tails below it, tau[j]).  T and the column-block workspace live
// in the CTA's shared GEMM buffers.
template <class E>
__device__ __noinline__ void cta_qr_wy(E* A, int m, int c, int64_t lda, E* tau, CtaShared& sh)
{
  E* T = reinterpret_cast<E*>(&sh.gemm_b[0][0]);
  E* Wk = reinterpret_cast<E*>(&sh.gemm_a[0][0]);
  const int k = m < c ? m : c;
  for (int j0 = 0; j0 < k; j0 += kWyB)
  {
    const int nb = k - j0 < kWyB ? k - j0 : kWyB;
    wy_panel<E>(A, m, j0, nb, lda, tau, sh);
    if (j0 + nb < c)
    {
      wy_build_t<E>(A, m, j0, nb, lda, tau, T);
      wy_apply<E>(A, m, j0, nb, lda, T, true, A, lda, j0 + nb, c - j0 - nb, Wk);
    }
  }
}

// Q (m x k, column-major, ldq) = H_0 ... H_{k-1} [I; 0] from the reflectors
// in A (a separate buffer; A is only read).  Block by block from the last:
// a block starting at j0 leaves columns < j0 of [I; 0] unchanged.
template <class E>
__device__ __noinline__ void cta_form_q_wy(const E* A, int m, int k, int64_t lda, const E* tau,
                                           E* Q, int64_t ldq, CtaShared& sh)
{
  using O = WyOps<E>;
  E* T = reinterpret_cast<E*>(&sh.gemm_b[0][0]);
  E* Wk = reinterpret_cast<E*>(&sh.gemm_a[0][0]);
  const int64_t total = static_cast<int64_t>(m) * k;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int64_t i = t % m, j = t / m;
    Q[i + j * ldq] = i == j ? O::one() : O::zero();
  }
  __syncthreads();
  if (k < 1)
    return;
  for (int j0 = ((k - 1) / kWyB) * kWyB; j0 >= 0; j0 -= kWyB)
  {
    const int nb = k - j0 < kWyB ? k - j0 : kWyB;
    wy_build_t<E>(A, m, j0, nb, lda, tau, T);
    wy_apply<E>(A, m, j0, nb, lda, T, false, Q, ldq, j0, k - j0, Wk);
  }
}

// B (m x p, column-major, ldb) <- H_0 ... H_{kref-1} B.
template <class E>
__device__ __noinline__ void cta_apply_q_wy(const E* A, int m, int kref, int64_t lda,
                                            const E* tau, E* B, int p, int64_t ldb, CtaShared& sh)
{
  E* T = reinterpret_cast<E*>(&sh.gemm_b[0][0]);
  E* Wk = reinterpret_cast<E*>(&sh.gemm_a[0][0]);
  if (kref < 1 || p < 1)
    return;
  for (int j0 = ((kref - 1) / kWyB) * kWyB; j0 >= 0; j0 -= kWyB)
  {
    const int nb = kref - j0 < kWyB ? kref - j0 : kWyB;
    wy_build_t<E>(A, m, j0, nb, lda, tau, T);
    wy_apply<E>(A, m, j0, nb, lda, T, false, B, ldb, 0, p, Wk);
  }
}

}  // namespace
}  // namespace ttg
