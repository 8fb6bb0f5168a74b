// Blocked (compact WY) Householder QR, Q formation and Q application in
// df64, for matrices that live in global memory (too large for the CTA's
// shared staging).  Same reflectors, same convention and the same products
// as cta_householder_qr_df / cta_form_q_df / cta_apply_q_df, summed in
// another order.
//
// A block of kWyB consecutive reflectors j0 .. j0+nb-1 acts as
//   H_j0 ... H_{j0+nb-1} = I - V T V^T      (forward, columnwise: LAPACK
//                                            dlarft; Schreiber & Van Loan,
//                                            SISC 10(1), 1989)
// with V the unit lower-trapezoidal (m - j0) x nb block of the reflector
// vectors and T upper triangular.  The one-reflector-at-a-time routines
// stream the trailing matrix from L2 three times per reflector; here the
// panel is factored in shared memory and the trailing matrix is streamed
// three times per block (W = V^T B, W <- T' W, B -= V W), with V staged in
// shared memory as an explicit column-major block (zeros above its unit
// diagonal, zero columns past nb) so the inner loops carry no branches and
// lanes read consecutive rows.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ttg_device.cuh"
#include "ttg_device_df.cuh"

namespace ttg
{
namespace
{

constexpr int kWyB = 8;  // reflectors per block

// Shared staging the blocked routines need for m rows (in doubles).
__device__ __forceinline__ int64_t wy_stage_need(int m)
{
  return static_cast<int64_t>(m) * kWyB;
}

// T (kWyB x kWyB, column-major, zero outside the leading nb x nb upper
// triangle) of the explicit block P (hp x kWyB, column-major, ld hp) and
// its scales tau[0..nb).  Ends with a barrier.
__device__ void wy_build_t_df(const df64* P, int hp, int nb, const df64* tau, df64* T)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < kWyB * kWyB; t += blockDim.x)
    T[t] = df64{0.0f, 0.0f};
  __syncthreads();
  // G(l, i) = v_l^T v_i for l < i, held above the diagonal of T.
  for (int pr = w; pr < kWyB * kWyB; pr += kWarps)
  {
    const int l = pr % kWyB, i = pr / kWyB;
    if (l >= i || i >= nb)
      continue;
    df64 acc{0.0f, 0.0f};
    for (int r = i + lane; r < hp; r += 32)  // v_i is zero above row i
      acc = df_fma(P[r + static_cast<int64_t>(l) * hp], P[r + static_cast<int64_t>(i) * hp], acc);
    acc = df_warp_sum(acc);
    if (lane == 0)
      T[l + i * kWyB] = acc;
  }
  __syncthreads();
  // T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i), T(i, i) = tau_i: column by
  // column on warp 0, lane l forming row l.
  if (w == 0)
  {
    for (int i = 0; i < nb; ++i)
    {
      const df64 nt = df_neg(tau[i]);
      df64 acc{0.0f, 0.0f};
      if (lane < i)
        for (int q = lane; q < i; ++q)
          acc = df_fma(T[lane + q * kWyB], df_mul(nt, T[q + i * kWyB]), acc);
      __syncwarp();
      if (lane < i)
        T[lane + i * kWyB] = acc;
      if (lane == 0)
        T[i + i * kWyB] = tau[i];
      __syncwarp();
    }
  }
  __syncthreads();
}

// B(0:hp, 0:ncols) <- (I - V T' V^T) B, T' = T^T (kTrans: the product
// H_{j0+nb-1} ... H_j0, as the factorisation applies the block) or T (the
// product H_j0 ... H_{j0+nb-1}).  B points at the block's first row,
// column stride ldb.  A group of hh_group(hp) lanes per column of B.  Ends
// with a barrier.
template <bool kTrans>
__device__ __noinline__ void wy_apply_df(const df64* P, int hp, const df64* T, df64* B, int64_t ldb,
                                         int ncols)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // G lanes per column (hh_group), 32 / G columns in flight per warp; the
  // loop bound is uniform over the warp (the group sums need every lane).
  const int G = hh_group(hp), gpw = 32 / G, gl = lane & (G - 1), gbase = lane & ~(G - 1);
  const int li = gl & (kWyB - 1);
  for (int cb = w * gpw; cb < ncols; cb += kWarps * gpw)
  {
    const int q = cb + lane / G;
    const bool act = q < ncols;
    df64* y = B + static_cast<int64_t>(act ? q : cb) * ldb;
    df64 acc[kWyB];
#pragma unroll
    for (int i = 0; i < kWyB; ++i)
      acc[i] = df64{0.0f, 0.0f};
    if (act)
      for (int r = gl; r < hp; r += G)
      {
        const df64 a = y[r];
#pragma unroll
        for (int i = 0; i < kWyB; ++i)
          acc[i] = df_fma(P[r + static_cast<int64_t>(i) * hp], a, acc[i]);
      }
#pragma unroll
    for (int i = 0; i < kWyB; ++i)
      acc[i] = df_group_sum(acc[i], G);  // W = V^T y on every lane of the group
    // Lane li of the group forms (T' W)_li; the group gathers all kWyB.
    df64 wp{0.0f, 0.0f};
#pragma unroll
    for (int l = 0; l < kWyB; ++l)
      wp = df_fma(kTrans ? T[l + li * kWyB] : T[li + l * kWyB], acc[l], wp);
#pragma unroll
    for (int i = 0; i < kWyB; ++i)
      acc[i] = df_neg(df64{__shfl_sync(0xffffffffu, wp.hi, gbase + i),
                           __shfl_sync(0xffffffffu, wp.lo, gbase + i)});
    if (act)
      for (int r = gl; r < hp; r += G)
      {
        df64 a = y[r];
#pragma unroll
        for (int i = 0; i < kWyB; ++i)
          a = df_fma(acc[i], P[r + static_cast<int64_t>(i) * hp], a);
        y[r] = a;
      }
  }
  __syncthreads();
}

// P (hp x kWyB, ld hp) <- the explicit V of the block of nb reflectors whose
// vectors lie below the diagonal of A(j0:, j0:j0+nb): zero above the unit
// diagonal, zero columns past nb.  Ends with a barrier.
__device__ void wy_stage_v_df(const df64* A, int64_t ld, int j0, int hp, int nb, df64* P)
{
  const int64_t total = static_cast<int64_t>(hp) * kWyB;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int r = static_cast<int>(t % hp), i = static_cast<int>(t / hp);
    df64 v{0.0f, 0.0f};
    if (i < nb)
      v = r > i ? A[(j0 + r) + static_cast<int64_t>(j0 + i) * ld] : (r == i ? df64{1.0f, 0.0f} : v);
    P[t] = v;
  }
  __syncthreads();
}

// Householder QR of A (m x c, column-major, ld) in place, as
// cta_householder_qr_df, in blocks of kWyB reflectors.  stage: shared
// memory for wy_stage_need(m) doubles; T: kWyB^2 df64 in shared memory.
__device__ __noinline__ void cta_householder_qr_df_wy(df64* A, int m, int c, int64_t ld, df64* tau,
                                                      df64* stage, df64* T, CtaShared& sh)
{
  const int k = m < c ? m : c;
  for (int j0 = 0; j0 < k; j0 += kWyB)
  {
    const int nb = k - j0 < kWyB ? k - j0 : kWyB;
    const int hp = m - j0;
    df64* P = stage;
    // The panel A(j0:m, j0:j0+nb) into shared memory, factored there.
    const int64_t pn = static_cast<int64_t>(hp) * nb;
    for (int64_t t = threadIdx.x; t < pn; t += blockDim.x)
    {
      const int r = static_cast<int>(t % hp), i = static_cast<int>(t / hp);
      P[t] = A[(j0 + r) + static_cast<int64_t>(j0 + i) * ld];
    }
    __syncthreads();
    cta_householder_qr_df(P, hp, nb, hp, tau + j0, sh);
    // R block and reflector vectors back to A; P becomes the explicit V.
    for (int64_t t = threadIdx.x; t < pn; t += blockDim.x)
    {
      const int r = static_cast<int>(t % hp), i = static_cast<int>(t / hp);
      A[(j0 + r) + static_cast<int64_t>(j0 + i) * ld] = P[t];
    }
    __syncthreads();
    if (j0 + nb >= c)
      break;
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(hp) * kWyB; t += blockDim.x)
    {
      const int r = static_cast<int>(t % hp), i = static_cast<int>(t / hp);
      if (i >= nb || r <= i)
        P[t] = (i < nb && r == i) ? df64{1.0f, 0.0f} : df64{0.0f, 0.0f};
    }
    __syncthreads();
    wy_build_t_df(P, hp, nb, tau + j0, T);
    wy_apply_df<true>(P, hp, T, A + j0 + static_cast<int64_t>(j0 + nb) * ld, ld, c - j0 - nb);
  }
}

// Thin Q (m x k) in place from the reflectors of cta_householder_qr_df_wy
// (or cta_householder_qr_df), as cta_form_q_df: blocks from the last, each
// applied to the columns already formed, then its own columns formed in
// shared memory (dorgqr order).
__device__ __noinline__ void cta_form_q_df_wy(df64* A, int m, int k, int64_t ld, const df64* tau,
                                              df64* stage, df64* T)
{
  for (int j0 = ((k - 1) / kWyB) * kWyB; j0 >= 0; j0 -= kWyB)
  {
    const int nb = k - j0 < kWyB ? k - j0 : kWyB;
    const int hp = m - j0;
    df64* P = stage;
    wy_stage_v_df(A, ld, j0, hp, nb, P);
    if (j0 + nb < k)
    {
      wy_build_t_df(P, hp, nb, tau + j0, T);
      wy_apply_df<false>(P, hp, T, A + j0 + static_cast<int64_t>(j0 + nb) * ld, ld, k - j0 - nb);
    }
    cta_form_q_df(P, hp, nb, hp, tau + j0);
    // The block's columns: rows j0.. from P, rows above j0 zero.
    const int64_t total = static_cast<int64_t>(m) * nb;
    for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
    {
      const int r = static_cast<int>(t % m), i = static_cast<int>(t / m);
      A[r + static_cast<int64_t>(j0 + i) * ld] =
        r >= j0 ? P[(r - j0) + static_cast<int64_t>(i) * hp] : df64{0.0f, 0.0f};
    }
    __syncthreads();
  }
}

// B (m x p, column-major df64, ldb) <- H_0 ... H_{kref-1} B, as
// cta_apply_q_df, one block pass at a time from the last block.
__device__ __noinline__ void cta_apply_q_df_wy(const df64* A, int m, int kref, int64_t lda,
                                               const df64* tau, df64* B, int p, int64_t ldb,
                                               df64* stage, df64* T)
{
  for (int j0 = ((kref - 1) / kWyB) * kWyB; j0 >= 0; j0 -= kWyB)
  {
    const int nb = kref - j0 < kWyB ? kref - j0 : kWyB;
    const int hp = m - j0;
    df64* P = stage;
    wy_stage_v_df(A, lda, j0, hp, nb, P);
    wy_build_t_df(P, hp, nb, tau + j0, T);
    wy_apply_df<false>(P, hp, T, B + j0, ldb, p);
  }
}

}  // namespace
}  // namespace ttg
