// CTA-level FP64 building blocks of the TT sweep kernels (sm_103a).
//
// Every routine here is executed by all threads of one CTA (kThreads) and
// works on matrices in global memory (the per-CTA scratch slab and the core
// slots, L2-resident for the shapes of the rounding workloads).  Each call
// ends with a __syncthreads(), so results are visible to the whole CTA.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "ttg_gemm_live.h"

namespace ttg
{
// Internal linkage: every translation unit that includes this header gets
// its own copy of these device functions.
namespace
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// FP64 Jacobi stops after a sweep whose largest relative rotation is below
// this (the following sweep's would be ~1e-20).
constexpr double kJacobiStopRel = 1e-10;

// Column-major / row-major strided view: element (i, j) at p[i*rs + j*cs].
struct View
{
  const double* p;
  int64_t rs, cs;
  __device__ double operator()(int64_t i, int64_t j) const { return p[i * rs + j * cs]; }
};

__device__ __forceinline__ View rowmajor(const double* p, int64_t ld) { return View{p, ld, 1}; }
__device__ __forceinline__ View colmajor(const double* p, int64_t ld) { return View{p, 1, ld}; }
__device__ __forceinline__ View transposed(View v) { return View{v.p, v.cs, v.rs}; }

// Static shared state of the CTA routines.
struct CtaShared
{
  double red[kWarps];
  double gemm_a[16][64 + 1];
  double gemm_b[16][64 + 1];
  int flag;
  unsigned int relbits;  // float bits of a sweep's largest relative rotation
  int item;
  int ival[4];
  double dval[4];
  double hh[4];       // Householder scalars broadcast by thread 0 (FP64 QR)
  double ldl_inv[2];  // inverse of the next LDL^T pivot, double-buffered
  int ldl_ok[2];      // that pivot is positive
};

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
struct Eps;
template <>
struct Eps<double>
{
  static __device__ __forceinline__ double value() { return DBL_EPSILON; }
};
template <>
struct Eps<float>
{
  static __device__ __forceinline__ float value() { return 4.0f * FLT_EPSILON; }
};

// Sum over the CTA; every thread gets the same value (the partials are
// added in a fixed order by every thread).
__device__ double cta_sum(double v, CtaShared& sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0)
    sh.red[w] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int i = 0; i < kWarps; ++i)
    t += sh.red[i];
  return t;
}

__device__ __forceinline__ void cta_fill(double* p, int64_t n, double v)
{
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    p[i] = v;
}

// dst(i, j) = src(i, j) for an (m x n) block; dst column-major with ld.
__device__ void cta_copy_to_colmajor(double* dst, int64_t ld, View src, int64_t m, int64_t n)
{
  const int64_t total = m * n;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int64_t i = t % m, j = t / m;
    dst[i + j * ld] = src(i, j);
  }
}

// dst row-major (m x n, ld) from a view.
__device__ void cta_copy_to_rowmajor(double* dst, int64_t ld, View src, int64_t m, int64_t n)
{
  const int64_t total = m * n;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int64_t i = t / n, j = t % n;
    dst[i * ld + j] = src(i, j);
  }
}

// Lanes per column in the column loops of the unblocked Householder
// routines, by the column's length: short columns put several columns in
// flight per warp (each with a shorter reduction: in FP64 every level is an
// add on the FP64 pipe, for all 32 lanes) instead of chaining five levels
// per column.  Uniform over the CTA.
__device__ __forceinline__ int hh_group(int len)
{
  return len > 256 ? 32 : (len > 96 ? 16 : 8);
}

// Sum over the G aligned lanes of a group (G = 8, 16 or 32); every lane of
// the group gets it.  All 32 lanes of the warp must call it.
__device__ __forceinline__ double group_sum(double v, int G)
{
  for (int o = G >> 1; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Householder QR, in place.  A column-major (m x c, ld).  On return the
// upper triangle of the leading (k x c) block holds R (k = min(m, c)), the
// strict lower part of column j holds the reflector tail v_j[1:] (v_j[0] = 1
// implicit) and tau[j] its scale: H_j = I - tau_j v_j v_j^T.  Reflector
// convention of Eigen's makeHouseholder (beta = -sign(x0)*||x||; an exactly
// zero tail gives tau = 0), as in qr_thin (types/tt_eigen_bridge.hpp:42-60).
// Thread 0 alone forms the reflector scalars (one FP64 square root and two
// divisions) and broadcasts t and 1 / (x0 - beta); the trailing update uses
// the unscaled column with that factor folded in, and the column's own
// scaling to v is deferred to the next reflector's norm pass.
// ---------------------------------------------------------------------------
__device__ __noinline__ void cta_householder_qr(double* A, int m, int c, int64_t ld, double* tau, CtaShared& sh)
{
  const int k = m < c ? m : c;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double inv_prev = 0.0;
  for (int j = 0; j < k; ++j)
  {
    double* x = A + j * ld + j;
    const int len = m - j;
    if (j > 0)
    {
      double* xp = x - ld - 1;  // column j - 1 from its diagonal
      for (int i = 1 + threadIdx.x; i <= len; i += blockDim.x)
        xp[i] *= inv_prev;
    }
    double part = 0.0;
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      part = fma(x[i], x[i], part);
    part = warp_sum(part);
    if (lane == 0)
      sh.red[w] = part;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      double tail2 = 0.0;
#pragma unroll
      for (int i = 0; i < kWarps; ++i)
        tail2 += sh.red[i];
      const double x0 = x[0];
      double beta, t, inv;
      if (tail2 <= DBL_MIN)
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
      x[0] = beta;
      tau[j] = t;
      sh.hh[0] = t;
      sh.hh[1] = inv;
    }
    __syncthreads();
    const double t = sh.hh[0], inv = sh.hh[1];
    if (t != 0.0)
    {
      // G lanes per column, 32 / G columns in flight per warp; the loop
      // bound is uniform over the warp (the group sum needs every lane).
      const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
      for (int cb = j + 1 + w * gpw; cb < c; cb += kWarps * gpw)
      {
        const int col = cb + lane / G;
        const bool act = col < c;
        double* y = A + (act ? col : cb) * ld + j;
        double dot = 0.0;
        if (act)
          for (int i = 1 + gl; i < len; i += G)
            dot = fma(x[i], y[i], dot);
        // t (y0 + v1..^T y1..), v = x * inv: the group's lane 0 alone reads
        // and writes y0.
        const double y0 = (act && gl == 0) ? y[0] : 0.0;
        dot = group_sum(fma(dot, inv, y0), G) * t;
        if (act)
        {
          const double nd = -dot * inv;
          if (gl == 0)
            y[0] = y0 - dot;
          for (int i = 1 + gl; i < len; i += G)
            y[i] = fma(nd, x[i], y[i]);
        }
      }
    }
    inv_prev = inv;
    __syncthreads();
  }
  if (k > 0)
  {
    double* xl = A + (k - 1) * ld + (k - 1);
    for (int i = 1 + threadIdx.x; i < m - (k - 1); i += blockDim.x)
      xl[i] *= inv_prev;
    __syncthreads();
  }
}

// Copy R (k x c upper triangular, zero below) out of a factored A into a
// column-major (k x c) buffer with leading dimension k.
__device__ void cta_extract_r(double* R, const double* A, int k, int c, int64_t ld)
{
  const int64_t total = static_cast<int64_t>(k) * c;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int i = static_cast<int>(t % k), j = static_cast<int>(t / k);
    R[t] = (i <= j) ? A[i + j * ld] : 0.0;
  }
  __syncthreads();
}

// Form the thin Q (m x k) in place from the reflectors (LAPACK dorg2r order).
// R must have been extracted before.
__device__ __noinline__ void cta_form_q(double* A, int m, int k, int64_t ld, const double* tau)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = k - 1; j >= 0; --j)
  {
    double* v = A + j * ld + j;
    const double t = tau[j];
    const int len = m - j;
    if (t != 0.0)
    {
      const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
      for (int cb = j + 1 + w * gpw; cb < k; cb += kWarps * gpw)
      {
        const int col = cb + lane / G;
        const bool act = col < k;
        double* y = A + (act ? col : cb) * ld + j;
        double dot = 0.0;
        if (act)
          for (int i = gl; i < len; i += G)
            dot = fma(i == 0 ? 1.0 : v[i], y[i], dot);
        dot = group_sum(dot, G) * t;
        if (act)
          for (int i = gl; i < len; i += G)
            y[i] = fma(-dot, i == 0 ? 1.0 : v[i], y[i]);
      }
    }
    __syncthreads();
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      v[i] *= -t;
    if (threadIdx.x == 0)
      v[0] = 1.0 - t;
    for (int i = threadIdx.x; i < j; i += blockDim.x)
      A[j * ld + i] = 0.0;
    __syncthreads();
  }
}

// B (m x p, column-major, ldb) <- H_0 H_1 ... H_{kref-1} B.
__device__ __noinline__ void cta_apply_q(const double* A, int m, int kref, int64_t lda, const double* tau,
                            double* B, int p, int64_t ldb)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = kref - 1; j >= 0; --j)
  {
    const double t = tau[j];
    if (t == 0.0)
      continue;
    const double* v = A + j * lda + j;
    const int len = m - j;
    const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
    for (int cb = w * gpw; cb < p; cb += kWarps * gpw)
    {
      const int col = cb + lane / G;
      const bool act = col < p;
      double* y = B + (act ? col : cb) * ldb + j;
      double dot = 0.0;
      if (act)
        for (int i = gl; i < len; i += G)
          dot = fma(i == 0 ? 1.0 : v[i], y[i], dot);
      dot = group_sum(dot, G) * t;
      if (act)
        for (int i = gl; i < len; i += G)
          y[i] = fma(-dot, i == 0 ? 1.0 : v[i], y[i]);
    }
    __syncthreads();
  }
}


// Column norms of A (m x n column-major) into sig[n].
__device__ void cta_col_norms(const double* A, int m, int n, int64_t lda, double* sig)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = w; j < n; j += kWarps)
  {
    const double* a = A + j * lda;
    double s = 0.0;
    for (int i = lane; i < m; i += 32)
      s += a[i] * a[i];
    s = warp_sum(s);
    if (lane == 0)
      sig[j] = sqrt(s);
  }
  __syncthreads();
}

// ord[0..n) = indices of sig sorted descending (stable).  sorted[k] = sig[ord[k]].
__device__ void cta_argsort_desc(const double* sig, int n, int* ord, double* sorted)
{
  for (int i = threadIdx.x; i < n; i += blockDim.x)
  {
    const double si = sig[i];
    int rank = 0;
    for (int j = 0; j < n; ++j)
    {
      const double sj = sig[j];
      rank += (sj > si) || (sj == si && j < i);
    }
    ord[rank] = i;
    sorted[rank] = si;
  }
  __syncthreads();
}

// truncate_eps_rank (types/tt_eigen_bridge.hpp:172-197) on descending s.
__device__ int trunc_rank_serial(const double* s, int n, double delta, int max_rank)
{
  if (n == 0)
    return 1;
  const double thresh = delta * delta;
  double tail2 = 0.0;
  int r_new = n;
  for (int i = n - 1; i >= 0; --i)
  {
    const double next = tail2 + s[i] * s[i];
    if (next > thresh)
      break;
    tail2 = next;
    r_new = i;
  }
  if (r_new < 1)
    r_new = 1;
  if (max_rank > 0 && r_new > max_rank)
    r_new = max_rank;
  return r_new;
}

// ---------------------------------------------------------------------------
// FP64 GEMM, one CTA: C(i, j) = sum_p A(i, p) B(p, j), C row-major/col-major
// through (c_rs, c_cs).  64x64 output tiles, 16-deep k slabs in shared
// memory, 4x4 register tile per thread.
// ---------------------------------------------------------------------------
// One 64x64 output tile at (i0, j0).
// Zero structure a GEMM may skip: A(i, p) = 0 for p < i (an upper-
// triangular left factor, R of a QR), or B(p, j) = 0 for p < j (a lower-
// triangular right factor, R^T).
enum GemmTri : int
{
  kTriNone = 0,
  kTriUpperA = 1,
  kTriLowerB = 2,
};

// One 64 x 64 tile of C = A B (FP64): k slabs of 16 staged in shared
// memory, 4 x 4 outputs per thread.  A thread multiplies only the rows and
// columns of its block that are inside the matrix and, under tri, not in
// the zero triangle of the slab; slabs left of the diagonal are skipped.
__device__ void cta_gemm_tile(int i0, int j0, int M, int N, int K, View A, View B, double* C,
                              int64_t c_rs, int64_t c_cs, CtaShared& sh, int tri)
{
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
      acc[a][b] = 0.0;
  const int pstart = tri == kTriUpperA ? i0 : (tri == kTriLowerB ? j0 : 0);
  for (int p0 = pstart; p0 < K; p0 += 16)
  {
    __syncthreads();
    for (int t = threadIdx.x; t < 16 * 64; t += blockDim.x)
    {
      const int kk = t / 64, ii = t % 64;
      const int gi = i0 + ii, gp = p0 + kk, gj = j0 + ii;
      sh.gemm_a[kk][ii] = (gi < M && gp < K) ? A(gi, gp) : 0.0;
      sh.gemm_b[kk][ii] = (gp < K && gj < N) ? B(gp, gj) : 0.0;
    }
    __syncthreads();
    const int na = gemm_live(M - i0, ty, tri == kTriUpperA, p0 - i0);
    const int nb = gemm_live(N - j0, tx, tri == kTriLowerB, p0 - j0);
    const int kmax = K - p0 < 16 ? K - p0 : 16;
#pragma unroll 4
    for (int kk = 0; kk < kmax; ++kk)
    {
      double av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
        av[a] = sh.gemm_a[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b)
        bv[b] = sh.gemm_b[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
        if (a < na)
        {
#pragma unroll
          for (int b = 0; b < 4; ++b)
            if (b < nb)
              acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
    {
      const int gi = i0 + ty + 16 * a, gj = j0 + tx + 16 * b;
      if (gi < M && gj < N)
        C[gi * c_rs + gj * c_cs] = acc[a][b];
    }
}

// C = A B, tile by tile (row tiles outer).  With tri = kTriUpperA a tile
// reads B only from its own first row down, and with kTriLowerB A only from
// its own first column right; so C may be B itself (upper A, M <= K, same
// layout) or A itself (lower B, N <= K, same layout): every element is read
// by the tiles that need it before a tile writes over it.
__device__ __noinline__ void cta_gemm(int M, int N, int K, View A, View B, double* C, int64_t c_rs,
                         int64_t c_cs, CtaShared& sh, int tri = kTriNone)
{
  for (int i0 = 0; i0 < M; i0 += 64)
    for (int j0 = 0; j0 < N; j0 += 64)
      cta_gemm_tile(i0, j0, M, N, K, A, B, C, c_rs, c_cs, sh, tri);
  __syncthreads();
}

}  // namespace
}  // namespace ttg
