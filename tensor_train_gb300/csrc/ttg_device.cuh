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

namespace ttg
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

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
  int item;
  int ival[4];
  double dval[4];
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

// ---------------------------------------------------------------------------
// Householder QR, in place.  A column-major (m x c, ld).  On return the
// upper triangle of the leading (k x c) block holds R (k = min(m, c)), the
// strict lower part of column j holds the reflector tail v_j[1:] (v_j[0] = 1
// implicit) and tau[j] its scale: H_j = I - tau_j v_j v_j^T.  Reflector
// convention of Eigen's makeHouseholder (beta = -sign(x0)*||x||; an exactly
// zero tail gives tau = 0), as in qr_thin (types/tt_eigen_bridge.hpp:42-60).
// ---------------------------------------------------------------------------
__device__ void cta_householder_qr(double* A, int m, int c, int64_t ld, double* tau, CtaShared& sh)
{
  const int k = m < c ? m : c;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < k; ++j)
  {
    double* x = A + j * ld + j;
    const int len = m - j;
    double part = 0.0;
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      part += x[i] * x[i];
    const double tail2 = cta_sum(part, sh);
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
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      x[i] *= inv;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      x[0] = beta;
      tau[j] = t;
    }
    if (t != 0.0)
    {
      for (int col = j + 1 + w; col < c; col += kWarps)
      {
        double* y = A + col * ld + j;
        double dot = 0.0;
        for (int i = lane; i < len; i += 32)
          dot += (i == 0 ? 1.0 : x[i]) * y[i];
        dot = warp_sum(dot) * t;
        for (int i = lane; i < len; i += 32)
          y[i] -= dot * (i == 0 ? 1.0 : x[i]);
      }
    }
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
__device__ void cta_form_q(double* A, int m, int k, int64_t ld, const double* tau)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = k - 1; j >= 0; --j)
  {
    double* v = A + j * ld + j;
    const double t = tau[j];
    const int len = m - j;
    if (t != 0.0)
    {
      for (int col = j + 1 + w; col < k; col += kWarps)
      {
        double* y = A + col * ld + j;
        double dot = 0.0;
        for (int i = lane; i < len; i += 32)
          dot += (i == 0 ? 1.0 : v[i]) * y[i];
        dot = warp_sum(dot) * t;
        for (int i = lane; i < len; i += 32)
          y[i] -= dot * (i == 0 ? 1.0 : v[i]);
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
__device__ void cta_apply_q(const double* A, int m, int kref, int64_t lda, const double* tau,
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
    for (int col = w; col < p; col += kWarps)
    {
      double* y = B + col * ldb + j;
      double dot = 0.0;
      for (int i = lane; i < len; i += 32)
        dot += (i == 0 ? 1.0 : v[i]) * y[i];
      dot = warp_sum(dot) * t;
      for (int i = lane; i < len; i += 32)
        y[i] -= dot * (i == 0 ? 1.0 : v[i]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// One-sided Jacobi (Hestenes) SVD, in place.  A column-major (m x n, lda):
// on return its columns are mutually orthogonal (A_final = U * diag(s)).
// V column-major (n x n, ldv) accumulates the rotations when non-null (it
// must hold the identity, or any start matrix, on entry).  Pairs are visited
// in the round-robin tournament order, n/2 disjoint pairs per round, one
// warp per pair.  Squared column norms are cached in nrm[n] (recomputed at
// the start of every sweep, updated after each rotation as
// alpha' = alpha - t*gamma, beta' = beta + t*gamma), so a pair costs one dot
// product and one rotation.  Returns the number of sweeps; *converged = 0 if
// the limit was reached.  Rotation as in Demmel & Veselic (1992), eq. (4.3).
// ---------------------------------------------------------------------------
template <class T>
__device__ int cta_jacobi(T* A, int m, int n, int64_t lda, T* V, int64_t ldv, int max_sweeps,
                          int* converged, T* nrm, CtaShared& sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = n + (n & 1);
  const int npairs = N / 2;
  const T tol = sqrt(static_cast<T>(m > 1 ? m : 1)) * Eps<T>::value();
  int sweep = 0;
  *converged = 0;
  if (n < 2)
  {
    *converged = 1;
    return 0;
  }
  for (; sweep < max_sweeps; ++sweep)
  {
    __syncthreads();
    if (threadIdx.x == 0)
      sh.flag = 0;
    for (int j = w; j < n; j += kWarps)
    {
      const T* a = A + j * lda;
      T s = 0;
      for (int i = lane; i < m; i += 32)
        s += a[i] * a[i];
      s = warp_sum(s);
      if (lane == 0)
        nrm[j] = s;
    }
    __syncthreads();
    for (int r = 0; r < N - 1; ++r)
    {
      for (int t = w; t < npairs; t += kWarps)
      {
        int p = (t == 0) ? 0 : ((t - 1 + r) % (N - 1)) + 1;
        int q = ((N - 2 - t + r) % (N - 1)) + 1;
        if (p >= n || q >= n)
          continue;
        if (p > q)
        {
          const int tmp = p;
          p = q;
          q = tmp;
        }
        T* ap = A + p * lda;
        T* aq = A + q * lda;
        const T al = nrm[p], be = nrm[q];
        T ga = 0;
        for (int i = lane; i < m; i += 32)
          ga += ap[i] * aq[i];
        ga = warp_sum(ga);
        if (ga == T(0) || fabs(ga) <= tol * sqrt(fmax(al, T(0)) * fmax(be, T(0))))
          continue;
        const T zeta = (be - al) / (T(2) * ga);
        T tt;
        if (fabs(zeta) > T(1.0e18))
          tt = T(0.5) / zeta;
        else
          tt = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + tt * tt);
        const T s = c * tt;
        for (int i = lane; i < m; i += 32)
        {
          const T x = ap[i], y = aq[i];
          ap[i] = c * x - s * y;
          aq[i] = s * x + c * y;
        }
        if (V)
        {
          T* vp = V + p * ldv;
          T* vq = V + q * ldv;
          for (int i = lane; i < n; i += 32)
          {
            const T x = vp[i], y = vq[i];
            vp[i] = c * x - s * y;
            vq[i] = s * x + c * y;
          }
        }
        if (lane == 0)
        {
          nrm[p] = al - tt * ga;
          nrm[q] = be + tt * ga;
          sh.flag = 1;
        }
      }
      __syncthreads();
    }
    const int any = sh.flag;
    __syncthreads();
    if (!any)
    {
      *converged = 1;
      ++sweep;
      break;
    }
  }
  __syncthreads();
  return sweep;
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
__device__ void cta_gemm(int M, int N, int K, View A, View B, double* C, int64_t c_rs,
                         int64_t c_cs, CtaShared& sh)
{
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int i0 = 0; i0 < M; i0 += 64)
    for (int j0 = 0; j0 < N; j0 += 64)
    {
      double acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          acc[a][b] = 0.0;
      for (int p0 = 0; p0 < K; p0 += 16)
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
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
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
#pragma unroll
            for (int b = 0; b < 4; ++b)
              acc[a][b] = fma(av[a], bv[b], acc[a][b]);
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
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Mixed-precision one-sided Jacobi: the sweeps that do most of the rotating
// run in FP32, one FP64 refinement restores FP64 accuracy.
//   1. FP32 copy of src (m x n, m >= n) and V32 = I in fbuf
//      (m*n + n*n floats); FP32 Jacobi sweeps accumulate V32.
//   2. V = V32 * (3I - V32^T V32)/2 in FP64 (one Newton-Schulz step: V is
//      orthogonal to FP64 accuracy), in tmp (3 n*n doubles).
//   3. A = src * V (FP64 GEMM) -- nearly orthogonal columns.
//   4. FP64 Jacobi sweeps on A (typically one rotating sweep and one check);
//      when Vout is given it starts from V and accumulates the rotations.
// src stays readable throughout; fbuf may alias A (it is dead before step 3).
// Returns the FP64 sweep count.
// ---------------------------------------------------------------------------
template <class Gemm>
__device__ int cta_jacobi_mixed(View src, int m, int n, double* A, int64_t lda, double* Vout,
                                int max_sweeps, int* converged, double* nrm, float* fbuf,
                                double* tmp, CtaShared& sh, Gemm gemm)
{
  float* Af = fbuf;
  float* Vf = fbuf + static_cast<int64_t>(m) * n;
  const int64_t mn = static_cast<int64_t>(m) * n, nn = static_cast<int64_t>(n) * n;
  for (int64_t t = threadIdx.x; t < mn; t += blockDim.x)
    Af[t] = static_cast<float>(src(t % m, t / m));
  for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
    Vf[t] = (t % n == t / n) ? 1.0f : 0.0f;
  __syncthreads();
  int conv32 = 0;
  cta_jacobi<float>(Af, m, n, m, Vf, n, 24, &conv32, reinterpret_cast<float*>(nrm), sh);
  double* Vd = tmp;
  double* P = tmp + nn;
  double* V2 = tmp + 2 * nn;
  for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
    Vd[t] = static_cast<double>(Vf[t]);
  __syncthreads();
  // P = Vd^T Vd ; P <- (3I - P)/2 ; V2 = Vd P.
  gemm(n, n, n, View{Vd, n, 1}, View{Vd, 1, n}, P, 1, n, sh);
  for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
    P[t] = ((t % n == t / n) ? 1.5 : 0.0) - 0.5 * P[t];
  __syncthreads();
  gemm(n, n, n, View{Vd, 1, n}, View{P, 1, n}, V2, 1, n, sh);
  gemm(m, n, n, src, View{V2, 1, n}, A, 1, lda, sh);
  if (Vout)
  {
    for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
      Vout[t] = V2[t];
    __syncthreads();
  }
  return cta_jacobi<double>(A, m, n, lda, Vout, n, max_sweeps, converged, nrm, sh);
}

}  // namespace ttg
