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
// Internal linkage: every translation unit that includes this header gets
// its own copy of these device functions.
namespace
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

// W (df64, column-major m x n, ld) = split(X * 2^k).
__device__ void cta_split_to_df(df64* W, int64_t ld, View X, int64_t m, int64_t n, int k)
{
  const int64_t total = m * n;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int64_t i = t % m, j = t / m;
    W[i + j * ld] = df_split_pow2(X(i, j), k);
  }
}

// W[t] (FP64) = A[t] (df64) for t < n, in place when W and A alias
// element for element.
__device__ void cta_join_from_df(double* W, const df64* A, int64_t n)
{
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x)
  {
    const df64 a = A[t];
    W[t] = df_join_pow2(a, 0);
  }
  __syncthreads();
}

// Sum over the G aligned lanes of a group (G = 8, 16 or 32); every lane of
// the group gets it.  All 32 lanes of the warp must call it.
__device__ __forceinline__ df64 df_group_sum(df64 v, int G)
{
  for (int o = G >> 1; o > 0; o >>= 1)
    v = df_add(v, df_shfl_xor(v, o));
  return v;
}

// The reflector of x = (x0, x1..) with ||x1..||^2 = tail2, in df64 on the
// FP32 pipes: H = I - t v v^T, v = (1, x1.. * inv), H x = (beta, 0..);
// t = 0 (no reflection) when the tail is negligible.
__device__ __forceinline__ void householder_scalars_df(df64 x0, df64 tail2, df64* beta, df64* t,
                                                       df64* inv)
{
  if (tail2.hi <= 1.0e-36f)
  {
    *beta = x0;
    *t = df64{0.0f, 0.0f};
    *inv = df64{0.0f, 0.0f};
    return;
  }
  df64 b = df_sqrt(df_fma(x0, x0, tail2));
  if (x0.hi >= 0.0f)
    b = df_neg(b);
  const df64 den = df_sub(x0, b);  // x0 and beta have opposite signs: no cancellation
  *beta = b;
  *inv = df_recip(den);
  *t = df_neg(df_mul(den, df_recip(b)));  // (beta - x0) / beta
}

// Householder QR in df64, in place (see cta_householder_qr for the layout
// and convention).  tau is kept in df64.  Every thread forms the reflector
// scalars itself from the warp partial sums (FP32 pipes, no broadcast), the
// trailing update uses the unscaled column with inv folded in, and the
// column's own scaling to v is deferred to the next reflector's norm pass:
// two barriers per reflector.
__device__ __noinline__ void cta_householder_qr_df(df64* A, int m, int c, int64_t ld, df64* tau, CtaShared& sh)
{
  const int k = m < c ? m : c;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  df64* red = reinterpret_cast<df64*>(sh.red);
  df64 inv_prev{0.0f, 0.0f};
  for (int j = 0; j < k; ++j)
  {
    df64* x = A + j * ld + j;
    const int len = m - j;
    if (j > 0)
    {
      df64* xp = x - ld - 1;  // column j - 1 from its diagonal
      for (int i = 1 + threadIdx.x; i <= len; i += blockDim.x)
        xp[i] = df_mul(xp[i], inv_prev);
    }
    df64 part{0.0f, 0.0f};
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
      part = df_fma(x[i], x[i], part);
    part = df_warp_sum(part);
    const df64 x0 = x[0];
    if (lane == 0)
      red[w] = part;
    __syncthreads();
    df64 tail2{0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < kWarps; ++i)
      tail2 = df_add(tail2, red[i]);
    df64 beta, td, inv;
    householder_scalars_df(x0, tail2, &beta, &td, &inv);
    if (threadIdx.x == 0)
    {
      x[0] = beta;
      tau[j] = td;
    }
    if (td.hi != 0.0f)
    {
      // G lanes per column, 32 / G columns in flight per warp; the loop
      // bound is uniform over the warp (the group sum needs every lane).
      const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
      for (int cb = j + 1 + w * gpw; cb < c; cb += kWarps * gpw)
      {
        const int col = cb + lane / G;
        const bool act = col < c;
        df64* y = A + (act ? col : cb) * ld + j;
        df64 dot{0.0f, 0.0f};
        if (act)
          for (int i = 1 + gl; i < len; i += G)
            dot = df_fma(x[i], y[i], dot);
        // t (y0 + v1..^T y1..), v = x * inv: the group's lane 0 alone reads
        // and writes y0.
        const df64 y0 = (act && gl == 0) ? y[0] : df64{0.0f, 0.0f};
        dot = df_mul(df_group_sum(df_fma(dot, inv, y0), G), td);
        if (act)
        {
          const df64 nd = df_neg(df_mul(dot, inv));
          if (gl == 0)
            y[0] = df_sub(y0, dot);
          for (int i = 1 + gl; i < len; i += G)
            y[i] = df_fma(nd, x[i], y[i]);
        }
      }
    }
    inv_prev = inv;
    __syncthreads();
  }
  if (k > 0)
  {
    df64* xl = A + (k - 1) * ld + (k - 1);
    for (int i = 1 + threadIdx.x; i < m - (k - 1); i += blockDim.x)
      xl[i] = df_mul(xl[i], inv_prev);
    __syncthreads();
  }
}

// R (k x c, column-major, FP64, ld k) = upper triangle of A, times 2^e.
__device__ void cta_extract_r_df(double* R, const df64* A, int k, int c, int64_t ld, int e)
{
  const int64_t total = static_cast<int64_t>(k) * c;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const int i = static_cast<int>(t % k), j = static_cast<int>(t / k);
    R[t] = (i <= j) ? df_join_pow2(A[i + j * ld], e) : 0.0;
  }
  __syncthreads();
}

// Thin Q (m x k) in place, df64 (dorg2r order, as cta_form_q).
__device__ __noinline__ void cta_form_q_df(df64* A, int m, int k, int64_t ld, const df64* tau)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = k - 1; j >= 0; --j)
  {
    df64* v = A + j * ld + j;
    const df64 t = tau[j];
    const int len = m - j;
    if (t.hi != 0.0f)
    {
      const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
      for (int cb = j + 1 + w * gpw; cb < k; cb += kWarps * gpw)
      {
        const int col = cb + lane / G;
        const bool act = col < k;
        df64* y = A + (act ? col : cb) * ld + j;
        df64 dot = (act && gl == 0) ? y[0] : df64{0.0f, 0.0f};
        if (act)
          for (int i = 1 + gl; i < len; i += G)
            dot = df_fma(v[i], y[i], dot);
        dot = df_mul(df_group_sum(dot, G), t);
        if (act)
        {
          const df64 nd = df_neg(dot);
          if (gl == 0)
            y[0] = df_add(y[0], nd);
          for (int i = 1 + gl; i < len; i += G)
            y[i] = df_fma(nd, v[i], y[i]);
        }
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
__device__ __noinline__ void cta_apply_q_df(const df64* A, int m, int kref, int64_t lda, const df64* tau,
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
    const int G = hh_group(len), gpw = 32 / G, gl = lane & (G - 1);
    for (int cb = w * gpw; cb < p; cb += kWarps * gpw)
    {
      const int col = cb + lane / G;
      const bool act = col < p;
      df64* y = B + (act ? col : cb) * ldb + j;
      df64 dot = (act && gl == 0) ? y[0] : df64{0.0f, 0.0f};
      if (act)
        for (int i = 1 + gl; i < len; i += G)
          dot = df_fma(v[i], y[i], dot);
      dot = df_mul(df_group_sum(dot, G), t);
      if (act)
      {
        const df64 nd = df_neg(dot);
        if (gl == 0)
          y[0] = df_add(y[0], nd);
        for (int i = 1 + gl; i < len; i += G)
          y[i] = df_fma(nd, v[i], y[i]);
      }
    }
    __syncthreads();
  }
}

// Element arithmetic of the one-sided Jacobi below, for FP32, FP64 and df64
// matrices.  S is the type of the cached squared norms and the rotation
// parameters (FP64 for df64), Acc the dot-product accumulator.
template <class E>
struct JOps;
template <>
struct JOps<float>
{
  using S = float;
  using Acc = float;
  struct Rot
  {
    float c, s;
  };
  static __device__ __forceinline__ Acc zero() { return 0.0f; }
  static __device__ __forceinline__ Acc fma(float a, float b, Acc c) { return fmaf(a, b, c); }
  static __device__ __forceinline__ Acc add(Acc a, Acc b) { return a + b; }
  static __device__ __forceinline__ Acc shfl(Acc v, int o)
  {
    return __shfl_xor_sync(0xffffffffu, v, o);
  }
  static __device__ __forceinline__ S to_s(Acc v) { return v; }
  static __device__ __forceinline__ S eps() { return 4.0f * FLT_EPSILON; }
  static __device__ __forceinline__ Rot rot(S c, S s) { return Rot{c, s}; }
  static __device__ __forceinline__ void apply(const Rot& r, float& x, float& y)
  {
    const float a = x, b = y;
    x = r.c * a - r.s * b;
    y = r.s * a + r.c * b;
  }
};
template <>
struct JOps<double>
{
  using S = double;
  using Acc = double;
  struct Rot
  {
    double c, s;
  };
  static __device__ __forceinline__ Acc zero() { return 0.0; }
  static __device__ __forceinline__ Acc fma(double a, double b, Acc c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ Acc add(Acc a, Acc b) { return a + b; }
  static __device__ __forceinline__ Acc shfl(Acc v, int o)
  {
    return __shfl_xor_sync(0xffffffffu, v, o);
  }
  static __device__ __forceinline__ S to_s(Acc v) { return v; }
  static __device__ __forceinline__ S eps() { return DBL_EPSILON; }
  static __device__ __forceinline__ Rot rot(S c, S s) { return Rot{c, s}; }
  static __device__ __forceinline__ void apply(const Rot& r, double& x, double& y)
  {
    const double a = x, b = y;
    x = r.c * a - r.s * b;
    y = r.s * a + r.c * b;
  }
};
template <>
struct JOps<df64>
{
  using S = double;
  using Acc = df64;
  struct Rot
  {
    df64 c, s, ns;
  };
  static __device__ __forceinline__ Acc zero() { return df64{0.0f, 0.0f}; }
  static __device__ __forceinline__ Acc fma(df64 a, df64 b, Acc c) { return df_fma(a, b, c); }
  static __device__ __forceinline__ Acc add(Acc a, Acc b) { return df_add(a, b); }
  static __device__ __forceinline__ Acc shfl(Acc v, int o) { return df_shfl_xor(v, o); }
  static __device__ __forceinline__ S to_s(Acc v) { return df_to(v); }
  // df64 carries 48 significand bits.
  static __device__ __forceinline__ S eps() { return 7.2e-15; }
  static __device__ __forceinline__ Rot rot(S c, S s)
  {
    return Rot{df_from(c), df_from(s), df_from(-s)};
  }
  static __device__ __forceinline__ void apply(const Rot& r, df64& x, df64& y)
  {
    const df64 a = x, b = y;
    x = df_fma(r.ns, b, df_mul(r.c, a));
    y = df_fma(r.s, a, df_mul(r.c, b));
  }
};

// ---------------------------------------------------------------------------
// One-sided Jacobi (Hestenes) SVD, in place.  A column-major (m x n, lda):
// on return its columns are mutually orthogonal (A_final = U * diag(s)).
// V column-major (vrows x n, ldv; vrows = n by default) accumulates the
// rotations when non-null (it must hold the identity, or any start matrix,
// on entry).  Pairs are visited
// in the round-robin tournament order, n/2 disjoint pairs per round, one
// group of G lanes per pair (G = 8, 16 or 32 by column length: short
// columns put several pairs in flight per warp, which is what bounds a
// latency-bound sweep).  Squared column norms are cached in nrm[n] (recomputed at
// the start of every sweep, updated after each rotation as
// alpha' = alpha - t*gamma, beta' = beta + t*gamma), so a pair costs one dot
// product and one rotation.  Returns the number of sweeps; *converged = 0 if
// the limit was reached.  Rotation as in Demmel & Veselic (1992), eq. (4.3).
// ---------------------------------------------------------------------------
//
// floor2: a column whose squared norm is <= floor2 is never rotated.  Such
// columns lie far below the truncation threshold (the caller picks floor2
// so that all of them together hold a negligible share of delta^2): leaving
// them out moves the kept singular values and vectors by O(their norm^2),
// and on rank-deficient inputs they would otherwise keep the sweeps going.
// (Freezing only pairs of tiny columns is not enough: a column just above
// the floor never becomes orthogonal to a mutually non-orthogonal frozen
// set, and the sweeps would cycle.)
// stop_rel > 0: a sweep whose largest rotated |a_p . a_q| / (|a_p| |a_q|)
// is below stop_rel ends the iteration (one-sided Jacobi converges
// quadratically, so the next sweep's rotations would be ~stop_rel^2).
template <class E>
__device__ __noinline__ int cta_jacobi(E* A, int m, int n, int64_t lda, E* V, int64_t ldv, int max_sweeps,
                          int* converged, typename JOps<E>::S* nrm, CtaShared& sh,
                          typename JOps<E>::S floor2 = 0, typename JOps<E>::S stop_rel = 0,
                          float* maxrel_out = nullptr, int vrows = -1)
{
  using O = JOps<E>;
  using S = typename O::S;
  using Acc = typename O::Acc;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // Group size by column length, widened while half the groups would
  // already cover all pairs of a round (short rows of few columns).
  int G = m <= 128 ? 8 : (m <= 512 ? 16 : 32);
  while (G < 32 && kWarps * (32 / G) >= 2 * ((n + 1) / 2))
    G *= 2;
  const int gpw = 32 / G, ngroups = kWarps * gpw;
  const int grp = w * gpw + lane / G, gl = lane & (G - 1);
  const int N = n + (n & 1);
  const int npairs = N / 2;
  const S tol = sqrt(static_cast<S>(m > 1 ? m : 1)) * O::eps();
  auto group_sum = [G](Acc v) {
    for (int o = G >> 1; o > 0; o >>= 1)
      v = O::add(v, O::shfl(v, o));
    return v;
  };
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
    {
      sh.flag = 0;
      sh.relbits = 0u;
    }
    for (int j0 = 0; j0 < n; j0 += ngroups)
    {
      const int j = j0 + grp;
      Acc acc = O::zero();
      if (j < n)
      {
        const E* a = A + j * lda;
        for (int i = gl; i < m; i += G)
          acc = O::fma(a[i], a[i], acc);
      }
      acc = group_sum(acc);
      if (j < n && gl == 0)
        nrm[j] = O::to_s(acc);
    }
    __syncthreads();
    for (int r = 0; r < N - 1; ++r)
    {
      for (int t0 = 0; t0 < npairs; t0 += ngroups)
      {
        const int t = t0 + grp;
        int p = 0, q = 0;
        bool act = t < npairs;
        if (act)
        {
          p = (t == 0) ? 0 : ((t - 1 + r) % (N - 1)) + 1;
          q = ((N - 2 - t + r) % (N - 1)) + 1;
          if (p >= n || q >= n)
            act = false;
          else if (p > q)
          {
            const int tmp = p;
            p = q;
            q = tmp;
          }
        }
        S al = 0, be = 0;
        if (act)
        {
          al = nrm[p];
          be = nrm[q];
          if (al <= floor2 || be <= floor2)
            act = false;
        }
        E* ap = A + p * lda;
        E* aq = A + q * lda;
        Acc acc = O::zero();
        if (act)
          for (int i = gl; i < m; i += G)
            acc = O::fma(ap[i], aq[i], acc);
        acc = group_sum(acc);
        const S ga = O::to_s(acc);
        if (!act || ga == S(0) || fabs(ga) <= tol * sqrt(fmax(al, S(0)) * fmax(be, S(0))))
          continue;
        const S zeta = (be - al) / (S(2) * ga);
        S tt;
        if (fabs(zeta) > S(1.0e18))
          tt = S(0.5) / zeta;
        else
          tt = (zeta >= S(0) ? S(1) : S(-1)) / (fabs(zeta) + sqrt(S(1) + zeta * zeta));
        const S c = S(1) / sqrt(S(1) + tt * tt);
        const typename O::Rot R = O::rot(c, c * tt);
        for (int i = gl; i < m; i += G)
          O::apply(R, ap[i], aq[i]);
        if (V)
        {
          E* vp = V + p * ldv;
          E* vq = V + q * ldv;
          const int vr = vrows < 0 ? n : vrows;
          for (int i = gl; i < vr; i += G)
            O::apply(R, vp[i], vq[i]);
        }
        if (gl == 0)
        {
          nrm[p] = al - tt * ga;
          nrm[q] = be + tt * ga;
          sh.flag = 1;
          const float rel =
            static_cast<float>(fabs(ga) / sqrt(fmax(al, S(0)) * fmax(be, S(0))));
          atomicMax(&sh.relbits, __float_as_uint(rel));
        }
      }
      __syncthreads();
    }
    const int any = sh.flag;
    const float maxrel = __uint_as_float(sh.relbits);
    __syncthreads();
    if (maxrel_out)
      *maxrel_out = maxrel;
    if (!any || (stop_rel > S(0) && maxrel < static_cast<float>(stop_rel)))
    {
      *converged = 1;
      ++sweep;
      break;
    }
  }
  __syncthreads();
  return sweep;
}

// ---------------------------------------------------------------------------
// No-truncation certificate of a truncated-SVD step.
//
// svd_step keeps all c singular values of a bond exactly when the smallest
// one alone exceeds the tail budget: sigma_c^2 > delta^2 (tail rule of
// truncate_eps_rank, types/tt_eigen_bridge.hpp:172-197, with no max_rank
// cap below c).  Then the SVD only rotates a basis: U diag(s) V^T = Q R gives
// the same represented tensor and the same rank whether the left factor is U
// and diag(s) V^T is absorbed, or Q and R.  These routines prove that case
// from the R factor of the step's QR, so the Jacobi SVD can be skipped.
//
// Test: R^T R - tau I is positive definite, shown by an LDL^T elimination
// that meets only positive pivots.  tau covers every rounding error between
// the bond matrix X and the computed pivots (u = unit roundoff of the
// arithmetic, gamma_n = n u / (1 - n u); Higham, Accuracy and Stability of
// Numerical Algorithms, 2nd ed.):
//   * sigma_min(X) >= sigma_min(R) - e_R, e_R = c h u_QR ||R||_F, a bound on
//     the backward error of the Householder QR that produced R (thm. 19.4,
//     constant taken generously);
//   * fl(R^T R) = R^T R + E1 with ||E1||_2 <= gamma_c ||R||_F^2 (inner
//     products of length <= c; || |R|^T |R| ||_F <= ||R||_F^2);
//   * an LDL^T elimination with positive pivots factors fl(R^T R) - tau I +
//     E2 with |E2| <= gamma_{c+1} |L||D||L^T| (thm. 10.3), and
//     || |L||D||L^T| ||_F <= trace(L D L^T) <= (1 + gamma_c) ||R||_F^2;
// so positive pivots with tau = (1 + 4u)(delta + e_R)^2 + 4 (c + 1) u
// ||R||_F^2 imply sigma_min(X) > delta.  u is 2^-53 for FP64 and 2^-44 for
// df64 (its operations are accurate to a few units of 2^-48: Joldes, Muller
// & Popescu, ACM TOMS 2017).  A NaN anywhere fails the test (a comparison
// with a NaN pivot is false) and the caller runs the SVD, which reports it.
// ---------------------------------------------------------------------------
template <class E>
struct CertOps;
template <>
struct CertOps<double>
{
  static __device__ __forceinline__ double from(double x) { return x; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double neg(double a) { return -a; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double recip(double a) { return 1.0 / a; }
  static __device__ __forceinline__ bool positive(double a) { return a > 0.0; }
  static constexpr double u = 1.1102230246251565e-16;  // 2^-53
};
template <>
struct CertOps<df64>
{
  static __device__ __forceinline__ df64 from(double x) { return df_split_pow2(x, 0); }
  static __device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) { return df_fma(a, b, c); }
  static __device__ __forceinline__ df64 mul(df64 a, df64 b) { return df_mul(a, b); }
  static __device__ __forceinline__ df64 neg(df64 a) { return df_neg(a); }
  static __device__ __forceinline__ df64 sub(df64 a, df64 b) { return df_sub(a, b); }
  static __device__ __forceinline__ df64 recip(df64 a) { return df_recip(a); }
  // hi carries the sign of a normalised pair; NaN compares false.
  static __device__ __forceinline__ bool positive(df64 a) { return a.hi > 0.0f; }
  static constexpr double u = 5.684341886080802e-14;  // 2^-44
};

// The shift tau (see above) for R / s with ||R / s||_F^2 = fro2, the
// threshold dl = delta / s, arithmetic unit roundoff u and QR unit roundoff uqr.
__device__ __forceinline__ double certify_tau(double dl, double fro2, int c, int h, double u,
                                              double uqr)
{
  const double eR = static_cast<double>(c) * h * uqr * sqrt(fro2);
  return (1.0 + 4.0 * u) * (dl + eR) * (dl + eR) + 4.0 * (c + 1.0) * u * fro2;
}

// (i, j), i >= j, of entry t of a lower triangle packed by rows.  The FP32
// square root lands within one of i for t < 2^21 (8t + 1 exact in FP32);
// the integer steps settle it, and any t.
__device__ __forceinline__ void tri_index(int64_t t, int* i_out, int* j_out)
{
  int i = static_cast<int>((sqrtf(8.0f * static_cast<float>(t) + 1.0f) - 1.0f) * 0.5f);
  while (static_cast<int64_t>(i) * (i + 1) / 2 > t)
    --i;
  while (static_cast<int64_t>(i + 1) * (i + 2) / 2 <= t)
    ++i;
  *i_out = i;
  *j_out = static_cast<int>(t - static_cast<int64_t>(i) * (i + 1) / 2);
}

// LDL^T elimination of G - shift I (G: lower triangle of a c x c matrix,
// column-major, ld c, eliminated in place without its shift); true when
// every pivot is positive.  Only the pivots are needed: G(i, k) -= G(i, j)
// G(k, j) / (G(j, j) - shift) for j < k <= i.  The diagonal is stored
// unshifted (the updates are linear, so the shift enters the pivots only).
// Thread 0 owns entry (j+1, j+1) of every trailing update, so it finishes
// the next pivot, tests it and broadcasts its inverse through shared memory
// (double-buffered by step parity): one barrier per step, and the FP64
// division of the plain path runs on one thread instead of all of them.
template <class E>
__device__ bool cta_ldl_positive(E* G, int c, E shift, CtaShared& sh)
{
  using O = CertOps<E>;
  static_assert(sizeof(E) == sizeof(double), "pivot slots hold 8-byte elements");
  E* inv_buf = reinterpret_cast<E*>(sh.ldl_inv);
  if (threadIdx.x == 0)
  {
    const E piv = O::sub(G[0], shift);
    sh.ldl_ok[0] = O::positive(piv) ? 1 : 0;
    inv_buf[0] = O::recip(piv);
  }
  __syncthreads();
  for (int j = 0; j < c; ++j)
  {
    const int b = j & 1;
    if (!sh.ldl_ok[b])
      return false;  // every thread reads the same flag: a uniform exit
    if (j == c - 1)
      break;
    const E inv = inv_buf[b];
    const int rem = c - 1 - j;  // trailing order
    const int64_t ntr = static_cast<int64_t>(rem) * (rem + 1) / 2;
    const E* gj = G + static_cast<int64_t>(j) * c;
    for (int64_t t = threadIdx.x; t < ntr; t += blockDim.x)
    {
      int a, bb;
      tri_index(t, &a, &bb);
      const int i = j + 1 + a, k = j + 1 + bb;  // i >= k > j
      E& g = G[i + static_cast<int64_t>(k) * c];
      g = O::fma(O::neg(O::mul(gj[i], inv)), gj[k], g);
      if (t == 0)
      {
        const E piv = O::sub(g, shift);
        sh.ldl_ok[b ^ 1] = O::positive(piv) ? 1 : 0;
        inv_buf[b ^ 1] = O::recip(piv);
      }
    }
    __syncthreads();
  }
  return true;
}

// R: c x c upper triangular, column-major (ld c), FP64.  G: c x c FP64
// scratch (lower triangle used).  h: rows of the step's matrix; uqr: unit
// roundoff of the QR that produced R.  The plain path's test.
__device__ __noinline__ bool cta_certify_no_truncation(const double* R, int c, int h, double delta,
                                                       double* G, CtaShared& sh, double uqr)
{
  if (c < 1)
    return false;
  // Scale by a power of two (exact) so that max |R| is ~1.
  const double s = cta_pow2_of_max(View{R, 1, c}, c, c, sh);
  const double is = 1.0 / s;
  const int64_t cc = static_cast<int64_t>(c) * c;
  double part = 0.0;
  for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
  {
    const double x = R[t] * is;
    part = fma(x, x, part);
  }
  const double fro2 = cta_sum(part, sh);  // ||R / s||_F^2
  if (!(fro2 > 0.0) || !isfinite(fro2))
    return false;
  // G = (R/s)^T (R/s), lower triangle: G(i, j) = sum_{p <= j} R(p, i) R(p, j) / s^2.
  const int64_t ntri = static_cast<int64_t>(c) * (c + 1) / 2;
  for (int64_t t = threadIdx.x; t < ntri; t += blockDim.x)
  {
    int i, j;
    tri_index(t, &i, &j);
    const double* ri = R + static_cast<int64_t>(i) * c;
    const double* rj = R + static_cast<int64_t>(j) * c;
    double acc = 0.0;
    for (int p = 0; p <= j; ++p)
      acc = fma(ri[p], rj[p], acc);
    G[i + static_cast<int64_t>(j) * c] = acc * is * is;
  }
  double shift = 0.0;
  if (threadIdx.x == 0)
    shift = certify_tau(delta * is, fro2, c, h, CertOps<double>::u, uqr);
  __syncthreads();
  return cta_ldl_positive<double>(G, c, shift, sh);  // only thread 0 reads shift
}

// The mixed path's test, on the df64 R of its QR as it lies in the
// factored panel: Rd(i, j) = Rd[i + j ld], i <= j, representing R / 2^e
// (dl = delta / 2^e).  No conversion: the Gram and the elimination run in
// df64 on the FP32 pipes; ||R||_F^2 and tau are formed once, by thread 0,
// in FP64.  The Gram entries stay far inside the FP32 range: the panel was
// scaled so that its largest entry is in [1, 2), so ||R / 2^e||_F >= 1 and
// every |Rd| <= sqrt(h c) * 2.
__device__ __noinline__ bool cta_certify_no_truncation_df(const df64* Rd, int64_t ld, int c, int h,
                                                          double dl, df64* G, CtaShared& sh,
                                                          double uqr)
{
  if (c < 1)
    return false;
  const int64_t cc = static_cast<int64_t>(c) * c;
  df64 part{0.0f, 0.0f};
  for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
  {
    const int i = static_cast<int>(t % c), j = static_cast<int>(t / c);
    if (i <= j)
    {
      const df64 r = Rd[i + static_cast<int64_t>(j) * ld];
      part = df_fma(r, r, part);
    }
  }
  const df64 f2 = cta_sum_df(part, sh);
  if (!(f2.hi > 0.0f) || !(f2.hi < 1.0e30f))
    return false;  // zero, overflowing or NaN: the SVD path decides (and reports a NaN)
  const int64_t ntri = static_cast<int64_t>(c) * (c + 1) / 2;
  for (int64_t t = threadIdx.x; t < ntri; t += blockDim.x)
  {
    int i, j;
    tri_index(t, &i, &j);
    const df64* ri = Rd + static_cast<int64_t>(i) * ld;
    const df64* rj = Rd + static_cast<int64_t>(j) * ld;
    df64 acc{0.0f, 0.0f};
    for (int p = 0; p <= j; ++p)
      acc = df_fma(ri[p], rj[p], acc);
    G[i + static_cast<int64_t>(j) * c] = acc;
  }
  df64 shift{0.0f, 0.0f};
  if (threadIdx.x == 0)
    shift = df_split_pow2(certify_tau(dl, df_join_pow2(f2, 0), c, h, CertOps<df64>::u, uqr), 0);
  __syncthreads();
  return cta_ldl_positive<df64>(G, c, shift, sh);  // only thread 0 reads shift
}

// The same test with G = R^T R already formed in FP64 (lower triangle
// used; the whole-GPU sweep forms it over the grid): G is scaled by 1/s^2
// in place, then eliminated in FP64 by this CTA.
__device__ __noinline__ bool cta_certify_from_gram(double* G, const double* R, int c, int h,
                                                   double delta, CtaShared& sh, double uqr)
{
  if (c < 1)
    return false;
  const double s = cta_pow2_of_max(View{R, 1, c}, c, c, sh);
  const double is = 1.0 / s;
  const int64_t cc = static_cast<int64_t>(c) * c;
  double part = 0.0;
  for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
  {
    const double x = R[t] * is;
    part = fma(x, x, part);
  }
  const double fro2 = cta_sum(part, sh);
  if (!(fro2 > 0.0) || !isfinite(fro2))
    return false;
  for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
  {
    const int64_t i = t % c, j = t / c;
    if (i >= j)
      G[t] = G[t] * is * is;
  }
  double shift = 0.0;
  if (threadIdx.x == 0)
    shift = certify_tau(delta * is, fro2, c, h, CertOps<double>::u, uqr);
  __syncthreads();
  return cta_ldl_positive<double>(G, c, shift, sh);
}

// ---------------------------------------------------------------------------
// Mixed-precision one-sided Jacobi: the sweeps that do most of the rotating
// run in FP32, a df64 refinement restores FP64-level accuracy.
//   1. FP32 copy of src (m x n, m >= n) and V32 = I in fbuf
//      (m*n + n*n floats); FP32 Jacobi sweeps accumulate V32.
//   2. V = V32 * (3I - V32^T V32)/2 in FP64 (one Newton-Schulz step: V is
//      orthogonal to FP64 accuracy), in tmp (3 n*n doubles).
//   3. A = src * V (FP64 GEMM) -- nearly orthogonal columns.
//   4. df64 Jacobi sweeps on A (typically one or two: the first rotates by
//      ~1e-7, the next by ~1e-14 and stops the iteration); when Vout is given
//      it starts from V and accumulates the rotations.
// src stays readable throughout; fbuf may alias A (it is dead before step 3).
// Returns the df64 sweep count.
// ---------------------------------------------------------------------------
template <class Gemm>
__device__ __noinline__ int cta_jacobi_mixed(View src, int m, int n, double* A, int64_t lda, double* Vout,
                                int max_sweeps, int* converged, double* nrm, float* fbuf,
                                double* tmp, CtaShared& sh, Gemm gemm, double floor2 = 0.0)
{
  float* Af = fbuf;
  float* Vf = fbuf + static_cast<int64_t>(m) * n;
  const int64_t mn = static_cast<int64_t>(m) * n, nn = static_cast<int64_t>(n) * n;
  for (int64_t t = threadIdx.x; t < mn; t += blockDim.x)
    Af[t] = static_cast<float>(src(t % m, t / m));
  for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
    Vf[t] = (t % n == t / n) ? 1.0f : 0.0f;
  __syncthreads();
  // FP32 sweeps leave alone columns below ~1e-6 of the RMS column norm
  // (FP32 cannot resolve them; the high-precision sweeps do) and stop once the
  // rotations are ~3e-4 (the next sweep would reach FP32 resolution).
  float ss = 0.f;
  for (int64_t t = threadIdx.x; t < mn; t += blockDim.x)
    ss += Af[t] * Af[t];
  ss = cta_sum(ss, sh);
  const float floor32 = fmaxf(static_cast<float>(floor2), 1e-12f * ss / static_cast<float>(n));
  int conv32 = 0;
  cta_jacobi<float>(Af, m, n, m, Vf, n, 24, &conv32, reinterpret_cast<float*>(nrm), sh, floor32,
                    3e-4f);
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
  // 4. Polish in df64: A / 2^e split once, df64 sweeps, back to FP64.
  const double sc = cta_pow2_of_max(View{A, 1, lda}, m, n, sh);
  const double isc = 1.0 / sc;
  const int esc = pow2_exponent(sc);
  df64* Ad = reinterpret_cast<df64*>(A);
  for (int64_t t = threadIdx.x; t < mn; t += blockDim.x)
  {
    const int64_t e = (t % m) + (t / m) * lda;
    Ad[e] = df_split_pow2(A[e], -esc);
  }
  df64* Vdd = reinterpret_cast<df64*>(Vout);
  if (Vout)
    for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
      Vdd[t] = df_split_pow2(Vout[t], 0);
  __syncthreads();
  const int sweeps = cta_jacobi<df64>(Ad, m, n, lda, Vdd, n, max_sweeps, converged, nrm, sh,
                                      floor2 * isc * isc, kJacobiStopRel);
  for (int64_t t = threadIdx.x; t < mn; t += blockDim.x)
  {
    const int64_t e = (t % m) + (t / m) * lda;
    A[e] = df_join_pow2(Ad[e], esc);
  }
  if (Vout)
    for (int64_t t = threadIdx.x; t < nn; t += blockDim.x)
      Vout[t] = df_join_pow2(Vdd[t], 0);
  __syncthreads();
  return sweeps;
}

// C(i, j) = sum_p A(i, p) B(p, j) in df64 (FP64 in, FP64 out).  A and B are
// scaled by powers of two (exact) so the split never leaves FP32 range.
// tri and in-place use as cta_gemm (the same tiles, rows and slabs).
// 64x64 output tiles, 16-deep k slabs in shared memory (the df64 slabs reuse
// the CtaShared GEMM buffers, one df64 per double slot), 4x4 per thread.
__device__ __noinline__ void cta_gemm_df(int M, int N, int K, View A, View B, double* C, int64_t c_rs,
                            int64_t c_cs, CtaShared& sh, int tri = kTriNone)
{
  const int ea = pow2_exponent(cta_pow2_of_max(A, M, K, sh));
  const int eb = pow2_exponent(cta_pow2_of_max(B, K, N, sh));
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
      const int pstart = tri == kTriUpperA ? i0 : (tri == kTriLowerB ? j0 : 0);
      for (int p0 = pstart; p0 < K; p0 += 16)
      {
        __syncthreads();
        for (int t = threadIdx.x; t < 16 * 64; t += blockDim.x)
        {
          const int kk = t / 64, ii = t % 64;
          const int gi = i0 + ii, gp = p0 + kk, gj = j0 + ii;
          as[kk][ii] = (gi < M && gp < K) ? df_split_pow2(A(gi, gp), -ea) : df64{0.0f, 0.0f};
          bs[kk][ii] = (gp < K && gj < N) ? df_split_pow2(B(gp, gj), -eb) : df64{0.0f, 0.0f};
        }
        __syncthreads();
        const int na = gemm_live(M - i0, ty, tri == kTriUpperA, p0 - i0);
        const int nb = gemm_live(N - j0, tx, tri == kTriLowerB, p0 - j0);
        const int kmax = K - p0 < 16 ? K - p0 : 16;
#pragma unroll 4
        for (int kk = 0; kk < kmax; ++kk)
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
            if (a < na)
            {
#pragma unroll
              for (int b = 0; b < 4; ++b)
                if (b < nb)
                  acc[a][b] = df_fma(av[a], bv[b], acc[a][b]);
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
            C[gi * c_rs + gj * c_cs] = df_join_pow2(acc[a][b], ea + eb);
        }
    }
  __syncthreads();
}

}  // namespace
}  // namespace ttg
