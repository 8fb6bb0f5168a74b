// Whole-GPU rounding of a few large TTs (or of many, by teams of CTAs).
//
// One cooperative launch, one CTA per SM; the CTAs work on one TT at a time
// and meet at a grid barrier between dependent phases.  Same algorithm and
// branch structure as round_tt (detail::round, round/tt_round.hpp:36-134),
// each step spread over the grid:
//   * Householder QR (qr_thin, types/tt_eigen_bridge.hpp:42-60): column l
//     belongs to CTA l mod P.  The owner of column j forms reflector j and
//     publishes it; after one barrier every CTA applies it to its own
//     columns.  Owned columns stay in shared memory when they fit.
//   * Q and Q [Uc; 0]: each CTA forms its own columns from the published
//     reflectors -- no barriers.
//   * One-sided Jacobi SVD: block-pair rounds.  Columns are cut into blocks
//     of b; in each round of the round-robin tournament over blocks a CTA
//     loads a block pair into shared memory, runs one local sweep over all
//     pairs of its 2b columns (cta_jacobi) and writes them back; a barrier
//     ends the round.  Outer sweeps stop when a sweep rotates nothing or its
//     largest relative rotation is below kJacobiStopRel.
//   * Contractions: 64x64 FP64 output tiles spread over the CTAs.
// QR, contractions and balancing are FP64.  The SVD is FP64 Jacobi on the
// plain path; on the mixed path FP32 sweeps do the bulk of the rotating and
// df64 sweeps (FP32 pipes) polish to FP64-level accuracy, as in the
// one-CTA-per-TT kernel.
//
// Every barrier wait is bounded (WideJob::wait_cycles, ~2 s by default): a CTA that gives up sets
// the shared error word, every other CTA sees it at its next barrier, and
// the kernel returns; the host reports TTG_ERR_TIMEOUT.
#include <cfloat>
#include <cstdint>

#include <cuda_runtime.h>

#include "ttg_device.cuh"
#include "ttg_device_df.cuh"
#include "ttg_job.h"
#include "ttg_kernels.h"
#include "ttg_ozaki.cuh"
#include "ttg_sweep_common.cuh"

namespace ttg
{

// Bounded barrier of the `count` CTAs of a team (the whole grid, or a group
// of it), by generation counter.  All CTAs are co-resident (cooperative
// launch).  Returns false once any CTA of the team timed out (after
// `limit` clock cycles of waiting).
__device__ bool grid_sync(GridBar* gb, unsigned int count, long long limit)
{
  __shared__ int ok_sh;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    int ok = 1;
    volatile unsigned int* genp = &gb->gen;
    volatile int* errp = &gb->err;
    const unsigned int g = *genp;
    __threadfence();
    if (atomicAdd(&gb->count, 1u) == count - 1)
    {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    }
    else
    {
      const long long t0 = clock64();
      while (*genp == g)
      {
        if (*errp)
          break;
        if (clock64() - t0 > limit)
        {
          atomicExch(&gb->err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*errp)
      ok = 0;
    ok_sh = ok;
  }
  __syncthreads();
  return ok_sh != 0;
}

// The team's barrier.  job.stall_waits (set only by the failure-path tests)
// counts one CTA more than the team holds, so that no barrier ever
// completes and every wait runs out after job.wait_cycles.
__device__ bool grid_sync(const WideJob& job)
{
  return grid_sync(job.bar, job.size + (job.stall_waits ? 1u : 0u), job.wait_cycles);
}

#define WSYNC()                 \
  do                            \
  {                             \
    if (!grid_sync(job)) \
      return false;             \
  } while (0)

struct WideSmem
{
  double* p;
  int64_t cap;  // doubles
  OzState* oz;  // TMEM accumulator and MMA barrier of this CTA (null: FP64 tiles only)
};

// dst[0..n) = src[0..n), spread over the grid.
__device__ void wide_copy(const WideJob& job, double* dst, const double* src, int64_t n)
{
  const int64_t stride = static_cast<int64_t>(job.size) * blockDim.x;
  for (int64_t t = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n; t += stride)
    dst[t] = src[t];
}

// C = A B over the grid, tile t on CTA t mod P: 128x64 sliced-BF16 tiles
// on the tensor cores (FP64-accurate, oz_tile) when the job allows them and
// K <= 512, else 64x64 FP64 tiles.  Returns false if a tensor-core wait
// timed out (the grid error word is set).
// fp64_only: FP64 tiles even when the sliced tensor-core tiles are on
// (products whose error bound is stated for FP64).
__device__ bool wide_gemm(const WideJob& job, int M, int N, int K, View A, View B, double* C,
                          int64_t c_rs, int64_t c_cs, WideSmem sm, CtaShared& sh,
                          bool fp64_only = false)
{
  if (!fp64_only && job.tc && sm.oz && K <= 512 &&
      static_cast<int64_t>(kOzSmemBytes) <= sm.cap * 8)
  {
    const int tm = (M + kOzM - 1) / kOzM, tn = (N + kOzN - 1) / kOzN;
    bool ok = true;
    for (int t = job.rank; t < tm * tn && ok; t += job.size)
      ok = oz_tile((t / tn) * kOzM, (t % tn) * kOzN, M, N, K, A, B, C, c_rs, c_cs,
                   reinterpret_cast<uint8_t*>(sm.p), *sm.oz, sh);
    if (!ok && threadIdx.x == 0)
      atomicExch(&job.bar->err, 1);
    return ok;
  }
  const int tm = (M + 63) / 64, tn = (N + 63) / 64;
  for (int t = job.rank; t < tm * tn; t += job.size)
    cta_gemm_tile((t / tn) * 64, (t % tn) * 64, M, N, K, A, B, C, c_rs, c_cs, sh, kTriNone);
  __syncthreads();
  return true;
}

// Householder QR of X (h x c), column-distributed.  Reflector tails go to
// job.W (column-major, ld h), scales to job.tau, R (k x c, column-major,
// ld k) to job.R.  Returns k = min(h, c); false in *ok on a barrier failure.
__device__ int wide_qr(const WideJob& job, View X, int h, int c, WideSmem sm, CtaShared& sh,
                       bool* ok)
{
  const int P = job.size, me = job.rank;
  const int k = h < c ? h : c;
  const int nown = (c - me + P - 1) / P > 0 ? (c - me + P - 1) / P : 0;
  const bool in_smem = static_cast<int64_t>(nown) * h <= sm.cap;
  auto col = [&](int l) -> double* {
    return in_smem ? sm.p + static_cast<int64_t>(l / P) * h : job.W + static_cast<int64_t>(l) * h;
  };
  for (int l = me; l < c; l += P)
  {
    double* y = col(l);
    for (int i = threadIdx.x; i < h; i += blockDim.x)
      y[i] = X(i, l);
  }
  __syncthreads();
  // Reflector j from column j (its owner has applied H_0..H_{j-1} to it),
  // published to W and tau.
  auto reflect = [&](int j) {
    const int len = h - j;
    double* x = col(j) + j;
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
    double* pub = job.W + static_cast<int64_t>(j) * h + j;
    for (int i = 1 + threadIdx.x; i < len; i += blockDim.x)
    {
      x[i] *= inv;
      pub[i] = x[i];
    }
    if (threadIdx.x == 0)
    {
      x[0] = beta;
      pub[0] = beta;
      job.tau[j] = t;
    }
  };
  // y <- H_j y on rows j.. of an owned column.
  auto apply = [&](int j, double t, const double* v, int l) {
    const int len = h - j;
    double* y = col(l) + j;
    double part = 0.0;
    for (int i = threadIdx.x; i < len; i += blockDim.x)
      part += (i == 0 ? 1.0 : v[i]) * y[i];
    const double dot = cta_sum(part, sh) * t;
    for (int i = threadIdx.x; i < len; i += blockDim.x)
      y[i] -= dot * (i == 0 ? 1.0 : v[i]);
    __syncthreads();
  };
  if (k > 0 && me == 0)
    reflect(0);
  for (int j = 0; j < k; ++j)
  {
    if (!grid_sync(job))
    {
      *ok = false;
      return k;
    }
    const double t = job.tau[j];
    const double* v = job.W + static_cast<int64_t>(j) * h + j;
    // Look-ahead: the owner of column j+1 brings it up to date and forms
    // reflector j+1 first (the next barrier waits for it), then updates
    // its other columns.
    const int nj = j + 1;
    const bool own_next = nj < k && nj % P == me;
    if (own_next)
    {
      if (t != 0.0)
        apply(j, t, v, nj);
      reflect(nj);
    }
    if (t != 0.0)
      for (int l = me; l < c; l += P)
        if (l > j && !(own_next && l == nj))
          apply(j, t, v, l);
  }
  // R columns from their owners.
  for (int l = me; l < c; l += P)
  {
    const double* y = col(l);
    for (int i = threadIdx.x; i < k; i += blockDim.x)
      job.R[i + static_cast<int64_t>(l) * k] = (i <= l) ? y[i] : 0.0;
  }
  if (!grid_sync(job))
    *ok = false;
  return k;
}

// Column l (l mod P == this CTA) of H_0 ... H_{kref-1} [B(:, l); 0] into
// out(i, l) = out[i*o_rs + l*o_cs], for l < ncols; B column-major (nb x
// ncols, ld nb), nb <= h.  y is a length-h work column.
__device__ void wide_apply_q(const WideJob& job, int h, int kref, const double* B, int nb,
                             int ncols, double* out, int64_t o_rs, int64_t o_cs, bool eye,
                             WideSmem sm, CtaShared& sh)
{
  const int P = job.size, me = job.rank;
  for (int l = me; l < ncols; l += P)
  {
    double* y = (h <= sm.cap) ? sm.p : job.Ub + static_cast<int64_t>(l) * h;
    for (int i = threadIdx.x; i < h; i += blockDim.x)
      y[i] = eye ? (i == l ? 1.0 : 0.0) : (i < nb ? B[i + static_cast<int64_t>(l) * nb] : 0.0);
    __syncthreads();
    // For the identity start, H_j with j > l leaves e_l unchanged.
    const int jtop = eye ? (l < kref - 1 ? l : kref - 1) : kref - 1;
    for (int j = jtop; j >= 0; --j)
    {
      const double t = job.tau[j];
      if (t == 0.0)
        continue;
      const double* v = job.W + static_cast<int64_t>(j) * h + j;
      double* yj = y + j;
      const int len = h - j;
      double part = 0.0;
      for (int i = threadIdx.x; i < len; i += blockDim.x)
        part += (i == 0 ? 1.0 : v[i]) * yj[i];
      const double dot = cta_sum(part, sh) * t;
      for (int i = threadIdx.x; i < len; i += blockDim.x)
        yj[i] -= dot * (i == 0 ? 1.0 : v[i]);
      __syncthreads();
    }
    for (int i = threadIdx.x; i < h; i += blockDim.x)
      out[i * o_rs + static_cast<int64_t>(l) * o_cs] = y[i];
    __syncthreads();
  }
}

// One-sided Jacobi of A (p x q, column-major, lda; element type E = float,
// double or df64) in block-pair rounds of b columns over the grid; V (q x q,
// ld q) accumulates the rotations when non-null.  Stops after a sweep
// without rotations or whose largest relative rotation is below stop_rel.
template <class E>
__device__ bool wide_jacobi(const WideJob& job, E* A, int p, int q, int64_t lda, E* V, int b,
                            typename JOps<E>::S floor2, typename JOps<E>::S stop_rel,
                            int max_sweeps, WideSmem sm, CtaShared& sh, int* sweeps_out,
                            int* conv)
{
  using S = typename JOps<E>::S;
  const int P = job.size, me = job.rank;
  const int nblk = (q + b - 1) / b;
  const int NB = nblk + (nblk & 1), npairs = NB / 2;
  E* As = reinterpret_cast<E*>(sm.p);
  E* Vs = As + static_cast<int64_t>(p) * 2 * b;
  S* ns = reinterpret_cast<S*>(Vs + (V ? static_cast<int64_t>(q) * 2 * b : 0));
  if (me == 0)
    for (int s = threadIdx.x; s < max_sweeps; s += blockDim.x)
    {
      job.sweep_rot[s] = 0u;
      job.sweep_rel[s] = 0u;
    }
  WSYNC();
  *conv = 0;
  *sweeps_out = max_sweeps;
  if (q < 2)
  {
    *conv = 1;
    *sweeps_out = 0;
    return true;
  }
  for (int sw = 0; sw < max_sweeps; ++sw)
  {
    for (int rr = 0; rr < NB - 1; ++rr)
    {
      for (int t = me; t < npairs; t += P)
      {
        const int bp = (t == 0) ? 0 : ((t - 1 + rr) % (NB - 1)) + 1;
        const int bq = ((NB - 2 - t + rr) % (NB - 1)) + 1;
        const int c0 = bp * b, c1 = bq * b;
        const int np = c0 < q ? (q - c0 < b ? q - c0 : b) : 0;
        const int nq = c1 < q ? (q - c1 < b ? q - c1 : b) : 0;
        const int nc = np + nq;
        if (nc < 2)
          continue;
        auto gcol = [&](int j) { return j < np ? c0 + j : c1 + (j - np); };
        // Warp per column, lanes down the rows (no integer division).
        const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
        for (int j = wp; j < nc; j += kWarps)
        {
          const E* src = A + static_cast<int64_t>(gcol(j)) * lda;
          E* dst = As + static_cast<int64_t>(j) * p;
          for (int i = lane; i < p; i += 32)
            dst[i] = src[i];
          if (V)
          {
            const E* vs = V + static_cast<int64_t>(gcol(j)) * q;
            E* vd = Vs + static_cast<int64_t>(j) * q;
            for (int i = lane; i < q; i += 32)
              vd[i] = vs[i];
          }
        }
        __syncthreads();
        int lconv = 1;
        float mr = 0.0f;
        cta_jacobi<E>(As, p, nc, p, V ? Vs : nullptr, q, 1, &lconv, ns, sh, floor2, S(0), &mr, q);
        if (!lconv && threadIdx.x == 0)
        {
          atomicOr(&job.sweep_rot[sw], 1u);
          atomicMax(&job.sweep_rel[sw], __float_as_uint(mr));
        }
        for (int j = wp; j < nc; j += kWarps)
        {
          E* dst = A + static_cast<int64_t>(gcol(j)) * lda;
          const E* src = As + static_cast<int64_t>(j) * p;
          for (int i = lane; i < p; i += 32)
            dst[i] = src[i];
          if (V)
          {
            E* vd = V + static_cast<int64_t>(gcol(j)) * q;
            const E* vs = Vs + static_cast<int64_t>(j) * q;
            for (int i = lane; i < q; i += 32)
              vd[i] = vs[i];
          }
        }
        __syncthreads();
      }
      WSYNC();
    }
    const unsigned int rot = *reinterpret_cast<volatile unsigned int*>(&job.sweep_rot[sw]);
    const unsigned int rel = *reinterpret_cast<volatile unsigned int*>(&job.sweep_rel[sw]);
    if (!rot || __uint_as_float(rel) < static_cast<float>(stop_rel))
    {
      *conv = 1;
      *sweeps_out = sw + 1;
      return true;
    }
  }
  return true;
}

// Grid-stride loop bounds of this thread.
#define WIDE_FOR(e, n)                                                                   \
  for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < (n); \
       e += static_cast<int64_t>(job.size) * blockDim.x)

// The SVD step of the mixed path over the grid, as cta_jacobi_mixed:
// FP32 block-pair sweeps on an FP32 copy of src (p x q) accumulating V32,
// two Newton-Schulz steps V <- V (3I - V^T V)/2 in FP64, A = src V
// (FP64 tiles), then df64 block-pair sweeps on A / 2^e (and on V when
// with_v) until the rotations fall below kJacobiStopRel.  A (double, p x
// q, ld p) and, when with_v, V (double, q x q) hold the result.  Returns
// the df64 sweep count in *sweeps.
__device__ bool wide_svd_mixed(const WideJob& job, View src, int p, int q, bool with_v,
                               double floor2, WideSmem sm, CtaShared& sh, int* sweeps, int* conv)
{
  const int me = job.rank;
  float* A32 = reinterpret_cast<float*>(job.Pb);
  float* V32 = reinterpret_cast<float*>(job.T1);
  const int64_t pq = static_cast<int64_t>(p) * q, qq = static_cast<int64_t>(q) * q;
  double part = 0.0;
  WIDE_FOR(e, pq)
  {
    const float x = static_cast<float>(src(e % p, e / p));
    A32[e] = x;
    part += static_cast<double>(x) * x;
  }
  WIDE_FOR(e, qq)
  V32[e] = (e % q == e / q) ? 1.0f : 0.0f;
  part = cta_sum(part, sh);
  if (threadIdx.x == 0)
    job.part[me] = part;
  if (me == 0 && threadIdx.x == 0)
    *job.umax = 0ull;
  WSYNC();
  double ss = 0.0;
  for (int i = 0; i < static_cast<int>(job.size); ++i)
    ss += job.part[i];
  const float floor32 = fmaxf(static_cast<float>(floor2), 1e-12f * static_cast<float>(ss / q));
  int sw32 = 0, cv32 = 0;
  if (!wide_jacobi<float>(job, A32, p, q, p, V32, 2 * job.jblock, floor32, 3e-4f,
                          job.max_sweeps < 24 ? job.max_sweeps : 24, sm, sh, &sw32, &cv32))
    return false;
  // Two Newton-Schulz steps V <- V (3I - V^T V)/2 in FP64 (M in F): the
  // FP32 rotations leave V32^T V32 - I at up to ~1e-5 for a few hundred
  // columns, one step squares that to ~1e-10, the second to FP64 level.
  double* Vd = job.T2;
  WIDE_FOR(e, qq)
  Vd[e] = static_cast<double>(V32[e]);
  WSYNC();
  for (int it = 0; it < 2; ++it)
  {
    double* Vin = it == 0 ? Vd : job.V;
    double* Vout = it == 0 ? job.V : Vd;
    if (!wide_gemm(job, q, q, q, View{Vin, q, 1}, View{Vin, 1, q}, job.F, 1, q, sm, sh))
      return false;
    WSYNC();
    WIDE_FOR(e, qq)
    job.F[e] = ((e % q == e / q) ? 1.5 : 0.0) - 0.5 * job.F[e];
    WSYNC();
    if (!wide_gemm(job, q, q, q, View{Vin, 1, q}, View{job.F, 1, q}, Vout, 1, q, sm, sh))
      return false;
    WSYNC();
  }
  // The result is in Vd (T2); V takes it.
  wide_copy(job, job.V, Vd, qq);
  WSYNC();
  if (!wide_gemm(job, p, q, q, src, View{job.V, 1, q}, job.A, 1, p, sm, sh))
    return false;
  WSYNC();
  // df64 polish on A / 2^e, 2^e <= max|A| < 2^(e+1) (bit-pattern max).
  {
    unsigned long long mx = 0ull;
    WIDE_FOR(e, pq)
    {
      const unsigned long long bits =
        static_cast<unsigned long long>(__double_as_longlong(job.A[e])) & 0x7fffffffffffffffull;
      mx = bits > mx ? bits : mx;
    }
    for (int o = 16; o > 0; o >>= 1)
    {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = y > mx ? y : mx;
    }
    if ((threadIdx.x & 31) == 0)
      atomicMax(job.umax, mx);
  }
  WSYNC();
  const int ex = static_cast<int>((*reinterpret_cast<volatile unsigned long long*>(job.umax) >> 52) &
                                  0x7ff);
  const double sc = (ex == 0 || ex == 0x7ff) ? 1.0 : __longlong_as_double(static_cast<long long>(ex) << 52);
  const double isc = 1.0 / sc;
  df64* Ad = reinterpret_cast<df64*>(job.A);
  df64* Vdd = reinterpret_cast<df64*>(job.V);
  WIDE_FOR(e, pq)
  Ad[e] = df_split_pow2(job.A[e], -pow2_exponent(sc));
  if (with_v)
  {
    WIDE_FOR(e, qq)
    Vdd[e] = df_split_pow2(job.V[e], 0);
  }
  WSYNC();
  if (!wide_jacobi<df64>(job, Ad, p, q, p, with_v ? Vdd : nullptr, job.jblock, floor2 * isc * isc,
                         kJacobiStopRel, job.max_sweeps, sm, sh, sweeps, conv))
    return false;
  WIDE_FOR(e, pq)
  job.A[e] = df_join_pow2(Ad[e], pow2_exponent(sc));
  if (with_v)
  {
    WIDE_FOR(e, qq)
    job.V[e] = df_join_pow2(Vdd[e], 0);
  }
  WSYNC();
  return true;
}

// Singular values = column norms of A (p x q); sorted/ord/r_new by CTA 0.
// Ends with a barrier; returns false on a barrier failure.
__device__ bool wide_truncate(const WideJob& job, const double* A, int p, int q, int64_t lda,
                              double delta, TTInfo& T, BondStat* bs, CtaShared& sh)
{
  const int P = job.size, me = job.rank;
  for (int j = me; j < q; j += P)
  {
    const double* a = A + static_cast<int64_t>(j) * lda;
    double s = 0.0;
    for (int i = threadIdx.x; i < p; i += blockDim.x)
      s += a[i] * a[i];
    s = cta_sum(s, sh);
    if (threadIdx.x == 0)
      job.sig[j] = sqrt(s);
  }
  WSYNC();
  if (me == 0)
  {
    cta_argsort_desc(job.sig, q, job.ord, job.sorted);
    if (threadIdx.x == 0)
    {
      job.ival[0] = trunc_rank_serial(job.sorted, q, delta, job.max_rank);
      if (!finite(job.sorted[0]))
        set_status(T, kStatusNan);
    }
    __syncthreads();
    record_bond(bs, job.sorted, q, job.ival[0]);
  }
  WSYNC();
  return true;
}

// Norm balancing (round/tt_round.hpp:65-124) over the grid: core k on CTA
// k mod P for the column norms and for the scaling; every CTA forms the
// geometric mean from all norms in the same order.
__device__ bool wide_balance(const WideJob& job, double* ar, CoreSlot* S, int d, CtaShared& sh)
{
  const int P = job.size, me = job.rank;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t base = 0;
  for (int k = 0; k < d - 1; ++k)
  {
    const int h = S[k].r * S[k].n, c = S[k].rp;
    if (k % P == me)
    {
      const double* p = ar + S[k].off;
      for (int col = w; col < c; col += kWarps)
      {
        double s = 0.0;
        for (int i = lane; i < h; i += 32)
          s += p[static_cast<int64_t>(i) * c + col] * p[static_cast<int64_t>(i) * c + col];
        s = warp_sum(s);
        if (lane == 0)
          job.cn[base + col] = sqrt(s);
      }
    }
    base += c;
  }
  WSYNC();
  double my_log = 0.0, my_cnt = 0.0;
  for (int64_t i = threadIdx.x; i < base; i += blockDim.x)
  {
    const double nc = job.cn[i];
    if (nc > 0.0)
    {
      my_log += log(nc);
      my_cnt += 1.0;
    }
  }
  const double tot_log = cta_sum(my_log, sh);
  const double tot_cnt = cta_sum(my_cnt, sh);
  if (tot_cnt <= 0.0)
    return true;
  const double geo = exp(tot_log / tot_cnt);
  base = 0;
  int64_t prev_base = 0;
  for (int k = 0; k < d; ++k)
  {
    const int r = S[k].r, n = S[k].n, c = S[k].rp;
    constexpr int kFactorCap = 16 * (64 + 1);  // doubles in each GEMM staging tile
    if (k % P == me && r <= kFactorCap && c <= kFactorCap)
    {
      // This core's row and column factors, once each, in the CTA's GEMM
      // staging tiles (free here): 1 / scl of bond k-1 per row block a,
      // scl = geo / nc of bond k per column (the reference divides by scl:
      // the same up to the last bit).
      double* rf = &sh.gemm_a[0][0];
      double* cf = &sh.gemm_b[0][0];
      for (int a = threadIdx.x; a < r; a += blockDim.x)
      {
        const double nr = k >= 1 ? job.cn[prev_base + a] : 0.0;
        rf[a] = nr > 0.0 ? nr / geo : 1.0;
      }
      for (int b = threadIdx.x; b < c; b += blockDim.x)
      {
        const double nc = k <= d - 2 ? job.cn[base + b] : 0.0;
        cf[b] = nc > 0.0 ? geo / nc : 1.0;
      }
      __syncthreads();
      int cg = 1;  // lanes per row: a power of two >= c, at most 32
      while (cg < c && cg < 32)
        cg <<= 1;
      const int rpw = 32 / cg, lb = lane & (cg - 1);
      double* p = ar + S[k].off;
      for (int row = w * rpw + lane / cg; row < r * n; row += kWarps * rpw)
      {
        const double f = rf[row / n];
        double* x = p + static_cast<int64_t>(row) * c;
        for (int b = lb; b < c; b += cg)
          x[b] *= f * cf[b];
      }
      __syncthreads();
    }
    else if (k % P == me)
    {
      double* p = ar + S[k].off;
      const int64_t sz = static_cast<int64_t>(r) * n * c;
      for (int64_t t = threadIdx.x; t < sz; t += blockDim.x)
      {
        const int a = static_cast<int>(t / (static_cast<int64_t>(n) * c));
        const int b = static_cast<int>(t % c);
        double x = p[t];
        if (k >= 1)
        {
          const double nr = job.cn[prev_base + a];
          if (nr > 0.0)
            x /= geo / nr;
        }
        if (k <= d - 2)
        {
          const double nc = job.cn[base + b];
          if (nc > 0.0)
            x *= geo / nc;
        }
        p[t] = x;
      }
    }
    if (k <= d - 2)
    {
      prev_base = base;
      base += c;
    }
  }
  return true;
}

// Right-to-left QR sweep (right_qr_step, detail/orthogonalize.hpp:63-100)
// over cores d-1..1 of S.
__device__ bool wide_right_orth(const WideJob& job, CoreSlot* S, int d, WideSmem sm,
                                CtaShared& sh)
{
  double* ar = job.arena;
  const bool lead = (job.rank == 0 && threadIdx.x == 0);
  for (int k = d - 1; k >= 1; --k)
  {
    const int r = S[k].r, n = S[k].n, rp = S[k].rp;
    const int w = n * rp;
    const int hp = S[k - 1].r * S[k - 1].n;
    double* cs = ar + S[k].off;
    double* ps = ar + S[k - 1].off;
    bool ok = true;
    const int kk = wide_qr(job, View{cs, 1, w}, w, r, sm, sh, &ok);
    if (!ok)
      return false;
    // core_k <- Q^T (Q column-major w x kk is the core's row-major layout);
    // prev (hp x kk) = left_unfold(prev) R^T.
    wide_apply_q(job, w, kk, nullptr, 0, kk, cs, 1, w, true, sm, sh);
    if (!wide_gemm(job, hp, kk, r, View{ps, r, 1}, View{job.R, kk, 1}, job.Pb, kk, 1, sm, sh))
      return false;
    WSYNC();
    wide_copy(job, ps, job.Pb, static_cast<int64_t>(hp) * kk);
    if (lead)
    {
      set_ranks(S[k], kk, rp);
      set_ranks(S[k - 1], S[k - 1].r, kk);
    }
    WSYNC();
  }
  return true;
}

// Truncated SVD of X (h x c) over the grid, as left_svd of the per-TT
// kernel (detail/truncate.hpp:61-99 branches): *r_new_out, U in job.Ub
// (column-major, h x r_new), diag(s) V^T rows in job.F (row-major, r_new x
// c).  X must not alias the work buffers (A, W, R, V, F, Ub, Pb, T1, T2).
__device__ bool wide_left_svd(const WideJob& job, View X, int h, int c, double delta, TTInfo& T,
                              BondStat* bs, WideSmem sm, CtaShared& sh, int* r_new_out)
{
  const int me = job.rank;
  const bool lead = (me == 0 && threadIdx.x == 0);
  const int nsv = h < c ? h : c;
  const double floor2 = 1e-6 * delta * delta / static_cast<double>(nsv > 1 ? nsv : 1);
  int sweeps = 0, conv = 1, r_new = 1;
  // No-truncation certificate (cta_certify_from_gram) as in the per-TT
  // left_svd: tried when no bond statistics are asked for and max_rank
  // cannot cut below c; for h >= c the step then takes the QR route.
  const bool certify = bs == nullptr && h >= c && c >= 2 &&
                       (job.max_rank <= 0 || job.max_rank >= c);
  if (h >= 2 * c || certify)
  {
    bool ok = true;
    wide_qr(job, X, h, c, sm, sh, &ok);
    if (!ok)
      return false;
    bool certified = false;
    if (certify)
    {
      // G = R^T R (FP64) over the grid into job.A, then one CTA eliminates
      // it (FP64) and proves sigma_min(R) > delta; the decision reaches every
      // CTA through job.ival[1].  The QR here is FP64 on both paths.
      if (!wide_gemm(job, c, c, c, View{job.R, c, 1}, View{job.R, 1, c}, job.A, 1, c, sm, sh,
                     true))
        return false;
      WSYNC();
      if (me == 0)
      {
        const bool yes =
          cta_certify_from_gram(job.A, job.R, c, h, delta, sh, CertOps<double>::u);
        if (threadIdx.x == 0)
          job.ival[1] = yes ? 1 : 0;
      }
      WSYNC();
      certified = *reinterpret_cast<volatile const int*>(job.ival + 1) != 0;
    }
    if (certified)
    {
      // Every singular value is kept: U = Q (Uc = I in V), F = R.
      r_new = c;
      const int64_t cc = static_cast<int64_t>(c) * c;
      for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < cc;
           e += static_cast<int64_t>(job.size) * blockDim.x)
      {
        const int64_t i = e % c, j = e / c;
        job.V[e] = i == j ? 1.0 : 0.0;
        job.F[i * c + j] = job.R[e];
      }
      WSYNC();
      wide_apply_q(job, h, c, job.V, c, r_new, job.Ub, 1, h, false, sm, sh);
      WSYNC();
    }
    else
    {
      // A = R (c x c), then Jacobi.
      wide_copy(job, job.A, job.R, static_cast<int64_t>(c) * c);
      WSYNC();
      if (job.mixed)
      {
        if (!wide_svd_mixed(job, View{job.R, 1, c}, c, c, false, floor2, sm, sh, &sweeps, &conv))
          return false;
      }
      else if (!wide_jacobi<double>(job, job.A, c, c, c, nullptr, job.jblock, floor2,
                                    kJacobiStopRel, job.max_sweeps, sm, sh, &sweeps, &conv))
        return false;
      if (!wide_truncate(job, job.A, c, c, c, delta, T, bs, sh))
        return false;
      r_new = job.ival[0];
      // Uc (c x r_new) = A(:, ord) / s, into V.
      for (int j = me; j < r_new; j += job.size)
      {
        const double s = job.sorted[j];
        const double* a = job.A + static_cast<int64_t>(job.ord[j]) * c;
        for (int i = threadIdx.x; i < c; i += blockDim.x)
          job.V[i + static_cast<int64_t>(j) * c] = s > 0.0 ? a[i] / s : 0.0;
      }
      WSYNC();
      // F = Uc^T R (r_new x c, row-major); U = Q [Uc; 0] (h x r_new).
      if (!wide_gemm(job, r_new, c, c, View{job.V, c, 1}, View{job.R, 1, c}, job.F, c, 1, sm,
                     sh))
        return false;
      wide_apply_q(job, h, c, job.V, c, r_new, job.Ub, 1, h, false, sm, sh);
      WSYNC();
    }
  }
  else if (h >= c)
  {
    for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x;
         e < static_cast<int64_t>(h) * c; e += static_cast<int64_t>(job.size) * blockDim.x)
      job.A[e] = X(e % h, e / h);
    WSYNC();
    if (job.mixed)
    {
      if (!wide_svd_mixed(job, X, h, c, false, floor2, sm, sh, &sweeps, &conv))
        return false;
    }
    else if (!wide_jacobi<double>(job, job.A, h, c, h, nullptr, job.jblock, floor2,
                                  kJacobiStopRel, job.max_sweeps, sm, sh, &sweeps, &conv))
      return false;
    if (!wide_truncate(job, job.A, h, c, h, delta, T, bs, sh))
      return false;
    r_new = job.ival[0];
    for (int j = me; j < r_new; j += job.size)
    {
      const double s = job.sorted[j];
      const double* a = job.A + static_cast<int64_t>(job.ord[j]) * h;
      for (int i = threadIdx.x; i < h; i += blockDim.x)
        job.Ub[i + static_cast<int64_t>(j) * h] = s > 0.0 ? a[i] / s : 0.0;
    }
    WSYNC();
    // F = U^T X.
    if (!wide_gemm(job, r_new, c, h, View{job.Ub, h, 1}, X, job.F, c, 1, sm, sh))
      return false;
    WSYNC();
  }
  else
  {
    // Jacobi on X^T (c x h); V (h x h) accumulates and becomes U.
    const int64_t stride = static_cast<int64_t>(job.size) * blockDim.x;
    for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x;
         e < static_cast<int64_t>(c) * h; e += stride)
      job.A[e] = X(e / c, e % c);
    for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x;
         e < static_cast<int64_t>(h) * h; e += stride)
      job.V[e] = (e % h == e / h) ? 1.0 : 0.0;
    WSYNC();
    if (job.mixed)
    {
      if (!wide_svd_mixed(job, transposed(X), c, h, true, floor2, sm, sh, &sweeps, &conv))
        return false;
    }
    else if (!wide_jacobi<double>(job, job.A, c, h, c, job.V, job.jblock, floor2,
                                  kJacobiStopRel, job.max_sweeps, sm, sh, &sweeps, &conv))
      return false;
    if (!wide_truncate(job, job.A, c, h, c, delta, T, bs, sh))
      return false;
    r_new = job.ival[0];
    for (int j = me; j < r_new; j += job.size)
    {
      const int o = job.ord[j];
      for (int i = threadIdx.x; i < h; i += blockDim.x)
        job.Ub[i + static_cast<int64_t>(j) * h] = job.V[i + static_cast<int64_t>(o) * h];
      for (int i = threadIdx.x; i < c; i += blockDim.x)
        job.F[static_cast<int64_t>(j) * c + i] = job.A[i + static_cast<int64_t>(o) * c];
    }
    WSYNC();
  }
  if (lead)
  {
    if (!conv)
      set_status(T, kStatusNotConverged);
    if (sweeps > T.sweeps)
      T.sweeps = sweeps;
  }
  *r_new_out = r_new;
  return true;
}

// Norm, NaN and zero checks after the right-to-left sweep; *delta = the
// truncation threshold.  Returns 0 to continue, 1 when the TT is finished
// (NaN recorded or zeroed), -1 on a barrier failure.
__device__ int wide_norm_step(const WideJob& job, TTInfo& T, CoreSlot* S, int d, double nrm,
                              CtaShared& sh, double* delta)
{
  const bool lead = (job.rank == 0 && threadIdx.x == 0);
  if (lead)
    T.norm = nrm;
  if (!isfinite(nrm))
  {
    if (job.rank == 0)
      set_status(T, kStatusNan);
    return 1;
  }
  if (nrm == 0.0)
  {
    if (job.rank == 0)
      zero_tt(job.arena, S, d);
    return grid_sync(job) ? 1 : -1;
  }
  *delta = job.eps * nrm / sqrt(static_cast<double>(d - 1 > 1 ? d - 1 : 1));
  if (lead)
    T.delta = *delta;
  return 0;
}

// detail::round (gauge none) of TT tti over the whole grid.
__device__ bool wide_round_tt(const WideJob& job, int tti, WideSmem sm, CtaShared& sh)
{
  TTInfo& T = job.tts[tti];
  const int d = T.d;
  CoreSlot* S = job.slots + T.first;
  double* ar = job.arena;
  const bool lead = (job.rank == 0 && threadIdx.x == 0);
  if (d <= 1)
    return true;
  if (!wide_right_orth(job, S, d, sm, sh))
    return false;
  double delta = 0.0;
  const int st = wide_norm_step(job, T, S, d, core_norm(ar + S[0].off, core_size(S[0]), sh), sh,
                                &delta);
  if (st != 0)
    return st > 0;
  // Left-to-right truncated SVD sweep (svd_step, detail/truncate.hpp:61-99).
  for (int k = 0; k < d - 1; ++k)
  {
    const int r = S[k].r, n = S[k].n, c = S[k].rp;
    const int h = r * n;
    const int wn = S[k + 1].n * S[k + 1].rp;
    double* cs = ar + S[k].off;
    double* ns = ar + S[k + 1].off;
    BondStat* bs = job.bond_stats ? job.bond_stats + T.first + k : nullptr;
    int r_new = 1;
    if (!wide_left_svd(job, View{cs, c, 1}, h, c, delta, T, bs, sm, sh, &r_new))
      return false;
    // next (r_new x wn) = F right_unfold(next); core_k <- U (row-major).
    if (!wide_gemm(job, r_new, wn, c, View{job.F, c, 1}, View{ns, wn, 1}, job.Pb, wn, 1, sm, sh))
      return false;
    WSYNC();
    wide_copy(job, ns, job.Pb, static_cast<int64_t>(r_new) * wn);
    {
      const int64_t stride = static_cast<int64_t>(job.size) * blockDim.x;
      for (int64_t e = job.rank * static_cast<int64_t>(blockDim.x) + threadIdx.x;
           e < static_cast<int64_t>(h) * r_new; e += stride)
      {
        const int64_t i = e / r_new, j = e % r_new;
        cs[e] = job.Ub[i + j * h];
      }
    }
    if (lead)
    {
      set_ranks(S[k], r, r_new);
      set_ranks(S[k + 1], r_new, S[k + 1].rp);
    }
    WSYNC();
  }
  if (!wide_balance(job, ar, S, d, sh))
    return false;
  WSYNC();
  return true;
}

// round_right_canonical (round/tt_round.hpp:151-190) of TT tti over the
// whole grid: the left-to-right QR sweep (left_qr_step,
// detail/orthogonalize.hpp:35-60), the norm of the last core, then the
// right-to-left truncated SVD sweep (svd_step_right, detail/truncate.hpp:
// 114-166, a left step on the transposed unfolding), as round_tt of the
// per-TT kernel does for kJobRoundRight.  No balancing.
__device__ bool wide_round_right_tt(const WideJob& job, int tti, WideSmem sm, CtaShared& sh)
{
  TTInfo& T = job.tts[tti];
  const int d = T.d;
  CoreSlot* S = job.slots + T.first;
  double* ar = job.arena;
  const bool lead = (job.rank == 0 && threadIdx.x == 0);
  if (d <= 1)
    return true;
  for (int k = 0; k < d - 1; ++k)
  {
    const int r = S[k].r, n = S[k].n, rp = S[k].rp;
    const int h = r * n;
    const int wn = S[k + 1].n * S[k + 1].rp;
    double* cs = ar + S[k].off;
    double* ns = ar + S[k + 1].off;
    bool ok = true;
    const int kk = wide_qr(job, View{cs, rp, 1}, h, rp, sm, sh, &ok);
    if (!ok)
      return false;
    // core_k <- Q (h x kk, row-major); next (kk x wn) = R right_unfold(next),
    // R (kk x rp) column-major in job.R.
    wide_apply_q(job, h, kk, nullptr, 0, kk, cs, kk, 1, true, sm, sh);
    if (!wide_gemm(job, kk, wn, rp, View{job.R, 1, kk}, View{ns, wn, 1}, job.Pb, wn, 1, sm, sh))
      return false;
    WSYNC();
    wide_copy(job, ns, job.Pb, static_cast<int64_t>(kk) * wn);
    if (lead)
    {
      set_ranks(S[k], r, kk);
      set_ranks(S[k + 1], kk, S[k + 1].rp);
    }
    WSYNC();
  }
  double delta = 0.0;
  const int st =
    wide_norm_step(job, T, S, d, core_norm(ar + S[d - 1].off, core_size(S[d - 1]), sh), sh, &delta);
  if (st != 0)
    return st > 0;
  for (int k = d - 1; k >= 1; --k)
  {
    const int r = S[k].r, n = S[k].n, rp = S[k].rp;
    const int w = n * rp;
    const int hp = S[k - 1].r * S[k - 1].n;
    double* cs = ar + S[k].off;
    double* ps = ar + S[k - 1].off;
    int r_new = 1;
    if (!wide_left_svd(job, View{cs, 1, w}, w, r, delta, T, nullptr, sm, sh, &r_new))
      return false;
    // prev (hp x r_new) = left_unfold(prev) F^T, F (r_new x r) row-major in
    // job.F; core_k <- U^T, whose row-major layout is U's column-major one.
    if (!wide_gemm(job, hp, r_new, r, View{ps, r, 1}, View{job.F, 1, r}, job.Pb, r_new, 1, sm, sh))
      return false;
    WSYNC();
    wide_copy(job, ps, job.Pb, static_cast<int64_t>(hp) * r_new);
    wide_copy(job, cs, job.Ub, static_cast<int64_t>(w) * r_new);
    if (lead)
    {
      set_ranks(S[k], r_new, rp);
      set_ranks(S[k - 1], S[k - 1].r, r_new);
    }
    WSYNC();
  }
  return true;
}

// Streaming apply-round (build_streaming_matvec / _matmat,
// detail/streaming_apply.hpp:39-202, fused cores detail/fused_apply_core.hpp:
// 33-272) over the whole grid: right-orthogonalise A and X, then per core
// C = F x A_k x X_k (two contractions and two permutations, never the full
// product TT) and a truncated SVD of C, F <- diag(s) V^T.  Same steps as
// stream_tt of the per-TT kernel.
__device__ bool wide_stream_tt(const WideJob& job, int item, WideSmem sm, CtaShared& sh)
{
  double* ar = job.arena;
  TTInfo& TA = job.tts[job.a_idx[item]];
  TTInfo& TX = job.tts[job.b_idx[item]];
  TTInfo& TO = job.tts[job.out_idx[item]];
  CoreSlot* SA = job.slots + TA.first;
  CoreSlot* SX = job.slots + TX.first;
  CoreSlot* SO = job.slots + TO.first;
  const int d = TA.d;
  const bool lead = (job.rank == 0 && threadIdx.x == 0);
  if (!wide_right_orth(job, SA, d, sm, sh) || !wide_right_orth(job, SX, d, sm, sh))
    return false;
  const double nA = core_norm(ar + SA[0].off, core_size(SA[0]), sh);
  const double nX = core_norm(ar + SX[0].off, core_size(SX[0]), sh);
  double delta = 0.0;
  const int st = wide_norm_step(job, TO, SO, d, nA * nX, sh, &delta);
  if (st != 0)
    return st > 0;
  if (lead)
    job.Fs[0] = 1.0;
  WSYNC();
  int alpha = 1;
  for (int k = 0; k < d; ++k)
  {
    const int a = SA[k].r, b = SA[k].rp;
    const int m = SA[k].m;
    const int p = SA[k].n / m;
    const int sx = SX[k].r, bx = SX[k].rp;
    const int nout = SX[k].n / p;
    const int64_t mpb = static_cast<int64_t>(m) * p * b;
    // Fp (alpha*sx x a): Fp[(al*sx + ax), aa] = F[al, aa*sx + ax].
    double* Fp = job.S1;
    WIDE_FOR(t, static_cast<int64_t>(alpha) * sx * a)
    {
      const int aa = static_cast<int>(t % a);
      const int64_t row = t / a;
      const int al = static_cast<int>(row / sx), ax = static_cast<int>(row % sx);
      Fp[t] = job.Fs[static_cast<int64_t>(al) * a * sx + static_cast<int64_t>(aa) * sx + ax];
    }
    WSYNC();
    // G1 (alpha*sx x m*p*b) = Fp A_k.
    double* G1 = job.S2;
    if (!wide_gemm(job, alpha * sx, static_cast<int>(mpb), a, View{Fp, a, 1},
                   View{ar + SA[k].off, mpb, 1}, G1, mpb, 1, sm, sh))
      return false;
    WSYNC();
    // G1p ((al, i, bb) x (ax, q)).
    const int64_t g1p_rows = static_cast<int64_t>(alpha) * m * b;
    const int64_t g1p_cols = static_cast<int64_t>(sx) * p;
    double* G1p = job.S1;
    WIDE_FOR(t, g1p_rows * g1p_cols)
    {
      const int64_t row = t / g1p_cols, col = t % g1p_cols;
      const int bb = static_cast<int>(row % b);
      const int i = static_cast<int>((row / b) % m);
      const int al = static_cast<int>(row / (static_cast<int64_t>(b) * m));
      const int ax = static_cast<int>(col / p), q = static_cast<int>(col % p);
      G1p[t] = G1[(static_cast<int64_t>(al) * sx + ax) * mpb +
                  (static_cast<int64_t>(i) * p + q) * b + bb];
    }
    WSYNC();
    // C2 ((al,i,bb) x (j,bx')) = G1p X_k.
    const int64_t c2_cols = static_cast<int64_t>(nout) * bx;
    double* C2 = job.S2;
    if (!wide_gemm(job, static_cast<int>(g1p_rows), static_cast<int>(c2_cols),
                   static_cast<int>(g1p_cols), View{G1p, g1p_cols, 1},
                   View{ar + SX[k].off, c2_cols, 1}, C2, c2_cols, 1, sm, sh))
      return false;
    WSYNC();
    // Cj (al, i, j, bb, bx') row-major.
    double* Cj = C2;
    if (nout > 1)
    {
      Cj = job.S1;
      WIDE_FOR(t, g1p_rows * c2_cols)
      {
        const int bxx = static_cast<int>(t % bx);
        const int bb = static_cast<int>((t / bx) % b);
        const int j = static_cast<int>((t / (static_cast<int64_t>(bx) * b)) % nout);
        const int64_t ai = t / (static_cast<int64_t>(bx) * b * nout);  // al*m + i
        Cj[t] = C2[(ai * b + bb) * c2_cols + static_cast<int64_t>(j) * bx + bxx];
      }
      WSYNC();
    }
    const int hrows = alpha * m * nout;
    const int ccols = b * bx;
    double* os = ar + SO[k].off;
    if (k == d - 1)
    {
      wide_copy(job, os, Cj, static_cast<int64_t>(hrows) * ccols);
      if (lead)
        set_ranks(SO[k], alpha, ccols);
      WSYNC();
      break;
    }
    int r_new = 1;
    if (!wide_left_svd(job, View{Cj, ccols, 1}, hrows, ccols, delta, TO, nullptr, sm, sh, &r_new))
      return false;
    // core_k <- U (row-major hrows x r_new); F <- diag(s) V^T.
    WIDE_FOR(e, static_cast<int64_t>(hrows) * r_new)
    {
      const int64_t i = e / r_new, j = e % r_new;
      os[e] = job.Ub[i + j * hrows];
    }
    wide_copy(job, job.Fs, job.F, static_cast<int64_t>(r_new) * ccols);
    if (lead)
      set_ranks(SO[k], alpha, r_new);
    WSYNC();
    alpha = r_new;
  }
  return true;
}

__global__ void __launch_bounds__(kThreads) wide_round_kernel(WideJob job)
{
  extern __shared__ double dyn_smem[];
  __shared__ CtaShared sh;
  __shared__ uint32_t tmem_base;
  __shared__ __align__(8) uint64_t mbar;
  OzState oz{0u, &mbar, 0u};
  if (job.tc)
  {
    // One CTA per SM: the whole TMEM (512 columns) is free for this CTA.
    if ((threadIdx.x >> 5) == 0)
      tc::tmem_alloc(&tmem_base, kOzTmemCols);
    if (threadIdx.x == 0)
      tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    oz.tmem = tmem_base;
  }
  const WideSmem sm{dyn_smem, job.smem_doubles, job.tc ? &oz : nullptr};
  // Teams: the grid splits into `teams` groups of equal size; group g owns
  // its own work buffers (one block of team_bytes each) and barrier word, and
  // rounds items g, g + teams, ... (the order is longest first).
  const int teams = job.teams > 0 ? job.teams : 1;
  const int tsize = static_cast<int>(gridDim.x) / teams;
  const int team = static_cast<int>(blockIdx.x) / tsize;
  __shared__ WideJob tj;  // the team's view of the job, read by every thread
  if (team < teams && threadIdx.x == 0)
  {
    tj = job;
    tj.rank = static_cast<int>(blockIdx.x) % tsize;
    tj.size = tsize;
    tj.bar = job.bar + team;
    const int64_t off = static_cast<int64_t>(team) * job.team_bytes;
    auto sh_ptr = [off](auto* p) { return reinterpret_cast<decltype(p)>(reinterpret_cast<char*>(p) + off); };
    tj.W = sh_ptr(job.W);
    tj.Ub = sh_ptr(job.Ub);
    tj.Pb = sh_ptr(job.Pb);
    tj.A = sh_ptr(job.A);
    tj.R = sh_ptr(job.R);
    tj.V = sh_ptr(job.V);
    tj.F = sh_ptr(job.F);
    tj.T1 = sh_ptr(job.T1);
    tj.T2 = sh_ptr(job.T2);
    tj.tau = sh_ptr(job.tau);
    tj.sig = sh_ptr(job.sig);
    tj.sorted = sh_ptr(job.sorted);
    tj.ord = sh_ptr(job.ord);
    tj.cn = sh_ptr(job.cn);
    tj.ival = sh_ptr(job.ival);
    tj.part = sh_ptr(job.part);
    tj.umax = sh_ptr(job.umax);
    tj.sweep_rot = sh_ptr(job.sweep_rot);
    tj.sweep_rel = sh_ptr(job.sweep_rel);
    tj.S1 = sh_ptr(job.S1);
    tj.S2 = sh_ptr(job.S2);
    tj.Fs = sh_ptr(job.Fs);
  }
  __syncthreads();
  if (team < teams)
  {
    const bool stream = job.kind == kJobStreamMatvec || job.kind == kJobStreamMatmat;
    for (int i = team; i < job.ntt; i += teams)
    {
      const int item = job.order ? job.order[i] : i;
      const bool ok = stream                        ? wide_stream_tt(tj, item, sm, sh)
                      : job.kind == kJobRoundRight ? wide_round_right_tt(tj, item, sm, sh)
                                                    : wide_round_tt(tj, item, sm, sh);
      if (!ok)
        break;
    }
  }
  if (job.tc)
  {
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
    {
      tc::fence_after_sync();
      tc::tmem_dealloc(oz.tmem, kOzTmemCols);
    }
  }
}

#undef WIDE_FOR
#undef WSYNC

cudaError_t launch_wide_round(const WideJob& job, int grid, cudaStream_t stream)
{
  WideJob j = job;
  void* args[] = {&j};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(wide_round_kernel), dim3(grid),
                                     dim3(kThreads), args,
                                     sizeof(double) * static_cast<size_t>(job.smem_doubles),
                                     stream);
}

cudaError_t wide_round_setup(int smem_doubles, int* max_grid)
{
  cudaError_t e = cudaFuncSetAttribute(wide_round_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(double) * smem_doubles));
  if (e != cudaSuccess)
    return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
    &per_sm, wide_round_kernel, kThreads, sizeof(double) * static_cast<size_t>(smem_doubles));
  if (e != cudaSuccess)
    return e;
  // One CTA per SM: the phases are latency-bound, more CTAs only add
  // barrier arrivals.
  *max_grid = per_sm >= 1 ? sms : 0;
  return cudaSuccess;
}

}  // namespace ttg
