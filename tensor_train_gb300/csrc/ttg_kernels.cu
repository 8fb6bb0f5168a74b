// FP64 TT sweep kernels for sm_103a.
//
// One CTA owns one tensor train for a whole sweep (persistent CTAs pull
// work items from an atomic queue, longest first).  Cores stay in their HBM
// slots for the whole call; each step reads a core, factors it in the CTA's
// scratch slab and writes the result back into the same slot.  Structure
// of a step follows the reference:
//   right_qr_step / left_qr_step     detail/orthogonalize.hpp:35-100
//   svd_step / svd_step_right        detail/truncate.hpp:61-166
//   detail::round                    round/tt_round.hpp:36-127
//   round_right_canonical            round/tt_round.hpp:151-183
//   build_streaming_matvec/matmat    detail/streaming_apply.hpp:39-202
//   fused_matvec/matmat_core         detail/fused_apply_core.hpp:33-272
//   matvec_core / matmat_core        apply/tt_matrix_apply.hpp:40-224
//   eval_at / eval_batch             algebra/tt_eval.hpp:32-112
//   inner (contract_inner_step)      algebra/tt_inner.hpp:33-47,
//                                    detail/contract.hpp:155-205
#include <cuda_runtime.h>

#include "ttg_device.cuh"
#include "ttg_device_df.cuh"
#include "ttg_wy_df.cuh"
#include "ttg_job.h"
#include "ttg_kernels.h"
#include "ttg_sweep_common.cuh"

namespace ttg
{

namespace
{


// The mixed path runs its contractions in df64 on the FP32 pipes.
struct GemmDf
{
  __device__ void operator()(int M, int N, int K, View A, View B, double* C, int64_t rs,
                             int64_t cs, CtaShared& sh) const
  {
    cta_gemm_df(M, N, K, A, B, C, rs, cs, sh);
  }
};

__device__ void gemm_sel(bool mixed, int M, int N, int K, View A, View B, double* C, int64_t rs,
                         int64_t cs, CtaShared& sh, int tri = kTriNone)
{
  if (mixed)
    cta_gemm_df(M, N, K, A, B, C, rs, cs, sh, tri);
  else
    cta_gemm(M, N, K, A, B, C, rs, cs, sh, tri);
}

// Dynamic shared memory of the CTA, used to stage the matrix a step works
// on when it fits (cap doubles).

// QR of X (h x c).  Q -> *W (h x k, column-major, ld h), R -> R (k x c,
// column-major, ld k), k = min(h, c).  The factorisation runs in shared
// memory when h*c fits there, else in Wg; *W tells the caller where Q is.
// qdst (mixed only, optional): Q is rounded to FP64 straight into qdst
// (h*k doubles; it may be X's storage, which is read before), and *W = qdst.
__device__ __noinline__ int qr_factor(View X, int h, int c, double* Wg, double* tau, double* R, Smem sm,
                         double** Wout, bool mixed, CtaShared& sh, double* qdst = nullptr)
{
  double* W = (static_cast<int64_t>(h) * c <= sm.cap) ? sm.p : Wg;
  *Wout = W;
  if (mixed)
  {
    // df64 factorisation of X / 2^e; R scaled back exactly; Q rounded to FP64.
    df64* Wd = reinterpret_cast<df64*>(W);
    df64* td = reinterpret_cast<df64*>(tau);
    const int e = pow2_exponent(cta_pow2_of_max(X, h, c, sh));
    cta_split_to_df(Wd, h, X, h, c, -e);
    __syncthreads();
    const int k = h < c ? h : c;
    // A panel in global memory is factored in blocks of kWyB reflectors
    // with the shared region as staging (it holds nothing else here).
    const bool wy = W != sm.p && c > kWyB && wy_stage_need(h) <= sm.cap;
    df64* stage = reinterpret_cast<df64*>(sm.p);
    df64* T = reinterpret_cast<df64*>(&sh.gemm_b[0][0]);
    if (wy)
      cta_householder_qr_df_wy(Wd, h, c, h, td, stage, T, sh);
    else
      cta_householder_qr_df(Wd, h, c, h, td, sh);
    cta_extract_r_df(R, Wd, k, c, h, e);
    if (wy)
      cta_form_q_df_wy(Wd, h, k, h, td, stage, T);
    else
      cta_form_q_df(Wd, h, k, h, td);
    if (qdst)
      *Wout = qdst;
    cta_join_from_df(qdst ? qdst : W, Wd, static_cast<int64_t>(h) * k);
    return k;
  }
  cta_copy_to_colmajor(W, h, X, h, c);
  __syncthreads();
  cta_householder_qr(W, h, c, h, tau, sh);
  const int k = h < c ? h : c;
  cta_extract_r(R, W, k, c, h);
  cta_form_q(W, h, k, h, tau);
  return k;
}

// Truncated SVD of X (h x c) = U S V^T, as used by svd_step
// (detail/truncate.hpp:61-99): returns r_new and
//   Ut (h x r_new, column-major, ld h): leading left singular vectors,
//   F  (r_new x c, row-major):         diag(s) * V^T leading rows.
// Branches as the reference: QR-condense when h >= 2c (truncate.hpp:76-85);
// otherwise decompose X directly -- by columns when h >= c, by rows (the
// transpose, accumulating V) when h < c.

// s_out (optional) receives the singular values, descending (c or h of them).
// f_upper (optional) is set when F is the upper-triangular R of the QR
// (a certified bond): the caller's absorption may skip its zero triangle.
__device__ __noinline__ int left_svd(View X, int h, int c, double delta, int max_rank, int max_sweeps,
                        bool mixed, Bump bump, Smem sm, double** Ut_out, double** F_out,
                        TTInfo& T, CtaShared& sh, BondStat* bs = nullptr,
                        double** s_out = nullptr, bool* f_upper = nullptr)
{
  if (f_upper)
    *f_upper = false;
  double* sig;
  double* sorted;
  int* ord;
  double* U;
  double* F;
  int sweeps = 0, conv = 1;
  // Columns below this squared norm hold < 1e-6 delta^2 all together, so
  // they always land in the truncated tail: Jacobi does not rotate them.
  const int nsv = h < c ? h : c;
  const double floor2 = 1e-6 * delta * delta / static_cast<double>(nsv > 1 ? nsv : 1);
  // No-truncation certificate (cta_certify_no_truncation): tried whenever no
  // singular value is asked for and max_rank cannot cut below c; for h >= c
  // the step then takes the QR route of the h >= 2c branch below.
  const bool certify = bs == nullptr && s_out == nullptr && h >= c && c >= 2 &&
                       (max_rank <= 0 || max_rank >= c);
  if (h >= 2 * c || certify)
  {
    double* W = bump.take(static_cast<int64_t>(h) * c);
    double* tau = bump.take(c);
    double* R = bump.take(static_cast<int64_t>(c) * c);
    double* A = bump.take(static_cast<int64_t>(c) * c);
    sig = bump.take(c);
    sorted = bump.take(c);
    ord = reinterpret_cast<int*>(bump.take(c));
    double* nrm = bump.take(c);
    double* Uc = bump.take(static_cast<int64_t>(c) * c);
    U = bump.take(static_cast<int64_t>(h) * c);
    F = bump.take(static_cast<int64_t>(c) * c);
    // Shared-memory staging: the Jacobi matrix first (it is touched most),
    // then the Householder panel when both fit.
    const int64_t cc = static_cast<int64_t>(c) * c, hc = static_cast<int64_t>(h) * c;
    if (cc + c <= sm.cap)
    {
      A = sm.p;
      nrm = sm.p + cc;
      if (hc + cc + c <= sm.cap)
        W = sm.p + cc + c;
    }
    const bool A_in_smem = (A == sm.p);
    df64* Wd = reinterpret_cast<df64*>(W);
    df64* td = reinterpret_cast<df64*>(tau);
    int eX = 0;  // mixed: the panel holds X / 2^eX
    // Mixed, panel in global memory: blocked Householder, Q formation and
    // Q application, staged in the shared region (free until the Jacobi /
    // certificate matrix A is written, and again once U is being formed).
    const bool wy = mixed && W != sm.p + cc + c && c > kWyB && wy_stage_need(h) <= sm.cap;
    df64* stage = reinterpret_cast<df64*>(sm.p);
    df64* Twy = reinterpret_cast<df64*>(&sh.gemm_b[0][0]);
    if (mixed)
    {
      eX = pow2_exponent(cta_pow2_of_max(X, h, c, sh));
      cta_split_to_df(Wd, h, X, h, c, -eX);
      __syncthreads();
      if (wy)
        cta_householder_qr_df_wy(Wd, h, c, h, td, stage, Twy, sh);
      else
        cta_householder_qr_df(Wd, h, c, h, td, sh);
      cta_extract_r_df(R, Wd, c, c, h, eX);
    }
    else
    {
      cta_copy_to_colmajor(W, h, X, h, c);
      __syncthreads();
      cta_householder_qr(W, h, c, h, tau, sh);
      cta_extract_r(R, W, c, c, h);
    }
    const bool certified =
      certify && (mixed ? cta_certify_no_truncation_df(Wd, h, c, h, ldexp(delta, -eX),
                                                       reinterpret_cast<df64*>(A), sh,
                                                       CertOps<df64>::u)
                        : cta_certify_no_truncation(R, c, h, delta, A, sh, CertOps<double>::u));
    int r_new = c;
    if (certified)
    {
      // sigma_min > delta: every singular value is kept, U = Q, F = R.
      for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
      {
        const int i = static_cast<int>(t % c), jj = static_cast<int>(t / c);
        Uc[t] = i == jj ? 1.0 : 0.0;
        F[static_cast<int64_t>(i) * c + jj] = R[t];
      }
      __syncthreads();
    }
    else
    {
      if (mixed)
      {
        float* fbuf =
          A_in_smem ? reinterpret_cast<float*>(A) : reinterpret_cast<float*>(bump.take(cc));
        double* tmp = bump.take(3 * cc);
        sweeps = cta_jacobi_mixed(View{R, 1, c}, c, c, A, c, nullptr, max_sweeps, &conv, nrm,
                                  fbuf, tmp, sh, GemmDf{}, floor2);
      }
      else
      {
        for (int64_t t = threadIdx.x; t < cc; t += blockDim.x)
          A[t] = R[t];
        __syncthreads();
        sweeps = cta_jacobi<double>(A, c, c, c, nullptr, 0, max_sweeps, &conv, nrm, sh, floor2,
                                    kJacobiStopRel);
      }
      cta_col_norms(A, c, c, c, sig);
      cta_argsort_desc(sig, c, ord, sorted);
      if (threadIdx.x == 0)
        sh.ival[0] = trunc_rank_serial(sorted, c, delta, max_rank);
      __syncthreads();
      r_new = sh.ival[0];
      for (int64_t t = threadIdx.x; t < static_cast<int64_t>(c) * r_new; t += blockDim.x)
      {
        const int i = static_cast<int>(t % c), jj = static_cast<int>(t / c);
        const double s = sorted[jj];
        Uc[t] = s > 0.0 ? A[i + static_cast<int64_t>(ord[jj]) * c] / s : 0.0;
      }
      __syncthreads();
      // F = Uc^T R  (= diag(s) V^T restricted to the kept rows).
      gemm_sel(mixed, r_new, c, c, View{Uc, c, 1}, View{R, 1, c}, F, c, 1, sh);
    }
    // U = Q [Uc; 0] by applying the reflectors.  A certified bond keeps
    // every column (Uc = I): U is Q itself, formed in place from the
    // reflectors (dorg2r order, which skips the zero structure of [I; 0]).
    if (certified)
    {
      if (mixed)
      {
        if (wy)
          cta_form_q_df_wy(Wd, h, c, h, td, stage, Twy);
        else
          cta_form_q_df(Wd, h, c, h, td);
        cta_join_from_df(W, Wd, hc);
      }
      else
        cta_form_q(W, h, c, h, tau);
      U = W;
    }
    else if (mixed)
    {
      df64* Ud = reinterpret_cast<df64*>(U);
      for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * r_new; t += blockDim.x)
      {
        const int i = static_cast<int>(t % h), jj = static_cast<int>(t / h);
        Ud[t] = i < c ? df_split_pow2(Uc[i + static_cast<int64_t>(jj) * c], 0) : df64{0.0f, 0.0f};
      }
      __syncthreads();
      if (wy)
        cta_apply_q_df_wy(Wd, h, c, h, td, Ud, r_new, h, stage, Twy);
      else
        cta_apply_q_df(Wd, h, c, h, td, Ud, r_new, h);
      cta_join_from_df(U, Ud, static_cast<int64_t>(h) * r_new);
    }
    else
    {
      for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * r_new; t += blockDim.x)
      {
        const int i = static_cast<int>(t % h), jj = static_cast<int>(t / h);
        U[t] = i < c ? Uc[i + static_cast<int64_t>(jj) * c] : 0.0;
      }
      __syncthreads();
      cta_apply_q(W, h, c, h, tau, U, r_new, h);
    }
    if (!certified)
      record_bond(bs, sorted, c, r_new);
    if (certified && f_upper)
      *f_upper = true;
    if (threadIdx.x == 0)
    {
      if (!certified && !finite(sorted[0]))
        set_status(T, kStatusNan);
      if (!conv)
        set_status(T, kStatusNotConverged);
      if (sweeps > T.sweeps)
        T.sweeps = sweeps;
    }
    __syncthreads();
    *Ut_out = U;
    *F_out = F;
    if (s_out)
      *s_out = sorted;
    return r_new;
  }
  if (h >= c)
  {
    double* A = bump.take(static_cast<int64_t>(h) * c);
    sig = bump.take(c);
    sorted = bump.take(c);
    ord = reinterpret_cast<int*>(bump.take(c));
    double* nrm = bump.take(c);
    U = bump.take(static_cast<int64_t>(h) * c);
    F = bump.take(static_cast<int64_t>(c) * c);
    const int64_t hc = static_cast<int64_t>(h) * c;
    bool A_in_smem = false;
    if (hc + c <= sm.cap)
    {
      A = sm.p;
      nrm = sm.p + hc;
      A_in_smem = true;
    }
    if (mixed)
    {
      float* fbuf = A_in_smem ? reinterpret_cast<float*>(A) : reinterpret_cast<float*>(bump.take(hc));
      double* tmp = bump.take(3 * static_cast<int64_t>(c) * c);
      sweeps = cta_jacobi_mixed(X, h, c, A, h, nullptr, max_sweeps, &conv, nrm, fbuf, tmp, sh,
                                GemmDf{}, floor2);
    }
    else
    {
      cta_copy_to_colmajor(A, h, X, h, c);
      __syncthreads();
      sweeps = cta_jacobi<double>(A, h, c, h, nullptr, 0, max_sweeps, &conv, nrm, sh, floor2,
                                  kJacobiStopRel);
    }
    cta_col_norms(A, h, c, h, sig);
    cta_argsort_desc(sig, c, ord, sorted);
    if (threadIdx.x == 0)
      sh.ival[0] = trunc_rank_serial(sorted, c, delta, max_rank);
    __syncthreads();
    const int r_new = sh.ival[0];
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * r_new; t += blockDim.x)
    {
      const int i = static_cast<int>(t % h), jj = static_cast<int>(t / h);
      const double s = sorted[jj];
      U[t] = s > 0.0 ? A[i + static_cast<int64_t>(ord[jj]) * h] / s : 0.0;
    }
    __syncthreads();
    // F = U^T X.
    gemm_sel(mixed, r_new, c, h, View{U, h, 1}, X, F, c, 1, sh);
    record_bond(bs, sorted, c, r_new);
    if (threadIdx.x == 0)
    {
      if (!finite(sorted[0]))
        set_status(T, kStatusNan);
      if (!conv)
        set_status(T, kStatusNotConverged);
      if (sweeps > T.sweeps)
        T.sweeps = sweeps;
    }
    __syncthreads();
    *Ut_out = U;
    *F_out = F;
    if (s_out)
      *s_out = sorted;
    return r_new;
  }
  // h < c: Jacobi on X^T (c x h), V (h x h) accumulates the rotations and
  // becomes U; the rotated columns are the rows of diag(s) V^T.
  double* A = bump.take(static_cast<int64_t>(c) * h);
  double* V = bump.take(static_cast<int64_t>(h) * h);
  sig = bump.take(h);
  sorted = bump.take(h);
  ord = reinterpret_cast<int*>(bump.take(h));
  double* nrm = bump.take(h);
  U = bump.take(static_cast<int64_t>(h) * h);
  F = bump.take(static_cast<int64_t>(h) * c);
  const int64_t ch = static_cast<int64_t>(c) * h, hh = static_cast<int64_t>(h) * h;
  bool A_in_smem = false;
  if (ch + h <= sm.cap)
  {
    A = sm.p;
    nrm = sm.p + ch;
    A_in_smem = true;
    if (ch + h + hh <= sm.cap)
      V = sm.p + ch + h;
  }
  if (mixed)
  {
    float* fbuf = A_in_smem ? reinterpret_cast<float*>(A) : reinterpret_cast<float*>(bump.take(ch));
    double* tmp = bump.take(3 * hh);
    sweeps = cta_jacobi_mixed(transposed(X), c, h, A, c, V, max_sweeps, &conv, nrm, fbuf, tmp, sh,
                              GemmDf{}, floor2);
  }
  else
  {
    cta_copy_to_colmajor(A, c, transposed(X), c, h);
    for (int64_t t = threadIdx.x; t < hh; t += blockDim.x)
      V[t] = (t % h == t / h) ? 1.0 : 0.0;
    __syncthreads();
    sweeps = cta_jacobi<double>(A, c, h, c, V, h, max_sweeps, &conv, nrm, sh, floor2,
                                kJacobiStopRel);
  }
  cta_col_norms(A, c, h, c, sig);
  cta_argsort_desc(sig, h, ord, sorted);
  if (threadIdx.x == 0)
    sh.ival[0] = trunc_rank_serial(sorted, h, delta, max_rank);
  __syncthreads();
  const int r_new = sh.ival[0];
  for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * r_new; t += blockDim.x)
  {
    const int i = static_cast<int>(t % h), jj = static_cast<int>(t / h);
    U[t] = V[i + static_cast<int64_t>(ord[jj]) * h];
  }
  for (int64_t t = threadIdx.x; t < static_cast<int64_t>(r_new) * c; t += blockDim.x)
  {
    const int jj = static_cast<int>(t / c), j = static_cast<int>(t % c);
    F[t] = A[j + static_cast<int64_t>(ord[jj]) * c];
  }
  record_bond(bs, sorted, h, r_new);
  if (threadIdx.x == 0)
  {
    if (!finite(sorted[0]))
      set_status(T, kStatusNan);
    if (!conv)
      set_status(T, kStatusNotConverged);
    if (sweeps > T.sweeps)
      T.sweeps = sweeps;
  }
  __syncthreads();
  *Ut_out = U;
  *F_out = F;
  if (s_out)
    *s_out = sorted;
  return r_new;
}

__device__ void cta_copy(double* dst, const double* src, int64_t n)
{
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x)
    dst[t] = src[t];
  __syncthreads();
}


// right_qr_step (detail/orthogonalize.hpp:63-100): QR of M^T (n*rp x r);
// r_eff = min(n*rp, r); L = R^T absorbed into prev.
__device__ __noinline__ void right_qr_step(double* ar, CoreSlot& cur, CoreSlot& prev, Bump bump, Smem sm,
                              bool mixed, CtaShared& sh)
{
  const int r = cur.r, n = cur.n, rp = cur.rp;
  const int w = n * rp;
  const int hp = prev.r * prev.n;
  double* cs = ar + cur.off;
  double* ps = ar + prev.off;
  double* W = bump.take(static_cast<int64_t>(w) * r);
  double* tau = bump.take(r);
  double* R = bump.take(static_cast<int64_t>(r) * r);
  double* P = bump.take(static_cast<int64_t>(hp) * r);
  double* Q;
  // Q (w x k column-major) is the new right_unfold(cur) (k x w row-major):
  // the mixed path writes it there directly.
  const int k = qr_factor(View{cs, 1, w}, w, r, W, tau, R, sm, &Q, mixed, sh, mixed ? cs : nullptr);
  // prev (hp x k) = left_unfold(prev) (hp x r) * L, L(a, e) = R(e, a)
  // (lower triangular); in place when the rank stays r.
  if (k == r)
    gemm_sel(mixed, hp, k, r, View{ps, r, 1}, View{R, k, 1}, ps, k, 1, sh, kTriLowerB);
  else
  {
    gemm_sel(mixed, hp, k, r, View{ps, r, 1}, View{R, k, 1}, P, k, 1, sh, kTriLowerB);
    cta_copy(ps, P, static_cast<int64_t>(hp) * k);
  }
  if (Q != cs)
    cta_copy(cs, Q, static_cast<int64_t>(w) * k);
  set_ranks(cur, k, rp);
  set_ranks(prev, prev.r, k);
  __syncthreads();
}

// left_qr_step (detail/orthogonalize.hpp:35-60).
__device__ __noinline__ void left_qr_step(double* ar, CoreSlot& cur, CoreSlot& next, Bump bump, Smem sm,
                             bool mixed, CtaShared& sh)
{
  const int r = cur.r, n = cur.n, rp = cur.rp;
  const int h = r * n;
  const int wn = next.n * next.rp;
  double* cs = ar + cur.off;
  double* ns = ar + next.off;
  double* W = bump.take(static_cast<int64_t>(h) * rp);
  double* tau = bump.take(rp);
  double* R = bump.take(static_cast<int64_t>(rp) * rp);
  double* P = bump.take(static_cast<int64_t>(rp) * wn);
  double* Q;
  const int k = qr_factor(View{cs, rp, 1}, h, rp, W, tau, R, sm, &Q, mixed, sh);
  // next (k x wn) = R (k x rp, upper triangular) * right_unfold(next)
  // (rp x wn); in place when the rank stays rp.
  if (k == rp)
    gemm_sel(mixed, k, wn, rp, View{R, 1, k}, View{ns, wn, 1}, ns, wn, 1, sh, kTriUpperA);
  else
  {
    gemm_sel(mixed, k, wn, rp, View{R, 1, k}, View{ns, wn, 1}, P, wn, 1, sh, kTriUpperA);
    cta_copy(ns, P, static_cast<int64_t>(k) * wn);
  }
  // cur row-major (h x k) <- Q column-major.
  cta_copy_to_rowmajor(cs, k, View{Q, 1, h}, h, k);
  set_ranks(cur, r, k);
  set_ranks(next, k, next.rp);
  __syncthreads();
}

// svd_step (detail/truncate.hpp:61-99).
__device__ __noinline__ void svd_step(const RoundJob& job, double* ar, CoreSlot& cur, CoreSlot& next,
                         double delta, Bump bump, Smem sm, TTInfo& T, CtaShared& sh,
                         BondStat* bs = nullptr)
{
  const int r = cur.r, n = cur.n, c = cur.rp;
  const int h = r * n;
  const int wn = next.n * next.rp;
  double* cs = ar + cur.off;
  double* ns = ar + next.off;
  double* P = bump.take(static_cast<int64_t>(c) * wn);
  double *U, *F;
  bool f_upper = false;
  const int r_new = left_svd(View{cs, c, 1}, h, c, delta, job.max_rank, job.max_sweeps,
                             job.mixed != 0, bump, sm, &U, &F, T, sh, bs, nullptr, &f_upper);
  // A certified bond keeps F = R (c x c, upper triangular): in place.
  if (f_upper)
    gemm_sel(job.mixed != 0, r_new, wn, c, View{F, c, 1}, View{ns, wn, 1}, ns, wn, 1, sh,
             kTriUpperA);
  else
  {
    gemm_sel(job.mixed != 0, r_new, wn, c, View{F, c, 1}, View{ns, wn, 1}, P, wn, 1, sh);
    cta_copy(ns, P, static_cast<int64_t>(r_new) * wn);
  }
  cta_copy_to_rowmajor(cs, r_new, View{U, 1, h}, h, r_new);
  set_ranks(cur, r, r_new);
  set_ranks(next, r_new, next.rp);
  __syncthreads();
}

// svd_step_right (detail/truncate.hpp:114-166) as a left step on M^T.
__device__ __noinline__ void svd_step_right(const RoundJob& job, double* ar, CoreSlot& cur, CoreSlot& prev,
                               double delta, Bump bump, Smem sm, TTInfo& T, CtaShared& sh)
{
  const int r = cur.r, n = cur.n, rp = cur.rp;
  const int w = n * rp;
  const int hp = prev.r * prev.n;
  double* cs = ar + cur.off;
  double* ps = ar + prev.off;
  double* P = bump.take(static_cast<int64_t>(hp) * r);
  double *U, *F;
  bool f_upper = false;
  const int r_new = left_svd(View{cs, 1, w}, w, r, delta, job.max_rank, job.max_sweeps,
                             job.mixed != 0, bump, sm, &U, &F, T, sh, nullptr, nullptr, &f_upper);
  // prev (hp x r_new) = left_unfold(prev) (hp x r) * F^T; a certified bond
  // keeps F = R (r x r), so F^T is lower triangular: in place.
  if (f_upper)
    gemm_sel(job.mixed != 0, hp, r_new, r, View{ps, r, 1}, View{F, 1, r}, ps, r_new, 1, sh,
             kTriLowerB);
  else
  {
    gemm_sel(job.mixed != 0, hp, r_new, r, View{ps, r, 1}, View{F, 1, r}, P, r_new, 1, sh);
    cta_copy(ps, P, static_cast<int64_t>(hp) * r_new);
  }
  cta_copy(cs, U, static_cast<int64_t>(w) * r_new);
  set_ranks(cur, r_new, rp);
  set_ranks(prev, prev.r, r_new);
  __syncthreads();
}




// One bond of soft_threshold (round/tt_soft_threshold.hpp:64-175): SVD of
// M = left_unfold(prev) right_unfold(cur) (h x c, FP64), s' = max(s - tau, 0);
// prev <- U diag(s') over the kept columns, cur <- V^T (the rows of
// diag(s) V^T that left_svd returns, divided by s).  All values at or below
// tau: both cores become rank-1 zero cores.  M = L R with an inner dimension
// of r has at most r nonzero singular values; any further ones are rounding
// noise (~1e-16 ||M||) and are never kept, so both cores fit their slots.
__device__ __noinline__ void soft_step(const RoundJob& job, double* ar, CoreSlot& prev,
                                       CoreSlot& cur, double tau, Bump bump, Smem sm, TTInfo& T,
                                       CtaShared& sh)
{
  const int rL = prev.r, np = prev.n, r = prev.rp, nc = cur.n, rR = cur.rp;
  const int h = rL * np, c = nc * rR;
  double* ps = ar + prev.off;
  double* cs = ar + cur.off;
  double* M = bump.take(static_cast<int64_t>(h) * c);
  cta_gemm(h, c, r, View{ps, r, 1}, View{cs, c, 1}, M, c, 1, sh);
  __syncthreads();
  double *U, *F, *s;
  const int rn = left_svd(View{M, c, 1}, h, c, 0.0, 0, job.max_sweeps, false, bump, sm, &U, &F,
                          T, sh, nullptr, &s);
  if (threadIdx.x == 0)
  {
    int keep = 0;
    for (int j = 0; j < rn; ++j)
      if (s[j] > tau)
        keep = j + 1;
    sh.ival[1] = keep < r ? keep : r;
  }
  __syncthreads();
  const int keep = sh.ival[1];
  if (keep == 0)
  {
    for (int64_t t = threadIdx.x; t < h; t += blockDim.x)
      ps[t] = 0.0;
    for (int64_t t = threadIdx.x; t < c; t += blockDim.x)
      cs[t] = 0.0;
    set_ranks(prev, rL, 1);
    set_ranks(cur, 1, rR);
    __syncthreads();
    return;
  }
  for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * keep; t += blockDim.x)
  {
    const int64_t i = t / keep;
    const int j = static_cast<int>(t % keep);
    ps[t] = U[i + static_cast<int64_t>(j) * h] * (s[j] - tau);
  }
  for (int64_t t = threadIdx.x; t < static_cast<int64_t>(keep) * c; t += blockDim.x)
    cs[t] = F[t] / s[t / c];
  set_ranks(prev, rL, keep);
  set_ranks(cur, keep, rR);
  __syncthreads();
}

// Norm balancing (round/tt_round.hpp:65-124).
__device__ __noinline__ void balance(double* ar, CoreSlot* S, int d, Bump bump, CtaShared& sh)
{
  int64_t total = 0;
  for (int k = 0; k < d - 1; ++k)
    total += S[k].rp;
  double* cn = bump.take(2 * (total + 1));  // norms -> scl, then 1 / scl
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double my_log = 0.0, my_cnt = 0.0;
  int64_t base = 0;
  for (int k = 0; k < d - 1; ++k)
  {
    const int h = S[k].r * S[k].n, c = S[k].rp;
    const double* p = ar + S[k].off;
    for (int col = w; col < c; col += kWarps)
    {
      double s = 0.0;
      for (int i = lane; i < h; i += 32)
        s += p[static_cast<int64_t>(i) * c + col] * p[static_cast<int64_t>(i) * c + col];
      s = warp_sum(s);
      const double nc = sqrt(s);
      if (lane == 0)
      {
        cn[base + col] = nc;
        if (nc > 0.0)
        {
          my_log += log(nc);
          my_cnt += 1.0;
        }
      }
    }
    base += c;
  }
  const double tot_log = cta_sum(my_log, sh);
  const double tot_cnt = cta_sum(my_cnt, sh);
  if (tot_cnt <= 0.0)
    return;
  const double geo = exp(tot_log / tot_cnt);
  // Per bond column: scl = geo / nc multiplies the column of left_unfold(c_k)
  // and 1 / scl the matching row of right_unfold(c_{k+1}) (the reference
  // divides by scl: the same up to the last bit), once per column here
  // rather than per element.
  double* inv = cn + total + 1;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
  {
    const double nc = cn[t];
    cn[t] = nc > 0.0 ? geo / nc : 1.0;
    inv[t] = nc > 0.0 ? nc / geo : 1.0;
  }
  __syncthreads();
  base = 0;
  int64_t prev_base = 0;
  for (int k = 0; k < d; ++k)
  {
    const int r = S[k].r, n = S[k].n, c = S[k].rp;
    double* p = ar + S[k].off;
    const int rows = r * n;
    // cg lanes per row (a power of two >= c, at most 32), 32 / cg rows per
    // warp at a time: no index division per element.
    int cg = 1;
    while (cg < c && cg < 32)
      cg <<= 1;
    const int rpw = 32 / cg, lb = lane & (cg - 1);
    const double* fc = k <= d - 2 ? cn + base : nullptr;
    const double* fr = k >= 1 ? inv + prev_base : nullptr;
    for (int row = w * rpw + lane / cg; row < rows; row += kWarps * rpw)
    {
      const double f = fr ? fr[row / n] : 1.0;
      double* x = p + static_cast<int64_t>(row) * c;
      for (int b = lb; b < c; b += cg)
        x[b] *= fc ? f * fc[b] : f;
    }
    if (k <= d - 2)
    {
      prev_base = base;
      base += c;
    }
  }
  __syncthreads();
}

// Scratch guard: the step needs `need` doubles of the CTA's slab.
__device__ bool fits(const RoundJob& job, int64_t need, TTInfo& T)
{
  if (need <= job.scratch_stride)
    return true;
  set_status(T, kStatusNoSpace);
  __syncthreads();
  return false;
}

__device__ int64_t balance_need(const CoreSlot* S, int d)
{
  int64_t total = 0;
  for (int k = 0; k < d - 1; ++k)
    total += S[k].rp;
  return a32(2 * (total + 1));
}

__device__ __noinline__ void round_tt(const RoundJob& job, int tti, double* scratch, Smem sm, CtaShared& sh,
                         double eps)
{
  TTInfo& T = job.tts[tti];
  const int d = T.d;
  CoreSlot* S = job.slots + T.first;
  double* ar = job.arena;
  if (d <= 1)
    return;
  // gauge none (detail::round) for plain, sketch-finishing and orthogonalise
  // jobs; round_right_canonical for kJobRoundRight, whose L->R QR sweep is
  // also left_orthogonalize (kJobLeftOrth).
  if (job.kind != kJobRoundRight && job.kind != kJobLeftOrth)
  {
    for (int k = d - 1; k >= 1; --k)
    {
      if (!fits(job, need_right_qr(S[k].r, static_cast<int64_t>(S[k].n) * S[k].rp,
                                   static_cast<int64_t>(S[k - 1].r) * S[k - 1].n), T))
        return;
      right_qr_step(ar, S[k], S[k - 1], Bump{scratch}, sm, job.mixed != 0, sh);
    }
    if (job.kind == kJobRightOrth)
      return;
    if (job.kind == kJobSoftThreshold)
    {
      // soft_threshold: eps carries tau.
      for (int k = d - 1; k >= 1; --k)
      {
        if (!fits(job, need_soft_step(static_cast<int64_t>(S[k - 1].r) * S[k - 1].n,
                                      static_cast<int64_t>(S[k].n) * S[k].rp), T))
          return;
        soft_step(job, ar, S[k - 1], S[k], eps, Bump{scratch}, sm, T, sh);
      }
      return;
    }
    const double nrm = core_norm(ar + S[0].off, core_size(S[0]), sh);
    if (threadIdx.x == 0)
      T.norm = nrm;
    if (!isfinite(nrm))
    {
      set_status(T, kStatusNan);
      return;
    }
    if (nrm == 0.0)
    {
      zero_tt(ar, S, d);
      return;
    }
    const double delta = eps * nrm / sqrt(static_cast<double>(d - 1 > 1 ? d - 1 : 1));
    if (threadIdx.x == 0)
      T.delta = delta;
    for (int k = 0; k < d - 1; ++k)
    {
      if (!fits(job, need_svd_step(static_cast<int64_t>(S[k].r) * S[k].n, S[k].rp,
                                   static_cast<int64_t>(S[k + 1].n) * S[k + 1].rp), T))
        return;
      svd_step(job, ar, S[k], S[k + 1], delta, Bump{scratch}, sm, T, sh,
               job.bond_stats ? job.bond_stats + T.first + k : nullptr);
    }
    if (!fits(job, balance_need(S, d), T))
      return;
    balance(ar, S, d, Bump{scratch}, sh);
    return;
  }
  // round_right_canonical.
  for (int k = 0; k < d - 1; ++k)
  {
    if (!fits(job, need_left_qr(static_cast<int64_t>(S[k].r) * S[k].n, S[k].rp,
                                static_cast<int64_t>(S[k + 1].n) * S[k + 1].rp), T))
      return;
    left_qr_step(ar, S[k], S[k + 1], Bump{scratch}, sm, job.mixed != 0, sh);
  }
  if (job.kind == kJobLeftOrth)
    return;
  const double nrm = core_norm(ar + S[d - 1].off, core_size(S[d - 1]), sh);
  if (threadIdx.x == 0)
    T.norm = nrm;
  if (!isfinite(nrm))
  {
    set_status(T, kStatusNan);
    return;
  }
  if (nrm == 0.0)
  {
    zero_tt(ar, S, d);
    return;
  }
  const double delta = eps * nrm / sqrt(static_cast<double>(d - 1 > 1 ? d - 1 : 1));
  if (threadIdx.x == 0)
    T.delta = delta;
  for (int k = d - 1; k >= 1; --k)
  {
    if (!fits(job, need_svd_step_right(static_cast<int64_t>(S[k].n) * S[k].rp, S[k].r,
                                       static_cast<int64_t>(S[k - 1].r) * S[k - 1].n), T))
      return;
    svd_step_right(job, ar, S[k], S[k - 1], delta, Bump{scratch}, sm, T, sh);
  }
}

// ---------------------------------------------------------------------------
// Randomised sketch rounding ("randomise-then-orthogonalise", Al Daas et al.,
// SIAM J. Sci. Comput. 2023) with an exact acceptance test.
//   1. ||X||^2 by the inner-product chain.
//   2. Right environments W_k (r_k x l_k) of X against a Gaussian TT with
//      bond ranks l_k (the sketch ranks, e.g. predicted by the rank model).
//   3. Left-to-right: Z = left_unfold(X_k) W_{k+1}, Q = qr(Z), X_k <- Q,
//      X_{k+1} <- (Q^T left_unfold(X_k)) right_unfold(X_{k+1}).  The result
//      Y is an orthogonal projection of X, so ||X - Y||^2 = ||X||^2 - ||Y||^2,
//      and ||Y|| = ||last core|| (the other cores are left-orthogonal).
//   4. Accept when ||X - Y|| <= eps/4 ||X||.  The final round of Y stays in
//      the range of the projection, so the two errors are orthogonal:
//      ||X - round(Y)||^2 = ||X - Y||^2 + ||Y - round(Y)||^2; Y is rounded
//      with eps_r = sqrt(eps^2 - rel^2) ||X|| / ||Y||, which keeps the total
//      within eps ||X|| and the per-bond threshold within 3% of the exact
//      rounder's.  Otherwise the inputs are restored from the pristine copy
//      and rounded exactly (the fallback that also validates the sketch).
// The acceptance test resolves ||X - Y||/||X|| down to ~1e-7 (FP64
// cancellation of the two squared norms): meant for eps >= 1e-6.
// ---------------------------------------------------------------------------
__device__ double sketch_gauss(uint64_t seed, uint64_t tti, uint64_t k, uint64_t i)
{
  uint64_t z = seed ^ (tti * 0x9E3779B97F4A7C15ull) ^ (k * 0xC2B2AE3D27D4EB4Full) ^
               (i * 0x165667B19E3779F9ull);
  auto mix = [](uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
  };
  const uint64_t a = mix(z), b = mix(z ^ 0xD6E8FEB86659FD93ull);
  const double u1 = (static_cast<double>(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = static_cast<double>(b >> 11) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

__device__ int sketch_rank_of(const RoundJob& job, const CoreSlot* S, int first, int k, int d)
{
  // bond k+1 (right of core k); clipped to [1, r_{k+1}]
  if (k >= d - 1)
    return 1;
  int l = job.sketch_ranks ? job.sketch_ranks[first + k] : S[k].rp;
  l = l < 1 ? 1 : l;
  return l > S[k].rp ? S[k].rp : l;
}

__device__ __noinline__ void round_sketch_tt(const RoundJob& job, int tti, double* scratch, Smem sm,
                                CtaShared& sh)
{
  TTInfo& T = job.tts[tti];
  const int d = T.d;
  CoreSlot* S = job.slots + T.first;
  double* ar = job.arena;
  const bool mixed = job.mixed != 0;
  if (d <= 1)
    return;
  int64_t rmax = 1, lsum = 0, lmax = 1, hmax = 1, nmax = 1, gsum = 0;
  for (int k = 0; k < d; ++k)
  {
    if (k >= 1)
      gsum += static_cast<int64_t>(S[k].r) * S[k].r;
    rmax = imax64(rmax, imax64(S[k].r, S[k].rp));
    hmax = imax64(hmax, static_cast<int64_t>(S[k].r) * S[k].n);
    nmax = imax64(nmax, S[k].n);
    if (k < d - 1)
    {
      const int l = sketch_rank_of(job, S, T.first, k, d);
      lsum += static_cast<int64_t>(S[k].rp) * l;
      lmax = imax64(lmax, l);
    }
  }
  if (!fits(job, need_sketch(rmax, lsum, lmax, hmax, nmax, gsum), T))
    return;
  Bump bump{scratch};
  // 1. Right Gram matrices G_k = X_{>=k} X_{>=k}^T (r_k x r_k; X_{>=k} the
  //    r_k x (n_k ... n_{d-1}) unfolding of cores k..d-1), from k = d-1 down
  //    (the contract_inner_step chain of detail/contract.hpp:155-205 run from
  //    the right); G_k for k = 1..d-1 stay in gbuf for step 3, and
  //    ||X||^2 = G_0.  gram_off(k): offset of G_k in gbuf, from the input ranks.
  auto gram_off = [&](int k) {
    int64_t off = 0;
    for (int j = 1; j < k; ++j)
      off += static_cast<int64_t>(job.pristine_slots[T.first + j].r) *
             job.pristine_slots[T.first + j].r;
    return off;
  };
  double* gbuf = bump.take(gsum);
  double* tmp = bump.take(rmax * nmax * rmax);
  double* g0 = bump.take(1);
  for (int k = d - 1; k >= 0; --k)
  {
    const int ra = S[k].r, n = S[k].n, rap = S[k].rp;
    const int64_t w = static_cast<int64_t>(n) * rap;
    const double* ca = ar + S[k].off;
    double* Gk = k >= 1 ? gbuf + gram_off(k) : g0;
    const double* Y = ca;  // cores k..d-1 applied to G_{k+1}: left_unfold(C_k) G_{k+1}
    if (k < d - 1)
    {
      gemm_sel(mixed, ra * n, rap, rap, View{ca, rap, 1}, View{gbuf + gram_off(k + 1), rap, 1},
               tmp, rap, 1, sh);
      Y = tmp;
    }
    // G_k (ra x ra) = right_unfold(C_k) right_unfold(Y)^T.
    gemm_sel(mixed, ra, ra, w, View{ca, w, 1}, View{Y, 1, w}, Gk, ra, 1, sh);
  }
  const double nx2 = g0[0];
  __syncthreads();
  // 2. Right environments, stored for bonds 1..d-1 (wbuf + woff, woff per core).
  double* wbuf = bump.take(lsum);
  double* Rk = bump.take(lmax * nmax * lmax);
  double* T1 = bump.take(hmax * lmax);
  double* Wnext = nullptr;  // environment of bond k+1 (1x1 identity for bond d)
  int64_t woff_next = lsum;
  for (int k = d - 1; k >= 1; --k)
  {
    const int r = S[k].r, n = S[k].n, rp = S[k].rp;
    const int lk = sketch_rank_of(job, S, T.first, k - 1, d);
    const int lk1 = sketch_rank_of(job, S, T.first, k, d);
    const int64_t woff = woff_next - static_cast<int64_t>(r) * lk;
    double* Wk = wbuf + woff;
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(lk) * n * lk1; t += blockDim.x)
      Rk[t] = sketch_gauss(job.sketch_seed, static_cast<uint64_t>(tti), static_cast<uint64_t>(k),
                           static_cast<uint64_t>(t));
    __syncthreads();
    const double* xk = ar + S[k].off;
    if (k == d - 1)
    {
      // W_d = 1: T1 = left_unfold(X_{d-1}) (r*n x 1).
      for (int64_t t = threadIdx.x; t < static_cast<int64_t>(r) * n; t += blockDim.x)
        T1[t] = xk[t];
      __syncthreads();
    }
    else
    {
      gemm_sel(mixed, r * n, lk1, rp, View{xk, rp, 1}, View{Wnext, lk1, 1}, T1, lk1, 1, sh);
    }
    // W_k (r x lk) = T1_as (r x n*lk1) * right_unfold(R_k)^T (n*lk1 x lk).
    gemm_sel(mixed, r, lk, n * lk1, View{T1, static_cast<int64_t>(n) * lk1, 1},
             View{Rk, 1, static_cast<int64_t>(n) * lk1}, Wk, lk, 1, sh);
    Wnext = Wk;
    woff_next = woff;
  }
  // 3. Left-to-right sketch-and-orthogonalise; err2 accumulates ||X - Y||^2.
  Bump step = bump;
  double err2 = 0.0;
  for (int k = 0; k < d - 1; ++k)
  {
    Bump b2 = step;
    CoreSlot& cur = S[k];
    CoreSlot& next = S[k + 1];
    const int r = cur.r, n = cur.n, rp = cur.rp;
    const int h = r * n;
    const int l = sketch_rank_of(job, S, T.first, k, d);
    // W_{k+1}: bond k+1 environment (rp x l), at its stored offset.
    int64_t off = 0;
    for (int j = 1; j < k + 1; ++j)
      off += static_cast<int64_t>(job.pristine_slots[T.first + j].r) *
             sketch_rank_of(job, job.pristine_slots + T.first, T.first, j - 1, d);
    const double* Wk1 = wbuf + off;
    double* Z = b2.take(static_cast<int64_t>(h) * l);
    gemm_sel(mixed, h, l, rp, View{ar + cur.off, rp, 1}, View{Wk1, l, 1}, Z, 1, h, sh);
    double* Wq = b2.take(static_cast<int64_t>(h) * l);
    double* tau = b2.take(l);
    double* Rq = b2.take(static_cast<int64_t>(l) * l);
    double* Q;
    // The CTA's shared region is free here: the sketched QR stages in it
    // (in place when h*l fits, else blocked with its panels staged there).
    const int lq = qr_factor(View{Z, 1, h}, h, l, Wq, tau, Rq, sm, &Q, mixed, sh);
    // M (lq x rp) = Q^T left_unfold(cur).
    double* M = b2.take(static_cast<int64_t>(lq) * rp);
    gemm_sel(mixed, lq, rp, h, View{Q, h, 1}, View{ar + cur.off, rp, 1}, M, rp, 1, sh);
    // What this projection discards: D = left_unfold(cur) - Q M (h x rp), a
    // difference of matrices, so it is accurate to the arithmetic's unit
    // roundoff times ||cur||.  With the cores left of k orthonormal and
    // cores k+1.. still those of X, ||X - Y||^2 is the sum over the steps of
    // ||D X_{>=k+1}||^2 = <D, D G_{k+1}> (the discarded parts of successive
    // steps are mutually orthogonal).
    double* D = b2.take(static_cast<int64_t>(h) * rp);
    double* DG = b2.take(static_cast<int64_t>(h) * rp);
    gemm_sel(mixed, h, rp, lq, View{Q, 1, h}, View{M, rp, 1}, D, rp, 1, sh);
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * rp; t += blockDim.x)
      D[t] = ar[cur.off + t] - D[t];
    __syncthreads();
    gemm_sel(mixed, h, rp, rp, View{D, rp, 1}, View{gbuf + gram_off(k + 1), rp, 1}, DG, rp, 1, sh);
    double part = 0.0;
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(h) * rp; t += blockDim.x)
      part = fma(D[t], DG[t], part);
    err2 += cta_sum(part, sh);
    const int wn = next.n * next.rp;
    double* P = b2.take(static_cast<int64_t>(lq) * wn);
    gemm_sel(mixed, lq, wn, rp, View{M, rp, 1}, View{ar + next.off, wn, 1}, P, wn, 1, sh);
    cta_copy(ar + next.off, P, static_cast<int64_t>(lq) * wn);
    cta_copy_to_rowmajor(ar + cur.off, lq, View{Q, 1, h}, h, lq);
    set_ranks(cur, r, lq);
    set_ranks(next, lq, next.rp);
    __syncthreads();
  }
  const double ny = core_norm(ar + S[d - 1].off, core_size(S[d - 1]), sh);
  const double rel = nx2 > 0.0 ? sqrt(fmax(err2, 0.0) / nx2) : 0.0;
  const bool accept = isfinite(rel) && rel <= 0.25 * job.eps;
  if (threadIdx.x == 0)
  {
    T.sketch_err = rel;
    T.sketch_state = accept ? 1 : 2;
  }
  __syncthreads();
  if (accept)
  {
    const double eps_r =
      ny > 0.0 ? sqrt(fmax(job.eps * job.eps - rel * rel, 0.0)) * sqrt(nx2) / ny : job.eps;
    round_tt(job, tti, scratch, sm, sh, eps_r);
    return;
  }
  // Fallback: restore the inputs and round exactly.
  for (int k = 0; k < d; ++k)
  {
    const CoreSlot& p = job.pristine_slots[T.first + k];
    const double* src = job.pristine_arena + p.off;
    cta_copy(ar + p.off, src, static_cast<int64_t>(p.r) * p.n * p.rp);
    set_ranks(S[k], p.r, p.rp);
  }
  __syncthreads();
  round_tt(job, tti, scratch, sm, sh, job.eps);
}

// build_streaming_matvec / build_streaming_matmat
// (detail/streaming_apply.hpp:39-202) for one (operator, operand) pair.
__device__ __noinline__ void stream_tt(const RoundJob& job, int item, double* scratch, Smem sm, CtaShared& sh)
{
  double* ar = job.arena;
  TTInfo& TA = job.tts[job.a_idx[item]];
  TTInfo& TX = job.tts[job.b_idx[item]];
  TTInfo& TO = job.tts[job.out_idx[item]];
  CoreSlot* SA = job.slots + TA.first;
  CoreSlot* SX = job.slots + TX.first;
  CoreSlot* SO = job.slots + TO.first;
  const int d = TA.d;
  for (int k = d - 1; k >= 1; --k)
  {
    if (!fits(job, need_right_qr(SA[k].r, static_cast<int64_t>(SA[k].n) * SA[k].rp,
                                 static_cast<int64_t>(SA[k - 1].r) * SA[k - 1].n), TO))
      return;
    right_qr_step(ar, SA[k], SA[k - 1], Bump{scratch}, sm, job.mixed != 0, sh);
  }
  for (int k = d - 1; k >= 1; --k)
  {
    if (!fits(job, need_right_qr(SX[k].r, static_cast<int64_t>(SX[k].n) * SX[k].rp,
                                 static_cast<int64_t>(SX[k - 1].r) * SX[k - 1].n), TO))
      return;
    right_qr_step(ar, SX[k], SX[k - 1], Bump{scratch}, sm, job.mixed != 0, sh);
  }
  const double nA = core_norm(ar + SA[0].off, core_size(SA[0]), sh);
  const double nX = core_norm(ar + SX[0].off, core_size(SX[0]), sh);
  const double nrm = nA * nX;
  if (threadIdx.x == 0)
    TO.norm = nrm;
  if (!isfinite(nrm))
  {
    set_status(TO, kStatusNan);
    return;
  }
  if (nrm == 0.0)
  {
    zero_tt(ar, SO, d);
    return;
  }
  const double delta = job.eps * nrm / sqrt(static_cast<double>(d - 1 > 1 ? d - 1 : 1));
  if (threadIdx.x == 0)
    TO.delta = delta;
  // Persistent F buffer at the front of the slab; per-step scratch after it.
  // F holds r_new x (b*bx) with r_new <= b*bx.
  int64_t fcap = 1;
  for (int k = 0; k < d; ++k)
  {
    const int64_t cap = static_cast<int64_t>(SA[k].rp) * SX[k].rp;
    fcap = fcap > cap * cap ? fcap : cap * cap;
  }
  double* Fbuf = scratch;
  Bump base{scratch + ((fcap + 31) & ~static_cast<int64_t>(31))};
  if (threadIdx.x == 0)
    Fbuf[0] = 1.0;
  int alpha = 1;
  __syncthreads();
  for (int k = 0; k < d; ++k)
  {
    Bump bump = base;
    const int a = SA[k].r, b = SA[k].rp;
    const int m = SA[k].m;
    const int p = SA[k].n / m;
    const int sx = SX[k].r, bx = SX[k].rp;
    const int nout = SX[k].n / p;
    if (!fits(job, need_stream_step(fcap, alpha, a, m, p, b, sx, nout, bx), TO))
      return;
    const int64_t mpb = static_cast<int64_t>(m) * p * b;
    // Fp (alpha*sx x a): Fp[(al*sx + ax), aa] = F[al, aa*sx + ax].
    double* Fp = bump.take(static_cast<int64_t>(alpha) * sx * a);
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(alpha) * sx * a; t += blockDim.x)
    {
      const int aa = static_cast<int>(t % a);
      const int64_t row = t / a;
      const int al = static_cast<int>(row / sx), ax = static_cast<int>(row % sx);
      Fp[t] = Fbuf[static_cast<int64_t>(al) * a * sx + static_cast<int64_t>(aa) * sx + ax];
    }
    __syncthreads();
    // G1 (alpha*sx x m*p*b) = Fp * A_k.
    double* G1 = bump.take(static_cast<int64_t>(alpha) * sx * mpb);
    gemm_sel(job.mixed != 0, alpha * sx, static_cast<int>(mpb), a, View{Fp, a, 1},
             View{ar + SA[k].off, mpb, 1}, G1, mpb, 1, sh);
    // G1p ((al, i, bb) x (ax, q)).
    const int64_t g1p_rows = static_cast<int64_t>(alpha) * m * b;
    const int64_t g1p_cols = static_cast<int64_t>(sx) * p;
    double* G1p = bump.take(g1p_rows * g1p_cols);
    for (int64_t t = threadIdx.x; t < g1p_rows * g1p_cols; t += blockDim.x)
    {
      const int64_t row = t / g1p_cols, col = t % g1p_cols;
      const int bb = static_cast<int>(row % b);
      const int i = static_cast<int>((row / b) % m);
      const int al = static_cast<int>(row / (static_cast<int64_t>(b) * m));
      const int ax = static_cast<int>(col / p), q = static_cast<int>(col % p);
      G1p[t] = G1[(static_cast<int64_t>(al) * sx + ax) * mpb + (static_cast<int64_t>(i) * p + q) * b + bb];
    }
    __syncthreads();
    // C2 ((al,i,bb) x (j,bx')) = G1p * X_k.
    const int64_t c2_cols = static_cast<int64_t>(nout) * bx;
    double* C2 = bump.take(g1p_rows * c2_cols);
    gemm_sel(job.mixed != 0, static_cast<int>(g1p_rows), static_cast<int>(c2_cols),
             static_cast<int>(g1p_cols), View{G1p, g1p_cols, 1}, View{ar + SX[k].off, c2_cols, 1},
             C2, c2_cols, 1, sh);
    // Cj (al, i, j, bb, bx') row-major.
    double* Cj = C2;
    if (nout > 1)
    {
      Cj = bump.take(g1p_rows * c2_cols);
      for (int64_t t = threadIdx.x; t < g1p_rows * c2_cols; t += blockDim.x)
      {
        const int bxx = static_cast<int>(t % bx);
        const int bb = static_cast<int>((t / bx) % b);
        const int j = static_cast<int>((t / (static_cast<int64_t>(bx) * b)) % nout);
        const int64_t ai = t / (static_cast<int64_t>(bx) * b * nout);  // al*m + i
        Cj[t] = C2[(ai * b + bb) * c2_cols + static_cast<int64_t>(j) * bx + bxx];
      }
      __syncthreads();
    }
    const int hrows = alpha * m * nout;
    const int ccols = b * bx;
    double* os = ar + SO[k].off;
    if (k == d - 1)
    {
      cta_copy(os, Cj, static_cast<int64_t>(hrows) * ccols);
      set_ranks(SO[k], alpha, ccols);
      __syncthreads();
      break;
    }
    double *U, *F;
    const int r_new = left_svd(View{Cj, ccols, 1}, hrows, ccols, delta, job.max_rank,
                               job.max_sweeps, job.mixed != 0, bump, sm, &U, &F, TO, sh);
    cta_copy_to_rowmajor(os, r_new, View{U, 1, hrows}, hrows, r_new);
    cta_copy(Fbuf, F, static_cast<int64_t>(r_new) * ccols);
    set_ranks(SO[k], alpha, r_new);
    alpha = r_new;
    __syncthreads();
  }
}

}  // namespace

// MinBlocks CTAs of 256 threads resident per SM (the register cap follows:
// 128, 85 or 64 per thread); the autotuner picks the instantiation.
// ---------------------------------------------------------------------------
// ALS and two-site DMRG rounding (round/tt_als.hpp:52-206,
// round/tt_dmrg.hpp:45-212), one CTA per (Y, X) pair: Y = TT a_idx[i] is the
// tensor to compress, X = TT b_idx[i] the start TT, overwritten in its slots
// (bond capacities fixed by the host).  The left and right environments,
// the bond spectra of two consecutive sweep pairs and the bond capacities
// live in the pair's region of the arena (TTInfo::env_off of X):
//   L[k] at env + k*es, R[k] at env + (d+1+k)*es (k = 0..d), then cmax,
//   s_prev / s_now ((d-1) bonds x cmax each), their counts and the bond
//   capacities cap[0..d], as doubles (written by the host).
// All arithmetic is FP64.
// ---------------------------------------------------------------------------

// contract_inner_step (detail/contract.hpp:155-205):
// out (rap x rbp) = sum_{a,b,i} E(a, b) ca(a, i, a') cb(b, i, b').
__device__ void env_left(const double* E, const double* ca, int ra, int n, int rap,
                         const double* cb, int rb, int rbp, double* out, Bump bump, CtaShared& sh)
{
  const int64_t w = static_cast<int64_t>(n) * rap;
  double* tmp = bump.take(static_cast<int64_t>(rb) * w);
  cta_gemm(rb, static_cast<int>(w), ra, View{E, 1, rb}, View{ca, w, 1}, tmp, w, 1, sh);
  cta_gemm(rap, rbp, rb * n, View{tmp, 1, rap}, View{cb, rbp, 1}, out, rbp, 1, sh);
}

// contract_inner_step_right (detail/contract.hpp:90-139):
// out (ra x rb) = sum_{i,a',b'} ca(a, i, a') F(a', b') cb(b, i, b').
__device__ void env_right(const double* ca, int ra, int n, int rap, const double* cb, int rb,
                          int rbp, const double* F, double* out, Bump bump, CtaShared& sh)
{
  const int64_t w = static_cast<int64_t>(n) * rbp;
  double* T1 = bump.take(static_cast<int64_t>(ra) * w);
  cta_gemm(ra * n, rbp, rap, View{ca, rap, 1}, View{F, rbp, 1}, T1, rbp, 1, sh);
  cta_gemm(ra, rb, static_cast<int>(w), View{T1, w, 1}, View{cb, 1, w}, out, rb, 1, sh);
}

// als_local_update (detail/als_local_solve.hpp): X (lr, n, rc) = L Y_k R.
__device__ void local_update(const double* L, int lr, const double* Y, int yr, int n, int yrp,
                             const double* R, int rc, double* X, Bump bump, CtaShared& sh)
{
  const int64_t w = static_cast<int64_t>(n) * yrp;
  double* T1 = bump.take(static_cast<int64_t>(lr) * w);
  cta_gemm(lr, static_cast<int>(w), yr, View{L, yr, 1}, View{Y, w, 1}, T1, w, 1, sh);
  cta_gemm(lr * n, rc, yrp, View{T1, yrp, 1}, View{R, rc, 1}, X, rc, 1, sh);
}

// merge_y_block (detail/dmrg_local_solve.hpp): Theta (rxl*n0, n1*rxr) =
// (L Y_k) (Y_k1 R).
__device__ double* merge_pair(const double* L, int rxl, const double* Y0, int yr0, int n0,
                              int yr1, const double* Y1, int n1, int yr2, const double* R,
                              int rxr, Bump& bump, CtaShared& sh)
{
  const int64_t w0 = static_cast<int64_t>(n0) * yr1;
  const int64_t cols = static_cast<int64_t>(n1) * rxr;
  double* T1 = bump.take(static_cast<int64_t>(rxl) * w0);
  double* T2 = bump.take(static_cast<int64_t>(yr1) * cols);
  double* Th = bump.take(static_cast<int64_t>(rxl) * n0 * cols);
  cta_gemm(rxl, static_cast<int>(w0), yr0, View{L, yr0, 1}, View{Y0, w0, 1}, T1, w0, 1, sh);
  cta_gemm(yr1 * n1, rxr, yr2, View{Y1, yr2, 1}, View{R, rxr, 1}, T2, rxr, 1, sh);
  cta_gemm(rxl * n0, static_cast<int>(cols), yr1, View{T1, yr1, 1}, View{T2, cols, 1}, Th, cols,
           1, sh);
  return Th;
}

__device__ __noinline__ void iter_round_tt(const RoundJob& job, int item, double* scratch, Smem sm,
                                           CtaShared& sh)
{
  const bool dmrg = job.kind == kJobDmrg;
  TTInfo& TY = job.tts[job.a_idx[item]];
  TTInfo& TX = job.tts[job.b_idx[item]];
  const int d = TY.d;
  CoreSlot* SY = job.slots + TY.first;
  CoreSlot* SX = job.slots + TX.first;
  double* ar = job.arena;
  const int64_t es = TX.env_stride;
  double* env = ar + TX.env_off;
  // After the environments: cmax, s_prev, s_now ((d-1) x cmax each),
  // cnt_prev, cnt_now (d-1 each), caps (d+1).
  double* base2 = env + 2 * static_cast<int64_t>(d + 1) * es;
  const int cmax = static_cast<int>(base2[0]);
  double* sp = base2 + 1;
  double* sn = sp + static_cast<int64_t>(d - 1) * cmax;
  double* cp = sn + static_cast<int64_t>(d - 1) * cmax;
  double* cn = cp + (d - 1);
  const double* caps = cn + (d - 1);
  auto Lk = [&](int k) { return env + static_cast<int64_t>(k) * es; };
  auto Rk = [&](int k) { return env + static_cast<int64_t>(d + 1 + k) * es; };
  auto core = [&](CoreSlot* S, int k) { return ar + S[k].off; };
  double* sdummy = nullptr;

  double delta = 0.0;
  if (dmrg)
  {
    // ||Y|| by the inner chain of Y with itself (algebra/tt_inner.hpp:33-47).
    if (threadIdx.x == 0)
      Lk(0)[0] = 1.0;
    __syncthreads();
    for (int k = 0; k < d; ++k)
      env_left(Lk(k), core(SY, k), SY[k].r, SY[k].n, SY[k].rp, core(SY, k), SY[k].r, SY[k].rp,
               Lk(k + 1), Bump{scratch}, sh);
    const double yy = Lk(d)[0];
    const double ynorm = sqrt(yy > 0.0 ? yy : 0.0);
    delta = job.eps * ynorm / sqrt(static_cast<double>(d - 1 > 1 ? d - 1 : 1));
    if (threadIdx.x == 0)
    {
      TX.norm = ynorm;
      TX.delta = delta;
    }
  }
  if (!job.x_right_canonical)
    for (int k = d - 1; k >= 1; --k)
    {
      if (!fits(job, need_right_qr(SX[k].r, static_cast<int64_t>(SX[k].n) * SX[k].rp,
                                   static_cast<int64_t>(SX[k - 1].r) * SX[k - 1].n), TX))
        return;
      right_qr_step(ar, SX[k], SX[k - 1], Bump{scratch}, sm, false, sh);
    }
  if (threadIdx.x == 0)
  {
    Rk(d)[0] = 1.0;
    Lk(0)[0] = 1.0;
  }
  __syncthreads();
  for (int k = d - 1; k >= 1; --k)
    env_right(core(SY, k), SY[k].r, SY[k].n, SY[k].rp, core(SX, k), SX[k].r, SX[k].rp, Rk(k + 1),
              Rk(k), Bump{scratch}, sh);

  int iters = 0, converged = 0;
  double change = 0.0;
  for (int it = 0; it < job.max_iters; ++it)
  {
    if (!dmrg)
    {
      for (int k = 0; k < d; ++k)
      {
        local_update(Lk(k), SX[k].r, core(SY, k), SY[k].r, SY[k].n, SY[k].rp, Rk(k + 1),
                     SX[k].rp, core(SX, k), Bump{scratch}, sh);
        if (k < d - 1)
        {
          if (!fits(job, need_left_qr(static_cast<int64_t>(SX[k].r) * SX[k].n, SX[k].rp,
                                      static_cast<int64_t>(SX[k + 1].n) * SX[k + 1].rp), TX))
            return;
          left_qr_step(ar, SX[k], SX[k + 1], Bump{scratch}, sm, false, sh);
          env_left(Lk(k), core(SX, k), SX[k].r, SX[k].n, SX[k].rp, core(SY, k), SY[k].r,
                   SY[k].rp, Lk(k + 1), Bump{scratch}, sh);
        }
      }
      for (int k = d - 1; k >= 0; --k)
      {
        if (k < d - 1)
          local_update(Lk(k), SX[k].r, core(SY, k), SY[k].r, SY[k].n, SY[k].rp, Rk(k + 1),
                       SX[k].rp, core(SX, k), Bump{scratch}, sh);
        if (k > 0)
        {
          if (!fits(job, need_right_qr(SX[k].r, static_cast<int64_t>(SX[k].n) * SX[k].rp,
                                       static_cast<int64_t>(SX[k - 1].r) * SX[k - 1].n), TX))
            return;
          right_qr_step(ar, SX[k], SX[k - 1], Bump{scratch}, sm, false, sh);
          env_right(core(SY, k), SY[k].r, SY[k].n, SY[k].rp, core(SX, k), SX[k].r, SX[k].rp,
                    Rk(k + 1), Rk(k), Bump{scratch}, sh);
        }
      }
      // Bond spectra of the cores (core_singular_values, tt_als.hpp:170-190).
      for (int k = 0; k < d - 1; ++k)
      {
        const int h = SX[k].r * SX[k].n, c = SX[k].rp;
        if (!fits(job, need_left_svd(h, c) + a32(static_cast<int64_t>(h) * c), TX))
          return;
        double *U, *F, *sv;
        left_svd(View{core(SX, k), c, 1}, h, c, 0.0, 0, job.max_sweeps, false, Bump{scratch}, sm,
                 &U, &F, TX, sh, nullptr, &sv);
        const int cnt = h < c ? h : c;
        for (int i = threadIdx.x; i < cnt; i += blockDim.x)
          sn[static_cast<int64_t>(k) * cmax + i] = sv[i];
        if (threadIdx.x == 0)
          cn[k] = cnt;
        __syncthreads();
      }
    }
    else
    {
      for (int k = 0; k < d - 1; ++k)
      {
        const int rxl = SX[k].r, rxr = SX[k + 1].rp, n0 = SY[k].n, n1 = SY[k + 1].n;
        const int rows = rxl * n0, cols = n1 * rxr;
        const int cap = static_cast<int>(caps[k + 1]);
        const int mr = job.max_rank > 0 && job.max_rank < cap ? job.max_rank : cap;
        if (!fits(job, a32(static_cast<int64_t>(rxl) * n0 * SY[k].rp) +
                         a32(static_cast<int64_t>(SY[k].rp) * cols) +
                         a32(static_cast<int64_t>(rows) * cols) + need_left_svd(rows, cols),
                  TX))
          return;
        Bump bump{scratch};
        double* Th = merge_pair(Lk(k), rxl, core(SY, k), SY[k].r, n0, SY[k].rp, core(SY, k + 1),
                                n1, SY[k + 1].rp, Rk(k + 2), rxr, bump, sh);
        double *U, *F, *sv;
        const int r = left_svd(View{Th, cols, 1}, rows, cols, delta, mr, job.max_sweeps, false,
                               bump, sm, &U, &F, TX, sh, nullptr, &sv);
        // X_k <- U, X_k1 <- diag(s) V^T (split_two_site_lr).
        cta_copy_to_rowmajor(core(SX, k), r, View{U, 1, rows}, rows, r);
        cta_copy(core(SX, k + 1), F, static_cast<int64_t>(r) * cols);
        set_ranks(SX[k], rxl, r);
        set_ranks(SX[k + 1], r, rxr);
        for (int i = threadIdx.x; i < r; i += blockDim.x)
          sn[static_cast<int64_t>(k) * cmax + i] = sv[i];
        if (threadIdx.x == 0)
          cn[k] = r;
        __syncthreads();
        env_left(Lk(k), core(SX, k), SX[k].r, SX[k].n, SX[k].rp, core(SY, k), SY[k].r, SY[k].rp,
                 Lk(k + 1), Bump{scratch}, sh);
      }
      for (int k = d - 2; k >= 0; --k)
      {
        const int rxl = SX[k].r, rxr = SX[k + 1].rp, n0 = SY[k].n, n1 = SY[k + 1].n;
        const int rows = rxl * n0, cols = n1 * rxr;
        const int cap = static_cast<int>(caps[k + 1]);
        const int mr = job.max_rank > 0 && job.max_rank < cap ? job.max_rank : cap;
        if (!fits(job, a32(static_cast<int64_t>(rxl) * n0 * SY[k].rp) +
                         a32(static_cast<int64_t>(SY[k].rp) * cols) +
                         a32(static_cast<int64_t>(rows) * cols) + need_left_svd(cols, rows),
                  TX))
          return;
        Bump bump{scratch};
        double* Th = merge_pair(Lk(k), rxl, core(SY, k), SY[k].r, n0, SY[k].rp, core(SY, k + 1),
                                n1, SY[k + 1].rp, Rk(k + 2), rxr, bump, sh);
        // split_two_site_rl through Theta^T = V S U^T: U' = V, F' = S U^T.
        double *U, *F;
        const int r = left_svd(View{Th, 1, cols}, cols, rows, delta, mr, job.max_sweeps, false,
                               bump, sm, &U, &F, TX, sh, nullptr, &sdummy);
        cta_copy(core(SX, k + 1), U, static_cast<int64_t>(r) * cols);         // V^T
        cta_copy_to_rowmajor(core(SX, k), r, View{F, 1, rows}, rows, r);    // U diag(s)
        set_ranks(SX[k], rxl, r);
        set_ranks(SX[k + 1], r, rxr);
        __syncthreads();
        env_right(core(SY, k + 1), SY[k + 1].r, SY[k + 1].n, SY[k + 1].rp, core(SX, k + 1),
                  SX[k + 1].r, SX[k + 1].rp, Rk(k + 2), Rk(k + 1), Bump{scratch}, sh);
      }
    }
    ++iters;
    // Largest relative change of the bond spectra (sv_change; a bond whose
    // count changed counts as 1, as tt_als.hpp:182-186 / tt_dmrg.hpp do).
    if (threadIdx.x == 0)
    {
      double worst = 0.0;
      for (int k = 0; k < d - 1; ++k)
      {
        const int a = static_cast<int>(cn[k]), b = static_cast<int>(cp[k]);
        if (it == 0)
          continue;
        if (a != b)
        {
          worst = 1.0;
          continue;
        }
        double dn = 0.0, nn = 0.0;
        for (int i = 0; i < a; ++i)
        {
          const double x = sn[static_cast<int64_t>(k) * cmax + i];
          const double y = sp[static_cast<int64_t>(k) * cmax + i];
          dn += (x - y) * (x - y);
          nn += x * x;
        }
        const double rel = sqrt(dn) / (sqrt(nn) + 1.0e-300);
        worst = rel > worst ? rel : worst;
      }
      sh.dval[0] = it == 0 ? 1.0 : worst;
    }
    __syncthreads();
    change = sh.dval[0];
    for (int64_t t = threadIdx.x; t < static_cast<int64_t>(d - 1) * (cmax + 1); t += blockDim.x)
    {
      if (t < static_cast<int64_t>(d - 1) * cmax)
        sp[t] = sn[t];
      else
        cp[t - static_cast<int64_t>(d - 1) * cmax] = cn[t - static_cast<int64_t>(d - 1) * cmax];
    }
    __syncthreads();
    if (change <= job.tol)
    {
      converged = 1;
      break;
    }
  }
  if (threadIdx.x == 0)
  {
    TX.iters_run = iters;
    TX.iter_conv = converged;
    TX.final_change = change;
  }
  __syncthreads();
}

template <int MinBlocks>
__global__ void __launch_bounds__(kThreads, MinBlocks) round_kernel(RoundJob job)
{
  __shared__ CtaShared sh;
  extern __shared__ double dyn_smem[];
  const Smem sm{dyn_smem, job.smem_doubles};
  double* scratch = job.scratch + static_cast<int64_t>(blockIdx.x) * job.scratch_stride;
  for (;;)
  {
    if (threadIdx.x == 0)
      sh.item = atomicAdd(job.queue, 1);
    __syncthreads();
    const int item = sh.item;
    __syncthreads();
    if (item >= job.ntt)
      break;
    if (job.kind == kJobStreamMatvec || job.kind == kJobStreamMatmat)
      stream_tt(job, job.order[item], scratch, sm, sh);
    else if (job.kind == kJobRoundSketch)
      round_sketch_tt(job, job.order[item], scratch, sm, sh);
    else if (job.kind == kJobAls || job.kind == kJobDmrg)
      iter_round_tt(job, job.order[item], scratch, sm, sh);
    else
      round_tt(job, job.order[item], scratch, sm, sh, job.eps);
  }
}

// matvec_core / matmat_core (apply/tt_matrix_apply.hpp:40-224):
// y(a*s+ax, i, j, b*sp+bx) = sum_q A(a, i, q, b) X(ax, q, j, bx), with j of
// size nout (1 for matvec).  One thread per output element.
__global__ void apply_core_kernel(const double* __restrict__ Ac, const double* __restrict__ Xc,
                                  double* __restrict__ Y, int r, int m, int p, int rp, int s,
                                  int nout, int sp)
{
  const int64_t total = static_cast<int64_t>(r) * s * m * nout * rp * sp;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
  {
    int64_t u = t;
    const int bx = static_cast<int>(u % sp);
    u /= sp;
    const int b = static_cast<int>(u % rp);
    u /= rp;
    const int j = static_cast<int>(u % nout);
    u /= nout;
    const int i = static_cast<int>(u % m);
    u /= m;
    const int ax = static_cast<int>(u % s);
    const int a = static_cast<int>(u / s);
    double acc = 0.0;
    for (int q = 0; q < p; ++q)
      acc = fma(Ac[((static_cast<int64_t>(a) * m + i) * p + q) * rp + b],
                Xc[((static_cast<int64_t>(ax) * p + q) * nout + j) * sp + bx], acc);
    Y[t] = acc;
  }
}

// eval_batch: one warp per multi-index; the running row vector lives in
// shared memory (two buffers per warp of `rcap` doubles).
__global__ void __launch_bounds__(kThreads) eval_kernel(const double* __restrict__ ar,
                                                        const CoreSlot* __restrict__ S, int d,
                                                        const int* __restrict__ idx, int64_t M,
                                                        double* __restrict__ out, int rcap,
                                                        int* __restrict__ bad)
{
  extern __shared__ double evbuf[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double* v = evbuf + static_cast<int64_t>(w) * 2 * rcap;
  double* vn = v + rcap;
  const int64_t warps_total = static_cast<int64_t>(gridDim.x) * kWarps;
  for (int64_t smp = blockIdx.x * static_cast<int64_t>(kWarps) + w; smp < M; smp += warps_total)
  {
    const int* ix = idx + smp * d;
    int i0 = ix[0];
    bool ok = (i0 >= 0 && i0 < S[0].n);
    for (int k = 1; k < d; ++k)
    {
      const int ik = ix[k];
      ok = ok && (ik >= 0 && ik < S[k].n);
    }
    if (!ok)
    {
      if (lane == 0)
      {
        out[smp] = __longlong_as_double(0x7ff8000000000000ll);
        atomicExch(bad, 1);
      }
      continue;
    }
    {
      const int r1 = S[0].rp;
      const double* c0 = ar + S[0].off + static_cast<int64_t>(i0) * r1;
      for (int b = lane; b < r1; b += 32)
        v[b] = c0[b];
    }
    __syncwarp();
    for (int k = 1; k < d; ++k)
    {
      const int r = S[k].r, n = S[k].n, rp = S[k].rp;
      const int ik = ix[k];
      const double* ck = ar + S[k].off + static_cast<int64_t>(ik) * rp;
      const int64_t stride = static_cast<int64_t>(n) * rp;
      for (int b0 = 0; b0 < rp; b0 += 32)
      {
        const int b = b0 + lane;
        double acc = 0.0;
        if (b < rp)
          for (int a = 0; a < r; ++a)
            acc = fma(v[a], ck[a * stride + b], acc);
        if (b < rp)
          vn[b] = acc;
      }
      __syncwarp();
      double* t = v;
      v = vn;
      vn = t;
    }
    if (lane == 0)
      out[smp] = v[0];
    __syncwarp();
  }
}

// inner (algebra/tt_inner.hpp:33-47): one CTA runs the left-to-right
// environment chain of contract_inner_step (detail/contract.hpp:155-205).
__global__ void __launch_bounds__(kThreads) inner_kernel(const double* __restrict__ ar,
                                                         const CoreSlot* __restrict__ SA,
                                                         const CoreSlot* __restrict__ SB, int d,
                                                         double* scratch, int64_t env_cap,
                                                         double* out)
{
  __shared__ CtaShared sh;
  double* E = scratch;
  double* En = scratch + env_cap;
  double* tmp = scratch + 2 * env_cap;
  if (threadIdx.x == 0)
    E[0] = 1.0;
  __syncthreads();
  for (int k = 0; k < d; ++k)
  {
    const int ra = SA[k].r, n = SA[k].n, rap = SA[k].rp;
    const int rb = SB[k].r, rbp = SB[k].rp;
    const double* ca = ar + SA[k].off;
    const double* cb = ar + SB[k].off;
    // tmp (rb x n*rap) = E^T * right_unfold(ca).
    cta_gemm(rb, n * rap, ra, View{E, 1, rb}, View{ca, static_cast<int64_t>(n) * rap, 1}, tmp,
             static_cast<int64_t>(n) * rap, 1, sh);
    // En (rap x rbp) = tmp_as^T (rap x rb*n) * left_unfold(cb) (rb*n x rbp).
    cta_gemm(rap, rbp, rb * n, View{tmp, 1, rap}, View{cb, rbp, 1}, En, rbp, 1, sh);
    double* t = E;
    E = En;
    En = t;
  }
  if (threadIdx.x == 0)
    *out = E[0];
}

void launch_round(const RoundJob& job, int grid, int ctas_per_sm, cudaStream_t stream)
{
  const size_t smem = sizeof(double) * static_cast<size_t>(job.smem_doubles);
  if (ctas_per_sm >= 4)
    round_kernel<4><<<grid, kThreads, smem, stream>>>(job);
  else if (ctas_per_sm == 3)
    round_kernel<3><<<grid, kThreads, smem, stream>>>(job);
  else
    round_kernel<2><<<grid, kThreads, smem, stream>>>(job);
}

cudaError_t round_smem_optin(int smem_doubles)
{
  const int bytes = static_cast<int>(sizeof(double) * smem_doubles);
  cudaError_t e = cudaFuncSetAttribute(round_kernel<2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(round_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(round_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

void launch_apply_core(const double* A, const double* X, double* Y, int r, int m, int p, int rp,
                       int s, int nout, int sp, cudaStream_t stream)
{
  const int64_t total = static_cast<int64_t>(r) * s * m * nout * rp * sp;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 65535)
    blocks = 65535;
  if (blocks < 1)
    blocks = 1;
  apply_core_kernel<<<static_cast<int>(blocks), 256, 0, stream>>>(A, X, Y, r, m, p, rp, s, nout,
                                                                  sp);
}

void launch_eval(const double* ar, const CoreSlot* S, int d, const int* idx, int64_t M,
                 double* out, int rcap, int* bad, int grid, cudaStream_t stream)
{
  const size_t smem = static_cast<size_t>(kWarps) * 2 * rcap * sizeof(double);
  eval_kernel<<<grid, kThreads, smem, stream>>>(ar, S, d, idx, M, out, rcap, bad);
}

void launch_inner(const double* ar, const CoreSlot* SA, const CoreSlot* SB, int d,
                  double* scratch, int64_t env_cap, double* out, cudaStream_t stream)
{
  inner_kernel<<<1, kThreads, 0, stream>>>(ar, SA, SB, d, scratch, env_cap, out);
}

// Eight independent DFMA chains per thread (operands from kernel
// parameters); one store per thread into out[grid*block].
__global__ void fp64_peak_kernel(double* out, int iters, double a, double b)
{
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k)
      x[k] = fma(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    s += x[k];
  out[static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

void launch_fp64_peak(double* out, int iters, int grid, int block, cudaStream_t stream)
{
  fp64_peak_kernel<<<grid, block, 0, stream>>>(out, iters, 0.999, 0.001);
}

cudaError_t eval_smem_optin(int rcap)
{
  const size_t smem = static_cast<size_t>(kWarps) * 2 * rcap * sizeof(double);
  return cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(smem));
}

}  // namespace ttg
