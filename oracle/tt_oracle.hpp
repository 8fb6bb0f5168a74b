// CPU oracle for the TT-rounding hot path -- TEST INFRASTRUCTURE ONLY.
//
// A plain-C++20 FP64 restatement of the reference's algorithms, used by the
// tests and by smoke() for the expected results, and by bench.py as the
// timed CPU baseline.  The product (the CUDA library) never links, calls or
// routes through this file.
//
// The reference delegates QR/SVD/GEMM to Eigen (libeigen/eigen; version
// unpinned: the submodule is empty in the reference tree), which is not
// available here.  This file restates the published algorithms Eigen uses:
//   * Householder thin QR (Golub & Van Loan, Alg. 5.2.1; Eigen's
//     makeHouseholder sign convention beta = -sign(x0)*||x||),
//   * one-sided Jacobi SVD (Hestenes 1958; Demmel & Veselic 1992) as the
//     stand-in for BDCSVD/JacobiSVD (same singular values to ~1e-15*s_max),
// and follows the reference's branch structure, delta formula, tail rule,
// early-outs and max_rank handling exactly.  Each function cites the
// reference file:line it follows (paths inside the reference project).
//
// Parity status: the reference ships no golden vectors; its tests are
// known-answer-by-construction (dense equality, invariants).  Every one of
// them on this path is restated against this oracle (tests/test_oracle*.py,
// tests/test_bindings_reference.py), and two independent numpy/LAPACK
// restatements (oracle/numpy_round.py, oracle/numpy_iter.py) agree with it.
// Bitwise agreement with Eigen is not claimed (QR/SVD sign conventions
// differ); results are compared as tensors (relative Frobenius error) and as
// ranks.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace ttor
{

struct oracle_error : std::runtime_error
{
  using std::runtime_error::runtime_error;
};

[[noreturn]] inline void fail(const std::string& msg)
{
  throw oracle_error(msg);
}

// ---------------------------------------------------------------------------
// Storage.  A core is (r, n, rp) row-major: idx = (a*n + i)*rp + b
// (types/tt_core.hpp:25-212).  A TT-matrix core (r, m, n, rp) is stored as a
// 3-axis core with mode m*n (types/tt_matrix.hpp:29-36); the TT keeps m and
// the column mode per site when it is a matrix.
// ---------------------------------------------------------------------------
struct Core
{
  int r = 0, n = 0, rp = 0;
  std::vector<double> v;
  Core() = default;
  Core(int r_, int n_, int rp_) : r(r_), n(n_), rp(rp_)
  {
    if (r <= 0 || n <= 0 || rp <= 0)
      fail("tt_core: dimensions must be positive");
    v.assign(static_cast<size_t>(r) * n * rp, 0.0);
  }
  double& operator()(int a, int i, int b)
  {
    return v[(static_cast<size_t>(a) * n + i) * rp + b];
  }
  double operator()(int a, int i, int b) const
  {
    return v[(static_cast<size_t>(a) * n + i) * rp + b];
  }
  size_t size() const { return v.size(); }
};

struct TT
{
  std::vector<Core> c;
  bool matrix = false;
  std::vector<int> mrow, ncol;  // per-site (m, n) when matrix

  int d() const { return static_cast<int>(c.size()); }
  std::vector<int> ranks() const
  {
    std::vector<int> rs;
    if (c.empty())
    {
      rs.push_back(1);
      return rs;
    }
    rs.push_back(c.front().r);
    for (auto& x : c)
      rs.push_back(x.rp);
    return rs;
  }
  std::vector<int> shape() const
  {
    std::vector<int> s;
    for (auto& x : c)
      s.push_back(x.n);
    return s;
  }
  // Boundary / bond validation (types/tt.hpp:35-70).
  void validate() const
  {
    const int dd = d();
    if (dd == 0)
      return;
    if (c[0].r != 1)
      fail("tt: r_0 must be 1");
    if (c[dd - 1].rp != 1)
      fail("tt: r_d must be 1");
    for (int k = 0; k + 1 < dd; ++k)
      if (c[k].rp != c[k + 1].r)
        fail("tt: rank mismatch at bond " + std::to_string(k + 1));
  }
};

// Optional per-step trace (shapes and chosen ranks) for the FLOP model.
struct Trace
{
  bool on = false;
  std::vector<std::string> lines;
  void add(const std::string& s)
  {
    if (on)
      lines.push_back(s);
  }
};
inline Trace& trace()
{
  static thread_local Trace t;
  return t;
}

// Row-major dense matrix helper.
struct Mat
{
  int64_t rows = 0, cols = 0;
  std::vector<double> v;
  Mat() = default;
  Mat(int64_t r, int64_t c) : rows(r), cols(c), v(static_cast<size_t>(r * c), 0.0) {}
  double& operator()(int64_t i, int64_t j) { return v[static_cast<size_t>(i * cols + j)]; }
  double operator()(int64_t i, int64_t j) const { return v[static_cast<size_t>(i * cols + j)]; }
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
};

// C(m,n) = A(m,k) * B(k,n), all row-major with explicit leading dimensions.
// i-k-j loop order so the inner loop is a contiguous axpy.
inline void gemm_nn(int64_t m, int64_t n, int64_t k,
                    const double* A, int64_t lda,
                    const double* B, int64_t ldb,
                    double* C, int64_t ldc)
{
  for (int64_t i = 0; i < m; ++i)
  {
    double* ci = C + i * ldc;
    for (int64_t j = 0; j < n; ++j)
      ci[j] = 0.0;
    const double* ai = A + i * lda;
    for (int64_t p = 0; p < k; ++p)
    {
      const double a = ai[p];
      const double* bp = B + p * ldb;
      for (int64_t j = 0; j < n; ++j)
        ci[j] += a * bp[j];
    }
  }
}

inline Mat matmul(const Mat& A, const Mat& B)
{
  if (A.cols != B.rows)
    fail("matmul: shape mismatch");
  Mat C(A.rows, B.cols);
  gemm_nn(A.rows, B.cols, A.cols, A.data(), A.cols, B.data(), B.cols, C.data(), C.cols);
  return C;
}

inline Mat transpose(const Mat& A)
{
  Mat T(A.cols, A.rows);
  for (int64_t i = 0; i < A.rows; ++i)
    for (int64_t j = 0; j < A.cols; ++j)
      T(j, i) = A(i, j);
  return T;
}

// ---------------------------------------------------------------------------
// Householder thin QR.  Restates qr_thin (types/tt_eigen_bridge.hpp:42-60):
// Q (rows x k) orthonormal columns, R (k x cols) upper triangular,
// k = min(rows, cols).  Reflector convention of Eigen's makeHouseholder:
// beta = -sign(x0) * ||x||, tau = (beta - x0)/beta, v = [1; x_tail/(x0-beta)];
// a column whose tail is exactly zero gets tau = 0 (identity reflector).
// ---------------------------------------------------------------------------
inline void qr_thin(const double* M, int64_t rows, int64_t cols, Mat& Q, Mat& R)
{
  if (rows <= 0 || cols <= 0)
  {
    Q = Mat();
    R = Mat();
    return;
  }
  const int64_t k = std::min(rows, cols);
  // Column-major working copy: W[j*rows + i] = M(i, j).
  std::vector<double> W(static_cast<size_t>(rows * cols));
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < cols; ++j)
      W[j * rows + i] = M[i * cols + j];
  std::vector<double> tau(static_cast<size_t>(k), 0.0);
  const double tiny = std::numeric_limits<double>::min();
  for (int64_t j = 0; j < k; ++j)
  {
    double* x = &W[j * rows + j];
    const int64_t len = rows - j;
    double tail2 = 0.0;
    for (int64_t i = 1; i < len; ++i)
      tail2 += x[i] * x[i];
    const double x0 = x[0];
    double beta, t;
    if (tail2 <= tiny)
    {
      t = 0.0;
      beta = x0;
      for (int64_t i = 1; i < len; ++i)
        x[i] = 0.0;
    }
    else
    {
      beta = std::sqrt(x0 * x0 + tail2);
      if (x0 >= 0.0)
        beta = -beta;
      const double inv = 1.0 / (x0 - beta);
      for (int64_t i = 1; i < len; ++i)
        x[i] *= inv;
      t = (beta - x0) / beta;
    }
    x[0] = beta;
    tau[j] = t;
    if (t == 0.0)
      continue;
    // Apply H = I - t v v^T to trailing columns.
    for (int64_t c = j + 1; c < cols; ++c)
    {
      double* y = &W[c * rows + j];
      double w = y[0];
      for (int64_t i = 1; i < len; ++i)
        w += x[i] * y[i];
      w *= t;
      y[0] -= w;
      for (int64_t i = 1; i < len; ++i)
        y[i] -= w * x[i];
    }
  }
  R = Mat(k, cols);
  for (int64_t i = 0; i < k; ++i)
    for (int64_t j = i; j < cols; ++j)
      R(i, j) = W[j * rows + i];
  // Q = H_0 ... H_{k-1} [I_k; 0], accumulated backwards (column-major work).
  std::vector<double> Qc(static_cast<size_t>(rows * k), 0.0);
  for (int64_t j = 0; j < k; ++j)
    Qc[j * rows + j] = 1.0;
  for (int64_t j = k - 1; j >= 0; --j)
  {
    const double t = tau[j];
    if (t == 0.0)
      continue;
    const double* x = &W[j * rows + j];
    const int64_t len = rows - j;
    for (int64_t c = j; c < k; ++c)
    {
      double* y = &Qc[c * rows + j];
      double w = y[0];
      for (int64_t i = 1; i < len; ++i)
        w += x[i] * y[i];
      w *= t;
      y[0] -= w;
      for (int64_t i = 1; i < len; ++i)
        y[i] -= w * x[i];
    }
  }
  Q = Mat(rows, k);
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < k; ++j)
      Q(i, j) = Qc[j * rows + i];
}

// ---------------------------------------------------------------------------
// One-sided Jacobi SVD (Hestenes).  Stand-in for svd_thin
// (types/tt_eigen_bridge.hpp:67-104): U (rows x k), s (k, descending),
// Vt (k x cols), k = min(rows, cols).  For rows < cols the transpose is
// decomposed.  Columns whose norm is exactly zero get an orthonormal
// completion so that U keeps orthonormal columns, as BDCSVD's U does.
// ---------------------------------------------------------------------------
inline void complete_orthonormal(std::vector<double>& Uc, int64_t rows, int64_t k,
                                 const std::vector<char>& good)
{
  // Uc column-major (rows x k).  Fill columns with good[j]==0 by
  // Gram-Schmidt (twice) of unit vectors against the accepted columns.
  std::vector<char> acc(good.begin(), good.end());
  int64_t e = 0;
  for (int64_t j = 0; j < k; ++j)
  {
    if (acc[j])
      continue;
    for (; e < rows; ++e)
    {
      std::vector<double> v(static_cast<size_t>(rows), 0.0);
      v[e] = 1.0;
      for (int pass = 0; pass < 2; ++pass)
        for (int64_t c = 0; c < k; ++c)
        {
          if (!acc[c])
            continue;
          const double* u = &Uc[c * rows];
          double dot = 0.0;
          for (int64_t i = 0; i < rows; ++i)
            dot += u[i] * v[i];
          for (int64_t i = 0; i < rows; ++i)
            v[i] -= dot * u[i];
        }
      double nv = 0.0;
      for (int64_t i = 0; i < rows; ++i)
        nv += v[i] * v[i];
      nv = std::sqrt(nv);
      if (nv > 0.5)
      {
        for (int64_t i = 0; i < rows; ++i)
          Uc[j * rows + i] = v[i] / nv;
        acc[j] = 1;
        ++e;
        break;
      }
    }
  }
}

inline void jacobi_svd_tall(const double* M, int64_t rows, int64_t cols,
                            Mat& U, std::vector<double>& s, Mat& Vt)
{
  // rows >= cols.  A column-major (rows x cols), V column-major (cols x cols).
  const int64_t k = cols;
  std::vector<double> A(static_cast<size_t>(rows * cols));
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < cols; ++j)
      A[j * rows + i] = M[i * cols + j];
  std::vector<double> V(static_cast<size_t>(cols * cols), 0.0);
  for (int64_t j = 0; j < cols; ++j)
    V[j * cols + j] = 1.0;
  const double eps = std::numeric_limits<double>::epsilon();
  const int max_sweeps = 80;
  for (int sweep = 0; sweep < max_sweeps; ++sweep)
  {
    bool rotated = false;
    for (int64_t p = 0; p + 1 < cols; ++p)
      for (int64_t q = p + 1; q < cols; ++q)
      {
        double* ap = &A[p * rows];
        double* aq = &A[q * rows];
        double alpha = 0.0, beta = 0.0, gamma = 0.0;
        for (int64_t i = 0; i < rows; ++i)
        {
          alpha += ap[i] * ap[i];
          beta += aq[i] * aq[i];
          gamma += ap[i] * aq[i];
        }
        if (gamma == 0.0 || std::fabs(gamma) <= eps * std::sqrt(alpha * beta))
          continue;
        rotated = true;
        const double zeta = (beta - alpha) / (2.0 * gamma);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t);
        const double sn = c * t;
        for (int64_t i = 0; i < rows; ++i)
        {
          const double x = ap[i], y = aq[i];
          ap[i] = c * x - sn * y;
          aq[i] = sn * x + c * y;
        }
        double* vp = &V[p * cols];
        double* vq = &V[q * cols];
        for (int64_t i = 0; i < cols; ++i)
        {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - sn * y;
          vq[i] = sn * x + c * y;
        }
      }
    if (!rotated)
      break;
  }
  std::vector<double> sig(static_cast<size_t>(k));
  for (int64_t j = 0; j < k; ++j)
  {
    double nn = 0.0;
    for (int64_t i = 0; i < rows; ++i)
      nn += A[j * rows + i] * A[j * rows + i];
    sig[j] = std::sqrt(nn);
  }
  std::vector<int64_t> order(static_cast<size_t>(k));
  for (int64_t j = 0; j < k; ++j)
    order[j] = j;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return sig[a] > sig[b]; });
  std::vector<double> Uc(static_cast<size_t>(rows * k), 0.0);
  std::vector<char> good(static_cast<size_t>(k), 0);
  s.assign(static_cast<size_t>(k), 0.0);
  Vt = Mat(k, cols);
  for (int64_t jj = 0; jj < k; ++jj)
  {
    const int64_t j = order[jj];
    s[jj] = sig[j];
    if (sig[j] > 0.0)
    {
      for (int64_t i = 0; i < rows; ++i)
        Uc[jj * rows + i] = A[j * rows + i] / sig[j];
      good[jj] = 1;
    }
    for (int64_t i = 0; i < cols; ++i)
      Vt(jj, i) = V[j * cols + i];
  }
  complete_orthonormal(Uc, rows, k, good);
  U = Mat(rows, k);
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < k; ++j)
      U(i, j) = Uc[j * rows + i];
}

inline void svd_thin(const double* M, int64_t rows, int64_t cols,
                     Mat& U, std::vector<double>& s, Mat& Vt)
{
  if (rows <= 0 || cols <= 0)
  {
    U = Mat();
    Vt = Mat();
    s.clear();
    return;
  }
  if (rows >= cols)
  {
    jacobi_svd_tall(M, rows, cols, U, s, Vt);
    return;
  }
  // M^T = U' s V'^T  =>  M = V' s U'^T.
  std::vector<double> MT(static_cast<size_t>(rows * cols));
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < cols; ++j)
      MT[j * rows + i] = M[i * cols + j];
  Mat U2, Vt2;
  jacobi_svd_tall(MT.data(), cols, rows, U2, s, Vt2);
  U = transpose(Vt2);   // (rows x k)
  Vt = transpose(U2);   // (k x cols)
}

// truncate_eps_rank (types/tt_eigen_bridge.hpp:172-197): scan the tail from
// the smallest singular value; keep the largest dropped set with
// sum s_i^2 <= delta^2; at least 1; cap at max_rank when > 0.
inline int truncate_eps_rank(const std::vector<double>& s, double delta, int max_rank = 0)
{
  const int n = static_cast<int>(s.size());
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

// frob_norm_buffer (detail/shape_check.hpp:164-172).
inline double frob_norm_buffer(const double* p, size_t n)
{
  double s2 = 0.0;
  for (size_t i = 0; i < n; ++i)
    s2 += p[i] * p[i];
  return std::sqrt(s2);
}

// ---------------------------------------------------------------------------
// Core contractions (detail/contract.hpp:33-77, detail/core_view.hpp:28-57).
// ---------------------------------------------------------------------------
// M (rows x c.r) * right_unfold(c) (c.r x n*rp)  ->  core (M.rows, n, rp).
inline Core apply_left_factor(const Mat& M, const Core& c)
{
  if (M.cols != c.r)
    fail("apply_left_factor: M.cols != c.r_left");
  Core out(static_cast<int>(M.rows), c.n, c.rp);
  const int64_t w = static_cast<int64_t>(c.n) * c.rp;
  gemm_nn(M.rows, w, c.r, M.data(), M.cols, c.v.data(), w, out.v.data(), w);
  return out;
}

// left_unfold(c) (r*n x rp) * M (rp x cols)  ->  core (r, n, M.cols).
inline Core apply_right_factor(const Core& c, const Mat& M)
{
  if (M.rows != c.rp)
    fail("apply_right_factor: M.rows != c.r_right");
  Core out(c.r, c.n, static_cast<int>(M.cols));
  const int64_t h = static_cast<int64_t>(c.r) * c.n;
  gemm_nn(h, M.cols, c.rp, c.v.data(), c.rp, M.data(), M.cols, out.v.data(), M.cols);
  return out;
}

// ---------------------------------------------------------------------------
// QR sweep steps (detail/orthogonalize.hpp:35-100).
// ---------------------------------------------------------------------------
inline void left_qr_step(Core& cur, Core& next)
{
  if (cur.rp != next.r)
    fail("left_qr_step: rank mismatch");
  const int64_t m = static_cast<int64_t>(cur.r) * cur.n;
  const int k = static_cast<int>(std::min<int64_t>(m, cur.rp));
  Mat Q, R;
  qr_thin(cur.v.data(), m, cur.rp, Q, R);
  Core nc(cur.r, cur.n, k);
  std::memcpy(nc.v.data(), Q.data(), sizeof(double) * nc.size());
  next = apply_left_factor(R, next);
  cur = std::move(nc);
}

// QR of M^T (n*rp x r); r_eff = min(n*rp, r) may shrink the bond
// (orthogonalize.hpp:84); L = R^T is absorbed into prev.
inline void right_qr_step(Core& cur, Core& prev)
{
  if (cur.r != prev.rp)
    fail("right_qr_step: rank mismatch");
  const int r = cur.r;
  const int64_t m = static_cast<int64_t>(cur.n) * cur.rp;
  // M^T row-major (m x r).
  std::vector<double> MT(static_cast<size_t>(m * r));
  for (int a = 0; a < r; ++a)
    for (int64_t j = 0; j < m; ++j)
      MT[j * r + a] = cur.v[a * m + j];
  Mat Q, R;
  qr_thin(MT.data(), m, r, Q, R);
  const int r_eff = static_cast<int>(std::min<int64_t>(m, r));
  trace().add("rqr m=" + std::to_string(m) + " c=" + std::to_string(r) +
              " reff=" + std::to_string(r_eff));
  Core nc(r_eff, cur.n, cur.rp);
  // right_unfold(new) (r_eff x m) = Q^T.
  for (int a = 0; a < r_eff; ++a)
    for (int64_t j = 0; j < m; ++j)
      nc.v[a * m + j] = Q(j, a);
  prev = apply_right_factor(prev, transpose(R));  // L = R^T (r x r_eff)
  cur = std::move(nc);
}

// ---------------------------------------------------------------------------
// Truncation steps (detail/truncate.hpp:27-166).
// ---------------------------------------------------------------------------
inline Mat diag_scale_rows(const Mat& M, const std::vector<double>& s, int r)
{
  Mat F(r, M.cols);
  for (int i = 0; i < r; ++i)
    for (int64_t j = 0; j < M.cols; ++j)
      F(i, j) = M(i, j) * s[i];
  return F;
}

inline Mat diag_scale_cols(const Mat& M, const std::vector<double>& s, int r)
{
  Mat F(M.rows, r);
  for (int64_t i = 0; i < M.rows; ++i)
    for (int j = 0; j < r; ++j)
      F(i, j) = M(i, j) * s[j];
  return F;
}

inline int svd_step(Core& cur, Core& next, double delta, int max_rank = 0)
{
  const int r = cur.r, n = cur.n, rp = cur.rp;
  const int64_t rows = static_cast<int64_t>(r) * n;
  const int cols = rp;
  Mat U, Vt;
  std::vector<double> s;
  if (rows >= 2 * static_cast<int64_t>(cols) && cols > 0)
  {
    Mat Q, R, Ur, Vtr;
    qr_thin(cur.v.data(), rows, cols, Q, R);
    svd_thin(R.data(), cols, cols, Ur, s, Vtr);
    U = matmul(Q, Ur);
    Vt = std::move(Vtr);
  }
  else
  {
    svd_thin(cur.v.data(), rows, cols, U, s, Vt);
  }
  const int r_new = truncate_eps_rank(s, delta, max_rank);
  trace().add("svd rows=" + std::to_string(rows) + " cols=" + std::to_string(cols) +
              " rnew=" + std::to_string(r_new));
  Core nc(r, n, r_new);
  for (int64_t i = 0; i < rows; ++i)
    for (int j = 0; j < r_new; ++j)
      nc.v[i * r_new + j] = U(i, j);
  cur = std::move(nc);
  next = apply_left_factor(diag_scale_rows(Vt, s, r_new), next);
  return r_new;
}

inline int svd_step_right(Core& cur, Core& prev, double delta, int max_rank = 0)
{
  const int r = cur.r, n = cur.n, rp = cur.rp;
  const int rows = r;
  const int64_t cols = static_cast<int64_t>(n) * rp;
  Mat U, Vt;
  std::vector<double> s;
  if (cols >= 2 * static_cast<int64_t>(rows) && rows > 0)
  {
    // Wide: M^T = Q R; svd(R^T) = Ur s Vtr; Vt = Vtr Q^T.
    std::vector<double> MT(static_cast<size_t>(cols * rows));
    for (int a = 0; a < rows; ++a)
      for (int64_t j = 0; j < cols; ++j)
        MT[j * rows + a] = cur.v[a * cols + j];
    Mat Q, R, Ur, Vtr;
    qr_thin(MT.data(), cols, rows, Q, R);
    Mat Rt = transpose(R);
    svd_thin(Rt.data(), rows, rows, Ur, s, Vtr);
    U = std::move(Ur);
    Vt = matmul(Vtr, transpose(Q));
  }
  else if (rows >= 2 * cols && cols > 0)
  {
    Mat Q, R, Ur, Vtr;
    qr_thin(cur.v.data(), rows, cols, Q, R);
    svd_thin(R.data(), cols, cols, Ur, s, Vtr);
    U = matmul(Q, Ur);
    Vt = std::move(Vtr);
  }
  else
  {
    svd_thin(cur.v.data(), rows, cols, U, s, Vt);
  }
  const int r_new = truncate_eps_rank(s, delta, max_rank);
  Core nc(r_new, n, rp);
  for (int a = 0; a < r_new; ++a)
    for (int64_t j = 0; j < cols; ++j)
      nc.v[a * cols + j] = Vt(a, j);
  cur = std::move(nc);
  prev = apply_right_factor(prev, diag_scale_cols(U, s, r_new));
  return r_new;
}

// Gauge sweeps (gauge/tt_orthogonalize.hpp:26-58).
inline void right_orthogonalize(TT& a)
{
  const int d = a.d();
  if (d <= 1)
    return;
  for (int k = d - 1; k >= 1; --k)
    right_qr_step(a.c[k], a.c[k - 1]);
}

inline void left_orthogonalize(TT& a)
{
  const int d = a.d();
  if (d <= 1)
    return;
  for (int k = 0; k < d - 1; ++k)
    left_qr_step(a.c[k], a.c[k + 1]);
}

// make_rank1_zero_tt (detail/shape_check.hpp:176-188).
inline TT make_rank1_zero(const TT& like)
{
  TT z;
  z.matrix = like.matrix;
  z.mrow = like.mrow;
  z.ncol = like.ncol;
  for (auto& c : like.c)
    z.c.emplace_back(1, c.n, 1);
  return z;
}

// ---------------------------------------------------------------------------
// detail::round (round/tt_round.hpp:36-127), by value.
// ---------------------------------------------------------------------------
inline TT round(TT acc, double eps = 1.0e-10, int max_rank = 0)
{
  const int d = acc.d();
  if (d <= 1)
    return acc;
  right_orthogonalize(acc);
  auto& cs = acc.c;
  const double norm = frob_norm_buffer(cs[0].v.data(), cs[0].size());
  if (norm == 0.0)
    return make_rank1_zero(acc);
  const double delta = eps * norm / std::sqrt(static_cast<double>(std::max(d - 1, 1)));
  trace().add("norm=" + std::to_string(norm) + " delta=" + std::to_string(delta));
  for (int k = 0; k < d - 1; ++k)
    svd_step(cs[k], cs[k + 1], delta, max_rank);

  // Norm balancing (tt_round.hpp:65-124): scale the columns of
  // left_unfold(c_k), k < d-1, to the geometric mean of all positive column
  // norms; divide the matching rows of right_unfold(c_{k+1}).
  std::vector<std::vector<double>> col_norms(static_cast<size_t>(d));
  double total_log = 0.0;
  int total_cols = 0;
  for (int k = 0; k < d - 1; ++k)
  {
    const Core& c = cs[k];
    const int64_t h = static_cast<int64_t>(c.r) * c.n;
    col_norms[k].assign(static_cast<size_t>(c.rp), 0.0);
    for (int col = 0; col < c.rp; ++col)
    {
      double s2 = 0.0;
      for (int64_t i = 0; i < h; ++i)
        s2 += c.v[i * c.rp + col] * c.v[i * c.rp + col];
      const double nc = std::sqrt(s2);
      col_norms[k][col] = nc;
      if (nc > 0.0)
      {
        total_log += std::log(nc);
        ++total_cols;
      }
    }
  }
  if (total_cols > 0)
  {
    const double geo = std::exp(total_log / static_cast<double>(total_cols));
    for (int k = 0; k < d - 1; ++k)
    {
      Core& c = cs[k];
      Core& cn = cs[k + 1];
      const int64_t h = static_cast<int64_t>(c.r) * c.n;
      const int64_t w = static_cast<int64_t>(cn.n) * cn.rp;
      for (int col = 0; col < c.rp; ++col)
      {
        const double nc = col_norms[k][col];
        if (nc > 0.0)
        {
          const double scl = geo / nc;
          for (int64_t i = 0; i < h; ++i)
            c.v[i * c.rp + col] *= scl;
          for (int64_t j = 0; j < w; ++j)
            cn.v[col * w + j] /= scl;
        }
      }
    }
  }
  return acc;
}

// detail::round_right_canonical (round/tt_round.hpp:151-183).
inline TT round_right_canonical(TT acc, double eps = 1.0e-10, int max_rank = 0)
{
  const int d = acc.d();
  if (d <= 1)
    return acc;
  left_orthogonalize(acc);
  auto& cs = acc.c;
  const double norm = frob_norm_buffer(cs[d - 1].v.data(), cs[d - 1].size());
  if (norm == 0.0)
    return make_rank1_zero(acc);
  const double delta = eps * norm / std::sqrt(static_cast<double>(std::max(d - 1, 1)));
  for (int k = d - 1; k >= 1; --k)
    svd_step_right(cs[k], cs[k - 1], delta, max_rank);
  return acc;
}

// ---------------------------------------------------------------------------
// MPO apply (apply/tt_matrix_apply.hpp:40-271).
// y(a*s+ax, i, b*sp+bx) = sum_j A(a,i,j,b) x(ax,j,bx).
// ---------------------------------------------------------------------------
inline Core matvec_core(const Core& A, int m, int n, const Core& x)
{
  if (x.n != n)
    fail("matvec: mode mismatch");
  const int r = A.r, rp = A.rp, s = x.r, sp = x.rp;
  Core out(r * s, m, rp * sp);
  for (int a = 0; a < r; ++a)
    for (int i = 0; i < m; ++i)
      for (int b = 0; b < rp; ++b)
        for (int ax = 0; ax < s; ++ax)
          for (int bx = 0; bx < sp; ++bx)
          {
            double acc = 0.0;
            for (int j = 0; j < n; ++j)
              acc += A.v[((static_cast<size_t>(a) * m + i) * n + j) * rp + b] *
                     x.v[(static_cast<size_t>(ax) * n + j) * sp + bx];
            out(a * s + ax, i, b * sp + bx) = acc;
          }
  return out;
}

// y(a*s+ax, i, j, b*sp+bx) = sum_p A(a,i,p,b) B(ax,p,j,bx).
inline Core matmat_core(const Core& A, int m, int p, const Core& B, int n)
{
  const int r = A.r, rp = A.rp, s = B.r, sp = B.rp;
  if (B.n != p * n)
    fail("matmat: mode mismatch");
  Core out(r * s, m * n, rp * sp);
  for (int a = 0; a < r; ++a)
    for (int i = 0; i < m; ++i)
      for (int b = 0; b < rp; ++b)
        for (int ax = 0; ax < s; ++ax)
          for (int j = 0; j < n; ++j)
            for (int bx = 0; bx < sp; ++bx)
            {
              double acc = 0.0;
              for (int q = 0; q < p; ++q)
                acc += A.v[((static_cast<size_t>(a) * m + i) * p + q) * rp + b] *
                       B.v[((static_cast<size_t>(ax) * p + q) * n + j) * sp + bx];
              out.v[((static_cast<size_t>(a * s + ax) * m + i) * n + j) * (rp * sp) +
                    b * sp + bx] = acc;
            }
  return out;
}

inline void check_matvec(const TT& A, const TT& x)
{
  if (!A.matrix || x.matrix)
    fail("matvec: operand kinds");
  if (A.d() != x.d())
    fail("matvec: d mismatch");
  for (int k = 0; k < A.d(); ++k)
    if (A.ncol[k] != x.c[k].n)
      fail("matvec: mode-size mismatch at axis " + std::to_string(k));
}

inline void check_matmat(const TT& A, const TT& B)
{
  if (!A.matrix || !B.matrix)
    fail("matmat: operand kinds");
  if (A.d() != B.d())
    fail("matmat: d mismatch");
  for (int k = 0; k < A.d(); ++k)
    if (A.ncol[k] != B.mrow[k])
      fail("matmat: inner-dimension mismatch at axis " + std::to_string(k));
}

inline TT matvec(const TT& A, const TT& x)
{
  check_matvec(A, x);
  TT y;
  for (int k = 0; k < A.d(); ++k)
    y.c.push_back(matvec_core(A.c[k], A.mrow[k], A.ncol[k], x.c[k]));
  return y;
}

inline TT matmat(const TT& A, const TT& B)
{
  check_matmat(A, B);
  TT y;
  y.matrix = true;
  for (int k = 0; k < A.d(); ++k)
  {
    y.c.push_back(matmat_core(A.c[k], A.mrow[k], A.ncol[k], B.c[k], B.ncol[k]));
    y.mrow.push_back(A.mrow[k]);
    y.ncol.push_back(B.ncol[k]);
  }
  return y;
}

// ---------------------------------------------------------------------------
// Fused streaming apply (detail/fused_apply_core.hpp:33-272,
// detail/streaming_apply.hpp:39-202).
// out(al, i, b*bx') = sum_{a, ax, j} F(al, a*sx+ax) A(a,i,j,b) x(ax,j,bx).
// Matmat: out(al, i, j, b*bx') = sum F(al, a*sx+ax) A(a,i,q,b) B(ax,q,j,bx).
// Both are computed here as the same contraction with the output's j axis
// of size `nout` (1 for matvec).
// ---------------------------------------------------------------------------
inline Core fused_apply_core(const Mat& F, const Core& A, int m, int p,
                             const Core& X, int nout)
{
  const int alpha = static_cast<int>(F.rows);
  const int a = A.r, b = A.rp, sx = X.r, bx = X.rp;
  if (F.cols != static_cast<int64_t>(a) * sx)
    fail("fused_apply: F cols != a*sx");
  if (X.n != p * nout)
    fail("fused_apply: mode mismatch");
  // G1(al, ax, i, q, b) = sum_a F(al, a*sx+ax) A(a, i, q, b).
  const int64_t mpb = static_cast<int64_t>(m) * p * b;
  std::vector<double> G1(static_cast<size_t>(alpha) * sx * mpb, 0.0);
  for (int al = 0; al < alpha; ++al)
    for (int ax = 0; ax < sx; ++ax)
    {
      double* g = &G1[(static_cast<size_t>(al) * sx + ax) * mpb];
      for (int aa = 0; aa < a; ++aa)
      {
        const double f = F(al, static_cast<int64_t>(aa) * sx + ax);
        const double* ar = &A.v[static_cast<size_t>(aa) * mpb];
        for (int64_t t = 0; t < mpb; ++t)
          g[t] += f * ar[t];
      }
    }
  // out(al, i, j, b, bx) = sum_{ax, q} G1(al, ax, i, q, b) X(ax, q, j, bx).
  Core out(alpha, m * nout, b * bx);
  for (int al = 0; al < alpha; ++al)
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < nout; ++j)
        for (int bb = 0; bb < b; ++bb)
        {
          double* o = &out.v[((static_cast<size_t>(al) * m + i) * nout + j) *
                                 (static_cast<size_t>(b) * bx) +
                             static_cast<size_t>(bb) * bx];
          for (int ax = 0; ax < sx; ++ax)
            for (int q = 0; q < p; ++q)
            {
              const double g = G1[((static_cast<size_t>(al) * sx + ax) * m + i) * (p * b) +
                                  static_cast<size_t>(q) * b + bb];
              const double* xr = &X.v[((static_cast<size_t>(ax) * p + q) * nout + j) * bx];
              for (int t = 0; t < bx; ++t)
                o[t] += g * xr[t];
            }
        }
  return out;
}

// Right-orthogonalize a TT-matrix (gauge/tt_matrix_orthogonalize.hpp:34-86):
// the packed 3-axis cores are swept exactly like a TT.
inline void right_orthogonalize_any(TT& a) { right_orthogonalize(a); }

// build_streaming_matvec / build_streaming_matmat
// (detail/streaming_apply.hpp:39-110, 115-202).
inline TT build_streaming(const TT& a_in, const TT& x_in, double eps, int max_rank,
                          bool matrix_out)
{
  if (matrix_out)
    check_matmat(a_in, x_in);
  else
    check_matvec(a_in, x_in);
  const int d = a_in.d();
  if (d == 0)
    fail("build_streaming: d=0 not supported");
  TT A = a_in, X = x_in;
  right_orthogonalize(A);
  right_orthogonalize(X);
  const double nA = frob_norm_buffer(A.c[0].v.data(), A.c[0].size());
  const double nX = frob_norm_buffer(X.c[0].v.data(), X.c[0].size());
  const double norm = nA * nX;
  TT out;
  out.matrix = matrix_out;
  if (matrix_out)
  {
    out.mrow = a_in.mrow;
    out.ncol = x_in.ncol;
  }
  if (norm == 0.0)
  {
    for (int k = 0; k < d; ++k)
      out.c.emplace_back(1, matrix_out ? a_in.mrow[k] * x_in.ncol[k] : a_in.mrow[k], 1);
    return out;
  }
  const double delta = eps * norm / std::sqrt(static_cast<double>(std::max(d - 1, 1)));
  Mat F(1, 1);
  F(0, 0) = 1.0;
  for (int k = 0; k < d; ++k)
  {
    const int nout = matrix_out ? x_in.ncol[k] : 1;
    Core Cj = fused_apply_core(F, A.c[k], a_in.mrow[k], a_in.ncol[k], X.c[k], nout);
    if (k == d - 1)
    {
      out.c.push_back(std::move(Cj));
      break;
    }
    const int64_t rows = static_cast<int64_t>(Cj.r) * Cj.n;
    Mat U, Vt;
    std::vector<double> s;
    svd_thin(Cj.v.data(), rows, Cj.rp, U, s, Vt);
    const int r_new = truncate_eps_rank(s, delta, max_rank);
    trace().add("stream rows=" + std::to_string(rows) + " cols=" + std::to_string(Cj.rp) +
                " rnew=" + std::to_string(r_new));
    Core nc(Cj.r, Cj.n, r_new);
    for (int64_t i = 0; i < rows; ++i)
      for (int j = 0; j < r_new; ++j)
        nc.v[i * r_new + j] = U(i, j);
    out.c.push_back(std::move(nc));
    F = diag_scale_rows(Vt, s, r_new);
  }
  return out;
}

// round_matrix via pack/unpack (round/tt_matrix_round.hpp:27-72): the
// packed cores are rounded as a TT; m/n per site are carried through.
inline TT round_matrix(const TT& a, double eps, int max_rank, bool right_canonical)
{
  TT packed = a;
  packed.matrix = false;
  TT r = right_canonical ? round_right_canonical(std::move(packed), eps, max_rank)
                         : round(std::move(packed), eps, max_rank);
  r.matrix = true;
  r.mrow = a.mrow;
  r.ncol = a.ncol;
  return r;
}

// matvec_round (round/tt_matrix_apply_round.hpp:32-62): svd = naive
// round(matvec(A, x)); svd_streaming = fused; d <= 1 falls back to naive.
inline TT matvec_round(const TT& A, const TT& x, double eps, int max_rank, bool streaming)
{
  if (!streaming || A.d() <= 1)
  {
    if (A.d() != x.d())
      fail("matvec_round: core count mismatch");
    return round(matvec(A, x), eps, max_rank);
  }
  return build_streaming(A, x, eps, max_rank, false);
}

// matmat_round (round/tt_matrix_apply_round.hpp:66-92): svd = streaming,
// svd_naive = round_matrix(matmat(A, B)); d <= 1 falls back to naive.
inline TT matmat_round(const TT& A, const TT& B, double eps, int max_rank, bool naive)
{
  if (A.d() != B.d())
    fail("matmat_round: core count mismatch");
  if (naive || A.d() <= 1)
    return round_matrix(matmat(A, B), eps, max_rank, false);
  return build_streaming(A, B, eps, max_rank, true);
}

// ---------------------------------------------------------------------------
// eval (algebra/tt_eval.hpp:32-112).
// ---------------------------------------------------------------------------
inline double eval_at(const TT& a, const int* idx)
{
  if (!idx)
    fail("eval_at: idx pointer is null");
  const int d = a.d();
  if (d == 0)
    fail("eval_at: TT is empty (d=0)");
  for (int k = 0; k < d; ++k)
    if (idx[k] < 0 || idx[k] >= a.c[k].n)
      fail("eval_at: idx[" + std::to_string(k) + "] out of range");
  std::vector<double> v(a.c[0].rp), w;
  for (int b = 0; b < a.c[0].rp; ++b)
    v[b] = a.c[0](0, idx[0], b);
  for (int k = 1; k < d; ++k)
  {
    const Core& c = a.c[k];
    w.assign(static_cast<size_t>(c.rp), 0.0);
    for (int aa = 0; aa < c.r; ++aa)
    {
      const double va = v[aa];
      const double* row = &c.v[(static_cast<size_t>(aa) * c.n + idx[k]) * c.rp];
      for (int b = 0; b < c.rp; ++b)
        w[b] += va * row[b];
    }
    v.swap(w);
  }
  return v[0];
}

inline std::vector<double> eval_batch(const TT& a, const int* idx, int M)
{
  if (!idx && M > 0)
    fail("eval_batch: idx pointer is null");
  if (M < 0)
    fail("eval_batch: M must be non-negative");
  if (a.d() == 0)
    fail("eval_batch: TT is empty (d=0)");
  std::vector<double> out(static_cast<size_t>(M), 0.0);
  for (int j = 0; j < M; ++j)
    out[j] = eval_at(a, idx + static_cast<ptrdiff_t>(j) * a.d());
  return out;
}

// contract_inner_step (detail/contract.hpp:155-205): E (ra x rb) ->
// E' (rap x rbp) = sum over (a, b, i) of E(a, b) ca(a, i, :) cb(b, i, :).
inline Mat contract_inner_step(const Mat& E, const Core& ca, const Core& cb)
{
  // tmp (rb, n*rap) = E^T (rb x ra) * right_unfold(ca).
  const int64_t nrap = static_cast<int64_t>(ca.n) * ca.rp;
  Mat Et = transpose(E);
  Mat tmp(cb.r, nrap);
  gemm_nn(cb.r, nrap, ca.r, Et.data(), Et.cols, ca.v.data(), nrap, tmp.data(), nrap);
  // E' (rap, rbp) = tmp_as^T (rap x rb*n) * left_unfold(cb) (rb*n x rbp).
  Mat En(ca.rp, cb.rp);
  const int64_t rbn = static_cast<int64_t>(cb.r) * cb.n;
  for (int64_t t = 0; t < rbn; ++t)
    for (int p = 0; p < ca.rp; ++p)
    {
      const double x = tmp.v[t * ca.rp + p];
      const double* brow = &cb.v[t * cb.rp];
      for (int q = 0; q < cb.rp; ++q)
        En(p, q) += x * brow[q];
    }
  return En;
}

// inner / norm (algebra/tt_inner.hpp:33-59, detail/contract.hpp:155-205).
inline double inner(const TT& a, const TT& b)
{
  if (a.d() != b.d())
    fail("inner: rank-d mismatch");
  for (int k = 0; k < a.d(); ++k)
    if (a.c[k].n != b.c[k].n)
      fail("inner: mode-size mismatch at axis " + std::to_string(k));
  const int d = a.d();
  if (d == 0)
    return 0.0;
  Mat E(1, 1);
  E(0, 0) = 1.0;
  for (int k = 0; k < d; ++k)
    E = contract_inner_step(E, a.c[k], b.c[k]);
  return E(0, 0);
}

inline double norm(const TT& a)
{
  const double s = inner(a, a);
  return std::sqrt(std::max(s, 0.0));
}

// frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98): ||A x||_F
// or ||A B||_F.  Per site the product core (matvec_core, or matmat_core read
// as a 3-axis core of mode m*n) goes straight into one contract_inner_step
// of the product with itself; the product TT is never held whole.
inline double frob_norm_apply(const TT& A, const TT& X)
{
  if (X.matrix)
    check_matmat(A, X);
  else
    check_matvec(A, X);
  const int d = A.d();
  if (d == 0)
    return 0.0;
  Mat E(1, 1);
  E(0, 0) = 1.0;
  for (int k = 0; k < d; ++k)
  {
    const Core y = X.matrix ? matmat_core(A.c[k], A.mrow[k], A.ncol[k], X.c[k], X.ncol[k])
                            : matvec_core(A.c[k], A.mrow[k], A.ncol[k], X.c[k]);
    E = contract_inner_step(E, y, y);
  }
  return std::sqrt(std::max(E(0, 0), 0.0));
}

// soft_threshold (round/tt_soft_threshold.hpp:42-178): proximal step of the
// nuclear norm, bond by bond.  d <= 1 or tau <= 0 returns the input.  Else
// right_orthogonalize, then for k = d-1 .. 1: M = left_unfold(c_{k-1})
// right_unfold(c_k) (rL*n_{k-1} x n_k*rR), its thin SVD, s' = max(s - tau, 0)
// and r_keep = the last index with s' > 0; c_{k-1} <- U[:, :r_keep]
// diag(s'), c_k <- V^T[:r_keep, :].  When every value shrinks to zero both
// cores become rank-1 zero cores.
inline TT soft_threshold(TT acc, double tau)
{
  const int d = acc.d();
  if (d <= 1 || tau <= 0.0)
    return acc;
  right_orthogonalize(acc);
  for (int k = d - 1; k >= 1; --k)
  {
    Core& prev = acc.c[k - 1];
    Core& cur = acc.c[k];
    const int rL = prev.r, np = prev.n, r = prev.rp, nc = cur.n, rR = cur.rp;
    const int64_t rows = static_cast<int64_t>(rL) * np, cols = static_cast<int64_t>(nc) * rR;
    Mat M(rows, cols);
    gemm_nn(rows, cols, r, prev.v.data(), r, cur.v.data(), cols, M.data(), cols);
    Mat U, Vt;
    std::vector<double> s;
    svd_thin(M.data(), rows, cols, U, s, Vt);
    int keep = 0;
    for (int j = 0; j < static_cast<int>(s.size()); ++j)
      if (s[j] > tau)
        keep = j + 1;
    if (keep == 0)
    {
      prev = Core(rL, np, 1);
      cur = Core(1, nc, rR);
      continue;
    }
    Core p2(rL, np, keep), c2(keep, nc, rR);
    for (int64_t i = 0; i < rows; ++i)
      for (int j = 0; j < keep; ++j)
        p2.v[static_cast<size_t>(i * keep + j)] = U(i, j) * (s[j] - tau);
    for (int j = 0; j < keep; ++j)
      for (int64_t q = 0; q < cols; ++q)
        c2.v[static_cast<size_t>(j * cols + q)] = Vt(j, q);
    prev = std::move(p2);
    cur = std::move(c2);
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Algebra used to build inputs (algebra/tt_ops.hpp:72-143,
// detail/block_concat.hpp:40-156).
// ---------------------------------------------------------------------------
inline Core axpby_core(int k, int d, const Core& ca, const Core& cb, double alpha, double beta)
{
  const int n = ca.n;
  if (n != cb.n)
    fail("axpby_core: mode size mismatch");
  const bool head = (k == 0), tail = (k == d - 1);
  if (head && (ca.r != 1 || cb.r != 1))
    fail("axpby_core: head rank must be 1");
  if (tail && (ca.rp != 1 || cb.rp != 1))
    fail("axpby_core: tail rank must be 1");
  const int rL = head ? 1 : ca.r + cb.r;
  const int rR = tail ? 1 : ca.rp + cb.rp;
  Core out(rL, n, rR);
  for (int aa = 0; aa < ca.r; ++aa)
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < ca.rp; ++b)
        out(aa, i, b) = (alpha == 1.0) ? ca(aa, i, b) : alpha * ca(aa, i, b);
  const int boff = head ? 0 : ca.r;
  const int coff = tail ? 0 : ca.rp;
  for (int bb = 0; bb < cb.r; ++bb)
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < cb.rp; ++b)
        out(boff + bb, i, coff + b) = (beta == 1.0) ? cb(bb, i, b) : beta * cb(bb, i, b);
  return out;
}

inline TT axpby(double alpha, const TT& a, double beta, const TT& b)
{
  if (a.d() != b.d())
    fail("axpby: rank-d mismatch");
  for (int k = 0; k < a.d(); ++k)
    if (a.c[k].n != b.c[k].n)
      fail("axpby: mode-size mismatch");
  TT out;
  out.matrix = a.matrix;
  out.mrow = a.mrow;
  out.ncol = a.ncol;
  const int d = a.d();
  if (d == 0)
    return out;
  if (d == 1)
  {
    Core c(1, a.c[0].n, 1);
    for (int i = 0; i < c.n; ++i)
      c.v[i] = alpha * a.c[0].v[i] + beta * b.c[0].v[i];
    out.c.push_back(std::move(c));
    return out;
  }
  for (int k = 0; k < d; ++k)
    out.c.push_back(axpby_core(k, d, a.c[k], b.c[k], k == 0 ? alpha : 1.0, k == 0 ? beta : 1.0));
  return out;
}

inline TT add(const TT& a, const TT& b) { return axpby(1.0, a, 1.0, b); }
inline TT sub(const TT& a, const TT& b) { return axpby(1.0, a, -1.0, b); }

// ---------------------------------------------------------------------------
// Factories (factory/tt_factory.hpp:32-207, factory/tt_matrix_factory.hpp:133-191).
// ---------------------------------------------------------------------------
inline TT ones(const std::vector<int>& shape)
{
  TT t;
  for (int n : shape)
  {
    if (n <= 0)
      fail("ones: mode size is not positive");
    Core c(1, n, 1);
    for (int i = 0; i < n; ++i)
      c.v[i] = 1.0;
    t.c.push_back(std::move(c));
  }
  return t;
}

inline TT zeros(const std::vector<int>& shape)
{
  TT t;
  for (int n : shape)
  {
    if (n <= 0)
      fail("zeros: mode size is not positive");
    t.c.emplace_back(1, n, 1);
  }
  return t;
}

// Forward/backward feasibility clipping of ranks (tt_factory.hpp:156-189);
// `mode[k]` is n_k for a TT and m_k*n_k for a TT-matrix.
inline std::vector<int> feasible_ranks(const std::vector<long long>& mode, int max_rank)
{
  const int d = static_cast<int>(mode.size());
  std::vector<int> ranks(static_cast<size_t>(d + 1), 1);
  for (int k = 0; k < d; ++k)
  {
    long long cap = static_cast<long long>(ranks[k]) * mode[k];
    if (cap > max_rank && max_rank > 0)
      cap = max_rank;
    if (cap > std::numeric_limits<int>::max())
      fail("random: rank cap exceeds INT_MAX");
    ranks[k + 1] = static_cast<int>(cap);
  }
  for (int k = d - 1; k >= 0; --k)
  {
    long long cap = static_cast<long long>(ranks[k + 1]) * mode[k];
    if (cap > max_rank && max_rank > 0)
      cap = max_rank;
    if (cap > std::numeric_limits<int>::max())
      fail("random: rank cap exceeds INT_MAX");
    if (cap < ranks[k])
      ranks[k] = static_cast<int>(cap);
  }
  ranks[0] = 1;
  ranks[d] = 1;
  return ranks;
}

inline TT random(const std::vector<int>& shape, int max_rank, uint64_t seed)
{
  std::vector<long long> mode;
  for (int n : shape)
  {
    if (n <= 0)
      fail("random: mode size is not positive");
    mode.push_back(n);
  }
  const std::vector<int> ranks = feasible_ranks(mode, max_rank);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  TT t;
  for (size_t k = 0; k < shape.size(); ++k)
  {
    Core c(ranks[k], shape[k], ranks[k + 1]);
    for (auto& x : c.v)
      x = nd(rng);
    t.c.push_back(std::move(c));
  }
  return t;
}

inline TT random_matrix(const std::vector<int>& rows, const std::vector<int>& cols,
                        int max_rank, uint64_t seed)
{
  if (rows.size() != cols.size())
    fail("random_matrix: row/col shape length mismatch");
  std::vector<long long> mode;
  for (size_t k = 0; k < rows.size(); ++k)
  {
    if (rows[k] <= 0 || cols[k] <= 0)
      fail("random_matrix: mode size is not positive");
    mode.push_back(static_cast<long long>(rows[k]) * cols[k]);
  }
  const std::vector<int> ranks = feasible_ranks(mode, max_rank);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  TT t;
  t.matrix = true;
  t.mrow = rows;
  t.ncol = cols;
  for (size_t k = 0; k < rows.size(); ++k)
  {
    Core c(ranks[k], rows[k] * cols[k], ranks[k + 1]);
    for (auto& x : c.v)
      x = nd(rng);
    t.c.push_back(std::move(c));
  }
  return t;
}

// Per-core scaling 1/sqrt(r_left * mode) applied after random() to give the
// configured N(0,1)/sqrt(r_k*n_k) entries (mode = m*n for a TT-matrix).
inline void scale_by_fan_in(TT& t)
{
  for (auto& c : t.c)
  {
    const double s = 1.0 / std::sqrt(static_cast<double>(c.r) * c.n);
    for (auto& x : c.v)
      x *= s;
  }
}

// Dense reconstruction (types/tt.hpp:145-198).
inline std::vector<double> to_dense(const TT& a)
{
  const int d = a.d();
  if (d == 0)
    return {1.0};
  std::vector<double> T(a.c[0].v);
  int64_t rows = a.c[0].n, cols = a.c[0].rp;
  for (int k = 1; k < d; ++k)
  {
    const Core& c = a.c[k];
    const int64_t w = static_cast<int64_t>(c.n) * c.rp;
    std::vector<double> Tn(static_cast<size_t>(rows * w));
    gemm_nn(rows, w, cols, T.data(), cols, c.v.data(), w, Tn.data(), w);
    T.swap(Tn);
    rows *= c.n;
    cols = c.rp;
  }
  return T;
}

// Stable distance between TTs: ||a - b|| = ||core0|| after right-
// orthogonalising sub(a, b) (the gauge argument of tt_round.hpp:47-52).
inline double norm_qr(const TT& a)
{
  if (a.d() == 0)
    return 0.0;
  TT t = a;
  right_orthogonalize(t);
  return frob_norm_buffer(t.c[0].v.data(), t.c[0].size());
}

inline double rel_err(const TT& y, const TT& yref)
{
  const double den = norm_qr(yref);
  const double num = norm_qr(sub(y, yref));
  return den == 0.0 ? num : num / den;
}

// ---------------------------------------------------------------------------
// Batched uneven workload (4096 TTs): TT i draws from mt19937_64(base + i):
// d ~ U{dmin..dmax}; n_k ~ U{2,4,8}; bond ranks r_k ~ U{rmin..rmax} for
// k = 1..d-1; feasibility clipping as in random(); entries N(0,1) from the
// same generator, then scaled by 1/sqrt(r_k * n_k).
// ---------------------------------------------------------------------------
inline TT random_uneven(uint64_t seed, int dmin, int dmax, int rmin, int rmax)
{
  std::mt19937_64 rng(seed);
  std::uniform_int_distribution<int> ud(dmin, dmax);
  std::uniform_int_distribution<int> un(0, 2);
  std::uniform_int_distribution<int> ur(rmin, rmax);
  const int d = ud(rng);
  std::vector<int> shape(static_cast<size_t>(d));
  for (int k = 0; k < d; ++k)
    shape[k] = 2 << un(rng);
  std::vector<int> ranks(static_cast<size_t>(d + 1), 1);
  for (int k = 1; k < d; ++k)
    ranks[k] = ur(rng);
  for (int k = 0; k < d; ++k)
    ranks[k + 1] = std::min<long long>(ranks[k + 1], static_cast<long long>(ranks[k]) * shape[k]);
  ranks[d] = 1;
  for (int k = d - 1; k >= 0; --k)
    ranks[k] = std::min<long long>(ranks[k], static_cast<long long>(ranks[k + 1]) * shape[k]);
  ranks[0] = 1;
  std::normal_distribution<double> nd(0.0, 1.0);
  TT t;
  for (int k = 0; k < d; ++k)
  {
    Core c(ranks[k], shape[k], ranks[k + 1]);
    for (auto& x : c.v)
      x = nd(rng);
    t.c.push_back(std::move(c));
  }
  scale_by_fan_in(t);
  return t;
}

// ---------------------------------------------------------------------------
// Iterative rounding: ALS and two-site DMRG (round/tt_als.hpp:27-306,
// round/tt_dmrg.hpp:27-309, detail/als_local_solve.hpp,
// detail/dmrg_local_solve.hpp, detail/warm_start.hpp).  Environments are
// the inner-product chains of X against Y from both ends; a local update
// solves for one core (ALS) or a merged pair (DMRG) in the mixed-canonical
// gauge.  Convergence: max over bonds of the relative change of the bond's
// singular values between sweeps.
// ---------------------------------------------------------------------------
struct IterOptions
{
  int max_rank = 0;       // 0: ALS derives it from an SVD round at eps
  double eps = 0.0;
  int max_iters = 20;
  double tol = 1.0e-12;
  uint64_t seed = 0;      // random cold start of the apply variants
  const TT* warm = nullptr;
};

struct IterResult
{
  int iters_run = 0;
  double final_change = 0.0;
  bool converged = false;
};

// contract_inner_step_right (detail/contract.hpp:90-139): F (ca.rp x cb.rp)
// -> F' (ca.r x cb.r) = sum over (i, a', b') ca(a, i, a') F(a', b') cb(b, i, b').
inline Mat contract_inner_step_right(const Core& ca, const Core& cb, const Mat& F)
{
  if (ca.n != cb.n)
    fail("contract_inner_step_right: n_phys mismatch");
  if (F.rows != ca.rp || F.cols != cb.rp)
    fail("contract_inner_step_right: environment shape mismatch");
  const int64_t rows = static_cast<int64_t>(ca.r) * ca.n;
  Mat T1(rows, cb.rp);
  gemm_nn(rows, cb.rp, ca.rp, ca.v.data(), ca.rp, F.data(), F.cols, T1.data(), T1.cols);
  // F' = T1 viewed as (ca.r, n*cb.rp) times right_unfold(cb)^T.
  const int64_t w = static_cast<int64_t>(ca.n) * cb.rp;
  Mat out(ca.r, cb.r);
  for (int a = 0; a < ca.r; ++a)
    for (int b = 0; b < cb.r; ++b)
    {
      double acc = 0.0;
      const double* t = &T1.v[static_cast<size_t>(a) * w];
      const double* c = &cb.v[static_cast<size_t>(b) * w];
      for (int64_t j = 0; j < w; ++j)
        acc += t[j] * c[j];
      out(a, b) = acc;
    }
  return out;
}

// als_local_update (detail/als_local_solve.hpp): X_k = L Y_k R as a core
// (L.rows, n, R.cols).
inline Core als_local_update(const Mat& L, const Core& Yk, const Mat& R)
{
  const int64_t w1 = static_cast<int64_t>(Yk.n) * Yk.rp;
  Mat T1(L.rows, w1);
  gemm_nn(L.rows, w1, Yk.r, L.data(), L.cols, Yk.v.data(), w1, T1.data(), w1);
  Core X(static_cast<int>(L.rows), Yk.n, static_cast<int>(R.cols));
  gemm_nn(L.rows * Yk.n, R.cols, Yk.rp, T1.data(), Yk.rp, R.data(), R.cols, X.v.data(), R.cols);
  return X;
}

inline std::vector<double> core_singular_values(const Core& c)
{
  Mat U, Vt;
  std::vector<double> s;
  svd_thin(c.v.data(), static_cast<int64_t>(c.r) * c.n, c.rp, U, s, Vt);
  return s;
}

// Max over bonds of ||s_now - s_prev|| / ||s_now||; a bond whose size
// changed sets the running value to 1.
inline double sv_change(const std::vector<std::vector<double>>& now,
                        const std::vector<std::vector<double>>& prev)
{
  double worst = 0.0;
  for (size_t k = 0; k < now.size(); ++k)
  {
    if (now[k].size() != prev[k].size())
    {
      worst = 1.0;  // overwrite, as the reference does (tt_als.hpp:182-186)
      continue;
    }
    double dn = 0.0, nn = 0.0;
    for (size_t i = 0; i < now[k].size(); ++i)
    {
      dn += (now[k][i] - prev[k][i]) * (now[k][i] - prev[k][i]);
      nn += now[k][i] * now[k][i];
    }
    worst = std::max(worst, std::sqrt(dn) / (std::sqrt(nn) + 1.0e-300));
  }
  return worst;
}

// als_engine (round/tt_als.hpp:52-206).
inline TT als_engine(const TT& Y, TT X, const IterOptions& o, IterResult* info,
                     bool x_right_canonical)
{
  const int d = Y.d();
  if (d <= 1)
  {
    if (info)
      *info = IterResult{0, 0.0, true};
    TT out;
    if (d == 1)
      out.c.push_back(Y.c[0]);
    return out;
  }
  if (!x_right_canonical)
    right_orthogonalize(X);
  std::vector<Mat> R(static_cast<size_t>(d + 1)), L(static_cast<size_t>(d + 1));
  R[d] = Mat(1, 1);
  R[d](0, 0) = 1.0;
  for (int k = d - 1; k >= 1; --k)
    R[k] = contract_inner_step_right(Y.c[k], X.c[k], R[k + 1]);
  L[0] = Mat(1, 1);
  L[0](0, 0) = 1.0;
  std::vector<std::vector<double>> s_prev;
  double change = 0.0;
  bool converged = false;
  int iters = 0;
  for (int it = 0; it < o.max_iters; ++it)
  {
    for (int k = 0; k < d; ++k)
    {
      X.c[k] = als_local_update(L[k], Y.c[k], R[k + 1]);
      if (k < d - 1)
      {
        left_qr_step(X.c[k], X.c[k + 1]);
        L[k + 1] = contract_inner_step(L[k], X.c[k], Y.c[k]);
      }
    }
    for (int k = d - 1; k >= 0; --k)
    {
      if (k < d - 1)
        X.c[k] = als_local_update(L[k], Y.c[k], R[k + 1]);
      if (k > 0)
      {
        right_qr_step(X.c[k], X.c[k - 1]);
        R[k] = contract_inner_step_right(Y.c[k], X.c[k], R[k + 1]);
      }
    }
    ++iters;
    std::vector<std::vector<double>> s_now;
    for (int k = 0; k < d - 1; ++k)
      s_now.push_back(core_singular_values(X.c[k]));
    change = s_prev.empty() ? 1.0 : sv_change(s_now, s_prev);
    s_prev = std::move(s_now);
    if (change <= o.tol)
    {
      converged = true;
      break;
    }
  }
  if (info)
    *info = IterResult{iters, change, converged};
  return X;
}

// warm_start_tt_compatible (detail/warm_start.hpp): same length and modes.
inline bool warm_compatible(const TT* w, const TT& ref)
{
  if (!w || w->d() != ref.d())
    return false;
  for (int k = 0; k < ref.d(); ++k)
    if (w->c[k].n != ref.c[k].n)
      return false;
  if (w->matrix != ref.matrix)
    return false;
  if (ref.matrix)
    for (int k = 0; k < ref.d(); ++k)
      if (w->mrow[k] != ref.mrow[k] || w->ncol[k] != ref.ncol[k])
        return false;
  return true;
}

inline int tt_max_rank(const TT& t)
{
  int m = 0;
  for (int r : t.ranks())
    m = std::max(m, r);
  return m;
}

inline TT as_packed(TT t)
{
  t.matrix = false;
  t.mrow.clear();
  t.ncol.clear();
  return t;
}

inline TT as_matrix_like(TT t, const TT& like)
{
  t.matrix = like.matrix;
  t.mrow = like.mrow;
  t.ncol = like.ncol;
  return t;
}

// als_round (round/tt_als.hpp:212-300) of a TT, or of a TT-matrix through
// its packed 3-axis cores (round/tt_matrix_als_round.hpp).  cold_random:
// the apply variants start from random(shape, max_rank, seed) instead of
// round_right_canonical (round/tt_matvec_als_round.hpp:88-95,
// round/tt_matmat_als_round.hpp).
inline TT als_round(const TT& Yin, IterOptions o, IterResult* info, bool cold_random = false)
{
  if (std::isnan(o.eps))
    fail("als_round: eps is NaN; must be a valid number");
  const TT Y = as_packed(Yin);
  const int d = Y.d();
  if (d <= 1)
  {
    if (info)
      *info = IterResult{0, 0.0, true};
    return as_matrix_like(round(Y, o.eps, o.max_rank), Yin);
  }
  TT svd_ref;
  TT warm_packed;
  const TT* warm = nullptr;
  if (o.warm && warm_compatible(o.warm, Yin))
  {
    warm_packed = as_packed(*o.warm);
    warm = &warm_packed;
  }
  if (o.max_rank <= 0)
  {
    if (o.eps <= 0.0)
      fail("als_round: max_rank <= 0 and eps <= 0; ALS requires either max_rank > 0 or "
           "eps > 0 to determine compression target");
    svd_ref = round(Y, o.eps, 0);
    o.max_rank = tt_max_rank(svd_ref);
    if (!warm)
      warm = &svd_ref;
  }
  if (warm)
    for (int r : warm->ranks())
      if (r > o.max_rank)
        fail("als_round: warm_start max rank " + std::to_string(r) + " exceeds max_rank " +
             std::to_string(o.max_rank));
  TT X0;
  bool rc = false;
  if (warm)
    X0 = *warm;
  else if (cold_random)
    X0 = random(Y.shape(), o.max_rank, o.seed);
  else
  {
    X0 = round_right_canonical(Y, 0.0, o.max_rank);
    rc = true;
  }
  return as_matrix_like(als_engine(Y, std::move(X0), o, info, rc), Yin);
}

// merge_y_block (detail/dmrg_local_solve.hpp): Theta (rXl*n_k, n_k1*rXr) =
// (L Y_k) (Y_k1 R) with the middle bond of Y contracted.
inline Mat merge_y_block(const Mat& L, const Core& Yk, const Core& Yk1, const Mat& R)
{
  const int64_t w1 = static_cast<int64_t>(Yk.n) * Yk.rp;
  Mat T1(L.rows, w1);
  gemm_nn(L.rows, w1, Yk.r, L.data(), L.cols, Yk.v.data(), w1, T1.data(), w1);
  const int64_t h2 = static_cast<int64_t>(Yk1.r) * Yk1.n;
  Mat T2(h2, R.cols);
  gemm_nn(h2, R.cols, Yk1.rp, Yk1.v.data(), Yk1.rp, R.data(), R.cols, T2.data(), R.cols);
  const int64_t rows = L.rows * Yk.n, cols = static_cast<int64_t>(Yk1.n) * R.cols;
  Mat Th(rows, cols);
  gemm_nn(rows, cols, Yk.rp, T1.data(), Yk.rp, T2.data(), cols, Th.data(), cols);
  return Th;
}

// split_two_site_lr / _rl (detail/dmrg_local_solve.hpp): truncated SVD of
// Theta; lr: X_k <- U, X_k1 <- diag(s) V^T (s_head receives s[:r]);
// rl: X_k <- U diag(s), X_k1 <- V^T.
inline int split_two_site(const Mat& Th, int rXl, int nk, int nk1, int rXr, double delta,
                          int max_rank, bool left_to_right, Core& Xk, Core& Xk1,
                          std::vector<double>* s_head)
{
  Mat U, Vt;
  std::vector<double> s;
  svd_thin(Th.data(), Th.rows, Th.cols, U, s, Vt);
  const int r = truncate_eps_rank(s, delta, max_rank);
  Core a(rXl, nk, r), b(r, nk1, rXr);
  for (int64_t i = 0; i < Th.rows; ++i)
    for (int j = 0; j < r; ++j)
      a.v[static_cast<size_t>(i * r + j)] = left_to_right ? U(i, j) : U(i, j) * s[j];
  for (int j = 0; j < r; ++j)
    for (int64_t q = 0; q < Th.cols; ++q)
      b.v[static_cast<size_t>(j * Th.cols + q)] = left_to_right ? s[j] * Vt(j, q) : Vt(j, q);
  Xk = std::move(a);
  Xk1 = std::move(b);
  if (s_head)
    s_head->assign(s.begin(), s.begin() + r);
  return r;
}

// dmrg_engine (round/tt_dmrg.hpp:45-212).
inline TT dmrg_engine(const TT& Y, TT X, const IterOptions& o, IterResult* info,
                      bool x_right_canonical)
{
  const int d = Y.d();
  if (d <= 1)
  {
    if (info)
      *info = IterResult{0, 0.0, true};
    TT out;
    if (d == 1)
      out.c.push_back(Y.c[0]);
    return out;
  }
  if (!x_right_canonical)
    right_orthogonalize(X);
  const double y_norm = std::sqrt(std::max(inner(Y, Y), 0.0));
  const double delta = o.eps * y_norm / std::sqrt(static_cast<double>(std::max(d - 1, 1)));
  std::vector<Mat> R(static_cast<size_t>(d + 1)), L(static_cast<size_t>(d + 1));
  R[d] = Mat(1, 1);
  R[d](0, 0) = 1.0;
  for (int k = d - 1; k >= 1; --k)
    R[k] = contract_inner_step_right(Y.c[k], X.c[k], R[k + 1]);
  L[0] = Mat(1, 1);
  L[0](0, 0) = 1.0;
  std::vector<std::vector<double>> s_prev, s_now(static_cast<size_t>(d - 1));
  double change = 0.0;
  bool converged = false;
  int iters = 0;
  for (int it = 0; it < o.max_iters; ++it)
  {
    for (int k = 0; k < d - 1; ++k)
    {
      const Mat Th = merge_y_block(L[k], Y.c[k], Y.c[k + 1], R[k + 2]);
      split_two_site(Th, static_cast<int>(L[k].rows), Y.c[k].n, Y.c[k + 1].n,
                     static_cast<int>(R[k + 2].cols), delta, o.max_rank, true, X.c[k],
                     X.c[k + 1], &s_now[k]);
      L[k + 1] = contract_inner_step(L[k], X.c[k], Y.c[k]);
    }
    for (int k = d - 2; k >= 0; --k)
    {
      const Mat Th = merge_y_block(L[k], Y.c[k], Y.c[k + 1], R[k + 2]);
      split_two_site(Th, static_cast<int>(L[k].rows), Y.c[k].n, Y.c[k + 1].n,
                     static_cast<int>(R[k + 2].cols), delta, o.max_rank, false, X.c[k],
                     X.c[k + 1], nullptr);
      R[k + 1] = contract_inner_step_right(Y.c[k + 1], X.c[k + 1], R[k + 2]);
    }
    ++iters;
    change = s_prev.empty() ? 1.0 : sv_change(s_now, s_prev);
    s_prev = s_now;
    if (change <= o.tol)
    {
      converged = true;
      break;
    }
  }
  if (info)
    *info = IterResult{iters, change, converged};
  return X;
}

// dmrg_round (round/tt_dmrg.hpp:217-300), and through packed cores
// (round/tt_matrix_dmrg_round.hpp).  cold_random as for als_round
// (round/tt_matvec_dmrg_round.hpp: random start when max_rank > 0).
inline TT dmrg_round(const TT& Yin, const IterOptions& o, IterResult* info,
                     bool cold_random = false)
{
  if (std::isnan(o.eps) || o.eps <= 0.0)
    fail("dmrg_round: eps must be > 0 for DMRG compression");
  const TT Y = as_packed(Yin);
  const int d = Y.d();
  if (d <= 1)
  {
    if (info)
      *info = IterResult{0, 0.0, true};
    return as_matrix_like(round(Y, o.eps, o.max_rank), Yin);
  }
  TT X0;
  bool rc = false;
  if (o.warm && warm_compatible(o.warm, Yin))
  {
    X0 = as_packed(*o.warm);
    if (o.max_rank > 0)
      for (int r : X0.ranks())
        if (r > o.max_rank)
          fail("dmrg_round: warm_start max rank " + std::to_string(r) + " exceeds max_rank " +
               std::to_string(o.max_rank));
  }
  else if (cold_random && o.max_rank > 0)
    X0 = random(Y.shape(), o.max_rank, o.seed);
  else
  {
    X0 = round_right_canonical(Y, o.eps, o.max_rank);
    rc = true;
  }
  return as_matrix_like(dmrg_engine(Y, std::move(X0), o, info, rc), Yin);
}

}  // namespace ttor
