// tensor_train_gb300.hpp -- the reference's C++20 interface for the TT
// rounding hot path, served by libttgpu.so (ttg.h).
//
// Drop-in for code written against mva::tensor_train (include/tensor_train.hpp
// of the reference) on this path: same namespace, types, option structs and
// free-function signatures.  Storage is host-side and row-major exactly as
// the reference's (types/tt_core.hpp:25-212, types/tt_matrix.hpp:29-36); every
// numerical call crosses the C-ABI into CUDA kernels.  Like the reference,
// invalid input is reported with fprintf(stderr) + abort().
//
// Link: -I<repo>/include -L<repo>/tensor_train_gb300/_build -lttgpu
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <utility>
#include <vector>

#include "ttg.h"

namespace mva
{
namespace tensor_train
{

namespace detail
{
[[noreturn]] inline void die(const char* what, int32_t status)
{
  std::fprintf(stderr, "%s: %s (%s)\n", what, ttg_last_error(), ttg_status_string(status));
  std::abort();
}
inline void check(int32_t status, const char* what)
{
  if (status != TTG_OK)
    die(what, status);
}
}  // namespace detail

// tt_core (types/tt_core.hpp:25-212): (r_left, n_phys, r_right) row-major.
class tt_core
{
 public:
  tt_core() = default;
  tt_core(int r_left, int n_phys, int r_right) : r_(r_left), n_(n_phys), rp_(r_right)
  {
    if (r_left <= 0 || n_phys <= 0 || r_right <= 0)
    {
      std::fprintf(stderr, "tt_core: dimensions must be positive (got %d, %d, %d)\n", r_left,
                   n_phys, r_right);
      std::abort();
    }
    v_.assign(static_cast<size_t>(r_left) * n_phys * r_right, 0.0);
  }
  int r_left() const { return r_; }
  int n_phys() const { return n_; }
  int r_right() const { return rp_; }
  int size() const { return static_cast<int>(v_.size()); }
  double* data() { return v_.data(); }
  const double* data() const { return v_.data(); }
  double& operator()(int a, int i, int b) { return v_[(static_cast<size_t>(a) * n_ + i) * rp_ + b]; }
  double operator()(int a, int i, int b) const
  {
    return v_[(static_cast<size_t>(a) * n_ + i) * rp_ + b];
  }
  void zero_clear() { std::fill(v_.begin(), v_.end(), 0.0); }

 private:
  int r_ = 0, n_ = 0, rp_ = 0;
  std::vector<double> v_;
};

// tt (types/tt.hpp:24-244).
class tt
{
 public:
  tt() = default;
  explicit tt(std::vector<tt_core> cores) : cores_(std::move(cores))
  {
    const int d = static_cast<int>(cores_.size());
    if (d == 0)
      return;
    if (cores_[0].r_left() != 1)
    {
      std::fprintf(stderr, "tt: r_0 must be 1 (got %d)\n", cores_[0].r_left());
      std::abort();
    }
    if (cores_[d - 1].r_right() != 1)
    {
      std::fprintf(stderr, "tt: r_d must be 1 (got %d)\n", cores_[d - 1].r_right());
      std::abort();
    }
    for (int k = 0; k < d - 1; ++k)
      if (cores_[k].r_right() != cores_[k + 1].r_left())
      {
        std::fprintf(stderr, "tt: rank mismatch at bond %d\n", k + 1);
        std::abort();
      }
  }
  int d() const { return static_cast<int>(cores_.size()); }
  std::vector<int> shape() const
  {
    std::vector<int> s;
    for (auto& c : cores_)
      s.push_back(c.n_phys());
    return s;
  }
  std::vector<int> ranks() const
  {
    std::vector<int> rs;
    if (cores_.empty())
      return {1};
    rs.push_back(cores_.front().r_left());
    for (auto& c : cores_)
      rs.push_back(c.r_right());
    return rs;
  }
  int max_rank() const
  {
    int m = 0;
    for (int r : ranks())
      m = r > m ? r : m;
    return m;
  }
  std::size_t num_params() const
  {
    std::size_t s = 0;
    for (auto& c : cores_)
      s += static_cast<std::size_t>(c.size());
    return s;
  }
  // Dense reconstruction (types/tt.hpp:145-198); small tensors only.
  std::vector<double> to_dense() const
  {
    if (cores_.empty())
      return {1.0};
    std::vector<double> T(cores_[0].data(), cores_[0].data() + cores_[0].size());
    size_t rows = static_cast<size_t>(cores_[0].n_phys());
    size_t cols = static_cast<size_t>(cores_[0].r_right());
    for (size_t k = 1; k < cores_.size(); ++k)
    {
      const tt_core& c = cores_[k];
      const size_t w = static_cast<size_t>(c.n_phys()) * c.r_right();
      std::vector<double> Tn(rows * w, 0.0);
      for (size_t i = 0; i < rows; ++i)
        for (size_t a = 0; a < cols; ++a)
        {
          const double t = T[i * cols + a];
          const double* src = c.data() + a * w;
          for (size_t j = 0; j < w; ++j)
            Tn[i * w + j] += t * src[j];
        }
      T.swap(Tn);
      rows *= static_cast<size_t>(c.n_phys());
      cols = static_cast<size_t>(c.r_right());
    }
    return T;
  }
  tt_core& core(int k) { return cores_.at(static_cast<size_t>(k)); }
  const tt_core& core(int k) const { return cores_.at(static_cast<size_t>(k)); }
  std::vector<tt_core>& cores() { return cores_; }
  const std::vector<tt_core>& cores() const { return cores_; }

 private:
  std::vector<tt_core> cores_;
};

// tt_matrix_core (types/tt_matrix.hpp:37-...): (r_left, m, n, r_right) row-major.
class tt_matrix_core
{
 public:
  tt_matrix_core() = default;
  tt_matrix_core(int r_left, int m_phys, int n_phys, int r_right)
    : r_(r_left), m_(m_phys), n_(n_phys), rp_(r_right)
  {
    if (r_left <= 0 || m_phys <= 0 || n_phys <= 0 || r_right <= 0)
    {
      std::fprintf(stderr, "tt_matrix_core: dimensions must be positive\n");
      std::abort();
    }
    v_.assign(static_cast<size_t>(r_left) * m_phys * n_phys * r_right, 0.0);
  }
  int r_left() const { return r_; }
  int m_phys() const { return m_; }
  int n_phys() const { return n_; }
  int r_right() const { return rp_; }
  std::size_t size() const { return v_.size(); }
  double* data() { return v_.data(); }
  const double* data() const { return v_.data(); }
  double& operator()(int a, int i, int j, int b)
  {
    return v_[((static_cast<size_t>(a) * m_ + i) * n_ + j) * rp_ + b];
  }
  double operator()(int a, int i, int j, int b) const
  {
    return v_[((static_cast<size_t>(a) * m_ + i) * n_ + j) * rp_ + b];
  }
  void zero_clear() { std::fill(v_.begin(), v_.end(), 0.0); }

 private:
  int r_ = 0, m_ = 0, n_ = 0, rp_ = 0;
  std::vector<double> v_;
};

class tt_matrix
{
 public:
  tt_matrix() = default;
  explicit tt_matrix(std::vector<tt_matrix_core> cores) : cores_(std::move(cores))
  {
    const int d = static_cast<int>(cores_.size());
    if (d == 0)
      return;
    if (cores_[0].r_left() != 1 || cores_[d - 1].r_right() != 1)
    {
      std::fprintf(stderr, "tt_matrix: boundary ranks must be 1\n");
      std::abort();
    }
    for (int k = 0; k < d - 1; ++k)
      if (cores_[k].r_right() != cores_[k + 1].r_left())
      {
        std::fprintf(stderr, "tt_matrix: rank mismatch at bond %d\n", k + 1);
        std::abort();
      }
  }
  int d() const { return static_cast<int>(cores_.size()); }
  std::vector<int> row_shape() const
  {
    std::vector<int> s;
    for (auto& c : cores_)
      s.push_back(c.m_phys());
    return s;
  }
  std::vector<int> col_shape() const
  {
    std::vector<int> s;
    for (auto& c : cores_)
      s.push_back(c.n_phys());
    return s;
  }
  std::vector<int> ranks() const
  {
    if (cores_.empty())
      return {1};
    std::vector<int> rs{cores_.front().r_left()};
    for (auto& c : cores_)
      rs.push_back(c.r_right());
    return rs;
  }
  tt_matrix_core& core(int k) { return cores_.at(static_cast<size_t>(k)); }
  const tt_matrix_core& core(int k) const { return cores_.at(static_cast<size_t>(k)); }
  std::vector<tt_matrix_core>& cores() { return cores_; }
  const std::vector<tt_matrix_core>& cores() const { return cores_; }

 private:
  std::vector<tt_matrix_core> cores_;
};

// round_method / round_gauge / round_options / round_result
// (round/round.hpp:33-119).
enum class round_method
{
  svd,
  svd_streaming,
  svd_naive,
  als,
  dmrg
};
enum class round_gauge
{
  none,
  right_canonical
};
struct round_options
{
  double eps = 0.0;
  int max_rank = 0;
  round_method method = round_method::svd;
  round_gauge gauge = round_gauge::none;
  int max_iters = 20;
  double tol = 1.0e-12;
  std::uint64_t seed = 0;
  const tt* warm_start_tt = nullptr;
  const tt_matrix* warm_start_tt_matrix = nullptr;
  // GB300 knobs (not in the reference): arithmetic of the bulk contractions
  // and the device schedule (one CTA per TT, or the whole GPU per TT).
  ttg_precision precision = TTG_PREC_FP64;
  ttg_schedule schedule = TTG_SCHED_AUTO;
};
struct round_result
{
  int iters_run = 0;
  double final_resid = 0.0;
  bool converged = false;
};

namespace detail
{

// Flat C-ABI view of a host tensor; keeps the arrays it points into.
struct flat
{
  std::vector<int32_t> ranks, rows, cols;
  std::vector<int64_t> offsets;
  std::vector<double> data;
  ttg_tensor t{};
  explicit flat(const tt& a)
  {
    const int d = a.d();
    ranks.push_back(d ? a.core(0).r_left() : 1);
    offsets.push_back(0);
    for (int k = 0; k < d; ++k)
    {
      const tt_core& c = a.core(k);
      ranks.push_back(c.r_right());
      rows.push_back(c.n_phys());
      data.insert(data.end(), c.data(), c.data() + c.size());
      offsets.push_back(static_cast<int64_t>(data.size()));
    }
    bind(d, false);
  }
  explicit flat(const tt_matrix& a)
  {
    const int d = a.d();
    ranks.push_back(d ? a.core(0).r_left() : 1);
    offsets.push_back(0);
    for (int k = 0; k < d; ++k)
    {
      const tt_matrix_core& c = a.core(k);
      ranks.push_back(c.r_right());
      rows.push_back(c.m_phys());
      cols.push_back(c.n_phys());
      data.insert(data.end(), c.data(), c.data() + c.size());
      offsets.push_back(static_cast<int64_t>(data.size()));
    }
    bind(d, true);
  }
  void bind(int d, bool matrix)
  {
    if (data.empty())
      data.push_back(0.0);
    if (rows.empty())
      rows.push_back(0);
    t.d = d;
    t.ranks = ranks.data();
    t.rows = rows.data();
    t.cols = matrix ? cols.data() : nullptr;
    t.offsets = offsets.data();
    t.data = data.data();
    t.owned = 0;
  }
};

struct owned
{
  ttg_tensor t{};
  ~owned() { ttg_free(&t); }
};

inline tt to_tt(const ttg_tensor& t)
{
  std::vector<tt_core> cs;
  for (int k = 0; k < t.d; ++k)
  {
    tt_core c(t.ranks[k], t.rows[k], t.ranks[k + 1]);
    std::memcpy(c.data(), t.data + t.offsets[k], sizeof(double) * static_cast<size_t>(c.size()));
    cs.push_back(std::move(c));
  }
  return tt(std::move(cs));
}

inline tt_matrix to_tt_matrix(const ttg_tensor& t)
{
  std::vector<tt_matrix_core> cs;
  for (int k = 0; k < t.d; ++k)
  {
    tt_matrix_core c(t.ranks[k], t.rows[k], t.cols[k], t.ranks[k + 1]);
    std::memcpy(c.data(), t.data + t.offsets[k], sizeof(double) * c.size());
    cs.push_back(std::move(c));
  }
  return tt_matrix(std::move(cs));
}

inline ttg_round_options to_c(const round_options& o)
{
  ttg_round_options c{};
  c.eps = o.eps;
  c.max_rank = o.max_rank;
  c.method = static_cast<int32_t>(o.method);
  c.gauge = static_cast<int32_t>(o.gauge);
  c.precision = o.precision;
  c.schedule = o.schedule;
  return c;
}

// svd_result_default (round/round.hpp:196-203).
inline void fill(const ttg_round_result& r, round_result* info)
{
  if (!info)
    return;
  info->iters_run = r.iters_run;
  info->final_resid = r.final_resid;
  info->converged = r.converged != 0;
}

inline bool iterative(const round_options& o)
{
  return o.method == round_method::als || o.method == round_method::dmrg;
}

// The iterative fields of round_options (round.hpp:84-104) with the warm
// start that matches the call's type (tt or tt_matrix), kept alive here.
struct iter_args
{
  std::unique_ptr<flat> warm;
  ttg_iter_options c{};
  template <class W>
  iter_args(const round_options& o, const W* w)
  {
    if (w)
      warm.reset(new flat(*w));
    c.max_iters = o.max_iters;
    c.tol = o.tol;
    c.seed = o.seed;
    c.warm = warm ? &warm->t : nullptr;
  }
};

}  // namespace detail

// ---- factories (factory/tt_factory.hpp, factory/tt_matrix_factory.hpp) ----
inline tt zeros(const std::vector<int>& shape)
{
  std::vector<tt_core> cs;
  for (int n : shape)
  {
    if (n <= 0)
    {
      std::fprintf(stderr, "zeros: mode size %d is not positive\n", n);
      std::abort();
    }
    cs.emplace_back(1, n, 1);
  }
  return tt(std::move(cs));
}

inline tt ones(const std::vector<int>& shape)
{
  std::vector<int32_t> s(shape.begin(), shape.end());
  detail::owned o;
  detail::check(ttg_host_ones(static_cast<int32_t>(s.size()), s.data(), &o.t), "ones");
  return detail::to_tt(o.t);
}

inline tt random(const std::vector<int>& shape, int max_rank, std::uint64_t seed)
{
  std::vector<int32_t> s(shape.begin(), shape.end());
  detail::owned o;
  detail::check(ttg_host_random(static_cast<int32_t>(s.size()), s.data(), nullptr, max_rank, seed,
                                0, &o.t),
                "random");
  return detail::to_tt(o.t);
}

inline tt_matrix random(const std::vector<int>& row_shape, const std::vector<int>& col_shape,
                        int max_rank, std::uint64_t seed)
{
  std::vector<int32_t> r(row_shape.begin(), row_shape.end()), c(col_shape.begin(), col_shape.end());
  if (r.size() != c.size())
  {
    std::fprintf(stderr, "random: row/col shape length mismatch\n");
    std::abort();
  }
  detail::owned o;
  detail::check(ttg_host_random(static_cast<int32_t>(r.size()), r.data(), c.data(), max_rank,
                                seed, 0, &o.t),
                "random");
  return detail::to_tt_matrix(o.t);
}

// ---- algebra (algebra/tt_ops.hpp:35-143) ----
inline tt axpby(double alpha, const tt& a, double beta, const tt& b)
{
  detail::flat fa(a), fb(b);
  detail::owned o;
  detail::check(ttg_host_axpby(alpha, &fa.t, beta, &fb.t, &o.t), "axpby");
  return detail::to_tt(o.t);
}
inline tt add(const tt& a, const tt& b) { return axpby(1.0, a, 1.0, b); }
inline tt sub(const tt& a, const tt& b) { return axpby(1.0, a, -1.0, b); }
inline tt scale(const tt& a, double alpha)
{
  std::vector<tt_core> cs(a.cores().begin(), a.cores().end());
  if (!cs.empty())
    for (int i = 0; i < cs[0].size(); ++i)
      cs[0].data()[i] *= alpha;
  return tt(std::move(cs));
}

// ---- the hot path -------------------------------------------------------
// round (round/round.hpp:230-312): every method on the GPU (svd; als and
// dmrg through ttg_round_iter with the options' iterative fields).
inline tt round(const tt& a, const round_options& opts, round_result* info = nullptr)
{
  detail::flat in(a);
  detail::owned out;
  ttg_round_options o = detail::to_c(opts);
  ttg_round_result r{};
  if (detail::iterative(opts))
  {
    detail::iter_args it(opts, opts.warm_start_tt);
    detail::check(ttg_round_iter(&in.t, &o, &it.c, &out.t, &r), "round(tt)");
  }
  else
    detail::check(ttg_round(&in.t, &o, &out.t, &r), "round(tt)");
  detail::fill(r, info);
  return detail::to_tt(out.t);
}
inline tt round(tt&& a, const round_options& opts, round_result* info = nullptr)
{
  const tt src(std::move(a));
  return round(src, opts, info);
}

// round(tt_matrix) (round/round.hpp:329-425; pack/unpack tt_matrix_round.hpp:27-72).
inline tt_matrix round(const tt_matrix& a, const round_options& opts, round_result* info = nullptr)
{
  detail::flat in(a);
  detail::owned out;
  ttg_round_options o = detail::to_c(opts);
  ttg_round_result r{};
  if (detail::iterative(opts))
  {
    detail::iter_args it(opts, opts.warm_start_tt_matrix);
    detail::check(ttg_round_iter(&in.t, &o, &it.c, &out.t, &r), "round(tt_matrix)");
  }
  else
    detail::check(ttg_round(&in.t, &o, &out.t, &r), "round(tt_matrix)");
  detail::fill(r, info);
  return detail::to_tt_matrix(out.t);
}
inline tt_matrix round(tt_matrix&& a, const round_options& opts, round_result* info = nullptr)
{
  const tt_matrix src(std::move(a));
  return round(src, opts, info);
}

// matvec_round (round/matvec_round.hpp:42-91).
inline tt matvec_round(const tt_matrix& a, const tt& x, const round_options& opts,
                       round_result* info = nullptr)
{
  detail::flat fa(a), fx(x);
  detail::owned out;
  ttg_round_options o = detail::to_c(opts);
  ttg_round_result r{};
  if (detail::iterative(opts))
  {
    detail::iter_args it(opts, opts.warm_start_tt);
    detail::check(ttg_apply_round_iter(&fa.t, &fx.t, &o, &it.c, &out.t, &r), "matvec_round");
  }
  else
    detail::check(ttg_matvec_round(&fa.t, &fx.t, &o, &out.t, &r), "matvec_round");
  detail::fill(r, info);
  return detail::to_tt(out.t);
}

// matmat_round (round/matmat_round.hpp:41-93).
inline tt_matrix matmat_round(const tt_matrix& a, const tt_matrix& b, const round_options& opts,
                              round_result* info = nullptr)
{
  detail::flat fa(a), fb(b);
  detail::owned out;
  ttg_round_options o = detail::to_c(opts);
  ttg_round_result r{};
  if (detail::iterative(opts))
  {
    detail::iter_args it(opts, opts.warm_start_tt_matrix);
    detail::check(ttg_apply_round_iter(&fa.t, &fb.t, &o, &it.c, &out.t, &r), "matmat_round");
  }
  else
    detail::check(ttg_matmat_round(&fa.t, &fb.t, &o, &out.t, &r), "matmat_round");
  detail::fill(r, info);
  return detail::to_tt_matrix(out.t);
}

// matvec / matmat (apply/tt_matrix_apply.hpp:237-271).
inline tt matvec(const tt_matrix& A, const tt& x)
{
  detail::flat fa(A), fx(x);
  detail::owned out;
  detail::check(ttg_matvec(&fa.t, &fx.t, &out.t), "matvec");
  return detail::to_tt(out.t);
}
inline tt_matrix matmat(const tt_matrix& A, const tt_matrix& B)
{
  detail::flat fa(A), fb(B);
  detail::owned out;
  detail::check(ttg_matmat(&fa.t, &fb.t, &out.t), "matmat");
  return detail::to_tt_matrix(out.t);
}

// eval_batch / eval_at (algebra/tt_eval.hpp:32-112).
inline std::vector<double> eval_batch(const tt& a, const int* idx, int M)
{
  detail::flat fa(a);
  std::vector<double> out(static_cast<size_t>(M > 0 ? M : 0), 0.0);
  detail::check(ttg_eval_batch(&fa.t, reinterpret_cast<const int32_t*>(idx), M, out.data()),
                "eval_batch");
  return out;
}
inline double eval_at(const tt& a, const int* idx)
{
  if (idx == nullptr)
  {
    std::fprintf(stderr, "eval_at: idx pointer is null\n");
    std::abort();
  }
  return eval_batch(a, idx, 1)[0];
}

// inner / norm (algebra/tt_inner.hpp:33-59).
inline double inner(const tt& a, const tt& b)
{
  detail::flat fa(a), fb(b);
  double v = 0.0;
  detail::check(ttg_inner(&fa.t, &fb.t, &v), "inner");
  return v;
}
inline double norm(const tt& a)
{
  detail::flat fa(a);
  double v = 0.0;
  detail::check(ttg_norm(&fa.t, &v), "norm");
  return v;
}

// frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98): ||A x||_F
// and ||A B||_F without a host copy of the product.
inline double frob_norm_apply(const tt_matrix& A, const tt& x)
{
  detail::flat fa(A), fx(x);
  double v = 0.0;
  detail::check(ttg_frob_norm_apply(&fa.t, &fx.t, &v), "frob_norm_apply");
  return v;
}
inline double frob_norm_apply(const tt_matrix& A, const tt_matrix& B)
{
  detail::flat fa(A), fb(B);
  double v = 0.0;
  detail::check(ttg_frob_norm_apply(&fa.t, &fb.t, &v), "frob_norm_apply");
  return v;
}

// soft_threshold (round/tt_soft_threshold.hpp:42-178): singular values of
// every bond shrunk by tau; tau <= 0 or d <= 1 returns a copy.
inline tt soft_threshold(const tt& a, double tau = 0.0)
{
  detail::flat fa(a);
  detail::owned out;
  detail::check(ttg_soft_threshold(&fa.t, tau, &out.t), "soft_threshold");
  return detail::to_tt(out.t);
}

// right_orthogonalize (gauge/tt_orthogonalize.hpp:26-37,
// gauge/tt_matrix_orthogonalize.hpp:34-86), in place.
inline void right_orthogonalize(tt& a)
{
  detail::flat fa(a);
  detail::owned out;
  detail::check(ttg_right_orthogonalize(&fa.t, &out.t), "right_orthogonalize");
  a = detail::to_tt(out.t);
}
inline void right_orthogonalize(tt_matrix& a)
{
  detail::flat fa(a);
  detail::owned out;
  detail::check(ttg_right_orthogonalize(&fa.t, &out.t), "right_orthogonalize");
  a = detail::to_tt_matrix(out.t);
}

}  // namespace tensor_train
}  // namespace mva
