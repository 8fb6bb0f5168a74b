// Reference-style test (printf FAIL/OK, exit code = failures) written against
// the reference's own C++ interface, served here by tensor_train_gb300.hpp.
// Mirrors tests/core/test_tt_invariants.cpp, test_tt_matrix_apply_round.cpp
// and test_tt_eval.cpp of the reference.
#include <cmath>
#include <cstdio>
#include <vector>

#include "tensor_train_gb300.hpp"

namespace tt = mva::tensor_train;

static int failed = 0;
#define CHECK(cond, msg)                 \
  do                                     \
  {                                      \
    if (!(cond))                         \
    {                                    \
      std::printf("FAIL: %s\n", msg);    \
      ++failed;                          \
    }                                    \
  } while (0)

static double frob(const std::vector<double>& a)
{
  double s = 0;
  for (double x : a)
    s += x * x;
  return std::sqrt(s);
}
static double frob_diff(const std::vector<double>& a, const std::vector<double>& b)
{
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i)
    s += (a[i] - b[i]) * (a[i] - b[i]);
  return std::sqrt(s);
}

int main()
{
  tt::round_options o;
  o.eps = 1.0e-10;
  {
    auto a = tt::random({2, 3, 4}, 4, 0), b = tt::random({2, 3, 4}, 4, 1);
    auto s = tt::round(tt::add(a, b), o);
    auto da = a.to_dense(), db = b.to_dense(), ds = s.to_dense();
    double md = 0;
    for (size_t i = 0; i < da.size(); ++i)
      md = std::fmax(md, std::fabs(ds[i] - da[i] - db[i]));
    CHECK(md < 1.0e-13, "round(add(a,b)) == a+b dense");
  }
  {
    auto z = tt::zeros({3, 4, 2});
    auto r = tt::round(z, o);
    CHECK(tt::norm(r) < 1e-300, "round(zeros): norm still 0");
    CHECK(r.ranks()[1] == 1, "round(zeros): bond ranks = 1");
  }
  {
    auto a = tt::random({2, 3, 4, 2}, 8, 99);
    tt::round_options e;
    e.eps = 0.01;
    auto ar = tt::round(a, e);
    CHECK(tt::norm(tt::sub(a, ar)) <= 0.01 * tt::norm(a) * 1.01, "round error bound");
  }
  {
    // ALS and DMRG through round_options (test_tt_round.cpp's iterative
    // cases): a rank-8 sum rounded back to its exact rank.
    auto a = tt::random({3, 4, 3, 4}, 4, 5), b = tt::random({3, 4, 3, 4}, 4, 6);
    auto s = tt::add(a, b);
    const int rmax = 8;
    for (tt::round_method m : {tt::round_method::als, tt::round_method::dmrg})
    {
      tt::round_options it;
      it.method = m;
      it.eps = m == tt::round_method::dmrg ? 1e-12 : 0.0;
      it.max_rank = rmax;
      it.max_iters = 3;
      tt::round_result info;
      auto y = tt::round(s, it, &info);
      CHECK(frob_diff(y.to_dense(), s.to_dense()) <= 1e-10 * frob(s.to_dense()),
            "als/dmrg round keeps the tensor");
      CHECK(info.iters_run >= 1 && info.iters_run <= 3, "als/dmrg iters_run");
      it.warm_start_tt = &y;
      auto y2 = tt::round(s, it, &info);
      CHECK(frob_diff(y2.to_dense(), s.to_dense()) <= 1e-10 * frob(s.to_dense()),
            "als/dmrg warm start");
    }
  }
  {
    auto A = tt::random(std::vector<int>{2, 3, 2, 3}, std::vector<int>{3, 2, 3, 2}, 3, 0xAA11ULL);
    auto x = tt::random({3, 2, 3, 2}, 3, 0xBB22ULL);
    tt::round_options s = o;
    s.method = tt::round_method::svd_streaming;
    tt::round_result info;
    auto ys = tt::matvec_round(A, x, s, &info);
    auto yn = tt::matvec_round(A, x, o);
    auto ym = tt::matvec(A, x);
    CHECK(info.iters_run == 1 && info.converged, "svd result defaults");
    CHECK(frob_diff(yn.to_dense(), ym.to_dense()) <= 1e-9 * frob(ym.to_dense()),
          "matvec_round vs matvec");
    CHECK(frob_diff(ys.to_dense(), yn.to_dense()) <= 10 * 1e-10 * frob(yn.to_dense()),
          "streaming vs naive");
  }
  {
    auto A = tt::random(std::vector<int>{2, 3, 2}, std::vector<int>{3, 2, 3}, 2, 0xC3ULL);
    auto B = tt::random(std::vector<int>{3, 2, 3}, std::vector<int>{2, 3, 2}, 2, 0xD4ULL);
    auto C = tt::matmat_round(A, B, o);
    auto F = tt::matmat(A, B);
    CHECK(C.ranks().size() == F.ranks().size(), "matmat_round order");
    auto Cr = tt::round(F, o);
    CHECK(Cr.d() == 3 && Cr.core(0).m_phys() == 2 && Cr.core(0).n_phys() == 2,
          "round(tt_matrix) keeps modes");
  }
  {
    auto a = tt::random({4, 5, 6, 4}, 6, 13);
    auto D = a.to_dense();
    std::vector<int> idx;
    std::vector<double> ref;
    for (int i = 0; i < 32; ++i)
    {
      int i0 = i % 4, i1 = (i * 7) % 5, i2 = (i * 11) % 6, i3 = (i * 3) % 4;
      idx.insert(idx.end(), {i0, i1, i2, i3});
      ref.push_back(D[((i0 * 5 + i1) * 6 + i2) * 4 + i3]);
    }
    auto v = tt::eval_batch(a, idx.data(), 32);
    double md = 0;
    for (int j = 0; j < 32; ++j)
      md = std::fmax(md, std::fabs(v[j] - ref[j]));
    CHECK(md < 1.0e-10, "eval_batch vs dense");
    CHECK(std::fabs(tt::inner(a, a) - frob(D) * frob(D)) <= 1e-12 * frob(D) * frob(D),
          "inner vs dense");
  }
  {
    // tests/core/test_tt_soft_threshold.cpp: tau = 0 is a copy, the norm
    // does not grow, cores 1..d-1 come out right-orthogonal
    auto a = tt::random({3, 4, 5}, 8, 7);
    auto s0 = tt::soft_threshold(a, 0.0);
    CHECK(frob_diff(s0.to_dense(), a.to_dense()) < 1e-14, "soft_threshold(a, 0) == a");
    auto s = tt::soft_threshold(a, 0.5);
    CHECK(tt::norm(s) <= tt::norm(a) * (1.0 + 1e-14), "soft_threshold: norm non-increasing");
    // tests/core/test_tt_matrix_frob_norm_apply.cpp
    auto A = tt::random(std::vector<int>{2, 3, 2}, std::vector<int>{3, 2, 3}, 3, 0xA10001ULL);
    auto x = tt::random({3, 2, 3}, 2, 0x55AA77ULL);
    const double ref = tt::norm(tt::matvec(A, x));
    CHECK(std::fabs(tt::frob_norm_apply(A, x) - ref) <= 1e-13 * ref, "frob_norm_apply(A, x)");
  }
  if (failed == 0)
    std::printf("test_header_round: OK\n");
  return failed;
}
