// C entry points of the CPU oracle (ctypes-callable) -- TEST INFRASTRUCTURE.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library.  Errors never abort: functions return NULL / a negative code
// and ttor_last_error() holds the message (the reference would abort).
#include <atomic>
#include <chrono>
#include <thread>

#include "tt_oracle.hpp"

using namespace ttor;

namespace
{
thread_local std::string g_err;

template <class F>
auto guard(F&& f) -> decltype(f())
{
  try
  {
    g_err.clear();
    return f();
  }
  catch (const std::exception& e)
  {
    g_err = e.what();
    return decltype(f())();
  }
}

std::vector<int> vec(const int* p, int n)
{
  return std::vector<int>(p, p + n);
}
}  // namespace

struct ttor_tt
{
  TT t;
};

extern "C" {

const char* ttor_last_error() { return g_err.c_str(); }

// Build from flat arrays.  `cols` == NULL for a TT; for a TT-matrix `rows`
// holds m_k and `cols` n_k, and core k is (r_k, m_k*n_k, r_{k+1}).
ttor_tt* ttor_make(int d, const int* ranks, const int* rows, const int* cols,
                   const double* data)
{
  return guard([&]() -> ttor_tt* {
    auto* h = new ttor_tt;
    size_t off = 0;
    h->t.matrix = (cols != nullptr);
    for (int k = 0; k < d; ++k)
    {
      const int mode = cols ? rows[k] * cols[k] : rows[k];
      Core c(ranks[k], mode, ranks[k + 1]);
      std::memcpy(c.v.data(), data + off, sizeof(double) * c.size());
      off += c.size();
      h->t.c.push_back(std::move(c));
      if (cols)
      {
        h->t.mrow.push_back(rows[k]);
        h->t.ncol.push_back(cols[k]);
      }
    }
    try
    {
      h->t.validate();
    }
    catch (...)
    {
      delete h;
      throw;
    }
    return h;
  });
}

void ttor_free(ttor_tt* h) { delete h; }
int ttor_d(const ttor_tt* h) { return h->t.d(); }
int ttor_is_matrix(const ttor_tt* h) { return h->t.matrix ? 1 : 0; }

void ttor_ranks(const ttor_tt* h, int* out)
{
  auto r = h->t.ranks();
  for (size_t i = 0; i < r.size(); ++i)
    out[i] = r[i];
}

// Mode of core k as stored (n_k, or m_k*n_k for a matrix).
void ttor_modes(const ttor_tt* h, int* out)
{
  for (int k = 0; k < h->t.d(); ++k)
    out[k] = h->t.c[k].n;
}

void ttor_matrix_modes(const ttor_tt* h, int* rows, int* cols)
{
  for (int k = 0; k < h->t.d(); ++k)
  {
    rows[k] = h->t.matrix ? h->t.mrow[k] : h->t.c[k].n;
    cols[k] = h->t.matrix ? h->t.ncol[k] : 1;
  }
}

long long ttor_numel(const ttor_tt* h)
{
  long long s = 0;
  for (auto& c : h->t.c)
    s += static_cast<long long>(c.size());
  return s;
}

void ttor_data(const ttor_tt* h, double* out)
{
  size_t off = 0;
  for (auto& c : h->t.c)
  {
    std::memcpy(out + off, c.v.data(), sizeof(double) * c.size());
    off += c.size();
  }
}

ttor_tt* ttor_random(int d, const int* shape, int max_rank, unsigned long long seed)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{random(vec(shape, d), max_rank, seed)}; });
}

ttor_tt* ttor_random_matrix(int d, const int* rows, const int* cols, int max_rank,
                            unsigned long long seed)
{
  return guard([&]() -> ttor_tt* {
    return new ttor_tt{random_matrix(vec(rows, d), vec(cols, d), max_rank, seed)};
  });
}

ttor_tt* ttor_random_uneven(unsigned long long seed, int dmin, int dmax, int rmin, int rmax)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{random_uneven(seed, dmin, dmax, rmin, rmax)}; });
}

ttor_tt* ttor_ones(int d, const int* shape)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{ones(vec(shape, d))}; });
}

ttor_tt* ttor_zeros(int d, const int* shape)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{zeros(vec(shape, d))}; });
}

void ttor_scale_by_fan_in(ttor_tt* h) { scale_by_fan_in(h->t); }

ttor_tt* ttor_axpby(double alpha, const ttor_tt* a, double beta, const ttor_tt* b)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{axpby(alpha, a->t, beta, b->t)}; });
}

// gauge: 0 = none (round), 1 = right_canonical.
ttor_tt* ttor_round(const ttor_tt* a, double eps, int max_rank, int gauge)
{
  return guard([&]() -> ttor_tt* {
    if (a->t.matrix)
      return new ttor_tt{round_matrix(a->t, eps, max_rank, gauge == 1)};
    return new ttor_tt{gauge == 1 ? round_right_canonical(a->t, eps, max_rank)
                                  : round(a->t, eps, max_rank)};
  });
}

ttor_tt* ttor_right_orthogonalize(const ttor_tt* a)
{
  return guard([&]() -> ttor_tt* {
    TT t = a->t;
    right_orthogonalize(t);
    return new ttor_tt{std::move(t)};
  });
}

ttor_tt* ttor_left_orthogonalize(const ttor_tt* a)
{
  return guard([&]() -> ttor_tt* {
    TT t = a->t;
    left_orthogonalize(t);
    return new ttor_tt{std::move(t)};
  });
}

ttor_tt* ttor_matvec(const ttor_tt* A, const ttor_tt* x)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{matvec(A->t, x->t)}; });
}

ttor_tt* ttor_matmat(const ttor_tt* A, const ttor_tt* B)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{matmat(A->t, B->t)}; });
}

// streaming: 0 = svd (naive), 1 = svd_streaming.
ttor_tt* ttor_matvec_round(const ttor_tt* A, const ttor_tt* x, double eps, int max_rank,
                           int streaming)
{
  return guard([&]() -> ttor_tt* {
    return new ttor_tt{matvec_round(A->t, x->t, eps, max_rank, streaming != 0)};
  });
}

// naive: 0 = svd (streaming), 1 = svd_naive.
ttor_tt* ttor_matmat_round(const ttor_tt* A, const ttor_tt* B, double eps, int max_rank,
                           int naive)
{
  return guard([&]() -> ttor_tt* {
    return new ttor_tt{matmat_round(A->t, B->t, eps, max_rank, naive != 0)};
  });
}

int ttor_eval_batch(const ttor_tt* a, const int* idx, int M, double* out)
{
  return guard([&]() -> int {
    auto v = eval_batch(a->t, idx, M);
    std::memcpy(out, v.data(), sizeof(double) * v.size());
    return 1;
  }) ? 0 : -1;
}

int ttor_inner(const ttor_tt* a, const ttor_tt* b, double* out)
{
  return guard([&]() -> int {
    *out = inner(a->t, b->t);
    return 1;
  }) ? 0 : -1;
}

int ttor_norm(const ttor_tt* a, double* out)
{
  return guard([&]() -> int {
    *out = norm(a->t);
    return 1;
  }) ? 0 : -1;
}

// Core-level products for the fused-apply known-answer test
// (tests/core/test_tt_fused_apply_core.cpp): A (a, m, p, b), X (sx, p*nout,
// bx); fused = 1 forms F (alpha x a*sx) x A x X through fused_apply_core,
// fused = 0 forms matvec_core (nout = 1) or matmat_core.  out holds
// alpha*m*nout*b*bx doubles (alpha = a*sx when not fused).
int ttor_apply_core(int fused, const double* F, int alpha, int a, int m, int p, int b,
                    const double* A, int sx, int nout, int bx, const double* X, double* out)
{
  return guard([&]() -> int {
    Core Ac(a, m * p, b), Xc(sx, p * nout, bx);
    std::memcpy(Ac.v.data(), A, sizeof(double) * Ac.size());
    std::memcpy(Xc.v.data(), X, sizeof(double) * Xc.size());
    Core y;
    if (fused)
    {
      Mat Fm(alpha, static_cast<int64_t>(a) * sx);
      std::memcpy(Fm.data(), F, sizeof(double) * Fm.v.size());
      y = fused_apply_core(Fm, Ac, m, p, Xc, nout);
    }
    else
      y = nout == 1 ? matvec_core(Ac, m, p, Xc) : matmat_core(Ac, m, p, Xc, nout);
    std::memcpy(out, y.v.data(), sizeof(double) * y.size());
    return 1;
  }) ? 0 : -1;
}

// Iterative rounding: method 3 = ALS, 4 = DMRG (round/round.hpp:237-250).
// warm may be NULL; cold_random = 1 starts from random(shape, max_rank,
// seed) as the apply variants do.  info = {iters_run, converged} and change.
ttor_tt* ttor_round_iter(const ttor_tt* a, int method, double eps, int max_rank, int max_iters,
                         double tol, unsigned long long seed, const ttor_tt* warm,
                         int cold_random, int* info, double* change)
{
  return guard([&]() -> ttor_tt* {
    IterOptions o;
    o.eps = eps;
    o.max_rank = max_rank;
    o.max_iters = max_iters;
    o.tol = tol;
    o.seed = seed;
    o.warm = warm ? &warm->t : nullptr;
    IterResult r;
    TT y = method == 4 ? dmrg_round(a->t, o, &r, cold_random != 0)
                       : als_round(a->t, o, &r, cold_random != 0);
    info[0] = r.iters_run;
    info[1] = r.converged ? 1 : 0;
    *change = r.final_change;
    return new ttor_tt{std::move(y)};
  });
}

int ttor_frob_norm_apply(const ttor_tt* A, const ttor_tt* x, double* out)
{
  return guard([&]() -> int {
    *out = frob_norm_apply(A->t, x->t);
    return 1;
  }) ? 0 : -1;
}

ttor_tt* ttor_soft_threshold(const ttor_tt* a, double tau)
{
  return guard([&]() -> ttor_tt* { return new ttor_tt{soft_threshold(a->t, tau)}; });
}

double ttor_norm_qr(const ttor_tt* a) { return norm_qr(a->t); }

double ttor_rel_err(const ttor_tt* y, const ttor_tt* yref)
{
  return guard([&]() -> double { return rel_err(y->t, yref->t); });
}

// Dense size when out == NULL; otherwise writes the dense tensor.
long long ttor_to_dense(const ttor_tt* a, double* out)
{
  long long n = 1;
  for (auto& c : a->t.c)
    n *= c.n;
  if (out)
  {
    auto v = to_dense(a->t);
    std::memcpy(out, v.data(), sizeof(double) * v.size());
  }
  return n;
}

// Per-step trace of the calling thread (shapes and chosen ranks).
void ttor_trace(int on)
{
  trace().on = (on != 0);
  trace().lines.clear();
}

int ttor_trace_count() { return static_cast<int>(trace().lines.size()); }

const char* ttor_trace_line(int i) { return trace().lines.at(static_cast<size_t>(i)).c_str(); }

// Dense kernels, exposed for cross-checks against LAPACK (numpy).
// Q: rows x k, R: k x cols, U: rows x k, s: k, Vt: k x cols, k = min(rows, cols).
int ttor_qr_thin(const double* M, int rows, int cols, double* Q, double* R)
{
  return guard([&]() -> int {
    Mat q, r;
    qr_thin(M, rows, cols, q, r);
    std::memcpy(Q, q.data(), sizeof(double) * q.v.size());
    std::memcpy(R, r.data(), sizeof(double) * r.v.size());
    return 1;
  }) ? 0 : -1;
}

int ttor_svd_thin(const double* M, int rows, int cols, double* U, double* sv, double* Vt)
{
  return guard([&]() -> int {
    Mat u, vt;
    std::vector<double> s;
    svd_thin(M, rows, cols, u, s, vt);
    std::memcpy(U, u.data(), sizeof(double) * u.v.size());
    std::memcpy(sv, s.data(), sizeof(double) * s.size());
    std::memcpy(Vt, vt.data(), sizeof(double) * vt.v.size());
    return 1;
  }) ? 0 : -1;
}

int ttor_truncate_eps_rank(const double* s, int n, double delta, int max_rank)
{
  return truncate_eps_rank(std::vector<double>(s, s + n), delta, max_rank);
}

// CPU baseline: round `count` TTs (oracle, plain FP64) on `threads` host
// threads, each thread taking TTs from a shared counter.  Returns the wall
// time in seconds.  `outs` may be NULL.
double ttor_round_many(int count, ttor_tt* const* tts, double eps, int max_rank, int threads,
                       ttor_tt** outs)
{
  std::atomic<int> next{0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&]() {
    for (;;)
    {
      const int i = next.fetch_add(1);
      if (i >= count)
        break;
      TT r = round(tts[i]->t, eps, max_rank);
      if (outs)
        outs[i] = new ttor_tt{std::move(r)};
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t)
    pool.emplace_back(work);
  work();
  for (auto& th : pool)
    th.join();
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// CPU baseline for apply-round: `reps` independent matvec_round calls on
// `threads` threads.  Returns wall seconds.
double ttor_matvec_round_many(const ttor_tt* A, const ttor_tt* x, double eps, int max_rank,
                              int streaming, int reps, int threads)
{
  std::atomic<int> next{0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&]() {
    for (;;)
    {
      if (next.fetch_add(1) >= reps)
        break;
      TT r = matvec_round(A->t, x->t, eps, max_rank, streaming != 0);
      (void)r;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t)
    pool.emplace_back(work);
  work();
  for (auto& th : pool)
    th.join();
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // extern "C"
