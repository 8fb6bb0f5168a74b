// Host-side input construction of libttgpu.so (no device work).
//
// The reference builds the hot path's inputs with its factories and TT
// algebra; these entry points restate them so a caller of this library can
// build the same seeded inputs without the reference:
//   random(shape, max_rank, seed)         factory/tt_factory.hpp:141-207
//   random(rows, cols, max_rank, seed)    factory/tt_matrix_factory.hpp:133-191
//   ones / zeros                          factory/tt_factory.hpp:32-78
//   axpby / add / sub                     algebra/tt_ops.hpp:72-143,
//                                         detail/block_concat.hpp:40-156
// The generator is one std::mt19937_64(seed) stream drawn through
// std::normal_distribution<double>, core by core in row-major order, after
// the forward/backward rank-feasibility passes -- so a build with the same
// standard library produces bit-identical inputs.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <vector>

#include "../../include/ttg.h"

namespace
{

thread_local std::string g_host_err;

int32_t host_fail(int32_t st, const char* msg)
{
  g_host_err = msg;
  return st;
}

int32_t emit(int d, const std::vector<int>& ranks, const std::vector<int>& rows,
             const std::vector<int>* cols, std::vector<double>&& data, ttg_tensor* out)
{
  std::memset(out, 0, sizeof(*out));
  out->d = d;
  out->owned = 1;
  out->ranks = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (d + 1)));
  out->rows = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (d > 0 ? d : 1)));
  out->offsets = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (d + 1)));
  if (cols)
    out->cols = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (d > 0 ? d : 1)));
  out->data = static_cast<double*>(std::malloc(sizeof(double) * (data.empty() ? 1 : data.size())));
  if (!out->ranks || !out->rows || !out->offsets || !out->data || (cols && !out->cols))
    return host_fail(TTG_ERR_OOM, "host allocation failed");
  int64_t off = 0;
  for (int k = 0; k <= d; ++k)
    out->ranks[k] = ranks[k];
  for (int k = 0; k < d; ++k)
  {
    out->rows[k] = rows[k];
    if (cols)
      out->cols[k] = (*cols)[k];
    out->offsets[k] = off;
    off += static_cast<int64_t>(ranks[k]) * rows[k] * (cols ? (*cols)[k] : 1) * ranks[k + 1];
  }
  out->offsets[d] = off;
  if (!data.empty())
    std::memcpy(out->data, data.data(), sizeof(double) * data.size());
  return TTG_OK;
}

// Forward then backward feasibility clipping (tt_factory.hpp:156-189).
bool feasible(const std::vector<long long>& mode, int max_rank, std::vector<int>& ranks)
{
  const int d = static_cast<int>(mode.size());
  ranks.assign(static_cast<size_t>(d + 1), 1);
  for (int k = 0; k < d; ++k)
  {
    long long cap = static_cast<long long>(ranks[k]) * mode[k];
    if (cap > max_rank && max_rank > 0)
      cap = max_rank;
    if (cap > std::numeric_limits<int>::max())
      return false;
    ranks[k + 1] = static_cast<int>(cap);
  }
  for (int k = d - 1; k >= 0; --k)
  {
    long long cap = static_cast<long long>(ranks[k + 1]) * mode[k];
    if (cap > max_rank && max_rank > 0)
      cap = max_rank;
    if (cap > std::numeric_limits<int>::max())
      return false;
    if (cap < ranks[k])
      ranks[k] = static_cast<int>(cap);
  }
  ranks[0] = 1;
  ranks[d] = 1;
  return true;
}

}  // namespace

extern "C" {

int32_t ttg_host_random(int32_t d, const int32_t* rows, const int32_t* cols, int32_t max_rank,
                        uint64_t seed, int32_t fan_in_scale, ttg_tensor* out)
{
  if (!out || d < 0 || (d > 0 && !rows))
    return host_fail(TTG_ERR_ARG, "random: bad arguments");
  std::vector<long long> mode;
  std::vector<int> rv, cv;
  for (int k = 0; k < d; ++k)
  {
    const int m = rows[k], n = cols ? cols[k] : 1;
    if (m <= 0 || n <= 0)
      return host_fail(TTG_ERR_SHAPE, "random: mode size is not positive");
    mode.push_back(static_cast<long long>(m) * n);
    rv.push_back(m);
    cv.push_back(n);
  }
  std::vector<int> ranks;
  if (!feasible(mode, max_rank, ranks))
    return host_fail(TTG_ERR_SHAPE, "random: rank cap exceeds INT_MAX; provide a finite max_rank");
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::vector<double> data;
  for (int k = 0; k < d; ++k)
  {
    const int64_t sz = static_cast<int64_t>(ranks[k]) * mode[k] * ranks[k + 1];
    const double s = fan_in_scale ? 1.0 / std::sqrt(static_cast<double>(ranks[k]) * mode[k]) : 1.0;
    for (int64_t i = 0; i < sz; ++i)
      data.push_back(fan_in_scale ? nd(rng) * s : nd(rng));
  }
  return emit(d, ranks, rv, cols ? &cv : nullptr, std::move(data), out);
}

int32_t ttg_host_random_uneven(uint64_t seed, int32_t dmin, int32_t dmax, int32_t rmin,
                               int32_t rmax, ttg_tensor* out)
{
  if (!out || dmin < 1 || dmax < dmin || rmin < 1 || rmax < rmin)
    return host_fail(TTG_ERR_ARG, "random_uneven: bad arguments");
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
    ranks[k + 1] = static_cast<int>(
      std::min<long long>(ranks[k + 1], static_cast<long long>(ranks[k]) * shape[k]));
  ranks[d] = 1;
  for (int k = d - 1; k >= 0; --k)
    ranks[k] = static_cast<int>(
      std::min<long long>(ranks[k], static_cast<long long>(ranks[k + 1]) * shape[k]));
  ranks[0] = 1;
  std::normal_distribution<double> nd(0.0, 1.0);
  std::vector<double> data;
  for (int k = 0; k < d; ++k)
  {
    const int64_t sz = static_cast<int64_t>(ranks[k]) * shape[k] * ranks[k + 1];
    const double s = 1.0 / std::sqrt(static_cast<double>(ranks[k]) * shape[k]);
    const size_t base = data.size();
    for (int64_t i = 0; i < sz; ++i)
      data.push_back(nd(rng));
    for (int64_t i = 0; i < sz; ++i)
      data[base + i] *= s;
  }
  return emit(d, ranks, shape, nullptr, std::move(data), out);
}

int32_t ttg_host_ones(int32_t d, const int32_t* shape, ttg_tensor* out)
{
  if (!out || d < 0 || (d > 0 && !shape))
    return host_fail(TTG_ERR_ARG, "ones: bad arguments");
  std::vector<int> ranks(static_cast<size_t>(d + 1), 1), rv;
  std::vector<double> data;
  for (int k = 0; k < d; ++k)
  {
    if (shape[k] <= 0)
      return host_fail(TTG_ERR_SHAPE, "ones: mode size is not positive");
    rv.push_back(shape[k]);
    for (int i = 0; i < shape[k]; ++i)
      data.push_back(1.0);
  }
  return emit(d, ranks, rv, nullptr, std::move(data), out);
}

// alpha*a + beta*b with block-diagonal core concatenation; the scalars are
// folded into core 0 (algebra/tt_ops.hpp:72-117, block_concat.hpp:40-156).
int32_t ttg_host_axpby(double alpha, const ttg_tensor* a, double beta, const ttg_tensor* b,
                       ttg_tensor* out)
{
  if (!a || !b || !out)
    return host_fail(TTG_ERR_ARG, "axpby: null argument");
  if (a->d != b->d)
    return host_fail(TTG_ERR_SHAPE, "tt::axpby: rank-d mismatch");
  const int d = a->d;
  std::vector<int> rows, cols, ranks(static_cast<size_t>(d + 1), 1);
  const bool matrix = a->cols != nullptr;
  auto mode = [&](const ttg_tensor* t, int k) { return t->rows[k] * (t->cols ? t->cols[k] : 1); };
  for (int k = 0; k < d; ++k)
  {
    if (mode(a, k) != mode(b, k))
      return host_fail(TTG_ERR_SHAPE, "tt::axpby: mode-size mismatch");
    rows.push_back(a->rows[k]);
    if (matrix)
      cols.push_back(a->cols[k]);
  }
  std::vector<double> data;
  if (d == 1)
  {
    const int n = mode(a, 0);
    for (int i = 0; i < n; ++i)
      data.push_back(alpha * a->data[a->offsets[0] + i] + beta * b->data[b->offsets[0] + i]);
    return emit(d, ranks, rows, matrix ? &cols : nullptr, std::move(data), out);
  }
  for (int k = 1; k < d; ++k)
    ranks[k] = a->ranks[k] + b->ranks[k];
  for (int k = 0; k < d; ++k)
  {
    const int n = mode(a, k);
    const int raL = a->ranks[k], raR = a->ranks[k + 1], rbL = b->ranks[k], rbR = b->ranks[k + 1];
    const bool head = k == 0, tail = k == d - 1;
    const int rL = ranks[k], rR = ranks[k + 1];
    const size_t base = data.size();
    data.resize(base + static_cast<size_t>(rL) * n * rR, 0.0);
    const double al = head ? alpha : 1.0, be = head ? beta : 1.0;
    const double* pa = a->data + a->offsets[k];
    const double* pb = b->data + b->offsets[k];
    for (int x = 0; x < raL; ++x)
      for (int i = 0; i < n; ++i)
        for (int y = 0; y < raR; ++y)
          data[base + (static_cast<size_t>(x) * n + i) * rR + y] =
            al == 1.0 ? pa[(x * n + i) * raR + y] : al * pa[(x * n + i) * raR + y];
    const int boff = head ? 0 : raL, coff = tail ? 0 : raR;
    for (int x = 0; x < rbL; ++x)
      for (int i = 0; i < n; ++i)
        for (int y = 0; y < rbR; ++y)
          data[base + (static_cast<size_t>(boff + x) * n + i) * rR + coff + y] =
            be == 1.0 ? pb[(x * n + i) * rbR + y] : be * pb[(x * n + i) * rbR + y];
  }
  return emit(d, ranks, rows, matrix ? &cols : nullptr, std::move(data), out);
}

const char* ttg_host_last_error(void) { return g_host_err.c_str(); }

}  // extern "C"
