// Multi-device batch entries (host code only): one batch of independent TTs
// partitioned across devices by estimated rounding cost, and eval_batch with
// the multi-indices split across devices.
//
// The reference rounds TTs one after another on one core; nothing in it is
// parallel (round/tt_round.hpp:60-63 is a strictly sequential sweep, and
// algebra/tt_eval.hpp:86-112 a loop over samples).  Across TTs and across
// samples there is no exchange step, so the split needs no collective: each
// device runs the single-device entry point on its part from its own host
// thread, and the results land in the caller's host arrays in input order.
//
// Cost model: the algorithmic FLOP count F_round of one TT with its input
// ranks as the output ranks (an upper bound: rounding only lowers ranks),
// the same model as tensor_train_gb300/flops.py.  Partition: longest
// processing time first -- TTs in decreasing cost (ties by index) each go to
// the part with the least cost so far (ties to the lowest part).  The result
// depends only on the shapes and the part count, so every process that
// computes it gets the same partition.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_kernels.h"

namespace ttg
{
namespace
{

double qr_f(double m, double c) { return 4.0 * m * c * c - (4.0 / 3.0) * c * c * c; }
double gemm_f(double m, double k, double n) { return 2.0 * m * k * n; }
double svd_f(double m, double c)
{
  if (m < c)
    std::swap(m, c);
  return 4.0 * m * m * c + 8.0 * m * c * c + 9.0 * c * c * c;
}

// F_round of one TT or TT-matrix (mode m_k n_k) with output ranks = input
// ranks after the R->L sweep's r_eff shrink.
double round_cost(const ttg_tensor& t)
{
  const int d = t.d;
  if (d <= 1 || !t.ranks || !t.rows)
    return 0.0;
  std::vector<double> r(t.ranks, t.ranks + d + 1), n(d);
  for (int k = 0; k < d; ++k)
    n[k] = static_cast<double>(t.rows[k]) * (t.cols ? t.cols[k] : 1);
  double F = 0.0;
  for (int k = d - 1; k >= 1; --k)
  {
    const double m = n[k] * r[k + 1], c = r[k], e = std::min(m, c);
    F += qr_f(std::max(m, c), std::min(m, c)) + gemm_f(r[k - 1] * n[k - 1], c, e);
    r[k] = e;
  }
  F += 2.0 * r[0] * n[0] * r[1];
  for (int k = 0; k + 1 < d; ++k)
  {
    const double rows = r[k] * n[k], cols = r[k + 1];
    const double w = n[k + 1] * r[k + 2];
    if (rows >= 2.0 * cols)
      F += qr_f(rows, cols) + 21.0 * cols * cols * cols + gemm_f(rows, cols, cols);
    else
      F += svd_f(rows, cols);
    F += gemm_f(cols, cols, w);
  }
  for (int k = 0; k < d; ++k)
    F += 4.0 * r[k] * n[k] * r[k + 1];
  return F;
}

int32_t sfail(int32_t st, const std::string& msg)
{
  set_last_error(msg);
  return st;
}

std::vector<int32_t> partition(int32_t count, const ttg_tensor* ins, int32_t parts)
{
  std::vector<double> cost(static_cast<size_t>(count));
  for (int32_t i = 0; i < count; ++i)
    cost[i] = round_cost(ins[i]);
  std::vector<int32_t> order(static_cast<size_t>(count));
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
  std::vector<double> load(static_cast<size_t>(parts), 0.0);
  std::vector<int32_t> part_of(static_cast<size_t>(count), 0);
  for (int32_t i : order)
  {
    int32_t best = 0;
    for (int32_t p = 1; p < parts; ++p)
      if (load[p] < load[best])
        best = p;
    part_of[i] = best;
    load[best] += cost[i];
  }
  return part_of;
}

}  // namespace
}  // namespace ttg

extern "C" {

int32_t ttg_shard_plan(int32_t count, const ttg_tensor* ins, int32_t parts, int32_t* part_of,
                       double* cost)
{
  using namespace ttg;
  set_last_error(std::string());
  if (count < 0 || parts < 1 || (count > 0 && (!ins || !part_of)))
    return sfail(TTG_ERR_ARG, "shard_plan: bad arguments");
  for (int32_t i = 0; i < count; ++i)
    if (ins[i].d < 0 || (ins[i].d > 0 && (!ins[i].ranks || !ins[i].rows)))
      return sfail(TTG_ERR_ARG, "shard_plan: tensor " + std::to_string(i) + " has no shape");
  const std::vector<int32_t> p = partition(count, ins, parts);
  std::copy(p.begin(), p.end(), part_of);
  if (cost)
    for (int32_t i = 0; i < count; ++i)
      cost[i] = round_cost(ins[i]);
  return TTG_OK;
}

int32_t ttg_round_batch_devices(int32_t count, const ttg_tensor* ins,
                                const ttg_round_options* opts, ttg_tensor* outs,
                                ttg_round_result* results, int32_t n_dev, const int32_t* devices)
{
  using namespace ttg;
  set_last_error(std::string());
  if (count < 0 || n_dev < 1 || !devices || !opts || (count > 0 && (!ins || !outs)))
    return sfail(TTG_ERR_ARG, "round_batch_devices: bad arguments");
  if (opts->bond_stats)
    return sfail(TTG_ERR_ARG, "round_batch_devices: bond_stats is served by ttg_round_batch only");
  for (int32_t i = 0; i < count; ++i)
  {
    std::memset(&outs[i], 0, sizeof(outs[i]));
    if (ins[i].d < 0 || (ins[i].d > 0 && (!ins[i].ranks || !ins[i].rows)))
      return sfail(TTG_ERR_SHAPE, "round_batch_devices: tensor " + std::to_string(i) +
                                      " has no shape");
  }
  int ndev_avail = 0;
  if (cudaGetDeviceCount(&ndev_avail) != cudaSuccess || ndev_avail <= 0)
  {
    cudaGetLastError();
    return sfail(TTG_ERR_CUDA, "round_batch_devices: no CUDA device");
  }
  for (int32_t p = 0; p < n_dev; ++p)
    if (devices[p] < 0 || devices[p] >= ndev_avail)
      return sfail(TTG_ERR_ARG, "round_batch_devices: device " + std::to_string(devices[p]) +
                                    " does not exist");
  const std::vector<int32_t> part_of = partition(count, ins, n_dev);
  // Sketch ranks are stored TT by TT (d_i - 1 bonds each): slice them.
  std::vector<int64_t> sk_off(static_cast<size_t>(count) + 1, 0);
  for (int32_t i = 0; i < count; ++i)
    sk_off[i + 1] = sk_off[i] + std::max(ins[i].d - 1, 0);

  struct Part
  {
    std::vector<int32_t> idx;
    std::vector<ttg_tensor> in, out;
    std::vector<ttg_round_result> res;
    std::vector<int32_t> sketch;
    int32_t status = TTG_OK;
    std::string err;
  };
  std::vector<Part> parts(static_cast<size_t>(n_dev));
  for (int32_t i = 0; i < count; ++i)
    parts[part_of[i]].idx.push_back(i);
  auto work = [&](int32_t p) {
    Part& P = parts[p];
    if (P.idx.empty())
      return;
    cudaError_t e = cudaSetDevice(devices[p]);
    if (e != cudaSuccess)
    {
      P.status = TTG_ERR_CUDA;
      P.err = std::string("round_batch_devices: cudaSetDevice: ") + cudaGetErrorString(e);
      return;
    }
    const size_t n = P.idx.size();
    P.in.resize(n);
    P.out.assign(n, ttg_tensor{});
    P.res.assign(n, ttg_round_result{});
    ttg_round_options o = *opts;
    for (size_t j = 0; j < n; ++j)
    {
      P.in[j] = ins[P.idx[j]];
      if (opts->sketch_ranks)
        for (int64_t b = sk_off[P.idx[j]]; b < sk_off[P.idx[j] + 1]; ++b)
          P.sketch.push_back(opts->sketch_ranks[b]);
    }
    if (opts->sketch_ranks)
      o.sketch_ranks = P.sketch.data();
    P.status = ttg_round_batch(static_cast<int32_t>(n), P.in.data(), &o, P.out.data(),
                               P.res.data());
    if (P.status != TTG_OK)
      P.err = ttg_last_error();
  };
  std::vector<std::thread> threads;
  for (int32_t p = 1; p < n_dev; ++p)
    threads.emplace_back(work, p);
  work(0);
  for (auto& t : threads)
    t.join();
  int32_t status = TTG_OK;
  std::string err;
  for (const Part& P : parts)
    if (P.status != TTG_OK && status == TTG_OK)
    {
      status = P.status;
      err = P.err;
    }
  for (Part& P : parts)
    for (size_t j = 0; j < P.idx.size() && j < P.out.size(); ++j)
    {
      if (status == TTG_OK)
      {
        outs[P.idx[j]] = P.out[j];
        if (results)
          results[P.idx[j]] = P.res[j];
      }
      else
        ttg_free(&P.out[j]);
    }
  if (status != TTG_OK)
    return sfail(status, err);
  return TTG_OK;
}

int32_t ttg_eval_batch_devices(const ttg_tensor* a, const int32_t* idx, int32_t M, double* out,
                               int32_t n_dev, const int32_t* devices)
{
  using namespace ttg;
  set_last_error(std::string());
  if (!a || M < 0 || n_dev < 1 || !devices || (M > 0 && (!idx || !out)))
    return sfail(TTG_ERR_ARG, "eval_batch_devices: bad arguments");
  int ndev_avail = 0;
  if (cudaGetDeviceCount(&ndev_avail) != cudaSuccess || ndev_avail <= 0)
  {
    cudaGetLastError();
    return sfail(TTG_ERR_CUDA, "eval_batch_devices: no CUDA device");
  }
  for (int32_t p = 0; p < n_dev; ++p)
    if (devices[p] < 0 || devices[p] >= ndev_avail)
      return sfail(TTG_ERR_ARG, "eval_batch_devices: device " + std::to_string(devices[p]) +
                                    " does not exist");
  const int64_t d = a->d;
  std::vector<int32_t> st(static_cast<size_t>(n_dev), TTG_OK);
  std::vector<std::string> errs(static_cast<size_t>(n_dev));
  auto work = [&](int32_t p) {
    // Contiguous slices of the samples, sizes differing by at most one.
    const int64_t lo = static_cast<int64_t>(M) * p / n_dev;
    const int64_t hi = static_cast<int64_t>(M) * (p + 1) / n_dev;
    cudaError_t e = cudaSetDevice(devices[p]);
    if (e != cudaSuccess)
    {
      st[p] = TTG_ERR_CUDA;
      errs[p] = std::string("eval_batch_devices: cudaSetDevice: ") + cudaGetErrorString(e);
      return;
    }
    st[p] = ttg_eval_batch(a, idx + lo * d, static_cast<int32_t>(hi - lo), out + lo);
    if (st[p] != TTG_OK)
      errs[p] = ttg_last_error();
  };
  std::vector<std::thread> threads;
  for (int32_t p = 1; p < n_dev; ++p)
    threads.emplace_back(work, p);
  work(0);
  for (auto& t : threads)
    t.join();
  for (int32_t p = 0; p < n_dev; ++p)
    if (st[p] != TTG_OK)
      return sfail(st[p], errs[p]);
  return TTG_OK;
}

}  // extern "C"
