// Host runtime of libttgpu.so: the C-ABI declared in include/ttg.h.
//
// Validation mirrors the reference's abort conditions (types/tt.hpp:35-70,
// detail/shape_check.hpp:29-149, round/round.hpp:124-134,
// algebra/tt_eval.hpp:34-104) but reports them as status codes.  Every
// compute path runs on the GPU; there is no host fallback.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_job.h"
#include "ttg_kernels.h"

using namespace ttg;

namespace
{

thread_local std::string g_err;
std::atomic<int64_t> g_launches{0};

int32_t fail(int32_t st, const std::string& msg)
{
  g_err = msg;
  return st;
}

#define TTG_CUDA(call)                                                               \
  do                                                                                 \
  {                                                                                  \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(e_ == cudaErrorMemoryAllocation ? TTG_ERR_OOM : TTG_ERR_CUDA,      \
                  std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

struct DeviceInfo
{
  int ok = 0;
  int sms = 0;
  std::string why;
};

const DeviceInfo& device()
{
  static DeviceInfo info = [] {
    DeviceInfo d;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
    {
      d.why = std::string("no CUDA device: ") + cudaGetErrorString(e);
      return d;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    d.ok = 1;
    return d;
  }();
  return info;
}

int32_t need_device()
{
  if (!device().ok)
    return fail(TTG_ERR_CUDA, device().why);
  return TTG_OK;
}

// --------------------------------------------------------------------------
// Tensor description and validation.
// --------------------------------------------------------------------------
struct Shape
{
  int d = 0;
  bool matrix = false;
  std::vector<int> r, m, n;  // r: d+1; m: row modes (n_k of a TT); n: col modes (1 for TT)
  std::vector<int64_t> size, src_off;
  const double* data = nullptr;
  int mode(int k) const { return m[k] * n[k]; }
};

int32_t describe(const ttg_tensor* t, const char* op, Shape& s)
{
  if (!t)
    return fail(TTG_ERR_ARG, std::string(op) + ": null tensor");
  if (t->d < 0)
    return fail(TTG_ERR_ARG, std::string(op) + ": negative d");
  s.d = t->d;
  s.matrix = (t->cols != nullptr);
  s.data = t->data;
  if (s.d == 0)
    return TTG_OK;
  if (!t->ranks || !t->rows || !t->data)
    return fail(TTG_ERR_ARG, std::string(op) + ": null ranks/rows/data");
  s.r.assign(t->ranks, t->ranks + s.d + 1);
  s.m.assign(t->rows, t->rows + s.d);
  s.n.assign(static_cast<size_t>(s.d), 1);
  if (s.matrix)
    s.n.assign(t->cols, t->cols + s.d);
  for (int k = 0; k <= s.d; ++k)
    if (s.r[k] <= 0)
      return fail(TTG_ERR_SHAPE, std::string(op) + ": tt_core: dimensions must be positive");
  for (int k = 0; k < s.d; ++k)
    if (s.m[k] <= 0 || s.n[k] <= 0)
      return fail(TTG_ERR_SHAPE, std::string(op) + ": tt_core: dimensions must be positive");
  if (s.r[0] != 1)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": tt: r_0 must be 1 (got " +
                                   std::to_string(s.r[0]) + ")");
  if (s.r[s.d] != 1)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": tt: r_d must be 1 (got " +
                                   std::to_string(s.r[s.d]) + ")");
  int64_t off = 0;
  for (int k = 0; k < s.d; ++k)
  {
    const int64_t sz = static_cast<int64_t>(s.r[k]) * s.mode(k) * s.r[k + 1];
    if (sz > INT32_MAX)
      return fail(TTG_ERR_SHAPE, std::string(op) + ": core size exceeds INT_MAX");
    s.size.push_back(sz);
    const int64_t o = t->offsets ? t->offsets[k] : off;
    if (t->offsets && t->offsets[k + 1] - t->offsets[k] != sz)
      return fail(TTG_ERR_SHAPE, std::string(op) + ": offsets do not match core " +
                                     std::to_string(k) + " size");
    s.src_off.push_back(o);
    off += sz;
  }
  return TTG_OK;
}

// --------------------------------------------------------------------------
// Device buffers.
// --------------------------------------------------------------------------
struct DevMem
{
  void* p = nullptr;
  size_t bytes = 0;
  ~DevMem() { release(); }
  void release()
  {
    if (p)
      cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b)
  {
    if (b <= bytes)
      return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess)
      bytes = b;
    return e;
  }
};

struct HostPinned
{
  void* p = nullptr;
  size_t bytes = 0;
  ~HostPinned() { release(); }
  void release()
  {
    if (p)
      cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b)
  {
    if (b <= bytes)
      return cudaSuccess;
    release();
    cudaError_t e = cudaHostAlloc(&p, b, cudaHostAllocDefault);
    if (e == cudaSuccess)
      bytes = b;
    return e;
  }
};

size_t align256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

// fn(i) for i in [0, n) on up to 16 host threads (packing and unpacking of
// many tensors is memcpy-bound; one thread would take longer than the
// sweep).  Returns the first non-OK status.
template <class Fn>
int32_t parallel_for(int64_t n, Fn fn)
{
  const int64_t hw = std::max<int64_t>(1, std::thread::hardware_concurrency());
  const int64_t nt = std::min<int64_t>({16, hw, n});
  if (nt <= 1)
  {
    for (int64_t i = 0; i < n; ++i)
      if (int32_t st = fn(i))
        return st;
    return TTG_OK;
  }
  std::atomic<int64_t> next{0};
  std::atomic<int32_t> first{TTG_OK};
  std::vector<std::string> errs(static_cast<size_t>(nt));
  std::vector<std::thread> pool;
  for (int64_t t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (int64_t i = next++; i < n; i = next++)
        if (int32_t st = fn(i))
        {
          int32_t expect = TTG_OK;
          if (first.compare_exchange_strong(expect, st))
            errs[static_cast<size_t>(t)] = g_err;
          return;
        }
    });
  for (auto& th : pool)
    th.join();
  if (first.load() != TTG_OK)
    for (auto& e : errs)
      if (!e.empty())
        g_err = e;
  return first.load();
}

// --------------------------------------------------------------------------
// Round plan: arena + tables + scratch in one device allocation; the
// uploaded prefix [arena | slots | tts | order | idx tables] mirrors a
// pinned host image so upload/download are single copies.
// --------------------------------------------------------------------------
enum PlanKind
{
  kPlanRound,
  kPlanMatvecNaive,
  kPlanStream,
  kPlanEval
};

}  // namespace

namespace ttg
{
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace ttg

struct ttg_plan
{
  PlanKind kind = kPlanRound;
  int job_kind = kJobRound;
  ttg_round_options opts{};
  std::vector<Shape> shapes;       // input tensors, in arena order
  std::vector<int> out_tts;        // TT indices returned to the caller
  std::vector<CoreSlot> slots;
  std::vector<TTInfo> tts;
  std::vector<int32_t> order, a_idx, b_idx, out_idx, sketch;
  size_t off_sketch = 0, off_stats = 0;
  std::vector<BondStat> stats_host;
  int64_t arena_doubles = 0;
  int64_t scratch_stride = 0;
  int grid = 1;
  int cps = 2;          // resident CTAs per SM of the sweep kernel instantiation
  int scratch_ctas = 1; // CTAs the scratch slabs were allocated for
  int smem_doubles = 0;
  // products computed on the device before the sweep (naive apply-round):
  struct Apply
  {
    int a_slot, x_slot, y_slot, r, m, p, rp, s, nout, sp;
  };
  std::vector<Apply> applies;
  // iterative rounding (ALS / DMRG)
  int iter_max = 20;
  double iter_tol = 1.0e-12;
  bool iter_rc = false;
  // whole-GPU schedule (wide_round_kernel)
  bool wide = false;
  int wide_grid = 0;
  int wide_teams = 1;      // teams of the whole-GPU kernel (1 = all CTAs on one TT)
  int wide_teams_max = 1;  // teams the work buffers were allocated for
  WideJob wjob{};
  DevMem wdev;
  // byte layout of the device buffer
  size_t off_arena = 0, off_slots = 0, off_tts = 0, off_order = 0, off_aidx = 0, off_bidx = 0,
         off_oidx = 0, prefix_bytes = 0, off_pristine = 0, off_queue = 0, off_scratch = 0,
         total_bytes = 0;
  DevMem dev;
  HostPinned host;
  // eval plans
  const int32_t* eval_idx = nullptr;
  int64_t M = 0;
  int rcap = 0;
  size_t off_idx = 0, off_out = 0, off_bad = 0;
  int64_t h2d = 0, d2h = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  bool kernel_timed = false;
  // one run captured as a CUDA graph (ttg_plan_graph)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_launches = 0;
  void drop_graph()
  {
    if (gexec)
      cudaGraphExecDestroy(gexec);
    if (graph)
      cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
  }
  ~ttg_plan()
  {
    drop_graph();
    for (cudaEvent_t e : {ev0, ev1, evk0, evk1})
      if (e)
        cudaEventDestroy(e);
  }
};

namespace
{

int add_tensor(ttg_plan& P, const Shape& s, bool upload, const std::vector<int64_t>* cap_sizes)
{
  TTInfo t{};
  t.first = static_cast<int32_t>(P.slots.size());
  t.d = s.d;
  for (int k = 0; k < s.d; ++k)
  {
    CoreSlot c{};
    c.off = P.arena_doubles;
    c.n = s.mode(k);
    c.r = s.r[k];
    c.rp = s.r[k + 1];
    c.m = s.matrix ? s.m[k] : 0;
    const int64_t cap = cap_sizes ? (*cap_sizes)[k] : s.size[k];
    P.arena_doubles += a32(cap);
    P.slots.push_back(c);
  }
  (void)upload;
  P.tts.push_back(t);
  return static_cast<int>(P.tts.size()) - 1;
}

// Scratch need of a round-type sweep over a TT with the given input dims.
int64_t round_need(const Shape& s, int job_kind)
{
  int64_t need = 0;
  const int d = s.d;
  if (d <= 1)
    return 64;
  int64_t cols = 0;
  for (int k = 0; k < d; ++k)
  {
    const int64_t r = s.r[k], n = s.mode(k), rp = s.r[k + 1];
    const int64_t hp = k > 0 ? static_cast<int64_t>(s.r[k - 1]) * s.mode(k - 1) : 0;
    const int64_t wn = k + 1 < d ? static_cast<int64_t>(s.mode(k + 1)) * s.r[k + 2] : 0;
    if (job_kind == kJobRound || job_kind == kJobRightOrth || job_kind == kJobSoftThreshold)
    {
      if (k >= 1)
        need = std::max(need, need_right_qr(r, n * rp, hp));
      if (k <= d - 2 && job_kind == kJobRound)
        need = std::max(need, need_svd_step(r * n, rp, wn));
      if (k >= 1 && job_kind == kJobSoftThreshold)
        need = std::max(need, need_soft_step(hp, n * rp));
    }
    else
    {
      if (k <= d - 2)
        need = std::max(need, need_left_qr(r * n, rp, wn));
      if (k >= 1)
        need = std::max(need, need_svd_step_right(n * rp, r, hp));
    }
    if (k <= d - 2)
      cols += rp;
  }
  need = std::max(need, a32(2 * (cols + 1)));  // balance: scale factors and inverses
  return need + 64;
}

int64_t stream_need(const Shape& A, const Shape& X)
{
  const int d = A.d;
  int64_t need = std::max(round_need(A, kJobRightOrth), round_need(X, kJobRightOrth));
  int64_t fcap = 1;
  for (int k = 0; k < d; ++k)
  {
    const int64_t cap = static_cast<int64_t>(A.r[k + 1]) * X.r[k + 1];
    fcap = std::max(fcap, cap * cap);
  }
  for (int k = 0; k < d; ++k)
  {
    const int64_t alpha = static_cast<int64_t>(A.r[k]) * X.r[k];
    need = std::max(need, need_stream_step(fcap, alpha, A.r[k], A.m[k], A.n[k], A.r[k + 1],
                                           X.r[k], X.mode(k) / A.n[k], X.r[k + 1]));
  }
  return need + 64;
}

double est_cost(const Shape& s)
{
  double c = 0.0;
  for (int k = 0; k < s.d; ++k)
    c += static_cast<double>(s.size[k]) * std::max(s.r[k], s.r[k + 1]);
  return c;
}

// Dynamic shared memory of the sweep kernel: two CTAs per SM share the
// SM's 228 KB (each also has ~17 KB of static shared state) when the grid
// is larger than the SM count, one CTA gets ~200 KB otherwise.
constexpr int kSmemTwoPerSm = 11776;  // 92 KB
constexpr int kSmemOnePerSm = 25600;  // 200 KB
constexpr int kSmemThreePerSm = 7168;  // 56 KB
constexpr int kSmemFourPerSm = 4864;   // 38 KB

// Whole-GPU schedule: chosen for round jobs (method svd, both gauges) by
// the options, or automatically for at most 4 TTs with a bond rank >= 64.
// Work buffers are sized for the largest core and rank of the TTs swept.
int32_t setup_wide(ttg_plan& P)
{
  P.wide = false;
  const bool stream = P.job_kind == kJobStreamMatvec || P.job_kind == kJobStreamMatmat;
  if ((P.job_kind != kJobRound && P.job_kind != kJobRoundRight && !stream) || P.order.empty() ||
      P.opts.schedule == TTG_SCHED_PER_TT)
    return TTG_OK;
  // TTs whose cores the sweep touches: the rounded TTs, or every operand and
  // output of the streaming items.
  std::vector<int> swept;
  if (stream)
    for (int it : P.order)
    {
      swept.push_back(P.a_idx[it]);
      swept.push_back(P.b_idx[it]);
      swept.push_back(P.out_idx[it]);
    }
  else
    swept = P.order;
  int64_t core_max = 1, c_max = 1, cols_max = 1, s_max = 1, f_max = 1;
  if (stream)
    for (int it : P.order)
    {
      const TTInfo& ta = P.tts[P.a_idx[it]];
      const TTInfo& tx = P.tts[P.b_idx[it]];
      for (int k = 0; k < ta.d; ++k)
      {
        const CoreSlot& A = P.slots[ta.first + k];
        const CoreSlot& X = P.slots[tx.first + k];
        const int64_t a = A.r, b = A.rp, m = A.m, p = A.n / std::max(A.m, 1);
        const int64_t sx = X.r, bx = X.rp, nout = X.n / std::max<int64_t>(p, 1);
        const int64_t alpha = a * sx;  // the output's left bond never exceeds this
        s_max = std::max({s_max, alpha * sx * a, alpha * sx * m * p * b, alpha * m * b * nout * bx});
        f_max = std::max(f_max, (b * bx) * (b * bx));
      }
    }
  for (int t : swept)
  {
    const TTInfo& ti = P.tts[t];
    int64_t cols = 0;
    for (int k = 0; k < ti.d; ++k)
    {
      const CoreSlot& c = P.slots[ti.first + k];
      core_max = std::max<int64_t>(core_max, static_cast<int64_t>(c.r) * c.n * c.rp);
      c_max = std::max<int64_t>(c_max, std::max(c.r, c.rp));
      cols += c.rp;
    }
    cols_max = std::max(cols_max, cols);
  }
  const int64_t items = static_cast<int64_t>(P.order.size());
  const bool force_whole = P.opts.schedule == TTG_SCHED_WHOLE_GPU;
  const bool force_teams = P.opts.schedule == TTG_SCHED_TEAMS;
  const bool big = c_max >= 64;
  // Whole grid on one TT at a time: forced, or AUTO for a few large TTs.
  // Teams: forced, or offered to the autotuner for 5..256 large TTs (the
  // default stays one CTA per TT).
  const bool want_whole = force_whole || (!force_teams && items <= 4 && big);
  const bool offer_teams = force_teams || (!force_whole && items > 4 && items <= 256 && big);
  if (stream)
    core_max = std::max(core_max, s_max);
  if (!want_whole && !offer_teams)
    return TTG_OK;
  // Jacobi block pairs: (2 c_max rows + c_max V rows) x 2b columns + 2b norms.
  int jb = 4;
  while (jb > 1 && (6 * c_max + 2) * jb > kSmemOnePerSm)
    jb /= 2;
  if ((6 * c_max + 2) * jb > kSmemOnePerSm)
    return TTG_OK;  // ranks beyond the block buffers: stay per TT
  const int64_t smem = kSmemOnePerSm;
  int grid = 0;
  const cudaError_t e = wide_round_setup(static_cast<int>(smem), &grid);
  if (e != cudaSuccess)
    return fail(TTG_ERR_CUDA, std::string("whole-GPU round setup: ") + cudaGetErrorString(e));
  if (grid < 2)
    return TTG_OK;
  // Team counts: up to one team per item, at least 4 CTAs per team, 32 teams.
  int teams_max = 1;
  if (offer_teams)
    teams_max = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>({items, static_cast<int64_t>(grid / 4), 32})));
  const int ms = P.opts.max_sweeps > 0 ? P.opts.max_sweeps : 40;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t r = o;
    o = align256(o + bytes);
    return r;
  };
  const size_t cc = sizeof(double) * static_cast<size_t>(c_max * c_max);
  const size_t cm = sizeof(double) * static_cast<size_t>(core_max);
  const size_t oW = take(cm), oU = take(cm), oP = take(cm), oA = take(cm), oR = take(cc),
               oV = take(cc), oF = take(cc), oT1 = take(cc), oT2 = take(cc),
               opart = take(8 * static_cast<size_t>(grid) + 8), oumax = take(8),
               otau = take(8 * c_max), osig = take(8 * c_max),
               osorted = take(8 * c_max), oord = take(4 * c_max), ocn = take(8 * (cols_max + 1)),
               oival = take(64), orot = take(4 * ms), orel = take(4 * ms),
               oS1 = take(stream ? 8 * static_cast<size_t>(s_max) : 8),
               oS2 = take(stream ? 8 * static_cast<size_t>(s_max) : 8),
               oFs = take(stream ? 8 * static_cast<size_t>(f_max) : 8);
  // One such block per team, then the teams' barrier words.
  const size_t team_bytes = o;
  const size_t obar = team_bytes * static_cast<size_t>(teams_max);
  o = align256(obar + sizeof(GridBar) * static_cast<size_t>(teams_max));
  TTG_CUDA(P.wdev.ensure(o));
  char* b = static_cast<char*>(P.wdev.p);
  char* d = static_cast<char*>(P.dev.p);
  WideJob& j = P.wjob;
  j = WideJob{};
  j.arena = reinterpret_cast<double*>(d + P.off_arena);
  j.slots = reinterpret_cast<CoreSlot*>(d + P.off_slots);
  j.tts = reinterpret_cast<TTInfo*>(d + P.off_tts);
  j.order = reinterpret_cast<const int32_t*>(d + P.off_order);
  j.ntt = static_cast<int32_t>(P.order.size());
  j.max_rank = P.opts.max_rank;
  j.max_sweeps = ms;
  j.jblock = jb;
  j.smem_doubles = smem;
  j.eps = P.opts.eps;
  j.W = reinterpret_cast<double*>(b + oW);
  j.Ub = reinterpret_cast<double*>(b + oU);
  j.Pb = reinterpret_cast<double*>(b + oP);
  j.A = reinterpret_cast<double*>(b + oA);
  j.R = reinterpret_cast<double*>(b + oR);
  j.V = reinterpret_cast<double*>(b + oV);
  j.F = reinterpret_cast<double*>(b + oF);
  j.T1 = reinterpret_cast<double*>(b + oT1);
  j.T2 = reinterpret_cast<double*>(b + oT2);
  j.part = reinterpret_cast<double*>(b + opart);
  j.umax = reinterpret_cast<unsigned long long*>(b + oumax);
  j.mixed = P.opts.precision == TTG_PREC_MIXED ? 1 : 0;
  // Sliced-BF16 tensor-core contractions (mixed path only): measured slower
  // than the FP64 tiles on these latency-bound sweeps, so off unless
  // TTG_WIDE_TENSOR_CORES=1 or the autotuner picks them.
  {
    const char* e = std::getenv("TTG_WIDE_TENSOR_CORES");
    j.tc = (j.mixed && e && e[0] == '1') ? 1 : 0;
  }
  // Failure-path tests only (TTG_TEST_STALL_DEVICE_WAITS=1): no grid barrier
  // completes and each wait gives up after ~1 ms, so that the call returns
  // TTG_ERR_TIMEOUT through the same path a real stall would take.
  {
    const char* e = std::getenv("TTG_TEST_STALL_DEVICE_WAITS");
    j.stall_waits = (e && e[0] == '1') ? 1 : 0;
    j.wait_cycles = j.stall_waits ? 2000000ll : 4000000000ll;  // ~1 ms / ~2 s at 2 GHz
  }
  j.tau = reinterpret_cast<double*>(b + otau);
  j.sig = reinterpret_cast<double*>(b + osig);
  j.sorted = reinterpret_cast<double*>(b + osorted);
  j.ord = reinterpret_cast<int*>(b + oord);
  j.cn = reinterpret_cast<double*>(b + ocn);
  j.ival = reinterpret_cast<int*>(b + oival);
  j.sweep_rot = reinterpret_cast<unsigned int*>(b + orot);
  j.sweep_rel = reinterpret_cast<unsigned int*>(b + orel);
  j.bar = reinterpret_cast<GridBar*>(b + obar);
  j.kind = P.job_kind;
  j.a_idx = reinterpret_cast<const int32_t*>(d + P.off_aidx);
  j.b_idx = reinterpret_cast<const int32_t*>(d + P.off_bidx);
  j.out_idx = reinterpret_cast<const int32_t*>(d + P.off_oidx);
  j.S1 = reinterpret_cast<double*>(b + oS1);
  j.S2 = reinterpret_cast<double*>(b + oS2);
  j.Fs = reinterpret_cast<double*>(b + oFs);
  j.bond_stats = P.opts.bond_stats ? reinterpret_cast<BondStat*>(d + P.off_stats) : nullptr;
  j.team_bytes = static_cast<int64_t>(team_bytes);
  P.wide_grid = grid;
  P.wide_teams_max = teams_max;
  if (want_whole)
  {
    P.wide = true;
    P.wide_teams = 1;
  }
  else if (force_teams)
  {
    P.wide = true;
    P.wide_teams = teams_max;
  }
  else
    P.wide_teams = teams_max;  // offered to the autotuner; per-TT stays the default
  return TTG_OK;
}

int32_t layout_and_alloc(ttg_plan& P)
{
  static const cudaError_t optin = round_smem_optin(kSmemOnePerSm);
  if (optin != cudaSuccess)
    return fail(TTG_ERR_CUDA, std::string("round kernel shared-memory opt-in: ") +
                                  cudaGetErrorString(optin));
  const int sms = std::max(device().sms, 1);
  P.smem_doubles = P.grid > sms ? kSmemTwoPerSm : kSmemOnePerSm;
  P.cps = P.grid > sms ? 2 : 1;
  // Large batches get scratch for up to 4 CTAs per SM (autotuner candidates).
  // FP64 sweeps start at 4 per SM (DFMA-bound: more resident TTs keep the
  // pipe fed); mixed sweeps at 3, whose 56 KB of shared staging still holds
  // the blocked df64 Householder panels -- the autotuner's picks on the
  // uneven 4096-TT batch.
  P.scratch_ctas = P.grid;
  if (static_cast<int64_t>(P.order.size()) > 2LL * sms && P.job_kind >= 0)
  {
    P.scratch_ctas = static_cast<int>(std::min<int64_t>(static_cast<int64_t>(P.order.size()),
                                                        4LL * sms));
    const bool mixed = P.opts.precision == TTG_PREC_MIXED;
    const int cps = mixed ? 3 : 4;
    if (static_cast<int64_t>(P.order.size()) >= static_cast<int64_t>(cps) * sms)
    {
      P.grid = cps * sms;
      P.cps = cps;
      P.smem_doubles = mixed ? kSmemThreePerSm : kSmemFourPerSm;
    }
  }
  size_t o = 0;
  P.off_arena = o;
  o = align256(o + sizeof(double) * static_cast<size_t>(P.arena_doubles));
  P.off_slots = o;
  o = align256(o + sizeof(CoreSlot) * P.slots.size());
  P.off_tts = o;
  o = align256(o + sizeof(TTInfo) * P.tts.size());
  P.off_order = o;
  o = align256(o + sizeof(int32_t) * P.order.size());
  P.off_aidx = o;
  o = align256(o + sizeof(int32_t) * P.a_idx.size());
  P.off_bidx = o;
  o = align256(o + sizeof(int32_t) * P.b_idx.size());
  P.off_oidx = o;
  o = align256(o + sizeof(int32_t) * P.out_idx.size());
  P.off_sketch = o;
  o = align256(o + sizeof(int32_t) * P.sketch.size());
  P.prefix_bytes = o;
  P.off_pristine = o;
  o = align256(o + P.prefix_bytes);
  P.off_queue = o;
  o = align256(o + 256);
  P.off_stats = o;
  o = align256(o + (P.opts.bond_stats ? sizeof(BondStat) * P.slots.size() : 0));
  P.off_scratch = o;
  o = align256(o + sizeof(double) * static_cast<size_t>(P.scratch_stride) *
                       static_cast<size_t>(std::max(P.grid, P.scratch_ctas)));
  P.total_bytes = o;
  TTG_CUDA(P.dev.ensure(P.total_bytes));
  TTG_CUDA(P.host.ensure(P.prefix_bytes));
  TTG_CUDA(cudaEventCreate(&P.ev0));
  TTG_CUDA(cudaEventCreate(&P.ev1));
  TTG_CUDA(cudaEventCreate(&P.evk0));
  TTG_CUDA(cudaEventCreate(&P.evk1));
  // Host image of the prefix: arena inputs + tables.  Only the tables are
  // cleared; every arena byte a sweep reads is a copied input.
  char* h = static_cast<char*>(P.host.p);
  std::memset(h + P.off_slots, 0, P.prefix_bytes - P.off_slots);
  double* arena = reinterpret_cast<double*>(h + P.off_arena);
  parallel_for(static_cast<int64_t>(P.shapes.size()), [&](int64_t t) -> int32_t {
    const Shape& s = P.shapes[static_cast<size_t>(t)];
    const TTInfo& ti = P.tts[static_cast<size_t>(t)];
    for (int k = 0; k < s.d; ++k)
      std::memcpy(arena + P.slots[ti.first + k].off, s.data + s.src_off[k],
                  sizeof(double) * static_cast<size_t>(s.size[k]));
    return TTG_OK;
  });
  std::memcpy(h + P.off_slots, P.slots.data(), sizeof(CoreSlot) * P.slots.size());
  std::memcpy(h + P.off_tts, P.tts.data(), sizeof(TTInfo) * P.tts.size());
  std::memcpy(h + P.off_order, P.order.data(), sizeof(int32_t) * P.order.size());
  if (!P.sketch.empty())
    std::memcpy(h + P.off_sketch, P.sketch.data(), sizeof(int32_t) * P.sketch.size());
  if (!P.a_idx.empty())
  {
    std::memcpy(h + P.off_aidx, P.a_idx.data(), sizeof(int32_t) * P.a_idx.size());
    std::memcpy(h + P.off_bidx, P.b_idx.data(), sizeof(int32_t) * P.b_idx.size());
    std::memcpy(h + P.off_oidx, P.out_idx.data(), sizeof(int32_t) * P.out_idx.size());
  }
  P.h2d = static_cast<int64_t>(P.prefix_bytes);
  P.d2h = static_cast<int64_t>(P.off_order);
  return setup_wide(P);
}

RoundJob make_job(ttg_plan& P)
{
  char* d = static_cast<char*>(P.dev.p);
  RoundJob j{};
  j.arena = reinterpret_cast<double*>(d + P.off_arena);
  j.slots = reinterpret_cast<CoreSlot*>(d + P.off_slots);
  j.tts = reinterpret_cast<TTInfo*>(d + P.off_tts);
  j.order = reinterpret_cast<const int32_t*>(d + P.off_order);
  j.ntt = static_cast<int32_t>(P.order.size());
  j.kind = P.job_kind;
  j.scratch = reinterpret_cast<double*>(d + P.off_scratch);
  j.scratch_stride = P.scratch_stride;
  j.queue = reinterpret_cast<int32_t*>(d + P.off_queue);
  j.eps = P.opts.eps;
  j.max_rank = P.opts.max_rank;
  j.max_sweeps = P.opts.max_sweeps > 0 ? P.opts.max_sweeps : 40;
  j.smem_doubles = P.smem_doubles;
  j.mixed = P.opts.precision == TTG_PREC_MIXED ? 1 : 0;
  j.a_idx = reinterpret_cast<const int32_t*>(d + P.off_aidx);
  j.b_idx = reinterpret_cast<const int32_t*>(d + P.off_bidx);
  j.out_idx = reinterpret_cast<const int32_t*>(d + P.off_oidx);
  j.sketch_ranks = P.sketch.empty() ? nullptr : reinterpret_cast<const int32_t*>(d + P.off_sketch);
  j.sketch_seed = P.opts.sketch_seed;
  j.pristine_arena = reinterpret_cast<const double*>(d + P.off_pristine + P.off_arena);
  j.pristine_slots = reinterpret_cast<const CoreSlot*>(d + P.off_pristine + P.off_slots);
  j.bond_stats = P.opts.bond_stats ? reinterpret_cast<BondStat*>(d + P.off_stats) : nullptr;
  j.max_iters = P.iter_max;
  j.tol = P.iter_tol;
  j.x_right_canonical = P.iter_rc ? 1 : 0;
  return j;
}

int32_t check_opts(const ttg_round_options* o, const char* op)
{
  if (!o)
    return fail(TTG_ERR_ARG, std::string(op) + ": null options");
  if (std::isnan(o->eps) || o->eps < 0.0)
    return fail(TTG_ERR_ARG, std::string(op) + ": eps must be >= 0");
  if (o->max_rank < 0)
    return fail(TTG_ERR_ARG, std::string(op) + ": max_rank must be >= 0");
  if (o->gauge != TTG_GAUGE_NONE && o->gauge != TTG_GAUGE_RIGHT_CANONICAL)
    return fail(TTG_ERR_ARG, std::string(op) + ": unknown gauge");
  if (o->precision != TTG_PREC_FP64 && o->precision != TTG_PREC_MIXED)
    return fail(TTG_ERR_ARG, std::string(op) + ": unknown precision");
  if (o->schedule < TTG_SCHED_AUTO || o->schedule > TTG_SCHED_TEAMS)
    return fail(TTG_ERR_ARG, std::string(op) + ": unknown schedule");
  if (o->method < 0 || o->method > TTG_METHOD_SKETCH)
    return fail(TTG_ERR_METHOD, std::string(op) + ": unknown method " + std::to_string(o->method));
  return TTG_OK;
}

int finish_grid(int64_t items)
{
  const int sms = std::max(device().sms, 1);
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(items, 2LL * sms)));
}

// job_kind >= 0 replaces the sweep the options select (right_orthogonalize,
// soft_threshold); it is fixed before the layout, which sizes the scratch
// and picks the schedule for it.
int32_t build_round_plan(ttg_plan& P, int32_t count, const ttg_tensor* ins,
                         const ttg_round_options* opts, const char* op, int job_kind = -1)
{
  if (int32_t st = check_opts(opts, op))
    return st;
  if (opts->method != TTG_METHOD_SVD && opts->method != TTG_METHOD_SKETCH)
    return fail(TTG_ERR_METHOD, std::string(op) +
                                    ": round_method::svd_streaming / svd_naive are only valid on "
                                    "matvec_round / matmat_round respectively.");
  const bool sketch = opts->method == TTG_METHOD_SKETCH;
  if (sketch && opts->gauge != TTG_GAUGE_NONE)
    return fail(TTG_ERR_ARG, std::string(op) + ": the sketch method serves gauge none only");
  P.opts = *opts;
  P.kind = kPlanRound;
  P.job_kind = sketch ? kJobRoundSketch
                      : (opts->gauge == TTG_GAUGE_RIGHT_CANONICAL ? kJobRoundRight : kJobRound);
  if (job_kind >= 0)
    P.job_kind = job_kind;
  P.shapes.resize(static_cast<size_t>(count));
  int64_t need = 64;
  std::vector<std::pair<double, int>> cost;
  for (int i = 0; i < count; ++i)
  {
    if (int32_t st = describe(&ins[i], op, P.shapes[i]))
      return st;
    add_tensor(P, P.shapes[i], true, nullptr);
    need = std::max(need, round_need(P.shapes[i], sketch ? kJobRound : P.job_kind));
    P.out_tts.push_back(i);
    if (P.shapes[i].d > 1)
      cost.emplace_back(est_cost(P.shapes[i]), i);
  }
  if (sketch)
  {
    // Sketch-rank table indexed by global core (the bond right of the core).
    P.sketch.assign(P.slots.size(), 1);
    int64_t pos = 0;
    for (int i = 0; i < count; ++i)
    {
      const Shape& sh = P.shapes[i];
      int64_t rmax = 1, lsum = 0, lmax = 1, hmax = 1, nmax = 1, gsum = 0;
      for (int k = 0; k < sh.d; ++k)
      {
        if (k >= 1)
          gsum += static_cast<int64_t>(sh.r[k]) * sh.r[k];
        rmax = std::max<int64_t>(rmax, std::max(sh.r[k], sh.r[k + 1]));
        hmax = std::max<int64_t>(hmax, static_cast<int64_t>(sh.r[k]) * sh.mode(k));
        nmax = std::max<int64_t>(nmax, sh.mode(k));
        if (k < sh.d - 1)
        {
          int l = opts->sketch_ranks ? opts->sketch_ranks[pos + k] : sh.r[k + 1];
          if (l < 1)
            return fail(TTG_ERR_ARG, std::string(op) + ": sketch ranks must be >= 1");
          l = std::min(l, sh.r[k + 1]);
          P.sketch[P.tts[i].first + k] = l;
          lsum += static_cast<int64_t>(sh.r[k + 1]) * l;
          lmax = std::max<int64_t>(lmax, l);
        }
      }
      pos += sh.d > 0 ? sh.d - 1 : 0;
      need = std::max(need, need_sketch(rmax, lsum, lmax, hmax, nmax, gsum) + 64);
    }
  }
  std::stable_sort(cost.begin(), cost.end(),
                   [](const auto& a, const auto& b) { return a.first > b.first; });
  for (auto& c : cost)
    P.order.push_back(c.second);
  P.scratch_stride = need;
  P.grid = finish_grid(static_cast<int64_t>(P.order.size()));
  return layout_and_alloc(P);
}

// Inputs land in the pristine copy; run() deep-copies them into the work
// region, so a plan can be run any number of times.
int32_t plan_upload(ttg_plan& P, cudaStream_t st)
{
  char* d = static_cast<char*>(P.dev.p);
  TTG_CUDA(cudaMemcpyAsync(d + P.off_pristine, P.host.p, P.prefix_bytes, cudaMemcpyHostToDevice,
                           st));
  return TTG_OK;
}

// Event record that also works inside a stream capture: there it becomes
// an event-record node of the graph, so every replay records the event.
cudaError_t record_event(cudaEvent_t ev, cudaStream_t st)
{
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
    return cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
  return cudaEventRecord(ev, st);
}

int32_t plan_run(ttg_plan& P, cudaStream_t st)
{
  char* d = static_cast<char*>(P.dev.p);
  if (P.kind == kPlanEval)
  {
    TTG_CUDA(cudaMemsetAsync(d + P.off_bad, 0, sizeof(int), st));
    const Shape& s = P.shapes[0];
    const int sms = std::max(device().sms, 1);
    const int64_t warps_needed = (P.M + 7) / 8;
    const int grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(warps_needed, 8LL * sms)));
    launch_eval(reinterpret_cast<double*>(d + P.off_arena),
                reinterpret_cast<CoreSlot*>(d + P.off_slots), s.d,
                reinterpret_cast<const int*>(d + P.off_idx), P.M,
                reinterpret_cast<double*>(d + P.off_out), P.rcap,
                reinterpret_cast<int*>(d + P.off_bad), grid, st);
    g_launches += 1;
    TTG_CUDA(cudaGetLastError());
    return TTG_OK;
  }
  TTG_CUDA(cudaMemcpyAsync(d, d + P.off_pristine, P.prefix_bytes, cudaMemcpyDeviceToDevice, st));
  double* arena = reinterpret_cast<double*>(d + P.off_arena);
  for (const auto& a : P.applies)
  {
    launch_apply_core(arena + P.slots[a.a_slot].off, arena + P.slots[a.x_slot].off,
                      arena + P.slots[a.y_slot].off, a.r, a.m, a.p, a.rp, a.s, a.nout, a.sp, st);
    g_launches += 1;
  }
  if (!P.order.empty() && P.job_kind >= 0)
  {
    TTG_CUDA(cudaMemsetAsync(d + P.off_queue, 0, sizeof(int32_t), st));
    if (P.opts.bond_stats)
      TTG_CUDA(cudaMemsetAsync(d + P.off_stats, 0, sizeof(BondStat) * P.slots.size(), st));
    TTG_CUDA(record_event(P.evk0, st));
    if (P.wide)
    {
      TTG_CUDA(cudaMemsetAsync(P.wjob.bar, 0, sizeof(GridBar) * P.wide_teams, st));
      WideJob j = P.wjob;
      j.teams = P.wide_teams;
      const int tsize = P.wide_grid / P.wide_teams;
      TTG_CUDA(launch_wide_round(j, tsize * P.wide_teams, st));
    }
    else
      launch_round(make_job(P), P.grid, P.cps, st);
    TTG_CUDA(record_event(P.evk1, st));
    P.kernel_timed = true;
    g_launches += 1;
  }
  TTG_CUDA(cudaGetLastError());
  return TTG_OK;
}

int32_t plan_download_raw(ttg_plan& P, cudaStream_t st)
{
  TTG_CUDA(cudaMemcpyAsync(P.host.p, P.dev.p, P.off_order, cudaMemcpyDeviceToHost, st));
  if (P.opts.bond_stats && !P.slots.empty())
  {
    P.stats_host.resize(P.slots.size());
    TTG_CUDA(cudaMemcpyAsync(P.stats_host.data(), static_cast<char*>(P.dev.p) + P.off_stats,
                             sizeof(BondStat) * P.slots.size(), cudaMemcpyDeviceToHost, st));
  }
  std::vector<GridBar> bars(static_cast<size_t>(std::max(P.wide_teams, 1)));
  if (P.wide)
    TTG_CUDA(cudaMemcpyAsync(bars.data(), P.wjob.bar, sizeof(GridBar) * bars.size(),
                             cudaMemcpyDeviceToHost, st));
  TTG_CUDA(cudaStreamSynchronize(st));
  if (P.wide)
    for (const GridBar& bar : bars)
      if (bar.err)
        return fail(TTG_ERR_TIMEOUT, "whole-GPU round: a grid barrier wait timed out");
  if (P.opts.bond_stats && !P.slots.empty())
  {
    // 4 doubles per bond, TT by TT.
    int64_t pos = 0;
    for (size_t t = 0; t < P.tts.size() && t < P.shapes.size(); ++t)
    {
      const TTInfo& ti = P.tts[t];
      for (int k = 0; k + 1 < ti.d; ++k, ++pos)
      {
        const BondStat& b = P.stats_host[ti.first + k];
        P.opts.bond_stats[4 * pos + 0] = b.s_max;
        P.opts.bond_stats[4 * pos + 1] = b.s_last;
        P.opts.bond_stats[4 * pos + 2] = b.r_new;
        P.opts.bond_stats[4 * pos + 3] = b.n_sv;
      }
    }
  }
  return TTG_OK;
}

// Builds an output tensor from TT `t` of the downloaded host image.
int32_t emit_tensor(ttg_plan& P, int t, bool matrix, const std::vector<int>& mrow,
                    const std::vector<int>& ncol, ttg_tensor* out)
{
  const char* h = static_cast<const char*>(P.host.p);
  const CoreSlot* S = reinterpret_cast<const CoreSlot*>(h + P.off_slots);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P.off_tts);
  const double* arena = reinterpret_cast<const double*>(h + P.off_arena);
  const TTInfo& ti = T[t];
  const int d = ti.d;
  std::memset(out, 0, sizeof(*out));
  out->d = d;
  out->owned = 1;
  out->ranks = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (d + 1)));
  out->rows = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max(d, 1)));
  out->offsets = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (d + 1)));
  if (matrix)
    out->cols = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max(d, 1)));
  if (!out->ranks || !out->rows || !out->offsets || (matrix && !out->cols))
    return fail(TTG_ERR_OOM, "host allocation failed");
  int64_t total = 0;
  out->ranks[0] = d > 0 ? S[ti.first].r : 1;
  for (int k = 0; k < d; ++k)
  {
    const CoreSlot& c = S[ti.first + k];
    out->ranks[k + 1] = c.rp;
    out->rows[k] = matrix ? mrow[k] : c.n;
    if (matrix)
      out->cols[k] = ncol[k];
    out->offsets[k] = total;
    total += static_cast<int64_t>(c.r) * c.n * c.rp;
  }
  out->offsets[d] = total;
  out->data = static_cast<double*>(std::malloc(sizeof(double) * std::max<int64_t>(total, 1)));
  if (!out->data)
    return fail(TTG_ERR_OOM, "host allocation failed");
  for (int k = 0; k < d; ++k)
  {
    const CoreSlot& c = S[ti.first + k];
    std::memcpy(out->data + out->offsets[k], arena + c.off,
                sizeof(double) * static_cast<size_t>(static_cast<int64_t>(c.r) * c.n * c.rp));
  }
  return TTG_OK;
}

void fill_result(const TTInfo& ti, float ms, ttg_round_result* r)
{
  if (!r)
    return;
  r->iters_run = 1;
  r->final_resid = 0.0;
  r->converged = ti.status == TTG_ERR_NOT_CONVERGED ? 0 : 1;
  r->norm = ti.norm;
  r->delta = ti.delta;
  r->device_ms = ms;
  r->status = ti.status;
  r->jacobi_sweeps = ti.sweeps;
  r->sketch_state = ti.sketch_state;
  r->sketch_rel_err = ti.sketch_err;
}

int32_t first_bad_status(const ttg_plan& P)
{
  const char* h = static_cast<const char*>(P.host.p);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P.off_tts);
  for (size_t i = 0; i < P.tts.size(); ++i)
    if (T[i].status != TTG_OK && T[i].status != TTG_ERR_NOT_CONVERGED)
      return T[i].status;
  return TTG_OK;
}

// State of the one-shot entry points, one set per device: the stream they
// run on, the lock that serialises them, and the buffers they reuse
// (grow-only, guarded by the lock), so repeated calls do not pay cudaMalloc /
// cudaHostAlloc again.  Calls on different devices (the multi-device batch
// entries run one host thread per device) proceed in parallel.
constexpr int kMaxDevices = 64;

struct DeviceState
{
  std::mutex mu;
  std::once_flag stream_once, stream2_once;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // the second chunk of a pipelined batch
  DevMem dev_pool, dev_pool2;
  HostPinned host_pool, host_pool2;
};

DeviceState g_devices[kMaxDevices];

DeviceState& dev_state()
{
  int dev = 0;
  cudaGetDevice(&dev);
  return g_devices[(dev >= 0 && dev < kMaxDevices) ? dev : 0];
}

cudaStream_t lib_stream()
{
  DeviceState& s = dev_state();
  std::call_once(s.stream_once,
                 [&] { cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking); });
  return s.stream;
}

cudaStream_t lib_stream2()
{
  DeviceState& s = dev_state();
  std::call_once(s.stream2_once,
                 [&] { cudaStreamCreateWithFlags(&s.stream2, cudaStreamNonBlocking); });
  return s.stream2;
}

// Lends the device's buffers (slot 0, or slot 1 for the second plan of a
// pipelined batch) to a plan for one call, and takes them back grown.
struct PoolLease
{
  ttg_plan& P;
  DevMem& dev;
  HostPinned& host;
  explicit PoolLease(ttg_plan& p, int slot = 0)
    : P(p), dev(slot ? dev_state().dev_pool2 : dev_state().dev_pool),
      host(slot ? dev_state().host_pool2 : dev_state().host_pool)
  {
    std::swap(P.dev.p, dev.p);
    std::swap(P.dev.bytes, dev.bytes);
    std::swap(P.host.p, host.p);
    std::swap(P.host.bytes, host.bytes);
  }
  ~PoolLease()
  {
    std::swap(P.dev.p, dev.p);
    std::swap(P.dev.bytes, dev.bytes);
    std::swap(P.host.p, host.p);
    std::swap(P.host.bytes, host.bytes);
  }
};

// Runs a plan end to end on the library stream with device timing.
int32_t execute(ttg_plan& P, float* ms)
{
  cudaStream_t st = lib_stream();
  if (int32_t e = plan_upload(P, st))
    return e;
  TTG_CUDA(cudaEventRecord(P.ev0, st));
  if (int32_t e = plan_run(P, st))
    return e;
  TTG_CUDA(cudaEventRecord(P.ev1, st));
  if (int32_t e = plan_download_raw(P, st))
    return e;
  TTG_CUDA(cudaEventElapsedTime(ms, P.ev0, P.ev1));
  return TTG_OK;
}

int32_t copy_through(const Shape& s, ttg_tensor* out)
{
  // d <= 1: round returns its input unchanged (round/tt_round.hpp:38-42).
  std::memset(out, 0, sizeof(*out));
  out->d = s.d;
  out->owned = 1;
  out->ranks = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (s.d + 1)));
  out->rows = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max(s.d, 1)));
  out->offsets = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (s.d + 1)));
  if (s.matrix)
    out->cols = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max(s.d, 1)));
  out->ranks[0] = 1;
  int64_t total = 0;
  for (int k = 0; k < s.d; ++k)
  {
    out->ranks[k + 1] = s.r[k + 1];
    out->rows[k] = s.m[k];
    if (s.matrix)
      out->cols[k] = s.n[k];
    out->offsets[k] = total;
    total += s.size[k];
  }
  out->offsets[s.d] = total;
  out->data = static_cast<double*>(std::malloc(sizeof(double) * std::max<int64_t>(total, 1)));
  for (int k = 0; k < s.d; ++k)
    std::memcpy(out->data + out->offsets[k], s.data + s.src_off[k],
                sizeof(double) * static_cast<size_t>(s.size[k]));
  return TTG_OK;
}

}  // namespace

extern "C" {

const char* ttg_version(void) { return "ttgpu 0.1 (sm_103a, fp64 sweep)"; }

const char* ttg_status_string(int32_t s)
{
  switch (s)
  {
    case TTG_OK: return "ok";
    case TTG_ERR_ARG: return "invalid argument";
    case TTG_ERR_SHAPE: return "shape mismatch";
    case TTG_ERR_METHOD: return "method not valid here";
    case TTG_ERR_INDEX: return "index out of range";
    case TTG_ERR_NAN: return "non-finite value";
    case TTG_ERR_NOT_CONVERGED: return "Jacobi SVD did not converge";
    case TTG_ERR_TIMEOUT: return "device wait timed out";
    case TTG_ERR_OOM: return "out of memory";
    case TTG_ERR_CUDA: return "CUDA error";
    case TTG_ERR_EMPTY: return "empty tensor (d = 0)";
    case TTG_ERR_NO_SPACE: return "size exceeds a fixed capacity";
    default: return "unknown status";
  }
}

const char* ttg_last_error(void) { return g_err.c_str(); }

int64_t ttg_kernel_launches(void) { return g_launches.load(); }

void ttg_free(ttg_tensor* t)
{
  if (!t || !t->owned)
    return;
  std::free(t->ranks);
  std::free(t->rows);
  std::free(t->cols);
  std::free(t->offsets);
  std::free(t->data);
  std::memset(t, 0, sizeof(*t));
}

int32_t ttg_plan_create_round(int32_t count, const ttg_tensor* ins, const ttg_round_options* opts,
                              ttg_plan** plan)
{
  g_err.clear();
  if (!plan || count < 0 || (count > 0 && !ins))
    return fail(TTG_ERR_ARG, "ttg_plan_create_round: bad arguments");
  if (int32_t st = need_device())
    return st;
  auto* P = new ttg_plan;
  const int32_t st = build_round_plan(*P, count, ins, opts, "round");
  if (st)
  {
    delete P;
    return st;
  }
  *plan = P;
  return TTG_OK;
}

static int32_t eval_upload(ttg_plan& P, cudaStream_t st);

int32_t ttg_plan_upload(ttg_plan* P, void* stream)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  if (P->kind == kPlanEval)
    return eval_upload(*P, static_cast<cudaStream_t>(stream));
  return plan_upload(*P, static_cast<cudaStream_t>(stream));
}

int32_t ttg_plan_run(ttg_plan* P, void* stream)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  if (P->gexec)
  {
    TTG_CUDA(cudaGraphLaunch(P->gexec, static_cast<cudaStream_t>(stream)));
    g_launches += P->graph_launches;
    return TTG_OK;
  }
  return plan_run(*P, static_cast<cudaStream_t>(stream));
}

// Autotuner: times each launch configuration of the plan's sweep on the
// plan itself (every run restarts from the pristine inputs) and keeps the
// fastest.  Per-TT schedule: one CTA per SM with 200 KB of shared staging,
// or two per SM with 92 KB each.  Whole-GPU schedule: Jacobi block widths
// 2, 4 and 8 columns, and the per-TT schedule as a contender.
int32_t ttg_plan_autotune(ttg_plan* P, void* stream, int32_t* choice)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  if (choice)
    *choice = 0;
  if (P->kind == kPlanEval || P->order.empty() || P->job_kind < 0)
    return TTG_OK;
  P->drop_graph();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sms = std::max(device().sms, 1);
  const int items = static_cast<int>(P->order.size());
  struct Cand
  {
    int code;  // 1/2: per TT, CTAs per SM; 100 + b (+ 1000 with tensor cores): whole GPU
    bool wide;
    int grid, smem, jblock, tc, cps, teams = 1;
  };
  std::vector<Cand> cands;
  const int g1 = std::max(1, std::min(items, sms)), g2 = std::max(1, std::min(items, 2 * sms));
  cands.push_back({1, false, g1, kSmemOnePerSm, P->wjob.jblock, P->wjob.tc, 1});
  if (g2 > g1)
    cands.push_back({2, false, g2, kSmemTwoPerSm, P->wjob.jblock, P->wjob.tc, 2});
  const int g3 = std::max(1, std::min(items, 3 * sms)), g4 = std::max(1, std::min(items, 4 * sms));
  if (g3 > g2 && g3 <= P->scratch_ctas)
    cands.push_back({3, false, g3, kSmemThreePerSm, P->wjob.jblock, P->wjob.tc, 3});
  if (g4 > g3 && g4 <= P->scratch_ctas)
    cands.push_back({4, false, g4, kSmemFourPerSm, P->wjob.jblock, P->wjob.tc, 4});
  const bool can_wide = P->wide_grid > 0 && P->wjob.W != nullptr;
  const int teams0 = P->wide_teams;
  if (can_wide)
  {
    int64_t c_max = 1;
    for (int t : P->order)
      for (int k = 0; k < P->tts[t].d; ++k)
      {
        const CoreSlot& c = P->slots[P->tts[t].first + k];
        c_max = std::max<int64_t>(c_max, std::max(c.r, c.rp));
      }
    if (P->wide_teams_max <= 1)
    {
      // The sliced-BF16 tensor-core tiles are tried only when they were
      // opted into (TTG_WIDE_TENSOR_CORES=1): they are no faster on these
      // barrier-bound sweeps and carry ~1e-12 instead of FP64 rounding per
      // product, which reached 2.6e-10 on the d=40 rank-257 round.
      for (int tcv = 0; tcv <= (P->wjob.mixed && P->wjob.tc ? 1 : 0); ++tcv)
        for (int b : {2, 4, 8})
          if ((6 * c_max + 2) * b <= kSmemOnePerSm)
            cands.push_back({100 + b + 1000 * tcv, true, P->wide_grid, kSmemOnePerSm, b, tcv, 1, 1});
    }
    else
      for (int t : {4, 8, 16, 32})
        if (t <= P->wide_teams_max)
          cands.push_back({10000 + t, true, P->wide_grid, kSmemOnePerSm, P->wjob.jblock, 0, 1, t});
  }
  const bool wide0 = P->wide;
  const int grid0 = P->grid, smem0 = P->smem_doubles, jb0 = P->wjob.jblock, tc0 = P->wjob.tc,
            cps0 = P->cps;
  float best = 0.0f;
  int bi = -1;
  for (size_t i = 0; i < cands.size(); ++i)
  {
    const Cand& c = cands[i];
    P->wide = c.wide;
    P->grid = c.grid;
    P->smem_doubles = c.smem;
    P->wjob.jblock = c.jblock;
    P->wjob.tc = c.tc;
    P->cps = c.cps;
    P->wide_teams = c.teams;
    float ms = 0.0f;
    for (int rep = 0; rep < 2; ++rep)  // warm, then timed
    {
      TTG_CUDA(cudaEventRecord(P->ev0, st));
      if (int32_t e = plan_run(*P, st))
        return e;
      TTG_CUDA(cudaEventRecord(P->ev1, st));
      TTG_CUDA(cudaEventSynchronize(P->ev1));
      TTG_CUDA(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
    }
    if (P->wide)
    {
      std::vector<GridBar> bars(static_cast<size_t>(P->wide_teams));
      TTG_CUDA(cudaMemcpy(bars.data(), P->wjob.bar, sizeof(GridBar) * bars.size(),
                          cudaMemcpyDeviceToHost));
      for (const GridBar& bar : bars)
        if (bar.err)
          return fail(TTG_ERR_TIMEOUT, "autotune: a grid barrier wait timed out");
    }
    if (bi < 0 || ms < best)
    {
      best = ms;
      bi = static_cast<int>(i);
    }
  }
  if (bi < 0)
  {
    P->wide = wide0;
    P->grid = grid0;
    P->smem_doubles = smem0;
    P->wjob.jblock = jb0;
    P->wjob.tc = tc0;
    P->cps = cps0;
    P->wide_teams = teams0;
    return TTG_OK;
  }
  const Cand& c = cands[static_cast<size_t>(bi)];
  P->wide = c.wide;
  P->grid = c.grid;
  P->smem_doubles = c.smem;
  P->wjob.jblock = c.jblock;
  P->wjob.tc = c.tc;
  P->cps = c.cps;
  P->wide_teams = c.teams;
  if (choice)
    *choice = c.code;
  return TTG_OK;
}

int32_t ttg_plan_graph(ttg_plan* P, int32_t enable)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  P->drop_graph();
  if (!enable)
    return TTG_OK;
  // Capture on a private stream: the legacy default stream cannot capture,
  // and the instantiated graph launches on any stream.
  cudaStream_t cap = nullptr;
  TTG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  const int64_t l0 = g_launches.load();
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int32_t st = TTG_OK;
  if (e == cudaSuccess)
  {
    st = plan_run(*P, cap);
    const cudaError_t e2 = cudaStreamEndCapture(cap, &P->graph);
    if (st == TTG_OK && e2 != cudaSuccess)
      e = e2;
  }
  P->graph_launches = g_launches.load() - l0;
  g_launches -= P->graph_launches;  // capture launches nothing
  if (e == cudaSuccess && st == TTG_OK)
    e = cudaGraphInstantiate(&P->gexec, P->graph, 0);
  cudaStreamDestroy(cap);
  if (st != TTG_OK)
  {
    P->drop_graph();
    return st;
  }
  if (e != cudaSuccess)
  {
    P->drop_graph();
    cudaGetLastError();
    return fail(TTG_ERR_CUDA, std::string("plan graph capture: ") + cudaGetErrorString(e));
  }
  return TTG_OK;
}

int32_t ttg_plan_kernel_ms(ttg_plan* P, float* ms)
{
  if (!P || !ms)
    return fail(TTG_ERR_ARG, "plan_kernel_ms: null argument");
  if (!P->kernel_timed)
    return fail(TTG_ERR_ARG, "plan_kernel_ms: no sweep launch recorded");
  TTG_CUDA(cudaEventSynchronize(P->evk1));
  TTG_CUDA(cudaEventElapsedTime(ms, P->evk0, P->evk1));
  return TTG_OK;
}

int32_t ttg_plan_schedule(const ttg_plan* P)
{
  if (!P || P->order.empty() || P->job_kind < 0)
    return 0;
  if (!P->wide)
    return TTG_SCHED_PER_TT;
  return P->wide_teams > 1 ? TTG_SCHED_TEAMS : TTG_SCHED_WHOLE_GPU;
}

int32_t ttg_plan_io_bytes(const ttg_plan* P, int64_t* h2d, int64_t* d2h)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  if (h2d)
    *h2d = P->h2d;
  if (d2h)
    *d2h = P->d2h;
  return TTG_OK;
}

void ttg_plan_destroy(ttg_plan* P) { delete P; }

int32_t ttg_plan_download(ttg_plan* P, void* stream, ttg_tensor* outs, double* values,
                          ttg_round_result* results)
{
  if (!P)
    return fail(TTG_ERR_ARG, "null plan");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (P->kind == kPlanEval)
  {
    char* d = static_cast<char*>(P->dev.p);
    int bad = 0;
    TTG_CUDA(cudaMemcpyAsync(values, d + P->off_out, sizeof(double) * P->M,
                             cudaMemcpyDeviceToHost, st));
    TTG_CUDA(cudaMemcpyAsync(&bad, d + P->off_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    TTG_CUDA(cudaStreamSynchronize(st));
    if (bad)
      return fail(TTG_ERR_INDEX, "eval_at: idx out of range");
    return TTG_OK;
  }
  if (int32_t e = plan_download_raw(*P, st))
    return e;
  const char* h = static_cast<const char*>(P->host.p);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P->off_tts);
  for (size_t i = 0; i < P->out_tts.size(); ++i)
  {
    const int t = P->out_tts[i];
    const Shape& s = P->shapes[P->kind == kPlanRound ? t : 0];
    bool matrix = s.matrix;
    std::vector<int> mrow = s.m, ncol = s.n;
    if (P->kind != kPlanRound)
    {
      // apply-round: rows from the operator, cols from the operand.
      matrix = P->shapes[1].matrix;
      mrow = P->shapes[0].m;
      ncol = P->shapes[1].n;
    }
    if (outs)
      if (int32_t e = emit_tensor(*P, t, matrix, mrow, ncol, &outs[i]))
        return e;
    fill_result(T[t], 0.0f, results ? &results[i] : nullptr);
  }
  return first_bad_status(*P) ? fail(first_bad_status(*P), "sweep reported a device status")
                              : TTG_OK;
}

// --------------------------------------------------------------------------
// ALS / two-site DMRG rounding (round/tt_als.hpp:212-300,
// round/tt_dmrg.hpp:217-300, and their matvec/matmat variants): the start TT
// is chosen on the host exactly as the reference chooses it (warm start,
// SVD round, round_right_canonical or a random TT), then one CTA runs the
// sweeps on the device (kJobAls / kJobDmrg, iter_round_tt).
// --------------------------------------------------------------------------
struct TensorView
{
  std::vector<int32_t> ranks, rows, cols;
  std::vector<int64_t> offsets;
  ttg_tensor t{};
  // A view of s with its column modes folded into the row modes (the packed
  // 3-axis cores of a TT-matrix) when `pack`.
  TensorView(const Shape& s, bool pack)
  {
    ranks.assign(s.r.begin(), s.r.end());
    if (ranks.empty())
      ranks.push_back(1);
    for (int k = 0; k < s.d; ++k)
    {
      rows.push_back(pack ? s.mode(k) : s.m[k]);
      cols.push_back(s.n[k]);
      offsets.push_back(s.src_off[k]);
    }
    offsets.push_back(s.d > 0 ? s.src_off[s.d - 1] + s.size[s.d - 1] : 0);
    t.d = s.d;
    t.ranks = ranks.data();
    t.rows = rows.empty() ? nullptr : rows.data();
    t.cols = (s.matrix && !pack) ? cols.data() : nullptr;
    t.offsets = offsets.data();
    t.data = const_cast<double*>(s.data);
  }
};

struct OwnedTensor
{
  ttg_tensor t{};
  ~OwnedTensor() { ttg_free(&t); }
};

int max_rank_of(const ttg_tensor& t)
{
  int m = 0;
  for (int k = 0; k <= t.d; ++k)
    m = std::max(m, t.ranks[k]);
  return m;
}

// Bond capacities of the start TT in DMRG: a merged pair L Y_k Y_k1 R has
// rank <= Y's middle rank, and the split keeps at most max_rank and what the
// unfolding allows; the start TT's own ranks always fit.
std::vector<int> dmrg_caps(const Shape& Y, const std::vector<int>& rx, int max_rank)
{
  const int d = Y.d;
  std::vector<int> cap(static_cast<size_t>(d + 1), 1);
  std::vector<double> left(static_cast<size_t>(d + 1), 1.0), right(static_cast<size_t>(d + 1), 1.0);
  for (int k = 0; k < d; ++k)
    left[k + 1] = std::min(left[k] * Y.mode(k), 1e18);
  for (int k = d - 1; k >= 0; --k)
    right[k] = std::min(right[k + 1] * Y.mode(k), 1e18);
  for (int k = 1; k < d; ++k)
  {
    double c = std::min({static_cast<double>(Y.r[k]), left[k], right[k]});
    if (max_rank > 0)
      c = std::min(c, static_cast<double>(max_rank));
    cap[k] = std::max(rx[k], static_cast<int>(c));
  }
  return cap;
}

int32_t run_iter_engine(const Shape& Y, const ttg_tensor& X0, bool dmrg, bool rc, int max_rank,
                        double eps, int max_iters, double tol, ttg_tensor* out,
                        ttg_round_result* result, const char* op)
{
  Shape XS;
  if (int32_t st = describe(&X0, op, XS))
    return st;
  if (XS.d != Y.d)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": start TT has a different order");
  const int d = Y.d;
  std::vector<int> rx(XS.r.begin(), XS.r.end());
  const std::vector<int> cap = dmrg ? dmrg_caps(Y, rx, max_rank) : rx;
  std::vector<int> ry(Y.r.begin(), Y.r.end()), nm(static_cast<size_t>(d));
  for (int k = 0; k < d; ++k)
    nm[k] = Y.mode(k);
  int cmax = 1, rymax = 1;
  for (int k = 0; k <= d; ++k)
  {
    cmax = std::max(cmax, cap[k]);
    rymax = std::max(rymax, ry[k]);
  }
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_plan P;
  PoolLease lease(P);
  P.opts = ttg_round_options{};
  P.opts.eps = eps;
  P.opts.max_rank = max_rank;
  P.opts.method = dmrg ? TTG_METHOD_DMRG : TTG_METHOD_ALS;
  P.kind = kPlanRound;
  P.job_kind = dmrg ? kJobDmrg : kJobAls;
  P.iter_max = max_iters;
  P.iter_tol = tol;
  P.iter_rc = rc;
  // Y as a plain TT of its packed modes; X in slots of capacity cap_k n_k cap_k+1.
  Shape Yp = Y;
  if (Yp.matrix)
  {
    for (int k = 0; k < d; ++k)
    {
      Yp.m[k] = Y.mode(k);
      Yp.n[k] = 1;
    }
    Yp.matrix = false;
  }
  Shape Xp = XS;
  Xp.matrix = false;
  for (int k = 0; k < d; ++k)
  {
    Xp.m[k] = XS.mode(k);
    Xp.n[k] = 1;
  }
  P.shapes = {Yp, Xp};
  add_tensor(P, Yp, true, nullptr);
  std::vector<int64_t> xcap(static_cast<size_t>(d));
  for (int k = 0; k < d; ++k)
    xcap[k] = static_cast<int64_t>(cap[k]) * nm[k] * cap[k + 1];
  add_tensor(P, Xp, true, &xcap);
  // The pair's environments, spectra and capacities after the cores.
  const int64_t es = a32(static_cast<int64_t>(std::max(cmax, rymax)) * rymax);
  const int64_t tail = 1 + 2 * static_cast<int64_t>(d - 1) * cmax + 2 * (d - 1) + (d + 1);
  const int64_t env_off = P.arena_doubles;
  P.arena_doubles += a32(2 * static_cast<int64_t>(d + 1) * es + tail);
  P.tts[1].env_off = env_off;
  P.tts[1].env_stride = es;
  P.order = {0};
  P.a_idx = {0};
  P.b_idx = {1};
  P.out_idx = {1};
  P.out_tts = {1};
  P.scratch_stride = need_iter(d, ry.data(), nm.data(), cap.data(), dmrg);
  P.grid = 1;
  if (int32_t st = layout_and_alloc(P))
    return st;
  double* tailp = reinterpret_cast<double*>(static_cast<char*>(P.host.p) + P.off_arena) +
                  env_off + 2 * static_cast<int64_t>(d + 1) * es;
  std::memset(tailp, 0, sizeof(double) * static_cast<size_t>(tail));
  tailp[0] = cmax;
  for (int k = 0; k <= d; ++k)
    tailp[tail - (d + 1) + k] = cap[k];
  float ms = 0.0f;
  if (int32_t st = execute(P, &ms))
    return st;
  if (int32_t st = emit_tensor(P, 1, Y.matrix, Y.m, Y.n, out))
    return st;
  const char* h = static_cast<const char*>(P.host.p);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P.off_tts);
  if (result)
  {
    fill_result(T[1], ms, result);
    result->iters_run = T[1].iters_run;
    result->converged = T[1].iter_conv;
    result->final_resid = T[1].final_change;
  }
  if (int32_t bad = first_bad_status(P))
  {
    ttg_free(out);
    return fail(bad, std::string(op) + ": device status " + ttg_status_string(bad));
  }
  return TTG_OK;
}

bool warm_compatible(const ttg_tensor* w, const Shape& Y)
{
  if (!w || w->d != Y.d || (w->cols != nullptr) != Y.matrix)
    return false;
  for (int k = 0; k < Y.d; ++k)
  {
    if (!w->rows || w->rows[k] != Y.m[k])
      return false;
    if (Y.matrix && w->cols[k] != Y.n[k])
      return false;
  }
  return true;
}

// The reference's start-TT rules, then the device engine.  cold_random: the
// matvec/matmat variants (round/tt_matvec_als_round.hpp:88-95 and the
// DMRG/matmat ones) start from random(shape, max_rank, seed).
int32_t round_iter_impl(const ttg_tensor* in, const ttg_round_options* opts,
                        const ttg_iter_options* it, bool cold_random, ttg_tensor* out,
                        ttg_round_result* result, const char* op)
{
  const bool dmrg = opts->method == TTG_METHOD_DMRG;
  const char* nm = dmrg ? "dmrg_round" : "als_round";
  if (dmrg && (std::isnan(opts->eps) || opts->eps <= 0.0))
    return fail(TTG_ERR_ARG, std::string(nm) + ": eps must be > 0 for DMRG compression");
  if (!dmrg && std::isnan(opts->eps))
    return fail(TTG_ERR_ARG, std::string(nm) + ": eps is NaN; must be a valid number");
  if (opts->gauge != TTG_GAUGE_NONE)
    return fail(TTG_ERR_ARG, std::string(op) + ": gauge is an svd-method option");
  if (opts->precision != TTG_PREC_FP64)
    return fail(TTG_ERR_METHOD, std::string(op) + ": ALS / DMRG run in FP64 only");
  const int max_iters = it && it->max_iters > 0 ? it->max_iters : 20;
  const double tol = it && it->tol > 0.0 ? it->tol : 1.0e-12;
  const uint64_t seed = it ? it->seed : 0;
  const ttg_tensor* warm = it ? it->warm : nullptr;
  Shape Y;
  if (int32_t st = describe(in, op, Y))
    return st;
  if (int32_t st = need_device())
    return st;
  ttg_round_options svd{};
  svd.eps = opts->eps;
  svd.max_rank = opts->max_rank;
  svd.method = TTG_METHOD_SVD;
  svd.max_sweeps = opts->max_sweeps;
  if (Y.d <= 1)
  {
    // d <= 1: the SVD round (tt_als.hpp:222-228, tt_dmrg.hpp:226-232).
    if (int32_t st = ttg_round(in, &svd, out, nullptr))
      return st;
    if (result)
    {
      std::memset(result, 0, sizeof(*result));
      result->converged = 1;
    }
    return TTG_OK;
  }
  const bool wc = warm_compatible(warm, Y);
  int max_rank = opts->max_rank;
  OwnedTensor ref, start;
  const ttg_tensor* X0 = nullptr;
  bool rc = false;
  TensorView packed(Y, true);
  if (!dmrg && max_rank <= 0)
  {
    if (opts->eps <= 0.0)
      return fail(TTG_ERR_ARG, std::string(nm) + ": max_rank <= 0 and eps <= 0; ALS requires "
                               "either max_rank > 0 or eps > 0 to determine compression target");
    if (int32_t st = ttg_round(&packed.t, &svd, &ref.t, nullptr))
      return st;
    max_rank = max_rank_of(ref.t);
    if (!wc)
      X0 = &ref.t;
  }
  if (wc)
  {
    // (ALS always has a max_rank here: given, or taken from the SVD round.)
    if (max_rank > 0)
      for (int k = 0; k <= warm->d; ++k)
        if (warm->ranks[k] > max_rank)
          return fail(TTG_ERR_ARG, std::string(nm) + ": warm_start max rank " +
                                       std::to_string(warm->ranks[k]) + " exceeds max_rank " +
                                       std::to_string(max_rank));
    X0 = warm;
  }
  if (!X0)
  {
    if (cold_random && (!dmrg || max_rank > 0))
    {
      if (int32_t st = ttg_host_random(Y.d, packed.rows.data(), nullptr, max_rank, seed, 0,
                                       &start.t))
        return fail(st, ttg_host_last_error());
    }
    else
    {
      ttg_round_options rco{};
      rco.eps = dmrg ? opts->eps : 0.0;
      rco.max_rank = max_rank;
      rco.method = TTG_METHOD_SVD;
      rco.gauge = TTG_GAUGE_RIGHT_CANONICAL;
      rco.max_sweeps = opts->max_sweeps;
      if (int32_t st = ttg_round(&packed.t, &rco, &start.t, nullptr))
        return st;
      rc = true;
    }
    X0 = &start.t;
  }
  // A warm start of a TT-matrix arrives with its 4-axis modes: view it packed.
  Shape W;
  if (int32_t st = describe(X0, op, W))
    return st;
  TensorView xview(W, true);
  return run_iter_engine(Y, xview.t, dmrg, rc, max_rank, opts->eps, max_iters, tol, out,
                         result, op);
}

// Host-side phase times of one batch call, printed to stderr when the
// environment sets TTG_TRACE (diagnostics only: with it set, each phase
// ends with a stream synchronize so that its time is its own).
struct CallTrace
{
  bool on = std::getenv("TTG_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  std::string line;
  void mark(const char* phase, cudaStream_t st = nullptr)
  {
    if (!on)
      return;
    if (st)
      cudaStreamSynchronize(st);
    const auto now = std::chrono::steady_clock::now();
    char buf[64];
    std::snprintf(buf, sizeof(buf), " %s=%.2fms", phase,
                  std::chrono::duration<double, std::milli>(now - t).count());
    line += buf;
    t = now;
  }
  void print(const char* op, int32_t count)
  {
    if (on)
      std::fprintf(stderr, "ttg_trace %s count=%d%s\n", op, count, line.c_str());
  }
};

// Outputs and results of a finished round plan; orig maps the plan's TT t
// to its index in the caller's arrays (null: the same).
static int32_t unpack_round(ttg_plan& P, const int32_t* orig, ttg_tensor* outs,
                            ttg_round_result* results, float ms)
{
  const char* h = static_cast<const char*>(P.host.p);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P.off_tts);
  const int64_t n = static_cast<int64_t>(P.shapes.size());
  return parallel_for(n, [&](int64_t ii) -> int32_t {
    const int t = static_cast<int>(ii);
    const int i = orig ? orig[t] : t;
    const Shape& s = P.shapes[t];
    if (s.d <= 1)
    {
      if (int32_t e = copy_through(s, &outs[i]))
        return e;
      if (results)
      {
        std::memset(&results[i], 0, sizeof(results[i]));
        results[i].iters_run = 1;
        results[i].converged = 1;
      }
      return TTG_OK;
    }
    if (int32_t e = emit_tensor(P, t, s.matrix, s.m, s.n, &outs[i]))
      return e;
    fill_result(T[t], ms, results ? &results[i] : nullptr);
    return TTG_OK;
  });
}

// A large batch with host buffers runs as a pipeline of plans whose host and
// device phases overlap: chunk c + 1 is packed and uploaded while chunk c
// sweeps, and chunk c is downloaded and unpacked while chunk c + 1 sweeps.
// Two chunks are in flight at a time, each on its own stream with its own
// pooled buffers (chunk c takes slot c % 2 once chunk c - 2 has been
// unpacked); chunk c + 1's CTAs take the SMs that chunk c's last TTs free.
// The chunks split the batch by estimated sweep cost (largest first, each TT
// to the lightest chunk) so that the sweeps take about as long; the first
// pack and the last unpack, a chunk each, are all that stays exposed.
constexpr int32_t kPipelineMinBatch = 1024;

static int32_t round_batch_pipelined(int32_t count, const ttg_tensor* ins,
                                     const ttg_round_options* opts, ttg_tensor* outs,
                                     ttg_round_result* results, const char* op,
                                     const std::vector<double>& cost)
{
  const int nch = std::max(2, std::min(4, count / kPipelineMinBatch));
  std::vector<int32_t> order(static_cast<size_t>(count));
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
  struct Chunk
  {
    std::vector<int32_t> part;
    std::vector<ttg_tensor> in;
    double load = 0.0;
    ttg_plan P;
    std::unique_ptr<PoolLease> lease;
  };
  std::vector<std::unique_ptr<Chunk>> ch;
  for (int c = 0; c < nch; ++c)
    ch.push_back(std::make_unique<Chunk>());
  for (int32_t i : order)
  {
    int c = 0;
    for (int j = 1; j < nch; ++j)
      if (ch[j]->load < ch[c]->load)
        c = j;
    ch[c]->part.push_back(i);
    ch[c]->in.push_back(ins[i]);
    ch[c]->load += cost[i];
  }
  CallTrace trace;
  const cudaStream_t st[2] = {lib_stream(), lib_stream2()};
  auto launch = [&](int c) -> int32_t {
    Chunk& k = *ch[c];
    k.lease = std::make_unique<PoolLease>(k.P, c & 1);
    if (int32_t e = build_round_plan(k.P, static_cast<int32_t>(k.in.size()), k.in.data(), opts, op))
      return e;
    trace.mark("pack");
    if (int32_t e = plan_upload(k.P, st[c & 1]))
      return e;
    TTG_CUDA(cudaEventRecord(k.P.ev0, st[c & 1]));
    if (int32_t e = plan_run(k.P, st[c & 1]))
      return e;
    TTG_CUDA(cudaEventRecord(k.P.ev1, st[c & 1]));
    return TTG_OK;
  };
  auto finish = [&](int c) -> int32_t {
    Chunk& k = *ch[c];
    if (int32_t e = plan_download_raw(k.P, st[c & 1]))
      return e;
    trace.mark("sweep+d2h");
    float ms = 0.0f;
    TTG_CUDA(cudaEventElapsedTime(&ms, k.P.ev0, k.P.ev1));
    if (int32_t e = unpack_round(k.P, k.part.data(), outs, results, ms))
      return e;
    trace.mark("unpack");
    const int32_t bad = first_bad_status(k.P);
    k.lease.reset();  // the slot's buffers back to the pool for chunk c + 2
    if (bad)
      return fail(bad, std::string(op) + ": device status " + ttg_status_string(bad));
    return TTG_OK;
  };
  auto run_all = [&]() -> int32_t {
    for (int c = 0; c < std::min(nch, 2); ++c)
      if (int32_t e = launch(c))
        return e;
    for (int c = 0; c < nch; ++c)
    {
      if (int32_t e = finish(c))
        return e;
      if (c + 2 < nch)
        if (int32_t e = launch(c + 2))
          return e;
    }
    return TTG_OK;
  };
  const int32_t e = run_all();
  if (e)
  {
    // Nothing of a chunk still in flight may outlive its buffers' return
    // to the pool.
    cudaStreamSynchronize(st[0]);
    cudaStreamSynchronize(st[1]);
    return e;
  }
  trace.print(op, count);
  return TTG_OK;
}

static int32_t round_common(int32_t count, const ttg_tensor* ins, const ttg_round_options* opts,
                            ttg_tensor* outs, ttg_round_result* results, const char* op)
{
  g_err.clear();
  if (count < 0 || (count > 0 && (!ins || !outs)))
    return fail(TTG_ERR_ARG, std::string(op) + ": bad arguments");
  if (int32_t st = check_opts(opts, op))
    return st;
  if (opts->method == TTG_METHOD_ALS || opts->method == TTG_METHOD_DMRG)
  {
    if (count != 1)
      return fail(TTG_ERR_METHOD, std::string(op) + ": ALS / DMRG are served for one tensor "
                                                    "at a time (ttg_round, ttg_round_iter)");
    return round_iter_impl(ins, opts, nullptr, false, outs, results, op);
  }
  if (opts->method != TTG_METHOD_SVD && opts->method != TTG_METHOD_SKETCH)
    return fail(TTG_ERR_METHOD, std::string(op) +
                                    ": round_method::svd_streaming / svd_naive are only valid on "
                                    "matvec_round / matmat_round respectively.");
  // Shapes first: an invalid tensor is an argument error with or without a
  // device (the reference aborts on it before any arithmetic).
  std::vector<double> cost(static_cast<size_t>(count), 0.0);
  for (int32_t i = 0; i < count; ++i)
  {
    Shape s;
    if (int32_t st = describe(&ins[i], op, s))
      return st;
    for (int k = 0; k < s.d; ++k)  // ~ flops of the step at core k
      cost[i] += static_cast<double>(s.r[k]) * s.mode(k) * s.r[k + 1] * std::max(s.r[k], s.r[k + 1]);
  }
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  if (count >= kPipelineMinBatch && opts->method == TTG_METHOD_SVD && !opts->bond_stats &&
      (opts->schedule == TTG_SCHED_AUTO || opts->schedule == TTG_SCHED_PER_TT))
    return round_batch_pipelined(count, ins, opts, outs, results, op, cost);
  CallTrace trace;
  ttg_plan P;
  PoolLease lease(P);
  if (int32_t st = build_round_plan(P, count, ins, opts, op))
    return st;
  trace.mark("plan+pack");
  float ms = 0.0f;
  if (trace.on)
  {
    cudaStream_t st = lib_stream();
    if (int32_t e = plan_upload(P, st))
      return e;
    trace.mark("h2d", st);
    TTG_CUDA(cudaEventRecord(P.ev0, st));
    if (int32_t e = plan_run(P, st))
      return e;
    TTG_CUDA(cudaEventRecord(P.ev1, st));
    trace.mark("run", st);
    if (int32_t e = plan_download_raw(P, st))
      return e;
    trace.mark("d2h", st);
    TTG_CUDA(cudaEventElapsedTime(&ms, P.ev0, P.ev1));
  }
  else if (int32_t st = execute(P, &ms))
    return st;
  const int32_t est = unpack_round(P, nullptr, outs, results, ms);
  trace.mark("unpack");
  trace.print(op, count);
  if (est)
    return est;
  if (int32_t bad = first_bad_status(P))
    return fail(bad, std::string(op) + ": device status " + ttg_status_string(bad));
  return TTG_OK;
}

int32_t ttg_round(const ttg_tensor* in, const ttg_round_options* opts, ttg_tensor* out,
                  ttg_round_result* result)
{
  return round_common(1, in, opts, out, result, "round");
}

int32_t ttg_round_batch(int32_t count, const ttg_tensor* ins, const ttg_round_options* opts,
                        ttg_tensor* outs, ttg_round_result* results)
{
  return round_common(count, ins, opts, outs, results, "round_batch");
}

int32_t ttg_right_orthogonalize(const ttg_tensor* in, ttg_tensor* out)
{
  g_err.clear();
  if (!in || !out)
    return fail(TTG_ERR_ARG, "right_orthogonalize: null argument");
  {
    Shape s;
    if (int32_t st = describe(in, "right_orthogonalize", s))
      return st;
  }
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_round_options o{};
  ttg_plan P;
  if (int32_t st = build_round_plan(P, 1, in, &o, "right_orthogonalize", kJobRightOrth))
    return st;
  if (P.shapes[0].d <= 1)
    return copy_through(P.shapes[0], out);
  float ms = 0.0f;
  if (int32_t st = execute(P, &ms))
    return st;
  return emit_tensor(P, 0, P.shapes[0].matrix, P.shapes[0].m, P.shapes[0].n, out);
}

// detail::left_orthogonalize (gauge/tt_orthogonalize.hpp:39-58): the L->R
// QR sweep, cores 0..d-2 left-orthogonal.
int32_t ttg_left_orthogonalize(const ttg_tensor* in, ttg_tensor* out)
{
  g_err.clear();
  if (!in || !out)
    return fail(TTG_ERR_ARG, "left_orthogonalize: null argument");
  {
    Shape s;
    if (int32_t st = describe(in, "left_orthogonalize", s))
      return st;
  }
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_round_options o{};
  ttg_plan P;
  if (int32_t st = build_round_plan(P, 1, in, &o, "left_orthogonalize", kJobLeftOrth))
    return st;
  if (P.shapes[0].d <= 1)
    return copy_through(P.shapes[0], out);
  float ms = 0.0f;
  if (int32_t st = execute(P, &ms))
    return st;
  return emit_tensor(P, 0, P.shapes[0].matrix, P.shapes[0].m, P.shapes[0].n, out);
}

// soft_threshold (round/tt_soft_threshold.hpp:42-178).  d <= 1 or
// tau <= 0 return a copy of the input, as the reference does; otherwise one
// CTA sweeps the TT: right_orthogonalize, then the soft step of every bond
// right to left (job kind kJobSoftThreshold, tau in the job's eps).
int32_t ttg_soft_threshold(const ttg_tensor* in, double tau, ttg_tensor* out)
{
  g_err.clear();
  if (!in || !out)
    return fail(TTG_ERR_ARG, "soft_threshold: null argument");
  if (std::isnan(tau))
    return fail(TTG_ERR_ARG, "soft_threshold: tau is NaN");
  Shape s;
  if (int32_t st = describe(in, "soft_threshold", s))
    return st;
  if (s.matrix)
    return fail(TTG_ERR_ARG, "soft_threshold: takes a tt, not a tt_matrix");
  if (s.d <= 1 || tau <= 0.0)
    return copy_through(s, out);
  for (int k = 1; k < s.d; ++k)
    if (static_cast<int64_t>(s.r[k - 1]) * s.mode(k - 1) > INT32_MAX ||
        static_cast<int64_t>(s.mode(k)) * s.r[k + 1] > INT32_MAX)
      return fail(TTG_ERR_SHAPE, "soft_threshold: dimension product exceeds INT_MAX");
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_round_options o{};
  o.eps = tau;
  o.precision = TTG_PREC_FP64;
  o.schedule = TTG_SCHED_PER_TT;
  ttg_plan P;
  PoolLease lease(P);
  if (int32_t st = build_round_plan(P, 1, in, &o, "soft_threshold", kJobSoftThreshold))
    return st;
  float ms = 0.0f;
  if (int32_t st = execute(P, &ms))
    return st;
  if (int32_t bad = first_bad_status(P))
    return fail(bad, std::string("soft_threshold: device status ") + ttg_status_string(bad));
  return emit_tensor(P, 0, false, s.m, s.n, out);
}

// ---------------------------------------------------------------------------
// Apply and apply-round.
// ---------------------------------------------------------------------------
static int32_t check_apply(const Shape& A, const Shape& X, bool matmat, const char* op)
{
  if (!A.matrix)
    return fail(TTG_ERR_ARG, std::string(op) + ": operator must be a TT-matrix");
  if (matmat != X.matrix)
    return fail(TTG_ERR_ARG, std::string(op) + ": operand kind mismatch");
  if (A.d != X.d)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": d mismatch (a.d=" + std::to_string(A.d) +
                                   ", x.d=" + std::to_string(X.d) + ")");
  for (int k = 0; k < A.d; ++k)
    if (A.n[k] != X.m[k])
      return fail(TTG_ERR_SHAPE, std::string(op) + ": mode-size mismatch at axis " +
                                     std::to_string(k));
  return TTG_OK;
}

// Plan with A, X uploaded and the product TT computed by apply kernels;
// when `round` the product is then rounded (gauge none).
static int32_t build_apply_plan(ttg_plan& P, const Shape& A, const Shape& X, bool round,
                                const ttg_round_options* opts)
{
  P.kind = kPlanMatvecNaive;
  if (opts)
    P.opts = *opts;
  P.shapes = {A, X};
  add_tensor(P, A, true, nullptr);
  add_tensor(P, X, true, nullptr);
  const int d = A.d;
  const int nout_all = 1;
  (void)nout_all;
  Shape Y;
  Y.d = d;
  Y.matrix = X.matrix;
  Y.r.resize(d + 1);
  for (int k = 0; k <= d; ++k)
    Y.r[k] = A.r[k] * X.r[k];
  for (int k = 0; k < d; ++k)
  {
    Y.m.push_back(A.m[k]);
    Y.n.push_back(X.n[k]);
    Y.size.push_back(static_cast<int64_t>(Y.r[k]) * Y.mode(k) * Y.r[k + 1]);
    Y.src_off.push_back(0);
  }
  const int y = add_tensor(P, Y, false, nullptr);
  for (int k = 0; k < d; ++k)
  {
    ttg_plan::Apply ap{};
    ap.a_slot = P.tts[0].first + k;
    ap.x_slot = P.tts[1].first + k;
    ap.y_slot = P.tts[y].first + k;
    ap.r = A.r[k];
    ap.m = A.m[k];
    ap.p = A.n[k];
    ap.rp = A.r[k + 1];
    ap.s = X.r[k];
    ap.nout = X.n[k];
    ap.sp = X.r[k + 1];
    P.applies.push_back(ap);
  }
  P.out_tts = {y};
  P.job_kind = round ? kJobRound : -1;
  if (round && d > 1)
  {
    P.order = {y};
    P.scratch_stride = round_need(Y, kJobRound);
  }
  else
  {
    P.scratch_stride = 64;
  }
  P.grid = 1;
  // The product shape has no host data; layout_and_alloc copies only A, X.
  Shape* keep = &P.shapes[0];
  (void)keep;
  return TTG_OK;
}

static int32_t build_stream_plan(ttg_plan& P, const Shape& A, const Shape& X,
                                 const ttg_round_options* opts)
{
  P.kind = kPlanStream;
  P.opts = *opts;
  P.shapes = {A, X};
  add_tensor(P, A, true, nullptr);
  add_tensor(P, X, true, nullptr);
  const int d = A.d;
  Shape Y;
  Y.d = d;
  Y.matrix = X.matrix;
  Y.r.resize(d + 1);
  for (int k = 0; k <= d; ++k)
    Y.r[k] = A.r[k] * X.r[k];
  std::vector<int64_t> caps;
  for (int k = 0; k < d; ++k)
  {
    Y.m.push_back(A.m[k]);
    Y.n.push_back(X.n[k]);
    Y.size.push_back(static_cast<int64_t>(Y.r[k]) * Y.mode(k) * Y.r[k + 1]);
    Y.src_off.push_back(0);
  }
  const int y = add_tensor(P, Y, false, nullptr);
  P.out_tts = {y};
  P.job_kind = X.matrix ? kJobStreamMatmat : kJobStreamMatvec;
  P.order = {0};
  P.a_idx = {0};
  P.b_idx = {1};
  P.out_idx = {y};
  P.scratch_stride = stream_need(A, X);
  P.grid = 1;
  return TTG_OK;
}

static int32_t apply_round_common(const ttg_tensor* a, const ttg_tensor* x,
                                  const ttg_round_options* opts, ttg_tensor* out,
                                  ttg_round_result* result, bool matmat, int mode, const char* op)
{
  // mode: 0 = raw apply, 1 = apply then round (naive), 2 = streaming.
  g_err.clear();
  if (!out)
    return fail(TTG_ERR_ARG, std::string(op) + ": null output");
  Shape A, X;
  if (int32_t st = describe(a, op, A))
    return st;
  if (int32_t st = describe(x, op, X))
    return st;
  if (A.d != X.d)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": core count mismatch " + std::to_string(A.d) +
                                   " vs " + std::to_string(X.d));
  if (A.d > 0)
    if (int32_t st = check_apply(A, X, matmat, op))
      return st;
  if (int32_t st = need_device())
    return st;
  if (A.d == 0)
  {
    std::memset(out, 0, sizeof(*out));
    out->owned = 1;
    out->ranks = static_cast<int32_t*>(std::malloc(sizeof(int32_t)));
    out->offsets = static_cast<int64_t*>(std::malloc(sizeof(int64_t)));
    out->ranks[0] = 1;
    out->offsets[0] = 0;
    if (result)
    {
      std::memset(result, 0, sizeof(*result));
      result->iters_run = 1;
      result->converged = 1;
    }
    return TTG_OK;
  }
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_plan P;
  PoolLease lease(P);
  int32_t st = (mode == 2) ? build_stream_plan(P, A, X, opts)
                           : build_apply_plan(P, A, X, mode == 1, opts);
  if (st)
    return st;
  // Only A and X carry host data: trim the shapes list for the upload.
  std::vector<Shape> all = P.shapes;
  if ((st = layout_and_alloc(P)))
    return st;
  float ms = 0.0f;
  if ((st = execute(P, &ms)))
    return st;
  const int y = P.out_tts[0];
  if ((st = emit_tensor(P, y, X.matrix, A.m, X.n, out)))
    return st;
  const char* h = static_cast<const char*>(P.host.p);
  const TTInfo* T = reinterpret_cast<const TTInfo*>(h + P.off_tts);
  fill_result(T[y], ms, result);
  if (int32_t bad = first_bad_status(P))
    return fail(bad, std::string(op) + ": device status " + ttg_status_string(bad));
  return TTG_OK;
}

// matvec/matmat ALS and DMRG rounding (round/tt_matvec_als_round.hpp,
// tt_matvec_dmrg_round.hpp, tt_matmat_als_round.hpp, tt_matmat_dmrg_round.hpp):
// the raw product on the device, then the iterative rounder started from a
// random TT (the SVD round when ALS has no max_rank).
static int32_t apply_round_iter(const ttg_tensor* A, const ttg_tensor* x,
                                const ttg_round_options* opts, const ttg_iter_options* it,
                                ttg_tensor* out, ttg_round_result* result, bool matmat,
                                const char* op)
{
  if (!out)
    return fail(TTG_ERR_ARG, std::string(op) + ": null output");
  OwnedTensor prod;
  if (int32_t st = apply_round_common(A, x, nullptr, &prod.t, nullptr, matmat, 0, op))
    return st;
  return round_iter_impl(&prod.t, opts, it, true, out, result, op);
}

int32_t ttg_round_iter(const ttg_tensor* in, const ttg_round_options* opts,
                       const ttg_iter_options* iter, ttg_tensor* out, ttg_round_result* result)
{
  g_err.clear();
  if (!out)
    return fail(TTG_ERR_ARG, "round_iter: null output");
  if (int32_t st = check_opts(opts, "round_iter"))
    return st;
  if (opts->method != TTG_METHOD_ALS && opts->method != TTG_METHOD_DMRG)
    return fail(TTG_ERR_METHOD, "round_iter: method must be als or dmrg");
  return round_iter_impl(in, opts, iter, false, out, result, "round_iter");
}

int32_t ttg_apply_round_iter(const ttg_tensor* A, const ttg_tensor* x,
                             const ttg_round_options* opts, const ttg_iter_options* iter,
                             ttg_tensor* out, ttg_round_result* result)
{
  g_err.clear();
  if (!A || !x)
    return fail(TTG_ERR_ARG, "apply_round_iter: null tensor");
  if (int32_t st = check_opts(opts, "apply_round_iter"))
    return st;
  if (opts->method != TTG_METHOD_ALS && opts->method != TTG_METHOD_DMRG)
    return fail(TTG_ERR_METHOD, "apply_round_iter: method must be als or dmrg");
  return apply_round_iter(A, x, opts, iter, out, result, x->cols != nullptr, "apply_round_iter");
}

int32_t ttg_matvec_round(const ttg_tensor* A, const ttg_tensor* x, const ttg_round_options* opts,
                         ttg_tensor* out, ttg_round_result* result)
{
  g_err.clear();
  if (int32_t st = check_opts(opts, "matvec_round"))
    return st;
  if (opts->method == TTG_METHOD_SVD_NAIVE)
    return fail(TTG_ERR_METHOD, "matvec_round: round_method::svd_naive is matmat-only");
  if (opts->method == TTG_METHOD_SKETCH)
    return fail(TTG_ERR_METHOD, "matvec_round: the sketch method serves round() only");
  if (opts->gauge != TTG_GAUGE_NONE)
    return fail(TTG_ERR_ARG, "matvec_round: gauge is a round() option");
  if (opts->method == TTG_METHOD_ALS || opts->method == TTG_METHOD_DMRG)
    return apply_round_iter(A, x, opts, nullptr, out, result, false, "matvec_round");
  const bool streaming = opts->method == TTG_METHOD_SVD_STREAMING && A && A->d > 1;
  return apply_round_common(A, x, opts, out, result, false, streaming ? 2 : 1, "matvec_round");
}

int32_t ttg_matmat_round(const ttg_tensor* A, const ttg_tensor* B, const ttg_round_options* opts,
                         ttg_tensor* out, ttg_round_result* result)
{
  g_err.clear();
  if (int32_t st = check_opts(opts, "matmat_round"))
    return st;
  if (opts->method == TTG_METHOD_SVD_STREAMING)
    return fail(TTG_ERR_METHOD, "matmat_round: round_method::svd_streaming is matvec-only");
  if (opts->method == TTG_METHOD_SKETCH)
    return fail(TTG_ERR_METHOD, "matmat_round: the sketch method serves round() only");
  if (opts->gauge != TTG_GAUGE_NONE)
    return fail(TTG_ERR_ARG, "matmat_round: gauge is a round() option");
  if (opts->method == TTG_METHOD_ALS || opts->method == TTG_METHOD_DMRG)
    return apply_round_iter(A, B, opts, nullptr, out, result, true, "matmat_round");
  const bool streaming = opts->method == TTG_METHOD_SVD && A && A->d > 1;
  return apply_round_common(A, B, opts, out, result, true, streaming ? 2 : 1, "matmat_round");
}

int32_t ttg_matvec(const ttg_tensor* A, const ttg_tensor* x, ttg_tensor* out)
{
  return apply_round_common(A, x, nullptr, out, nullptr, false, 0, "matvec");
}

int32_t ttg_matmat(const ttg_tensor* A, const ttg_tensor* B, ttg_tensor* out)
{
  return apply_round_common(A, B, nullptr, out, nullptr, true, 0, "matmat");
}

// frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98): the
// product cores (matvec_core, or matmat_core packed as 3-axis cores of mode
// m*n) are formed in the arena by the apply kernels, then one CTA runs the
// contract_inner_step chain of the product with itself.  The product stays
// on the device (the reference avoids holding it for host-memory reasons;
// it is sum_k r_k^A r_k^x m_k r_{k+1}^A r_{k+1}^x doubles of HBM here).
int32_t ttg_frob_norm_apply(const ttg_tensor* a, const ttg_tensor* x, double* out)
{
  g_err.clear();
  const char* op = "frob_norm_apply";
  if (!out)
    return fail(TTG_ERR_ARG, std::string(op) + ": null output");
  Shape A, X;
  if (int32_t st = describe(a, op, A))
    return st;
  if (int32_t st = describe(x, op, X))
    return st;
  if (A.d != X.d)
    return fail(TTG_ERR_SHAPE, std::string(op) + ": d mismatch (a.d=" + std::to_string(A.d) +
                                   ", x.d=" + std::to_string(X.d) + ")");
  if (A.d == 0)
  {
    *out = 0.0;
    return TTG_OK;
  }
  if (int32_t st = check_apply(A, X, X.matrix, op))
    return st;
  for (int k = 0; k < A.d; ++k)
    if (static_cast<int64_t>(A.m[k]) * (X.matrix ? X.n[k] : 1) > INT32_MAX)
      return fail(TTG_ERR_SHAPE, std::string(op) + ": m*n product exceeds INT_MAX");
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_plan P;
  PoolLease lease(P);
  if (int32_t st = build_apply_plan(P, A, X, false, nullptr))
    return st;
  const TTInfo ty = P.tts[P.out_tts[0]];
  int64_t env = 1, tmp = 1;
  for (int k = 0; k < ty.d; ++k)
  {
    const CoreSlot& c = P.slots[ty.first + k];
    env = std::max(env, static_cast<int64_t>(c.r) * c.r);
    env = std::max(env, static_cast<int64_t>(c.rp) * c.rp);
    tmp = std::max(tmp, static_cast<int64_t>(c.r) * c.n * c.rp);
  }
  env = a32(env);
  P.scratch_stride = 2 * env + a32(tmp) + 32;
  if (int32_t st = layout_and_alloc(P))
    return st;
  cudaStream_t st = lib_stream();
  if (int32_t e = plan_upload(P, st))
    return e;
  if (int32_t e = plan_run(P, st))
    return e;
  char* d = static_cast<char*>(P.dev.p);
  double* scratch = reinterpret_cast<double*>(d + P.off_scratch);
  const CoreSlot* S = reinterpret_cast<const CoreSlot*>(d + P.off_slots);
  launch_inner(reinterpret_cast<double*>(d + P.off_arena), S + ty.first, S + ty.first, ty.d,
               scratch, env, scratch + P.scratch_stride - 8, st);
  g_launches += 1;
  TTG_CUDA(cudaGetLastError());
  double v = 0.0;
  TTG_CUDA(cudaMemcpyAsync(&v, scratch + P.scratch_stride - 8, sizeof(double),
                           cudaMemcpyDeviceToHost, st));
  TTG_CUDA(cudaStreamSynchronize(st));
  *out = std::sqrt(std::max(v, 0.0));
  return TTG_OK;
}

int32_t ttg_plan_create_matvec_round(const ttg_tensor* a, const ttg_tensor* x,
                                     const ttg_round_options* opts, ttg_plan** plan)
{
  g_err.clear();
  if (!plan)
    return fail(TTG_ERR_ARG, "null plan");
  if (int32_t st = check_opts(opts, "matvec_round"))
    return st;
  if (opts->method == TTG_METHOD_SVD_NAIVE)
    return fail(TTG_ERR_METHOD, "matvec_round: round_method::svd_naive is matmat-only");
  if (int32_t st = need_device())
    return st;
  Shape A, X;
  if (int32_t st = describe(a, "matvec_round", A))
    return st;
  if (int32_t st = describe(x, "matvec_round", X))
    return st;
  if (A.d < 2)
    return fail(TTG_ERR_SHAPE, "plan: matvec_round plans need d >= 2");
  if (int32_t st = check_apply(A, X, false, "matvec_round"))
    return st;
  auto* P = new ttg_plan;
  int32_t st = (opts->method == TTG_METHOD_SVD_STREAMING) ? build_stream_plan(*P, A, X, opts)
                                                          : build_apply_plan(*P, A, X, true, opts);
  if (!st)
    st = layout_and_alloc(*P);
  if (st)
  {
    delete P;
    return st;
  }
  *plan = P;
  return TTG_OK;
}

// ---------------------------------------------------------------------------
// eval_batch, inner, norm.
// ---------------------------------------------------------------------------
static int32_t build_eval_plan(ttg_plan& P, const ttg_tensor* a, const int32_t* idx, int32_t M)
{
  Shape s;
  if (int32_t st = describe(a, "eval_batch", s))
    return st;
  if (s.matrix)
    return fail(TTG_ERR_ARG, "eval_batch: expects a TT");
  if (!idx && M > 0)
    return fail(TTG_ERR_ARG, "eval_batch: idx pointer is null with M=" + std::to_string(M) +
                                 " > 0");
  if (M < 0)
    return fail(TTG_ERR_ARG, "eval_batch: M must be non-negative (got " + std::to_string(M) + ")");
  if (s.d == 0)
    return fail(TTG_ERR_EMPTY, "eval_batch: TT is empty (d=0)");
  P.kind = kPlanEval;
  P.shapes = {s};
  add_tensor(P, s, true, nullptr);
  P.M = M;
  P.eval_idx = idx;
  int rmax = 1;
  for (int k = 0; k <= s.d; ++k)
    rmax = std::max(rmax, s.r[k]);
  P.rcap = (rmax + 31) / 32 * 32;
  if (P.rcap > 1536)
    return fail(TTG_ERR_NO_SPACE, "eval_batch: ranks above 1536 are not served");
  TTG_CUDA(eval_smem_optin(P.rcap));
  // layout: [arena | slots | tts | idx] prefix, then [out | bad].
  size_t o = 0;
  P.off_arena = o;
  o = align256(o + sizeof(double) * static_cast<size_t>(P.arena_doubles));
  P.off_slots = o;
  o = align256(o + sizeof(CoreSlot) * P.slots.size());
  P.off_tts = o;
  o = align256(o + sizeof(TTInfo) * P.tts.size());
  P.off_order = o;
  const size_t table_end = o;
  P.off_idx = o;
  o = align256(o + sizeof(int32_t) * static_cast<size_t>(M) * s.d);
  P.prefix_bytes = o;
  P.off_out = o;
  o = align256(o + sizeof(double) * static_cast<size_t>(std::max<int64_t>(M, 1)));
  P.off_bad = o;
  o = align256(o + 256);
  P.total_bytes = o;
  TTG_CUDA(P.dev.ensure(P.total_bytes));
  TTG_CUDA(P.host.ensure(table_end));
  char* h = static_cast<char*>(P.host.p);
  std::memset(h, 0, table_end);
  double* arena = reinterpret_cast<double*>(h + P.off_arena);
  for (int k = 0; k < s.d; ++k)
    std::memcpy(arena + P.slots[k].off, s.data + s.src_off[k],
                sizeof(double) * static_cast<size_t>(s.size[k]));
  std::memcpy(h + P.off_slots, P.slots.data(), sizeof(CoreSlot) * P.slots.size());
  std::memcpy(h + P.off_tts, P.tts.data(), sizeof(TTInfo) * P.tts.size());
  P.h2d = static_cast<int64_t>(table_end + sizeof(int32_t) * static_cast<size_t>(M) * s.d);
  P.d2h = static_cast<int64_t>(sizeof(double) * M + sizeof(int));
  return TTG_OK;
}

static int32_t eval_upload(ttg_plan& P, cudaStream_t st)
{
  char* d = static_cast<char*>(P.dev.p);
  TTG_CUDA(cudaMemcpyAsync(d, P.host.p, P.off_order, cudaMemcpyHostToDevice, st));
  if (P.M > 0)
    TTG_CUDA(cudaMemcpyAsync(d + P.off_idx, P.eval_idx,
                             sizeof(int32_t) * static_cast<size_t>(P.M) * P.shapes[0].d,
                             cudaMemcpyHostToDevice, st));
  return TTG_OK;
}

int32_t ttg_plan_create_eval(const ttg_tensor* a, const int32_t* idx, int32_t M, ttg_plan** plan)
{
  g_err.clear();
  if (!plan)
    return fail(TTG_ERR_ARG, "null plan");
  if (int32_t st = need_device())
    return st;
  auto* P = new ttg_plan;
  if (int32_t st = build_eval_plan(*P, a, idx, M))
  {
    delete P;
    return st;
  }
  *plan = P;
  return TTG_OK;
}

int32_t ttg_eval_batch(const ttg_tensor* a, const int32_t* idx, int32_t M, double* out)
{
  g_err.clear();
  if (!out && M > 0)
    return fail(TTG_ERR_ARG, "eval_batch: null output");
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_plan P;
  if (int32_t st = build_eval_plan(P, a, idx, M))
    return st;
  if (M == 0)
    return TTG_OK;
  cudaStream_t st = lib_stream();
  if (int32_t e = eval_upload(P, st))
    return e;
  if (int32_t e = plan_run(P, st))
    return e;
  return ttg_plan_download(&P, st, nullptr, out, nullptr);
}

int32_t ttg_inner(const ttg_tensor* a, const ttg_tensor* b, double* out)
{
  g_err.clear();
  if (!out)
    return fail(TTG_ERR_ARG, "inner: null output");
  Shape A, B;
  if (int32_t st = describe(a, "inner", A))
    return st;
  if (int32_t st = describe(b, "inner", B))
    return st;
  if (A.d != B.d)
    return fail(TTG_ERR_SHAPE, "tt::inner: rank-d mismatch (a.d=" + std::to_string(A.d) +
                                   ", b.d=" + std::to_string(B.d) + ")");
  for (int k = 0; k < A.d; ++k)
    if (A.mode(k) != B.mode(k))
      return fail(TTG_ERR_SHAPE, "tt::inner: mode-size mismatch at axis " + std::to_string(k));
  if (A.d == 0)
  {
    *out = 0.0;
    return TTG_OK;
  }
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  ttg_plan P;
  P.shapes = {A, B};
  add_tensor(P, A, true, nullptr);
  add_tensor(P, B, true, nullptr);
  int64_t env = 1, tmp = 1;
  for (int k = 0; k < A.d; ++k)
  {
    env = std::max(env, static_cast<int64_t>(A.r[k + 1]) * B.r[k + 1]);
    env = std::max(env, static_cast<int64_t>(A.r[k]) * B.r[k]);
    tmp = std::max(tmp, static_cast<int64_t>(B.r[k]) * A.mode(k) * A.r[k + 1]);
  }
  env = a32(env);
  P.scratch_stride = 2 * env + a32(tmp) + 32;
  P.grid = 1;
  P.job_kind = -1;
  if (int32_t st = layout_and_alloc(P))
    return st;
  cudaStream_t st = lib_stream();
  if (int32_t e = plan_upload(P, st))
    return e;
  char* d = static_cast<char*>(P.dev.p);
  TTG_CUDA(cudaMemcpyAsync(d, d + P.off_pristine, P.prefix_bytes, cudaMemcpyDeviceToDevice, st));
  double* scratch = reinterpret_cast<double*>(d + P.off_scratch);
  const CoreSlot* S = reinterpret_cast<const CoreSlot*>(d + P.off_slots);
  launch_inner(reinterpret_cast<double*>(d + P.off_arena), S + P.tts[0].first,
               S + P.tts[1].first, A.d, scratch, env, scratch + P.scratch_stride - 8, st);
  g_launches += 1;
  TTG_CUDA(cudaGetLastError());
  TTG_CUDA(cudaMemcpyAsync(out, scratch + P.scratch_stride - 8, sizeof(double),
                           cudaMemcpyDeviceToHost, st));
  TTG_CUDA(cudaStreamSynchronize(st));
  return TTG_OK;
}

int32_t ttg_device_fp64_peak(double* tflops)
{
  g_err.clear();
  if (!tflops)
    return fail(TTG_ERR_ARG, "fp64_peak: null output");
  if (int32_t st = need_device())
    return st;
  std::lock_guard<std::mutex> lk(dev_state().mu);
  const int grid = 4 * std::max(device().sms, 1), block = 256, iters = 1 << 14;
  DevMem buf;
  TTG_CUDA(buf.ensure(sizeof(double) * static_cast<size_t>(grid) * block));
  cudaStream_t st = lib_stream();
  cudaEvent_t e0, e1;
  TTG_CUDA(cudaEventCreate(&e0));
  TTG_CUDA(cudaEventCreate(&e1));
  launch_fp64_peak(static_cast<double*>(buf.p), 64, grid, block, st);
  TTG_CUDA(cudaEventRecord(e0, st));
  launch_fp64_peak(static_cast<double*>(buf.p), iters, grid, block, st);
  TTG_CUDA(cudaEventRecord(e1, st));
  TTG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.0f;
  TTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = 2.0 * 8 * iters * static_cast<double>(grid) * block / (ms * 1e-3) / 1e12;
  return TTG_OK;
}

int32_t ttg_norm(const ttg_tensor* a, double* out)
{
  double s = 0.0;
  const int32_t st = ttg_inner(a, a, &s);
  if (st)
    return st;
  *out = std::sqrt(std::max(s, 0.0));
  return TTG_OK;
}

}  // extern "C"
