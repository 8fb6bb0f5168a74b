// ttg_round_noalloc: TT rounding for callers that cannot allocate device
// memory -- code running inside another runtime's allocator (a framework
// plugin that must not call cudaMalloc), work enqueued while device
// allocation is forbidden, or processes that run with a fixed memory budget.
// The caller passes the input cores and an output buffer, both already on
// the device; every other byte the sweep needs (slot tables, the work copy of
// the cores and the sweep's scratch slab) comes from one file-scope device
// array of kNoallocScratchBytes, which every GPU that loads this library
// holds until the process exits.
//
// The sweep itself is the library's round kernel (round_kernel, one CTA),
// unchanged; this file only adds the table set-up, the packing of the result
// and the host entry point.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_job.h"
#include "ttg_kernels.h"

namespace ttg
{
namespace
{

constexpr size_t kNoallocScratchBytes = TTG_NOALLOC_SCRATCH_BYTES;
constexpr int kNoallocMaxD = TTG_NOALLOC_MAX_D;
constexpr int kMaxDevices = 64;

// The only device memory this entry point uses besides the caller's buffers.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct NoallocShape
{
  int32_t d;
  int32_t ranks[kNoallocMaxD + 1];
  int32_t modes[kNoallocMaxD];
};

// Byte layout inside the scratch array (all offsets 256-byte aligned):
// [slots | tt info | order | queue | result ranks+status | arena | slab].
struct NoallocLayout
{
  size_t slots, tt, order, queue, result, arena, slab, end;
  int64_t slab_doubles;
};

size_t al256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

// Writes the slot table for the input shape and resets every field a
// previous call may have left behind (queue counter, status, sweeps).
__global__ void noalloc_prepare(NoallocShape s, CoreSlot* slots, TTInfo* tt, int32_t* order,
                                int32_t* queue)
{
  if (threadIdx.x != 0)
    return;
  int64_t off = 0;
  for (int k = 0; k < s.d; ++k)
  {
    CoreSlot c{};
    c.off = off;
    c.n = s.modes[k];
    c.r = s.ranks[k];
    c.rp = s.ranks[k + 1];
    c.m = 0;
    slots[k] = c;
    off += static_cast<int64_t>(s.ranks[k]) * s.modes[k] * s.ranks[k + 1];
  }
  TTInfo t{};
  t.first = 0;
  t.d = s.d;
  *tt = t;
  order[0] = 0;
  *queue = 0;
}

// Packs the rounded cores from their slots into `out` back to back and
// records the final ranks and the sweep status (result[0..d], result[d+1]).
__global__ void noalloc_pack(const double* arena, const CoreSlot* slots, const TTInfo* tt, int d,
                             double* out, int32_t* result)
{
  __shared__ int64_t dst_off[kNoallocMaxD + 1];
  if (threadIdx.x == 0)
  {
    int64_t off = 0;
    for (int k = 0; k < d; ++k)
    {
      dst_off[k] = off;
      off += static_cast<int64_t>(slots[k].r) * slots[k].n * slots[k].rp;
    }
    dst_off[d] = off;
    result[0] = d > 0 ? slots[0].r : 1;
    for (int k = 0; k < d; ++k)
      result[k + 1] = slots[k].rp;
    result[d + 1] = tt->status;
  }
  __syncthreads();
  for (int k = 0; k < d; ++k)
  {
    const double* src = arena + slots[k].off;
    double* dst = out + dst_off[k];
    const int64_t n = dst_off[k + 1] - dst_off[k];
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
      dst[i] = src[i];
  }
}

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};
unsigned long long g_noalloc_ctx[kMaxDevices] = {};

int32_t nfail(int32_t st, const std::string& msg)
{
  set_last_error(msg);
  return st;
}

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the context current on this thread (0 if the driver cannot
// tell).  A cudaDeviceReset ends the device's primary context; the next
// runtime call makes a new one with a new id, in which the array has a new
// address.  The driver functions are fetched through the runtime, so the
// library does not link libcuda itself.
unsigned long long current_context_id()
{
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx &&
      get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of the scratch array for the current device.  Looked up
// with that device current on the first call in each context of the device
// (the first call on the device, and the first after a cudaDeviceReset) and
// cached; later calls reuse the cached address.
int32_t scratch_for_device(unsigned char** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return nfail(TTG_ERR_CUDA, std::string("round_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return nfail(TTG_ERR_NO_SPACE, "round_noalloc: device index above 63");
  // cudaSetDevice makes the device's primary context current on this thread
  // (cudaGetDevice alone does not), so the context id read next is the one
  // the kernels of this call will run in.
  e = cudaSetDevice(dev);
  if (e != cudaSuccess)
    return nfail(TTG_ERR_CUDA, std::string("round_noalloc: cudaSetDevice: ") + cudaGetErrorString(e));
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || ctx != g_noalloc_ctx[dev])
  {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return nfail(TTG_ERR_CUDA, std::string("round_noalloc: cudaGetSymbolAddress: ") +
                                     cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    // Looked up after the symbol so that a context made by the lookup
    // itself is the one recorded.
    g_noalloc_ctx[dev] = current_context_id();
  }
  *out = g_noalloc_ptr[dev];
  return TTG_OK;
}

// Scratch slab of one sweep over the input shape (upper bounds: ranks only
// shrink), for gauge none or right_canonical.
int64_t slab_need(const NoallocShape& s, bool right_canonical)
{
  int64_t need = 64, cols = 0;
  const int d = s.d;
  for (int k = 0; k < d; ++k)
  {
    const int64_t r = s.ranks[k], n = s.modes[k], rp = s.ranks[k + 1];
    const int64_t hp = k > 0 ? static_cast<int64_t>(s.ranks[k - 1]) * s.modes[k - 1] : 0;
    const int64_t wn = k + 1 < d ? static_cast<int64_t>(s.modes[k + 1]) * s.ranks[k + 2] : 0;
    if (!right_canonical)
    {
      if (k >= 1)
        need = imax64(need, need_right_qr(r, n * rp, hp));
      if (k <= d - 2)
        need = imax64(need, need_svd_step(r * n, rp, wn));
    }
    else
    {
      if (k <= d - 2)
        need = imax64(need, need_left_qr(r * n, rp, wn));
      if (k >= 1)
        need = imax64(need, need_svd_step_right(n * rp, r, hp));
    }
    if (k <= d - 2)
      cols += rp;
  }
  need = imax64(need, a32(2 * (cols + 1)));  // balance: scale factors and inverses
  return need + 64;
}

}  // namespace
}  // namespace ttg

extern "C" {

int32_t ttg_round_noalloc(int32_t d, const int32_t* ranks, const int32_t* modes,
                          const double* in_dev, double* out_dev, int32_t* out_ranks,
                          const ttg_round_options* opts, void* stream)
{
  using namespace ttg;
  set_last_error(std::string());
  if (d < 0 || !out_ranks || !opts || (d > 0 && (!ranks || !modes || !in_dev || !out_dev)))
    return nfail(TTG_ERR_ARG, "round_noalloc: null pointer or negative d");
  if (d > kNoallocMaxD)
    return nfail(TTG_ERR_NO_SPACE, "round_noalloc: d = " + std::to_string(d) + " exceeds the " +
                                       std::to_string(kNoallocMaxD) + "-core limit");
  if (std::isnan(opts->eps) || opts->eps < 0.0 || opts->max_rank < 0)
    return nfail(TTG_ERR_ARG, "round_noalloc: eps must be >= 0 and max_rank >= 0");
  if (opts->method != TTG_METHOD_SVD)
    return nfail(TTG_ERR_METHOD, "round_noalloc: only round_method::svd is served");
  if (opts->precision != TTG_PREC_FP64)
    return nfail(TTG_ERR_METHOD, "round_noalloc: only FP64 precision is served");
  if (opts->gauge != TTG_GAUGE_NONE && opts->gauge != TTG_GAUGE_RIGHT_CANONICAL)
    return nfail(TTG_ERR_ARG, "round_noalloc: unknown gauge");
  if (d == 0)
  {
    out_ranks[0] = 1;
    return TTG_OK;
  }
  NoallocShape s{};
  s.d = d;
  int64_t total = 0;
  for (int k = 0; k <= d; ++k)
  {
    if (ranks[k] <= 0)
      return nfail(TTG_ERR_SHAPE, "round_noalloc: tt_core: dimensions must be positive");
    s.ranks[k] = ranks[k];
  }
  if (d > 0 && (ranks[0] != 1 || ranks[d] != 1))
    return nfail(TTG_ERR_SHAPE, "round_noalloc: tt: r_0 and r_d must be 1");
  // Sizes are bounded before any of them is multiplied further: no factor
  // of a core (r*n, n*r', r*n*r') and no running total may exceed the
  // doubles the array holds, so every later product of two such terms
  // stays far inside int64.
  constexpr int64_t kCapDoubles = static_cast<int64_t>(kNoallocScratchBytes / sizeof(double));
  for (int k = 0; k < d; ++k)
  {
    if (modes[k] <= 0)
      return nfail(TTG_ERR_SHAPE, "round_noalloc: tt_core: dimensions must be positive");
    s.modes[k] = modes[k];
    const int64_t rn = static_cast<int64_t>(ranks[k]) * modes[k];
    const int64_t nrp = static_cast<int64_t>(modes[k]) * ranks[k + 1];
    if (rn > kCapDoubles || nrp > kCapDoubles || rn * ranks[k + 1] > kCapDoubles ||
        total + rn * ranks[k + 1] > kCapDoubles)
      return nfail(TTG_ERR_NO_SPACE,
                   "round_noalloc: core " + std::to_string(k) + " does not fit the fixed scratch of " +
                       std::to_string(kNoallocScratchBytes) + " bytes (use ttg_round instead)");
    total += rn * ranks[k + 1];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (d <= 1)
  {
    // round() returns d <= 1 inputs unchanged (round/tt_round.hpp:38-42).
    for (int k = 0; k <= d; ++k)
      out_ranks[k] = ranks[k];
    if (d == 1)
    {
      cudaError_t e = cudaMemcpyAsync(out_dev, in_dev, sizeof(double) * total,
                                      cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
      if (e != cudaSuccess)
        return nfail(TTG_ERR_CUDA, std::string("round_noalloc: ") + cudaGetErrorString(e));
    }
    return TTG_OK;
  }
  const bool right = opts->gauge == TTG_GAUGE_RIGHT_CANONICAL;
  NoallocLayout L{};
  size_t o = 0;
  L.slots = o;
  o = al256(o + sizeof(CoreSlot) * d);
  L.tt = o;
  o = al256(o + sizeof(TTInfo));
  L.order = o;
  o = al256(o + sizeof(int32_t));
  L.queue = o;
  o = al256(o + sizeof(int32_t));
  L.result = o;
  o = al256(o + sizeof(int32_t) * (d + 2));
  L.arena = o;
  o = al256(o + sizeof(double) * static_cast<size_t>(total));
  L.slab = o;
  L.slab_doubles = slab_need(s, right);
  o = al256(o + sizeof(double) * static_cast<size_t>(L.slab_doubles));
  L.end = o;
  if (L.end > kNoallocScratchBytes)
    return nfail(TTG_ERR_NO_SPACE,
                 "round_noalloc: this TT needs " + std::to_string(L.end) +
                     " bytes of device scratch; the fixed scratch holds " +
                     std::to_string(kNoallocScratchBytes) + " bytes (use ttg_round instead)");
  unsigned char* base = nullptr;
  if (int32_t rc = scratch_for_device(&base))
    return rc;
  CoreSlot* slots = reinterpret_cast<CoreSlot*>(base + L.slots);
  TTInfo* tt = reinterpret_cast<TTInfo*>(base + L.tt);
  int32_t* order = reinterpret_cast<int32_t*>(base + L.order);
  int32_t* queue = reinterpret_cast<int32_t*>(base + L.queue);
  int32_t* result = reinterpret_cast<int32_t*>(base + L.result);
  double* arena = reinterpret_cast<double*>(base + L.arena);
  cudaError_t e = cudaMemcpyAsync(arena, in_dev, sizeof(double) * total,
                                  cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess)
    return nfail(TTG_ERR_CUDA, std::string("round_noalloc: ") + cudaGetErrorString(e));
  noalloc_prepare<<<1, 32, 0, st>>>(s, slots, tt, order, queue);
  RoundJob job{};
  job.arena = arena;
  job.slots = slots;
  job.tts = tt;
  job.order = order;
  job.ntt = 1;
  job.kind = right ? kJobRoundRight : kJobRound;
  job.scratch = reinterpret_cast<double*>(base + L.slab);
  job.scratch_stride = L.slab_doubles;
  job.queue = queue;
  job.eps = opts->eps;
  job.max_rank = opts->max_rank;
  job.max_sweeps = opts->max_sweeps > 0 ? opts->max_sweeps : 40;
  launch_round(job, 1, 1, st);
  noalloc_pack<<<1, 256, 0, st>>>(arena, slots, tt, d, out_dev, result);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return nfail(TTG_ERR_CUDA, std::string("round_noalloc: launch: ") + cudaGetErrorString(e));
  int32_t host_result[kNoallocMaxD + 2];
  e = cudaMemcpyAsync(host_result, result, sizeof(int32_t) * (d + 2), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return nfail(TTG_ERR_CUDA, std::string("round_noalloc: ") + cudaGetErrorString(e));
  for (int k = 0; k <= d; ++k)
    out_ranks[k] = host_result[k];
  const int32_t status = host_result[d + 1];
  if (status == TTG_ERR_NOT_CONVERGED)
    // The result is complete (out_dev and out_ranks are written); Jacobi hit
    // its sweep limit on at least one bond, which ttg_round reports through
    // round_result.converged = false.
    return nfail(status, "round_noalloc: a Jacobi SVD reached max_sweeps before converging; the "
                         "rounded TT was written");
  if (status != TTG_OK)
    return nfail(status, std::string("round_noalloc: device status ") + ttg_status_string(status));
  return TTG_OK;
}

}  // extern "C"
