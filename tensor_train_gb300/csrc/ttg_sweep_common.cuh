// Small device helpers shared by the sweep kernels (ttg_kernels.cu) and the
// whole-GPU sweep (ttg_wide.cu): status codes, the scratch bump allocator,
// shared-memory staging descriptor, slot updates, norms.
#pragma once

#include "ttg_device.cuh"
#include "ttg_job.h"

namespace ttg
{
// Internal linkage: every translation unit that includes this header gets
// its own copy of these device functions.
namespace
{

constexpr int kStatusOk = 0;
constexpr int kStatusNan = 5;
constexpr int kStatusNotConverged = 6;
constexpr int kStatusNoSpace = 11;

// Bump allocator over the CTA's scratch slab (256-byte aligned chunks).
struct Bump
{
  double* p;
  __device__ double* take(int64_t n)
  {
    double* r = p;
    p += (n + 31) & ~static_cast<int64_t>(31);
    return r;
  }
};

__device__ __forceinline__ bool finite(double x) { return isfinite(x); }

// Records a status on the TT (first error wins) -- thread 0 only.
__device__ void set_status(TTInfo& T, int st)
{
  if (threadIdx.x == 0 && T.status == kStatusOk)
    T.status = st;
}

struct Smem
{
  double* p;
  int64_t cap;
};

__device__ void record_bond(BondStat* bs, const double* sorted, int nsv, int r_new)
{
  if (bs && threadIdx.x == 0)
  {
    bs->s_max = sorted[0];
    bs->s_last = sorted[r_new - 1];
    bs->r_new = r_new;
    bs->n_sv = nsv;
  }
}

__device__ void set_ranks(CoreSlot& s, int r, int rp)
{
  if (threadIdx.x == 0)
  {
    s.r = r;
    s.rp = rp;
  }
}

__device__ double core_norm(const double* p, int64_t n, CtaShared& sh)
{
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x)
    s += p[t] * p[t];
  return sqrt(cta_sum(s, sh));
}

__device__ int64_t core_size(const CoreSlot& s)
{
  return static_cast<int64_t>(s.r) * s.n * s.rp;
}

// make_rank1_zero_tt (detail/shape_check.hpp:176-188).
__device__ void zero_tt(double* ar, CoreSlot* S, int d)
{
  for (int k = 0; k < d; ++k)
  {
    for (int i = threadIdx.x; i < S[k].n; i += blockDim.x)
      ar[S[k].off + i] = 0.0;
    set_ranks(S[k], 1, 1);
  }
  __syncthreads();
}

}  // namespace
}  // namespace ttg
