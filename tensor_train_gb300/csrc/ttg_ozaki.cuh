// FP64-accurate GEMM tiles on the tcgen05 tensor cores by exact slicing:
// scheme I of Ozaki, Ogita, Oishi & Rump (Numer. Algorithms 59, 2012) with
// fixed-point BF16 slices.
//
// A row i of A (K entries) is scaled by 2^(7 - e_i), e_i the exponent of
// its largest entry, and cut into kOzS integer slices of 8 bits,
//   A(i, k) = 2^(e_i - 7) sum_s 2^(-8 s) a_s(i, k),  a_s integer in [-128, 128],
// each exactly representable in BF16.  B's columns likewise (f_j, b_t).
// Products a_s b_t are integers below 2^14; the tensor core accumulates them
// in FP32 in TMEM, one accumulator per diagonal g = s + t (kOzS groups of
// kOzN columns).  Groups 0 and 1 stay exact for K <= 512 (sums below 2^24);
// higher groups carry rounding of 2^-24 of a term already 2^-16 below the
// leading one.  Pairs with s + t >= kOzS are dropped (2^-40 relative to the
// row and column scales).  The epilogue forms
//   C(i, j) = 2^(e_i + f_j - 14) sum_g 2^(-8 g) acc_g(i, j)
// in FP64: ~1e-12 relative to |A(i,:)| |B(:,j)|.
//
// One CTA (any multiple of 4 warps, here 8) computes a 128 x 64 tile in
// K-chunks of 64: threads slice into shared memory (K-major, no swizzle),
// one thread issues the MMAs (15 per 16-deep step), a tcgen05.commit to an
// mbarrier ends the chunk.  Every wait is bounded.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

#include "ttg_device.cuh"
#include "ttg_tc.cuh"

namespace ttg
{
namespace
{

constexpr int kOzM = 128, kOzN = 64, kOzK = 64, kOzS = 5;
constexpr int kOzTmemCols = 512;  // kOzS * kOzN = 320 used
constexpr int kOzSliceA = kOzM * kOzK * 2, kOzSliceB = kOzN * kOzK * 2;
// slices of A and B, then the row and column exponents
constexpr int kOzSmemBytes = kOzS * (kOzSliceA + kOzSliceB) + (kOzM + kOzN) * 4;
constexpr long long kOzWaitCycles = 4000000000ll;

struct OzState
{
  uint32_t tmem;
  uint64_t* mbar;
  uint32_t phase;
};

__device__ bool oz_wait(OzState& st)
{
  const long long t0 = clock64();
  while (!tc::mbar_wait(st.mbar, st.phase, 64))
    if (clock64() - t0 > kOzWaitCycles)
      return false;
  st.phase ^= 1u;
  return true;
}

// Exponent e with max|x| < 2^e over the entries, from the bit patterns
// (0 for an all-zero set).
__device__ __forceinline__ int oz_exp_of_bits(unsigned long long mx)
{
  const int ex = static_cast<int>((mx >> 52) & 0x7ff);
  return ex == 0 ? 0 : ex - 1022;
}

// One 128 x 64 tile at (i0, j0) of C = A B (FP64 in and out, views as in
// cta_gemm).  Returns false if an MMA completion wait timed out (the MMAs
// in flight were drained, bounded).
__device__ __noinline__ bool oz_tile(int i0, int j0, int M, int N, int K, View A, View B,
                                     double* C, int64_t c_rs, int64_t c_cs, uint8_t* smem,
                                     OzState& st, CtaShared& sh)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (K <= 0)
  {
    for (int t = threadIdx.x; t < kOzM * kOzN; t += blockDim.x)
    {
      const int gi = i0 + t / kOzN, gj = j0 + t % kOzN;
      if (gi < M && gj < N)
        C[gi * c_rs + gj * c_cs] = 0.0;
    }
    __syncthreads();
    return true;
  }
  int* erow = reinterpret_cast<int*>(smem + kOzS * (kOzSliceA + kOzSliceB));
  int* ecol = erow + kOzM;
  // Row exponents of A and column exponents of B over the whole K.
  for (int r = warp; r < kOzM + kOzN; r += nw)
  {
    unsigned long long mx = 0ull;
    const bool is_row = r < kOzM;
    const int gi = is_row ? i0 + r : j0 + (r - kOzM);
    if (gi < (is_row ? M : N))
      for (int k = lane; k < K; k += 32)
      {
        const double x = is_row ? A(gi, k) : B(k, gi);
        const unsigned long long b =
          static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull;
        mx = b > mx ? b : mx;
      }
    for (int o = 16; o > 0; o >>= 1)
    {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = y > mx ? y : mx;
    }
    if (lane == 0)
    {
      if (is_row)
        erow[r] = oz_exp_of_bits(mx);
      else
        ecol[r - kOzM] = oz_exp_of_bits(mx);
    }
  }
  __syncthreads();
  constexpr uint32_t idesc = tc::idesc_bf16_f32(kOzM, kOzN);
  constexpr uint32_t sbo = (kOzK / 8) * 128;
  uint32_t written = 0u;  // accumulator groups already initialised (thread 0)
  bool ok = true;
  for (int k0 = 0; k0 < K; k0 += kOzK)
  {
    // Slice A (128 x 64) and B^T (64 x 64) into kOzS BF16 planes each.
    for (int t = threadIdx.x; t < (kOzM + kOzN) * kOzK; t += blockDim.x)
    {
      const bool is_a = t < kOzM * kOzK;
      const int u = is_a ? t : t - kOzM * kOzK;
      const int r = u / kOzK, kk = u % kOzK;
      const int gk = k0 + kk;
      double y = 0.0;
      int e = 0;
      if (is_a)
      {
        const int gi = i0 + r;
        if (gi < M && gk < K)
          y = A(gi, gk);
        e = erow[r];
      }
      else
      {
        const int gj = j0 + r;
        if (gj < N && gk < K)
          y = B(gk, gj);
        e = ecol[r];
      }
      y = ldexp(y, 7 - e);
      uint8_t* base = is_a ? smem : smem + kOzS * kOzSliceA;
      const int plane = is_a ? kOzSliceA : kOzSliceB;
      const uint32_t off = tc::kmajor_offset(r, kk, kOzK);
#pragma unroll
      for (int s = 0; s < kOzS; ++s)
      {
        const double v = rint(y);
        *reinterpret_cast<__nv_bfloat16*>(base + s * plane + off) =
          __float2bfloat16_rn(static_cast<float>(v));
        y = (y - v) * 256.0;
      }
    }
    tc::fence_async_shared();
    __syncthreads();
    if (threadIdx.x == 0)
    {
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_u32(smem), sb = tc::smem_u32(smem + kOzS * kOzSliceA);
      for (int kk = 0; kk < kOzK / 16; ++kk)
        for (int s = 0; s < kOzS; ++s)
          for (int t = 0; s + t < kOzS; ++t)
          {
            const int g = s + t;
            const uint64_t ad = tc::smem_desc(sa + s * kOzSliceA + kk * 256, 128, sbo);
            const uint64_t bd = tc::smem_desc(sb + t * kOzSliceB + kk * 256, 128, sbo);
            tc::mma_bf16(st.tmem + g * kOzN, ad, bd, idesc, (written >> g) & 1u);
            written |= 1u << g;
          }
      tc::mma_commit(st.mbar);
    }
    // The next chunk overwrites the planes: wait for these MMAs.
    if (!oz_wait(st))
      ok = false;
    __syncthreads();
    if (!ok)
      break;
  }
  if (!ok)
  {
    // Drain: the MMAs already issued still target this CTA's TMEM.
    if (threadIdx.x == 0)
      oz_wait(st);
    __syncthreads();
    return false;
  }
  // Epilogue: warp w reads lanes 32 (w % 4).. (tile rows) and columns
  // 32 (w / 4).. of every group, when the CTA has 8 warps; with 4 warps each
  // warp covers all 64 columns.
  tc::fence_after_sync();
  const int quarter = warp & 3;
  const int row = i0 + quarter * 32 + lane;
  const int r_local = quarter * 32 + lane;
  const int halves = nw >= 8 ? 2 : 1;
  const int h = warp / 4;
  if (h < halves)
  {
    const int cspan = kOzN / halves;
    for (int c0 = h * cspan; c0 < (h + 1) * cspan; c0 += 16)
    {
      double acc[16];
#pragma unroll
      for (int q = 0; q < 16; ++q)
        acc[q] = 0.0;
      for (int g = kOzS - 1; g >= 0; --g)
      {
        float v[16];
        tc::tmem_ld16(st.tmem + (static_cast<uint32_t>(quarter * 32) << 16) + g * kOzN + c0, v);
#pragma unroll
        for (int q = 0; q < 16; ++q)
          acc[q] = ldexp(acc[q], -8) + static_cast<double>(v[q]);
      }
      if (row < M)
      {
        const int er = erow[r_local];
#pragma unroll
        for (int q = 0; q < 16; ++q)
        {
          const int col = j0 + c0 + q;
          if (col < N)
            C[row * c_rs + col * c_cs] = ldexp(acc[q], er + ecol[c0 + q] - 14);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  return true;
}

}  // namespace
}  // namespace ttg
