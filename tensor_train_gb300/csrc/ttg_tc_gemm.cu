// FP32 GEMM on the tcgen05 tensor cores with split-precision BF16 operands:
//   C (M x N) = A (M x K) * B (K x N) (+ bias[j]) (relu) (+ C),
// A(i, p) = A[i*a_rs + p*a_cs], B(p, j) = B[p*b_rs + j*b_cs] (any strides,
// so transposed operands need no copy).
//
// Each FP32 operand is split while it is staged into shared memory:
// x = hi + lo + O(2^-17 |x|), hi = bf16(x), lo = bf16(x - hi).  With
// `splits` = 3 the tile accumulates hi*hi + hi*lo + lo*hi in one FP32 TMEM
// accumulator (the dropped lo*lo term is 2^-16 relative), which gives
// ~1e-5 relative products at three times the BF16 MMA count; `splits` = 1 is
// plain BF16.
//
// One CTA (4 warps) computes a 128 x BN tile: warps stage K-chunks of 64 into
// the canonical K-major no-swizzle layout, one thread issues the MMAs
// (kind::f16, BF16 x BF16 -> FP32, M = 128, N = BN, K = 16 each), a
// tcgen05.commit arrives on an mbarrier when they complete, and every warp
// reads its 32 TMEM lanes (= tile rows) back with tcgen05.ld for the
// epilogue.  Every mbarrier wait is bounded: on timeout the kernel records
// the failure in *err, waits (bounded) once more for the MMAs in flight,
// frees its TMEM and returns.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_kernels.h"
#include "ttg_tc.cuh"

namespace ttg
{
namespace
{

constexpr int kBM = 128, kBK = 64, kTcThreads = 128;
// ~2 s at 2 GHz: far beyond any MMA group's latency.
constexpr long long kWaitCycles = 4000000000ll;
// ~1 ms: the stalled wait of the failure-path tests.
constexpr long long kStallWaitCycles = 2000000ll;

struct TcGemmArgs
{
  int M, N, K;
  const float* A;
  int64_t a_rs, a_cs;
  const float* B;
  int64_t b_rs, b_cs;
  float* C;
  int64_t ldc;
  const float* bias;
  int relu, accumulate, splits;
  int* err;
  // Failure-path tests only: before each MMA completion wait, wait on an
  // mbarrier nothing arrives on, so that the wait runs out (~1 ms) and the
  // kernel takes its timeout path.
  int stall_waits;
};

__device__ bool wait_bounded(uint64_t* mbar, uint32_t parity, long long limit = kWaitCycles)
{
  const long long t0 = clock64();
  while (!tc::mbar_wait(mbar, parity, 64))
    if (clock64() - t0 > limit)
      return false;
  return true;
}

__device__ __forceinline__ void split_store(uint8_t* hi, uint8_t* lo, uint32_t off, float x)
{
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
  *reinterpret_cast<__nv_bfloat16*>(lo + off) = l;
}

template <int BN>
__global__ void __launch_bounds__(kTcThreads) tc_gemm_kernel(TcGemmArgs g)
{
  extern __shared__ __align__(128) uint8_t tc_smem[];
  constexpr int kTileA = kBM * kBK * 2, kTileB = BN * kBK * 2;
  uint8_t* a_hi = tc_smem;
  uint8_t* a_lo = a_hi + kTileA;
  uint8_t* b_hi = a_lo + kTileA;
  uint8_t* b_lo = b_hi + kTileB;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t stall_mbar;  // never arrived on
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;

  if (warp == 0)
    tc::tmem_alloc(&tmem_base, BN);
  if (threadIdx.x == 0)
  {
    tc::mbar_init(&mbar, 1);
    tc::mbar_init(&stall_mbar, 1);
    failed = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, BN);
  constexpr uint32_t sbo = (kBK / 8) * 128;
  const bool a_row_fast = g.a_rs == 1;  // consecutive i contiguous in memory
  const bool b_col_fast = g.b_cs == 1;  // consecutive j contiguous in memory
  uint32_t phase = 0;
  bool issued = false;

  for (int k0 = 0; k0 < g.K; k0 += kBK)
  {
    // Stage A (rows m0.., K-chunk k0..) and B^T (rows n0..) as hi/lo BF16.
    for (int t = threadIdx.x; t < kBM * kBK; t += kTcThreads)
    {
      const int i = a_row_fast ? t % kBM : t / kBK;
      const int p = a_row_fast ? t / kBM : t % kBK;
      const int gi = m0 + i, gp = k0 + p;
      const float x = (gi < g.M && gp < g.K) ? g.A[gi * g.a_rs + gp * g.a_cs] : 0.f;
      split_store(a_hi, a_lo, tc::kmajor_offset(i, p, kBK), x);
    }
    for (int t = threadIdx.x; t < BN * kBK; t += kTcThreads)
    {
      const int j = b_col_fast ? t % BN : t / kBK;
      const int p = b_col_fast ? t / BN : t % kBK;
      const int gj = n0 + j, gp = k0 + p;
      const float x = (gj < g.N && gp < g.K) ? g.B[gp * g.b_rs + gj * g.b_cs] : 0.f;
      split_store(b_hi, b_lo, tc::kmajor_offset(j, p, kBK), x);
    }
    tc::fence_async_shared();
    __syncthreads();
    if (threadIdx.x == 0)
    {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk)
      {
        const uint32_t step = kk * 256;
        const uint64_t ah = tc::smem_desc(tc::smem_u32(a_hi) + step, 128, sbo);
        const uint64_t bh = tc::smem_desc(tc::smem_u32(b_hi) + step, 128, sbo);
        tc::mma_bf16(tmem, ah, bh, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
        if (g.splits == 3)
        {
          const uint64_t al = tc::smem_desc(tc::smem_u32(a_lo) + step, 128, sbo);
          const uint64_t bl = tc::smem_desc(tc::smem_u32(b_lo) + step, 128, sbo);
          tc::mma_bf16(tmem, ah, bl, idesc, 1u);
          tc::mma_bf16(tmem, al, bh, idesc, 1u);
        }
      }
      tc::mma_commit(&mbar);
    }
    issued = true;
    // The next chunk overwrites the operands: wait for these MMAs.
    bool done = !g.stall_waits || wait_bounded(&stall_mbar, 0, kStallWaitCycles);
    done = done && wait_bounded(&mbar, phase);
    if (!done)
    {
      if (lane == 0)
        atomicExch(&failed, 1);
    }
    phase ^= 1u;
    __syncthreads();
    if (failed)
      break;
  }

  if (!failed && issued)
  {
    tc::fence_after_sync();
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_addr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16)
    {
      float v[16];
      tc::tmem_ld16(lane_addr + c0, v);
      if (row < g.M)
      {
#pragma unroll
        for (int q = 0; q < 16; ++q)
        {
          const int col = n0 + c0 + q;
          if (col < g.N)
          {
            float y = v[q] + (g.bias ? g.bias[col] : 0.f);
            if (g.relu)
              y = fmaxf(y, 0.f);
            float* dst = g.C + static_cast<int64_t>(row) * g.ldc + col;
            if (g.accumulate)
              y += *dst;
            *dst = y;
          }
        }
      }
    }
  }
  else if (!issued)
  {
    // K == 0: C = bias (relu) (+ C).
    for (int t = threadIdx.x; t < kBM * BN; t += kTcThreads)
    {
      const int row = m0 + t / BN, col = n0 + t % BN;
      if (row < g.M && col < g.N)
      {
        float y = g.bias ? g.bias[col] : 0.f;
        if (g.relu)
          y = fmaxf(y, 0.f);
        float* dst = g.C + static_cast<int64_t>(row) * g.ldc + col;
        if (g.accumulate)
          y += *dst;
        *dst = y;
      }
    }
  }
  if (failed && threadIdx.x == 0)
  {
    atomicExch(g.err, 1);
    // Drain: the MMAs already issued still target this CTA's TMEM.
    wait_bounded(&mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0)
  {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, BN);
  }
}

template <int BN>
constexpr int tc_smem_bytes()
{
  return 2 * kBM * kBK * 2 + 2 * BN * kBK * 2;
}

template <int BN>
cudaError_t launch_bn(const TcGemmArgs& g, cudaStream_t st)
{
  static std::once_flag once[64];
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t attr = cudaSuccess;
  std::call_once(once[dev & 63], [&] {
    attr = cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                tc_smem_bytes<BN>());
  });
  if (attr != cudaSuccess)
    return attr;
  dim3 grid((g.M + kBM - 1) / kBM, (g.N + BN - 1) / BN);
  tc_gemm_kernel<BN><<<grid, kTcThreads, tc_smem_bytes<BN>(), st>>>(g);
  return cudaGetLastError();
}

std::mutex g_flag_mu;
int* g_flags[64] = {};

int* error_flag()
{
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_flag_mu);
  int*& f = g_flags[dev & 63];
  if (!f && cudaMalloc(&f, sizeof(int)) == cudaSuccess)
    cudaMemset(f, 0, sizeof(int));
  return f;
}

}  // namespace

cudaError_t tc_gemm_f32(cudaStream_t st, int M, int N, int K, const float* A, int64_t a_rs,
                        int64_t a_cs, const float* B, int64_t b_rs, int64_t b_cs, float* C,
                        int64_t ldc, const float* bias, bool relu, bool accumulate, int splits)
{
  if (M <= 0 || N <= 0)
    return cudaSuccess;
  int* err = error_flag();
  if (!err)
    return cudaErrorMemoryAllocation;
  const char* stall = std::getenv("TTG_TEST_STALL_DEVICE_WAITS");
  TcGemmArgs g{M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, bias,
               relu ? 1 : 0, accumulate ? 1 : 0, splits, err,
               (stall && stall[0] == '1') ? 1 : 0};
  if (N > 64)
    return launch_bn<128>(g, st);
  if (N > 32)
    return launch_bn<64>(g, st);
  return launch_bn<32>(g, st);
}

// Reads and clears the timeout flag of the current device (synchronises st).
bool tc_gemm_timed_out(cudaStream_t st)
{
  int* err = error_flag();
  if (!err)
    return false;
  int h = 0;
  cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  if (h)
    cudaMemsetAsync(err, 0, sizeof(int), st);
  return h != 0;
}

}  // namespace ttg

extern "C" int32_t ttg_tc_gemm_f32(int32_t M, int32_t N, int32_t K, const float* A, int64_t a_rs,
                                   int64_t a_cs, const float* B, int64_t b_rs, int64_t b_cs,
                                   float* C, int64_t ldc, int32_t splits, void* stream)
{
  ttg::set_last_error(std::string());
  if (M < 0 || N < 0 || K < 0 || (splits != 1 && splits != 3))
  {
    ttg::set_last_error("tc_gemm_f32: negative size or splits not in {1, 3}");
    return TTG_ERR_ARG;
  }
  if (M == 0 || N == 0)
    return TTG_OK;
  if (!C || (K > 0 && (!A || !B)))
  {
    ttg::set_last_error("tc_gemm_f32: null operand");
    return TTG_ERR_ARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = ttg::tc_gemm_f32(st, M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, nullptr,
                                   false, false, splits);
  if (e != cudaSuccess)
  {
    ttg::set_last_error(std::string("tc_gemm_f32: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TTG_ERR_OOM : TTG_ERR_CUDA;
  }
  if (ttg::tc_gemm_timed_out(st))
  {
    ttg::set_last_error("tc_gemm_f32: an MMA completion wait timed out");
    return TTG_ERR_TIMEOUT;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    ttg::set_last_error(std::string("tc_gemm_f32: ") + cudaGetErrorString(e));
    return TTG_ERR_CUDA;
  }
  return TTG_OK;
}
