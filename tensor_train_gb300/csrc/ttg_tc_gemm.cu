// FP32 GEMM on the tcgen05 tensor cores with split-precision BF16 operands:
//   C (M x N) = A (M x K) * B (K x N) (+ bias[j]) (relu) (+ C),
// A(i, p) = A[i*a_rs + p*a_cs], B(p, j) = B[p*b_rs + j*b_cs] (any strides,
// so transposed operands need no copy).
//
// Two kernels on the caller's stream:
//   1. split_planes_kernel: each FP32 operand is split into BF16 planes,
//      x = hi + lo + O(2^-17 |x|), hi = bf16(x), lo = bf16(x - hi), stored
//      K-major (A as M x K, B as its transpose N x K), zero-padded to whole
//      tiles, in a stream-ordered workspace.
//   2. tc_gemm_tma_kernel: one CTA (4 warps) per 128 x BN tile of C.  Warp 0
//      is the TMA producer: cp.async.bulk.tensor copies 64-wide K slabs of
//      the planes into a 3-stage ring of 128-byte-swizzled shared tiles,
//      each stage signalled on a "full" mbarrier with its byte count.  Warp 1
//      issues the MMAs from one thread (kind::f16, BF16 x BF16 -> FP32 in
//      TMEM, M = 128, N = BN, K = 16 each; with splits = 3 the products
//      hi*hi + hi*lo + lo*hi, ~1e-5 relative, the dropped lo*lo term being
//      2^-16; splits = 1 is plain BF16) and frees each stage with
//      tcgen05.commit on its "empty" mbarrier.  All four warps then read
//      their 32 TMEM lanes (= tile rows) with tcgen05.ld for the epilogue.
// Every mbarrier wait is bounded: on timeout the kernel records the failure
// in *err, stops both loops, waits (bounded) for the MMAs and copies in
// flight, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_kernels.h"
#include "ttg_tc.cuh"

namespace ttg
{
namespace
{

constexpr int kBM = 128, kBK = 64, kTcThreads = 128, kStages = 3;
// ~2 s at 2 GHz: far beyond any MMA group's or copy's latency.
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
  // Failure-path tests only: before its first MMA the issuing thread waits
  // on an mbarrier nothing arrives on, so that the wait runs out (~1 ms)
  // and the kernel takes its timeout path.
  int stall_waits;
};

// Bounded wait for a phase; gives up early once *abort is set (another
// role of the CTA failed).
__device__ bool wait_bounded(uint64_t* mbar, uint32_t parity, long long limit = kWaitCycles,
                             volatile int* abort = nullptr)
{
  const long long t0 = clock64();
  while (!tc::mbar_wait(mbar, parity, 64))
  {
    if (abort && *abort)
      return false;
    if (clock64() - t0 > limit)
      return false;
  }
  return true;
}

// BF16 planes (rows_pad x kpad, row-major) of X(i, p) = X[i*rs + p*cs],
// i < rows, p < K, zero elsewhere.
__global__ void split_planes_kernel(const float* __restrict__ X, int64_t rs, int64_t cs, int rows,
                                    int K, int rows_pad, int kpad, __nv_bfloat16* hi,
                                    __nv_bfloat16* lo)
{
  const int64_t total = static_cast<int64_t>(rows_pad) * kpad;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
  {
    const int i = static_cast<int>(t / kpad), p = static_cast<int>(t % kpad);
    const float x = (i < rows && p < K) ? X[i * rs + p * cs] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[t] = h;
    if (lo)
      lo[t] = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

template <int BN>
__global__ void __launch_bounds__(kTcThreads)
  tc_gemm_tma_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                     const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl,
                     TcGemmArgs g, int nk)
{
  extern __shared__ uint8_t tc_smem_raw[];
  constexpr int kTileA = kBM * kBK * 2, kTileB = BN * kBK * 2;
  constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;
  // 128-byte swizzled tiles want 1024-byte aligned bases.
  uint8_t* smem = reinterpret_cast<uint8_t*>(
    (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ __align__(8) uint64_t empty[kStages];
  __shared__ __align__(8) uint64_t done;
  __shared__ __align__(8) uint64_t stall_mbar;  // never arrived on
  __shared__ uint32_t tmem_base;
  __shared__ int failed, issued, consumed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const bool three = g.splits == 3;
  auto a_hi = [&](int s) { return smem + s * kStageBytes; };
  auto a_lo = [&](int s) { return smem + s * kStageBytes + kTileA; };
  auto b_hi = [&](int s) { return smem + s * kStageBytes + 2 * kTileA; };
  auto b_lo = [&](int s) { return smem + s * kStageBytes + 2 * kTileA + kTileB; };

  if (warp == 0)
    tc::tmem_alloc(&tmem_base, BN);
  if (threadIdx.x == 0)
  {
    for (int s = 0; s < kStages; ++s)
    {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::mbar_init(&stall_mbar, 1);
    failed = 0;
    issued = 0;
    consumed = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  volatile int* vfailed = &failed;

  if (warp == 0 && lane == 0 && nk > 0)
  {
    // TMA producer.
    const uint32_t tx = three ? kStageBytes : (kTileA + kTileB);
    for (int kb = 0; kb < nk; ++kb)
    {
      const int s = kb % kStages;
      if (kb >= kStages && !wait_bounded(&empty[s], ((kb / kStages) - 1) & 1, kWaitCycles, vfailed))
      {
        atomicExch(&failed, 1);
        break;
      }
      if (*vfailed)
        break;
      tc::mbar_arrive_expect_tx(&full[s], tx);
      tc::tma_load_2d(a_hi(s), &mAh, &full[s], kb * kBK, m0);
      tc::tma_load_2d(b_hi(s), &mBh, &full[s], kb * kBK, n0);
      if (three)
      {
        tc::tma_load_2d(a_lo(s), &mAl, &full[s], kb * kBK, m0);
        tc::tma_load_2d(b_lo(s), &mBl, &full[s], kb * kBK, n0);
      }
      issued = kb + 1;
    }
  }
  else if (warp == 1 && lane == 0)
  {
    // MMA issuer.
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, BN);
    bool ok = !g.stall_waits || wait_bounded(&stall_mbar, 0, kStallWaitCycles);
    for (int kb = 0; ok && kb < nk; ++kb)
    {
      const int s = kb % kStages;
      if (!wait_bounded(&full[s], (kb / kStages) & 1, kWaitCycles, vfailed))
      {
        ok = false;
        break;
      }
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk)
      {
        const uint32_t step = kk * 32;
        const uint64_t ah = tc::smem_desc_sw128(tc::smem_u32(a_hi(s)) + step);
        const uint64_t bh = tc::smem_desc_sw128(tc::smem_u32(b_hi(s)) + step);
        tc::mma_bf16(tmem, ah, bh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
        if (three)
        {
          const uint64_t al = tc::smem_desc_sw128(tc::smem_u32(a_lo(s)) + step);
          const uint64_t bl = tc::smem_desc_sw128(tc::smem_u32(b_lo(s)) + step);
          tc::mma_bf16(tmem, ah, bl, idesc, 1u);
          tc::mma_bf16(tmem, al, bh, idesc, 1u);
        }
      }
      tc::mma_commit(&empty[s]);
      consumed = kb + 1;
    }
    if (!ok)
      atomicExch(&failed, 1);
    // Arrives once every MMA issued above has completed.
    tc::mma_commit(&done);
  }
  __syncthreads();
  // Every thread waits for the MMAs (done), bounded.
  const bool mma_done = wait_bounded(&done, 0);
  if (!mma_done && lane == 0)
    atomicExch(&failed, 1);
  __syncthreads();
  if (failed)
  {
    if (threadIdx.x == 0)
    {
      atomicExch(g.err, 1);
      // Copies issued but never consumed still target the shared tiles:
      // wait (bounded) for them to land before the CTA leaves.
      for (int kb = consumed; kb < issued; ++kb)
        wait_bounded(&full[kb % kStages], (kb / kStages) & 1);
    }
  }
  else if (nk > 0)
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
  else
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
  return kStages * (2 * kBM * kBK * 2 + 2 * BN * kBK * 2) + 1024;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda itself).
EncodeTiledFn encode_tiled()
{
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<EncodeTiledFn>(nullptr);
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// 2-D map of a BF16 plane (rows x kpad, row-major), boxes of 64 x box_rows,
// 128-byte swizzle.  kpad is a multiple of 64, so every box starts at a
// multiple of 128 bytes along K.
bool make_plane_map(CUtensorMap* map, void* base, int rows, int kpad, int box_rows)
{
  EncodeTiledFn fn = encode_tiled();
  if (!fn)
    return false;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kpad), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kpad) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_bn(const TcGemmArgs& g, cudaStream_t st)
{
  static std::once_flag once[64];
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t attr = cudaSuccess;
  std::call_once(once[dev & 63], [&] {
    attr = cudaFuncSetAttribute(tc_gemm_tma_kernel<BN>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem_bytes<BN>());
  });
  if (attr != cudaSuccess)
    return attr;
  const int mt = (g.M + kBM - 1) / kBM, nt = (g.N + BN - 1) / BN;
  const int mpad = mt * kBM, npad = nt * BN;
  const int kpad = ((g.K + kBK - 1) / kBK) * kBK;
  const int nk = kpad / kBK;
  const bool three = g.splits == 3;
  CUtensorMap mAh{}, mAl{}, mBh{}, mBl{};
  __nv_bfloat16* ws = nullptr;
  if (nk > 0)
  {
    // Stream-ordered workspace: calls on other streams get their own.
    const size_t a_elems = static_cast<size_t>(mpad) * kpad, b_elems = static_cast<size_t>(npad) * kpad;
    const size_t bytes = (a_elems + b_elems) * (three ? 2 : 1) * sizeof(__nv_bfloat16);
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, st);
    if (e != cudaSuccess)
      return e;
    __nv_bfloat16* ah = ws;
    __nv_bfloat16* bh = ah + a_elems;
    __nv_bfloat16* al = three ? bh + b_elems : nullptr;
    __nv_bfloat16* bl = three ? al + a_elems : nullptr;
    const int threads = 256;
    const int blocks_a = static_cast<int>(std::min<size_t>((a_elems + threads - 1) / threads, 4096));
    const int blocks_b = static_cast<int>(std::min<size_t>((b_elems + threads - 1) / threads, 4096));
    split_planes_kernel<<<blocks_a, threads, 0, st>>>(g.A, g.a_rs, g.a_cs, g.M, g.K, mpad, kpad,
                                                      ah, al);
    // B^T (N x K): element (j, p) = B(p, j) = B[p*b_rs + j*b_cs].
    split_planes_kernel<<<blocks_b, threads, 0, st>>>(g.B, g.b_cs, g.b_rs, g.N, g.K, npad, kpad,
                                                      bh, bl);
    if (!make_plane_map(&mAh, ah, mpad, kpad, kBM) || !make_plane_map(&mBh, bh, npad, kpad, BN) ||
        (three && (!make_plane_map(&mAl, al, mpad, kpad, kBM) ||
                   !make_plane_map(&mBl, bl, npad, kpad, BN))))
    {
      cudaFreeAsync(ws, st);
      return cudaErrorInvalidValue;
    }
    if (!three)
    {
      mAl = mAh;
      mBl = mBh;
    }
  }
  dim3 grid(mt, nt);
  tc_gemm_tma_kernel<BN><<<grid, kTcThreads, tc_smem_bytes<BN>(), st>>>(mAh, mAl, mBh, mBl, g, nk);
  cudaError_t e = cudaGetLastError();
  if (ws)
    cudaFreeAsync(ws, st);
  return e;
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
