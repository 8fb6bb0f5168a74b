// tcgen05 (5th-generation tensor core) building blocks for sm_103a, written
// as inline PTX: TMEM allocation, single-thread MMA issue with operands in
// shared memory, completion through an mbarrier, TMEM -> register loads, and
// TMA (cp.async.bulk.tensor) copies into the 128-byte swizzled layout.
//
// Operand layout: K-major, no swizzle ("interleaved" canonical layout).  A
// tile of R rows x K columns of 16-bit elements is stored as 8x8 core
// matrices of 128 contiguous bytes (8 rows x 16 bytes); core (i, j) -- rows
// 8i..8i+7, columns 8j..8j+7 -- sits at byte (i * K/8 + j) * 128.  In the
// shared-memory descriptor the leading byte offset (LBO) is the distance
// between neighbouring core matrices along K (128 bytes) and the stride byte
// offset (SBO) the distance between 8-row groups (K/8 * 128 bytes).  One
// kind::f16 MMA consumes K = 16 (two core matrices along K); the descriptor
// start address advances by 256 bytes per MMA.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ttg
{
namespace tc
{

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, col) of a K-major no-swizzle tile with K
// columns (K a multiple of 8), 16-bit elements.
__device__ __forceinline__ uint32_t kmajor_offset(int row, int col, int K)
{
  return static_cast<uint32_t>(((row >> 3) * (K >> 3) + (col >> 3)) * 128 + (row & 7) * 16 +
                               (col & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 in bits
// [0,14), LBO >> 4 in [16,30), SBO >> 4 in [32,46), version 1 in [46,48),
// base offset 0, layout type 0 (no swizzle) in [61,64).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) |
         (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D,
// M x N tile.  M = 128 needs N a multiple of 16 in [16, 256].
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

// Whole warp: allocate ncols TMEM columns (power of two >= 32); the base
// address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                 smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// Single thread: D(tmem) (+)= A(smem) * B(smem)^T.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
    : "memory");
}

// Single thread: arrive on the mbarrier once every MMA issued so far by
// this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                 smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_polls)
{
  const uint32_t a = smem_u32(mbar);
  for (uint32_t i = 0; i < max_polls; ++i)
  {
    uint32_t done;
    asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(a), "r"(parity)
      : "memory");
    if (done)
      return true;
  }
  return false;
}

// Single thread: arrive on the mbarrier and add `bytes` to the transaction
// count that the TMA copies signalling it must complete.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}

// Single thread: TMA copy of the box at (x, y) of a 2-D tensor map into
// shared memory; completion is signalled on the mbarrier (complete_tx).
// x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, uint64_t* mbar, int x,
                                            int y)
{
  asm volatile(
    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
    "%4}], [%2];" ::"r"(smem_u32(dst)),
    "l"(reinterpret_cast<uint64_t>(tmap)), "r"(smem_u32(mbar)), "r"(x), "r"(y)
    : "memory");
}

// Shared-memory matrix descriptor for a K-major tile in the 128-byte
// swizzled layout that a TMA copy with 128-byte swizzle writes: rows of
// 64 BF16 (128 bytes), 8-row atoms of 1024 bytes (SBO), layout type 2
// (128B swizzle) in [61,64), version 1; the tile base 1024-byte aligned.
// A K step of 16 elements inside the atom advances the start by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) | (1ull << 16) |
         (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

// Generic-proxy shared-memory writes become visible to the tensor core.
__device__ __forceinline__ void fence_async_shared()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_before_sync()
{
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync()
{
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Warp: 32 lanes x 16 consecutive FP32 columns from TMEM (lane quarter of
// this warp, columns starting at the address's column field).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
  uint32_t r[16];
  asm volatile(
    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
    "%15}, [%16];\n"
    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
      "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
      "=r"(r[14]), "=r"(r[15])
    : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i)
    v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace ttg
