// The live-row rule of the CTA GEMM tiles (cta_gemm_tile, cta_gemm_df):
// which rows (or columns) of a thread's 4 x 4 block a k slab can touch.
// Host-callable so the rule is tested on the CPU against brute force.
#pragma once

#include <cuda_runtime.h>

namespace ttg
{

// Rows (or columns) ty + 16 a, a < result, of a thread's 4 x 4 block that
// lie inside the matrix (extent m from the tile start) and, for a
// triangular factor, can be non-zero in the k slab [p0, p0 + 16) (index
// <= p0 + 15 - tile start).
__host__ __device__ __forceinline__ int gemm_live(int m_from_tile, int t, bool tri, int p0_from_tile)
{
  int n = (m_from_tile - t + 15) >> 4;
  if (tri)
  {
    const int q = p0_from_tile + 15 - t;
    const int nt = q < 0 ? 0 : (q >> 4) + 1;
    n = nt < n ? nt : n;
  }
  return n < 0 ? 0 : (n > 4 ? 4 : n);
}

}  // namespace ttg
