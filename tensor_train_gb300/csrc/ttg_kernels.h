// Host-side launchers of the sweep, apply, eval and inner kernels.
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "ttg_job.h"

namespace ttg
{

// ctas_per_sm: 1-2 (128 registers), 3 (85) or 4 (64): the instantiation.
void launch_round(const RoundJob& job, int grid, int ctas_per_sm, cudaStream_t stream);
// Whole-GPU rounding (cooperative launch, grid <= the value from setup).
cudaError_t launch_wide_round(const WideJob& job, int grid, cudaStream_t stream);
// Opt-in to the dynamic shared memory and the co-resident grid size.
cudaError_t wide_round_setup(int smem_doubles, int* max_grid);
void launch_apply_core(const double* A, const double* X, double* Y, int r, int m, int p, int rp,
                       int s, int nout, int sp, cudaStream_t stream);
void launch_eval(const double* ar, const CoreSlot* S, int d, const int* idx, int64_t M,
                 double* out, int rcap, int* bad, int grid, cudaStream_t stream);
void launch_inner(const double* ar, const CoreSlot* SA, const CoreSlot* SB, int d,
                  double* scratch, int64_t env_cap, double* out, cudaStream_t stream);
cudaError_t eval_smem_optin(int rcap);
cudaError_t round_smem_optin(int smem_doubles);
void launch_fp64_peak(double* out, int iters, int grid, int block, cudaStream_t stream);
// tcgen05 split-BF16 GEMM (ttg_tc_gemm.cu): C = A B (+ bias) (relu) (+ C).
cudaError_t tc_gemm_f32(cudaStream_t st, int M, int N, int K, const float* A, int64_t a_rs,
                        int64_t a_cs, const float* B, int64_t b_rs, int64_t b_cs, float* C,
                        int64_t ldc, const float* bias, bool relu, bool accumulate, int splits);
// Reads and clears the tensor-core GEMM timeout flag (synchronises st).
bool tc_gemm_timed_out(cudaStream_t st);
// Sets the message returned by ttg_last_error() on this thread.
void set_last_error(const std::string& msg);

}  // namespace ttg
