// Device-side job tables shared by the host runtime and the kernels.
//
// HBM layout of a job: one arena of FP64 core slots.  Slot capacity is the
// core's input size; rounding never grows a core (ranks only shrink along a
// sweep), so every step writes its result back into the slot it came from.
// The tables below are small and live next to the arena.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define TTG_HD __host__ __device__
#else
#define TTG_HD
#endif

namespace ttg
{

// Scratch sizes (doubles) of the sweep steps.  The host sizes each CTA's
// slab with these functions evaluated at the input dimensions (upper bounds:
// ranks only shrink during a sweep) and the device checks the same functions
// at the actual dimensions before every step, so a step can never run past
// its slab.  Each bump allocation is rounded up to 32 doubles (256 bytes).
TTG_HD inline int64_t a32(int64_t n) { return (n + 31) & ~static_cast<int64_t>(31); }
TTG_HD inline int64_t imax64(int64_t a, int64_t b) { return a > b ? a : b; }

// left_svd on an (h x c) matrix, all three branches.
TTG_HD inline int64_t need_left_svd(int64_t h, int64_t c)
{
  const int64_t mn = h < c ? h : c;
  // + FP32 staging (m*n + n*n floats) and 3 n*n FP64 temporaries of the
  // mixed-precision Jacobi (n = min(h, c)).
  return 2 * a32(h * c) + 4 * a32(c * c) + 2 * a32(h * h) + 6 * a32(imax64(h, c)) +
         a32(h * c) + 4 * a32(mn * mn);
}
// right_qr_step on a core (r, w = n*rp) with previous core of h_prev rows.
TTG_HD inline int64_t need_right_qr(int64_t r, int64_t w, int64_t h_prev)
{
  return a32(w * r) + a32(r) + a32(r * r) + a32(h_prev * r);
}
// left_qr_step on a core (h = r*n, rp) with next core of w_next columns.
TTG_HD inline int64_t need_left_qr(int64_t h, int64_t rp, int64_t w_next)
{
  return a32(h * rp) + a32(rp) + a32(rp * rp) + a32(rp * w_next);
}
TTG_HD inline int64_t need_svd_step(int64_t h, int64_t c, int64_t w_next)
{
  return a32(c * w_next) + need_left_svd(h, c);
}
TTG_HD inline int64_t need_svd_step_right(int64_t w, int64_t r, int64_t h_prev)
{
  return a32(h_prev * r) + need_left_svd(w, r);
}
// One bond of soft_threshold: the merged pair M (h = rL*n_prev rows,
// c = n_cur*rR columns) and its SVD.
TTG_HD inline int64_t need_soft_step(int64_t h, int64_t c)
{
  return a32(h * c) + need_left_svd(h, c);
}
// One streaming step: F buffer capacity fcap, F rows alpha, operator core
// (a, m, p, b), operand core (sx, p*nout, bx).
TTG_HD inline int64_t need_stream_step(int64_t fcap, int64_t alpha, int64_t a, int64_t m,
                                       int64_t p, int64_t b, int64_t sx, int64_t nout,
                                       int64_t bx)
{
  const int64_t g1p = alpha * m * b * sx * p;
  const int64_t c2 = alpha * m * b * nout * bx;
  return a32(fcap) + a32(alpha * sx * a) + a32(alpha * sx * m * p * b) + a32(g1p) + 2 * a32(c2) +
         need_left_svd(alpha * m * nout, b * bx);
}

struct CoreSlot
{
  int64_t off;  // slot start in the arena (doubles)
  int32_t n;    // mode size as stored (n, or m*n for a TT-matrix core)
  int32_t r;    // current left rank (updated by the sweeps)
  int32_t rp;   // current right rank
  int32_t m;    // row mode of a TT-matrix core (0 for a TT core)
};

struct TTInfo
{
  int32_t first;   // index of core 0 in the slot table
  int32_t d;
  int32_t status;  // ttg_status
  int32_t sweeps;  // largest Jacobi sweep count met
  double norm;     // ||T|| computed by the sweep
  double delta;    // truncation threshold used
  int32_t sketch_state;  // 0 exact round, 1 sketch accepted, 2 sketch rejected -> exact
  int32_t pad;
  double sketch_err;     // ||X - Y|| / ||X|| of the sketch projection
  // Iterative rounding (kJobAls / kJobDmrg), on the start TT's record:
  int32_t iters_run;     // sweeps pairs run
  int32_t iter_conv;     // 1 when the change fell to tol
  double final_change;   // last max relative change of the bond spectra
  int64_t env_off;       // arena offset of the item's environments and spectra
  int64_t env_stride;    // doubles per environment matrix (>= max X rank * max Y rank)
};

// Per-bond record written by the exact rounder when RoundJob::bond_stats is
// set: the bond's largest singular value, the smallest kept one, the chosen
// rank and the number of singular values (indexed by the core left of the
// bond).
struct BondStat
{
  double s_max;
  double s_last;
  int32_t r_new;
  int32_t n_sv;
};

enum JobKind : int32_t
{
  kJobRound = 0,          // round (gauge none): R->L QR, L->R SVD, balance
  kJobRoundRight = 1,     // round_right_canonical: L->R QR, R->L SVD
  kJobRightOrth = 2,      // right_orthogonalize only
  kJobStreamMatvec = 3,   // build_streaming_matvec (pairs of TTs)
  kJobStreamMatmat = 4,   // build_streaming_matmat
  kJobRoundSketch = 5,    // randomised sketch rounding with an exact check and fallback
  kJobSoftThreshold = 6,  // right_orthogonalize, then R->L singular-value soft thresholding
  kJobLeftOrth = 7,       // left_orthogonalize only (the L->R QR sweep)
  kJobAls = 8,            // ALS rounding of TT a_idx[i] into the start TT b_idx[i]
  kJobDmrg = 9,           // two-site DMRG rounding, same pairing
};

// Grid barrier word of the whole-GPU kernel (zeroed before each launch).
struct GridBar
{
  unsigned int count;
  unsigned int gen;
  int err;
  int pad;
};

// Whole-GPU rounding of a few large TTs (wide_round_kernel): the arena,
// slots and TT records as in RoundJob, plus grid-shared work buffers sized
// for the largest core (core_max doubles) and rank (c_max).
struct WideJob
{
  double* arena;
  CoreSlot* slots;
  TTInfo* tts;
  const int* order;
  int ntt;
  int max_rank;
  int max_sweeps;
  int jblock;          // Jacobi block width (columns)
  int teams;           // groups of CTAs, each rounding its own TTs (1 = whole grid)
  int rank, size;      // this CTA's rank in its team and the team size (set on the device)
  int64_t team_bytes;  // stride between the teams' work-buffer blocks
  int mixed;           // 1: FP32 + df64 SVD sweeps
  int tc;              // 1: contractions with K <= 512 on the tensor cores (sliced BF16)
  int kind;            // kJobRound or kJobStreamMatvec / kJobStreamMatmat
  int stall_waits;     // failure-path tests only: no grid barrier completes
  long long wait_cycles;  // limit of one grid-barrier wait (clock cycles)
  const int* a_idx;    // streaming: operand and output TT of each item
  const int* b_idx;
  const int* out_idx;
  double* S1;          // streaming: two contraction/permutation buffers
  double* S2;
  double* Fs;          // streaming: the running F factor
  int64_t smem_doubles;
  double eps;
  double* W;           // core_max: reflectors
  double* Ub;          // core_max: U / work columns
  double* Pb;          // core_max: contraction output
  double* A;           // core_max: Jacobi matrix
  double* R;           // c_max^2
  double* V;           // c_max^2
  double* F;           // c_max^2
  double* T1;          // c_max^2: FP32 V of the mixed SVD
  double* T2;          // c_max^2: FP64 copy of it
  double* tau;         // c_max
  double* sig;         // c_max
  double* sorted;      // c_max
  int* ord;            // c_max
  double* cn;          // sum of ranks: balancing column norms
  int* ival;           // [0] = truncation rank of the current bond
  double* part;        // one partial sum per CTA
  unsigned long long* umax;  // grid-wide max of |x| bit patterns
  unsigned int* sweep_rot;  // max_sweeps
  unsigned int* sweep_rel;  // max_sweeps
  GridBar* bar;        // one barrier word per team
  BondStat* bond_stats;
};

struct RoundJob
{
  double* arena;
  CoreSlot* slots;
  TTInfo* tts;
  const int32_t* order;  // processing order (longest first)
  int32_t ntt;           // number of work items
  int32_t kind;
  double* scratch;
  int64_t scratch_stride;  // doubles per CTA
  int32_t* queue;          // work counter (reset before each run)
  double eps;
  int32_t max_rank;
  int32_t max_sweeps;
  int32_t smem_doubles;  // dynamic shared memory per CTA (doubles) for staging
  int32_t mixed;         // 1: FP32 Jacobi sweeps + FP64 refinement in the SVD steps
  // Streaming jobs: item i rounds the product of TT a_idx[i] (operator) and
  // b_idx[i] (operand) into output TT out_idx[i].  Row/col modes of the
  // operator cores come from CoreSlot::m and n/m.
  const int32_t* a_idx;
  const int32_t* b_idx;
  const int32_t* out_idx;
  // Sketch rounding: per core k (< d-1) the sketch rank of the bond to its
  // right; seed of the Gaussian sketch; the untouched inputs for the exact
  // fallback (arena and slot table of the pristine copy).
  const int32_t* sketch_ranks;
  uint64_t sketch_seed;
  const double* pristine_arena;
  const CoreSlot* pristine_slots;
  BondStat* bond_stats;  // optional per-bond spectrum summary of the exact rounder
  // Iterative rounding: sweep-pair limit, convergence tolerance on the
  // change of the bond spectra, and whether the start TT is already
  // right-orthogonal (round_right_canonical cold start).
  int32_t max_iters;
  int32_t x_right_canonical;
  double tol;
};

// Scratch of one CTA for ALS / DMRG on a TT with Y's dims (ry, n) and the
// start TT's bond capacities (cx): environments, local updates, QR steps,
// merged pairs and their SVDs.
TTG_HD inline int64_t need_iter(int d, const int* ry, const int* n, const int* cx, bool dmrg)
{
  int64_t need = 64;
  for (int k = 0; k < d; ++k)
  {
    const int64_t yr = ry[k], yrp = ry[k + 1], nk = n[k], xr = cx[k], xrp = cx[k + 1];
    const int64_t big = (yr > xr ? yr : xr) * (yrp > xrp ? yrp : xrp) * nk;
    int64_t t = 3 * a32(big) + a32(yr * xr) + a32(yrp * xrp);
    const int64_t hp = k > 0 ? static_cast<int64_t>(cx[k - 1]) * n[k - 1] : 0;
    const int64_t wn = k + 1 < d ? static_cast<int64_t>(n[k + 1]) * cx[k + 2] : 0;
    t = imax64(t, need_left_qr(xr * nk, xrp, wn));
    t = imax64(t, need_right_qr(xr, nk * xrp, hp));
    t = imax64(t, need_left_svd(xr * nk, xrp) + a32(xr * nk * xrp));
    if (dmrg && k + 1 < d)
    {
      const int64_t n1 = n[k + 1], yr2 = ry[k + 2], xr2 = cx[k + 2];
      const int64_t rows = xr * nk, cols = n1 * xr2;
      const int64_t m = a32(xr * nk * yrp) + a32(yrp * n1 * xr2) + a32(rows * cols);
      t = imax64(t, m + need_left_svd(rows, cols) + need_left_svd(cols, rows));
      (void)yr2;
    }
    need = imax64(need, t);
  }
  return need + 64;
}

// Scratch of the sketch phase of one TT (inner-product chain, stored right
// environments, one L->R sketch step); the deterministic round that follows
// uses the ordinary round need.  rmax = largest bond rank, lsum = sum over
// bonds of r_k * l_k, lmax = largest sketch rank, hmax = largest r_k * n_k,
// nmax = largest mode.
// gsum: sum of r_k^2 over the bonds k = 1..d-1 (the stored right Grams).
TTG_HD inline int64_t need_sketch(int64_t rmax, int64_t lsum, int64_t lmax, int64_t hmax,
                                  int64_t nmax, int64_t gsum)
{
  return a32(gsum) + a32(rmax * nmax * rmax) + a32(1) + a32(lsum) + a32(lmax * nmax * lmax) +
         a32(hmax * lmax) + 3 * a32(hmax * lmax) + a32(lmax) + a32(lmax * lmax) +
         a32(lmax * rmax) + a32(lmax * nmax * rmax) + 2 * a32(hmax * rmax) + 64 * 8;
}

}  // namespace ttg
