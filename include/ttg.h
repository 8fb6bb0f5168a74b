/* ttg.h -- C-ABI of the GB300 (sm_103a) TT-rounding library (libttgpu.so).
 *
 * Drop-in boundary for the reference's hot path (mva::tensor_train, a
 * header-only C++20 library).  Each entry point names the reference
 * interface it replaces (paths inside the reference project).  The C++20
 * header tensor_train_gb300.hpp re-exposes the reference's own signatures on
 * top of these functions.
 *
 * Data layout (identical to the reference, types/tt_core.hpp:25-212 and
 * types/tt_matrix.hpp:29-36): a TT of order d has ranks r_0..r_d
 * (r_0 = r_d = 1); core k is (r_k, n_k, r_{k+1}) row-major,
 * idx = (a*n_k + i)*r_{k+1} + b.  A TT-matrix core is (r_k, m_k, n_k, r_{k+1})
 * row-major, bit-identical to a TT core of mode m_k*n_k.  Cores are stored
 * back to back in `data`; core k starts at data + offsets[k].
 *
 * Errors: every function returns a ttg_status.  The reference aborts on
 * invalid input (fprintf + abort); the C++ header maps status != TTG_OK to
 * exactly that, while C/ctypes callers get the code and ttg_last_error().
 *
 * No function here falls back to the CPU: without a usable CUDA device every
 * compute entry point returns TTG_ERR_CUDA.
 */
#ifndef TTG_H
#define TTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ttg_status {
  TTG_OK = 0,
  TTG_ERR_ARG = 1,           /* null pointer, negative size, bad enum value */
  TTG_ERR_SHAPE = 2,         /* rank/mode mismatch (shape_check.hpp:29-149) */
  TTG_ERR_METHOD = 3,        /* method not valid for this entry (round.hpp:124-134) */
  TTG_ERR_INDEX = 4,         /* eval index out of range (tt_eval.hpp:34-53) */
  TTG_ERR_NAN = 5,           /* non-finite value met in the sweep */
  TTG_ERR_NOT_CONVERGED = 6, /* Jacobi SVD hit its sweep limit */
  TTG_ERR_TIMEOUT = 7,       /* a bounded device wait gave up */
  TTG_ERR_OOM = 8,           /* device or host allocation failed */
  TTG_ERR_CUDA = 9,          /* CUDA runtime error / no device */
  TTG_ERR_EMPTY = 10,        /* d = 0 where the reference rejects it */
  TTG_ERR_NO_SPACE = 11      /* a size exceeds a fixed capacity */
} ttg_status;

/* round_method (round/round.hpp:33-44). */
typedef enum ttg_method {
  TTG_METHOD_SVD = 0,
  TTG_METHOD_SVD_STREAMING = 1,
  TTG_METHOD_SVD_NAIVE = 2,
  TTG_METHOD_ALS = 3,
  TTG_METHOD_DMRG = 4,
  /* Not in the reference: randomised sketch rounding sized by per-bond
   * sketch ranks (round/ttg_round_batch only).  The sketch is accepted when
   * its projection error is <= eps/4 (checked exactly); the result is then
   * rounded with the remaining budget sqrt(eps^2 - err^2), otherwise the
   * exact SVD round runs. */
  TTG_METHOD_SKETCH = 5
} ttg_method;

/* round_gauge (round/round.hpp:49-53). */
typedef enum ttg_gauge { TTG_GAUGE_NONE = 0, TTG_GAUGE_RIGHT_CANONICAL = 1 } ttg_gauge;

/* Arithmetic of the sweeps.  FP64: every operation in FP64 (the plain
 * rounder).  MIXED: the Jacobi SVD sweeps run in FP32, a Newton-Schulz
 * re-orthogonalisation of the FP32 rotations and df64 (two-float) polish
 * sweeps restore FP64-level accuracy of the singular vectors and values;
 * on the one-CTA-per-TT schedule the Householder QR and the contractions
 * run in df64 as well (FP32 pipes), on the whole-GPU schedule they stay
 * FP64.  Ranks, norms and truncation thresholds are FP64 throughout. */
typedef enum ttg_precision { TTG_PREC_FP64 = 0, TTG_PREC_MIXED = 1 } ttg_precision;

/* Device schedule of a round (gauge none, method svd): one CTA per TT with
 * many TTs in flight, or the whole GPU on one TT at a time (cooperative
 * launch; for a few large TTs).  AUTO picks the whole GPU when a call
 * holds at most 4 TTs with a bond rank of 64 or more. */
typedef enum ttg_schedule {
  TTG_SCHED_AUTO = 0,
  TTG_SCHED_PER_TT = 1,
  TTG_SCHED_WHOLE_GPU = 2,
  TTG_SCHED_TEAMS = 3 /* groups of CTAs (>= 4 each), each on its own TT */
} ttg_schedule;

/* round_options (round/round.hpp:55-105), SVD-relevant fields plus the
 * device-side knobs.  Zero-initialise and set what you need. */
typedef struct ttg_round_options {
  double eps;          /* truncation tolerance (0 = exact up to rounding) */
  int32_t max_rank;    /* 0 = unlimited */
  int32_t method;      /* ttg_method */
  int32_t gauge;       /* ttg_gauge */
  int32_t precision;   /* ttg_precision */
  int32_t max_sweeps;  /* Jacobi sweep limit, 0 = default (40) */
  int32_t schedule;    /* ttg_schedule */
  /* TTG_METHOD_SKETCH: sketch rank of every bond, TT by TT (sum over the
   * tensors of d_i - 1 entries); NULL = the input ranks (no compression). */
  const int32_t* sketch_ranks;
  uint64_t sketch_seed;
  /* Optional: per-bond spectrum summary of the exact rounder, 4 doubles per
   * bond (largest singular value, smallest kept one, chosen rank, number of
   * singular values), TT by TT as sketch_ranks.  Filled when non-NULL. */
  double* bond_stats;
} ttg_round_options;

/* round_result (round/round.hpp:114-119) plus per-call diagnostics. */
typedef struct ttg_round_result {
  int32_t iters_run;     /* 1 for the SVD path (round.hpp:196-203) */
  int32_t converged;     /* 1 unless a Jacobi SVD hit its sweep limit */
  double final_resid;    /* 0 for the SVD path */
  double norm;           /* ||input|| as computed by the sweep */
  double delta;          /* eps*||T||/sqrt(d-1) used for truncation */
  double device_ms;      /* device time of the call's kernels */
  int32_t status;        /* ttg_status of this tensor */
  int32_t jacobi_sweeps; /* largest Jacobi sweep count met */
  int32_t sketch_state;  /* 0 exact round, 1 sketch accepted, 2 sketch rejected (exact ran) */
  int32_t reserved;
  double sketch_rel_err; /* ||X - sketch(X)|| / ||X|| when a sketch ran */
} ttg_round_result;

/* A TT (cols == NULL) or TT-matrix (rows = m_k, cols = n_k) in host memory.
 * Inputs are read only.  Outputs written by the library own their arrays;
 * release them with ttg_free(). */
typedef struct ttg_tensor {
  int32_t d;
  int32_t* ranks;   /* d+1 */
  int32_t* rows;    /* d: n_k (TT) or m_k (TT-matrix) */
  int32_t* cols;    /* d: n_k of a TT-matrix; NULL for a TT */
  int64_t* offsets; /* d+1: core k = data[offsets[k] .. offsets[k+1]) */
  double* data;
  int32_t owned;    /* set by the library on outputs */
} ttg_tensor;

/* ---- library ---------------------------------------------------------- */
const char* ttg_version(void);
const char* ttg_status_string(int32_t status);
/* Message of the last failing call on this thread ("" if none). */
const char* ttg_last_error(void);
/* Number of kernel launches issued by this library since load. */
int64_t ttg_kernel_launches(void);
/* Releases arrays that the library allocated in *t and zeroes *t. */
void ttg_free(ttg_tensor* t);

/* ---- rounding ----------------------------------------------------------
 * Replaces: tt round(const tt&, const round_options&, round_result*)
 *           (round/round.hpp:230-266; engine round/tt_round.hpp:36-134 and
 *           round_right_canonical tt_round.hpp:151-190) and the tt_matrix
 *           overloads (round.hpp:329-425, via pack/unpack
 *           round/tt_matrix_round.hpp:27-72) when in->cols != NULL.
 * Rejects svd_streaming / svd_naive like round_assert_method_for_value
 * (round.hpp:124-134).  Method ALS / DMRG runs the engine of ttg_round_iter
 * with its default iteration options. */
int32_t ttg_round(const ttg_tensor* in, const ttg_round_options* opts, ttg_tensor* out,
                  ttg_round_result* result);

/* ALS and two-site DMRG rounding.
 * Replaces: round(tt, opts) with method als / dmrg (round/round.hpp:230-266
 *           -> round/tt_als.hpp:212-300, round/tt_dmrg.hpp:217-300) and the
 *           tt_matrix overloads (round/tt_matrix_als_round.hpp,
 *           tt_matrix_dmrg_round.hpp), with the iterative fields of
 *           round_options (round.hpp:84-104) in ttg_iter_options.
 * ttg_round / ttg_matvec_round / ttg_matmat_round with method ALS or DMRG
 * use the defaults below.  Start TT as the reference picks it: a compatible
 * warm start; for ALS without max_rank the SVD round at eps (its largest
 * rank becomes max_rank); else round_right_canonical (ALS at eps 0, DMRG at
 * eps) -- or, in ttg_apply_round_iter and the matvec/matmat entries,
 * random(shape, max_rank, seed) when a max_rank is known.  FP64 only.
 * round_result: iters_run, converged, final_resid = the last change of the
 * bond spectra.  DMRG keeps at most min(Y's bond rank, max_rank) per bond
 * (the merged pair has no larger rank; further singular values are
 * rounding noise). */
typedef struct ttg_iter_options {
  int32_t max_iters;      /* sweep pairs, 0 = 20 */
  int32_t reserved;
  double tol;             /* stop when the spectra change by <= tol; 0 = 1e-12 */
  uint64_t seed;          /* random start of the apply variants */
  const ttg_tensor* warm; /* optional warm start (same modes), borrowed */
} ttg_iter_options;
int32_t ttg_round_iter(const ttg_tensor* in, const ttg_round_options* opts,
                       const ttg_iter_options* iter, ttg_tensor* out, ttg_round_result* result);
/* Replaces: matvec_round / matmat_round with method als / dmrg
 * (round/tt_matvec_als_round.hpp, tt_matvec_dmrg_round.hpp,
 * tt_matmat_als_round.hpp, tt_matmat_dmrg_round.hpp): y = round(A x) by the
 * iterative method from a random start (x a TT-matrix: matmat). */
int32_t ttg_apply_round_iter(const ttg_tensor* A, const ttg_tensor* x,
                             const ttg_round_options* opts, const ttg_iter_options* iter,
                             ttg_tensor* out, ttg_round_result* result);

/* Many independent TTs (uneven d, n, ranks) rounded in one persistent
 * launch.  No reference counterpart takes a batch; each element follows
 * round(const tt&, ...) (round/round.hpp:230-266).  `results` may be NULL. */
int32_t ttg_round_batch(int32_t count, const ttg_tensor* ins, const ttg_round_options* opts,
                        ttg_tensor* outs, ttg_round_result* results);

/* Replaces: void right_orthogonalize(tt&) (gauge/tt_orthogonalize.hpp:26-37)
 * and right_orthogonalize(tt_matrix&) (gauge/tt_matrix_orthogonalize.hpp:34-86). */
int32_t ttg_right_orthogonalize(const ttg_tensor* in, ttg_tensor* out);

/* Replaces: void detail::left_orthogonalize(tt&) (gauge/tt_orthogonalize.hpp:39-58),
 *           the gauge sweep of round_right_canonical and of the Python
 *           binding's left_orthogonalize (bind_py/tensor_train/__init__.py:662). */
int32_t ttg_left_orthogonalize(const ttg_tensor* in, ttg_tensor* out);

/* ---- apply + round -----------------------------------------------------
 * Replaces: tt matvec_round(const tt_matrix&, const tt&, const round_options&,
 *           round_result*) (round/matvec_round.hpp:42-91): svd = round(matvec)
 *           (round/tt_matrix_apply_round.hpp:32-38), svd_streaming =
 *           build_streaming_matvec (detail/streaming_apply.hpp:39-110). */
int32_t ttg_matvec_round(const ttg_tensor* A, const ttg_tensor* x, const ttg_round_options* opts,
                         ttg_tensor* out, ttg_round_result* result);

/* Replaces: tt_matrix matmat_round(const tt_matrix&, const tt_matrix&, ...)
 *           (round/matmat_round.hpp:41-93): svd = build_streaming_matmat
 *           (detail/streaming_apply.hpp:115-202), svd_naive =
 *           round_matrix(matmat) (round/tt_matrix_apply_round.hpp:66-72). */
int32_t ttg_matmat_round(const ttg_tensor* A, const ttg_tensor* B, const ttg_round_options* opts,
                         ttg_tensor* out, ttg_round_result* result);

/* Replaces: tt matvec(const tt_matrix&, const tt&) and
 *           tt_matrix matmat(const tt_matrix&, const tt_matrix&)
 *           (apply/tt_matrix_apply.hpp:237-271): the raw rank-multiplying
 *           products, no rounding. */
int32_t ttg_matvec(const ttg_tensor* A, const ttg_tensor* x, ttg_tensor* out);
int32_t ttg_matmat(const ttg_tensor* A, const ttg_tensor* B, ttg_tensor* out);

/* ---- evaluation and inner products ------------------------------------
 * Replaces: std::vector<double> eval_batch(const tt&, const int* idx, int M)
 *           (algebra/tt_eval.hpp:86-112); idx is M x d row-major; out has M
 *           entries (caller-owned). */
int32_t ttg_eval_batch(const ttg_tensor* a, const int32_t* idx, int32_t M, double* out);

/* Replaces: double inner(const tt&, const tt&) and double norm(const tt&)
 *           (algebra/tt_inner.hpp:33-59). */
int32_t ttg_inner(const ttg_tensor* a, const ttg_tensor* b, double* out);
int32_t ttg_norm(const ttg_tensor* a, double* out);

/* Replaces: double frob_norm_apply(const tt_matrix&, const tt&) and
 *           double frob_norm_apply(const tt_matrix&, const tt_matrix&)
 *           (algebra/tt_matrix_frob_norm_apply.hpp:36-98): ||A x||_F, or
 *           ||A B||_F when x is a TT-matrix (cols != NULL). */
int32_t ttg_frob_norm_apply(const ttg_tensor* A, const ttg_tensor* x, double* out);

/* ---- soft thresholding -------------------------------------------------
 * Replaces: tt soft_threshold(const tt&, double tau = 0.0)
 *           (round/tt_soft_threshold.hpp:42-178).  tau <= 0 or d <= 1
 *           return a copy (no device work); a NaN tau is TTG_ERR_ARG (the
 *           reference propagates it into the cores).  Singular values beyond
 *           a bond's current rank (rounding noise of the merged pair) are
 *           never kept. */
int32_t ttg_soft_threshold(const ttg_tensor* in, double tau, ttg_tensor* out);

/* ---- host-side input construction (no device work) --------------------
 * Replaces: tt random(const std::vector<int>& shape, int max_rank,
 *           std::uint64_t seed) (factory/tt_factory.hpp:141-207) when
 *           cols == NULL, and tt_matrix random(row_shape, col_shape, max_rank,
 *           seed) (factory/tt_matrix_factory.hpp:133-191) otherwise.  With
 *           fan_in_scale != 0 each core is multiplied by 1/sqrt(r_k*mode_k)
 *           after drawing. */
int32_t ttg_host_random(int32_t d, const int32_t* rows, const int32_t* cols, int32_t max_rank,
                        uint64_t seed, int32_t fan_in_scale, ttg_tensor* out);
/* The uneven batch member: mt19937_64(seed) draws d ~ U{dmin..dmax},
 * n_k ~ U{2,4,8}, bond ranks ~ U{rmin..rmax}, clips them for feasibility,
 * then fills N(0,1)/sqrt(r_k*n_k) entries from the same stream.  No
 * reference counterpart (the reference has no batched workload). */
int32_t ttg_host_random_uneven(uint64_t seed, int32_t dmin, int32_t dmax, int32_t rmin,
                               int32_t rmax, ttg_tensor* out);
/* Replaces: tt ones(const std::vector<int>&) (factory/tt_factory.hpp:60-78). */
int32_t ttg_host_ones(int32_t d, const int32_t* shape, ttg_tensor* out);
/* Replaces: tt axpby(double, const tt&, double, const tt&)
 *           (algebra/tt_ops.hpp:72-117); add = axpby(1,a,1,b), sub = axpby(1,a,-1,b). */
int32_t ttg_host_axpby(double alpha, const ttg_tensor* a, double beta, const ttg_tensor* b,
                       ttg_tensor* out);
const char* ttg_host_last_error(void);

/* Measured FP64 FMA throughput of the current device (TFLOP/s): a
 * dependent-chain DFMA loop over all SMs, timed with CUDA events.  Used as
 * the roofline denominator of the FP64 kernels.  No reference counterpart. */
int32_t ttg_device_fp64_peak(double* tflops);

/* ---- device-resident plans (inputs already in HBM) --------------------
 * A plan owns a device arena holding a set of tensors; run() executes the
 * sweep on `stream` (a cudaStream_t, NULL = legacy default) without host
 * synchronisation, so it can be timed with events or captured in a graph.
 * No reference counterpart: the reference has no device. */
typedef struct ttg_plan ttg_plan;

int32_t ttg_plan_create_round(int32_t count, const ttg_tensor* ins, const ttg_round_options* opts,
                              ttg_plan** plan);
int32_t ttg_plan_create_matvec_round(const ttg_tensor* A, const ttg_tensor* x,
                                     const ttg_round_options* opts, ttg_plan** plan);
int32_t ttg_plan_create_eval(const ttg_tensor* a, const int32_t* idx, int32_t M, ttg_plan** plan);
/* Re-uploads the inputs given at creation (host -> device) on `stream` into
 * the plan's input arena. */
int32_t ttg_plan_upload(ttg_plan* plan, void* stream);
/* One pass of the hot path: copies the input arena into the work arena
 * (the deep copy of round(const tt&), round/tt_round.hpp:129-134) and runs
 * the sweep on it.  Idempotent: repeated runs give the same result. */
int32_t ttg_plan_run(ttg_plan* plan, void* stream);
/* Autotuner: times the plan's launch configurations on the plan itself
 * (per-TT schedule: 1, 2, 3 or 4 CTAs per SM, i.e. 200, 92, 56 or 38 KB of
 * shared staging and 128, 128, 85 or 64 registers per thread; whole-GPU schedule: Jacobi block widths 2/4/8, and the per-TT
 * schedule as a contender; on the mixed path also with and without the
 * sliced-BF16 tensor-core contractions) and keeps the fastest.  *choice
 * (optional): 1-4 = per TT with that many CTAs per SM, 100 + b = whole
 * GPU with block width b (+1000 with tensor-core contractions), 10000 + t =
 * t teams of CTAs, 0 = nothing to tune.  Synchronises `stream`; drops a captured
 * graph (capture again afterwards). */
int32_t ttg_plan_autotune(ttg_plan* plan, void* stream, int32_t* choice);
/* enable != 0: capture one run (deep copy from the pristine inputs, the
 * sweep launch, its timing events) as a CUDA graph; later ttg_plan_run calls
 * replay it with one cudaGraphLaunch.  enable == 0 drops the graph. */
int32_t ttg_plan_graph(ttg_plan* plan, int32_t enable);
/* Copies results back (device -> host) and synchronises `stream`.
 * For round plans `outs` receives `count` tensors; for eval plans
 * `values` receives M doubles. */
int32_t ttg_plan_download(ttg_plan* plan, void* stream, ttg_tensor* outs, double* values,
                          ttg_round_result* results);
/* Device time (ms) of the sweep kernel of the last run(), from events
 * recorded on the run's stream around that launch alone. */
int32_t ttg_plan_kernel_ms(ttg_plan* plan, float* ms);
/* Schedule the plan's sweep runs on: TTG_SCHED_PER_TT, TTG_SCHED_WHOLE_GPU
 * or TTG_SCHED_TEAMS (0 for plans without a rounding sweep). */
int32_t ttg_plan_schedule(const ttg_plan* plan);
/* Bytes moved host->device by upload and device->host by download. */
int32_t ttg_plan_io_bytes(const ttg_plan* plan, int64_t* h2d, int64_t* d2h);
void ttg_plan_destroy(ttg_plan* plan);

/* ---- rank model of the learned-sketch rounding ---------------------------
 * No reference counterpart.  A 3-layer MLP (in_features -> hidden -> hidden
 * -> 1, ReLU, FP32 parameters and activations, GEMMs on the tensor cores
 * with split-BF16 operands as in ttg_tc_gemm_f32) that maps per-bond
 * features to log(rank); trained on the GPU by these kernels
 * (mean-squared-error gradient + Adam).  forward, gradients and train_step
 * synchronise `stream`.  All row
 * buffers (x: rows x in_features row-major, targets/outputs: rows) are
 * device pointers; parameters (W1|b1|W2|b2|W3|b3, row-major) live on the
 * device and cross to the host only through get/set_params. */
typedef struct ttg_mlp ttg_mlp;
int32_t ttg_mlp_create(int32_t in_features, int32_t hidden, uint64_t seed, ttg_mlp** out);
void ttg_mlp_destroy(ttg_mlp* m);
int32_t ttg_mlp_num_params(const ttg_mlp* m);
int32_t ttg_mlp_get_params(ttg_mlp* m, float* host);
int32_t ttg_mlp_set_params(ttg_mlp* m, const float* host);
int32_t ttg_mlp_forward(ttg_mlp* m, const float* x_dev, int32_t rows, float* y_dev, void* stream);
/* Gradient of the mean squared error at the current parameters (host copy,
 * same layout as the parameters) and the loss; synchronises `stream`. */
int32_t ttg_mlp_gradients(ttg_mlp* m, const float* x_dev, const float* t_dev, int32_t rows,
                          float* grads_host, double* loss_host, void* stream);
/* One Adam step (beta 0.9/0.999) on the mean squared error. */
int32_t ttg_mlp_train_step(ttg_mlp* m, const float* x_dev, const float* t_dev, int32_t rows,
                           float lr, double* loss_host, void* stream);
int64_t ttg_mlp_kernel_launches(const ttg_mlp* m);

/* ---- several devices ---------------------------------------------------
 * No counterpart in the reference, which rounds TTs and evaluates samples
 * one after another on one core (round/tt_round.hpp:60-63,
 * algebra/tt_eval.hpp:86-112).  Independent TTs and independent samples
 * split across devices without any exchange step: each device runs the
 * single-device entry point on its part from its own host thread, and the
 * results land in the caller's host arrays in input order.
 *
 * ttg_shard_plan: the partition used by ttg_round_batch_devices.  TT i goes
 * to part part_of[i] in [0, parts); cost[i] (optional) receives its
 * estimated rounding cost, the algorithmic FLOP count F_round with the input
 * ranks as output ranks.  Longest first, each TT to the least-loaded part
 * (ties to the lower index): the result depends only on the shapes and
 * `parts`, so every process computes the same partition.  Host code only;
 * needs no device. */
int32_t ttg_shard_plan(int32_t count, const ttg_tensor* ins, int32_t parts, int32_t* part_of,
                       double* cost);
/* ttg_round_batch with the TTs partitioned by ttg_shard_plan over the
 * n_dev devices listed in devices[] (a device may appear more than once;
 * its parts then run one after another).  Same options and results as
 * ttg_round_batch, except that opts->bond_stats must be NULL.  On error no
 * output is left allocated. */
int32_t ttg_round_batch_devices(int32_t count, const ttg_tensor* ins,
                                const ttg_round_options* opts, ttg_tensor* outs,
                                ttg_round_result* results, int32_t n_dev, const int32_t* devices);
/* ttg_eval_batch with the M multi-indices split into n_dev contiguous
 * slices (sizes differing by at most one), slice p on devices[p]; the TT is
 * copied to every device. */
int32_t ttg_eval_batch_devices(const ttg_tensor* a, const int32_t* idx, int32_t M, double* out,
                               int32_t n_dev, const int32_t* devices);

/* ---- tensor-core GEMM ---------------------------------------------------
 * No counterpart in the reference (its GEMMs are Eigen products, e.g.
 * detail/contract.hpp:50).  C (M x N, row-major, ldc) = A (M x K) * B (K x N)
 * on the tcgen05 tensor cores, FP32 in and out, FP32 accumulation in TMEM.
 * A(i, p) = A[i*a_rs + p*a_cs], B(p, j) = B[p*b_rs + j*b_cs]; all device
 * pointers.  splits = 1: operands rounded to BF16; splits = 3: each operand
 * split into BF16 hi + lo and the tile accumulates hi*hi + hi*lo + lo*hi
 * (~1e-5 relative).  The rank model's forward and backward GEMMs use this
 * kernel.  Synchronises `stream`; TTG_ERR_TIMEOUT if an MMA completion wait
 * gave up. */
int32_t ttg_tc_gemm_f32(int32_t M, int32_t N, int32_t K, const float* A, int64_t a_rs,
                        int64_t a_cs, const float* B, int64_t b_rs, int64_t b_cs, float* C,
                        int64_t ldc, int32_t splits, void* stream);

/* ---- rounding without device allocation -------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: code running inside another runtime's allocator (a framework
 * plugin that must not call cudaMalloc), work issued while allocation is
 * forbidden, or processes with a fixed device-memory budget.  Rounds one TT
 * (round(const tt&, round_options) semantics, gauge none or right_canonical,
 * FP64) whose cores are already on the device:
 *   ranks[d+1], modes[d]  host arrays describing the input;
 *   in_dev                the input cores back to back (offsets as in
 *                         ttg_tensor), read only;
 *   out_dev               caller-provided device buffer with room for the
 *                         input's total size; receives the rounded cores
 *                         back to back;
 *   out_ranks[d+1]        host array receiving the output ranks.
 * The call allocates nothing: its tables, work copy and scratch live in one
 * file-scope __device__ array of TTG_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this library holds until the process exits.  A TT whose work copy
 * plus scratch exceeds that size, or with d > TTG_NOALLOC_MAX_D, is rejected
 * with TTG_ERR_NO_SPACE and a message in ttg_last_error(); so is any core
 * whose r*n, n*r' or r*n*r' alone exceeds the array.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current, and so does the first call after a cudaDeviceReset
 * (the address is cached per device and context).  No call can be
 * captured into a graph: each copies the ranks to the host and waits for
 * its stream.  All calls share the array and it keeps the
 * last call's contents (every call resets what must start at zero); calls
 * that overlap on the GPU -- on different streams or threads -- race on it
 * and must be serialised by the caller.  The call waits for its own stream
 * to finish (it returns ranks).  Returns TTG_OK, or TTG_ERR_NOT_CONVERGED
 * when a Jacobi SVD reached opts->max_sweeps (ttg_round reports this as
 * round_result.converged = false): the rounded TT is written to out_dev and
 * out_ranks in both cases. */
#define TTG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define TTG_NOALLOC_MAX_D 256
int32_t ttg_round_noalloc(int32_t d, const int32_t* ranks, const int32_t* modes,
                          const double* in_dev, double* out_dev, int32_t* out_ranks,
                          const ttg_round_options* opts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TTG_H */
