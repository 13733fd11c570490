/*
 * hsrq3in_gb300.h -- C ABI of the GB300 (sm_103a) robust level-3 inverse
 * iteration library (libhsrq3in_gb300.so).
 *
 * All entry points use plain C types: pointers, sizes and status codes.
 * Matrices are column-major, FP64.  Citations name the interface of the
 * reference (hsrq3in) that each entry point replaces or extends.
 */
#ifndef HSRQ3IN_GB300_H
#define HSRQ3IN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
    HSR_OK = 0,
    HSR_ERR_ARG = -1,          /* invalid argument (n, ld, tlsz, ...)            */
    HSR_ERR_NOMEM = -2,        /* device or host allocation failed               */
    HSR_ERR_CUDA = -3,         /* a CUDA runtime call failed                     */
    HSR_ERR_DEVICE = -4,       /* a kernel reported an internal error            */
    HSR_ERR_NOT_CONVERGED = 1  /* finished; some columns did not converge        */
};

/* Status of the last call made on this host thread (0 = success). */
int hsr_last_status(void);
/* Human-readable text for a status code. */
const char *hsr_status_string(int status);

/* ---------------------------------------------------------- drop-in call */
/* Replaces tiled_inverse_iteration (inverse_iteration.h:19-22, implemented at
 * inverse_iteration.c:128-335).  Same arguments, layout and semantics:
 *   n       order of the upper-Hessenberg matrix H, n > 0
 *   H       n x n, column-major, leading dimension ldH >= n (read only)
 *   nrhs    number of real shifts
 *   wr      [nrhs] shifts; reordered (converged columns first) only when some
 *           columns needed a restart, as inverse_iteration.h:10 allows
 *   tlsz    row tile size, a positive multiple of 4; the first tile is the
 *           short one (partition.c:7-17)
 *   rhs_tlsz  column tile size (> 0); accepted for compatibility -- the
 *           device path computes every column independently
 *   vr      n x nrhs output, leading dimension ldvr >= n; column k is the
 *           unit-2-norm eigenvector for wr[k]
 * Runs on the current CUDA device.  Returns nothing, like the reference;
 * hsr_last_status() reports errors and non-convergence. */
void tiled_inverse_iteration(int n, const double *H, int ldH, int nrhs,
                             double *wr, int tlsz, int rhs_tlsz, double *vr,
                             int ldvr);

/* ---------------------------------------------------- extended host call */
/* Representation of the overflow-protection scaling factors
 * (robust.c:24-121, utils.h:17-21). */
enum {
    HSR_SCALING_POW2 = 0,   /* default: exact powers of two, kept as base-2 exponents
                               (the reference's -DINTSCALING build).  Scale factors
                               cannot underflow, so heavily rescaled columns stay
                               finite. */
    HSR_SCALING_DOUBLE = 1  /* the reference's default build: factors such as 0.5/x
                               kept as doubles; products of many of them underflow
                               to 0 and give NaN, exactly as the reference does.   */
};
/* On every input where no protection decision fires (all unreduced Hessenberg
 * inputs of the benchmark configurations) both representations give
 * bit-identical results. */

typedef struct hsr_options {
    int scaling;       /* HSR_SCALING_POW2 (0, default) or HSR_SCALING_DOUBLE    */
    int user_rhs;      /* 0: eps3 start vectors (inverse_iteration.c:19-34);
                          1: vr holds caller right-hand sides on entry, one
                             solve, no restart (shifted_Hessenberg_solve.h:26) */
    int max_restarts;  /* < 0: up to n rounds as inverse_iteration.c:229       */
    double hbm_budget_bytes; /* workspace cap for shift batching; 0 = auto    */
} hsr_options;

/* Per-column outputs (each pointer optional, arrays of length nrhs, in the
 * final column order). */
typedef struct hsr_column_info {
    int *status;            /* 1 converged, 0 not (vrnorms(k,0), shifted_Hessenberg_solve.c:263-273) */
    unsigned char *perturbed; /* 1 if a 1x1 solve was lifted to smin (robust.c:432-435) */
    double *scale;          /* reconciled scaling factor smin (robust.c:58-82); a base-2
                               exponent under HSR_SCALING_POW2 */
    double *tile_scales;    /* optional [num_tiles x nrhs] per-tile scaling factors
                               before reconciliation (shifted_Hessenberg_solve.c:105-123) */
    double *norm;           /* 2-norm before normalisation (shifted_Hessenberg_solve.c:229-260) */
} hsr_column_info;

/* Extended twin of tiled_inverse_iteration with options, per-column outputs
 * (the scaling factors the reference keeps internal) and a status code. */
int hsr_inverse_iteration_ex(int n, const double *H, int ldH, int nrhs,
                             double *wr, int tlsz, int rhs_tlsz, double *vr,
                             int ldvr, const hsr_options *opt,
                             hsr_column_info *info);

/* ------------------------------------------------ device-resident call */
/* Same computation on device pointers (inputs already in HBM), enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  The GEMM reads
 * dH through TMA, which needs an even lddH and a 16-byte aligned base; other
 * inputs are first copied to a padded device buffer.  Synchronises
 * the stream once at the end to read convergence status.  Device arrays
 * d_status/d_scale may be NULL.  Replaces solve_Hessenberg_system_real_shift
 * (shifted_Hessenberg_solve.h:26-30) plus the driver loop. */
int hsr_inverse_iteration_device(int n, const double *dH, int lddH, int nrhs,
                                 double *dwr, int tlsz, double *dvr, int lddvr,
                                 const hsr_options *opt, void *stream,
                                 int *d_status, double *d_scale);

/* ------------------------------------------ complex-conjugate shifts */
/* Extends tiled_inverse_iteration (inverse_iteration.h:19-22) to complex
 * shifts mu_k = wr[k] + i*wi[k], one per conjugate pair, which the reference
 * declares (problemgenerator.h:12-19 returns wi; main.c:95-97 stops at
 * "only real eigenvalues are supported") and provides the robust kernels for
 * (robust.c:370-773) without a driver.  Same tiled Givens RQ of H - mu I and
 * robust back-substitution, in complex arithmetic, on the current device.
 *   vr   n x 2*npairs output (ldvr >= n), the LAPACK dhsein layout: column 2k
 *        holds the real part and column 2k+1 the imaginary part of the
 *        unit-2-norm eigenvector for mu_k (the conjugate vector belongs to
 *        conj(mu_k))
 *   wr, wi  [npairs], not modified: pairs that need a restart are solved
 *        again in place (opt->max_restarts rounds), so column order is kept
 *   info  per pair (status, perturbed, scale, norm; tile_scales unused)
 * One scaling factor per pair (robust.c:370-417); magnitude bounds use
 * |Re| + |Im|.  opt->user_rhs is not supported (HSR_ERR_ARG).            */
int hsr_inverse_iteration_cplx_ex(int n, const double *H, int ldH, int npairs,
                                  const double *wr, const double *wi, int tlsz,
                                  int rhs_tlsz, double *vr, int ldvr,
                                  const hsr_options *opt, hsr_column_info *info);
/* Device-pointer form: dwr, dwi [npairs], dvr n x 2*npairs, enqueued on
 * `stream`; d_status (int) and d_scale (double) are per pair and optional. */
int hsr_inverse_iteration_cplx_device(int n, const double *dH, int lddH, int npairs,
                                      const double *dwr, const double *dwi, int tlsz,
                                      double *dvr, int lddvr, const hsr_options *opt,
                                      void *stream, int *d_status, double *d_scale);

/* Mixed real and complex shifts in one call, as LAPACK dhsein takes them
 * from a real Schur spectrum: m entries (wr[k], wi[k]); a real shift has
 * wi[k] == 0 and gets column k of vr; a conjugate pair occupies entries k,
 * k+1 with wi[k] > 0, wr[k+1] == wr[k], wi[k+1] == -wi[k], and columns k and
 * k+1 receive the real and imaginary parts of the vector for wr[k] + i wi[k].
 * Real shifts run through tiled_inverse_iteration's path and may be
 * reordered among the real positions when a restart was needed (wr updated,
 * columns follow); pairs run through hsr_inverse_iteration_cplx_ex and keep
 * their positions.  status (optional, [m]) is per column.  A malformed pair
 * returns HSR_ERR_ARG.  Extends inverse_iteration.h:19-22 to the wi that
 * problemgenerator.h:12-19 produces. */
int hsr_inverse_iteration_mixed(int n, const double *H, int ldH, int m,
                                double *wr, double *wi, int tlsz, int rhs_tlsz,
                                double *vr, int ldvr, const hsr_options *opt,
                                int *status);

/* Number of kernel launches the last call on this thread enqueued. */
long hsr_last_launch_count(void);

/* Per-kernel-class device timing (CUDA events on the launching stream
 * around every launch and copy), off by default.  hsr_last_kernel_times
 * fills ms[9] and launches[9] for the classes {setup, diagonal, part1, gemm
 * (rows above the next diagonal tile), finalize, other, host-to-device copy,
 * device-to-host copy, gemm of the next diagonal tile's rows} of the last
 * call, and the algorithmic FMA count of its gemm-class launches; returns
 * the number of classes.  No reference counterpart. */
void hsr_set_kernel_timing(int enable);
int hsr_last_kernel_times(double *ms, long *launches, double *gemm_fma);

/* Release cached device workspaces of this thread. */
void hsr_release_workspace(void);

/* ------------------------------------------ Hessenberg reduction (device) */
/* The input step of the solver, on the GPU: replaces the LAPACK dgehrd call
 * of the reference's problem generator (problemgenerator.c:344) for dense
 * inputs.  In place, with LAPACK's layout and reflector convention (dgehd2,
 * dlarfg): on exit the upper-Hessenberg part of dA holds H, column k below
 * the subdiagonal holds v_k(k+2 .. n-1) (v_k(k+1) = 1 implied), dtau[n] the
 * factors, and A = Q H Q^T with Q = H_0 ... H_{n-3}, H_k = I - tau_k v_k v_k^T.
 * Enqueued on `stream`; all pointers are device pointers.  No reference
 * counterpart in the solver itself. */
int hsr_hessenberg_device(int n, double *dA, int lda, double *dtau, void *stream);
/* X <- Q X for the Q of hsr_hessenberg_device (LAPACK dormhr 'L','N'):
 * back-transforms eigenvectors of H to eigenvectors of A, or forms Q from
 * X = I.  dX is n x ncols, leading dimension ldx. */
int hsr_hessenberg_apply_q_device(int n, const double *dA, int lda, const double *dtau,
                                  int ncols, double *dX, int ldx, void *stream);

/* ------------------------------------------------- residuals on the device */
/* Replaces the residual check of validate_real_eigenvectors
 * (validation.c:145-166) for device-resident results: d_res[k] =
 * ||H x_k - wr[k] x_k||_2 / (||H||_F ||x_k||_2) over the Hessenberg part of H,
 * computed with exact power-of-two prescaling so that no input magnitude
 * overflows (NaN for a non-finite H or x_k, +Inf for a zero x_k).  Costs about
 * n^2/2 FMAs per column.  Enqueued on `stream` without synchronising; all
 * pointers are device pointers. */
int hsr_residuals_device(int n, const double *dH, int lddH, int ncols,
                         const double *dwr, const double *dX, int lddX,
                         double *d_res, void *stream);

/* ------------------------------------------------------- batched solves */
/* No counterpart in the reference (it solves one H per call).  Thousands of
 * independent problems of different orders and shift counts are solved
 * together: every problem advances one tile stage per "tick" and each tick
 * launches one batched kernel per phase over all problems, so small problems
 * fill the GPU together.  Per column the arithmetic is exactly that of
 * hsr_inverse_iteration_device with the same tlsz, so each problem's result
 * is bit-identical to solving it alone.  All pointers are device pointers. */
typedef struct hsr_batch_problem {
    int n;              /* order of H, n > 0                                  */
    const double *dH;   /* n x n, leading dimension lddH (even, 16-byte aligned) */
    int lddH;
    int nrhs;           /* number of shifts                                   */
    double *dwr;        /* [nrhs] shifts (reordered only on restart)          */
    double *dvr;        /* n x nrhs output, leading dimension lddvr           */
    int lddvr;
} hsr_batch_problem;

typedef struct hsr_batch_plan hsr_batch_plan;

/* Lay out one device workspace for all problems, build the tick schedule and
 * capture it in one CUDA graph (replayed by every execute).  tlsz: row tile
 * size (multiple of 4, at most 384); 0 picks the autotuned size for this GPU
 * (hsr_autotune_tlsz).  Returns a status code. */
int hsr_batch_plan_create(hsr_batch_plan **plan, int nprob, const hsr_batch_problem *probs,
                          int tlsz, const hsr_options *opt, void *stream);
/* Run the plan on `stream` (one graph launch), then restart the columns that
 * did not converge, problem by problem.  Synchronises the stream. */
int hsr_batch_plan_execute(hsr_batch_plan *plan, void *stream);
/* Tile size, ticks and kernel launches captured in the plan's graph. */
int hsr_batch_plan_info(const hsr_batch_plan *plan, int *tlsz, int *ticks, long *launches);
void hsr_batch_plan_destroy(hsr_batch_plan *plan);

/* Engines of a plan (no reference counterpart; the reference's equivalent is
 * the dependency-driven OpenMP task DAG of shifted_Hessenberg_solve.c:95-313):
 *   HSR_BATCH_ENGINE_TICKS  one CUDA graph of per-phase batched launches; all
 *                           problems advance one stage per tick in lock step.
 *   HSR_BATCH_ENGINE_QUEUE  one persistent cooperative launch (captured in a
 *                           graph with the set-up memsets) that works through a
 *                           device work queue of (problem, stage, block) items;
 *                           an item starts as soon as the items of its own
 *                           problem that it depends on have finished, tracked
 *                           by per-problem counters with bounded waits.
 * Both give bit-identical results.  set_engine builds the queue on first use;
 * `stream` orders that set-up. */
#define HSR_BATCH_ENGINE_TICKS 0
#define HSR_BATCH_ENGINE_QUEUE 1
int hsr_batch_plan_set_engine(hsr_batch_plan *plan, int engine, void *stream);
/* Current engine, work items in the queue, persistent grid size, diagonal
 * blocks per queue item (0 before the queue is built), and whether the
 * persistent launch was captured in the plan's graph (1) or, where the
 * runtime cannot capture a cooperative launch, is issued directly (0). */
int hsr_batch_plan_queue_info(const hsr_batch_plan *plan, int *engine, long *items, int *grid,
                              int *diag_warps, int *in_graph);

/* Plain-path autotuner: times hsr_inverse_iteration_device on the caller's
 * problem (device pointers; dwr is restored, dvr overwritten) for each
 * candidate tlsz in `cand` (ms_out[i], optional, gets candidate i's time),
 * then, at the fastest tlsz, for 8, 16 and 32 shifts per diagonal CTA
 * (spc_ms[0..2], optional), and, where the fastest of those is 8 or 16,
 * with the GEMM of each tile's own rows run inside the diagonal CTAs or as
 * its own launch (fused_ms[1] and fused_ms[0], optional; -1 where it does
 * not apply).  It records the fastest tlsz for order n, the fastest shifts
 * per CTA and top-GEMM form for nrhs shifts (*shifts_per_cta, *top_fused,
 * optional), and returns the tlsz.  A tlsz of 0 passed to
 * tiled_inverse_iteration, hsr_inverse_iteration_ex or
 * hsr_inverse_iteration_device then selects the recorded size of the nearest
 * tuned order within a factor of two (hsr_autotune_plain_tlsz), else a
 * default by order; the diagonal kernel likewise uses the recorded shifts per
 * CTA and top-GEMM form of the nearest tuned shift count.  Every choice gives
 * the same result bit for bit.  The reference takes tlsz from its caller only
 * (main.c:40-44); no reference counterpart. */
int hsr_autotune_plain(int n, const double *dH, int lddH, int nrhs, double *dwr, double *dvr, int lddvr,
                       const int *cand, int ncand, double *ms_out, int *shifts_per_cta, double *spc_ms,
                       int *top_fused, double *fused_ms, void *stream);
int hsr_autotune_plain_tlsz(int n);

/* Tile size for batches whose orders lie in [n_lo, n_hi]: the size that
 * hsr_autotune_batch measured fastest on this GPU for the sample whose order
 * range overlaps [n_lo, n_hi] the most, else a default. */
int hsr_autotune_tlsz(int n_lo, int n_hi);
/* Time a sample batch for each candidate tile size in `cand` and record the
 * fastest for [n_lo, n_hi]; returns it.  ms_out[i] gets candidate i's time. */
int hsr_autotune_batch(int nprob, const hsr_batch_problem *probs, const int *cand, int ncand,
                       double *ms_out, void *stream);

/* ------------------------------------------------------- served requests */
/* A request loop with continuous batching.  Requests (host buffers) are
 * admitted in arrival order while their device footprint fits the HBM budget,
 * copied to the device, and advanced one tile stage per tick together with
 * every other admitted request; requests that arrive while others are on the
 * GPU join at the next tick.  Results are copied back to the request's host
 * vr and wr. */
typedef struct hsr_server_config {
    double hbm_budget_bytes;   /* device pool for admitted requests (0: 40% of free) */
    int tlsz;                  /* row tile size (0: autotuned)                        */
    int max_active;            /* admission cap on concurrent requests (0: 4096)      */
    int scaling;               /* HSR_SCALING_POW2 or HSR_SCALING_DOUBLE             */
} hsr_server_config;

typedef struct hsr_request {
    int n;
    const double *H;        /* host, column-major, leading dimension ldH */
    int ldH;
    int nrhs;
    double *wr;             /* host [nrhs], in/out                         */
    double *vr;             /* host n x nrhs output, leading dimension ldvr */
    int ldvr;
    double arrival_s;       /* arrival time, seconds after the replay starts */
} hsr_request;

typedef struct hsr_server_stats {
    double wall_s;          /* replay wall time                          */
    long ticks;             /* ticks run                                 */
    long launches;          /* kernel launches                           */
    int max_active;         /* largest number of concurrently admitted requests */
    double peak_bytes;      /* largest pool footprint                    */
    double phase_ms[9];     /* device time per phase (norms, init, first
                               diagonal, part1, gemm of tile J-1's rows,
                               next diagonal -- these two on a side stream
                               beside the next phase -- gemm of the rows
                               above, finalize, normalize) when
                               hsr_set_kernel_timing(1) is on; else 0    */
    double flops;           /* 2 n^2 nrhs summed over served requests    */
    double host_wait_s;     /* host time blocked on the device's ticks   */
} hsr_server_stats;

typedef struct hsr_server hsr_server;
int hsr_server_create(hsr_server **srv, const hsr_server_config *cfg);
/* Serve `nreq` requests, each admitted no earlier than its arrival time
 * (wall clock, measured from the call); latency_s[i] = completion time of
 * request i (result on the host) minus its arrival time.  status[i] (optional)
 * is the request's status code. */
int hsr_server_replay(hsr_server *srv, int nreq, hsr_request *reqs, double *latency_s, int *status,
                      hsr_server_stats *stats);
void hsr_server_destroy(hsr_server *srv);

/* ------------------------------------------- no-allocation device call */
/* No counterpart in the reference.  For callers that may not allocate device
 * memory while they run -- a serving process whose device memory is owned by
 * a caching allocator or a fixed pool (where a cudaMalloc would fail or
 * synchronise the device), or a plug-in host that forbids its plug-ins to
 * allocate.  Same computation and results as hsr_inverse_iteration_device with
 * default options (eps3 start vectors, restarts), on device pointers, enqueued
 * on `stream`; every other buffer comes from one file-scope __device__ array
 * of HSR_NOALLOC_SCRATCH_BYTES that each GPU loading the library keeps until
 * the process exits.  Calls no cudaMalloc/cudaFree and allocates no host
 * memory.  Limits: n <= HSR_NOALLOC_MAX_N, nrhs <= HSR_NOALLOC_MAX_NRHS, and
 * the workspace of (n, nrhs, tlsz) must fit the array; anything larger returns
 * HSR_ERR_ARG before any work is enqueued.  The array is shared by all calls:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on a device looks up the array's address on that device;
 * make that first call before any stream capture.  Under CUDA's default lazy
 * module loading that first call also loads the library's kernels and commits
 * the array on the device, so make it before a pool takes the free memory (or
 * set CUDA_MODULE_LOADING=EAGER).  The call returns after the solve has
 * finished (it synchronises `stream`); after a failure it first waits for the
 * work it had enqueued.  hsr_last_status() reports its status.  `status`
 * (host, optional, [nrhs]) receives 1 for converged columns. */
#define HSR_NOALLOC_MAX_N 256
#define HSR_NOALLOC_MAX_NRHS 256
#define HSR_NOALLOC_SCRATCH_BYTES (8u << 20)
int hsr_inverse_iteration_noalloc(int n, const double *dH, int lddH, int nrhs,
                                  double *dwr, int tlsz, double *dvr, int lddvr,
                                  int scaling, void *stream, int *status);

/* ----------------------------------------------------------- diagnostics */
/* Measured FP64 throughput of this GPU (GFLOP/s): a DFMA stream and a DMMA
 * (mma.sync m8n8k4 f64) stream, each timed with CUDA events over `ms_target`
 * milliseconds.  Used as the roofline denominator; no reference counterpart. */
int hsr_probe_fp64_peak(double ms_target, double *dfma_gflops,
                        double *dmma_gflops);

/* Failure-detection self-test: launches one wait on a barrier that can never
 * complete, through the same bounded wait the GEMM uses on its TMA copies.
 * The wait gives up after a short poll limit and records its error bit, the
 * kernel returns, and the call reports HSR_ERR_DEVICE -- the status a real
 * stalled copy would produce -- while the context stays usable.  Returns
 * HSR_OK only if the wait did not report.  No reference counterpart. */
int hsr_selftest_bounded_wait(void *stream);

/* Self-test of the integer-pipe division the diagonal solve's Givens
 * rotation uses for its two quotients in place of two FP64 divisions:
 * 256 threads x 4 per SM each try `per_thread` seeded operand sets (random
 * significands and exponents over the whole normal range, divisor
 * significands near 1 and 2, dividends equal or next to the divisor), divide
 * two dividends by one divisor, and compare both quotients bit for bit with
 * the FP64 division.  counts[0..1] receive the mismatches of the first and
 * second quotient, counts[2] the sets that took the integer path (the rest
 * fall back to the FP64 division), counts[3] the sets tried.  Blocks until
 * done.  No reference counterpart. */
int hsr_selftest_arith(long long per_thread, unsigned long long seed, long long counts[4]);

/* Library version string. */
const char *hsr_version(void);

#ifdef __cplusplus
}
#endif
#endif
