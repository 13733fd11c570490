// hsr_kernels.h -- kernel argument block and launch wrappers shared by the
// host orchestration (hsr_host.cu) and the kernels (hsr_kernels.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace hsr {

// Device-resident state of one solve over S shifts.  Layouts:
//   H   n x n column-major (ldh even, 16-byte aligned base: TMA source)
//   X   n x S column-major, the eigenvector block (ldx)
//   R   n x S column-major, running crossover columns (ldr)
//   Cr, Sr  Givens rotations, row-major [n][Spad]: Cr[i*Spad + k]
//   beta, ynorm  per-(tile, shift) scaling factor and bound, [T][Spad]
//   W, Zs  stage operands [tlsz][Spad]: crossover coefficients and the
//          rotated solved tile (row 0 of Zs is zero)
//   Zslow  rescaled copies of Ytilde2 for columns needing overflow
//          protection, [(T*tlsz)][Spad] indexed by (I*tlsz + q)
// For complex shifts (hsr_cplx.cu) S counts real columns: pair p occupies
// columns 2p (real part) and 2p+1 (imaginary part) of every array above and
// of the per-column scalars; wr holds (Re mu_p, Im mu_p) at 2p, 2p+1; the
// cosine of a rotation is Cr[.][2p] and its complex sine Sr[.][2p] +
// i Sr[.][2p+1]; beta, ynorm, slow and pert of pair p sit at column 2p.
struct DevProblem {
    int n, T, S, Spad, tlsz;
    const int *fr;             // first row of each tile, [T+1]
    const double *H;
    long long ldh;
    const double *wr;          // shifts [S]
    double *X;
    long long ldx;
    double *R;
    long long ldr;
    double *Cr, *Sr;
    double *beta, *ynorm;
    const double *Hn;          // ||H(I,J)||_oo, [T*T], Hn[I + J*T]
    const double *hn;          // ||H(I, fr[J]-1)||_oo, [T*T]
    double *W, *Zs;
    double *pi, *ytil, *z2n, *zlast;   // per-shift stage scalars [Spad]
    double *Zslow;
    unsigned char *slow;       // [T][Spad], column needs the protected path
    unsigned char *pert;       // [Spad], 1x1 solve perturbed
    double smlnum;
    int is;                    // integer (base-2 exponent) scaling factors
    int *err;                  // device error word
    // Used by the batched kernels, where every problem carries its own:
    double *colnorm;           // [S] 2-norm before normalisation
    int *status;               // [S] 1 converged
    double *scale;             // [S] reconciled scaling factor
    unsigned long long *nbits; // [2*T*T + 2]: Hn, hn, ||H||_oo, eps3 (as bit patterns)
    int *nanflag;              // [2]
};

// Work item of a batched kernel: x = problem, y = tile stage J (or -1),
// z, w = block indices whose meaning depends on the kernel.
typedef int4 BatchItem;

// Raise a kernel's dynamic shared-memory limit to at least `smem`; the limit
// only grows (one lock for all kernels).  `configured` is the kernel's cache.
cudaError_t raise_smem_limit(const void *func, size_t *configured, size_t smem);

// Setup: tile norms, eps3 = ||H||_oo * eps/2.  hnbits/Hnbits/hnorm_bits are
// zeroed by the caller.
cudaError_t launch_norms(const DevProblem &P, unsigned long long *Hn_bits,
                         unsigned long long *hn_bits, unsigned long long *hinf_bits,
                         int *nan_flag, cudaStream_t st);
// Initial state.  mode 0: start vector eps3; 1: restart vector (its);
// 2: caller right-hand sides already in X.
cudaError_t launch_init(const DevProblem &P, int mode, const double *eps3_dev,
                        int its, cudaStream_t st);
cudaError_t launch_diag(const DevProblem &P, int J, int b, double *gscratch, cudaStream_t st);
// Few shifts: tile J's diagonal solve preceded, in the same CTAs, by the GEMM
// of stage J+1 over tile J's rows (Pg: the descriptor with stage J+1's
// operands; b: tile J's height).  Returns false, launching nothing, where
// the wide diagonal form applies; otherwise *err holds the launch status.
bool launch_diag_fused(const DevProblem &P, const DevProblem &Pg, int J, int b, cudaStream_t st,
                       cudaError_t *err);
// Top-GEMM form of the narrow diagonal kernel: fused (true) or a separate
// launch -- the HSR_FUSED_TOP override, else this thread's autotuning trial
// (-1: none), else the tuned entry of the nearest shift count, else fused.
bool fused_top_for(int S);
void set_fused_top_trial(int on);
void record_fused_top(int S, bool on);
// Shifts per CTA the diagonal kernel uses for S shifts: 8, 16 or 32 -- the
// HSR_DIAG_SHIFTS_PER_CTA override, else this thread's autotuning trial, else
// the tuned entry of the nearest shift count (record_diag_shifts), else a rule
// by how many SMs the 32-shift CTAs would fill.
int diag_shifts_per_cta(int S);
void set_diag_shifts_trial(int sc);      // 0 ends the trial
void record_diag_shifts(int S, int sc);
size_t diag_smem_bytes(int b);
// CTAs per SM of the diagonal kernels with v/y in shared memory (0: v/y do
// not fit).  More CTAs than one resident wave -> v/y go to global scratch.
int diag_ctas_per_sm(int b);
int diag_c_ctas_per_sm(int b);
cudaError_t launch_part1(const DevProblem &P, int J, cudaStream_t st);
// Crossover/update GEMM of stage J over rows [row_lo, row_hi) (row_hi <= fr[J]).
cudaError_t launch_gemm(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                        const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st);
size_t gemm_smem_bytes();
// The same GEMM with 16-column tiles (tmW/tmZ with a 16 x 16 box), for the
// short GEMM that gates the next diagonal solve when 64-column tiles would
// leave most SMs idle (gemm_prefers_narrow).
cudaError_t launch_gemm_narrow(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                               const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st);
bool gemm_prefers_narrow(int rows, int S);
cudaError_t launch_finalize(const DevProblem &P, double *colnorm, int *status,
                            double *scale_out, cudaStream_t st);
cudaError_t launch_normalize(const DevProblem &P, const double *colnorm,
                             const int *status, cudaStream_t st);
// Column gather: dst(:, j) = src(:, perm[j]) for j < cnt.
cudaError_t launch_gather_cols(double *dst, long long ldd, const double *src,
                               long long lds, int n, const int *perm, int cnt,
                               cudaStream_t st);
// Batched kernels: one launch covers work items of many problems.  p indexes
// the descriptor array; a problem has two descriptors (stage operands of
// even and odd tiles, as in the single-problem look-ahead).
//   norms:    (p, 0, row block, 0)       row sums over all columns and per tile
//   init:     (p, 0, column, 0)          start vector eps3 (from the norms)
//   diag:     (p, J, shift block, 0)
//   part1:    (p, J, shift block of kPart1Shifts, 0) over all tiles I < J
//   gemm:     (p, J, row block [| kGemmTopFlag], column block): rows of tile
//             J-1, [fr[J-1], fr[J]), with the flag; rows [0, fr[J-1]) without
//   finalize: (p, 0, shift block, 0)
//   normalize:(p, 0, column block of 8, 0)
// `maps` holds three tensor maps per descriptor: H, W, Zs.
cudaError_t launch_norms_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st);
cudaError_t launch_init_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st);
cudaError_t launch_diag_b(const DevProblem *probs, const BatchItem *items, int n_items, int bmax,
                          cudaStream_t st);
cudaError_t launch_part1_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st);
cudaError_t launch_gemm_b(const DevProblem *probs, const BatchItem *items, int n_items, const CUtensorMap *maps,
                          cudaStream_t st);
cudaError_t launch_finalize_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st);
cudaError_t launch_normalize_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st);
constexpr int kNormRows = 128;        // rows per norms item
constexpr int kNormalizeCols = 8;     // columns per normalize item
constexpr int kPart1Shifts = 256;     // shifts per part-1 block (a lane per shift)

// Persistent batched engine.  One cooperative launch of `grid` CTAs (all
// resident at once) works through `items` in list order: each CTA takes the
// next index from *ticket, waits until the counters its item depends on reach
// their targets, runs the item, and adds one to the item's own counter.  The
// list is in a topological order of those dependencies, so the lowest
// unfinished item can always run.  Waits are bounded: a wait that gives up
// records kErrQueueTimeout in *err, and every other wait then stops at once,
// so the launch always ends.
enum QueueKind : int { qkNorms = 0, qkInit, qkDiag, qkPart1, qkGemm, qkFinal, qkNormalize };
struct QueueItem {
    BatchItem it;     // as in the batched kernels; qkInit: z = group of kQueueInitCols columns,
                      // qkDiag: z = group of queue_diag_warps() 32-shift blocks,
                      // qkFinal: z = group of kQueueFinalBlocks 32-shift blocks
    int kind, ctr;    // what runs; the counter it completes
    int dep0, tgt0;   // wait until ctr[dep0] >= tgt0 (dep0 < 0: none)
    int dep1, tgt1;
    int pad0, pad1;
};
constexpr int kQueueInitCols = 8;
constexpr int kQueueFinalBlocks = 2;
constexpr int kQueueThreads = 256;
// Diagonal blocks one item runs (a warp each, v/y in shared memory) for tile
// height up to bmax, and the shared memory of the persistent kernel.
int queue_diag_warps(int bmax);
size_t queue_smem_bytes(int bmax);
// Largest grid that keeps every CTA resident (0 when the kernel cannot run).
int queue_max_grid(int bmax);
cudaError_t launch_queue(const DevProblem *probs, const QueueItem *items, int n_items, const CUtensorMap *maps,
                         int *ctr, int *ticket, int *err, int bmax, int grid, cudaStream_t st);

// Complex-conjugate shifts (hsr_cplx.cu).  The problem's S counts real
// columns: pair p owns columns 2p (real part) and 2p+1 (imaginary part), and
// P.wr holds the shifts interleaved the same way.
cudaError_t launch_init_c(const DevProblem &P, int mode, const double *eps3_dev, int its, cudaStream_t st);
// Shared memory of k_diag_c for tile height b; *global_vy tells whether v/y
// need the global scratch region of 4*32*b doubles per 32 pairs instead.
size_t diag_c_smem_bytes(int b, bool *global_vy);
cudaError_t launch_diag_c(const DevProblem &P, int J, int b, double *gscratch, cudaStream_t st);
cudaError_t launch_part1_c(const DevProblem &P, int J, cudaStream_t st);
cudaError_t launch_gemm_c(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                          const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st);
// colnorm/status per column (both columns of a pair), scale_out per pair.
cudaError_t launch_finalize_c(const DevProblem &P, double *colnorm, int *status, double *scale_out,
                              cudaStream_t st);

// Bounded-wait self-test: a wait that cannot complete, given up after
// `limit` polls with kErrWaitTimeout recorded in *err.
cudaError_t launch_wait_selftest(int *err, long limit, cudaStream_t st);

// FP64 throughput probe kernels.
cudaError_t launch_probe_dfma(double *out, int blocks, int iters, cudaStream_t st);
cudaError_t launch_probe_dmma(double *out, int blocks, int iters, cudaStream_t st);
// Integer-pipe two-quotient division against the FP64 division; cnt[4]
// (zeroed by the caller) receives the mismatch counts, the integer-path
// count and the total.
cudaError_t launch_selftest_arith(unsigned long long per_thread, unsigned long long seed, unsigned long long *cnt,
                                  int blocks, cudaStream_t st);

constexpr int kGemmBM = 64, kGemmBN = 64, kGemmKC = 16, kGemmStages = 3;
constexpr int kGemmBNNarrow = 16;       // column tile of the narrow GEMM (launch_gemm_narrow)
constexpr int kGemmTopFlag = 1 << 30;   // batched GEMM item: rows of tile J-1

}  // namespace hsr
