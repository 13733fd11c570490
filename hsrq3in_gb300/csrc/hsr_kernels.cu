// hsr_kernels.cu -- sm_103a kernels of the robust level-3 inverse iteration.
//
// One solve sweeps the row tiles J = T-1 .. 0 (tile 0 is the short one,
// partition.c:7-17).  For every J >= 1 three kernels run:
//   k_diag   lane-per-shift: Givens generation of the diagonal tile fused with
//            the robust back-substitution (reduce.c:27-68 + solve-task.c:19-119),
//            then the stage operands W (crossover coefficients) and Zs (rotated
//            solved tile, update-task.c:170-198).
//   k_part1  warp-per-(tile, shift): scale consistency and the rank-1 update
//            with the column left of tile J (update-task.c:68-174), and the
//            Part-2 overflow decision (update-task.c:206-226).
//   k_gemm   TMA-fed DFMA GEMM over H(0:fr[J], fr[J]-1 : fr[J+1]-1) against
//            [W | Zs]; the epilogue advances the crossover columns
//            (reduceOffdiagBlocked, reduce.c:73-143, in prefix-product form)
//            and applies the tile update with its rank-1 crossover term
//            (update-task.c:233-248), folding the new ||Y||_oo bounds.
// Tile 0 runs k_diag in its factor_and_solve_R11 form (solve-task.c:123-225),
// then k_finalize reconciles the scaling factors and back-transforms
// (shifted_Hessenberg_solve.c:153-260) and k_normalize divides by the norm.
//
// FP64 on this part issues at ~2 lane-FMA per clock per SM whether or not a
// lane is active, so sequential per-shift work runs one shift per lane, and
// magnitude maxima run on the integer pipe over |x| bit patterns.
#include "hsr_device.cuh"
#include "hsr_kernels.h"

#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>

namespace hsr {

// Raise a kernel's dynamic shared-memory limit to at least `smem`.  The
// limit only grows, under one lock, so a host thread never lowers it below
// what another thread's launch already relies on.
cudaError_t raise_smem_limit(const void *func, size_t *configured, size_t smem) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (smem <= *configured) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) *configured = smem;
    return e;
}

// Ask for the largest shared-memory carveout for a kernel of the plain
// path's look-ahead.  The GEMM of the rows above (two 74 KB CTAs per SM) and
// the diagonal kernel of the next tile run at the same time; an SM set up
// with a small carveout for whichever CTA arrived first could not take the
// other kernel's CTAs beside it.  HSR_CARVEOUT=0 leaves the default.
cudaError_t prefer_max_shared(const void *func, bool *done) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (*done) return cudaSuccess;
    const char *env = getenv("HSR_CARVEOUT");
    const cudaError_t e = (env && env[0] == '0')
                              ? cudaSuccess
                              : cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                     (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) *done = true;
    return e;
}

// --------------------------------------------------------------- norms
// Row sums of |H| accumulated column by column in order, as LAPACK dlange
// 'I' does (utils.c:155-174): per (row, tile J >= tile(row)) for the tile
// norms, and over all columns for ||H||_oo.
__global__ void k_tile_rowsums(DevProblem P, unsigned long long *Hn_bits,
                               unsigned long long *hn_bits, int *nan_flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y;
    if (i >= P.n) return;
    const int T = P.T;
    int I = T - 1 - (P.n - 1 - i) / P.tlsz;
    if (I < 0) I = 0;
    if (J < I) return;
    const int c0 = P.fr[J], c1 = P.fr[J + 1];
    double sum = 0.0;
    const double *row = P.H + i;
    for (int c = c0; c < c1; ++c) sum += absd(row[(size_t)c * P.ldh]);
    if (sum != sum) atomicOr(nan_flag, 1 << 1);
    atomicMax(&Hn_bits[I + (size_t)J * T], (unsigned long long)__double_as_longlong(sum));
    if (J > I) {
        // hnrm: |H(i, fr[J]-1)| for the Part-1 column (update-task.c:124)
        atomicMax(&hn_bits[I + (size_t)J * T], abs_bits(row[(size_t)(c0 - 1) * P.ldh]));
    }
}

// One thread per row, 32 rows per CTA so the rows spread over many SMs; each
// group of eight columns is loaded before it is added, in column order.
__global__ void __launch_bounds__(32) k_full_rowsums(DevProblem P, unsigned long long *hinf_bits, int *nan_flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double sum = 0.0;
    const double *row = P.H + i;
    const size_t ldh = (size_t)P.ldh;
    int c = 0;
    for (; c + 8 <= P.n; c += 8) {
        double a[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = row[(size_t)(c + q) * ldh];
#pragma unroll
        for (int q = 0; q < 8; ++q) sum += absd(a[q]);
    }
    for (; c < P.n; ++c) sum += absd(row[(size_t)c * ldh]);
    if (sum != sum) atomicOr(nan_flag, 1);
    atomicMax(hinf_bits, (unsigned long long)__double_as_longlong(sum));
}

cudaError_t launch_norms(const DevProblem &P, unsigned long long *Hn_bits,
                         unsigned long long *hn_bits, unsigned long long *hinf_bits,
                         int *nan_flag, cudaStream_t st) {
    dim3 g((P.n + 127) / 128, P.T);
    k_tile_rowsums<<<g, 128, 0, st>>>(P, Hn_bits, hn_bits, nan_flag);
    k_full_rowsums<<<(P.n + 31) / 32, 32, 0, st>>>(P, hinf_bits, nan_flag);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- init
// Start vectors (inverse_iteration.c:19-34 and the dlaein-style restart
// vector :36-57), bounds, unit scaling factors, and the initial crossover
// columns H(:, n-1) with the shift in the last row (reduce.c:276-308).
__global__ void k_init(DevProblem P, int mode, const double *eps3_dev, int its) {
    const int k = blockIdx.y;
    if (k >= P.S) return;
    const double eps3 = *eps3_dev;
    const int n = P.n;
    const double sq = sqrt((double)n);
    const double tmp = eps3 / (sq + 1.0);
    double *x = P.X + (size_t)k * P.ldx;
    double *r = P.R + (size_t)k * P.ldr;
    const double *hl = P.H + (size_t)(n - 1) * P.ldh;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double h = hl[i];
        if (i == n - 1) h = h - P.wr[k];
        r[i] = h;
        if (mode == 0) {
            x[i] = eps3;
        } else if (mode == 1) {
            double v = (i == 0) ? eps3 : tmp;
            if (i == n - 1 - its) v -= eps3 * sq;
            x[i] = v;
        }
    }
    if (blockIdx.x == 0) {
        const double ub = fmax(fmax(eps3, tmp), absd(tmp - eps3 / sq));
        for (int I = threadIdx.x; I < P.T; I += blockDim.x) {
            P.beta[(size_t)I * P.Spad + k] = sc_one(P.is);
            if (mode == 0) P.ynorm[(size_t)I * P.Spad + k] = eps3;
            else if (mode == 1) P.ynorm[(size_t)I * P.Spad + k] = ub;
        }
        if (threadIdx.x == 0) P.pert[k] = 0;
    }
}

// Bounds of caller right-hand sides: ||X(I, k)||_oo (mode 2).
__global__ void k_rhs_bounds(DevProblem P) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + warp;
    const int I = blockIdx.y;
    if (k >= P.S) return;
    const int r0 = P.fr[I], m = P.fr[I + 1] - r0;
    const double *x = P.X + r0 + (size_t)k * P.ldx;
    unsigned long long mx = 0;
    for (int i = lane; i < m; i += 32) mx = umax64(mx, abs_bits(x[i]));
    for (int o = 16; o; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) P.ynorm[(size_t)I * P.Spad + k] = from_bits(mx);
}

cudaError_t launch_init(const DevProblem &P, int mode, const double *eps3_dev, int its,
                        cudaStream_t st) {
    int bx = (P.n + 255) / 256;
    if (bx > 64) bx = 64;
    dim3 g(bx, P.S);
    k_init<<<g, 256, 0, st>>>(P, mode, eps3_dev, its);
    if (mode == 2) {
        dim3 g2((P.S + 7) / 8, P.T);
        k_rhs_bounds<<<g2, 256, 0, st>>>(P);
    }
    return cudaGetLastError();
}

// -------------------------------------------------------------- diagonal
// 32 shifts per CTA, one per lane, and NW warps per CTA.  The FP64 unit is
// per SM sub-partition, so the single-problem kernel (k_diag) runs NW = 4
// or 8 warps and a lone CTA keeps all four sub-partitions busy: warp 0
// evaluates the short scalar chain of each step (Givens, 1x1 solve, overflow
// decisions) and warps 1 .. NW-1 split the vector part (the updates of
// y(0:j-2) and of the running column) by row, one step behind the chain
// (diag_body_pipe).  Where many CTAs share the GPU (the batched engine) one
// warp per CTA does the same work with the fewest FP64 instructions
// (diag_body_1w).  v (running column) and y (solution tile) live in shared
// memory as [row][lane]; columns of H are staged ahead with cp.async and
// read as broadcasts.  Per-warp maxima of |y| and |v| meet in shared memory
// once per step.  When 2*32*b doubles do not fit, v/y live in a global
// scratch region instead (same code, generic pointers).
constexpr int kDiagWarps = 4;     // single-problem path, v/y in global scratch
constexpr int kDiagWarpsSmem = 8; // single-problem path, v/y in shared memory
constexpr int kDiagWarpsB = 1;    // batched path
// Single-problem path, 8 or 16 shifts per CTA: three warps (the chain and
// two row warps) need 3 x 32 x 120 registers, which fit beside the two
// 256-thread CTAs of the concurrent GEMM on one SM (a fourth warp would not,
// and the diagonal CTA would wait for a GEMM CTA to finish).
constexpr int kDiagWarpsNarrow = 3;

constexpr int kDiagBcast = 8;      // per-lane step results broadcast by warp 0
// Staging buffers for columns of H: the pipelined multi-warp body keeps three
// in flight (rows of step j, chain of step j-1, copy for step j-2), the
// single-warp body two.
__host__ __device__ constexpr int diag_col_bufs(int nw) { return nw > 1 ? 3 : 2; }
// Shared memory of everything but v/y: column buffers, per-warp maxima
// [2][nw][2][32] and, with several warps, the broadcast slots.
__host__ __device__ constexpr size_t diag_small_bytes(int b, int nw) {
    return (size_t)(diag_col_bufs(nw) * (b + 1)) * sizeof(double) + (size_t)2 * nw * 2 * 32 * 8 +
           (nw > 1 ? (size_t)kDiagBcast * 32 * 8 : 0);
}
size_t diag_smem_bytes_nw(int b, int nw) {
    const size_t small = diag_small_bytes(b, nw);
    const size_t full = small + (size_t)64 * b * sizeof(double);
    return full <= 200 * 1024 ? full : small;
}
size_t diag_smem_bytes(int b) { return diag_smem_bytes_nw(b, kDiagWarpsSmem); }

// One-warp body of the diagonal kernel for the 32 shifts of block bx, one
// per lane: each step's scalar chain and the row updates run on the same
// warp.  `sm` is the warp's own shared-memory region (diag_small_bytes(b, 1),
// then v/y unless vy_scratch is given); the warp orders its shared-memory
// accesses with __syncwarp only, so several warps of one CTA may each run
// their own block.
__device__ __forceinline__ void diag_body_1w(const DevProblem &P, int J, int bx, double *sm, double *vy_scratch) {
    const int lane = threadIdx.x & 31;
    const int k0 = bx * 32;
    const int k = k0 + lane;
    const bool act = k < P.S;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;

    double *hc = sm;                                          // [2][b+1]
    // Maxima of |y| and |v| over rows 0 .. j-2, double-buffered by step parity: [2][2][32].
    unsigned long long *pmax = reinterpret_cast<unsigned long long *>(sm + 2 * (b + 1));
    double *v, *y;
    if (vy_scratch) {
        v = vy_scratch;
    } else {
        v = sm + 2 * (b + 1) + 2 * 2 * 32;
    }
    y = v + (size_t)32 * b;
#define V(i) v[(size_t)(i) * 32 + lane]
#define Y(i) y[(size_t)(i) * 32 + lane]
#define PMAX(par, which) pmax[((par) * 2 + (which)) * 32 + lane]

    // Load the crossover column and the right-hand side tile, transposed.
    for (int c = 0; c < 32; ++c) {
        const int kc = k0 + c;
        if (kc < P.S) {
            const double *rc = P.R + l + (size_t)kc * P.ldr;
            const double *xc = P.X + l + (size_t)kc * P.ldx;
            for (int i = lane; i < b; i += 32) {
                v[(size_t)i * 32 + c] = rc[i];
                y[(size_t)i * 32 + c] = xc[i];
            }
        } else {
            for (int i = lane; i < b; i += 32) {
                v[(size_t)i * 32 + c] = 1.0;
                y[(size_t)i * 32 + c] = 0.0;
            }
        }
    }

    const double mu = act ? P.wr[k] : 0.0;
    const double smin = fmax(DBL_EPSILON / 2 * absd(mu), P.smlnum);
    const double Hnorm = P.Hn[J + (size_t)J * P.T];
    double beta = act ? P.beta[(size_t)J * Spad + k] : sc_one(is);
    int pert = 0;

    const double *Hd = P.H + l + (size_t)l * P.ldh;          // H(l, l)
    auto stage_col = [&](int col, double *dst) {              // H(l : l+col+1, l+col)
        int rows = col + 2;
        if (rows > b) rows = b;
        const double *src = Hd + (size_t)col * P.ldh;
        for (int i = lane; i < rows; i += 32) cp_async8(dst + i, src + i);
        cp_async_commit();
    };
    if (b >= 2) stage_col(b - 2, hc);
    __syncwarp();                                             // tiles loaded

    // Maxima of |y(0:b-3)| and |v(0:b-3)| for the first step.
    {
        unsigned long long ym = 0, vm = 0;
        for (int i = 0; i < b - 2; ++i) {
            ym = umax64(ym, abs_bits(Y(i)));
            vm = umax64(vm, abs_bits(V(i)));
        }
        PMAX(0, 0) = ym;
        PMAX(0, 1) = vm;
    }
    // v(j) and y(j) of the current step are carried in registers.
    double vcar = V(b - 1), ycar = Y(b - 1);

    int buf = 0, par = 0;
    for (int j = b - 1; j >= 1; --j) {
        cp_async_wait_all();
        __syncwarp();                                         // previous step's rows and column j-1 visible
        const double *hcol = hc + buf * (b + 1);              // column j-1 of the tile
        if (j >= 2) stage_col(j - 2, hc + (buf ^ 1) * (b + 1));
        double c, s, yc, ys, a1, a2, a3, yj, yjm1, hdiag, vjm1;
        {
            unsigned long long ymax = PMAX(par, 0), vmax = PMAX(par, 1);
            const double hsub = hcol[j];
            hdiag = hcol[j - 1] - mu;
            const double vj = vcar;
            vjm1 = V(j - 1);
            yj = ycar;
            yjm1 = Y(j - 1);

            givens(vj, hsub, c, s);
            if (act) {
                P.Cr[(size_t)(l + j) * Spad + k] = c;
                P.Sr[(size_t)(l + j) * Spad + k] = s;
            }
            // y(j) := y(j) / R(j,j) robustly (solve-task.c:76-81).
            double phi = sc_one(is);
            pert |= solve_1x1(smin, c * vj, s * hsub, yj, phi, is);
            beta = sc_combine(beta, phi, is);
            a1 = sc_value(phi, is);
            if (!is_one(a1)) {
                yjm1 = mul_rare(a1, yjm1);
                ymax = abs_bits(mul_rare(a1, from_bits(ymax)));
            }
            // y(j-1) (solve-task.c:84-90).
            phi = protect_double_update(absd(vjm1), absd(yj), absd(hdiag), absd(yj), absd(yjm1), is);
            a2 = sc_value(phi, is);
            if (!is_one(a2)) {
                yj = mul_rare(a2, yj);
                yjm1 = mul_rare(a2, yjm1);
                ymax = abs_bits(mul_rare(a2, from_bits(ymax)));
            }
            beta = sc_combine(beta, phi, is);
            yc = yj * c;
            ys = yj * s;
            yjm1 = fma(ys, hdiag, fma(-yc, vjm1, yjm1));
            // y(0:j-2) (solve-task.c:92-100).
            phi = protect_double_update(from_bits(vmax), absd(yj), Hnorm, absd(yj), from_bits(ymax), is);
            a3 = sc_value(phi, is);
            if (!is_one(a3)) {
                yj = mul_rare(a3, yj);
                yjm1 = mul_rare(a3, yjm1);
                yc = mul_rare(yj, c);
                ys = mul_rare(yj, s);
            }
            beta = sc_combine(beta, phi, is);
        }
        const bool scaled = (!is_one(a1)) || (!is_one(a2)) || (!is_one(a3));
        if (scaled) {
            // Rare: the whole-vector scale() also reaches the solved rows j+1 .. b-1.
            for (int i = j + 1; i < b; ++i) {
                double t = Y(i);
                t = scale_by(a1, t);
                t = scale_by(a2, t);
                t = scale_by(a3, t);
                Y(i) = t;
            }
        }
        unsigned long long ymx = 0, vmx = 0;
        const int lim = j - 1;
        // Rows 0 .. j-2 in batches of 4: loads first, then the independent
        // FMA chains, then the stores.
        int i = 0;
        for (; i + 3 < lim; i += 4) {
            double hh[4], yy[4], vv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                hh[q] = hcol[i + q];
                yy[q] = Y(i + q);
                vv[q] = V(i + q);
            }
            if (scaled) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    yy[q] = scale_by(a1, yy[q]);
                    yy[q] = scale_by(a2, yy[q]);
                    yy[q] = scale_by(a3, yy[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                yy[q] = fma(ys, hh[q], fma(-yc, vv[q], yy[q]));
                vv[q] = fma(c, hh[q], s * vv[q]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = i + q;
                Y(r) = yy[q];
                V(r) = vv[q];
                if (r < lim - 1) {
                    ymx = umax64(ymx, abs_bits(yy[q]));
                    vmx = umax64(vmx, abs_bits(vv[q]));
                }
            }
        }
        for (; i < lim; ++i) {
            const double h = hcol[i];
            double yi = Y(i), vi = V(i);
            if (scaled) {
                yi = scale_by(a1, yi);
                yi = scale_by(a2, yi);
                yi = scale_by(a3, yi);
            }
            yi = fma(ys, h, fma(-yc, vi, yi));
            vi = fma(c, h, s * vi);
            Y(i) = yi;
            V(i) = vi;
            if (i < lim - 1) {
                ymx = umax64(ymx, abs_bits(yi));
                vmx = umax64(vmx, abs_bits(vi));
            }
        }
        PMAX(par ^ 1, 0) = ymx;
        PMAX(par ^ 1, 1) = vmx;
        Y(j) = yj;                                            // the solved entry
        // Next annihilation column entry (solve-task.c:105-108) and y(j-1).
        vcar = fma(c, hdiag, s * vjm1);
        ycar = yjm1;
        buf ^= 1;
        par ^= 1;
    }

    double c0 = 0.0, s0 = 0.0;
    {
        double v0 = b >= 2 ? vcar : V(0);
        const double y0 = b >= 2 ? ycar : Y(0);
        double y0s = y0;
        if (J > 0) {
            // Final rotation with H(l, l-1) (reduce.c:53-61, solve-task.c:111-118).
            const double hleft = P.H[l + (size_t)(l - 1) * P.ldh];
            if (hleft != 0) {
                givens(v0, hleft, c0, s0);
            } else {
                c0 = 1.0;
                s0 = 0.0;
            }
            if (act) {
                P.Cr[(size_t)l * Spad + k] = c0;
                P.Sr[(size_t)l * Spad + k] = s0;
            }
            v0 = fma(v0, c0, -(hleft * s0));
        }
        double phi = sc_one(is);
        pert |= solve_1x1(smin, v0, 0.0, y0s, phi, is);
        beta = sc_combine(beta, phi, is);
        const double a = sc_value(phi, is);
        __syncwarp();                                         // last step's rows written
        if (!is_one(a))
            for (int i = 1; i < b; ++i) Y(i) = a * Y(i);
        Y(0) = y0s;
    }
    __syncwarp();

    // Store the solved tile, its scaling factor and the perturbation flag.
    for (int c = 0; c < 32; ++c) {
        const int kc = k0 + c;
        if (kc < P.S) {
            double *xc = P.X + l + (size_t)kc * P.ldx;
            for (int i = lane; i < b; i += 32) xc[i] = y[(size_t)i * 32 + c];
        }
    }
    if (act) {
        P.beta[(size_t)J * Spad + k] = beta;
        if (pert) P.pert[k] = 1;
    }
    if (J == 0 || !act) return;

    // W(q) = c_q * prod_{p<q} s_p, pi = prod s (crossover propagation).
    {
        double pk = 1.0;
        for (int q = 0; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            P.W[(size_t)q * Spad + k] = cq * pk;
            pk = pk * sq;
        }
        P.pi[k] = pk;
    }
    {
        // Ytilde2 = G_{b-1}^T ... G_1^T (c_0 x_0, x_1, ...) (update-task.c:193-220);
        // Zs(q) = Ytilde2(q-1), Zs(0) = 0, zlast = Ytilde2(b-1).
        unsigned long long zmx = 0;
        double z = c0 * Y(0);
        P.Zs[k] = 0.0;
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            const double t1 = z, t2 = Y(q);
            const double zo = fma(cq, t1, -(sq * t2));
            z = fma(sq, t1, cq * t2);
            P.Zs[(size_t)q * Spad + k] = zo;
            zmx = umax64(zmx, abs_bits(zo));
        }
        zmx = umax64(zmx, abs_bits(z));
        P.zlast[k] = z;
        P.z2n[k] = from_bits(zmx);
        P.ytil[k] = -s0 * Y(0);
    }
#undef V
#undef Y
#undef PMAX
}

// The four-warp diagonal kernel, software-pipelined by one step.  Step j's
// scalar chain (Givens, 1x1 solve, three overflow decisions) runs on warp 0
// and feeds the row updates of step j, which run on warps 1-3; warp 0 first
// updates row j-2 itself and then evaluates the first two parts of step
// j-1's chain -- everything that does not need the new row maxima -- while
// warps 1-3 are still updating rows 0 .. j-3.  After a barrier warp 0 folds
// their maxima into the third decision of step j-1 and publishes that step's
// scalars; a second barrier hands them to warps 1-3.  Every row sees the
// same operations in the same order as in the unpipelined form (and the
// oracle), and the maxima cover the same rows, so the result is unchanged
// bit for bit.  The H column of step j-1 is staged with cp.async two steps
// ahead (three buffers: the rows of step j, the chain of step j-1, the copy
// for step j-2).
template <int NW>
__device__ __forceinline__ void diag_body_pipe(const DevProblem &P, int J, int bx, double *vy_scratch) {
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int k0 = bx * 32;
    const int k = k0 + lane;
    const bool act = k < P.S;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;

    constexpr int NB = diag_col_bufs(NW);                                     // 3 column buffers
    double *hc = sm;                                                          // [NB][b+1]
    unsigned long long *pmax = reinterpret_cast<unsigned long long *>(sm + NB * (b + 1));  // [NW][2][32]
    double *bc = sm + NB * (b + 1) + 2 * NW * 2 * 32;                         // [kDiagBcast][32]
    double *v, *y;
    if (vy_scratch) {
        v = vy_scratch;
        y = v + (size_t)32 * b;
    } else {
        v = bc + kDiagBcast * 32;
        y = v + (size_t)32 * b;
    }
#define V(i) v[(size_t)(i) * 32 + lane]
#define Y(i) y[(size_t)(i) * 32 + lane]
#define PM(w, which) pmax[(((w) * 2) + (which)) * 32 + lane]
#define BC(q) bc[(q) * 32 + lane]
#define HCOL(col) (hc + (size_t)((col) % NB) * (b + 1))

    for (int c = wid; c < 32; c += NW) {
        const int kc = k0 + c;
        if (kc < P.S) {
            const double *rc = P.R + l + (size_t)kc * P.ldr;
            const double *xc = P.X + l + (size_t)kc * P.ldx;
            for (int i = lane; i < b; i += 32) {
                v[(size_t)i * 32 + c] = rc[i];
                y[(size_t)i * 32 + c] = xc[i];
            }
        } else {
            for (int i = lane; i < b; i += 32) {
                v[(size_t)i * 32 + c] = 1.0;
                y[(size_t)i * 32 + c] = 0.0;
            }
        }
    }

    const double mu = act ? P.wr[k] : 0.0;
    const double smin = fmax(DBL_EPSILON / 2 * absd(mu), P.smlnum);
    const double Hnorm = P.Hn[J + (size_t)J * P.T];
    double beta = act ? P.beta[(size_t)J * Spad + k] : sc_one(is);
    int pert = 0;

    const double *Hd = P.H + l + (size_t)l * P.ldh;                           // H(l, l)
    auto stage_col = [&](int col) {                                           // H(l : l+col+1, l+col), warp 0
        int rows = col + 2;
        if (rows > b) rows = b;
        const double *src = Hd + (size_t)col * P.ldh;
        double *dst = HCOL(col);
        for (int i = lane; i < rows; i += 32) cp_async8(dst + i, src + i);
        cp_async_commit();
    };
    if (wid == 0 && b >= 2) stage_col(b - 2);
    if (wid == 0 && b >= 3) stage_col(b - 3);
    if (wid == 0) cp_async_wait_all();
    __syncthreads();                                                          // tiles and columns loaded

    // Maxima of |y(0:b-3)| and |v(0:b-3)| for the first step, by warps 1-3.
    {
        unsigned long long ym = 0, vm = 0;
        if (wid > 0)
            for (int i = wid - 1; i < b - 2; i += NW - 1) {
                ym = umax64(ym, abs_bits(Y(i)));
                vm = umax64(vm, abs_bits(V(i)));
            }
        PM(wid, 0) = ym;
        PM(wid, 1) = vm;
    }

    // Chain state of warp 0.
    double vcar = V(b - 1), ycar = Y(b - 1);
    double c = 0.0, s = 0.0, yc = 0.0, ys = 0.0, a1 = 1.0, a2 = 1.0, a3 = 1.0, yj = 0.0, yjm1 = 0.0;

    // Parts 1-2 of step jj's chain: Givens, the 1x1 solve and the y(jj-1)
    // decision and update (solve-task.c:76-90), and the next running column
    // entry (solve-task.c:105-108).  vjm1, yjm1 enter as row jj-1.
    auto chain12 = [&](int jj, double vjm1, double yjm1_in) {
        const double *hcol = HCOL(jj - 1);
        const double hsub = hcol[jj];
        const double hdiag = hcol[jj - 1] - mu;
        const double vj = vcar;
        yj = ycar;
        yjm1 = yjm1_in;
        givens(vj, hsub, c, s);
        if (act) {
            P.Cr[(size_t)(l + jj) * Spad + k] = c;
            P.Sr[(size_t)(l + jj) * Spad + k] = s;
        }
        double phi = sc_one(is);
        pert |= solve_1x1(smin, c * vj, s * hsub, yj, phi, is);
        beta = sc_combine(beta, phi, is);
        a1 = sc_value(phi, is);
        yjm1 = scale_by(a1, yjm1);
        phi = protect_double_update(absd(vjm1), absd(yj), absd(hdiag), absd(yj), absd(yjm1), is);
        a2 = sc_value(phi, is);
        if (!is_one(a2)) {
            yj = mul_rare(a2, yj);
            yjm1 = mul_rare(a2, yjm1);
        }
        beta = sc_combine(beta, phi, is);
        yc = yj * c;
        ys = yj * s;
        yjm1 = fma(ys, hdiag, fma(-yc, vjm1, yjm1));
        vcar = fma(c, hdiag, s * vjm1);
    };
    // Part 3 of step jj's chain: the y(0:jj-2) decision (solve-task.c:92-100)
    // with the maxima of rows 0 .. jj-2 folded by warps 1-3, then the step's
    // scalars for the row warps, the solved entry y(jj) and y(jj-1).
    auto chain3 = [&](int jj) {
        unsigned long long ymb = 0, vmb = 0;
#pragma unroll
        for (int w = 1; w < NW; ++w) {
            ymb = umax64(ymb, PM(w, 0));
            vmb = umax64(vmb, PM(w, 1));
        }
        double ymax = from_bits(ymb);
        if (!is_one(a1)) ymax = from_bits(abs_bits(mul_rare(a1, ymax)));
        if (!is_one(a2)) ymax = from_bits(abs_bits(mul_rare(a2, ymax)));
        const double phi = protect_double_update(from_bits(vmb), absd(yj), Hnorm, absd(yj), ymax, is);
        a3 = sc_value(phi, is);
        if (!is_one(a3)) {
            yj = mul_rare(a3, yj);
            yjm1 = mul_rare(a3, yjm1);
            yc = mul_rare(yj, c);
            ys = mul_rare(yj, s);
        }
        beta = sc_combine(beta, phi, is);
        BC(0) = c;
        BC(1) = s;
        BC(2) = yc;
        BC(3) = ys;
        BC(4) = a1;
        BC(5) = a2;
        BC(6) = a3;
        Y(jj) = yj;
        ycar = yjm1;
    };

    if (wid == 0 && b >= 2) chain12(b - 1, V(b - 2), Y(b - 2));
    __syncthreads();                                                          // first maxima in
    if (wid == 0 && b >= 2) chain3(b - 1);
    __syncthreads();                                                          // step b-1's scalars visible

    for (int j = b - 1; j >= 1; --j) {
        // Step j's scalars: registers on warp 0, shared memory for the rest.
        double sc_c = c, sc_s = s, sc_yc = yc, sc_ys = ys, s1 = a1, s2 = a2, s3 = a3;
        if (wid != 0) {
            sc_c = BC(0);
            sc_s = BC(1);
            sc_yc = BC(2);
            sc_ys = BC(3);
            s1 = BC(4);
            s2 = BC(5);
            s3 = BC(6);
        }
        const bool scaled = (!is_one(s1)) || (!is_one(s2)) || (!is_one(s3));
        const double *hcol = HCOL(j - 1);
        if (wid == 0) {
            // Row j-2 first: it enters step j-1's chain.
            double vn = 0.0, yn = 0.0;
            if (j >= 2) {
                const double h = hcol[j - 2];
                double yi = Y(j - 2);
                const double vi = V(j - 2);
                if (scaled) {
                    yi = scale_by(s1, yi);
                    yi = scale_by(s2, yi);
                    yi = scale_by(s3, yi);
                }
                yn = fma(sc_ys, h, fma(-sc_yc, vi, yi));
                vn = fma(sc_c, h, sc_s * vi);
                Y(j - 2) = yn;
                V(j - 2) = vn;
            }
            if (j >= 2) {
                cp_async_wait_all();                                          // column j-2, staged last step
                __syncwarp();                                                 // ... by all lanes of warp 0
                chain12(j - 1, vn, yn);
            }
            if (j >= 3) stage_col(j - 3);                                     // for step j-2's chain
        } else {
            if (scaled) {
                for (int i = j + 1 + ((wid - 1 - (j + 1)) % (NW - 1) + (NW - 1)) % (NW - 1); i < b; i += NW - 1) {
                    double t = Y(i);
                    t = scale_by(s1, t);
                    t = scale_by(s2, t);
                    t = scale_by(s3, t);
                    Y(i) = t;
                }
            }
            unsigned long long ymx = 0, vmx = 0;
            const int lim = j - 2;                                            // rows 0 .. j-3
            int i = wid - 1;
            for (; i + 3 * (NW - 1) < lim; i += 4 * (NW - 1)) {
                double hh[4], yy[4], vv[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    hh[q] = hcol[i + q * (NW - 1)];
                    yy[q] = Y(i + q * (NW - 1));
                    vv[q] = V(i + q * (NW - 1));
                }
                if (scaled) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        yy[q] = scale_by(s1, yy[q]);
                        yy[q] = scale_by(s2, yy[q]);
                        yy[q] = scale_by(s3, yy[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    yy[q] = fma(sc_ys, hh[q], fma(-sc_yc, vv[q], yy[q]));
                    vv[q] = fma(sc_c, hh[q], sc_s * vv[q]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = i + q * (NW - 1);
                    Y(r) = yy[q];
                    V(r) = vv[q];
                    ymx = umax64(ymx, abs_bits(yy[q]));
                    vmx = umax64(vmx, abs_bits(vv[q]));
                }
            }
            for (; i < lim; i += NW - 1) {
                const double h = hcol[i];
                double yi = Y(i), vi = V(i);
                if (scaled) {
                    yi = scale_by(s1, yi);
                    yi = scale_by(s2, yi);
                    yi = scale_by(s3, yi);
                }
                yi = fma(sc_ys, h, fma(-sc_yc, vi, yi));
                vi = fma(sc_c, h, sc_s * vi);
                Y(i) = yi;
                V(i) = vi;
                ymx = umax64(ymx, abs_bits(yi));
                vmx = umax64(vmx, abs_bits(vi));
            }
            PM(wid, 0) = ymx;
            PM(wid, 1) = vmx;
        }
        __syncthreads();                                                      // rows of step j done, maxima in
        if (wid == 0 && j >= 2) chain3(j - 1);
        __syncthreads();                                                      // step j-1's scalars visible
    }

    constexpr bool kBcast = true;
    double c0 = 0.0, s0 = 0.0;
    {
        double y0 = 0.0, a = 1.0;
        if (!kBcast || wid == 0) {
            double v0 = b >= 2 ? vcar : V(0);
            y0 = b >= 2 ? ycar : Y(0);
            double hleft = 0.0;
            if (J > 0) {
                // Final rotation with H(l, l-1) (reduce.c:53-61, solve-task.c:111-118).
                hleft = P.H[l + (size_t)(l - 1) * P.ldh];
                if (hleft != 0) {
                    givens(v0, hleft, c0, s0);
                } else {
                    c0 = 1.0;
                    s0 = 0.0;
                }
                if (act && wid == 0) {
                    P.Cr[(size_t)l * Spad + k] = c0;
                    P.Sr[(size_t)l * Spad + k] = s0;
                }
                v0 = fma(v0, c0, -(hleft * s0));
            }
            double phi = sc_one(is);
            pert |= solve_1x1(smin, v0, 0.0, y0, phi, is);
            beta = sc_combine(beta, phi, is);
            a = sc_value(phi, is);
            if (kBcast) {
                BC(0) = c0;
                BC(1) = s0;
                BC(2) = a;
            }
        }
        __syncthreads();                                       // last step's rows (and the scalars) written
        if (kBcast && wid != 0) {
            c0 = BC(0);
            s0 = BC(1);
            a = BC(2);
        }
        if (!is_one(a))
            for (int i = 1 + ((wid - 1) % NW + NW) % NW; i < b; i += NW)
                Y(i) = a * Y(i);
        if (wid == 0) Y(0) = y0;
    }
    __syncthreads();

    // Store the solved tile, its scaling factor and the perturbation flag.
    for (int c = wid; c < 32; c += NW) {
        const int kc = k0 + c;
        if (kc < P.S) {
            double *xc = P.X + l + (size_t)kc * P.ldx;
            for (int i = lane; i < b; i += 32) xc[i] = y[(size_t)i * 32 + c];
        }
    }
    if (act && wid == 0) {
        P.beta[(size_t)J * Spad + k] = beta;
        if (pert) P.pert[k] = 1;
    }
    if (J == 0 || !act) return;

    if (wid == 0) {
        // W(q) = c_q * prod_{p<q} s_p, pi = prod s (crossover propagation).
        double pk = 1.0;
        for (int q = 0; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            P.W[(size_t)q * Spad + k] = cq * pk;
            pk = pk * sq;
        }
        P.pi[k] = pk;
    }
    if (wid == (NW > 1 ? 1 : 0)) {
        // Ytilde2 = G_{b-1}^T ... G_1^T (c_0 x_0, x_1, ...) (update-task.c:193-220);
        // Zs(q) = Ytilde2(q-1), Zs(0) = 0, zlast = Ytilde2(b-1).
        unsigned long long zmx = 0;
        double z = c0 * Y(0);
        P.Zs[k] = 0.0;
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            const double t1 = z, t2 = Y(q);
            const double zo = fma(cq, t1, -(sq * t2));
            z = fma(sq, t1, cq * t2);
            P.Zs[(size_t)q * Spad + k] = zo;
            zmx = umax64(zmx, abs_bits(zo));
        }
        zmx = umax64(zmx, abs_bits(z));
        P.zlast[k] = z;
        P.z2n[k] = from_bits(zmx);
        P.ytil[k] = -s0 * Y(0);
    }
#undef V
#undef Y
#undef PM
#undef HCOL
#undef BC
}


// One element (row, col) of the real GEMM epilogue of the stage whose
// diagonal tile starts at row l (height b): the crossover column advanced by
// pi and the accumulated H W (aw), Part 1 applied where flagged, the tile
// update with the accumulated H Zs (az) or, for protected columns, with the
// rescaled Ytilde2 (update-task.c:233-243), in place in R and X.  I is the
// row's tile and hl1 = H(row, l-1).  Returns |y| as bits for the tile's norm
// bound.
__device__ __forceinline__ unsigned long long gemm_epilogue_elem(const DevProblem &P, int l, int b, int row, int I,
                                                                 int col, double hl1, double aw, double az) {
    const size_t Spad = (size_t)P.Spad;
    const double pik = P.pi[col], w0 = P.W[col], zl = P.zlast[col], mu = P.wr[col], yt = P.ytil[col];
    const size_t ir = row + (size_t)col * P.ldr;
    const size_t ix = row + (size_t)col * P.ldx;
    const double rold = P.R[ir];
    double rnew = fma(pik, rold, aw);
    if (row == l - 1) rnew = fma(-mu, w0, rnew);
    P.R[ir] = rnew;
    double yv = P.X[ix];
    const unsigned char fl = P.slow[(size_t)I * Spad + col];
    if (fl & 2) {
        // Part 1 (update-task.c:134-139): y -= (H(i, l-1) - mu [i == l-1]) ytilde.
        yv = fma(-hl1, yt, yv);
        if (row == l - 1) yv = fma(mu, yt, yv);
    }
    if (fl & 1) {
        // Protected path: rescaled Ytilde2 of this (tile, shift).
        const double *zs = P.Zslow + (size_t)I * P.tlsz * Spad + col;
        const double *hr = P.H + row + (size_t)l * P.ldh;
        double acc = 0.0;
        for (int q = 0; q < b - 1; ++q) acc = fma(hr[(size_t)q * P.ldh], zs[(size_t)q * Spad], acc);
        yv = yv - acc;
        yv = fma(-rold, zs[(size_t)(b - 1) * Spad], yv);
    } else {
        yv = yv - az;
        yv = fma(-rold, zl, yv);
    }
    P.X[ix] = yv;
    return abs_bits(yv);
}

// Narrow form of the pipelined body for solves with few shifts: SC (< 32)
// shifts per CTA, so that a small shift count still spreads over many SMs.
// The scalar chain of each step runs on warp 0, lane s (and its duplicates
// s + SC, s + 2 SC, ..., which compute the same values and store nothing);
// the row warps 1 .. NW-1 hold RL = 32 / SC rows x SC shifts per
// instruction, so a step's vector work takes RL times fewer instructions than
// with a lane per shift.  Every (row, shift) element sees the same operations
// in the same order as in diag_body_pipe, and the maxima cover the same rows
// (a maximum does not depend on the order it is taken in), so the result is
// bit-identical to the wide form.  v/y live in shared memory as [row][SC].
template <int SC>
__host__ __device__ constexpr size_t diag_narrow_smem_bytes(int b, int nw) {
    return (size_t)(3 * (b + 1) + nw * 2 * SC + kDiagBcast * SC + 2 * SC * b) * sizeof(double);
}

template <int SC, int NW>
__device__ __forceinline__ void diag_body_narrow(const DevProblem &P, int J, int bx) {
    static_assert(32 % SC == 0 && SC >= 4 && SC < 32, "shifts per CTA");
    static_assert(NW >= 2, "a chain warp and at least one row warp");
    constexpr int RL = 32 / SC;                                               // rows per row-warp instruction
    // Warps w = 0, 4, ... share sub-partition 0, whose FP64 unit the scalar
    // chain (warp 0) needs to itself: rows go to the other warps only.
    constexpr int NR = NW - (NW + 3) / 4;                                     // row warps
    extern __shared__ double sm[];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int wid = tid >> 5;
    const int sh = lane % SC;                                                 // shift slot
    const int rs = lane / SC;                                                 // row slot (row warps)
    const bool store_lane = lane < SC;                                        // chain results are stored once
    const bool row_warp = (wid & 3) != 0;
    const int rw = wid - 1 - wid / 4;                                         // row-warp index, 0 .. NR-1
    const int k0 = bx * SC;
    const int k = k0 + sh;
    const bool act = k < P.S;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;

    double *hc = sm;                                                          // [3][b+1]
    unsigned long long *pm = reinterpret_cast<unsigned long long *>(sm + 3 * (b + 1));   // [NW][2][SC]
    double *bc = sm + 3 * (b + 1) + NW * 2 * SC;                              // [kDiagBcast][SC]
    double *v = bc + kDiagBcast * SC;                                         // [b][SC]
    double *y = v + (size_t)SC * b;                                           // [b][SC]
#define V(i) v[(size_t)(i) * SC + sh]
#define Y(i) y[(size_t)(i) * SC + sh]
#define PM(w, which) pm[(((w) * 2) + (which)) * SC + sh]
#define BC(q) bc[(q) * SC + sh]
#define HCOL(col) (hc + (size_t)((col) % 3) * (b + 1))

    for (int idx = tid; idx < SC * b; idx += 32 * NW) {
        const int c = idx / b, i = idx - c * b;
        const int kc = k0 + c;
        if (kc < P.S) {
            v[(size_t)i * SC + c] = P.R[l + i + (size_t)kc * P.ldr];
            y[(size_t)i * SC + c] = P.X[l + i + (size_t)kc * P.ldx];
        } else {
            v[(size_t)i * SC + c] = 1.0;
            y[(size_t)i * SC + c] = 0.0;
        }
    }

    const double mu = act ? P.wr[k] : 0.0;
    const double smin = fmax(DBL_EPSILON / 2 * absd(mu), P.smlnum);
    const double Hnorm = P.Hn[J + (size_t)J * P.T];
    double beta = act ? P.beta[(size_t)J * Spad + k] : sc_one(is);
    int pert = 0;

    const double *Hd = P.H + l + (size_t)l * P.ldh;                           // H(l, l)
    auto stage_col = [&](int col) {                                           // H(l : l+col+1, l+col), warp 0
        int rows = col + 2;
        if (rows > b) rows = b;
        const double *src = Hd + (size_t)col * P.ldh;
        double *dst = HCOL(col);
        for (int i = lane; i < rows; i += 32) cp_async8(dst + i, src + i);
        cp_async_commit();
    };
    if (wid == 0 && b >= 2) stage_col(b - 2);
    if (wid == 0 && b >= 3) stage_col(b - 3);
    if (wid == 0) cp_async_wait_all();
    __syncthreads();                                                          // tiles and columns loaded

    // Maxima over the RL row slots of one shift (lanes sh, sh + SC, ...).
    auto slot_max = [&](unsigned long long m) {
#pragma unroll
        for (int o = SC; o < 32; o <<= 1) m = umax64(m, __shfl_xor_sync(0xffffffffu, m, o));
        return m;
    };
    // Maxima of |y(0:b-3)| and |v(0:b-3)| for the first step, by the row warps.
    {
        unsigned long long ym = 0, vm = 0;
        if (row_warp)
            for (int i = rw * RL + rs; i < b - 2; i += NR * RL) {
                ym = umax64(ym, abs_bits(Y(i)));
                vm = umax64(vm, abs_bits(V(i)));
            }
        ym = slot_max(ym);
        vm = slot_max(vm);
        if (store_lane) {
            PM(wid, 0) = ym;
            PM(wid, 1) = vm;
        }
    }

    // Chain state of warp 0.
    double vcar = V(b - 1), ycar = Y(b - 1);
    double c = 0.0, s = 0.0, yc = 0.0, ys = 0.0, a1 = 1.0, a2 = 1.0, a3 = 1.0, yj = 0.0, yjm1 = 0.0;

    auto chain12 = [&](int jj, double vjm1, double yjm1_in) {
        const double *hcol = HCOL(jj - 1);
        const double hsub = hcol[jj];
        const double hdiag = hcol[jj - 1] - mu;
        const double vj = vcar;
        yj = ycar;
        yjm1 = yjm1_in;
        givens(vj, hsub, c, s);
        if (act && store_lane) {
            P.Cr[(size_t)(l + jj) * Spad + k] = c;
            P.Sr[(size_t)(l + jj) * Spad + k] = s;
        }
        double phi = sc_one(is);
        pert |= solve_1x1(smin, c * vj, s * hsub, yj, phi, is);
        beta = sc_combine(beta, phi, is);
        a1 = sc_value(phi, is);
        yjm1 = scale_by(a1, yjm1);
        phi = protect_double_update(absd(vjm1), absd(yj), absd(hdiag), absd(yj), absd(yjm1), is);
        a2 = sc_value(phi, is);
        if (!is_one(a2)) {
            yj = mul_rare(a2, yj);
            yjm1 = mul_rare(a2, yjm1);
        }
        beta = sc_combine(beta, phi, is);
        yc = yj * c;
        ys = yj * s;
        yjm1 = fma(ys, hdiag, fma(-yc, vjm1, yjm1));
        vcar = fma(c, hdiag, s * vjm1);
    };
    auto chain3 = [&](int jj) {
        unsigned long long ymb = 0, vmb = 0;
#pragma unroll
        for (int w = 1; w < NW; ++w) {
            ymb = umax64(ymb, PM(w, 0));
            vmb = umax64(vmb, PM(w, 1));
        }
        double ymax = from_bits(ymb);
        if (!is_one(a1)) ymax = from_bits(abs_bits(mul_rare(a1, ymax)));
        if (!is_one(a2)) ymax = from_bits(abs_bits(mul_rare(a2, ymax)));
        const double phi = protect_double_update(from_bits(vmb), absd(yj), Hnorm, absd(yj), ymax, is);
        a3 = sc_value(phi, is);
        if (!is_one(a3)) {
            yj = mul_rare(a3, yj);
            yjm1 = mul_rare(a3, yjm1);
            yc = mul_rare(yj, c);
            ys = mul_rare(yj, s);
        }
        beta = sc_combine(beta, phi, is);
        if (store_lane) {
            BC(0) = c;
            BC(1) = s;
            BC(2) = yc;
            BC(3) = ys;
            BC(4) = a1;
            BC(5) = a2;
            BC(6) = a3;
            Y(jj) = yj;
        }
        ycar = yjm1;
    };

    if (wid == 0 && b >= 2) chain12(b - 1, V(b - 2), Y(b - 2));
    __syncthreads();                                                          // first maxima in
    if (wid == 0 && b >= 2) chain3(b - 1);
    __syncthreads();                                                          // step b-1's scalars visible

    for (int j = b - 1; j >= 1; --j) {
        double sc_c = c, sc_s = s, sc_yc = yc, sc_ys = ys, s1 = a1, s2 = a2, s3 = a3;
        if (wid != 0) {
            sc_c = BC(0);
            sc_s = BC(1);
            sc_yc = BC(2);
            sc_ys = BC(3);
            s1 = BC(4);
            s2 = BC(5);
            s3 = BC(6);
        }
        const bool scaled = (!is_one(s1)) || (!is_one(s2)) || (!is_one(s3));
        const double *hcol = HCOL(j - 1);
        if (wid == 0) {
            // Row j-2 first: it enters step j-1's chain.
            double vn = 0.0, yn = 0.0;
            if (j >= 2) {
                const double h = hcol[j - 2];
                double yi = Y(j - 2);
                const double vi = V(j - 2);
                if (scaled) {
                    yi = scale_by(s1, yi);
                    yi = scale_by(s2, yi);
                    yi = scale_by(s3, yi);
                }
                yn = fma(sc_ys, h, fma(-sc_yc, vi, yi));
                vn = fma(sc_c, h, sc_s * vi);
                __syncwarp();                                                 // every lane read row j-2
                if (store_lane) {
                    Y(j - 2) = yn;
                    V(j - 2) = vn;
                }
            }
            if (j >= 2) {
                cp_async_wait_all();                                          // column j-2, staged last step
                __syncwarp();                                                 // ... by all lanes of warp 0
                chain12(j - 1, vn, yn);
            }
            if (j >= 3) stage_col(j - 3);                                     // for step j-2's chain
        } else if (row_warp) {
            if (scaled) {
                for (int i = j + 1 + rw * RL + rs; i < b; i += NR * RL) {
                    double t = Y(i);
                    t = scale_by(s1, t);
                    t = scale_by(s2, t);
                    t = scale_by(s3, t);
                    Y(i) = t;
                }
            }
            unsigned long long ymx = 0, vmx = 0;
            const int lim = j - 2;                                            // rows 0 .. j-3
            int i = rw * RL + rs;
            constexpr int ST = NR * RL;                                       // row stride of one lane
            for (; i + 3 * ST < lim; i += 4 * ST) {
                double hh[4], yy[4], vv[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    hh[q] = hcol[i + q * ST];
                    yy[q] = Y(i + q * ST);
                    vv[q] = V(i + q * ST);
                }
                if (scaled) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        yy[q] = scale_by(s1, yy[q]);
                        yy[q] = scale_by(s2, yy[q]);
                        yy[q] = scale_by(s3, yy[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    yy[q] = fma(sc_ys, hh[q], fma(-sc_yc, vv[q], yy[q]));
                    vv[q] = fma(sc_c, hh[q], sc_s * vv[q]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = i + q * ST;
                    Y(r) = yy[q];
                    V(r) = vv[q];
                    ymx = umax64(ymx, abs_bits(yy[q]));
                    vmx = umax64(vmx, abs_bits(vv[q]));
                }
            }
            for (; i < lim; i += ST) {
                const double h = hcol[i];
                double yi = Y(i), vi = V(i);
                if (scaled) {
                    yi = scale_by(s1, yi);
                    yi = scale_by(s2, yi);
                    yi = scale_by(s3, yi);
                }
                yi = fma(sc_ys, h, fma(-sc_yc, vi, yi));
                vi = fma(sc_c, h, sc_s * vi);
                Y(i) = yi;
                V(i) = vi;
                ymx = umax64(ymx, abs_bits(yi));
                vmx = umax64(vmx, abs_bits(vi));
            }
            ymx = slot_max(ymx);
            vmx = slot_max(vmx);
            if (store_lane) {
                PM(wid, 0) = ymx;
                PM(wid, 1) = vmx;
            }
        }
        __syncthreads();                                                      // rows of step j done, maxima in
        if (wid == 0 && j >= 2) chain3(j - 1);
        __syncthreads();                                                      // step j-1's scalars visible
    }

    double c0 = 0.0, s0 = 0.0;
    {
        double y0 = 0.0, a = 1.0;
        if (wid == 0) {
            double v0 = b >= 2 ? vcar : V(0);
            y0 = b >= 2 ? ycar : Y(0);
            if (J > 0) {
                // Final rotation with H(l, l-1) (reduce.c:53-61, solve-task.c:111-118).
                const double hleft = P.H[l + (size_t)(l - 1) * P.ldh];
                if (hleft != 0) {
                    givens(v0, hleft, c0, s0);
                } else {
                    c0 = 1.0;
                    s0 = 0.0;
                }
                if (act && store_lane) {
                    P.Cr[(size_t)l * Spad + k] = c0;
                    P.Sr[(size_t)l * Spad + k] = s0;
                }
                v0 = fma(v0, c0, -(hleft * s0));
            }
            double phi = sc_one(is);
            pert |= solve_1x1(smin, v0, 0.0, y0, phi, is);
            beta = sc_combine(beta, phi, is);
            a = sc_value(phi, is);
            if (store_lane) {
                BC(0) = c0;
                BC(1) = s0;
                BC(2) = a;
            }
        }
        __syncthreads();                                       // last step's rows (and the scalars) written
        if (wid != 0) {
            c0 = BC(0);
            s0 = BC(1);
            a = BC(2);
        }
        if (!is_one(a))
            for (int i = 1 + wid * RL + rs; i < b; i += NW * RL)
                Y(i) = a * Y(i);
        if (wid == 0 && store_lane) Y(0) = y0;
    }
    __syncthreads();

    // Store the solved tile, its scaling factor and the perturbation flag.
    for (int idx = tid; idx < SC * b; idx += 32 * NW) {
        const int cc = idx / b, i = idx - cc * b;
        const int kc = k0 + cc;
        if (kc < P.S) P.X[l + i + (size_t)kc * P.ldx] = y[(size_t)i * SC + cc];
    }
    if (act && wid == 0 && store_lane) {
        P.beta[(size_t)J * Spad + k] = beta;
        if (pert) P.pert[k] = 1;
    }
    if (J == 0 || !act || !store_lane) return;

    if (wid == 0) {
        // W(q) = c_q * prod_{p<q} s_p, pi = prod s (crossover propagation).
        double pk = 1.0;
        for (int q = 0; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            P.W[(size_t)q * Spad + k] = cq * pk;
            pk = pk * sq;
        }
        P.pi[k] = pk;
    }
    if (wid == 1) {
        // Ytilde2 = G_{b-1}^T ... G_1^T (c_0 x_0, x_1, ...) (update-task.c:193-220);
        // Zs(q) = Ytilde2(q-1), Zs(0) = 0, zlast = Ytilde2(b-1).
        unsigned long long zmx = 0;
        double z = c0 * Y(0);
        P.Zs[k] = 0.0;
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            const double t1 = z, t2 = Y(q);
            const double zo = fma(cq, t1, -(sq * t2));
            z = fma(sq, t1, cq * t2);
            P.Zs[(size_t)q * Spad + k] = zo;
            zmx = umax64(zmx, abs_bits(zo));
        }
        zmx = umax64(zmx, abs_bits(z));
        P.zlast[k] = z;
        P.z2n[k] = from_bits(zmx);
        P.ytil[k] = -s0 * Y(0);
    }
#undef V
#undef Y
#undef PM
#undef HCOL
#undef BC
}

// The GEMM of stage J+1 over the rows of tile J, for the CTA's own columns
// k0 .. k0+SC-1 (Pg: the descriptor with stage J+1's operands).  Every
// (row, column) element sums k = 0 .. b-1 in order with fma, as gemm_body
// does, then goes through the same epilogue (gemm_epilogue_elem), so the
// result is bit-identical to the top GEMM launch it replaces and the tile's
// rows are ready in this CTA without waiting for another kernel.
//
// The H block (rows x b) and the CTA's columns of W and Zs move through
// shared memory in chunks of kTopChunk k-columns, double-buffered with
// cp.async (every request of a chunk in flight at once), so the FP64 sums
// read shared memory instead of paying a global-load latency every few fmas.
// Thread t takes column t % SC and rows g, g + G, ..., g + (EB-1) G (g = t /
// SC, G = threads / SC), its sums in registers across the chunks; a pass
// covers G * EB rows (72 with 8 shifts per CTA), a taller tile takes more
// passes.  The two buffers, (rows + 2 SC) x kTopChunk doubles each (10 KB at
// tlsz 64), are no larger than the diagonal solve's own shared memory from
// 16 rows on; the solve reuses them afterwards, so the CTA still fits beside
// two GEMM CTAs on one SM.
constexpr int kTopChunk = 8, kTopRowsPerThread = 6;
template <int SC>
__host__ __device__ constexpr size_t top_staged_bytes(int rows) {
    return 2 * ((size_t)rows + 2 * SC) * kTopChunk * sizeof(double);
}

template <int SC, int NW>
__device__ __forceinline__ void top_rows_staged(const DevProblem &Pg, int J, int k0, double *sm) {
    constexpr int NT = 32 * NW, G = NT / SC, EB = kTopRowsPerThread;
    const int Js = J + 1;                                   // the stage whose GEMM this is
    const int l = Pg.fr[Js], b = Pg.fr[Js + 1] - l;
    const int r_lo = Pg.fr[J], rows = l - r_lo;
    const size_t Spad = (size_t)Pg.Spad;
    const size_t bufd = ((size_t)rows + 2 * SC) * kTopChunk;  // doubles per buffer
    // Buffer layout: hs[kk][rows] = H(r_lo + r, l - 1 + k), then ws[kk][SC], zs[kk][SC].
    auto stage = [&](int ch) {
        double *hs = sm + (size_t)(ch & 1) * bufd;
        double *ws = hs + (size_t)kTopChunk * rows;
        double *zs = ws + kTopChunk * SC;
        const int kb = ch * kTopChunk, kn = min(kTopChunk, b - kb);
        for (int idx = threadIdx.x; idx < kn * rows; idx += NT) {
            const int kk = idx / rows, r = idx - kk * rows;
            cp_async8(hs + idx, Pg.H + (r_lo + r) + (size_t)(l - 1 + kb + kk) * Pg.ldh);
        }
        for (int idx = threadIdx.x; idx < kn * SC; idx += NT) {
            const int kk = idx / SC, c = idx - kk * SC;
            const int col = k0 + c;
            if (col < Pg.S) {
                cp_async8(ws + idx, Pg.W + (size_t)(kb + kk) * Spad + col);
                cp_async8(zs + idx, Pg.Zs + (size_t)(kb + kk) * Spad + col);
            } else {
                ws[idx] = 0.0;
                zs[idx] = 0.0;
            }
        }
        cp_async_commit();
    };

    const int c = threadIdx.x % SC, g = threadIdx.x / SC;
    const int col = k0 + c;
    const int nch = (b + kTopChunk - 1) / kTopChunk;
    unsigned long long m = 0;
    for (int p0 = 0; p0 < rows; p0 += G * EB) {
        int ri[EB];
#pragma unroll
        for (int e = 0; e < EB; ++e) ri[e] = min(p0 + g + e * G, rows - 1);   // rows past the tile: computed, dropped
        double aw[EB], az[EB], hl1[EB];
#pragma unroll
        for (int e = 0; e < EB; ++e) aw[e] = az[e] = hl1[e] = 0.0;
        stage(0);
        for (int ch = 0; ch < nch; ++ch) {
            if (ch + 1 < nch) {
                stage(ch + 1);
                cp_async_wait_one();
            } else {
                cp_async_wait_all();
            }
            __syncthreads();                                    // chunk ch in shared memory
            const double *hs = sm + (size_t)(ch & 1) * bufd;
            const double *ws = hs + (size_t)kTopChunk * rows;
            const double *zs = ws + kTopChunk * SC;
            if (ch == 0) {
#pragma unroll
                for (int e = 0; e < EB; ++e) hl1[e] = hs[ri[e]];  // H(row, l-1), the epilogue's operand
            }
            const int kn = min(kTopChunk, b - ch * kTopChunk);
            for (int kk = 0; kk < kn; ++kk) {
                const double w = ws[kk * SC + c], z = zs[kk * SC + c];
                const double *hk = hs + (size_t)kk * rows;
#pragma unroll
                for (int e = 0; e < EB; ++e) {
                    const double a = hk[ri[e]];
                    aw[e] = fma(a, w, aw[e]);
                    az[e] = fma(a, z, az[e]);
                }
            }
            __syncthreads();                                    // buffer ch & 1 free for chunk ch + 2
        }
        if (col < Pg.S) {
#pragma unroll
            for (int e = 0; e < EB; ++e)
                if (p0 + g + e * G < rows)
                    m = umax64(m, gemm_epilogue_elem(Pg, l, b, r_lo + ri[e], J, col, hl1[e], aw[e], az[e]));
        }
    }
    if (col < Pg.S && m) atomicMax(reinterpret_cast<unsigned long long *>(Pg.ynorm) + (size_t)J * Spad + col, m);
}

// Fused form: the GEMM of stage J+1 over this tile's rows (top_rows_staged),
// then the diagonal solve of tile J, in one CTA.  The launch gives the larger
// of the two shared-memory footprints; a launch given less records a shape
// error and touches nothing.
template <int SC, int NW>
__global__ void __launch_bounds__(32 * NW) k_diag_nf(DevProblem P, DevProblem Pg, int J) {
    const int b = P.fr[J + 1] - P.fr[J];
    const size_t have = dynamic_smem_bytes();
    if (diag_narrow_smem_bytes<SC>(b, NW) > have || top_staged_bytes<SC>(b) > have) {
        if (threadIdx.x == 0) atomicOr(P.err, kErrShape);
        return;
    }
    extern __shared__ double sm[];
    top_rows_staged<SC, NW>(Pg, J, blockIdx.x * SC, sm);
    __syncthreads();                     // this CTA's rows of tile J are final; shared memory free
    diag_body_narrow<SC, NW>(P, J, blockIdx.x);
}

template <int SC, int NW>
__global__ void __launch_bounds__(32 * NW) k_diag_n(DevProblem P, int J) {
    const int b = P.fr[J + 1] - P.fr[J];
    if (diag_narrow_smem_bytes<SC>(b, NW) > dynamic_smem_bytes()) {
        if (threadIdx.x == 0) atomicOr(P.err, kErrShape);
        return;
    }
    diag_body_narrow<SC, NW>(P, J, blockIdx.x);
}

// NW warps: 8 (two per sub-partition, hiding FP64 latency) when v/y sit in
// shared memory and the CTA has its SM mostly to itself; 4 when v/y are in
// global scratch, where the CTAs share SMs with the concurrent GEMM's and a
// smaller register footprint lets them co-reside.
template <int NW>
__global__ void __launch_bounds__(32 * NW) k_diag(DevProblem P, int J, double *gscratch) {
    const int b = P.fr[J + 1] - P.fr[J];
    // The layout needs diag_small_bytes (+ v/y unless they are in global
    // scratch); a launch given less records a shape error and touches nothing.
    const size_t need = diag_small_bytes(b, NW) + (gscratch ? 0 : (size_t)64 * b * sizeof(double));
    if (need > dynamic_smem_bytes()) {
        if (threadIdx.x == 0) atomicOr(P.err, kErrShape);
        return;
    }
    diag_body_pipe<NW>(P, J, blockIdx.x, gscratch ? gscratch + (size_t)blockIdx.x * 64 * b : nullptr);
}

// The dynamic shared-memory limit of each k_diag form only ever grows: a
// launch must never find it lowered below what an earlier launch configured.
template <int NW>
cudaError_t diag_smem_attr(size_t smem) {
    static size_t configured = 0;
    static bool carve = false;
    const cudaError_t e = prefer_max_shared((const void *)k_diag<NW>, &carve);
    if (e != cudaSuccess) return e;
    return raise_smem_limit((const void *)k_diag<NW>, &configured, smem);
}

template <int SC, int NW>
cudaError_t launch_diag_narrow(const DevProblem &P, int J, int b, cudaStream_t st) {
    static size_t configured = 0;
    static bool carve = false;
    const size_t smem = diag_narrow_smem_bytes<SC>(b, NW);
    cudaError_t e = prefer_max_shared((const void *)k_diag_n<SC, NW>, &carve);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_diag_n<SC, NW>, &configured, smem);
    if (e != cudaSuccess) return e;
    k_diag_n<SC, NW><<<(P.S + SC - 1) / SC, 32 * NW, smem, st>>>(P, J);
    return cudaGetLastError();
}

template <int SC, int NW>
cudaError_t launch_diag_narrow_fused(const DevProblem &P, const DevProblem &Pg, int J, int b, cudaStream_t st) {
    static size_t configured = 0;
    const size_t smem = std::max(diag_narrow_smem_bytes<SC>(b, NW), top_staged_bytes<SC>(b));
    static bool carve = false;
    cudaError_t e = prefer_max_shared((const void *)k_diag_nf<SC, NW>, &carve);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_diag_nf<SC, NW>, &configured, smem);
    if (e != cudaSuccess) return e;
    k_diag_nf<SC, NW><<<(P.S + SC - 1) / SC, 32 * NW, smem, st>>>(P, Pg, J);
    return cudaGetLastError();
}

// Tile J's diagonal solve preceded by stage J+1's GEMM over tile J's rows,
// in one launch, when the narrow forms apply; false (nothing launched) when
// the wide form is used and the caller runs the two launches.
bool launch_diag_fused(const DevProblem &P, const DevProblem &Pg, int J, int b, cudaStream_t st,
                       cudaError_t *err) {
    if (!fused_top_for(P.S)) return false;
    switch (diag_shifts_per_cta(P.S)) {
    case 8: *err = launch_diag_narrow_fused<8, kDiagWarpsNarrow>(P, Pg, J, b, st); return true;
    case 16: *err = launch_diag_narrow_fused<16, kDiagWarpsNarrow>(P, Pg, J, b, st); return true;
    default: return false;
    }
}

// Shifts per CTA and top-GEMM form recorded by the plain-path autotuner, by
// shift count, and per-thread trial values the autotuner sets while it times
// the candidates.
namespace {
std::mutex g_spc_mu;
std::map<int, int> g_spc_tuned;
std::map<int, int> g_fused_tuned;
thread_local int t_spc_trial = 0;
thread_local int t_fused_trial = -1;

// The entry of the nearest shift count within a factor of two, or 0.
int nearest_tuned(const std::map<int, int> &m, int S) {
    int best = 0;
    double bd = 1e300;
    for (auto &kv : m) {
        const double d = std::fabs(std::log((double)kv.first / S));
        if (d < bd) {
            bd = d;
            best = kv.second;
        }
    }
    return bd <= std::log(2.0) ? best : 0;
}
}  // namespace

void set_diag_shifts_trial(int sc) { t_spc_trial = sc; }
void record_diag_shifts(int S, int sc) {
    std::lock_guard<std::mutex> g(g_spc_mu);
    g_spc_tuned[S] = sc;
}
void set_fused_top_trial(int on) { t_fused_trial = on; }
void record_fused_top(int S, bool on) {
    std::lock_guard<std::mutex> g(g_spc_mu);
    g_fused_tuned[S] = on ? 1 : 2;
}
// Whether the narrow diagonal kernel also computes the top GEMM of its own
// rows: HSR_FUSED_TOP (0 or 1) first, then the autotuner's trial value, then
// its recorded choice for the nearest shift count within a factor of two,
// else yes.  Either form gives the same result bit for bit.
bool fused_top_for(int S) {
    const char *env = getenv("HSR_FUSED_TOP");
    if (env && (env[0] == '0' || env[0] == '1')) return env[0] == '1';
    if (t_fused_trial >= 0) return t_fused_trial != 0;
    std::lock_guard<std::mutex> g(g_spc_mu);
    return nearest_tuned(g_fused_tuned, S) != 2;
}

// Shifts per diagonal CTA.  HSR_DIAG_SHIFTS_PER_CTA (8, 16 or 32) first,
// then the autotuner's trial value, then its recorded choice for the nearest
// shift count within a factor of two; otherwise 32 (a lane per shift) while
// the 32-shift CTAs cover the GPU, fewer when they would leave most SMs idle
// -- 16 below half the SMs, 8 below a quarter.  Every choice gives the same
// result bit for bit.
int diag_shifts_per_cta(int S) {
    const char *env = getenv("HSR_DIAG_SHIFTS_PER_CTA");   // read per launch: tests switch it
    const int forced = env ? atoi(env) : 0;
    if (forced == 8 || forced == 16 || forced == 32) return forced;
    if (t_spc_trial) return t_spc_trial;
    {
        std::lock_guard<std::mutex> g(g_spc_mu);
        const int best = nearest_tuned(g_spc_tuned, S);
        if (best) return best;
    }
    static const int sms = []() {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        return n;
    }();
    const int wide = (S + 31) / 32;
    if (sms <= 0) return 32;
    if (4 * wide <= sms) return 8;
    if (2 * wide <= sms) return 16;
    return 32;
}

cudaError_t launch_diag(const DevProblem &P, int J, int b, double *gscratch, cudaStream_t st) {
    const int grid = (P.S + 31) / 32;
    switch (diag_shifts_per_cta(P.S)) {
    case 8: return launch_diag_narrow<8, kDiagWarpsNarrow>(P, J, b, st);
    case 16: return launch_diag_narrow<16, kDiagWarpsNarrow>(P, J, b, st);
    default: break;
    }
    if (gscratch) {
        const size_t smem = diag_small_bytes(b, kDiagWarps);
        const cudaError_t e = diag_smem_attr<kDiagWarps>(smem);
        if (e != cudaSuccess) return e;
        k_diag<kDiagWarps><<<grid, 32 * kDiagWarps, smem, st>>>(P, J, gscratch);
    } else {
        const size_t smem = diag_smem_bytes(b);
        const cudaError_t e = diag_smem_attr<kDiagWarpsSmem>(smem);
        if (e != cudaSuccess) return e;
        k_diag<kDiagWarpsSmem><<<grid, 32 * kDiagWarpsSmem, smem, st>>>(P, J, gscratch);
    }
    return cudaGetLastError();
}

// CTAs of k_diag that one SM holds with v/y in shared memory (tile height b).
int diag_ctas_per_sm(int b) {
    const size_t smem = diag_smem_bytes(b);
    if (diag_smem_attr<kDiagWarpsSmem>(smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_diag<kDiagWarpsSmem>, 32 * kDiagWarpsSmem, smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

// --------------------------------------------------------------- Part 1
// Part 1 of stage J for tile I < J and shift k (update-task.c:68-174, with
// the Part-2 decision of :206-226) is the rank-1 update
//   y(I) -= (H(I, l-1) - mu e_last) * ytilde,   ytilde = -s_0 x_0,
// bracketed by three scaling decisions.  Where the operands' exponents show
// that none of the decisions can fire (part1_fast), each returns 1 exactly,
// and the update itself is left to the GEMM epilogue of stage J, which
// applies it to every row right before the tile update -- the same
// operations in the same order.  Otherwise the warp runs the full Part 1 for
// that (tile, shift) here (part1_full).  The flag byte of (I, k) tells the
// GEMM epilogue what remains:
//   bit 0  protected path: Ytilde2 rescaled in Zslow
//   bit 1  apply the Part-1 update in the epilogue

// Exact test for the case where no decision fires.  Xs == Ys: neither
// consistency branch runs.  hn, |mu|, |ytilde| < 2^496 and Yn < 2^993: the
// Part-1 protect_update takes its shortcut (factor 1), and every updated
// entry has |y'| <= (2^993 + 2^992)(1+u) < 2^994, the shift row
// |y''| <= (2^994 + 2^992)(1+u) < 2^995, so with Hn, ||Ytilde2||_oo < 2^497
// the Part-2 protect_update takes its shortcut as well.  NaN fails every
// comparison and takes the full path.
__device__ __forceinline__ bool part1_fast(double Xs, double Ys, double hn, double mu, double yt, double Yn,
                                           double Hn, double z2) {
    return ubits(Xs) == ubits(Ys) && mag(hn) < pow2_bits(496) && mag(mu) < pow2_bits(496) &&
           mag(yt) < pow2_bits(496) && mag(Yn) < pow2_bits(993) && mag(Hn) < pow2_bits(497) &&
           mag(z2) < pow2_bits(497);
}

// Full Part 1 for (tile I, shift k), by the whole warp.  Columns that need a
// rescaled Ytilde2 (Y scale below X scale, or a Part-2 factor != 1) get it
// written to Zslow and are flagged for the protected path of the epilogue.
__device__ __noinline__ void part1_full(const DevProblem &P, int J, int I, int k) {
    const int lane = threadIdx.x & 31;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    const int T = P.T;
    const int r0 = P.fr[I], m = P.fr[I + 1] - r0;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool applyShift = (I == J - 1);
    double *y = P.X + r0 + (size_t)k * P.ldx;
    const double *h = P.H + r0 + (size_t)(l - 1) * P.ldh;
    const double mu = P.wr[k];
    double Ys = P.beta[(size_t)I * Spad + k];
    const double Xs = P.beta[(size_t)J * Spad + k];
    double Yn = P.ynorm[(size_t)I * Spad + k];

    // Part 0: consistent scaling.
    if (Xs < Ys) {
        const double a = sc_upscale(Xs, Ys, is);
        for (int i = lane; i < m; i += 32) y[i] = a * y[i];
        Yn = a * Yn;
        Ys = Xs;
    }
    // Part 1: y -= (H(I, l-1) - mu e_last) * ytilde.
    double ytilde;
    const double x0 = P.X[l + (size_t)k * P.ldx];
    const double s0 = P.Sr[(size_t)l * Spad + k];
    if (Ys < Xs) {
        const double a = sc_upscale(Ys, Xs, is);
        ytilde = -s0 * (a * x0);
    } else {
        ytilde = -s0 * x0;
    }
    const double hnrm = P.hn[I + (size_t)J * T];
    const double alpha = protect_update(fmax(hnrm, absd(mu)), absd(ytilde), Yn, is);
    const double a = sc_value(alpha, is);
    unsigned long long mx = 0;
    if (!is_one(a)) {
        const double at = a * ytilde;
        for (int i = lane; i < m; i += 32) {
            double yi = fma(-h[i], at, a * y[i]);
            if (applyShift && i == m - 1) yi = fma(mu, at, yi);
            y[i] = yi;
            mx = umax64(mx, abs_bits(yi));
        }
    } else {
        for (int i = lane; i < m; i += 32) {
            double yi = fma(-h[i], ytilde, y[i]);
            if (applyShift && i == m - 1) yi = fma(mu, ytilde, yi);
            y[i] = yi;
            mx = umax64(mx, abs_bits(yi));
        }
    }
    Ys = sc_combine(Ys, alpha, is);
    for (int o = 16; o; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    Yn = from_bits(mx);

    // Part 2 decision.  Fast path: Ytilde2 from the unscaled solved tile.
    bool slow = false;
    double z2 = P.z2n[k];
    double *zs = P.Zslow + (size_t)I * P.tlsz * Spad + k;   // zs[q*Spad]
    if (Ys < Xs) {
        // X scaled to the Y scale before rotation (update-task.c:196-203).
        slow = true;
        const double a2 = sc_upscale(Ys, Xs, is);
        const double *x = P.X + l + (size_t)k * P.ldx;
        unsigned long long zmx = 0;
        double z = P.Cr[(size_t)l * Spad + k] * (a2 * x[0]);
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const double sq = P.Sr[(size_t)(l + q) * Spad + k];
            const double t1 = z, t2 = a2 * x[q];
            const double zo = fma(cq, t1, -(sq * t2));
            z = fma(sq, t1, cq * t2);
            if (lane == 0) zs[(size_t)(q - 1) * Spad] = zo;
            zmx = umax64(zmx, abs_bits(zo));
        }
        zmx = umax64(zmx, abs_bits(z));
        if (lane == 0) zs[(size_t)(b - 1) * Spad] = z;
        z2 = from_bits(zmx);
    }
    const double tsc = protect_update(P.Hn[I + (size_t)J * T], z2, Yn, is);
    const double ta = sc_value(tsc, is);
    if (!is_one(ta)) {
        if (!slow) {
            // Materialise Ytilde2 from the fast-path operand.
            for (int q = lane; q < b - 1; q += 32) zs[(size_t)q * Spad] = P.Zs[(size_t)(q + 1) * Spad + k];
            if (lane == 0) zs[(size_t)(b - 1) * Spad] = P.zlast[k];
            __syncwarp();
        }
        slow = true;
        __syncwarp();
        for (int q = lane; q < b; q += 32) zs[(size_t)q * Spad] = ta * zs[(size_t)q * Spad];
        for (int i = lane; i < m; i += 32) y[i] = ta * y[i];
        Ys = sc_combine(Ys, tsc, is);
    }
    __syncwarp();
    if (lane == 0) {
        P.beta[(size_t)I * Spad + k] = Ys;
        P.ynorm[(size_t)I * Spad + k] = 0.0;   // the GEMM epilogue folds the new bound
        P.slow[(size_t)I * Spad + k] = slow ? 1 : 0;
    }
    __syncwarp();
}

// Part 1 of stage J for the shifts [k0, k0 + kPart1Shifts), a lane per shift
// and 32 shifts per warp, over every tile I < J.  First pass: the exact
// test, and for the (tile, shift) pairs that pass, the flag for the epilogue
// and the reset of the tile's norm bound (the epilogue folds the new one).
// Second pass, only in warps where some pair failed: the full Part 1 for
// each failed pair in turn.
__device__ __forceinline__ void part1_block(const DevProblem &P, int J, int k0) {
    const int lane = threadIdx.x & 31;
    const int kw = k0 + (threadIdx.x >> 5) * 32;
    if (kw >= P.S) return;                                    // warp-uniform
    const int k = kw + lane;
    const bool act = k < P.S;
    const size_t Spad = (size_t)P.Spad;
    const size_t T = (size_t)P.T;
    double mu = 0.0, yt = 0.0, z2 = 0.0, Xs = 0.0;
    if (act) {
        mu = P.wr[k];
        yt = P.ytil[k];
        z2 = P.z2n[k];
        Xs = P.beta[(size_t)J * Spad + k];
    }
    bool any = false;
    if (act) {
#pragma unroll 4
        for (int I = 0; I < J; ++I) {
            const size_t ik = (size_t)I * Spad + k;
            if (part1_fast(Xs, P.beta[ik], P.hn[I + J * T], mu, yt, P.ynorm[ik], P.Hn[I + J * T], z2)) {
                P.ynorm[ik] = 0.0;
                P.slow[ik] = 2;
            } else {
                any = true;
            }
        }
    }
    if (!__any_sync(0xffffffffu, any)) return;
    for (int I = 0; I < J; ++I) {
        bool pend = false;
        if (act) {
            // Pairs that passed keep passing: their norm bound is now 0.
            const size_t ik = (size_t)I * Spad + k;
            pend = !part1_fast(Xs, P.beta[ik], P.hn[I + J * T], mu, yt, P.ynorm[ik], P.Hn[I + J * T], z2);
        }
        unsigned m = __ballot_sync(0xffffffffu, pend);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            part1_full(P, J, I, kw + src);
        }
    }
}

__global__ void __launch_bounds__(256) k_part1(DevProblem P, int J) { part1_block(P, J, blockIdx.x * kPart1Shifts); }

cudaError_t launch_part1(const DevProblem &P, int J, cudaStream_t st) {
    k_part1<<<(P.S + kPart1Shifts - 1) / kPart1Shifts, 256, 0, st>>>(P, J);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ GEMM
// CTA tile: 64 rows x 64 shifts, both operand halves; 256 threads, each with
// a 4x4 block of both accumulators.  A = H(rows, l-1 .. l+b-2) and the two
// B tiles arrive by TMA in 16-column chunks through a 3-stage mbarrier ring.
// Each accumulator sums k = 0 .. b-1 in order with fma, the same order as
// the oracle's dot products.  Warp w owns rows 8w .. 8w+7 of the tile, so a
// warp whose rows all lie outside [row_lo, row_hi) -- the partial blocks at
// the ragged first tile and at unaligned tile starts -- skips the FMA loop:
// masked lanes would cost the FP64 pipe as much as live ones.
// BN = 64 is the main tile.  BN = 16 serves the short GEMM over the rows of
// the next diagonal tile when the 64-column tiles would leave most SMs idle:
// that GEMM gates the next diagonal solve, and 16-column tiles spread its
// sequential K loop over four times as many CTAs.  Every accumulator sums
// the same products in the same order in both shapes.
template <int BN>
struct GemmSmemT {
    double A[kGemmStages][kGemmKC][kGemmBM];
    double W[kGemmStages][kGemmKC][BN];
    double Z[kGemmStages][kGemmKC][BN];
    uint64_t full[kGemmStages];
};
using GemmSmem = GemmSmemT<kGemmBN>;

size_t gemm_smem_bytes() { return sizeof(GemmSmem) + 128; }
size_t gemm_narrow_smem_bytes() { return sizeof(GemmSmemT<kGemmBNNarrow>) + 128; }

// Complex-shift epilogue: columns (2p, 2p+1) hold the real and imaginary
// parts of pair p, the same thread owns both, and every scalar of the real
// epilogue becomes its complex counterpart (crossover coefficient pi, Part-1
// ytilde, shift mu, zlast, the old crossover column); the bound folded into
// ynorm is the largest cabs1 of the pair's rows, kept at column 2p.
__device__ __forceinline__ void gemm_epilogue_cplx(const DevProblem &P, int J, int row_lo, int row_hi, int row0,
                                                   int col0, const double *eaw, const double *eaz, int kEpiLd) {
    const int tid = threadIdx.x;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const size_t Spad = (size_t)P.Spad;
    unsigned long long *ynb = reinterpret_cast<unsigned long long *>(P.ynorm);
    const int lane = tid & 31;
    const int er = tid & (kGemmBM - 1), cg = tid >> 6;
    const int row = row0 + er;
    const bool rowok = row >= row_lo && row < row_hi;
    int I = P.T - 1 - (P.n - 1 - row) / P.tlsz;
    if (I < 0) I = 0;
    const int key = rowok ? I : -1;
    const double hl1 = rowok ? P.H[row + (size_t)(l - 1) * P.ldh] : 0.0;
    for (int j = 0; j < kGemmBN / 4; j += 2) {
        const int cc = cg * (kGemmBN / 4) + j;
        const int col = col0 + cc;
        if (col >= P.S) break;
        const dcplx pik = cmk(P.pi[col], P.pi[col + 1]);
        const dcplx w0 = cmk(P.W[col], P.W[col + 1]);
        const dcplx zl = cmk(P.zlast[col], P.zlast[col + 1]);
        const dcplx mu = cmk(P.wr[col], P.wr[col + 1]);
        const dcplx yt = cmk(P.ytil[col], P.ytil[col + 1]);
        unsigned long long m = 0;
        if (rowok) {
            const size_t ir = row + (size_t)col * P.ldr;
            const size_t ix = row + (size_t)col * P.ldx;
            const dcplx rold = cmk(P.R[ir], P.R[ir + P.ldr]);
            dcplx rnew = cfma(pik, rold, cmk(eaw[cc * kEpiLd + er], eaw[(cc + 1) * kEpiLd + er]));
            if (row == l - 1) rnew = cfnma(mu, w0, rnew);
            P.R[ir] = rnew.re;
            P.R[ir + P.ldr] = rnew.im;
            dcplx yv = cmk(P.X[ix], P.X[ix + P.ldx]);
            const unsigned char fl = P.slow[(size_t)I * Spad + col];
            if (fl & 2) {
                yv = cmk(fma(-hl1, yt.re, yv.re), fma(-hl1, yt.im, yv.im));
                if (row == l - 1) yv = cfma(mu, yt, yv);
            }
            if (fl & 1) {
                const double *zs = P.Zslow + (size_t)I * P.tlsz * Spad + col;
                const double *hr = P.H + row + (size_t)l * P.ldh;
                double ar = 0.0, ai = 0.0;
                for (int q = 0; q < b - 1; ++q) {
                    const double h = hr[(size_t)q * P.ldh];
                    ar = fma(h, zs[(size_t)q * Spad], ar);
                    ai = fma(h, zs[(size_t)q * Spad + 1], ai);
                }
                yv = cmk(yv.re - ar, yv.im - ai);
                yv = cfnma(rold, cmk(zs[(size_t)(b - 1) * Spad], zs[(size_t)(b - 1) * Spad + 1]), yv);
            } else {
                yv = cmk(yv.re - eaz[cc * kEpiLd + er], yv.im - eaz[(cc + 1) * kEpiLd + er]);
                yv = cfnma(rold, zl, yv);
            }
            P.X[ix] = yv.re;
            P.X[ix + P.ldx] = yv.im;
            m = abs_bits(cabs1(yv));
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long mo = __shfl_up_sync(0xffffffffu, m, d);
            const int ko = __shfl_up_sync(0xffffffffu, key, d);
            if (lane >= d && ko == key) m = umax64(m, mo);
        }
        const int kn = __shfl_down_sync(0xffffffffu, key, 1);
        if (rowok && (lane == 31 || kn != key)) atomicMax(&ynb[(size_t)I * Spad + col], m);
    }
}

template <bool kCplx, int BN = kGemmBN>
__device__ __forceinline__ void gemm_body(const DevProblem &P, int J, int row_lo, int row_hi, int bx, int by,
                                          const CUtensorMap *tmH, const CUtensorMap *tmW,
                                          const CUtensorMap *tmZ) {
    static_assert(BN == kGemmBN || (BN == kGemmBNNarrow && !kCplx), "tile widths");
    // Threads per row of the tile (4 columns each) and rows per thread.
    constexpr int TC = BN / 4, RPT = kGemmBM * TC / 256;
    static_assert(RPT == 4 || RPT == 1, "thread tile");
    extern __shared__ unsigned char smraw[];
    GemmSmemT<BN> &sm = *reinterpret_cast<GemmSmemT<BN> *>(
        (reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x;
    // Row blocks start at row_lo rounded down to 8, so the TMA x coordinate
    // is always 16-byte aligned; rows outside [row_lo, row_hi) are not stored.
    const int row0 = (row_lo & ~7) + bx * kGemmBM;
    const int col0 = by * BN;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const int nk = (b + kGemmKC - 1) / kGemmKC;
    const uint32_t bytes = (uint32_t)((kGemmBM + 2 * BN) * kGemmKC * sizeof(double));

    if (tid == 0) {
        for (int s = 0; s < kGemmStages; ++s) mbar_init(&sm.full[s], 1);
        mbar_fence_init();
        prefetch_tensormap(tmH);
        prefetch_tensormap(tmW);
        prefetch_tensormap(tmZ);
    }
    __syncthreads();
    auto issue = [&](int s, int kc) {
        mbar_expect_tx(&sm.full[s], bytes);
        tma_load_2d(&sm.A[s][0][0], tmH, &sm.full[s], row0, l - 1 + kc * kGemmKC);
        tma_load_2d(&sm.W[s][0][0], tmW, &sm.full[s], col0, kc * kGemmKC);
        tma_load_2d(&sm.Z[s][0][0], tmZ, &sm.full[s], col0, kc * kGemmKC);
    };
    if (tid == 0)
        for (int s = 0; s < kGemmStages && s < nk; ++s) issue(s, s);

    // Thread (tr, tc) owns rows RPT*tr .. RPT*tr+RPT-1 and columns 4*tc ..
    // 4*tc+3; either way warp w owns rows 8w .. 8w+7.
    const int tc = tid % TC, tr = tid / TC;
    const int wrow = row0 + 8 * (tid >> 5);
    const bool live = wrow + 8 > row_lo && wrow < row_hi;      // warp-uniform
    double aw[RPT][4], az[RPT][4];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) aw[r][c] = az[r][c] = 0.0;

    int issued = nk < kGemmStages ? nk : kGemmStages;
    bool ok = true;
    for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kGemmStages;
        const uint32_t par = (uint32_t)((kc / kGemmStages) & 1);
        const bool got = mbar_wait(&sm.full[s], par, P.err);
        if (!__syncthreads_and(got)) { ok = false; break; }
        const int kmax = live ? min(kGemmKC, b - kc * kGemmKC) : 0;
        for (int kk = 0; kk < kmax; ++kk) {
            double a[RPT];
            if constexpr (RPT == 4) {
                const double2 a01 = *reinterpret_cast<const double2 *>(&sm.A[s][kk][4 * tr]);
                const double2 a23 = *reinterpret_cast<const double2 *>(&sm.A[s][kk][4 * tr + 2]);
                a[0] = a01.x;
                a[1] = a01.y;
                a[2] = a23.x;
                a[3] = a23.y;
            } else {
                a[0] = sm.A[s][kk][tr];
            }
            const double2 w01 = *reinterpret_cast<const double2 *>(&sm.W[s][kk][4 * tc]);
            const double2 w23 = *reinterpret_cast<const double2 *>(&sm.W[s][kk][4 * tc + 2]);
            const double2 z01 = *reinterpret_cast<const double2 *>(&sm.Z[s][kk][4 * tc]);
            const double2 z23 = *reinterpret_cast<const double2 *>(&sm.Z[s][kk][4 * tc + 2]);
            const double w[4] = {w01.x, w01.y, w23.x, w23.y};
            const double z[4] = {z01.x, z01.y, z23.x, z23.y};
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    aw[r][c] = fma(a[r], w[c], aw[r][c]);
                    az[r][c] = fma(a[r], z[c], az[r][c]);
                }
        }
        __syncthreads();
        if (tid == 0 && kc + kGemmStages < nk) {
            issue(s, kc + kGemmStages);
            ++issued;
        }
    }
    if (!ok) {
        // Drain the copies still in flight (bounded) before the CTA exits.
        if (tid == 0)
            for (int kc = 0; kc < issued; ++kc)
                mbar_wait(&sm.full[kc % kGemmStages], (uint32_t)((kc / kGemmStages) & 1), P.err, 1L << 20);
        return;
    }

    // Epilogue.  The accumulators go through shared memory (the operand ring
    // is free once every warp has left the k-loop), so that each thread then
    // owns one row of 16 columns: the reads and writes of R and X coalesce
    // along the rows, and the per-tile maxima of |y| are reduced across the
    // warp before one atomic per (tile, column).
    constexpr int kEpiLd = kGemmBM + 2;                       // padded pitch: spreads the banks
    static_assert(2 * BN * kEpiLd * sizeof(double) <= sizeof(sm.A) + sizeof(sm.W) + sizeof(sm.Z),
                  "epilogue staging must fit the operand ring");
    __syncthreads();
    double *eaw = &sm.A[0][0][0];
    double *eaz = eaw + BN * kEpiLd;
    if (live) {
        if constexpr (RPT == 4) {
#pragma unroll
            for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int r = 0; r < 4; r += 2) {
                    const int at = (4 * tc + c) * kEpiLd + 4 * tr + r;
                    *reinterpret_cast<double2 *>(&eaw[at]) = make_double2(aw[r][c], aw[r + 1][c]);
                    *reinterpret_cast<double2 *>(&eaz[at]) = make_double2(az[r][c], az[r + 1][c]);
                }
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                eaw[(4 * tc + c) * kEpiLd + tr] = aw[0][c];
                eaz[(4 * tc + c) * kEpiLd + tr] = az[0][c];
            }
        }
    }
    __syncthreads();
    if constexpr (kCplx) {
        gemm_epilogue_cplx(P, J, row_lo, row_hi, row0, col0, eaw, eaz, kEpiLd);
        return;
    }

    const size_t Spad = (size_t)P.Spad;
    unsigned long long *ynb = reinterpret_cast<unsigned long long *>(P.ynorm);
    const int lane = tid & 31;
    const int er = tid & (kGemmBM - 1), cg = tid >> 6;       // row; BN/4-column group (warp-uniform)
    const int row = row0 + er;
    const bool rowok = row >= row_lo && row < row_hi;
    int I = P.T - 1 - (P.n - 1 - row) / P.tlsz;
    if (I < 0) I = 0;
    const int key = rowok ? I : -1;                           // tile of the row; rows are consecutive
    const double hl1 = rowok ? P.H[row + (size_t)(l - 1) * P.ldh] : 0.0;   // Part-1 column
    for (int j = 0; j < BN / 4; ++j) {
        const int cc = cg * (BN / 4) + j;
        const int col = col0 + cc;
        if (col >= P.S) break;
        unsigned long long m =
            rowok ? gemm_epilogue_elem(P, l, b, row, I, col, hl1, eaw[cc * kEpiLd + er], eaz[cc * kEpiLd + er]) : 0;
        // Segmented max over runs of lanes in the same tile (inclusive scan);
        // the last lane of each run holds its maximum.
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long mo = __shfl_up_sync(0xffffffffu, m, d);
            const int ko = __shfl_up_sync(0xffffffffu, key, d);
            if (lane >= d && ko == key) m = umax64(m, mo);
        }
        const int kn = __shfl_down_sync(0xffffffffu, key, 1);
        if (rowok && (lane == 31 || kn != key)) atomicMax(&ynb[(size_t)I * Spad + col], m);
    }
}

__global__ void __launch_bounds__(256, 2)
k_gemm(DevProblem P, int J, int row_lo, int row_hi, const __grid_constant__ CUtensorMap tmH,
       const __grid_constant__ CUtensorMap tmW, const __grid_constant__ CUtensorMap tmZ) {
    gemm_body<false>(P, J, row_lo, row_hi, blockIdx.x, blockIdx.y, &tmH, &tmW, &tmZ);
}

__global__ void __launch_bounds__(256, 2)
k_gemm_n(DevProblem P, int J, int row_lo, int row_hi, const __grid_constant__ CUtensorMap tmH,
         const __grid_constant__ CUtensorMap tmW, const __grid_constant__ CUtensorMap tmZ) {
    gemm_body<false, kGemmBNNarrow>(P, J, row_lo, row_hi, blockIdx.x, blockIdx.y, &tmH, &tmW, &tmZ);
}

// The GEMM over [row_lo, row_hi) with 16-column tiles; tmW/tmZ must have a
// 16 x 16 box.
cudaError_t launch_gemm_narrow(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                               const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st) {
    if (row_hi <= row_lo || P.S <= 0) return cudaSuccess;
    static size_t configured = 0;
    static bool carve = false;
    const size_t smem = gemm_narrow_smem_bytes();
    cudaError_t e = prefer_max_shared((const void *)k_gemm_n, &carve);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_gemm_n, &configured, smem);
    if (e != cudaSuccess) return e;
    const int span = row_hi - (row_lo & ~7);
    dim3 g((span + kGemmBM - 1) / kGemmBM, (P.S + kGemmBNNarrow - 1) / kGemmBNNarrow);
    k_gemm_n<<<g, 256, smem, st>>>(P, J, row_lo, row_hi, tmH, tmW, tmZ);
    return cudaGetLastError();
}

// Whether the 16-column tiles should serve a GEMM over `rows` rows: when the
// 64-column tiles would fill fewer than half of the SMs.
bool gemm_prefers_narrow(int rows, int S) {
    static const int sms = []() {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        return n;
    }();
    const long ctas = (long)((rows + kGemmBM - 1) / kGemmBM) * ((S + kGemmBN - 1) / kGemmBN);
    return sms > 0 && 2 * ctas < sms;
}

__global__ void __launch_bounds__(256, 2)
k_gemm_c(DevProblem P, int J, int row_lo, int row_hi, const __grid_constant__ CUtensorMap tmH,
         const __grid_constant__ CUtensorMap tmW, const __grid_constant__ CUtensorMap tmZ) {
    gemm_body<true>(P, J, row_lo, row_hi, blockIdx.x, blockIdx.y, &tmH, &tmW, &tmZ);
}

cudaError_t launch_gemm(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                        const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st) {
    static size_t configured = 0;
    static bool carve = false;
    const size_t smem = gemm_smem_bytes();
    {
        cudaError_t e = prefer_max_shared((const void *)k_gemm, &carve);
        if (e == cudaSuccess) e = raise_smem_limit((const void *)k_gemm, &configured, smem);
        if (e != cudaSuccess) return e;
    }
    if (row_hi <= row_lo) return cudaSuccess;
    const int span = row_hi - (row_lo & ~7);
    dim3 g((span + kGemmBM - 1) / kGemmBM, (P.S + kGemmBN - 1) / kGemmBN);
    k_gemm<<<g, 256, smem, st>>>(P, J, row_lo, row_hi, tmH, tmW, tmZ);
    return cudaGetLastError();
}

cudaError_t launch_gemm_c(const DevProblem &P, int J, int row_lo, int row_hi, const CUtensorMap &tmH,
                          const CUtensorMap &tmW, const CUtensorMap &tmZ, cudaStream_t st) {
    static size_t configured = 0;
    const size_t smem = gemm_smem_bytes();
    {
        const cudaError_t e = raise_smem_limit((const void *)k_gemm_c, &configured, smem);
        if (e != cudaSuccess) return e;
    }
    if (row_hi <= row_lo) return cudaSuccess;
    const int span = row_hi - (row_lo & ~7);
    dim3 g((span + kGemmBM - 1) / kGemmBM, (P.S + kGemmBN - 1) / kGemmBN);
    k_gemm_c<<<g, 256, smem, st>>>(P, J, row_lo, row_hi, tmH, tmW, tmZ);
    return cudaGetLastError();
}

// -------------------------------------------------------------- finalize
// Lane per shift: smin = min_I beta(I,k) (robust.c:58-82), back-transform
// y <- Q^T y with the tile upscalings (shifted_Hessenberg_solve.c:153-215),
// three-accumulator 2-norm and the convergence test ||y|| > 0.1/sqrt(n)
// (:33-40, :229-273).  Rows move through shared memory 32 at a time so that
// the column-major block is read and written coalesced.
// Per-warp staging of finalize_body_buf: a 32-row block of X (transposed)
// and the rotations of those rows, each loaded coalesced with all its loads
// in flight at once, so the sequential row loop reads shared memory only.
struct FinalizeBuf {
    double x[32][33];
    double c[32][33];
    double s[32][33];
};

__device__ __forceinline__ void finalize_body_buf(const DevProblem &P, int bx, double *colnorm, int *status,
                                                  double *scale_out, FinalizeBuf &fb) {
    double (*buf)[33] = fb.x;
    const int lane = threadIdx.x & 31;
    const int k0 = bx * 32;
    const int k = k0 + lane;
    const bool act = k < P.S;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    const int n = P.n;

    double smin = act ? P.beta[k] : sc_one(is);
    for (int I = 1; I < P.T; ++I)
        if (act) smin = sc_min(smin, P.beta[(size_t)I * Spad + k], is);

    Nrm3 acc;
    acc.init();
    double tau1 = 0.0;
    int I = 0;
    double alpha = act ? sc_upscale(smin, P.beta[k], is) : 1.0;
    for (int r0 = 0; r0 < n; r0 += 32) {
        const int rows = min(32, n - r0);
        __syncwarp();
        for (int c = 0; c < 32; ++c) {
            const int kc = k0 + c;
            if (kc < P.S && lane < rows) buf[lane][c] = P.X[r0 + lane + (size_t)kc * P.ldx];
        }
        for (int t = 0; t < rows; ++t) {
            const size_t at = (size_t)(r0 + t) * Spad + k;
            fb.c[t][lane] = act ? P.Cr[at] : 0.0;
            fb.s[t][lane] = act ? P.Sr[at] : 0.0;
        }
        __syncwarp();
        for (int t = 0; t < rows; ++t) {
            const int i = r0 + t;
            if (i == P.fr[I + 1]) {
                ++I;
                alpha = act ? sc_upscale_rare(smin, P.beta[(size_t)I * Spad + k], is) : 1.0;
            }
            if (i == 0) {
                tau1 = scale_by(alpha, buf[0][lane]);
                continue;
            }
            const double tau2 = scale_by(alpha, buf[t][lane]);
            const double c = fb.c[t][lane];
            const double s = fb.s[t][lane];
            const double out = fma(c, tau1, -(s * tau2));
            tau1 = fma(c, tau2, s * tau1);
            acc.add(out);
            if (t == 0) {
                if (act) P.X[(i - 1) + (size_t)k * P.ldx] = out;
            } else {
                buf[t - 1][lane] = out;
            }
        }
        __syncwarp();
        // rows r0 .. r0+rows-2 hold outputs; row r0-1 was written directly.
        for (int c = 0; c < 32; ++c) {
            const int kc = k0 + c;
            if (kc < P.S && lane < rows - 1) P.X[r0 + lane + (size_t)kc * P.ldx] = buf[lane][c];
        }
    }
    if (act) {
        P.X[(n - 1) + (size_t)k * P.ldx] = tau1;
        acc.add(tau1);
        const double ynrm = acc.finish();
        colnorm[k] = ynrm;
        status[k] = (ynrm > 0.1 / sqrt((double)n)) ? 1 : 0;
        if (scale_out) scale_out[k] = smin;
    }
}

__device__ __forceinline__ void finalize_body(const DevProblem &P, int bx, double *colnorm, int *status,
                                              double *scale_out) {
    __shared__ FinalizeBuf fb;
    finalize_body_buf(P, bx, colnorm, status, scale_out, fb);
}

// The plain path's form of finalize_body_buf, on two warps for the same 32
// shifts.  Warp 0 runs only the per-row recurrence (the back-transform
// rotation of each row, reading X, the cosines and the sines from shared
// memory) and leaves each row's result in an output buffer.  Warp 1 brings
// the next 32-row block in with cp.async, and for the block warp 0 finished
// one step earlier adds the results to the three-accumulator norm in row
// order and writes them back to X.  The two warps meet at one barrier per
// block, with double-buffered inputs and outputs.  Every value sees the
// operations of finalize_body_buf in the same order, so the result is the
// same bit for bit; the recurrence's warp no longer carries the loads, the
// norm and the stores between one row's rotation and the next.
struct FinalizeWs {
    double x[2][32][33];                 // X rows of the block, [row][shift]
    double c[2][32][33];                 // cosines, [row][shift]
    double s[2][32][33];                 // sines, [row][shift]
    double o[2][32][33];                 // results: o[t] is row r0 - 1 + t
    double tail[32];                     // the last row's result, for warp 1
};

__device__ __forceinline__ void finalize_body_ws(const DevProblem &P, int bx, double *colnorm, int *status,
                                                 double *scale_out, FinalizeWs &fw) {
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int k0 = bx * 32;
    const int k = k0 + lane;
    const bool act = k < P.S;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    const int n = P.n;
    const int nb = (n + 31) / 32;

    auto stage = [&](int blk) {                                // warp 1
        const int r0 = blk * 32, rows = min(32, n - r0), q = blk & 1;
        for (int c = 0; c < 32; ++c) {
            const int kc = k0 + c;
            if (kc < P.S && lane < rows) cp_async8(&fw.x[q][lane][c], P.X + r0 + lane + (size_t)kc * P.ldx);
        }
        for (int t = 0; t < rows; ++t) {
            const size_t at = (size_t)(r0 + t) * Spad + k;
            if (act) {
                cp_async8(&fw.c[q][t][lane], P.Cr + at);
                cp_async8(&fw.s[q][t][lane], P.Sr + at);
            } else {
                fw.c[q][t][lane] = 0.0;
                fw.s[q][t][lane] = 0.0;
            }
        }
        cp_async_commit();
        cp_async_wait_all();
    };

    // Warp 0: the recurrence.
    double tau1 = 0.0, alpha = 1.0, smin = 0.0;
    int I = 0, nbound = 0;
    if (wid == 0) {
        smin = act ? P.beta[k] : sc_one(is);
        for (int J = 1; J < P.T; ++J)
            if (act) smin = sc_min(smin, P.beta[(size_t)J * Spad + k], is);
        alpha = act ? sc_upscale(smin, P.beta[k], is) : 1.0;
        nbound = P.fr[1];
    }
    // Warp 1: the norm.
    Nrm3 acc;
    acc.init();

    if (wid == 1) stage(0);
    __syncthreads();                                           // block 0 in
    for (int blk = 0; blk <= nb; ++blk) {
        if (wid == 0 && blk < nb) {
            const int r0 = blk * 32, rows = min(32, n - r0), q = blk & 1;
            double (*xb)[33] = fw.x[q];
            double (*cb)[33] = fw.c[q];
            double (*sb)[33] = fw.s[q];
            double (*ob)[33] = fw.o[q];
            for (int t = 0; t < rows; ++t) {
                const int i = r0 + t;
                if (i == nbound) {                             // tile boundary: the next tile's upscaling
                    ++I;
                    nbound = P.fr[I + 1];
                    alpha = act ? sc_upscale_rare(smin, P.beta[(size_t)I * Spad + k], is) : 1.0;
                }
                if (i == 0) {
                    tau1 = scale_by(alpha, xb[0][lane]);
                    continue;
                }
                const double tau2 = scale_by(alpha, xb[t][lane]);
                const double c = cb[t][lane];
                const double s = sb[t][lane];
                ob[t][lane] = fma(c, tau1, -(s * tau2));       // row i - 1
                tau1 = fma(c, tau2, s * tau1);
            }
        }
        if (wid == 1) {
            if (blk >= 1) {
                // Results of block blk-1: rows r0-1 .. r0+rows-2 (row -1 does not exist).
                const int p = blk - 1, r0 = p * 32, rows = min(32, n - r0), q = p & 1;
                double (*ob)[33] = fw.o[q];
                for (int t = (r0 == 0 ? 1 : 0); t < rows; ++t) acc.add(ob[t][lane]);
                __syncwarp();
                const int lo = r0 == 0 ? 1 : 0;
                for (int c = 0; c < 32; ++c) {
                    const int kc = k0 + c;
                    if (kc < P.S && lane >= lo && lane < rows)
                        P.X[(r0 - 1 + lane) + (size_t)kc * P.ldx] = ob[lane][c];
                }
            }
            if (blk + 1 < nb) stage(blk + 1);
        }
        __syncthreads();
    }
    if (wid == 0) {
        fw.tail[lane] = tau1;
        if (act) {
            P.X[(n - 1) + (size_t)k * P.ldx] = tau1;
            if (scale_out) scale_out[k] = smin;
        }
    }
    __syncthreads();
    if (wid == 1 && act) {
        acc.add(fw.tail[lane]);
        const double ynrm = acc.finish();
        colnorm[k] = ynrm;
        status[k] = (ynrm > 0.1 / sqrt((double)n)) ? 1 : 0;
    }
}

__global__ void __launch_bounds__(64) k_finalize(DevProblem P, double *colnorm, int *status,
                                                 double *scale_out) {
    extern __shared__ double fsm[];
    finalize_body_ws(P, blockIdx.x, colnorm, status, scale_out, *reinterpret_cast<FinalizeWs *>(fsm));
}

cudaError_t launch_finalize(const DevProblem &P, double *colnorm, int *status, double *scale_out,
                            cudaStream_t st) {
    static size_t configured = 0;
    const size_t smem = sizeof(FinalizeWs);
    const cudaError_t e = raise_smem_limit((const void *)k_finalize, &configured, smem);
    if (e != cudaSuccess) return e;
    k_finalize<<<(P.S + 31) / 32, 64, smem, st>>>(P, colnorm, status, scale_out);
    return cudaGetLastError();
}

__global__ void k_normalize(DevProblem P, const double *colnorm, const int *status) {
    const int k = blockIdx.y;
    if (k >= P.S || !status[k]) return;
    const double nrm = colnorm[k];
    double *x = P.X + (size_t)k * P.ldx;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        x[i] = x[i] / nrm;
}

cudaError_t launch_normalize(const DevProblem &P, const double *colnorm, const int *status,
                             cudaStream_t st) {
    int bx = (P.n + 255) / 256;
    if (bx > 64) bx = 64;
    dim3 g(bx, P.S);
    k_normalize<<<g, 256, 0, st>>>(P, colnorm, status);
    return cudaGetLastError();
}

__global__ void k_gather_cols(double *dst, long long ldd, const double *src, long long lds, int n,
                              const int *perm) {
    const int j = blockIdx.y;
    const double *s = src + (size_t)perm[j] * lds;
    double *d = dst + (size_t)j * ldd;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s[i];
}

cudaError_t launch_gather_cols(double *dst, long long ldd, const double *src, long long lds, int n,
                               const int *perm, int cnt, cudaStream_t st) {
    if (cnt <= 0) return cudaSuccess;
    int bx = (n + 255) / 256;
    if (bx > 64) bx = 64;
    dim3 g(bx, cnt);
    k_gather_cols<<<g, 256, 0, st>>>(dst, ldd, src, lds, n, perm);
    return cudaGetLastError();
}

// ------------------------------------------------------------ batched
// Each block reads its work item and its problem's descriptor, then runs the
// same body as the single-problem kernel, so a column computes exactly what
// it computes when its problem is solved alone.

// One pass per row: the row sum over all columns (||H||_oo) and, at every
// tile boundary at or right of the row's own tile, that tile's row sum; each
// sum accumulates its columns in order, as dlange does.
__device__ __forceinline__ void norms_rows(const DevProblem &P, int rb) {
    const int i = rb * kNormRows + threadIdx.x;
    if (i >= P.n || threadIdx.x >= kNormRows) return;
    const double *row = P.H + i;
    const int T = P.T;
    int I = T - 1 - (P.n - 1 - i) / P.tlsz;
    if (I < 0) I = 0;
    double full = 0.0;
    for (int J = 0; J < T; ++J) {
        const int c0 = P.fr[J], c1 = P.fr[J + 1];
        double tsum = 0.0;
        for (int c = c0; c < c1; ++c) {
            const double a = absd(row[(size_t)c * P.ldh]);
            full += a;
            tsum += a;
        }
        if (J >= I) {
            atomicMax(&P.nbits[I + (size_t)J * T], (unsigned long long)__double_as_longlong(tsum));
            if (J > I)
                atomicMax(&P.nbits[(size_t)T * T + I + (size_t)J * T], abs_bits(row[(size_t)(c0 - 1) * P.ldh]));
        }
    }
    if (full != full) atomicOr(P.nanflag, 1);
    atomicMax(&P.nbits[2 * (size_t)T * T], (unsigned long long)__double_as_longlong(full));
}

__global__ void k_norms_b(const DevProblem *probs, const BatchItem *items) {
    const BatchItem it = items[blockIdx.x];
    norms_rows(probs[it.x], it.z);
}

// Start vector eps3 = ||H||_oo * eps/2 (inverse_iteration.c:154-158, 19-34),
// computed on the device from the norm accumulators: column k's start vector
// and bounds, by `nth` threads numbered t = 0 .. nth-1.
__device__ __forceinline__ void init_column(const DevProblem &P, int k, int t, int nth) {
    const int T = P.T, n = P.n;
    double hinf = from_bits(P.nbits[2 * (size_t)T * T]);
    if (P.nanflag[0] & 1) hinf = __longlong_as_double(0x7ff8000000000000LL);
    const double eps3 = hinf * (DBL_EPSILON / 2);
    double *x = P.X + (size_t)k * P.ldx;
    double *r = P.R + (size_t)k * P.ldr;
    const double *hl = P.H + (size_t)(n - 1) * P.ldh;
    for (int i = t; i < n; i += nth) {
        double h = hl[i];
        if (i == n - 1) h = h - P.wr[k];
        r[i] = h;
        x[i] = eps3;
    }
    for (int I = t; I < T; I += nth) {
        P.beta[(size_t)I * P.Spad + k] = sc_one(P.is);
        P.ynorm[(size_t)I * P.Spad + k] = eps3;
    }
    if (t == 0) P.pert[k] = 0;
}

__global__ void k_init_b(const DevProblem *probs, const BatchItem *items) {
    const BatchItem it = items[blockIdx.x];
    init_column(probs[it.x], it.z, threadIdx.x, blockDim.x);
}

__global__ void __launch_bounds__(32 * kDiagWarpsB) k_diag_b(const DevProblem *probs, const BatchItem *items) {
    extern __shared__ double sm[];
    const BatchItem it = items[blockIdx.x];
    diag_body_1w(probs[it.x], it.y, it.z, sm, nullptr);
}

// One block per (problem, stage, 8 shifts); the tiles above the diagonal
// tile are visited in turn.
__global__ void __launch_bounds__(256) k_part1_b(const DevProblem *probs, const BatchItem *items) {
    const BatchItem it = items[blockIdx.x];
    part1_block(probs[it.x], it.y, it.z * kPart1Shifts);
}

__global__ void __launch_bounds__(256, 2) k_gemm_b(const DevProblem *__restrict__ probs,
                                                  const BatchItem *__restrict__ items,
                                                  const CUtensorMap *maps) {
    // The descriptor is staged in shared memory: its fields are reloaded
    // where used instead of occupying registers next to the accumulators.
    __shared__ DevProblem Ps;
    static_assert(sizeof(DevProblem) % 8 == 0 && sizeof(DevProblem) / 8 <= 256, "descriptor copy");
    const BatchItem it = items[blockIdx.x];
    if (threadIdx.x < sizeof(DevProblem) / 8)
        reinterpret_cast<long long *>(&Ps)[threadIdx.x] =
            reinterpret_cast<const long long *>(probs + it.x)[threadIdx.x];
    __syncthreads();
    const DevProblem &P = Ps;
    const CUtensorMap *m = maps + 3 * (size_t)it.x;
    const int J = it.y;
    const bool top = (it.z & kGemmTopFlag) != 0;
    const int lo = top ? P.fr[J - 1] : 0, hi = top ? P.fr[J] : P.fr[J - 1];
    gemm_body<false>(P, J, lo, hi, it.z & ~kGemmTopFlag, it.w, m, m + 1, m + 2);
}

__global__ void __launch_bounds__(32) k_finalize_b(const DevProblem *probs, const BatchItem *items) {
    const BatchItem it = items[blockIdx.x];
    const DevProblem &P = probs[it.x];
    finalize_body(P, it.z, P.colnorm, P.status, P.scale);
}

__global__ void k_normalize_b(const DevProblem *probs, const BatchItem *items) {
    const BatchItem it = items[blockIdx.x];
    const DevProblem &P = probs[it.x];
    const int k = it.z * kNormalizeCols + (threadIdx.x >> 5);
    if (k >= P.S || !P.status[k]) return;
    const double nrm = P.colnorm[k];
    double *x = P.X + (size_t)k * P.ldx;
    for (int i = threadIdx.x & 31; i < P.n; i += 32) x[i] = x[i] / nrm;
}

cudaError_t launch_norms_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_norms_b<<<n_items, kNormRows, 0, st>>>(probs, items);
    return cudaGetLastError();
}
cudaError_t launch_init_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_init_b<<<n_items, 128, 0, st>>>(probs, items);
    return cudaGetLastError();
}
cudaError_t launch_diag_b(const DevProblem *probs, const BatchItem *items, int n_items, int bmax,
                          cudaStream_t st) {
    const size_t smem = diag_smem_bytes_nw(bmax, kDiagWarpsB);
    if (smem < (size_t)64 * bmax * sizeof(double)) return cudaErrorInvalidValue;   // must fit shared memory
    static size_t configured = 0;
    {
        const cudaError_t e = raise_smem_limit((const void *)k_diag_b, &configured, smem);
        if (e != cudaSuccess) return e;
    }
    if (n_items <= 0) return cudaSuccess;
    k_diag_b<<<n_items, 32 * kDiagWarpsB, smem, st>>>(probs, items);
    return cudaGetLastError();
}
cudaError_t launch_part1_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_part1_b<<<n_items, 256, 0, st>>>(probs, items);
    return cudaGetLastError();
}
cudaError_t launch_gemm_b(const DevProblem *probs, const BatchItem *items, int n_items, const CUtensorMap *maps,
                          cudaStream_t st) {
    static size_t configured = 0;
    const size_t smem = gemm_smem_bytes();
    {
        const cudaError_t e = raise_smem_limit((const void *)k_gemm_b, &configured, smem);
        if (e != cudaSuccess) return e;
    }
    if (n_items <= 0) return cudaSuccess;
    k_gemm_b<<<n_items, 256, smem, st>>>(probs, items, maps);
    return cudaGetLastError();
}
cudaError_t launch_finalize_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_finalize_b<<<n_items, 32, 0, st>>>(probs, items);
    return cudaGetLastError();
}
cudaError_t launch_normalize_b(const DevProblem *probs, const BatchItem *items, int n_items, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_normalize_b<<<n_items, 32 * kNormalizeCols, 0, st>>>(probs, items);
    return cudaGetLastError();
}

// ------------------------------------------------------ persistent queue
// The batched work as one cooperative launch: CTAs take items in list order
// from a ticket counter, wait (bounded) for the per-problem counters their
// item depends on, run the same body the batched kernels run, and complete
// their own counter.  A stage of one problem thus starts as soon as its own
// predecessors are done, instead of at the next tick of the whole batch.
// Producers publish with a fence before the counter increment; consumers
// fence after observing it (and, before TMA reads of data other CTAs wrote,
// a generic-to-async proxy fence).

// Diagonal blocks per item: as many warps as fit beside the GEMM's operand
// ring with v/y in shared memory, at least one, at most eight.
__host__ __device__ inline size_t queue_diag_warp_bytes(int b) {
    return diag_small_bytes(b, 1) + (size_t)64 * b * sizeof(double);
}
int queue_diag_warps(int bmax) {
    const size_t budget = gemm_smem_bytes();
    int w = (int)(budget / queue_diag_warp_bytes(bmax));
    return w < 1 ? 1 : (w > 8 ? 8 : w);
}
size_t queue_smem_bytes(int bmax) {
    size_t need = gemm_smem_bytes();
    const size_t diag = queue_diag_warps(bmax) * queue_diag_warp_bytes(bmax);
    const size_t fin = (size_t)kQueueFinalBlocks * sizeof(FinalizeBuf);
    if (diag + 128 > need) need = diag + 128;     // + room to align the base to 128 bytes
    if (fin + 128 > need) need = fin + 128;
    return need;
}

__device__ __forceinline__ bool queue_wait(const int *ctr, int dep, int tgt, int *err, long limit) {
    if (dep < 0 || tgt <= 0) return true;
    const volatile int *c = ctr + dep;
    const volatile int *e = err;
    unsigned ns = 32;
    for (long it = 0; it < limit; ++it) {
        if (*c >= tgt) return true;
        if (*e & kErrQueueTimeout) return false;
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
    }
    atomicOr(err, kErrQueueTimeout);
    return false;
}

__global__ void __launch_bounds__(kQueueThreads, 2) k_queue(const DevProblem *__restrict__ probs,
                                                           const QueueItem *__restrict__ items, int n_items,
                                                           const CUtensorMap *maps, int *ctr, int *ticket, int *err,
                                                           int diag_warps, long spin_limit) {
    extern __shared__ unsigned char smraw[];
    __shared__ DevProblem Ps;
    __shared__ int s_idx, s_ok;
    static_assert(sizeof(DevProblem) % 8 == 0 && sizeof(DevProblem) / 8 <= kQueueThreads, "descriptor copy");
    const int tid = threadIdx.x, wid = tid >> 5;
    double *smd = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    for (;;) {
        if (tid == 0) {
            const int idx = atomicAdd(ticket, 1);
            int ok = 1;
            if (idx < n_items) {
                const QueueItem &q = items[idx];
                ok = queue_wait(ctr, q.dep0, q.tgt0, err, spin_limit) && queue_wait(ctr, q.dep1, q.tgt1, err, spin_limit);
                __threadfence();
            }
            s_idx = idx;
            s_ok = ok;
        }
        __syncthreads();
        const int idx = s_idx;
        if (idx >= n_items) break;
        const QueueItem q = items[idx];
        const BatchItem it = q.it;
        if (tid < (int)(sizeof(DevProblem) / 8))
            reinterpret_cast<long long *>(&Ps)[tid] = reinterpret_cast<const long long *>(probs + it.x)[tid];
        __syncthreads();
        const DevProblem &P = Ps;
        if (s_ok) {
            switch (q.kind) {
            case qkNorms:
                norms_rows(P, it.z);
                break;
            case qkInit: {
                const int k = it.z * kQueueInitCols + wid;
                if (wid < kQueueInitCols && k < P.S) init_column(P, k, tid & 31, 32);
                break;
            }
            case qkDiag: {
                const int blk = it.z * diag_warps + wid;
                const int b = P.fr[it.y + 1] - P.fr[it.y];
                if (wid < diag_warps && blk * 32 < P.S)
                    diag_body_1w(P, it.y, blk, smd + (size_t)wid * (queue_diag_warp_bytes(b) / sizeof(double)),
                                 nullptr);
                break;
            }
            case qkPart1:
                part1_block(P, it.y, it.z * kPart1Shifts);
                break;
            case qkGemm: {
                if (tid == 0) {
                    fence_proxy_async_global();    // operands other CTAs wrote, read by TMA below
                    fence_proxy_async_smem();      // this CTA's earlier generic use of the ring
                }
                const CUtensorMap *m = maps + 3 * (size_t)it.x;
                const int J = it.y;
                const bool top = (it.z & kGemmTopFlag) != 0;
                const int lo = top ? P.fr[J - 1] : 0, hi = top ? P.fr[J] : P.fr[J - 1];
                gemm_body<false>(P, J, lo, hi, it.z & ~kGemmTopFlag, it.w, m, m + 1, m + 2);
                __syncthreads();
                if (tid == 0) {
                    GemmSmem &gs = *reinterpret_cast<GemmSmem *>(smd);
                    for (int st = 0; st < kGemmStages; ++st) mbar_inval(&gs.full[st]);
                }
                break;
            }
            case qkFinal: {
                const int blk = it.z * kQueueFinalBlocks + wid;
                if (wid < kQueueFinalBlocks && blk * 32 < P.S)
                    finalize_body_buf(P, blk, P.colnorm, P.status, P.scale,
                                      reinterpret_cast<FinalizeBuf *>(smd)[wid]);
                break;
            }
            case qkNormalize: {
                const int k = it.z * kNormalizeCols + wid;
                if (k < P.S && P.status[k]) {
                    const double nrm = P.colnorm[k];
                    double *x = P.X + (size_t)k * P.ldx;
                    for (int i = tid & 31; i < P.n; i += 32) x[i] = x[i] / nrm;
                }
                break;
            }
            default:
                break;
            }
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&ctr[q.ctr], 1);
        }
    }
}

int queue_max_grid(int bmax) {
    static size_t configured = 0;
    const size_t smem = queue_smem_bytes(bmax);
    if (raise_smem_limit((const void *)k_queue, &configured, smem) != cudaSuccess) return 0;
    int nb = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_queue, kQueueThreads, smem) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return nb * sms;
}

cudaError_t launch_queue(const DevProblem *probs, const QueueItem *items, int n_items, const CUtensorMap *maps,
                         int *ctr, int *ticket, int *err, int bmax, int grid, cudaStream_t st) {
    const int maxg = queue_max_grid(bmax);
    if (maxg <= 0 || grid <= 0 || grid > maxg) return cudaErrorInvalidConfiguration;
    int dw = queue_diag_warps(bmax);
    long spin = 1L << 22;      // ~4 s of polls with the back-off: far above any item's wait
    void *args[] = {(void *)&probs, (void *)&items, (void *)&n_items, (void *)&maps, (void *)&ctr,
                    (void *)&ticket, (void *)&err, (void *)&dw, (void *)&spin};
    return cudaLaunchCooperativeKernel((const void *)k_queue, dim3(grid), dim3(kQueueThreads), args,
                                       queue_smem_bytes(bmax), st);
}

// ------------------------------------------------ bounded-wait self-test
// One thread initialises an mbarrier that expects two arrivals, arrives once
// and waits with the library's bounded wait: the phase can never complete, so
// the wait gives up after `limit` polls and records kErrWaitTimeout, exactly
// as a GEMM wait on a TMA copy that never lands would.  Nothing faults and
// the kernel returns.
__global__ void k_wait_selftest(int *err, long limit) {
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 2);
    mbar_fence_init();
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
    mbar_wait(&bar, 0, err, limit);
}

cudaError_t launch_wait_selftest(int *err, long limit, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(err, limit);
    return cudaGetLastError();
}

// ------------------------------------------------------- FP64 peak probe
// Eight independent FMA chains per thread; a and b are launch arguments so
// the chains cannot be folded.
__global__ void k_probe_dfma(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int it = 0; it < iters; ++it) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 123456.789) out[0] = s;
}

__global__ void k_probe_dmma(double *out, int iters) {
    const double a = threadIdx.x * 1e-3, bb = 1.0 - threadIdx.x * 1e-4;
    double c[4][2];
#pragma unroll
    for (int t = 0; t < 4; ++t) c[t][0] = c[t][1] = 0.0;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int t = 0; t < 4; ++t)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                         : "+d"(c[t][0]), "+d"(c[t][1])
                         : "d"(a), "d"(bb));
    }
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < 4; ++t) s += c[t][0] + c[t][1];
    if (s == 123456.789) out[0] = s;
}

cudaError_t launch_probe_dfma(double *out, int blocks, int iters, cudaStream_t st) {
    k_probe_dfma<<<blocks, 256, 0, st>>>(out, iters, 0.999, 1e-3);
    return cudaGetLastError();
}
cudaError_t launch_probe_dmma(double *out, int blocks, int iters, cudaStream_t st) {
    k_probe_dmma<<<blocks, 256, 0, st>>>(out, iters);
    return cudaGetLastError();
}

// ------------------------------------------ integer-pipe division self-test
// Seeded operands (splitmix64 per thread) compared bit for bit with the FP64
// division: random significands and exponents within 2^+-100 and over the
// whole normal range, divisor significands near 1 and near 2, dividends equal
// or next to the divisor.  Each set divides two dividends by one divisor
// through ddiv2_rn.  cnt: [first-quotient mismatches, second-quotient
// mismatches, sets that took the integer path, sets tried].
__device__ __forceinline__ unsigned long long st_mix(unsigned long long &s) {
    unsigned long long z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__global__ void k_selftest_arith(unsigned long long per_thread, unsigned long long seed, unsigned long long *cnt) {
    const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    unsigned long long sd = seed ^ (tid * 0x2545f4914f6cdd1dULL);
    unsigned long long bad1 = 0, bad2 = 0, fast = 0;
    for (unsigned long long i = 0; i < per_thread; ++i) {
        const unsigned long long ra = st_mix(sd), rb = st_mix(sd), rc = st_mix(sd);
        const int mode = (int)(rc & 7);
        unsigned long long fa = ra & kSigMask, fb = rb & kSigMask;
        if (mode == 1) fb |= 0xffffffffff000ULL;
        if (mode == 2) fb &= 0xffULL;
        if (mode == 3) fa = fb;
        if (mode == 4) fa = (fb + ((rc >> 8) & 0xf)) & kSigMask;
        if (mode == 5) fa = (fb - ((rc >> 8) & 0xf)) & kSigMask;
        if (mode == 6) fa |= 0xfffffffffff00ULL;
        int ea = 1023 + (int)((rc >> 16) % 200) - 100, eb = 1023 + (int)((rc >> 32) % 200) - 100;
        if (mode == 7) {
            ea = 1 + (int)((rc >> 16) % 2046);
            eb = 1 + (int)((rc >> 32) % 2046);
        }
        const double a = from_bits((((rc >> 60) & 1ULL) << 63) | ((unsigned long long)ea << 52) | fa);
        const double b = from_bits((((rc >> 61) & 1ULL) << 63) | ((unsigned long long)eb << 52) | fb);
        const double a2 = from_bits(ubits(a) ^ ((rc >> 40) & 0xffffULL));
        double q1, q2;
        if (ddiv2_rn(a, a2, b, q1, q2)) ++fast;
        if (ubits(q1) != ubits(div_fp64(a, b))) ++bad1;
        if (ubits(q2) != ubits(div_fp64(a2, b))) ++bad2;
    }
    if (bad1) atomicAdd(&cnt[0], bad1);
    if (bad2) atomicAdd(&cnt[1], bad2);
    atomicAdd(&cnt[2], fast);
    atomicAdd(&cnt[3], per_thread);
}

cudaError_t launch_selftest_arith(unsigned long long per_thread, unsigned long long seed, unsigned long long *cnt,
                                  int blocks, cudaStream_t st) {
    k_selftest_arith<<<blocks, 256, 0, st>>>(per_thread, seed, cnt);
    return cudaGetLastError();
}

}  // namespace hsr
