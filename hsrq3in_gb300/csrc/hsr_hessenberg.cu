// hsr_hessenberg.cu -- reduction of a dense matrix to upper-Hessenberg form
// on the device, and application of its orthogonal factor.
//
// The input step of the solver: the reference's problem generator reduces
// Q T Q^T with LAPACK dgehrd (problemgenerator.c:344), and dense requests
// need the same reduction before inverse iteration.  The layout and the
// reflector convention are LAPACK's (dgehd2 with dlarfg and dlarf): on exit
// the upper-Hessenberg part of A holds H, the entries below the subdiagonal
// of column k hold v_k(k+2 : n-1) with v_k(k+1) = 1 implied, and
// A_in = Q H Q^T with Q = H_0 H_1 ... H_{n-3}, H_k = I - tau_k v_k v_k^T.
//
// Blocked as LAPACK dgehrd/dlahr2 do it, in panels of kHbNb reflectors.  For
// a panel starting at column k0, Q_p = H_k0 ... H_{k0+nb-1} = I - V T V^T
// (compact WY, T upper triangular) and Y = A V T over the panel-start A.
// Column j = k0 + i of the panel is first brought up to date with the
// panel's earlier reflectors, a_j - Y V(j,:)^T from the right and
// (I - V T^T V^T) from the left; then its reflector is generated, and
// Y(:, i) = tau (A v - Y (V^T v)), T(:, i) = -tau T (V^T v), T(i,i) = tau.
// Three launches per column:
//   k_hb_step    rows in parallel: finishes the previous column (Y, V and T
//                columns, its reflector into A) and starts this one,
//                c = a_j - Y V(j,:)^T, with partial V^T c; the last block to
//                finish reduces them and forms w' = T^T V^T c
//   k_hb_larfg   rows in parallel: c -= V w' (rows > k0), the H entries of
//                column j, partial three-accumulator norms; the last block
//                runs dlarfg (with its safe-minimum rescaling)
//   k_hb_gemv    A(:, j+1 : n-1) v in column chunks, and partial V^T v
// After the panel the trailing columns c1 = k0 + nb ... get both sides of
// the block reflector with FP64 GEMMs (k_hb_gemm, DFMA, 64x64 tiles):
//   A(:, c1:) -= Y V(c1:, :)^T;  W = T^T V^T A(k0+1:, c1:);  A(k0+1:, c1:) -= V W
// The "last block" reductions use a completion counter and a fixed summation
// order: no block waits for another, and results are reproducible run to run.
#include "../../include/hsrq3in_gb300.h"
#include "hsr_device.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cuda_runtime.h>

namespace hsr {
namespace {


__device__ __forceinline__ double block_sum3(double v, double *red) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < nw; ++i) t += red[i];   // fixed order, every thread
    return t;
}

// dlapy2 (LAPACK >= 3.10): sqrt(x^2 + y^2) without overflow; NaN propagates.
__device__ __forceinline__ double lapy2(double x, double y) {
    if (x != x) return x;
    if (y != y) return y;
    const double xa = fabs(x), ya = fabs(y);
    const double w = fmax(xa, ya), z = fmin(xa, ya);
    if (z == 0.0 || w > DBL_MAX) return w;
    const double q = z / w;
    return w * sqrt(1.0 + q * q);
}


constexpr int kHbNb = 64;         // reflectors per panel
constexpr int kHbRows = 256;      // rows per CTA of the row-parallel kernels
constexpr int kHbChunk = 64;      // columns per CTA of the panel GEMV
constexpr int kHbMaxSplit = 8;    // split-K factor of the thin left-update GEMM

// Device state of one reduction.  Y, V: n x kHbNb (leading dimension n);
// T: kHbNb x kHbNb; c: the working column; part / part2: per-block partial
// sums [nblk][kHbNb]; partn: per-block norm accumulators [nblk][3]; gpart:
// GEMV partials [nchunk][n]; sc[0 .. kHbNb): w', sc[kHbNb]: the reflector's
// scale 1/(alpha - beta), sc[kHbNb+1]: tau; cnt: completion counters.
struct HbState {
    double *A;
    long long lda;
    int n;
    double *Y, *V, *T, *c, *part, *part2, *partn, *gpart, *sc, *tau;
    unsigned int *cnt;
};

// True in the block that finished last; its partial sums see every other
// block's (threadfence before the count).
__device__ __forceinline__ bool last_block(unsigned int *counter) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// Sum over the 256 rows of a block of V(r, q) * cs[r - r0] for q < i, a warp
// per q; writes out[q].
__device__ __forceinline__ void block_vdot(const HbState &S, int r0, int i, const double *cs, double *out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = warp; q < i; q += kHbRows / 32) {
        double s = 0.0;
        for (int t = lane; t < kHbRows; t += 32) {
            const int r = r0 + t;
            if (r < S.n) s = fma(S.V[r + (size_t)q * S.n], cs[t], s);
        }
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[q] = s;
    }
}

// v(r) of the current reflector: 1 at j+1, c(r) * rs below, 0 above.
__device__ __forceinline__ double hb_v(const HbState &S, int j, double rs, int r) {
    return r == j + 1 ? 1.0 : (r >= j + 2 ? S.c[r] * rs : 0.0);
}

// Sum_{q < m} x[q * stride] * w[q] in four interleaved fma chains, combined
// in a fixed order (independent chains hide the FP64 latency).
__device__ __forceinline__ double dot4(const double *x, long long stride, const double *w, int m) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int q = 0;
    for (; q + 3 < m; q += 4) {
        s0 = fma(x[(size_t)q * stride], w[q], s0);
        s1 = fma(x[(size_t)(q + 1) * stride], w[q + 1], s1);
        s2 = fma(x[(size_t)(q + 2) * stride], w[q + 2], s2);
        s3 = fma(x[(size_t)(q + 3) * stride], w[q + 3], s3);
    }
    for (; q < m; ++q) s0 = fma(x[(size_t)q * stride], w[q], s0);
    return (s0 + s1) + (s2 + s3);
}

// The same with eight chains, for the panel GEMV: eight independent loads in
// flight per thread.
__device__ __forceinline__ double dot8(const double *x, long long stride, const double *w, int m) {
    double s[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int q = 0;
    for (; q + 7 < m; q += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) s[u] = fma(x[(size_t)(q + u) * stride], w[q + u], s[u]);
    }
    for (; q < m; ++q) s[0] = fma(x[(size_t)q * stride], w[q], s[0]);
    return ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
}

// Sum of m partials p[ch * stride], four chains in a fixed order.
__device__ __forceinline__ double sum4(const double *p, long long stride, int m) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int q = 0;
    for (; q + 3 < m; q += 4) {
        s0 += p[(size_t)q * stride];
        s1 += p[(size_t)(q + 1) * stride];
        s2 += p[(size_t)(q + 2) * stride];
        s3 += p[(size_t)(q + 3) * stride];
    }
    for (; q < m; ++q) s0 += p[(size_t)q * stride];
    return (s0 + s1) + (s2 + s3);
}

// T(0:ip, ip) = -tau T(0:ip, 0:ip) vv, T(ip, ip) = tau, by one block.
__device__ __forceinline__ void hb_tcol(const HbState &S, int ip, double t, const double *vv) {
    for (int p = threadIdx.x; p < ip; p += blockDim.x) {
        double s = 0.0;
        for (int q = p; q < ip; ++q) s = fma(S.T[p + (size_t)q * kHbNb], vv[q], s);
        S.T[p + (size_t)ip * kHbNb] = -t * s;
    }
    if (threadIdx.x == 0) S.T[ip + (size_t)ip * kHbNb] = t;
}

// One launch between two reflectors.  Phase A (ip >= 0) finishes column
// jp = k0 + ip: Y(:, ip) = tau (A v - Y (V^T v)), V(:, ip), the reflector
// into A, T(:, ip).  Phase B (i >= 0) starts column j = k0 + i: c = a_j -
// Y V(j,:)^T and the partial sums of V^T c, reduced by the last block into
// w' = T^T V^T c.  Row r of both phases is one thread's, so phase B reads the
// Y(r, ip) that phase A just wrote; V(j, ip) = v_jp(jp + 1) is 1.
__global__ void __launch_bounds__(kHbRows) k_hb_step(HbState S, int k0, int ip, int i, int nchp) {
    __shared__ double vv[kHbNb], vrow[kHbNb], cs[kHbRows], ws[kHbNb];
    const int tid = threadIdx.x, r0 = blockIdx.x * kHbRows, r = r0 + tid, n = S.n;
    const int nblk = gridDim.x;
    if (ip >= 0) {
        const int jp = k0 + ip;
        for (int q = tid; q < ip; q += blockDim.x) {
            double s = 0.0;
            for (int b = 0; b < nblk; ++b) s += S.part2[(size_t)b * kHbNb + q];
            vv[q] = s;
        }
        __syncthreads();
        const double t = S.sc[kHbNb + 1], rs = S.sc[kHbNb];
        if (r < n) {
            const double av = sum4(S.gpart + r, n, nchp);
            const double y = av - dot4(S.Y + r, n, vv, ip);
            S.Y[r + (size_t)ip * n] = t * y;
            if (r >= jp + 1) {
                const double v = hb_v(S, jp, rs, r);
                S.V[r + (size_t)ip * n] = v;
                if (r >= jp + 2) S.A[r + (size_t)jp * S.lda] = v;
            }
        }
        if (i < 0) {
            if (blockIdx.x == 0) hb_tcol(S, ip, t, vv);
            return;
        }
    }
    const int j = k0 + i;
    for (int q = tid; q < i; q += blockDim.x) vrow[q] = (q == i - 1) ? 1.0 : S.V[j + (size_t)q * n];
    __syncthreads();
    double x = 0.0;
    if (r < n) {
        x = S.A[r + (size_t)j * S.lda] - dot4(S.Y + r, n, vrow, i);
        S.c[r] = x;
    }
    if (i == 0) return;
    cs[tid] = (r < n && r >= k0 + 1) ? x : 0.0;
    __syncthreads();
    block_vdot(S, r0, i, cs, S.part + (size_t)blockIdx.x * kHbNb);
    if (!last_block(&S.cnt[0])) return;
    hb_tcol(S, ip, S.sc[kHbNb + 1], vv);
    __syncthreads();
    for (int q = tid; q < i; q += blockDim.x) {
        double w = 0.0;
        for (int b = 0; b < nblk; ++b) w += S.part[(size_t)b * kHbNb + q];
        ws[q] = w;
    }
    __syncthreads();
    for (int p = tid; p < i; p += blockDim.x) {            // (T^T w)_p = sum_{q <= p} T(q, p) w_q
        double t = 0.0;
        for (int q = 0; q <= p; ++q) t = fma(S.T[q + (size_t)p * kHbNb], ws[q], t);
        S.sc[p] = t;
    }
    if (tid == 0) S.cnt[0] = 0;
}

__global__ void __launch_bounds__(kHbRows) k_hb_larfg(HbState S, int k0, int i, int j) {
    __shared__ double red[32];
    const int tid = threadIdx.x, r = blockIdx.x * kHbRows + tid, n = S.n;
    double x = 0.0;
    if (r < n) {
        x = S.c[r];
        if (r >= k0 + 1 && i > 0) {
            x = x - dot4(S.V + r, n, S.sc, i);
            S.c[r] = x;
        }
        if (r <= j) S.A[r + (size_t)j * S.lda] = x;          // final entries of H above the subdiagonal
    }
    Nrm3 acc;
    acc.init();
    if (r < n && r >= j + 2) acc.add(x);
    const double a0 = block_sum3(acc.asml, red), a1 = block_sum3(acc.amed, red), a2 = block_sum3(acc.abig, red);
    if (tid == 0) {
        S.partn[(size_t)blockIdx.x * 3] = a0;
        S.partn[(size_t)blockIdx.x * 3 + 1] = a1;
        S.partn[(size_t)blockIdx.x * 3 + 2] = a2;
    }
    if (!last_block(&S.cnt[1])) return;
    // dlarfg on alpha = c(j+1), x = c(j+2 : n-1), as the reference's LAPACK.
    double *xv = S.c + (j + 2);
    const int nx = n - j - 2;
    Nrm3 tot;
    tot.init();
    for (int b = 0; b < (int)gridDim.x; ++b) {
        tot.asml += S.partn[(size_t)b * 3];
        tot.amed += S.partn[(size_t)b * 3 + 1];
        tot.abig += S.partn[(size_t)b * 3 + 2];
    }
    double xnorm = tot.finish();
    double alpha = S.c[j + 1];
    double t = 0.0, rs = 1.0, beta = alpha;
    if (xnorm != 0.0) {
        const double safmin = 0x1p-969;                        // dlamch('S') / dlamch('E')
        const double rsafmn = 0x1p+969;
        beta = -copysign(lapy2(alpha, xnorm), alpha);
        int knt = 0;
        if (fabs(beta) < safmin) {
            do {
                ++knt;
                __syncthreads();
                for (int q = tid; q < nx; q += blockDim.x) xv[q] = xv[q] * rsafmn;
                beta = beta * rsafmn;
                alpha = alpha * rsafmn;
            } while (fabs(beta) < safmin && knt < 20);
            __syncthreads();
            Nrm3 a;
            a.init();
            for (int q = tid; q < nx; q += blockDim.x) a.add(xv[q]);
            Nrm3 s2;
            s2.asml = block_sum3(a.asml, red);
            s2.amed = block_sum3(a.amed, red);
            s2.abig = block_sum3(a.abig, red);
            xnorm = s2.finish();
            beta = -copysign(lapy2(alpha, xnorm), alpha);
        }
        t = (beta - alpha) / beta;
        rs = 1.0 / (alpha - beta);
        for (int q = 0; q < knt; ++q) beta = beta * safmin;
    }
    if (tid == 0) {
        S.tau[j] = t;
        S.A[(j + 1) + (size_t)j * S.lda] = beta;
        S.sc[kHbNb] = rs;
        S.sc[kHbNb + 1] = t;
        S.cnt[1] = 0;
    }
}

__global__ void __launch_bounds__(kHbRows) k_hb_gemv(HbState S, int k0, int i, int j) {
    __shared__ double vs[kHbChunk], cs[kHbRows];
    const int tid = threadIdx.x, n = S.n;
    const double rs = S.sc[kHbNb];
    const int c0 = j + 1 + blockIdx.y * kHbChunk, c1 = min(n, c0 + kHbChunk);
    for (int t = tid; t < c1 - c0; t += blockDim.x) vs[t] = hb_v(S, j, rs, c0 + t);
    __syncthreads();
    const int r0 = blockIdx.x * kHbRows, r = r0 + tid;
    if (r < n) S.gpart[(size_t)blockIdx.y * n + r] = dot8(S.A + r + (size_t)c0 * S.lda, S.lda, vs, c1 - c0);
    if (blockIdx.y != 0 || i == 0) return;
    cs[tid] = r < n ? hb_v(S, j, rs, r) : 0.0;
    __syncthreads();
    block_vdot(S, r0, i, cs, S.part2 + (size_t)blockIdx.x * kHbNb);
}

// C(i, j) = beta C(i, j) + alpha sum_k A(i, k) B(k, j) over k in this block's
// split-K range, with A(i, k) = A[i*sai + k*sak], B(k, j) = B[k*sbk + j*sbj]
// (one of each pair of strides is 1: loads coalesce along it) and
// C(i, j) = C[i + j*ldc + blockIdx.z*cz].  64x64 tiles, 256 threads with a
// 4x4 block each, K in chunks of 16 through shared memory; the sum over k is
// one fma chain in k order.
constexpr int kHbTm = 64, kHbTk = 16;
__global__ void __launch_bounds__(256, 2)
k_hb_gemm(int M, int N, int K, int kc, double alpha, const double *A, long long sai, long long sak,
          const double *B, long long sbk, long long sbj, double beta, double *C, long long ldc, long long cz) {
    __shared__ __align__(16) double As[kHbTk][kHbTm + 2];
    __shared__ __align__(16) double Bs[kHbTk][kHbTm + 2];
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * kHbTm, j0 = blockIdx.y * kHbTm;
    const int kb = blockIdx.z * kc, ke = min(K, kb + kc);
    const int tr = tid >> 4, tc = tid & 15;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    const bool a_i = sai == 1;                 // A contiguous along i (else along k)
    const bool b_k = sbk == 1;                 // B contiguous along k (else along j)
    for (int k = kb; k < ke; k += kHbTk) {
        double ra[4], rb[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int ii, kk;
            if (a_i) { ii = tid & 63; kk = (tid >> 6) + 4 * e; }
            else { kk = tid & 15; ii = (tid >> 4) + 16 * e; }
            const int gi = i0 + ii, gk = k + kk;
            ra[e] = (gi < M && gk < ke) ? A[(size_t)gi * sai + (size_t)gk * sak] : 0.0;
            int jj, kq;
            if (b_k) { kq = tid & 15; jj = (tid >> 4) + 16 * e; }
            else { jj = tid & 63; kq = (tid >> 6) + 4 * e; }
            const int gj = j0 + jj, gq = k + kq;
            rb[e] = (gj < N && gq < ke) ? B[(size_t)gq * sbk + (size_t)gj * sbj] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (a_i) As[(tid >> 6) + 4 * e][tid & 63] = ra[e];
            else As[tid & 15][(tid >> 4) + 16 * e] = ra[e];
            if (b_k) Bs[tid & 15][(tid >> 4) + 16 * e] = rb[e];
            else Bs[(tid >> 6) + 4 * e][tid & 63] = rb[e];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kHbTk; ++kk) {
            const double2 a01 = *reinterpret_cast<const double2 *>(&As[kk][4 * tr]);
            const double2 a23 = *reinterpret_cast<const double2 *>(&As[kk][4 * tr + 2]);
            const double2 b01 = *reinterpret_cast<const double2 *>(&Bs[kk][4 * tc]);
            const double2 b23 = *reinterpret_cast<const double2 *>(&Bs[kk][4 * tc + 2]);
            const double av[4] = {a01.x, a01.y, a23.x, a23.y};
            const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
    }
    double *Cz = C + (size_t)blockIdx.z * cz;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int gj = j0 + 4 * tc + b;
        if (gj >= N) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int gi = i0 + 4 * tr + a;
            if (gi >= M) continue;
            double *cp = Cz + gi + (size_t)gj * ldc;
            const double v = alpha * acc[a][b];
            *cp = beta == 0.0 ? v : fma(beta, *cp, v);
        }
    }
}

// W(q, j) = sum over s of Wp[s](q, j), in order.
__global__ void k_hb_sumk(int M, int N, int nsplit, const double *Wp, long long ldw, long long cz, double *W) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * N) return;
    const int q = e % M, j = e / M;
    double s = 0.0;
    for (int z = 0; z < nsplit; ++z) s += Wp[(size_t)z * cz + q + (size_t)j * ldw];
    W[q + (size_t)j * ldw] = s;
}

cudaError_t hb_gemm(int M, int N, int K, double alpha, const double *A, long long sai, long long sak,
                    const double *B, long long sbk, long long sbj, double beta, double *C, long long ldc,
                    int nsplit, long long cz, cudaStream_t st) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    int kc = K;
    if (nsplit > 1) kc = (((K + nsplit - 1) / nsplit) + kHbTk - 1) / kHbTk * kHbTk;
    const int nz = kc > 0 ? (K + kc - 1) / kc : 1;
    dim3 g((M + kHbTm - 1) / kHbTm, (N + kHbTm - 1) / kHbTm, nz < 1 ? 1 : nz);
    k_hb_gemm<<<g, 256, 0, st>>>(M, N, K, kc > 0 ? kc : 1, alpha, A, sai, sak, B, sbk, sbj, beta, C, ldc, cz);
    return cudaGetLastError();
}

// Back-transform Q X, blocked like LAPACK dormhr ('L', 'N'): the panels of
// the reduction in reverse order, X(k0+1:, :) -= V (T (V^T X(k0+1:, :))), with
// V rebuilt from the reflectors stored in A and T from V and tau (dlarft:
// T(0:i, i) = -tau_i T(0:i, 0:i) (V^T V)(0:i, i), T(i, i) = tau_i).
__global__ void k_hq_vpanel(int n, const double *A, long long lda, int k0, double *V) {
    const int i = blockIdx.y, j = k0 + i;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        V[r + (size_t)i * n] = r == j + 1 ? 1.0 : (r >= j + 2 ? A[r + (size_t)j * lda] : 0.0);
}

__global__ void k_hq_tfactor(int ib, const double *tau, const double *G, double *T) {
    for (int i = 0; i < ib; ++i) {
        const double t = tau[i];
        for (int p = threadIdx.x; p < i; p += blockDim.x) {
            double s = 0.0;
            for (int q = p; q < i; ++q) s = fma(T[p + (size_t)q * kHbNb], G[q + (size_t)i * kHbNb], s);
            T[p + (size_t)i * kHbNb] = -t * s;
        }
        if (threadIdx.x == 0) {
            T[i + (size_t)i * kHbNb] = t;
            for (int p = i + 1; p < kHbNb; ++p) T[p + (size_t)i * kHbNb] = 0.0;
        }
        __syncthreads();
    }
}

struct HhScratch {
    int device = -1;
    double *p = nullptr;
    size_t bytes = 0;
    ~HhScratch() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t b, int dev) {
        if (device == dev && b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) {
            bytes = b;
            device = dev;
        }
        return e;
    }
};

}  // namespace
}  // namespace hsr

using namespace hsr;

extern "C" int hsr_hessenberg_device(int n, double *dA, int lda, double *dtau, void *stream) {
    if (n <= 0 || lda < n || !dA || !dtau) return HSR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(dtau, 0, (size_t)n * sizeof(double), st) != cudaSuccess) return HSR_ERR_CUDA;
    if (n <= 2) return HSR_OK;
    static thread_local HhScratch sc;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HSR_ERR_CUDA;
    const int nblk = (n + kHbRows - 1) / kHbRows;
    const int maxch = (n + kHbChunk - 1) / kHbChunk;
    const size_t nb = kHbNb;
    const size_t need = 2 * (size_t)n * nb           // Y, V
                        + nb * nb                     // T
                        + (size_t)n                   // c
                        + 2 * (size_t)nblk * nb       // part, part2
                        + 3 * (size_t)nblk            // partn
                        + (size_t)maxch * n           // gpart
                        + nb + 8                      // sc
                        + (size_t)(kHbMaxSplit + 2) * nb * n   // W partials, W, W2
                        + 4;                          // counters
    if (sc.ensure(need * sizeof(double), dev) != cudaSuccess) return HSR_ERR_NOMEM;
    HbState S{};
    S.A = dA;
    S.lda = lda;
    S.n = n;
    double *p = sc.p;
    S.Y = p; p += (size_t)n * nb;
    S.V = p; p += (size_t)n * nb;
    S.T = p; p += nb * nb;
    S.c = p; p += n;
    S.part = p; p += (size_t)nblk * nb;
    S.part2 = p; p += (size_t)nblk * nb;
    S.partn = p; p += 3 * (size_t)nblk;
    S.gpart = p; p += (size_t)maxch * n;
    S.sc = p; p += nb + 8;
    double *Wp = p; p += (size_t)kHbMaxSplit * nb * n;
    double *W = p; p += nb * (size_t)n;
    double *W2 = p; p += nb * (size_t)n;
    S.cnt = reinterpret_cast<unsigned int *>(p);
    S.tau = dtau;
    if (cudaMemsetAsync(S.cnt, 0, 4 * sizeof(double), st) != cudaSuccess) return HSR_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int k0 = 0; k0 < n - 2; k0 += kHbNb) {
        const int ib = std::min(kHbNb, n - 2 - k0);
        if (cudaMemsetAsync(S.V, 0, (size_t)n * nb * sizeof(double), st) != cudaSuccess ||
            cudaMemsetAsync(S.T, 0, nb * nb * sizeof(double), st) != cudaSuccess)
            return HSR_ERR_CUDA;
        int nchp = 0;
        for (int i = 0; i < ib; ++i) {
            const int j = k0 + i;
            const int nch = (n - j - 1 + kHbChunk - 1) / kHbChunk;
            k_hb_step<<<nblk, kHbRows, 0, st>>>(S, k0, i - 1, i, nchp);
            k_hb_larfg<<<nblk, kHbRows, 0, st>>>(S, k0, i, j);
            k_hb_gemv<<<dim3(nblk, nch), kHbRows, 0, st>>>(S, k0, i, j);
            nchp = nch;
        }
        k_hb_step<<<nblk, kHbRows, 0, st>>>(S, k0, ib - 1, -1, nchp);
        const int c1 = k0 + ib, m = n - c1;
        if (m <= 0) continue;
        // Right: A(:, c1:) -= Y V(c1:, :)^T
        if (hb_gemm(n, m, ib, -1.0, S.Y, 1, n, S.V + c1, n, 1, 1.0, dA + (size_t)c1 * lda, lda, 1, 0, st) !=
            cudaSuccess)
            return HSR_ERR_CUDA;
        // Left: W = T^T (V(k0+1:, :)^T A(k0+1:, c1:)); A(k0+1:, c1:) -= V(k0+1:, :) W
        const int kr = n - k0 - 1;
        const int tiles = ((m + kHbTm - 1) / kHbTm) * ((ib + kHbTm - 1) / kHbTm);
        int split = (2 * sms + tiles - 1) / tiles;
        split = std::max(1, std::min(split, std::min(kHbMaxSplit, (kr + kHbTk - 1) / kHbTk)));
        if (hb_gemm(ib, m, kr, 1.0, S.V + (k0 + 1), n, 1, dA + (k0 + 1) + (size_t)c1 * lda, 1, lda, 0.0, Wp, nb,
                    split, nb * (long long)m, st) != cudaSuccess)
            return HSR_ERR_CUDA;
        {
            int kc = (((kr + split - 1) / split) + kHbTk - 1) / kHbTk * kHbTk;
            const int nz = (kr + kc - 1) / kc;
            const int tot = ib * m;
            k_hb_sumk<<<(tot + 255) / 256, 256, 0, st>>>(ib, m, nz, Wp, nb, nb * (long long)m, W);
        }
        if (hb_gemm(ib, m, ib, 1.0, S.T, nb, 1, W, 1, nb, 0.0, W2, nb, 1, 0, st) != cudaSuccess ||
            hb_gemm(kr, m, ib, -1.0, S.V + (k0 + 1), 1, n, W2, 1, nb, 1.0, dA + (k0 + 1) + (size_t)c1 * lda, lda, 1,
                    0, st) != cudaSuccess)
            return HSR_ERR_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? HSR_OK : HSR_ERR_CUDA;
}

extern "C" int hsr_hessenberg_apply_q_device(int n, const double *dA, int lda, const double *dtau, int ncols,
                                             double *dX, int ldx, void *stream) {
    if (n <= 0 || lda < n || ncols < 0 || ldx < n || !dA || !dtau || (ncols > 0 && !dX)) return HSR_ERR_ARG;
    if (ncols == 0 || n <= 2) return HSR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    static thread_local HhScratch sc;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HSR_ERR_CUDA;
    const size_t nb = kHbNb;
    const size_t need = (size_t)n * nb + 2 * nb * nb + (size_t)kHbMaxSplit * nb * nb +
                        (size_t)(kHbMaxSplit + 2) * nb * ncols;
    if (sc.ensure(need * sizeof(double), dev) != cudaSuccess) return HSR_ERR_NOMEM;
    double *V = sc.p, *G = V + (size_t)n * nb, *T = G + nb * nb, *Gp = T + nb * nb;
    double *Wp = Gp + (size_t)kHbMaxSplit * nb * nb, *W = Wp + (size_t)kHbMaxSplit * nb * ncols,
           *W2 = W + nb * (size_t)ncols;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto split_for = [&](int tiles, int kr) {
        int sp = (2 * sms + tiles - 1) / tiles;
        return std::max(1, std::min(sp, std::min(kHbMaxSplit, (kr + kHbTk - 1) / kHbTk)));
    };
    auto sum_parts = [&](int M, int N, int kr, int sp, const double *parts, double *out) {
        const int kc = (((kr + sp - 1) / sp) + kHbTk - 1) / kHbTk * kHbTk;
        const int nz = (kr + kc - 1) / kc;
        k_hb_sumk<<<(M * N + 255) / 256, 256, 0, st>>>(M, N, nz, parts, nb, nb * (long long)N, out);
    };
    const int last = ((n - 3) / kHbNb) * kHbNb;
    for (int k0 = last; k0 >= 0; k0 -= kHbNb) {
        const int ib = std::min(kHbNb, n - 2 - k0);
        const int kr = n - k0 - 1;
        k_hq_vpanel<<<dim3((n + 255) / 256 < 64 ? (n + 255) / 256 : 64, ib), 256, 0, st>>>(n, dA, lda, k0, V);
        // G = V^T V over rows k0+1 .., then T (dlarft, forward, columnwise).
        const int sg = split_for(1, kr);
        if (hb_gemm(ib, ib, kr, 1.0, V + (k0 + 1), n, 1, V + (k0 + 1), 1, n, 0.0, Gp, nb, sg, nb * (long long)ib,
                    st) != cudaSuccess)
            return HSR_ERR_CUDA;
        sum_parts(ib, ib, kr, sg, Gp, G);
        k_hq_tfactor<<<1, 64, 0, st>>>(ib, dtau + k0, G, T);
        // X(k0+1:, :) -= V (T (V^T X(k0+1:, :)))
        const int tiles = (ncols + kHbTm - 1) / kHbTm;
        const int sp = split_for(tiles, kr);
        if (hb_gemm(ib, ncols, kr, 1.0, V + (k0 + 1), n, 1, dX + (k0 + 1), 1, ldx, 0.0, Wp, nb, sp,
                    nb * (long long)ncols, st) != cudaSuccess)
            return HSR_ERR_CUDA;
        sum_parts(ib, ncols, kr, sp, Wp, W);
        if (hb_gemm(ib, ncols, ib, 1.0, T, 1, nb, W, 1, nb, 0.0, W2, nb, 1, 0, st) != cudaSuccess ||
            hb_gemm(kr, ncols, ib, -1.0, V + (k0 + 1), 1, n, W2, 1, nb, 1.0, dX + (k0 + 1), ldx, 1, 0, st) !=
                cudaSuccess)
            return HSR_ERR_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? HSR_OK : HSR_ERR_CUDA;
}
