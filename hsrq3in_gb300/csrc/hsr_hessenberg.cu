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
// One Householder step k per four launches on the caller's stream:
//   k_hh_larfg   one CTA: the reflector of A(k+1 : n-1, k), with the
//                three-accumulator 2-norm and the safe-minimum rescaling of
//                dlarfg, so no input magnitude overflows
//   k_hh_gemv    w = A(:, k+1 : n-1) v in column chunks (partial sums)
//   k_hh_reduce  w = sum of the chunks, in chunk order (deterministic)
//   k_hh_update  one CTA per column j > k: the right reflector
//                a(:, j) -= tau w v_j, then the left one on rows > k,
//                a(k+1:, j) -= tau v (v^T a(k+1:, j)); the column passes
//                through shared memory, so it is read and written once
// Every product is an FMA on FP64; the result is reproducible run to run.
#include "../../include/hsrq3in_gb300.h"
#include "hsr_device.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cuda_runtime.h>

namespace hsr {
namespace {

constexpr int kHhChunk = 256;     // columns per partial GEMV block
constexpr int kHhThreads = 256;
constexpr int kHhMaxSmemRows = 27000;   // column staged in shared memory up to this n

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

// v(i) of reflector k for i >= k+1 (1 at k+1, stored entries below).
__device__ __forceinline__ double vk(const double *A, long long lda, int k, int i) {
    return i == k + 1 ? 1.0 : A[i + (size_t)k * lda];
}

// dlarfg on alpha = A(k+1, k), x = A(k+2 : n-1, k).
__global__ void __launch_bounds__(1024) k_hh_larfg(int n, double *A, long long lda, int k, double *tau) {
    __shared__ double red[32];
    const int m = n - k - 1;                                   // reflector length
    double *x = A + (k + 2) + (size_t)k * lda;
    const int nx = m - 1;
    if (m <= 1) {
        if (threadIdx.x == 0) tau[k] = 0.0;
        return;
    }
    auto xnorm_of = [&]() {
        Nrm3 acc;
        acc.init();
        for (int i = threadIdx.x; i < nx; i += blockDim.x) acc.add(x[i]);
        Nrm3 tot;
        tot.asml = block_sum3(acc.asml, red);
        tot.amed = block_sum3(acc.amed, red);
        tot.abig = block_sum3(acc.abig, red);
        return tot.finish();
    };
    double alpha = A[(k + 1) + (size_t)k * lda];
    double xnorm = xnorm_of();
    if (xnorm == 0.0) {
        if (threadIdx.x == 0) tau[k] = 0.0;
        return;
    }
    const double safmin = 0x1p-969;                            // dlamch('S') / dlamch('E')
    const double rsafmn = 0x1p+969;
    double beta = -copysign(lapy2(alpha, xnorm), alpha);
    int knt = 0;
    if (fabs(beta) < safmin) {
        do {
            ++knt;
            __syncthreads();
            for (int i = threadIdx.x; i < nx; i += blockDim.x) x[i] = x[i] * rsafmn;
            beta = beta * rsafmn;
            alpha = alpha * rsafmn;
        } while (fabs(beta) < safmin && knt < 20);
        __syncthreads();
        xnorm = xnorm_of();
        beta = -copysign(lapy2(alpha, xnorm), alpha);
    }
    const double t = (beta - alpha) / beta;
    const double r = 1.0 / (alpha - beta);
    __syncthreads();
    for (int i = threadIdx.x; i < nx; i += blockDim.x) x[i] = x[i] * r;
    for (int j = 0; j < knt; ++j) beta = beta * safmin;
    if (threadIdx.x == 0) {
        tau[k] = t;
        A[(k + 1) + (size_t)k * lda] = beta;
    }
}

// partial[c][i] = sum over the columns j of chunk c (j > k) of A(i, j) v(j).
__global__ void __launch_bounds__(kHhThreads) k_hh_gemv(int n, const double *A, long long lda, int k,
                                                       double *partial) {
    __shared__ double vs[kHhChunk];
    const int c = blockIdx.y;
    const int j0 = k + 1 + c * kHhChunk;
    const int j1 = min(n, j0 + kHhChunk);
    for (int t = threadIdx.x; t < j1 - j0; t += blockDim.x) vs[t] = vk(A, lda, k, j0 + t);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    const double *a = A + i + (size_t)j0 * lda;
    for (int j = 0; j < j1 - j0; ++j) s = fma(a[(size_t)j * lda], vs[j], s);
    partial[(size_t)c * n + i] = s;
}

__global__ void k_hh_reduce(int n, int nchunks, const double *partial, double *w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += partial[(size_t)c * n + i];
    w[i] = s;
}

// Column j = k+1+blockIdx.x: right reflector on all rows, then the left one
// on rows k+1 .. n-1.
template <bool kStage>
__global__ void __launch_bounds__(kHhThreads) k_hh_update(int n, double *A, long long lda, int k,
                                                         const double *tau, const double *w) {
    extern __shared__ double colbuf[];
    __shared__ double red[32];
    const int j = k + 1 + blockIdx.x;
    double *col = A + (size_t)j * lda;
    const double tk = tau[k];
    const double tj = -tk * vk(A, lda, k, j);
    double d = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double a = fma(w[i], tj, col[i]);
        if (kStage) colbuf[i] = a;
        else col[i] = a;
        if (i > k) d = fma(vk(A, lda, k, i), a, d);
    }
    d = block_sum3(d, red);
    const double td = -tk * d;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double a = kStage ? colbuf[i] : col[i];
        if (i > k) a = fma(vk(A, lda, k, i), td, a);
        col[i] = a;
    }
}

// X(k+1 :, c) = H_k X(k+1 :, c) for every column c of X.
__global__ void __launch_bounds__(kHhThreads) k_hh_apply(int n, const double *A, long long lda, int k,
                                                        const double *tau, double *X, long long ldx) {
    __shared__ double red[32];
    double *x = X + (size_t)blockIdx.x * ldx;
    double d = 0.0;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) d = fma(vk(A, lda, k, i), x[i], d);
    d = block_sum3(d, red);
    const double td = -tau[k] * d;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) x[i] = fma(vk(A, lda, k, i), td, x[i]);
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
    const int max_chunks = (n + kHhChunk - 1) / kHhChunk;
    if (sc.ensure(((size_t)max_chunks + 1) * n * sizeof(double), dev) != cudaSuccess) return HSR_ERR_NOMEM;
    double *partial = sc.p, *w = sc.p + (size_t)max_chunks * n;
    const bool stage = n <= kHhMaxSmemRows;
    const size_t smem = stage ? (size_t)n * sizeof(double) : 0;
    if (stage && smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_hh_update<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return HSR_ERR_CUDA;
    const int rb = (n + kHhThreads - 1) / kHhThreads;
    for (int k = 0; k + 2 < n; ++k) {
        const int cols = n - k - 1;
        const int nch = (cols + kHhChunk - 1) / kHhChunk;
        k_hh_larfg<<<1, 1024, 0, st>>>(n, dA, lda, k, dtau);
        k_hh_gemv<<<dim3(rb, nch), kHhThreads, 0, st>>>(n, dA, lda, k, partial);
        k_hh_reduce<<<rb, kHhThreads, 0, st>>>(n, nch, partial, w);
        if (stage) k_hh_update<true><<<cols, kHhThreads, smem, st>>>(n, dA, lda, k, dtau, w);
        else k_hh_update<false><<<cols, kHhThreads, 0, st>>>(n, dA, lda, k, dtau, w);
    }
    return cudaGetLastError() == cudaSuccess ? HSR_OK : HSR_ERR_CUDA;
}

extern "C" int hsr_hessenberg_apply_q_device(int n, const double *dA, int lda, const double *dtau, int ncols,
                                             double *dX, int ldx, void *stream) {
    if (n <= 0 || lda < n || ncols < 0 || ldx < n || !dA || !dtau || (ncols > 0 && !dX)) return HSR_ERR_ARG;
    if (ncols == 0 || n <= 2) return HSR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int k = n - 3; k >= 0; --k) k_hh_apply<<<ncols, kHhThreads, 0, st>>>(n, dA, lda, k, dtau, dX, ldx);
    return cudaGetLastError() == cudaSuccess ? HSR_OK : HSR_ERR_CUDA;
}
