// hsr_validate.cu -- residuals of computed eigenpairs on the device.
//
// For every column k:  res_k = ||H x_k - lambda_k x_k||_2 / (||H||_F ||x_k||_2),
// the bound form of validation.c:145-166 (without |lambda| in the denominator,
// which makes it the stricter of the two).  Only the Hessenberg part of H
// (i <= j+1) enters, as in the solver.  Inputs of any magnitude are safe:
// H is scaled by 2^-e(max|H|) and each x_k by 2^-e(max|x_k|) before anything
// is multiplied, so every product and partial sum stays below 4n; the ratio
// is invariant under those exact power-of-two scalings.  A non-finite entry
// of H or x_k gives NaN for the column, a zero x_k gives +Inf.
//
// Four launches on the caller's stream, no synchronisation:
//   k_val_max    max |H_ij| over the Hessenberg part and max |x_ik| per column
//   k_val_sums   sum of squares of the scaled H and of each scaled x_k
//   k_val_gemm   r = H x - lambda x on 64 x 32 tiles (DFMA, K in chunks of
//                32 from the subdiagonal on), sum of squares of r per column
//   k_val_final  the ratio
// The sums use floating-point atomics, so the last bits of a residual may
// differ between runs; the residual is a diagnostic, not a solver output.
#include "../../include/hsrq3in_gb300.h"
#include "hsr_device.cuh"

#include <cmath>
#include <cuda_runtime.h>

namespace hsr {
namespace {

constexpr int kValRows = 64, kValCols = 32, kValK = 32;

__device__ __forceinline__ unsigned long long block_umax(unsigned long long v, unsigned long long *red) {
    for (int o = 16; o; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? red[lane] : 0ULL;
        for (int o = 16; o; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;   // valid in warp 0
}

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;   // valid in warp 0
}

// |x| bit pattern with NaN kept above +Inf (any non-finite value wins).
__device__ __forceinline__ unsigned long long mag_bits(double x) { return mag(x); }

// 2^-e(m) for the largest magnitude m (as bits): the exact power of two that
// brings m into [1, 2), at most 2^1022 (a subnormal m stays below 1); 1 for
// m = 0 or a non-finite m.
__device__ __forceinline__ double inv_pow2_of(unsigned long long m) {
    if (m == 0 || m >= kInfBits) return 1.0;
    return ldexp(1.0, -max(ilogb(from_bits(m)), -1022));
}

// Blocks [0, n): column j of H, rows 0 .. min(j+1, n-1).  Blocks [n, n+ncols): column of X.
__global__ void k_val_max(int n, const double *H, long long ldh, int ncols, const double *X, long long ldx,
                          unsigned long long *hmax, unsigned long long *xmax) {
    __shared__ unsigned long long red[32];
    const int j = blockIdx.x;
    unsigned long long m = 0;
    if (j < n) {
        const int rows = min(j + 2, n);
        const double *c = H + (size_t)j * ldh;
        for (int i = threadIdx.x; i < rows; i += blockDim.x) m = umax64(m, mag_bits(c[i]));
    } else {
        const double *c = X + (size_t)(j - n) * ldx;
        for (int i = threadIdx.x; i < n; i += blockDim.x) m = umax64(m, mag_bits(c[i]));
    }
    m = block_umax(m, red);
    if (threadIdx.x == 0) {
        if (j < n) atomicMax(hmax, m);
        else xmax[j - n] = m;
    }
}

__global__ void k_val_sums(int n, const double *H, long long ldh, int ncols, const double *X, long long ldx,
                           const unsigned long long *hmax, const unsigned long long *xmax, double *hsum,
                           double *xsum) {
    __shared__ double red[32];
    const int j = blockIdx.x;
    double s = 0.0;
    if (j < n) {
        const double sc = inv_pow2_of(*hmax);
        const int rows = min(j + 2, n);
        const double *c = H + (size_t)j * ldh;
        for (int i = threadIdx.x; i < rows; i += blockDim.x) {
            const double t = c[i] * sc;
            s = fma(t, t, s);
        }
    } else {
        const double sc = inv_pow2_of(xmax[j - n]);
        const double *c = X + (size_t)(j - n) * ldx;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double t = c[i] * sc;
            s = fma(t, t, s);
        }
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) {
        if (j < n) atomicAdd(hsum, s);
        else xsum[j - n] = s;
    }
}

// CTA: rows [r0, r0+64) x columns [c0, c0+32); thread: one row, 8 columns.
__global__ void __launch_bounds__(256) k_val_gemm(int n, const double *H, long long ldh, int ncols,
                                                  const double *wr, const double *X, long long ldx,
                                                  const unsigned long long *hmax, const unsigned long long *xmax,
                                                  double *rsum) {
    __shared__ double As[kValK][kValRows];
    __shared__ double Bs[kValK][kValCols + 1];
    __shared__ double xsc[kValCols];
    const int tid = threadIdx.x;
    const int r0 = blockIdx.x * kValRows, c0 = blockIdx.y * kValCols;
    const int row = tid & (kValRows - 1), cg = tid >> 6;       // 4 groups of 8 columns
    const double sh = inv_pow2_of(*hmax);
    if (tid < kValCols) xsc[tid] = c0 + tid < ncols ? inv_pow2_of(xmax[c0 + tid]) : 1.0;
    __syncthreads();
    double acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = 0.0;
    const int kstart = (max(r0 - 1, 0) / kValK) * kValK;      // H(i, k) = 0 for k < i-1
    for (int k0 = kstart; k0 < n; k0 += kValK) {
        // H(r0 .. r0+63, k0 .. k0+31), Hessenberg part only, scaled.
        for (int e = tid; e < kValK * kValRows; e += blockDim.x) {
            const int i = e & (kValRows - 1), kk = e >> 6;
            const int gi = r0 + i, gk = k0 + kk;
            double v = 0.0;
            if (gi < n && gk < n && gk >= gi - 1) v = H[gi + (size_t)gk * ldh] * sh;
            As[kk][i] = v;
        }
        // X(k0 .. k0+31, c0 .. c0+31), each column scaled.
        for (int e = tid; e < kValK * kValCols; e += blockDim.x) {
            const int kk = e & (kValK - 1), c = e >> 5;
            const int gk = k0 + kk, gc = c0 + c;
            Bs[kk][c] = (gk < n && gc < ncols) ? X[gk + (size_t)gc * ldx] * xsc[c] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kValK; ++kk) {
            const double a = As[kk][row];
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[c] = fma(a, Bs[kk][cg * 8 + c], acc[c]);
        }
        __syncthreads();
    }
    const int gi = r0 + row;
    const int lane = tid & 31;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int gc = c0 + cg * 8 + c;
        double r2 = 0.0;
        if (gi < n && gc < ncols) {
            const double xs = X[gi + (size_t)gc * ldx] * xsc[cg * 8 + c];
            const double r = fma(-(wr[gc] * sh), xs, acc[c]);
            r2 = r * r;
        }
        for (int o = 16; o; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        if (lane == 0 && gc < ncols) atomicAdd(&rsum[gc], r2);
    }
}

__global__ void k_val_final(int ncols, const unsigned long long *hmax, const unsigned long long *xmax,
                            const double *hsum, const double *xsum, const double *rsum, double *res) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncols) return;
    const unsigned long long hm = *hmax, xm = xmax[k];
    double r;
    if (hm >= kInfBits || xm >= kInfBits) r = __longlong_as_double(0x7ff8000000000000LL);   // NaN
    else if (xm == 0) r = __longlong_as_double(0x7ff0000000000000LL);                      // +Inf
    else if (hm == 0) r = sqrt(rsum[k]) / sqrt(xsum[k]);                                    // H = 0: ||lambda x||/||x||
    else r = sqrt(rsum[k]) / (sqrt(*hsum) * sqrt(xsum[k]));
    res[k] = r;
}

struct ValScratch {
    int device = -1;
    void *p = nullptr;
    size_t bytes = 0;
    ~ValScratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace
}  // namespace hsr

using namespace hsr;

extern "C" int hsr_residuals_device(int n, const double *dH, int lddH, int ncols, const double *dwr,
                                    const double *dX, int lddX, double *d_res, void *stream) {
    if (n <= 0 || lddH < n || ncols < 0 || lddX < n || !dH || (ncols > 0 && (!dwr || !dX || !d_res)))
        return HSR_ERR_ARG;
    if (ncols == 0) return HSR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    static thread_local ValScratch sc;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HSR_ERR_CUDA;
    const size_t need = (size_t)(2 + 3 * (size_t)ncols) * 8;
    if (sc.device != dev || sc.bytes < need) {
        if (sc.p) cudaFree(sc.p);
        sc.p = nullptr;
        sc.bytes = 0;
        if (cudaMalloc(&sc.p, need) != cudaSuccess) return HSR_ERR_NOMEM;
        sc.bytes = need;
        sc.device = dev;
    }
    unsigned long long *hmax = static_cast<unsigned long long *>(sc.p);
    double *hsum = reinterpret_cast<double *>(hmax + 1);
    unsigned long long *xmax = hmax + 2;
    double *xsum = reinterpret_cast<double *>(xmax + ncols);
    double *rsum = xsum + ncols;
    if (cudaMemsetAsync(hmax, 0, 16, st) != cudaSuccess ||
        cudaMemsetAsync(rsum, 0, (size_t)ncols * 8, st) != cudaSuccess)
        return HSR_ERR_CUDA;
    k_val_max<<<n + ncols, 256, 0, st>>>(n, dH, lddH, ncols, dX, lddX, hmax, xmax);
    k_val_sums<<<n + ncols, 256, 0, st>>>(n, dH, lddH, ncols, dX, lddX, hmax, xmax, hsum, xsum);
    dim3 g((n + kValRows - 1) / kValRows, (ncols + kValCols - 1) / kValCols);
    k_val_gemm<<<g, 256, 0, st>>>(n, dH, lddH, ncols, dwr, dX, lddX, hmax, xmax, rsum);
    k_val_final<<<(ncols + 127) / 128, 128, 0, st>>>(ncols, hmax, xmax, hsum, xsum, rsum, d_res);
    return cudaGetLastError() == cudaSuccess ? HSR_OK : HSR_ERR_CUDA;
}
