// hsr_device.cuh -- device-side building blocks for the sm_103a kernels.
//
// The whole library is compiled with --fmad=false: a product followed by a
// sum is never fused unless the source calls fma() explicitly.  The scalar
// routines below therefore round exactly like their C restatements, and the
// kernels reproduce the CPU oracle's "fma" arithmetic bit for bit.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace hsr {

// Error bits reported by kernels through a device status word.
enum : int {
    kErrWaitTimeout = 1,   // an mbarrier wait gave up
    kErrShape = 2,         // a kernel was launched with an impossible shape
};

// Overflow threshold Omega and its reciprocal (robust.c:14-15).
constexpr double kOmega = 1.e+300;
constexpr double kOmegaInv = 1.e-300;

// ---------------------------------------------------------------- |x| bits
// |x| as an unsigned 64-bit pattern.  For non-NaN doubles the order of these
// patterns equals the order of the magnitudes, so a max over them is an
// integer-pipe max; NaN patterns map to 0 so that NaN never wins, matching
// vector_infnorm (utils.h:75-85).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
    return b > 0x7ff0000000000000ULL ? 0ULL : b;
}
__device__ __forceinline__ double from_bits(unsigned long long b) {
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
    return a > b ? a : b;
}

// ------------------------------------------------ scaling-factor algebra
// robust.c:24-121.  `is` selects base-2 exponents (INTSCALING) at run time.
__device__ __forceinline__ double sc_one(bool is) { return is ? 0.0 : 1.0; }
__device__ __forceinline__ double sc_value(double a, bool is) { return is ? ldexp(1.0, (int)a) : a; }
__device__ __forceinline__ double sc_combine(double g, double phi, bool is) { return is ? phi + g : phi * g; }
__device__ __forceinline__ double sc_upscale(double amin, double a, bool is) {
    return is ? ldexp(1.0, (int)(amin - a)) : amin / a;
}
__device__ __forceinline__ double sc_min(double a, double b, bool is) { return is ? (a < b ? a : b) : fmin(a, b); }

// ------------------------------------------------- robust scalar kernels
// protect_real_division (robust.c:144-166)
__device__ __forceinline__ double protect_real_division(double b, double t) {
    double scale = 1.0;
    const double at = fabs(t), ab = fabs(b);
    if (at < kOmegaInv) {
        if (ab > at * kOmega) scale = (at * kOmega) / ab;
    } else {
        if (1.0 > at && ab > at * kOmega) scale = 1.0 / ab;
    }
    return scale;
}
// protect_sum (robust.c:175-185)
__device__ __forceinline__ double protect_sum(double x, double y) {
    double scale = 1.0;
    if ((x > 0 && y > 0) || (x < 0 && y < 0))
        if (fabs(x) > kOmega - fabs(y)) scale = 0.5;
    return scale;
}
// protect_update (robust.c:220-262)
__device__ __forceinline__ double protect_update(double tnorm, double xnorm, double ynorm, bool is) {
    double scale = 1.0;
    if (xnorm <= 1.0) {
        if (tnorm * xnorm > kOmega - ynorm) scale = 0.5;
    } else {
        if (tnorm > (kOmega - ynorm) / xnorm) scale = 0.5 / xnorm;
    }
    return is ? (double)ilogb(scale) : scale;
}
// protect_double_update (robust.c:270-285)
__device__ __forceinline__ double protect_double_update(double t1, double x1, double t2, double x2,
                                                        double y, bool is) {
    const double a1 = protect_update(t1, x1, y, is);
    const double a2 = protect_update(t2, x2, y, is);
    return is ? (a1 < a2 ? a1 : a2) : fmin(a1, a2);
}
// solve_1x1_real_system (robust.c:422-479); returns 1 if |t-lambda| < smin.
__device__ __forceinline__ int solve_1x1(double smin, double t, double lambda, double &x,
                                         double &scale, bool is) {
    int info = 0;
    const double s = protect_sum(t, -lambda);
    double csr = (s * t) - (s * lambda);
    if (fabs(csr) < smin) {
        csr = smin;
        info = 1;
    }
    const double alpha = protect_real_division(x, csr);
    x = (alpha * x) / csr;
    scale = is ? (double)ilogb(alpha / s) : alpha / s;
    return info;
}

// ------------------------------------------------------------- Givens
// LAPACK >= 3.10 dlartg (E. Anderson, "Algorithm 978: Safe scaling in the
// Level 1 BLAS", ACM TOMS 44(1), 2017), transposed as in reduce.c:14-24.
__device__ __forceinline__ void givens(double f, double g, double &c, double &s) {
    const double safmin = 2.2250738585072014e-308;   // 2^-1022
    const double safmax = 1.0 / safmin;               // 2^1022
    const double rtmin = sqrt(safmin);
    const double rtmax = sqrt(safmax / 2);
    const double f1 = fabs(f), g1 = fabs(g);
    double sv;
    if (g == 0.0) {
        c = 1.0; sv = 0.0;
    } else if (f == 0.0) {
        c = 0.0; sv = copysign(1.0, g);
    } else if (f1 > rtmin && f1 < rtmax && g1 > rtmin && g1 < rtmax) {
        const double d = sqrt(f * f + g * g);
        c = f1 / d;
        const double r = copysign(d, f);
        sv = g / r;
    } else {
        const double u = fmin(safmax, fmax(safmin, fmax(f1, g1)));
        const double fs = f / u, gs = g / u;
        const double d = sqrt(fs * fs + gs * gs);
        c = fabs(fs) / d;
        const double r = copysign(d, f);
        sv = gs / r;
    }
    s = (-1.0) * sv;
}

// ------------------------------------------- 2-norm, three accumulators
// LAPACK 3.10 dnrm2 as used in shifted_Hessenberg_solve.c:135-260.  Blue's
// thresholds for IEEE double (Anderson 2017): powers of two.
constexpr double kTsml = 0x1p-511;
constexpr double kTbig = 0x1p+486;
constexpr double kSsml = 0x1p+537;
constexpr double kSbig = 0x1p-538;

struct Nrm3 {
    double asml, amed, abig;
    __device__ __forceinline__ void init() { asml = amed = abig = 0.0; }
    __device__ __forceinline__ void add(double x) {
        const double ax = fabs(x);
        if (ax > kTbig) { const double t = ax * kSbig; abig = fma(t, t, abig); }
        else if (ax < kTsml) { const double t = ax * kSsml; asml = fma(t, t, asml); }
        else amed = fma(ax, ax, amed);
    }
    __device__ __forceinline__ double finish() const {
        double ynrm, scale = 1.0;
        if (abig > 0.0) {
            ynrm = abig + (amed * kSbig) * kSbig;
            scale = 1.0 / kSbig;
        } else if (asml > 0.0) {
            if (amed > 0.0) {
                const double am = sqrt(amed);
                const double as = sqrt(asml) / kSsml;
                double ymin, ymax;
                if (as > am) { ymin = am; ymax = as; } else { ymin = as; ymax = am; }
                ynrm = ymax * ymax * (1.0 + (ymin / ymax) * (ymin / ymax));
            } else {
                scale = 1.0 / kSsml;
                ynrm = asml;
            }
        } else {
            ynrm = amed;
        }
        return scale * sqrt(ynrm);
    }
};

// ------------------------------------------------ mbarrier + TMA (PTX)
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after `limit` polls (each poll may suspend the
// thread for a hardware-chosen interval) and records kErrWaitTimeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, long limit = (1L << 24)) {
    for (long it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, kErrWaitTimeout);
    return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ------------------------------------------------------------ cp.async
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace hsr
