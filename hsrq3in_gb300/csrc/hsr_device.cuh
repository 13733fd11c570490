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
    kErrQueueTimeout = 4,  // a work-queue item gave up waiting for its dependencies
};

// Overflow threshold Omega and its reciprocal (robust.c:14-15).
constexpr double kOmega = 1.e+300;
constexpr double kOmegaInv = 1.e-300;

// ---------------------------------------------------------------- |x| bits
// |x| as an unsigned 64-bit pattern.  For non-NaN doubles the order of these
// patterns equals the order of the magnitudes, so a max over them is an
// integer-pipe max; NaN patterns map to 0 so that NaN never wins, matching
// vector_infnorm (utils.h:75-85).
// |x| by clearing the sign bit on the integer pipe: the same bits as fabs(x)
// for every input (NaN included), without an FP64-pipe instruction, which on
// this part costs as much issue time as a multiply.
__device__ __forceinline__ double absd(double x) {
    return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
}
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

// ------------------------------------------ exact integer-pipe shortcuts
// FP64 issues at a fraction of the integer rate here, so comparisons against
// fixed thresholds run on IEEE bit patterns (for non-negative finite values
// the order of the patterns is the order of the numbers; NaN patterns sort
// above +Inf and every shortcut below is written so that NaN fails it and
// takes the exact path), and multiplications or divisions by a factor that
// is exactly 1.0 are skipped (1*x == x bit for bit).  Each shortcut returns
// exactly what the full expression returns.
__device__ __forceinline__ unsigned long long ubits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ unsigned long long mag(double x) { return ubits(x) & 0x7fffffffffffffffULL; }
constexpr unsigned long long kOneBits = 0x3ff0000000000000ULL;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ULL;
__host__ __device__ constexpr unsigned long long pow2_bits(int e) { return (unsigned long long)(1023 + e) << 52; }
__device__ __forceinline__ bool is_one(double a) { return ubits(a) == kOneBits; }
__device__ __forceinline__ bool is_zero(double a) { return (ubits(a) << 1) == 0ULL; }
__device__ __forceinline__ double neg(double a) { return __longlong_as_double((long long)(ubits(a) ^ 0x8000000000000000ULL)); }

// ------------------------------------------------------- rare branches
// Every FP64 instruction, taken or not, costs its sub-partition 64 issue
// cycles on this part (a dependent chain and independent operations alike),
// so the compiler must not evaluate a rarely taken branch speculatively and
// select.  Rare branches therefore call non-inlined functions, which it
// cannot evaluate ahead of the branch.  Each returns exactly the expression
// the inline code would have computed.
static __device__ __noinline__ double mul_rare(double a, double b) { return a * b; }
static __device__ __noinline__ double add_rare(double a, double b) { return a + b; }
// x scaled by a, skipping the multiplication when a == 1 (1*x == x bit for bit).
__device__ __forceinline__ double scale_by(double a, double x) { return is_one(a) ? x : mul_rare(a, x); }

// ---------------------------------------- two quotients on the integer pipe
// The rotation divides |f| and g by the same d.  An FP64 division issues
// about nine FP64 instructions here (some 560 cycles of its sub-partition,
// dependent or not), so the two cost about 1,100 cycles of each step of the
// diagonal solve's chain.  ddiv2_rn returns the same two correctly rounded
// (round-to-nearest-even) quotients from integer arithmetic and one shared
// reciprocal: the reciprocal of d's significand, seeded by the FP32
// approximation and refined by two fixed-point Newton-Raphson steps to about
// 62 bits; each quotient truncated from it and corrected to the exact floor
// by its integer remainder, which also gives the rounding (the
// remainder-corrected Newton division of Muller et al., Handbook of
// Floating-Point Arithmetic, 2nd ed., 2018, ch. 4, in 64-bit integers).
// IEEE division is correctly rounded, so any correct method returns the same
// bits.  Measured on one warp: 741 cycles for both quotients against 1,438
// for two FP64 divisions.  Operands outside the common range (zero,
// subnormal, infinite, NaN, a divisor whose significand is a power of two, a
// quotient near the exponent limits) take the FP64 instruction.
// The integer parts below also compile for the host (a test checks them
// there against the host's IEEE division), with the FP32 seed from a
// correctly rounded division and the high product from a 128-bit one.
static __device__ __noinline__ double div_fp64(double a, double b) { return a / b; }
__host__ __device__ __forceinline__ float rcp_approx_f32(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
__host__ __device__ __forceinline__ unsigned long long umulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}
// One Newton step for y ~ 2^116 / mb, mb in (2^52, 2^53): with the 128-bit
// error E = 2^116 - mb y, y' = y + y E / 2^116.
__host__ __device__ __forceinline__ unsigned long long ip_recip_step(unsigned long long mb, unsigned long long y) {
    const unsigned long long lo = mb * y;
    const unsigned long long hi = umulhi64(mb, y);
    const long long ehi = (long long)((1ULL << 52) - hi) - (lo != 0ULL ? 1 : 0);
    const unsigned long long elo = 0ULL - lo;
    const long long e = (long long)(((unsigned long long)ehi << 12) | (elo >> 52));   // E / 2^52
    const unsigned long long ae = e < 0 ? (unsigned long long)(-e) : (unsigned long long)e;
    const unsigned long long d = umulhi64(y, ae);
    return e < 0 ? y - d : y + d;
}
// y ~ 2^116 / mb within a few units (about 2^-62 relative).
__host__ __device__ __forceinline__ unsigned long long ip_recip(unsigned long long mb) {
    float r = rcp_approx_f32((float)(unsigned)(mb >> 29)) * 0x1p87f;
    r = fminf(r, 0x1.fffffep63f);
    unsigned long long y = (unsigned long long)r;
    y = ip_recip_step(mb, y);
    return ip_recip_step(mb, y);
}
// Bits of the correctly rounded ma / mb (significands with the hidden bit),
// given y = ip_recip(mb), the biased exponent ea - eb + 1023 and the sign.
// q estimates floor(ma 2^sh / mb) (54 bits) within two; the remainder
// r = ma 2^sh - q mb, exact modulo 2^64 because |r| < 2^56, moves q to the
// floor; its last bit and r != 0 round the 53-bit result to nearest even.
__host__ __device__ __forceinline__ unsigned long long ip_quot(unsigned long long ma, unsigned long long mb,
                                                               unsigned long long y, int ebias,
                                                               unsigned long long sign) {
    const int sh = ma < mb ? 54 : 53;
    const unsigned long long hi = umulhi64(ma, y);
    const unsigned long long lo = ma * y;
    unsigned long long q = sh == 53 ? ((hi << 1) | (lo >> 63)) : ((hi << 2) | (lo >> 62));
    long long r = (long long)((ma << sh) - q * mb);
#pragma unroll
    for (int i = 0; i < 2; ++i)
        if (r < 0) {
            q -= 1;
            r += (long long)mb;
        }
#pragma unroll
    for (int i = 0; i < 2; ++i)
        if (r >= (long long)mb) {
            q += 1;
            r -= (long long)mb;
        }
    const unsigned long long guard = q & 1ULL;
    unsigned long long Q = q >> 1;
    Q += guard & ((r != 0 ? 1ULL : 0ULL) | (Q & 1ULL));
    const int eo = ebias - (sh == 54 ? 1 : 0);
    return sign | (((unsigned long long)(eo - 1) << 52) + Q);   // a carry out of Q raises the exponent
}
constexpr unsigned long long kSigMask = 0xfffffffffffffULL, kHidden = 1ULL << 52;
__host__ __device__ __forceinline__ bool ip_div_ok(int ea, int eb, unsigned long long fb) {
    const int eq = ea - eb + 1023;
    return ea != 0 && ea != 0x7ff && eb != 0 && eb != 0x7ff && fb != 0 && eq >= 2 && eq <= 2045;
}
// q1 = a1 / b and q2 = a2 / b, correctly rounded, one reciprocal of b for
// both.  Returns whether the integer path was taken (the self-test counts it).
__device__ __forceinline__ bool ddiv2_rn(double a1, double a2, double b, double &q1, double &q2) {
    const unsigned long long u1 = ubits(a1), u2 = ubits(a2), ub = ubits(b);
    const int e1 = (int)((u1 >> 52) & 0x7ff), e2 = (int)((u2 >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
    const unsigned long long fb = ub & kSigMask;
    if (!ip_div_ok(e1, eb, fb) || !ip_div_ok(e2, eb, fb)) {
        q1 = div_fp64(a1, b);
        q2 = div_fp64(a2, b);
        return false;
    }
    const unsigned long long mb = fb | kHidden;
    const unsigned long long y = ip_recip(mb);
    q1 = from_bits(ip_quot((u1 & kSigMask) | kHidden, mb, y, e1 - eb + 1023, (u1 ^ ub) & 0x8000000000000000ULL));
    q2 = from_bits(ip_quot((u2 & kSigMask) | kHidden, mb, y, e2 - eb + 1023, (u2 ^ ub) & 0x8000000000000000ULL));
    return true;
}

// ------------------------------------------------ scaling-factor algebra
// robust.c:24-121.  `is` selects base-2 exponents (INTSCALING) at run time.
__device__ __forceinline__ double sc_one(bool is) { return is ? 0.0 : 1.0; }
static __device__ __noinline__ double pow2_rare(double a) { return ldexp(1.0, (int)a); }
__device__ __forceinline__ double sc_value(double a, bool is) {
    if (is) return is_zero(a) ? 1.0 : pow2_rare(a);
    return a;
}
__device__ __forceinline__ double sc_combine(double g, double phi, bool is) {
    if (is) return is_zero(phi) ? g : add_rare(phi, g);
    return is_one(phi) ? g : mul_rare(phi, g);
}
__device__ __forceinline__ double sc_upscale(double amin, double a, bool is) {
    return is ? ldexp(1.0, (int)(amin - a)) : amin / a;
}
__device__ __forceinline__ double sc_min(double a, double b, bool is) { return is ? (a < b ? a : b) : fmin(a, b); }
// The upscaling at a tile boundary of the back-transform (once per tile, not
// per row): out of line so the per-row loop evaluates none of it.
static __device__ __noinline__ double sc_upscale_rare(double amin, double a, bool is) { return sc_upscale(amin, a, is); }
static __device__ __noinline__ double sc_min_rare(double a, double b, bool is) { return sc_min(a, b, is); }

// ------------------------------------------------- robust scalar kernels
// protect_real_division (robust.c:144-166).  Shortcut: with t normal and
// exponent(b) <= exponent(t) + 989, |b| < 2^990 |t| <= fl(|t| Omega), so
// neither branch rescales.
static __device__ __noinline__ double protect_real_division_full(double b, double t) {
    double scale = 1.0;
    const double at = absd(t), ab = absd(b);
    if (at < kOmegaInv) {
        if (ab > at * kOmega) scale = (at * kOmega) / ab;
    } else {
        if (1.0 > at && ab > at * kOmega) scale = 1.0 / ab;
    }
    return scale;
}
__device__ __forceinline__ double protect_real_division(double b, double t) {
    const unsigned long long mb = mag(b), mt = mag(t);
    if (mt >= pow2_bits(-1022) && mt <= kInfBits && mb <= kInfBits && (mb >> 52) < (mt >> 52) + 990)
        return 1.0;
    return protect_real_division_full(b, t);
}
// protect_sum (robust.c:175-185).  Shortcut: |x|, |y| < 2^995 gives
// Omega - |y| > 2^995 > |x|.
static __device__ __noinline__ double protect_sum_full(double x, double y) {
    double scale = 1.0;
    if ((x > 0 && y > 0) || (x < 0 && y < 0))
        if (absd(x) > kOmega - absd(y)) scale = 0.5;
    return scale;
}
__device__ __forceinline__ double protect_sum(double x, double y) {
    if (mag(x) < pow2_bits(995) && mag(y) < pow2_bits(995)) return 1.0;
    return protect_sum_full(x, y);
}
// protect_update (robust.c:220-262), for t, x, y >= 0.  Shortcut: t, x <
// 2^497 and y < 2^995 give t*x < 2^994 < Omega - y and t < (Omega - y)/x.
static __device__ __noinline__ double protect_update_full(double tnorm, double xnorm, double ynorm, bool is) {
    double scale = 1.0;
    if (xnorm <= 1.0) {
        if (tnorm * xnorm > kOmega - ynorm) scale = 0.5;
    } else {
        if (tnorm > (kOmega - ynorm) / xnorm) scale = 0.5 / xnorm;
    }
    return is ? (double)ilogb(scale) : scale;
}
__device__ __forceinline__ double protect_update(double tnorm, double xnorm, double ynorm, bool is) {
    if (mag(tnorm) < pow2_bits(497) && mag(xnorm) < pow2_bits(497) && mag(ynorm) < pow2_bits(995))
        return sc_one(is);
    return protect_update_full(tnorm, xnorm, ynorm, is);
}
// protect_double_update (robust.c:270-285)
__device__ __forceinline__ double protect_double_update(double t1, double x1, double t2, double x2,
                                                        double y, bool is) {
    const double a1 = protect_update(t1, x1, y, is);
    const double a2 = protect_update(t2, x2, y, is);
    if (ubits(a1) == ubits(a2)) return a1;
    return sc_min_rare(a1, a2, is);
}
// Rare parts of solve_1x1: the rescaled difference and the scaling factor.
static __device__ __noinline__ double solve_1x1_scaled_diff(double s, double t, double lambda) {
    return (s * t) - (s * lambda);
}
static __device__ __noinline__ double solve_1x1_scale(double alpha, double s, bool is) {
    return is ? (double)ilogb(alpha / s) : alpha / s;
}
// solve_1x1_real_system (robust.c:422-479); returns 1 if |t-lambda| < smin.
__device__ __forceinline__ int solve_1x1(double smin, double t, double lambda, double &x,
                                         double &scale, bool is) {
    int info = 0;
    const double s = protect_sum(t, neg(lambda));
    double csr = is_one(s) ? t - lambda : solve_1x1_scaled_diff(s, t, lambda);
    if (mag(csr) < ubits(smin)) {          // absd(csr) < smin, smin > 0
        csr = smin;
        info = 1;
    }
    const double alpha = protect_real_division(x, csr);
    x = scale_by(alpha, x) / csr;
    if (is_one(alpha) && is_one(s)) scale = sc_one(is);
    else scale = solve_1x1_scale(alpha, s, is);
    return info;
}

// ------------------------------------------------------------- Givens
// LAPACK >= 3.10 dlartg (E. Anderson, "Algorithm 978: Safe scaling in the
// Level 1 BLAS", ACM TOMS 44(1), 2017), transposed as in reduce.c:14-24.
// rtmin = sqrt(2^-1022) = 2^-511 and rtmax = sqrt(2^1021) = 2^510 * sqrt(2)
// (correctly rounded), as bit patterns.
constexpr unsigned long long kRtminBits = 0x2000000000000000ULL;
constexpr unsigned long long kRtmaxBits = 0x5fd6a09e667f3bcdULL;
// The safe-scaled branch of the rotation (operands near underflow or
// overflow), out of line: rarely taken.  Returns (c, s before negation).
struct RotCS {
    double c, sv;
};
static __device__ __noinline__ RotCS givens_scaled(double f, double g) {
    const double safmin = 2.2250738585072014e-308;   // 2^-1022
    const double safmax = 1.0 / safmin;               // 2^1022
    const double f1 = absd(f), g1 = absd(g);
    const double u = fmin(safmax, fmax(safmin, fmax(f1, g1)));
    const double fs = f / u, gs = g / u;
    const double d = sqrt(fs * fs + gs * gs);
    RotCS r;
    r.c = absd(fs) / d;
    r.sv = gs / copysign(d, f);
    return r;
}
__device__ __forceinline__ void givens(double f, double g, double &c, double &s) {
    const unsigned long long mf = mag(f), mg = mag(g);
    double sv;
    if (is_zero(g)) {
        c = 1.0; sv = 0.0;
    } else if (is_zero(f)) {
        c = 0.0; sv = copysign(1.0, g);
    } else if (mf > kRtminBits && mf < kRtmaxBits && mg > kRtminBits && mg < kRtmaxBits) {
        // c = |f| / d and sv = g / copysign(d, f) = +-(g / d), exactly as the
        // FP64 divisions round them, from one reciprocal of d.
        const double d = sqrt(f * f + g * g);
        ddiv2_rn(absd(f), g, d, c, sv);
        if (ubits(f) >> 63) sv = neg(sv);
    } else {
        const RotCS r = givens_scaled(f, g);
        c = r.c;
        sv = r.sv;
    }
    s = neg(sv);
}

// ------------------------------------------- 2-norm, three accumulators
// LAPACK 3.10 dnrm2 as used in shifted_Hessenberg_solve.c:135-260.  Blue's
// thresholds for IEEE double (Anderson 2017): powers of two.
constexpr double kTsml = 0x1p-511;
constexpr double kTbig = 0x1p+486;
constexpr double kSsml = 0x1p+537;
constexpr double kSbig = 0x1p-538;

// Scaled square accumulation of the rare big and small ranges (not inlined,
// so the common middle range evaluates one fma).
static __device__ __noinline__ double nrm3_scaled_sq(double ax, double sc, double acc) {
    const double t = ax * sc;
    return fma(t, t, acc);
}

struct Nrm3 {
    double asml, amed, abig;
    __device__ __forceinline__ void init() { asml = amed = abig = 0.0; }
    __device__ __forceinline__ void add(double x) {
        const double ax = absd(x);
        const unsigned long long m = mag(x);
        if (m > pow2_bits(486) && m <= kInfBits) abig = nrm3_scaled_sq(ax, kSbig, abig);
        else if (m < pow2_bits(-511)) asml = nrm3_scaled_sq(ax, kSsml, asml);
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

// ------------------------------------------------ complex-shift helpers
// Complex values as (re, im) pairs; every product and update has one fixed
// fma shape, the same one the oracle spells, so results match bit for bit.
struct dcplx {
    double re, im;
};
__device__ __forceinline__ dcplx cmk(double re, double im) { return dcplx{re, im}; }
// LAPACK's CABS1: |Re z| + |Im z|, an upper bound of |z| and of each part.
__device__ __forceinline__ double cabs1(dcplx z) { return absd(z.re) + absd(z.im); }
__device__ __forceinline__ dcplx cmul(dcplx a, dcplx b) {           // a b
    return cmk(fma(a.re, b.re, -(a.im * b.im)), fma(a.re, b.im, a.im * b.re));
}
__device__ __forceinline__ dcplx cmulc(dcplx a, dcplx b) {          // conj(a) b
    return cmk(fma(a.re, b.re, a.im * b.im), fma(a.re, b.im, -(a.im * b.re)));
}
__device__ __forceinline__ dcplx cfma(dcplx a, dcplx b, dcplx y) {  // y + a b
    return cmk(fma(a.re, b.re, fma(-a.im, b.im, y.re)), fma(a.re, b.im, fma(a.im, b.re, y.im)));
}
__device__ __forceinline__ dcplx cfnma(dcplx a, dcplx b, dcplx y) { // y - a b
    return cmk(fma(-a.re, b.re, fma(a.im, b.im, y.re)), fma(-a.re, b.im, fma(-a.im, b.re, y.im)));
}
__device__ __forceinline__ dcplx cfmar(dcplx a, double h, dcplx y) { // y + a h, h real
    return cmk(fma(a.re, h, y.re), fma(a.im, h, y.im));
}
__device__ __forceinline__ dcplx cscal(double c, dcplx a) { return cmk(c * a.re, c * a.im); }
// Rotation pair of the back-transform and of Ytilde2:
//   out = c t1 - conj(s) t2,   next = c t2 + s t1.
__device__ __forceinline__ dcplx crot_out(double c, dcplx s, dcplx t1, dcplx t2) {
    const dcplx q = cmulc(s, t2);
    return cmk(fma(c, t1.re, -q.re), fma(c, t1.im, -q.im));
}
__device__ __forceinline__ dcplx crot_next(double c, dcplx s, dcplx t1, dcplx t2) {
    const dcplx p = cmul(s, t1);
    return cmk(fma(c, t2.re, p.re), fma(c, t2.im, p.im));
}

// protect_mul (robust.c:194-212): alpha with t (alpha x) safe.  Shortcut:
// |t|, |x| < 2^497 give |t||x| < 2^994 < Omega and |t| < Omega / |x|.
__device__ __forceinline__ double protect_mul(double tnorm, double xnorm) {
    if (mag(tnorm) < pow2_bits(497) && mag(xnorm) < pow2_bits(497)) return 1.0;
    double scale = 1.0;
    if (absd(xnorm) <= 1.0) {
        if (absd(tnorm) * absd(xnorm) > kOmega) scale = 0.5;
    } else {
        if (absd(tnorm) > kOmega / absd(xnorm)) scale = 0.5 / absd(xnorm);
    }
    return scale;
}

// Robust complex division in real arithmetic (robust.c:486-637): dladiv2,
// dladiv1, dladiv, every intermediate protected by protect_sum,
// protect_mul and protect_real_division.
__device__ __forceinline__ void c_dladiv2(double a, double b, double c, double d, double r, double t,
                                          double &ret, double &scale) {
    double res, alpha = 1.0;
    if (r != 0.0) {
        const double br = b * r;
        if (br != 0.0) {
            // (a + b r) t
            double s = protect_sum(a, br);
            res = (s * a) + (s * br);
            alpha = s * alpha;
            s = protect_mul(absd(t), absd(res));
            res = (s * res) * t;
            alpha = s * alpha;
        } else {
            // a t + (b t) r
            const double s1 = protect_mul(absd(t), absd(a));
            double tmp1 = (s1 * a) * t;
            const double s2 = protect_mul(absd(t), absd(b));
            double tmp2 = (s2 * b) * t;
            tmp2 = tmp2 * r;
            const double smin = fmin(s1, s2);
            tmp1 = tmp1 * (s1 / smin);
            tmp2 = tmp2 * (s2 / smin);
            alpha = smin * alpha;
            const double s = protect_sum(tmp1, tmp2);
            res = (s * tmp1) + (s * tmp2);
            alpha = s * alpha;
        }
    } else {
        // (a + d (b / c)) t
        const double s1 = protect_real_division(b, c);
        alpha = s1 * alpha;
        double tmp = (s1 * b) / c;
        const double s2 = protect_mul(absd(d), absd(tmp));
        alpha = s2 * alpha;
        tmp = d * (s2 * tmp);
        a = (s1 * s2) * a;
        double s = protect_sum(a, tmp);
        alpha = s * alpha;
        tmp = (s * a) + (s * tmp);
        s = protect_mul(absd(tmp), absd(t));
        alpha = s * alpha;
        res = (s * tmp) * t;
    }
    scale = alpha;
    ret = res;
}
__device__ __forceinline__ void c_dladiv1(double a, double b, double c, double d, double &p, double &q,
                                          double &scale) {
    const double r = d / c;
    const double dr = d * r;
    const double s1 = protect_sum(c, dr);
    const double sum = (s1 * c) + (s1 * dr);
    const double s2 = protect_real_division(1.0, sum);
    const double t = 1.0 / (s2 * sum);
    const double alpha = 1.0 / (s1 * s2);
    double beta1 = 1.0, beta2 = 1.0;
    c_dladiv2(a, b, c, d, r, t, p, beta1);
    c_dladiv2(b, -a, c, d, r, t, q, beta2);
    double beta = 1.0;
    if (!((beta1 > 1.0 && beta2 < 1.0) || (beta1 < 1.0 && beta2 > 1.0))) {
        beta = fmin(beta1, beta2);
        p = p * (beta / beta1);
        q = q * (beta / beta2);
    }
    scale = alpha * beta;
}
__device__ __forceinline__ void c_dladiv(double a, double b, double c, double d, double &xr, double &xi,
                                         double &scale) {
    if (absd(d) < absd(c)) {
        c_dladiv1(a, b, c, d, xr, xi, scale);
    } else {
        c_dladiv1(b, a, d, c, xr, xi, scale);
        xi = -xi;
    }
}
// Complex 1x1 solve x := (scale x) / (t - l) (solve_1x1_cmplx_system,
// robust.c:677-773, with a complex t); returns 1 if |t - l| was lifted to smin.
__device__ __forceinline__ int csolve_1x1(double smin, double tr, double ti, double lr, double li, dcplx &x,
                                          double &scale, bool is) {
    int info = 0;
    const double s = fmin(protect_sum(tr, -lr), protect_sum(ti, -li));
    double csr = (s * tr) - (s * lr);
    double csi = (s * ti) - (s * li);
    if (absd(csr) + absd(csi) < smin) {
        csr = smin;
        csi = 0.0;
        info = 1;
    }
    double alpha = 1.0;
    c_dladiv(x.re, x.im, csr, csi, x.re, x.im, alpha);
    scale = is ? (double)ilogb((1.0 / s) * alpha) : (1.0 / s) * alpha;
    return info;
}

// Complex Givens rotation of (f, g), f complex, g real: c real >= 0 and
// sigma with sigma f + c g = 0.  Exact power-of-two scaling: the phase of f
// from f scaled by its own exponent, |f| and g on the exponent of the larger
// (E. Anderson, "Algorithm 978: Safe scaling in the Level 1 BLAS", 2017);
// c = 0 when |f| < 2^-600 |g|.
__device__ __forceinline__ int exp_clamped(double m) {
    int e = (int)((ubits(m) >> 52) & 0x7ff) - 1023;
    return e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
}
__device__ __forceinline__ double pow2d(int e) { return __longlong_as_double((long long)pow2_bits(e)); }
__device__ __forceinline__ void cgivens(dcplx f, double g, double &c, dcplx &sg) {
    if (is_zero(g)) {
        c = 1.0;
        sg = cmk(0.0, 0.0);
        return;
    }
    if (is_zero(f.re) && is_zero(f.im)) {
        c = 0.0;
        sg = cmk(-copysign(1.0, g), 0.0);
        return;
    }
    const int ef = exp_clamped(fmax(absd(f.re), absd(f.im)));
    const int eg = exp_clamped(absd(g));
    const int e = ef > eg ? ef : eg;
    const double uf = pow2d(-ef);
    const double fsr = f.re * uf, fsi = f.im * uf;
    const double af1 = sqrt(fma(fsr, fsr, fsi * fsi));
    const double pr = fsr / af1, pi = fsi / af1;
    const double af = (ef - e < -600) ? 0.0 : af1 * pow2d(ef - e);
    const double gs = g * pow2d(-e);
    const double d = sqrt(fma(af, af, gs * gs));
    c = af / d;
    const double t = gs / d;
    sg = cmk(-(t * pr), t * pi);
}

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
// Invalidate an mbarrier whose memory is about to serve another purpose.
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Order earlier generic-proxy accesses before later async-proxy (TMA) ones:
// shared memory the CTA wrote itself, and global memory written by other
// CTAs whose completion this thread has observed.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
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
// Waits until at most one committed group is still in flight.
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
// Dynamic shared memory this launch was given, in bytes.
__device__ __forceinline__ unsigned dynamic_smem_bytes() {
    unsigned r;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
    return r;
}

}  // namespace hsr
