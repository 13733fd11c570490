// hsr_cplx.cu -- sm_103a kernels for complex-conjugate shifts.
//
// A shift mu = wr + i wi makes H - mu I complex on its diagonal only.  The
// sweep is the real one (hsr_kernels.cu) in complex arithmetic:
//   k_init_c    start vector eps3 in the real part, crossover columns
//               H(:, n-1) - mu e_n
//   k_diag_c    lane-per-pair: complex Givens generation of the diagonal tile
//               fused with the robust back-substitution (reduce.c:27-68 +
//               solve-task.c:19-225), the complex 1x1 solves going through the
//               robust complex division of robust.c:486-773; then the stage
//               operands W and Zs
//   k_part1_c   the exact no-rescale test per (tile, pair), the full complex
//               Part 1 of update-task.c:68-226 where a decision can fire
//   k_gemm_c    the real GEMM over H (hsr_kernels.cu) with a complex epilogue:
//               the imaginary parts are just more columns of W and Zs
//   k_finalize_c  reconciliation, complex back-transform, 2-norm, convergence
// Layout: pair p holds its real part in column 2p and its imaginary part in
// column 2p+1 of X, R, W, Zs, Zslow and of the per-column scalars pi, ytil,
// zlast and the shifts; the cosine of a rotation is Cr[.][2p], the complex
// sine Sr[.][2p] + i Sr[.][2p+1]; the per-pair scaling factor, norm bound,
// perturbation and protected-path flags live at column 2p.
//
// Magnitude bounds use cabs1 = |Re| + |Im| (LAPACK's CABS1).  Every complex
// operation has one fma shape (hsr_device.cuh) shared with the oracle's
// complex path, which the device reproduces bit for bit.
#include "hsr_device.cuh"
#include "hsr_kernels.h"

#include <cfloat>

namespace hsr {

// ---------------------------------------------------------------- init
// Start vectors: mode 0 eps3 (inverse_iteration.c:19-34), mode 1 the
// dlaein-style restart vector of round `its` (:36-57), both real; crossover
// columns H(:, n-1) - mu e_n (reduce.c:276-308); unit scaling factors.
__global__ void k_init_c(DevProblem P, int mode, const double *eps3_dev, int its) {
    const int p = blockIdx.y;
    if (2 * p >= P.S) return;
    const int k = 2 * p;
    const double eps3 = *eps3_dev;
    const int n = P.n;
    const double sq = sqrt((double)n);
    const double tmp = eps3 / (sq + 1.0);
    double *xr = P.X + (size_t)k * P.ldx, *xi = xr + P.ldx;
    double *rr = P.R + (size_t)k * P.ldr, *ri = rr + P.ldr;
    const double *hl = P.H + (size_t)(n - 1) * P.ldh;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double h = hl[i], hi = 0.0;
        if (i == n - 1) {
            h = h - P.wr[k];
            hi = -P.wr[k + 1];
        }
        rr[i] = h;
        ri[i] = hi;
        double v = eps3;
        if (mode == 1) {
            v = (i == 0) ? eps3 : tmp;
            if (i == n - 1 - its) v -= eps3 * sq;
        }
        xr[i] = v;
        xi[i] = 0.0;
    }
    if (blockIdx.x == 0) {
        const double ub = mode == 1 ? fmax(fmax(eps3, tmp), absd(tmp - eps3 / sq)) : eps3;
        for (int I = threadIdx.x; I < P.T; I += blockDim.x) {
            P.beta[(size_t)I * P.Spad + k] = sc_one(P.is);
            P.beta[(size_t)I * P.Spad + k + 1] = sc_one(P.is);
            P.ynorm[(size_t)I * P.Spad + k] = ub;
            P.ynorm[(size_t)I * P.Spad + k + 1] = ub;
        }
        if (threadIdx.x == 0) P.pert[k] = P.pert[k + 1] = 0;
    }
}

cudaError_t launch_init_c(const DevProblem &P, int mode, const double *eps3_dev, int its, cudaStream_t st) {
    int bx = (P.n + 255) / 256;
    if (bx > 64) bx = 64;
    dim3 g(bx, P.S / 2);
    k_init_c<<<g, 256, 0, st>>>(P, mode, eps3_dev, its);
    return cudaGetLastError();
}

// -------------------------------------------------------------- diagonal
// 32 pairs per CTA, one per lane, on NW warps (at least one per SM
// sub-partition).  Warp 0 evaluates each step's scalar chain -- complex
// Givens, the robust complex 1x1 solve, the three overflow decisions -- and
// hands its results to the others through shared memory; warps 1 .. NW-1
// update the rows of y and of the running column v, one step behind the
// chain: in step j warp 0 first updates row j-2 itself and then evaluates
// everything of step j-1's chain that does not need the new bounds, while
// the other warps update rows 0 .. j-3; after a barrier warp 0 folds their
// maxima into step j-1's third decision.  Every row sees the same operations
// in the same order as in the unpipelined form, so the result is unchanged
// bit for bit.  v and y live in shared memory as [row][lane] (real and
// imaginary parts in separate arrays); when 4*32*b doubles do not fit, in a
// global scratch region.  The bound of y(0:j-2) is the largest cabs1 at the
// start of the step, times the step's scaling factors.
//   NW = 8 with v/y in shared memory (two warps per sub-partition hide the
//   FP64 latency), NW = 4 with v/y in global scratch, where the CTAs share
//   SMs with the concurrent GEMM.
constexpr int kDiagWarpsC = 4;       // v/y in global scratch
constexpr int kDiagWarpsCSmem = 8;   // v/y in shared memory
constexpr int kDiagBcastC = 12;

// Everything but v/y: three staged columns of H, per-warp maxima [NW][2][32]
// and the broadcast slots.
__host__ __device__ constexpr size_t diagc_small_bytes(int b, int nw) {
    return (size_t)(3 * (b + 1)) * sizeof(double) + (size_t)nw * 2 * 32 * 8 + (size_t)kDiagBcastC * 32 * 8;
}
size_t diag_c_smem_bytes(int b, bool *global_vy) {
    const size_t small = diagc_small_bytes(b, kDiagWarpsCSmem);
    const size_t full = small + (size_t)4 * 32 * b * sizeof(double);
    const bool fits = full <= 220 * 1024;
    if (global_vy) *global_vy = !fits;
    return fits ? full : small;
}

template <int NW>
__global__ void __launch_bounds__(32 * NW) k_diag_c(DevProblem P, int J, double *gscratch) {
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int np = P.S / 2;
    const int p0 = blockIdx.x * 32;
    const int pidx = p0 + lane;
    const bool act = pidx < np;
    const int k = 2 * pidx;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    constexpr int NR = NW - 1;                                         // row warps
    {
        // A launch given less shared memory than the layout needs records a
        // shape error and touches nothing.
        const size_t need = diagc_small_bytes(b, NW) + (gscratch ? 0 : (size_t)4 * 32 * b * sizeof(double));
        if (need > dynamic_smem_bytes()) {
            if (threadIdx.x == 0) atomicOr(P.err, kErrShape);
            return;
        }
    }

    double *hc = sm;                                                   // [3][b+1]
    unsigned long long *pmax = reinterpret_cast<unsigned long long *>(sm + 3 * (b + 1));   // [NW][2][32]
    double *bc = sm + 3 * (b + 1) + NW * 2 * 32;                       // [kDiagBcastC][32]
    double *vr_, *vi_, *yr_, *yi_;
    if (gscratch) {
        vr_ = gscratch + (size_t)blockIdx.x * 4 * 32 * b;
    } else {
        vr_ = bc + kDiagBcastC * 32;
    }
    vi_ = vr_ + (size_t)32 * b;
    yr_ = vi_ + (size_t)32 * b;
    yi_ = yr_ + (size_t)32 * b;
#define VR(i) vr_[(size_t)(i) * 32 + lane]
#define VI(i) vi_[(size_t)(i) * 32 + lane]
#define YR(i) yr_[(size_t)(i) * 32 + lane]
#define YI(i) yi_[(size_t)(i) * 32 + lane]
#define PM(w, which) pmax[((w) * 2 + (which)) * 32 + lane]
#define BC(q) bc[(q) * 32 + lane]
#define HCOL(col) (hc + (size_t)((col) % 3) * (b + 1))

    // Load the crossover column and the solution tile, transposed.
    for (int c = wid; c < 32; c += NW) {
        const int pc = p0 + c;
        if (pc < np) {
            const double *rr = P.R + l + (size_t)(2 * pc) * P.ldr, *ri = rr + P.ldr;
            const double *xr = P.X + l + (size_t)(2 * pc) * P.ldx, *xi = xr + P.ldx;
            for (int i = lane; i < b; i += 32) {
                vr_[(size_t)i * 32 + c] = rr[i];
                vi_[(size_t)i * 32 + c] = ri[i];
                yr_[(size_t)i * 32 + c] = xr[i];
                yi_[(size_t)i * 32 + c] = xi[i];
            }
        } else {
            for (int i = lane; i < b; i += 32) {
                vr_[(size_t)i * 32 + c] = 1.0;
                vi_[(size_t)i * 32 + c] = 0.0;
                yr_[(size_t)i * 32 + c] = 0.0;
                yi_[(size_t)i * 32 + c] = 0.0;
            }
        }
    }

    const dcplx mu = act ? cmk(P.wr[k], P.wr[k + 1]) : cmk(0.0, 0.0);
    const double smin = fmax(DBL_EPSILON / 2 * cabs1(mu), P.smlnum);
    const double Hnorm = P.Hn[J + (size_t)J * P.T];
    double beta = act ? P.beta[(size_t)J * Spad + k] : sc_one(is);
    int pert = 0;

    const double *Hd = P.H + l + (size_t)l * P.ldh;
    auto stage_col = [&](int col) {                                    // H(l : l+col+1, l+col), warp 0
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
    __syncthreads();                                                   // tiles and columns loaded

    // Largest cabs1 of y(0:b-3) and v(0:b-3) for the first step.
    {
        unsigned long long ym = 0, vm = 0;
        if (wid > 0)
            for (int i = wid - 1; i < b - 2; i += NR) {
                ym = umax64(ym, abs_bits(cabs1(cmk(YR(i), YI(i)))));
                vm = umax64(vm, abs_bits(cabs1(cmk(VR(i), VI(i)))));
            }
        PM(wid, 0) = ym;
        PM(wid, 1) = vm;
    }

    // Chain state of warp 0.
    dcplx vcar = cmk(VR(b - 1), VI(b - 1)), ycar = cmk(YR(b - 1), YI(b - 1));
    double c = 0.0, a1 = 1.0, a2 = 1.0, a3 = 1.0;
    dcplx sg = cmk(0.0, 0.0), yc = sg, ys = sg, yj = sg, yjm1 = sg;

    // Parts 1-2 of step jj's chain: Givens, the 1x1 solve, the y(jj-1)
    // decision and update (solve-task.c:76-90), the next running column entry
    // (solve-task.c:105-108).  vjm1, yjm1_in are row jj-1.
    auto chain12 = [&](int jj, dcplx vjm1, dcplx yjm1_in) {
        const double *hcol = HCOL(jj - 1);
        const double hsub = hcol[jj];
        const dcplx hd = cmk(hcol[jj - 1] - mu.re, -mu.im);
        const dcplx vj = vcar;
        yj = ycar;
        yjm1 = yjm1_in;
        cgivens(vj, hsub, c, sg);
        if (act) {
            P.Cr[(size_t)(l + jj) * Spad + k] = c;
            P.Sr[(size_t)(l + jj) * Spad + k] = sg.re;
            P.Sr[(size_t)(l + jj) * Spad + k + 1] = sg.im;
        }
        // y(j) := y(j) / R(j,j), R(j,j) = c v(j) - conj(sigma) H(j,j-1).
        double phi = sc_one(is);
        pert |= csolve_1x1(smin, c * vj.re, c * vj.im, sg.re * hsub, (-sg.im) * hsub, yj, phi, is);
        beta = sc_combine(beta, phi, is);
        a1 = sc_value(phi, is);
        if (!is_one(a1)) yjm1 = cscal(a1, yjm1);
        phi = protect_double_update(cabs1(vjm1), cabs1(yj), cabs1(hd), cabs1(yj), cabs1(yjm1), is);
        a2 = sc_value(phi, is);
        if (!is_one(a2)) {
            yj = cscal(a2, yj);
            yjm1 = cscal(a2, yjm1);
        }
        beta = sc_combine(beta, phi, is);
        yc = cscal(c, yj);
        ys = cmulc(sg, yj);
        yjm1 = cfma(ys, hd, cfnma(yc, vjm1, yjm1));
        const dcplx sv = cmul(sg, vjm1);
        vcar = cmk(fma(c, hd.re, sv.re), fma(c, hd.im, sv.im));
    };
    // Part 3 of step jj's chain: the y(0:jj-2) decision (solve-task.c:92-100)
    // with the maxima of rows 0 .. jj-2 folded by the row warps, then the
    // step's scalars for the row warps, the solved entry y(jj) and y(jj-1).
    auto chain3 = [&](int jj) {
        unsigned long long ymb = 0, vmb = 0;
#pragma unroll
        for (int w = 1; w < NW; ++w) {
            ymb = umax64(ymb, PM(w, 0));
            vmb = umax64(vmb, PM(w, 1));
        }
        double ymax = from_bits(ymb);
        if (!is_one(a1)) ymax = a1 * ymax;
        if (!is_one(a2)) ymax = a2 * ymax;
        const double phi = protect_double_update(from_bits(vmb), cabs1(yj), Hnorm, cabs1(yj), ymax, is);
        a3 = sc_value(phi, is);
        if (!is_one(a3)) {
            yj = cscal(a3, yj);
            yjm1 = cscal(a3, yjm1);
            yc = cscal(c, yj);
            ys = cmulc(sg, yj);
        }
        beta = sc_combine(beta, phi, is);
        BC(0) = c;
        BC(1) = sg.re;
        BC(2) = sg.im;
        BC(3) = yc.re;
        BC(4) = yc.im;
        BC(5) = ys.re;
        BC(6) = ys.im;
        BC(7) = a1;
        BC(8) = a2;
        BC(9) = a3;
        YR(jj) = yj.re;
        YI(jj) = yj.im;
        ycar = yjm1;
    };

    if (wid == 0 && b >= 2) chain12(b - 1, cmk(VR(b - 2), VI(b - 2)), cmk(YR(b - 2), YI(b - 2)));
    __syncthreads();                                                   // first maxima in
    if (wid == 0 && b >= 2) chain3(b - 1);
    __syncthreads();                                                   // step b-1's scalars visible

    for (int j = b - 1; j >= 1; --j) {
        // Step j's scalars: registers on warp 0, shared memory for the rest.
        double sc_c = c, s1 = a1, s2 = a2, s3 = a3;
        dcplx sc_sg = sg, sc_yc = yc, sc_ys = ys;
        if (wid != 0) {
            sc_c = BC(0);
            sc_sg = cmk(BC(1), BC(2));
            sc_yc = cmk(BC(3), BC(4));
            sc_ys = cmk(BC(5), BC(6));
            s1 = BC(7);
            s2 = BC(8);
            s3 = BC(9);
        }
        const bool scaled = (!is_one(s1)) || (!is_one(s2)) || (!is_one(s3));
        const double *hcol = HCOL(j - 1);
        // Row i of step j (the unpipelined loop body).
        auto row = [&](int i, dcplx &yo, dcplx &vo) {
            const double h = hcol[i];
            dcplx yv = cmk(YR(i), YI(i));
            const dcplx vv = cmk(VR(i), VI(i));
            if (scaled) {
                if (!is_one(s1)) yv = cscal(s1, yv);
                if (!is_one(s2)) yv = cscal(s2, yv);
                if (!is_one(s3)) yv = cscal(s3, yv);
            }
            yo = cfmar(sc_ys, h, cfnma(sc_yc, vv, yv));
            const dcplx sv = cmul(sc_sg, vv);
            vo = cmk(fma(sc_c, h, sv.re), sv.im);
            YR(i) = yo.re;
            YI(i) = yo.im;
            VR(i) = vo.re;
            VI(i) = vo.im;
        };
        if (wid == 0) {
            if (j >= 2) {
                dcplx yn, vn;
                row(j - 2, yn, vn);                                    // enters step j-1's chain
                cp_async_wait_all();                                   // column j-2, staged last step
                __syncwarp();                                          // ... by all lanes of warp 0
                chain12(j - 1, vn, yn);
            }
            if (j >= 3) stage_col(j - 3);                              // for step j-2's chain
        } else {
            if (scaled) {
                for (int i = j + 1 + ((wid - 1 - (j + 1)) % NR + NR) % NR; i < b; i += NR) {
                    dcplx t = cmk(YR(i), YI(i));
                    if (!is_one(s1)) t = cscal(s1, t);
                    if (!is_one(s2)) t = cscal(s2, t);
                    if (!is_one(s3)) t = cscal(s3, t);
                    YR(i) = t.re;
                    YI(i) = t.im;
                }
            }
            unsigned long long ymx = 0, vmx = 0;
            for (int i = wid - 1; i < j - 2; i += NR) {                // rows 0 .. j-3
                dcplx yo, vo;
                row(i, yo, vo);
                ymx = umax64(ymx, abs_bits(cabs1(yo)));
                vmx = umax64(vmx, abs_bits(cabs1(vo)));
            }
            PM(wid, 0) = ymx;
            PM(wid, 1) = vmx;
        }
        __syncthreads();                                               // rows of step j done, maxima in
        if (wid == 0 && j >= 2) chain3(j - 1);
        __syncthreads();                                               // step j-1's scalars visible
    }

    double c0 = 1.0;
    dcplx s0 = cmk(0.0, 0.0);
    {
        dcplx y0 = cmk(0.0, 0.0);
        double a = 1.0;
        if (wid == 0) {
            dcplx v0 = b >= 2 ? vcar : cmk(VR(0), VI(0));
            y0 = b >= 2 ? ycar : cmk(YR(0), YI(0));
            if (J > 0) {
                // Final rotation with H(l, l-1) (reduce.c:53-61).
                const double hleft = P.H[l + (size_t)(l - 1) * P.ldh];
                if (hleft != 0) {
                    cgivens(v0, hleft, c0, s0);
                } else {
                    c0 = 1.0;
                    s0 = cmk(0.0, 0.0);
                }
                if (act) {
                    P.Cr[(size_t)l * Spad + k] = c0;
                    P.Sr[(size_t)l * Spad + k] = s0.re;
                    P.Sr[(size_t)l * Spad + k + 1] = s0.im;
                }
                v0 = cmk(fma(v0.re, c0, -(hleft * s0.re)), fma(v0.im, c0, hleft * s0.im));
            }
            double phi = sc_one(is);
            pert |= csolve_1x1(smin, v0.re, v0.im, 0.0, 0.0, y0, phi, is);
            beta = sc_combine(beta, phi, is);
            a = sc_value(phi, is);
            BC(0) = c0;
            BC(1) = s0.re;
            BC(2) = s0.im;
            BC(3) = a;
        }
        __syncthreads();
        if (wid != 0) {
            c0 = BC(0);
            s0 = cmk(BC(1), BC(2));
            a = BC(3);
        }
        if (!is_one(a))
            for (int i = 1 + ((wid - 1) % NW + NW) % NW; i < b; i += NW) {
                YR(i) = a * YR(i);
                YI(i) = a * YI(i);
            }
        if (wid == 0) {
            YR(0) = y0.re;
            YI(0) = y0.im;
        }
    }
    __syncthreads();

    for (int c = wid; c < 32; c += NW) {
        const int pc = p0 + c;
        if (pc < np) {
            double *xr = P.X + l + (size_t)(2 * pc) * P.ldx, *xi = xr + P.ldx;
            for (int i = lane; i < b; i += 32) {
                xr[i] = yr_[(size_t)i * 32 + c];
                xi[i] = yi_[(size_t)i * 32 + c];
            }
        }
    }
    if (act && wid == 0) {
        P.beta[(size_t)J * Spad + k] = beta;
        if (pert) P.pert[k] = P.pert[k + 1] = 1;
    }
    if (J == 0 || !act) return;

    if (wid == 0) {
        // W(q) = c_q prod_{p<q} sigma_p, pi = prod sigma (crossover propagation).
        dcplx pk = cmk(1.0, 0.0);
        for (int q = 0; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const dcplx sq = cmk(P.Sr[(size_t)(l + q) * Spad + k], P.Sr[(size_t)(l + q) * Spad + k + 1]);
            const dcplx w = cscal(cq, pk);
            P.W[(size_t)q * Spad + k] = w.re;
            P.W[(size_t)q * Spad + k + 1] = w.im;
            pk = cmul(pk, sq);
        }
        P.pi[k] = pk.re;
        P.pi[k + 1] = pk.im;
    }
    if (wid == 1) {
        // Ytilde2 (update-task.c:170-198): Zs(q) = Ytilde2(q-1), Zs(0) = 0,
        // zlast = Ytilde2(b-1); ytilde = -conj(sigma_0) x_0 for Part 1.
        unsigned long long zmx = 0;
        dcplx z = cscal(c0, cmk(YR(0), YI(0)));
        P.Zs[k] = 0.0;
        P.Zs[k + 1] = 0.0;
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const dcplx sq = cmk(P.Sr[(size_t)(l + q) * Spad + k], P.Sr[(size_t)(l + q) * Spad + k + 1]);
            const dcplx t2 = cmk(YR(q), YI(q));
            const dcplx zo = crot_out(cq, sq, z, t2);
            z = crot_next(cq, sq, z, t2);
            P.Zs[(size_t)q * Spad + k] = zo.re;
            P.Zs[(size_t)q * Spad + k + 1] = zo.im;
            zmx = umax64(zmx, abs_bits(cabs1(zo)));
        }
        zmx = umax64(zmx, abs_bits(cabs1(z)));
        P.zlast[k] = z.re;
        P.zlast[k + 1] = z.im;
        P.z2n[k] = from_bits(zmx);
        const dcplx q0 = cmulc(s0, cmk(YR(0), YI(0)));
        P.ytil[k] = -q0.re;
        P.ytil[k + 1] = -q0.im;
    }
#undef VR
#undef VI
#undef YR
#undef YI
#undef PM
#undef HCOL
#undef BC
}

// The dynamic shared-memory limit of each k_diag_c form only ever grows.
template <int NW>
cudaError_t diag_c_smem_attr(size_t smem) {
    static size_t configured = 0;
    return raise_smem_limit((const void *)k_diag_c<NW>, &configured, smem);
}

cudaError_t launch_diag_c(const DevProblem &P, int J, int b, double *gscratch, cudaStream_t st) {
    bool gvy = false;
    const size_t smem = diag_c_smem_bytes(b, &gvy);
    if (gvy && !gscratch) return cudaErrorInvalidValue;
    const int grid = (P.S / 2 + 31) / 32;
    if (gscratch) {
        const size_t small = diagc_small_bytes(b, kDiagWarpsC);
        const cudaError_t e = diag_c_smem_attr<kDiagWarpsC>(small);
        if (e != cudaSuccess) return e;
        k_diag_c<kDiagWarpsC><<<grid, 32 * kDiagWarpsC, small, st>>>(P, J, gscratch);
    } else {
        const cudaError_t e = diag_c_smem_attr<kDiagWarpsCSmem>(smem);
        if (e != cudaSuccess) return e;
        k_diag_c<kDiagWarpsCSmem><<<grid, 32 * kDiagWarpsCSmem, smem, st>>>(P, J, nullptr);
    }
    return cudaGetLastError();
}

int diag_c_ctas_per_sm(int b) {
    bool gvy = false;
    const size_t smem = diag_c_smem_bytes(b, &gvy);
    if (gvy) return 0;
    if (diag_c_smem_attr<kDiagWarpsCSmem>(smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_diag_c<kDiagWarpsCSmem>, 32 * kDiagWarpsCSmem,
                                                      smem) != cudaSuccess)
        return 0;
    return nb;
}

// --------------------------------------------------------------- Part 1
// The real k_part1 in complex arithmetic: lane per pair for the exact
// no-rescale test, one warp per (tile, pair) for the full Part 1.  The test
// of hsr_kernels.cu (part1_fast) holds with cabs1 bounds: with hn,
// cabs1(mu), cabs1(ytilde) < 2^496 and Yn < 2^993, each updated entry has
// cabs1 <= (2^993 + 2^992 + 2^992)(1+u)^3 < 2^995, so with Hn, ||Ytilde2|| <
// 2^497 neither decision can fire.
__device__ __forceinline__ bool part1_fast_c(double Xs, double Ys, double hn, double mu1, double yt1, double Yn,
                                             double Hn, double z2) {
    return ubits(Xs) == ubits(Ys) && mag(hn) < pow2_bits(496) && mag(mu1) < pow2_bits(496) &&
           mag(yt1) < pow2_bits(496) && mag(Yn) < pow2_bits(993) && mag(Hn) < pow2_bits(497) &&
           mag(z2) < pow2_bits(497);
}

__device__ __noinline__ void part1_full_c(const DevProblem &P, int J, int I, int pidx) {
    const int lane = threadIdx.x & 31;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    const int T = P.T;
    const int k = 2 * pidx;
    const int r0 = P.fr[I], m = P.fr[I + 1] - r0;
    const int l = P.fr[J], b = P.fr[J + 1] - l;
    const bool applyShift = (I == J - 1);
    double *yr = P.X + r0 + (size_t)k * P.ldx, *yi = yr + P.ldx;
    const double *h = P.H + r0 + (size_t)(l - 1) * P.ldh;
    const dcplx mu = cmk(P.wr[k], P.wr[k + 1]);
    double Ys = P.beta[(size_t)I * Spad + k];
    const double Xs = P.beta[(size_t)J * Spad + k];
    double Yn = P.ynorm[(size_t)I * Spad + k];

    // Part 0: consistent scaling.
    if (Xs < Ys) {
        const double a = sc_upscale(Xs, Ys, is);
        if (!is_one(a))
            for (int i = lane; i < m; i += 32) {
                yr[i] = a * yr[i];
                yi[i] = a * yi[i];
            }
        Yn = a * Yn;
        Ys = Xs;
    }
    // Part 1: y -= (H(I, l-1) - mu e_last) ytilde, ytilde = -conj(sigma_0) x_0.
    dcplx x0 = cmk(P.X[l + (size_t)k * P.ldx], P.X[l + (size_t)(k + 1) * P.ldx]);
    if (Ys < Xs) x0 = cscal(sc_upscale(Ys, Xs, is), x0);
    const dcplx s0 = cmk(P.Sr[(size_t)l * Spad + k], P.Sr[(size_t)l * Spad + k + 1]);
    const dcplx q0 = cmulc(s0, x0);
    const dcplx yt = cmk(-q0.re, -q0.im);
    const double hnrm = P.hn[I + (size_t)J * T];
    const double alpha = protect_update(fmax(hnrm, cabs1(mu)), cabs1(yt), Yn, is);
    const double a = sc_value(alpha, is);
    unsigned long long mx = 0;
    if (!is_one(a)) {
        const dcplx at = cscal(a, yt);
        for (int i = lane; i < m; i += 32) {
            dcplx v = cmk(fma(-h[i], at.re, a * yr[i]), fma(-h[i], at.im, a * yi[i]));
            if (applyShift && i == m - 1) v = cfma(mu, at, v);
            yr[i] = v.re;
            yi[i] = v.im;
            mx = umax64(mx, abs_bits(cabs1(v)));
        }
    } else {
        for (int i = lane; i < m; i += 32) {
            dcplx v = cmk(fma(-h[i], yt.re, yr[i]), fma(-h[i], yt.im, yi[i]));
            if (applyShift && i == m - 1) v = cfma(mu, yt, v);
            yr[i] = v.re;
            yi[i] = v.im;
            mx = umax64(mx, abs_bits(cabs1(v)));
        }
    }
    Ys = sc_combine(Ys, alpha, is);
    for (int o = 16; o; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    Yn = from_bits(mx);

    // Part 2 decision.
    bool slow = false;
    double z2 = P.z2n[k];
    double *zs = P.Zslow + (size_t)I * P.tlsz * Spad + k;      // re at zs[q*Spad], im at +1
    if (Ys < Xs) {
        slow = true;
        const double a2 = sc_upscale(Ys, Xs, is);
        const double *xr = P.X + l + (size_t)k * P.ldx, *xi = xr + P.ldx;
        unsigned long long zmx = 0;
        dcplx z = cscal(P.Cr[(size_t)l * Spad + k], cscal(a2, cmk(xr[0], xi[0])));
        for (int q = 1; q < b; ++q) {
            const double cq = P.Cr[(size_t)(l + q) * Spad + k];
            const dcplx sq = cmk(P.Sr[(size_t)(l + q) * Spad + k], P.Sr[(size_t)(l + q) * Spad + k + 1]);
            const dcplx t2 = cscal(a2, cmk(xr[q], xi[q]));
            const dcplx zo = crot_out(cq, sq, z, t2);
            z = crot_next(cq, sq, z, t2);
            if (lane == 0) {
                zs[(size_t)(q - 1) * Spad] = zo.re;
                zs[(size_t)(q - 1) * Spad + 1] = zo.im;
            }
            zmx = umax64(zmx, abs_bits(cabs1(zo)));
        }
        zmx = umax64(zmx, abs_bits(cabs1(z)));
        if (lane == 0) {
            zs[(size_t)(b - 1) * Spad] = z.re;
            zs[(size_t)(b - 1) * Spad + 1] = z.im;
        }
        z2 = from_bits(zmx);
    }
    const double tsc = protect_update(P.Hn[I + (size_t)J * T], z2, Yn, is);
    const double ta = sc_value(tsc, is);
    if (!is_one(ta)) {
        if (!slow) {
            for (int q = lane; q < b - 1; q += 32) {
                zs[(size_t)q * Spad] = P.Zs[(size_t)(q + 1) * Spad + k];
                zs[(size_t)q * Spad + 1] = P.Zs[(size_t)(q + 1) * Spad + k + 1];
            }
            if (lane == 0) {
                zs[(size_t)(b - 1) * Spad] = P.zlast[k];
                zs[(size_t)(b - 1) * Spad + 1] = P.zlast[k + 1];
            }
            __syncwarp();
        }
        slow = true;
        __syncwarp();
        for (int q = lane; q < b; q += 32) {
            zs[(size_t)q * Spad] = ta * zs[(size_t)q * Spad];
            zs[(size_t)q * Spad + 1] = ta * zs[(size_t)q * Spad + 1];
        }
        for (int i = lane; i < m; i += 32) {
            yr[i] = ta * yr[i];
            yi[i] = ta * yi[i];
        }
        Ys = sc_combine(Ys, tsc, is);
    }
    __syncwarp();
    if (lane == 0) {
        P.beta[(size_t)I * Spad + k] = Ys;
        P.ynorm[(size_t)I * Spad + k] = 0.0;
        P.slow[(size_t)I * Spad + k] = slow ? 1 : 0;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(256) k_part1_c(DevProblem P, int J) {
    const int lane = threadIdx.x & 31;
    const int np = P.S / 2;
    const int pw = blockIdx.x * kPart1Shifts + (threadIdx.x >> 5) * 32;
    if (pw >= np) return;
    const int pidx = pw + lane;
    const bool act = pidx < np;
    const int k = 2 * pidx;
    const size_t Spad = (size_t)P.Spad;
    const size_t T = (size_t)P.T;
    double mu1 = 0.0, yt1 = 0.0, z2 = 0.0, Xs = 0.0;
    if (act) {
        mu1 = cabs1(cmk(P.wr[k], P.wr[k + 1]));
        yt1 = cabs1(cmk(P.ytil[k], P.ytil[k + 1]));
        z2 = P.z2n[k];
        Xs = P.beta[(size_t)J * Spad + k];
    }
    bool any = false;
    if (act) {
        for (int I = 0; I < J; ++I) {
            const size_t ik = (size_t)I * Spad + k;
            if (part1_fast_c(Xs, P.beta[ik], P.hn[I + J * T], mu1, yt1, P.ynorm[ik], P.Hn[I + J * T], z2)) {
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
            const size_t ik = (size_t)I * Spad + k;
            pend = !part1_fast_c(Xs, P.beta[ik], P.hn[I + J * T], mu1, yt1, P.ynorm[ik], P.Hn[I + J * T], z2);
        }
        unsigned msk = __ballot_sync(0xffffffffu, pend);
        while (msk) {
            const int src = __ffs(msk) - 1;
            msk &= msk - 1;
            part1_full_c(P, J, I, pw + src);
        }
    }
}

cudaError_t launch_part1_c(const DevProblem &P, int J, cudaStream_t st) {
    const int np = P.S / 2;
    k_part1_c<<<(np + kPart1Shifts - 1) / kPart1Shifts, 256, 0, st>>>(P, J);
    return cudaGetLastError();
}

// -------------------------------------------------------------- finalize
// Lane per pair: smin = min_I beta (robust.c:58-82), complex back-transform
// with the tile upscalings (shifted_Hessenberg_solve.c:153-215), the
// three-accumulator 2-norm over real and imaginary parts, convergence
// ||y|| > 0.1/sqrt(n) (:33-40).  Rows pass through shared memory 32 at a
// time so that both columns of every pair are read and written coalesced.
__global__ void __launch_bounds__(32) k_finalize_c(DevProblem P, double *colnorm, int *status,
                                                   double *scale_out) {
    __shared__ double bre[32][33], bim[32][33];
    const int lane = threadIdx.x;
    const int np = P.S / 2;
    const int p0 = blockIdx.x * 32;
    const int pidx = p0 + lane;
    const bool act = pidx < np;
    const int k = 2 * pidx;
    const bool is = P.is != 0;
    const size_t Spad = (size_t)P.Spad;
    const int n = P.n;

    double smin = act ? P.beta[k] : sc_one(is);
    for (int I = 1; I < P.T; ++I)
        if (act) smin = sc_min(smin, P.beta[(size_t)I * Spad + k], is);

    Nrm3 acc;
    acc.init();
    dcplx tau1 = cmk(0.0, 0.0);
    int I = 0;
    double alpha = act ? sc_upscale(smin, P.beta[k], is) : 1.0;
    for (int r0 = 0; r0 < n; r0 += 32) {
        const int rows = min(32, n - r0);
        __syncwarp();
        for (int c = 0; c < 32; ++c) {
            const int pc = p0 + c;
            if (pc < np && lane < rows) {
                bre[lane][c] = P.X[r0 + lane + (size_t)(2 * pc) * P.ldx];
                bim[lane][c] = P.X[r0 + lane + (size_t)(2 * pc + 1) * P.ldx];
            }
        }
        __syncwarp();
        for (int t = 0; t < rows; ++t) {
            const int i = r0 + t;
            if (i == P.fr[I + 1]) {
                ++I;
                alpha = act ? sc_upscale(smin, P.beta[(size_t)I * Spad + k], is) : 1.0;
            }
            if (i == 0) {
                tau1 = cscal(alpha, cmk(bre[0][lane], bim[0][lane]));
                continue;
            }
            const dcplx tau2 = cscal(alpha, cmk(bre[t][lane], bim[t][lane]));
            const double c = act ? P.Cr[(size_t)i * Spad + k] : 0.0;
            const dcplx s = act ? cmk(P.Sr[(size_t)i * Spad + k], P.Sr[(size_t)i * Spad + k + 1]) : cmk(0.0, 0.0);
            const dcplx out = crot_out(c, s, tau1, tau2);
            tau1 = crot_next(c, s, tau1, tau2);
            acc.add(out.re);
            acc.add(out.im);
            if (t == 0) {
                if (act) {
                    P.X[(i - 1) + (size_t)k * P.ldx] = out.re;
                    P.X[(i - 1) + (size_t)(k + 1) * P.ldx] = out.im;
                }
            } else {
                bre[t - 1][lane] = out.re;
                bim[t - 1][lane] = out.im;
            }
        }
        __syncwarp();
        for (int c = 0; c < 32; ++c) {
            const int pc = p0 + c;
            if (pc < np && lane < rows - 1) {
                P.X[r0 + lane + (size_t)(2 * pc) * P.ldx] = bre[lane][c];
                P.X[r0 + lane + (size_t)(2 * pc + 1) * P.ldx] = bim[lane][c];
            }
        }
    }
    if (act) {
        P.X[(n - 1) + (size_t)k * P.ldx] = tau1.re;
        P.X[(n - 1) + (size_t)(k + 1) * P.ldx] = tau1.im;
        acc.add(tau1.re);
        acc.add(tau1.im);
        const double ynrm = acc.finish();
        const int ok = (ynrm > 0.1 / sqrt((double)n)) ? 1 : 0;
        colnorm[k] = colnorm[k + 1] = ynrm;
        status[k] = status[k + 1] = ok;
        if (scale_out) scale_out[pidx] = smin;
    }
}

cudaError_t launch_finalize_c(const DevProblem &P, double *colnorm, int *status, double *scale_out,
                              cudaStream_t st) {
    k_finalize_c<<<(P.S / 2 + 31) / 32, 32, 0, st>>>(P, colnorm, status, scale_out);
    return cudaGetLastError();
}

}  // namespace hsr
