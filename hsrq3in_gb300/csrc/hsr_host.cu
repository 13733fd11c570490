// hsr_host.cu -- C ABI and host orchestration of the GB300 inverse iteration.
//
// The drop-in tiled_inverse_iteration (inverse_iteration.h:19-22) copies H and
// the shifts to the device, runs the sweep of tile columns, the convergence
// check and the restart rounds (inverse_iteration.c:176-205, restated with the
// intended semantics), and copies vr and wr back.  Workspaces are cached per
// host thread and grow on demand.
#include "hsr_common.h"
#include "hsr_device.cuh"
#include "hsr_kernels.h"
#include "../../include/hsrq3in_gb300.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace hsr {
namespace {

thread_local int g_last_status = HSR_OK;
thread_local long g_launches = 0;

// Optional per-kernel-class device timing: an event pair around every launch
// on the launching stream, resolved after the call's final synchronisation.
enum KernelClass { kcSetup = 0, kcDiag, kcPart1, kcGemm, kcFinal, kcOther, kcH2D, kcD2H, kcGemmTop, kcCount };
struct Timing {
    bool enabled = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<int> cls;
    double ms[kcCount] = {0};
    long launches[kcCount] = {0};
    double gemm_fma[1] = {0};   // algorithmic FMAs of the timed kcGemm launches
    void reset() {
        used = 0;
        cls.clear();
        for (int i = 0; i < kcCount; ++i) ms[i] = 0.0, launches[i] = 0;
        gemm_fma[0] = 0.0;
    }
    cudaEvent_t next() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(int c, cudaStream_t st) {
        if (!enabled) return;
        cls.push_back(c);
        cudaEventRecord(next(), st);
    }
    void end(cudaStream_t st) {
        if (!enabled) return;
        cudaEventRecord(next(), st);
    }
    // Forget the last begin/end pair (a launch that did not happen).
    void drop_last() {
        if (!enabled || cls.empty()) return;
        cls.pop_back();
        used -= 2;
    }
    void resolve() {
        if (!enabled) return;
        for (size_t i = 0; i < cls.size(); ++i) {
            float t = 0.f;
            if (2 * i + 1 < used && cudaEventElapsedTime(&t, pool[2 * i], pool[2 * i + 1]) == cudaSuccess) {
                ms[cls[i]] += t;
                launches[cls[i]] += 1;
            }
        }
        used = 0;
        cls.clear();
    }
};
thread_local Timing g_timing;

#define HSR_CK(x)                                  \
    do {                                           \
        cudaError_t e_ = (x);                      \
        if (e_ != cudaSuccess) {                   \
            last_cuda_error() = e_;                \
            return HSR_ERR_CUDA;                   \
        }                                          \
    } while (0)
#define HSR_LAUNCH_C(c, stream, x)                 \
    do {                                           \
        ++g_launches;                              \
        g_timing.begin((c), (stream));             \
        cudaError_t le_ = (x);                     \
        g_timing.end((stream));                    \
        HSR_CK(le_);                               \
    } while (0)

cudaError_t &last_cuda_error() {
    static thread_local cudaError_t e = cudaSuccess;
    return e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library does not link libcuda directly.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Looked up once; the initialiser of a function-local static runs exactly
// once even when several host threads make their first call together.
EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        return nullptr;
    }();
    return fn;
}

}  // namespace

// 2-D FP64 tensor map: inner extent `inner` (contiguous), outer extent
// `outer`, row pitch `ld` elements, box {bx, by}; out-of-range reads are 0.
bool encode_tensor_map(CUtensorMap *m, const double *base, unsigned long long inner, unsigned long long outer,
                       unsigned long long ld, unsigned bx, unsigned by) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {ld * sizeof(double)};
    cuuint32_t box[2] = {bx, by};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {

bool make_map(CUtensorMap *m, const double *base, unsigned long long inner, unsigned long long outer,
              unsigned long long ld, unsigned bx, unsigned by) {
    return encode_tensor_map(m, base, inner, outer, ld, bx, by);
}

inline long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

// Device buffer that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

struct Workspace {
    int device = -1;
    cudaStream_t stream = nullptr;
    // Look-ahead: the diagonal kernel of the next tile runs on a
    // high-priority side stream while the current stage's GEMM finishes.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_top = nullptr, ev_diag = nullptr;
    cudaError_t ensure_side() {
        if (side) return cudaSuccess;
        int lo = 0, hi = 0;
        cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_top, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_diag, cudaEventDisableTiming);
        return e;
    }
    DevBuf H, X, wr, R, Cr, Sr, beta, ynorm, W, Zs, vecs, Zslow, slow, pert, fr, bits, err, colnorm,
        status, scale, tmpX, perm, gscratch, probe;
    ~Workspace() { release(); }
    void release() {
        DevBuf *all[] = {&H, &X, &wr, &R, &Cr, &Sr, &beta, &ynorm, &W, &Zs, &vecs, &Zslow, &slow, &pert,
                         &fr, &bits, &err, &colnorm, &status, &scale, &tmpX, &perm, &gscratch, &probe};
        for (DevBuf *b : all) b->release();
        if (stream) cudaStreamDestroy(stream);
        if (side) cudaStreamDestroy(side);
        if (ev_top) cudaEventDestroy(ev_top);
        if (ev_diag) cudaEventDestroy(ev_diag);
        stream = side = nullptr;
        ev_top = ev_diag = nullptr;
    }
};

Workspace &ws() {
    static thread_local Workspace w;
    int dev = 0;
    cudaGetDevice(&dev);
    if (w.device != dev) {
        w.release();
        w.device = dev;
    }
    return w;
}

// Where the diagonal kernels keep v and y for a pass of `ctas` CTAs: in
// shared memory when all CTAs are resident in one wave, else in global
// scratch.  Beyond one wave the shared-memory form would run a second wave
// of the latency-bound diagonal solve, and its large CTAs would keep the
// concurrent GEMM's CTAs off their SMs; with v/y in global scratch a CTA
// needs ~10 KB and shares each SM with two GEMM CTAs (measured at n = 10^4:
// 1800 -> 1784 ms real, 1980 -> 1877 ms complex; at n <= 6144, where one
// wave suffices, shared memory is faster).
bool diag_vy_global(int ctas, int per_sm) {
    if (per_sm <= 0) return true;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return ctas > per_sm * sms;
}

// One solve over a column range: the sweep J = T-1 .. 0, finalize, normalize.
struct Solver {
    int n, T, tlsz, is;
    std::vector<int> fr;
    const double *H;
    long long ldh;
    double *X;      // column 0 of the whole block
    long long ldx;
    double *wr;     // device shifts of the whole block
    int S;          // columns of the whole block
    int Scap;       // columns per pass (workspace capacity)
    int Spad;
    double smlnum;
    cudaStream_t st;
    Workspace *w;
    CUtensorMap tmH, tmW[2], tmZ[2];
    CUtensorMap tmWn[2], tmZn[2];   // 16-column boxes for launch_gemm_narrow
    double *eps3_dev;
    int *d_status;     // [S] per final column
    double *d_colnorm; // [S]
    double *d_scale;   // [S] or null
    unsigned char *d_pert;  // [S]
};

// Stage operands (W, Zs and the per-shift scalars) are double-buffered by
// tile parity so that the diagonal kernel of tile J-1 can write its operands
// while the GEMM of stage J still reads those of tile J.
DevProblem problem_for(const Solver &s, int off, int cnt, int parity = 0) {
    Workspace &w = *s.w;
    DevProblem P{};
    P.n = s.n;
    P.T = s.T;
    P.S = cnt;
    P.Spad = s.Spad;
    P.tlsz = s.tlsz;
    P.fr = w.fr.as<int>();
    P.H = s.H;
    P.ldh = s.ldh;
    P.wr = s.wr + off;
    P.X = s.X + (size_t)off * s.ldx;
    P.ldx = s.ldx;
    P.R = w.R.as<double>();
    P.ldr = round_up(s.n, 4);
    P.Cr = w.Cr.as<double>();
    P.Sr = w.Sr.as<double>();
    P.beta = w.beta.as<double>();
    P.ynorm = w.ynorm.as<double>();
    P.Hn = w.bits.as<double>();
    P.hn = w.bits.as<double>() + (size_t)s.T * s.T;
    const size_t stage = (size_t)s.tlsz * s.Spad;
    P.W = w.W.as<double>() + parity * stage;
    P.Zs = w.Zs.as<double>() + parity * stage;
    double *v = w.vecs.as<double>() + parity * 4 * (size_t)s.Spad;
    P.pi = v;
    P.ytil = v + s.Spad;
    P.z2n = v + 2 * (size_t)s.Spad;
    P.zlast = v + 3 * (size_t)s.Spad;
    P.Zslow = w.Zslow.as<double>();
    P.slow = w.slow.as<unsigned char>();
    P.pert = s.d_pert + off;
    P.smlnum = s.smlnum;
    P.is = s.is;
    P.err = w.err.as<int>();
    return P;
}

// Runs columns [off, off+cnt) through one pass; mode as launch_init.
// Per stage J (main stream M, high-priority side stream D):
//   M: part1(J) -> [ev_top] -> gemm(J) on rows above tile J-1 -> wait ev_diag
//   D: wait ev_top -> gemm(J) on the rows of tile J-1 -> diag(J-1) -> [ev_diag]
// so the short GEMM of tile J-1's rows and then diag(J-1), a latency-bound
// sequential kernel, run beside the bulk of the FP64-bound GEMM of stage J,
// and the last wave of the short GEMM leaves no SM idle.  Stage operands
// alternate buffers by parity.
int run_pass(Solver &s, int mode, int its, int off, int cnt) {
    Workspace &w = *s.w;
    HSR_CK(w.ensure_side());
    cudaStream_t M = s.st, D = w.side;
    for (int c0 = 0; c0 < cnt; c0 += s.Scap) {
        const int cc = std::min(s.Scap, cnt - c0);
        DevProblem P0 = problem_for(s, off + c0, cc, 0);
        HSR_LAUNCH_C(kcSetup, M, launch_init(P0, mode, s.eps3_dev, its, M));
        if (mode == 2) ++g_launches;
        const int b = s.tlsz;
        const bool big = diag_smem_bytes(b) < (size_t)64 * b * sizeof(double) ||
                         diag_vy_global((cc + 31) / 32, diag_ctas_per_sm(b));
        double *gs = big ? w.gscratch.as<double>() : nullptr;
        {
            const int J = s.T - 1;
            DevProblem P = problem_for(s, off + c0, cc, J & 1);
            HSR_LAUNCH_C(kcDiag, M, launch_diag(P, J, s.fr[J + 1] - s.fr[J], gs, M));
        }
        for (int J = s.T - 1; J >= 1; --J) {
            const int bj = s.fr[J + 1] - s.fr[J];
            DevProblem P = problem_for(s, off + c0, cc, J & 1);
            DevProblem Pn = problem_for(s, off + c0, cc, (J - 1) & 1);
            HSR_LAUNCH_C(kcPart1, M, launch_part1(P, J, M));
            HSR_CK(cudaEventRecord(w.ev_top, M));
            HSR_CK(cudaStreamWaitEvent(D, w.ev_top, 0));
            cudaError_t fe = cudaSuccess;
            ++g_launches;
            g_timing.begin(kcDiag, D);
            const bool fused = launch_diag_fused(Pn, P, J - 1, s.fr[J] - s.fr[J - 1], D, &fe);
            g_timing.end(D);
            if (!fused) {
                --g_launches;
                g_timing.drop_last();
            }
            HSR_CK(fe);
            if (fused) {
                // Few shifts: the top GEMM ran inside the diagonal CTAs.
            } else if (gemm_prefers_narrow(s.fr[J] - s.fr[J - 1], cc))
                HSR_LAUNCH_C(kcGemmTop, D, launch_gemm_narrow(P, J, s.fr[J - 1], s.fr[J], s.tmH, s.tmWn[J & 1],
                                                              s.tmZn[J & 1], D));
            else
                HSR_LAUNCH_C(kcGemmTop, D,
                             launch_gemm(P, J, s.fr[J - 1], s.fr[J], s.tmH, s.tmW[J & 1], s.tmZ[J & 1], D));
            if (!fused) HSR_LAUNCH_C(kcDiag, D, launch_diag(Pn, J - 1, s.fr[J] - s.fr[J - 1], gs, D));
            HSR_CK(cudaEventRecord(w.ev_diag, D));
            if (s.fr[J - 1] > 0)
                HSR_LAUNCH_C(kcGemm, M, launch_gemm(P, J, 0, s.fr[J - 1], s.tmH, s.tmW[J & 1], s.tmZ[J & 1], M));
            HSR_CK(cudaStreamWaitEvent(M, w.ev_diag, 0));
            if (g_timing.enabled) g_timing.gemm_fma[0] += (double)s.fr[J - 1] * (2.0 * bj - 1.0) * cc;
        }
        DevProblem P = problem_for(s, off + c0, cc, 0);
        HSR_LAUNCH_C(kcFinal, M, launch_finalize(P, s.d_colnorm + off + c0, s.d_status + off + c0,
                                                 s.d_scale ? s.d_scale + off + c0 : nullptr, M));
        HSR_LAUNCH_C(kcFinal, M, launch_normalize(P, s.d_colnorm + off + c0, s.d_status + off + c0, M));
    }
    return HSR_OK;
}

void partition(int n, int T, int tlsz, std::vector<int> &p) {
    p.assign(T + 1, 0);
    for (int i = 1; i < T; ++i) p[i] = n - (T - i) * tlsz;
    p[0] = 0;
    p[T] = n;
}

// Core: device H (ldh even, aligned), device X (n x S, ldx), device wr.
int solve_device(int n, const double *dH, long long ldh, int S, double *dwr, int tlsz, double *dX,
                 long long ldx, const hsr_options *opt, cudaStream_t st, double *d_scale_user,
                 int *d_status_user, std::vector<int> *h_status, std::vector<unsigned char> *h_pert,
                 std::vector<double> *h_scale, std::vector<double> *h_norm, std::vector<double> *h_tile_scales) {
    Workspace &w = ws();
    hsr_options o{};
    if (opt) o = *opt;
    Solver s{};
    s.n = n;
    s.tlsz = tlsz;
    s.T = (n + tlsz - 1) / tlsz;
    s.is = o.scaling == HSR_SCALING_DOUBLE ? 0 : 1;
    partition(n, s.T, tlsz, s.fr);
    s.H = dH;
    s.ldh = ldh;
    s.X = dX;
    s.ldx = ldx;
    s.wr = dwr;
    s.S = S;
    s.st = st;
    s.w = &w;
    {
        const double eps = DBL_EPSILON / 2;
        s.smlnum = std::fmax(2 * DBL_MIN, DBL_MIN * ((double)n / eps));
    }
    const int T = s.T;
    // Workspace per column: R, Cr, Sr, Zslow (~n each), W/Zs (tlsz each),
    // beta/ynorm (T each), slow (T bytes).  Cap the pass width by the budget.
    {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        double budget = o.hbm_budget_bytes > 0 ? o.hbm_budget_bytes : 0.6 * (double)free_b;
        const double per_col = 8.0 * (4.0 * round_up(n, 4) + 4.0 * tlsz + 2.0 * T + 16) + T;
        long long cap = (long long)(budget / per_col);
        cap = std::max<long long>(32, std::min<long long>(cap, S));
        cap = std::min<long long>(cap, 65535);  // grid.y extent of the per-column kernels
        s.Scap = (int)cap;
    }
    s.Spad = (int)round_up(s.Scap, 64);
    const size_t Sp = (size_t)s.Spad;
    const size_t ldr = (size_t)round_up(n, 4);
    HSR_CK(w.R.ensure(ldr * Sp * 8));
    HSR_CK(w.Cr.ensure((size_t)n * Sp * 8));
    HSR_CK(w.Sr.ensure((size_t)n * Sp * 8));
    HSR_CK(w.beta.ensure((size_t)T * Sp * 8));
    HSR_CK(w.ynorm.ensure((size_t)T * Sp * 8));
    HSR_CK(w.W.ensure(2 * (size_t)tlsz * Sp * 8));
    HSR_CK(w.Zs.ensure(2 * (size_t)tlsz * Sp * 8));
    HSR_CK(w.vecs.ensure(2 * 4 * Sp * 8));
    HSR_CK(w.Zslow.ensure((size_t)T * tlsz * Sp * 8));
    HSR_CK(w.slow.ensure((size_t)T * Sp));
    HSR_CK(w.fr.ensure((size_t)(T + 1) * sizeof(int)));
    HSR_CK(w.bits.ensure((2 * (size_t)T * T + 2) * 8));
    HSR_CK(w.err.ensure(16));
    HSR_CK(w.colnorm.ensure((size_t)S * 8));
    HSR_CK(w.status.ensure((size_t)S * sizeof(int)));
    HSR_CK(w.pert.ensure((size_t)S));
    if (!d_scale_user && (h_scale || h_tile_scales)) HSR_CK(w.scale.ensure((size_t)S * 8));
    if (diag_smem_bytes(tlsz) < (size_t)64 * tlsz * sizeof(double) ||
        diag_vy_global((s.Scap + 31) / 32, diag_ctas_per_sm(tlsz)))
        HSR_CK(w.gscratch.ensure((size_t)((Sp + 31) / 32) * 64 * tlsz * 8));
    HSR_CK(cudaMemsetAsync(w.W.p, 0, 2 * (size_t)tlsz * Sp * 8, st));
    HSR_CK(cudaMemsetAsync(w.Zs.p, 0, 2 * (size_t)tlsz * Sp * 8, st));
    HSR_CK(cudaMemsetAsync(w.err.p, 0, 16, st));
    HSR_CK(cudaMemcpyAsync(w.fr.p, s.fr.data(), (T + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    s.d_status = d_status_user ? d_status_user : w.status.as<int>();
    s.d_colnorm = w.colnorm.as<double>();
    // The workspace scale buffer only when this call sized it: one left by an
    // earlier call may hold fewer than S entries.
    const bool own_scale = !d_scale_user && (h_scale || h_tile_scales);
    s.d_scale = d_scale_user ? d_scale_user : (own_scale ? w.scale.as<double>() : nullptr);
    s.d_pert = w.pert.as<unsigned char>();

    if (!make_map(&s.tmH, dH, (unsigned long long)n, (unsigned long long)n, (unsigned long long)ldh, kGemmBM,
                  kGemmKC) ||
        !make_map(&s.tmW[0], w.W.as<double>(), Sp, (unsigned long long)tlsz, Sp, kGemmBN, kGemmKC) ||
        !make_map(&s.tmW[1], w.W.as<double>() + (size_t)tlsz * Sp, Sp, (unsigned long long)tlsz, Sp, kGemmBN,
                  kGemmKC) ||
        !make_map(&s.tmZ[0], w.Zs.as<double>(), Sp, (unsigned long long)tlsz, Sp, kGemmBN, kGemmKC) ||
        !make_map(&s.tmZ[1], w.Zs.as<double>() + (size_t)tlsz * Sp, Sp, (unsigned long long)tlsz, Sp, kGemmBN,
                  kGemmKC))
        return HSR_ERR_CUDA;
    for (int par = 0; par < 2; ++par)
        if (!make_map(&s.tmWn[par], w.W.as<double>() + (size_t)par * tlsz * Sp, Sp, (unsigned long long)tlsz, Sp,
                      kGemmBNNarrow, kGemmKC) ||
            !make_map(&s.tmZn[par], w.Zs.as<double>() + (size_t)par * tlsz * Sp, Sp, (unsigned long long)tlsz, Sp,
                      kGemmBNNarrow, kGemmKC))
            return HSR_ERR_CUDA;

    // Norms and eps3.
    unsigned long long *bits = w.bits.as<unsigned long long>();
    HSR_CK(cudaMemsetAsync(bits, 0, (2 * (size_t)T * T + 2) * 8, st));
    {
        DevProblem P0 = problem_for(s, 0, std::min(S, s.Scap));
        HSR_LAUNCH_C(kcSetup, st, launch_norms(P0, bits, bits + (size_t)T * T, bits + 2 * (size_t)T * T,
                                               w.err.as<int>() + 1, st));
        ++g_launches;
    }
    double hinf = 0.0;
    HSR_CK(cudaMemcpyAsync(&hinf, bits + 2 * (size_t)T * T, 8, cudaMemcpyDeviceToHost, st));
    int nanflag[2] = {0, 0};
    HSR_CK(cudaMemcpyAsync(nanflag, w.err.as<int>(), 8, cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaStreamSynchronize(st));
    if (nanflag[1] & 1) hinf = NAN;
    const double eps3 = hinf * (DBL_EPSILON / 2);
    s.eps3_dev = reinterpret_cast<double *>(bits + 2 * (size_t)T * T + 1);
    HSR_CK(cudaMemcpyAsync(s.eps3_dev, &eps3, 8, cudaMemcpyHostToDevice, st));

    const bool user_rhs = o.user_rhs != 0;
    if (S > 0) {
        int rc = run_pass(s, user_rhs ? 2 : 0, 0, 0, S);
        if (rc) return rc;
    }

    // Convergence and restarts (intended semantics of inverse_iteration.c:176-205).
    std::vector<int> st_h(S);
    std::vector<double> wr_h;
    int front = 0, its = 0;
    const int max_its = o.max_restarts < 0 ? n : std::min(o.max_restarts, n);
    int result = HSR_OK;
    while (S > 0) {
        HSR_CK(cudaMemcpyAsync(st_h.data() + front, s.d_status + front, (S - front) * sizeof(int),
                               cudaMemcpyDeviceToHost, st));
        HSR_CK(cudaStreamSynchronize(st));
        int all = 1;
        for (int k = front; k < S; ++k)
            if (!st_h[k]) all = 0;
        if (all || user_rhs || its >= max_its) break;
        // Stable partition of [front, S): converged first.
        const int m = S - front;
        std::vector<int> perm;
        perm.reserve(m);
        for (int k = 0; k < m; ++k)
            if (st_h[front + k]) perm.push_back(k);
        const int nc = (int)perm.size();
        for (int k = 0; k < m; ++k)
            if (!st_h[front + k]) perm.push_back(k);
        HSR_CK(w.tmpX.ensure((size_t)n * m * 8));
        HSR_CK(w.perm.ensure((size_t)m * sizeof(int)));
        HSR_CK(cudaMemcpyAsync(w.perm.p, perm.data(), m * sizeof(int), cudaMemcpyHostToDevice, st));
        HSR_LAUNCH_C(kcOther, st, launch_gather_cols(w.tmpX.as<double>(), n, dX + (size_t)front * ldx, ldx, n,
                                                     w.perm.as<int>(), m, st));
        HSR_CK(cudaMemcpy2DAsync(dX + (size_t)front * ldx, ldx * 8, w.tmpX.p, (size_t)n * 8, (size_t)n * 8, m,
                                 cudaMemcpyDeviceToDevice, st));
        // Permute the small per-column arrays on the host.
        auto permute = [&](auto *dptr, size_t elem) -> int {
            if (!dptr) return HSR_OK;
            std::vector<unsigned char> a((size_t)m * elem), b((size_t)m * elem);
            HSR_CK(cudaMemcpyAsync(a.data(), reinterpret_cast<unsigned char *>(dptr) + (size_t)front * elem,
                                   (size_t)m * elem, cudaMemcpyDeviceToHost, st));
            HSR_CK(cudaStreamSynchronize(st));
            for (int j = 0; j < m; ++j) memcpy(&b[(size_t)j * elem], &a[(size_t)perm[j] * elem], elem);
            HSR_CK(cudaMemcpyAsync(reinterpret_cast<unsigned char *>(dptr) + (size_t)front * elem, b.data(),
                                   (size_t)m * elem, cudaMemcpyHostToDevice, st));
            HSR_CK(cudaStreamSynchronize(st));
            return HSR_OK;
        };
        int rc;
        if ((rc = permute(dwr, 8))) return rc;
        if ((rc = permute(s.d_scale, 8))) return rc;
        if ((rc = permute(s.d_pert, 1))) return rc;
        if ((rc = permute(s.d_status, sizeof(int)))) return rc;
        if ((rc = permute(s.d_colnorm, 8))) return rc;
        for (int j = 0; j < nc; ++j) st_h[front + j] = 1;
        front += nc;
        rc = run_pass(s, 1, its, front, S - front);
        if (rc) return rc;
        ++its;
    }
    int nonconv = 0;
    for (int k = 0; k < S; ++k) nonconv += !st_h[k];
    if (nonconv) result = HSR_ERR_NOT_CONVERGED;

    int errw = 0;
    HSR_CK(cudaMemcpyAsync(&errw, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaStreamSynchronize(st));
    g_timing.resolve();
    if (errw) return HSR_ERR_DEVICE;
    if (h_status) *h_status = st_h;
    if (h_pert) {
        h_pert->resize(S);
        HSR_CK(cudaMemcpy(h_pert->data(), s.d_pert, S, cudaMemcpyDeviceToHost));
    }
    if (h_scale && s.d_scale) {
        h_scale->resize(S);
        HSR_CK(cudaMemcpy(h_scale->data(), s.d_scale, (size_t)S * 8, cudaMemcpyDeviceToHost));
    }
    if (h_norm) {
        h_norm->resize(S);
        HSR_CK(cudaMemcpy(h_norm->data(), s.d_colnorm, (size_t)S * 8, cudaMemcpyDeviceToHost));
    }
    if (h_tile_scales) {
        // Per-tile factors of the last pass of each column (valid when one
        // pass covered every column).
        h_tile_scales->assign((size_t)T * S, 0.0);
        if (S <= s.Scap) {
            std::vector<double> tmp((size_t)T * Sp);
            HSR_CK(cudaMemcpy(tmp.data(), w.beta.p, (size_t)T * Sp * 8, cudaMemcpyDeviceToHost));
            for (int I = 0; I < T; ++I)
                for (int k = 0; k < S; ++k) (*h_tile_scales)[(size_t)I * S + k] = tmp[(size_t)I * Sp + k];
        }
    }
    return result;
}

// Tile sizes of the plain path recorded by hsr_autotune_plain, by order.
std::mutex g_plain_tune_mu;
std::map<int, int> g_plain_tune;

// Default tile size by order, from sweeps of the plain path on GB300 (all
// shifts): 64 at n = 1000 and 2048, 128 at n = 4096, 160 at n = 10^4.
int plain_default_tlsz(int n) { return n <= 2560 ? 64 : (n <= 6144 ? 128 : 160); }

// tlsz for order n: the tuned entry of the nearest order within a factor of
// two, else the default.
int plain_tlsz_for(int n) {
    std::lock_guard<std::mutex> g(g_plain_tune_mu);
    int best = 0;
    double bd = 1e300;
    for (auto &kv : g_plain_tune) {
        const double d = std::fabs(std::log((double)kv.first / n));
        if (d < bd) {
            bd = d;
            best = kv.second;
        }
    }
    return (best > 0 && bd <= std::log(2.0)) ? best : plain_default_tlsz(n);
}

int check_args(int n, int ldH, int nrhs, int tlsz, int ldvr, const void *H, const void *wr, const void *vr) {
    if (n <= 0 || ldH < n || nrhs < 0 || tlsz <= 0 || (tlsz % 4) != 0 || ldvr < n || !H) return HSR_ERR_ARG;
    if (nrhs > 0 && (!wr || !vr)) return HSR_ERR_ARG;
    return HSR_OK;
}

}  // namespace

// ----------------------------------------------------- caller's host blocks
// A column block moved between a caller's host buffer and device memory by SM
// loads and stores: dst(i, j) = src(i, j) for i < rows, j < cols, both
// column-major.  Used when the host buffer is page-locked and mapped into the
// device's address space; after long solves the copy engines were measured
// running far below their idle rate on this path, the SMs were not.
template <typename V>
__global__ void __launch_bounds__(256) k_copy_cols(V *__restrict__ dst, long long ldd, const V *__restrict__ src,
                                                   long long lds, int rows, int cols) {
    for (int j = blockIdx.x; j < cols; j += gridDim.x) {
        const V *s = src + (size_t)j * lds;
        V *d = dst + (size_t)j * ldd;
        for (int i = threadIdx.x; i < rows; i += blockDim.x) d[i] = s[i];
    }
}

// Device address of a page-locked host buffer mapped into the current
// device's address space, or null: cudaPointerAttributes::devicePointer is
// the address the current device may dereference, null where there is none
// (pageable memory, or a block pinned for another device without the
// portable flag), and those buffers keep the copy engines.
void *mapped_view(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

cudaError_t copy_cols(double *dst, long long ldd, const double *src, long long lds, int rows, int cols,
                      cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const int grid = cols < 1216 ? cols : 1216;
    const bool wide = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 16 == 0) &&
                      rows % 2 == 0 && ldd % 2 == 0 && lds % 2 == 0;
    ++g_launches;
    if (wide)
        k_copy_cols<double2><<<grid, 256, 0, st>>>(reinterpret_cast<double2 *>(dst), ldd / 2,
                                                    reinterpret_cast<const double2 *>(src), lds / 2, rows / 2, cols);
    else
        k_copy_cols<double><<<grid, 256, 0, st>>>(dst, ldd, src, lds, rows, cols);
    return cudaGetLastError();
}

namespace {

int host_call(int n, const double *H, int ldH, int nrhs, double *wr, int tlsz, int rhs_tlsz, double *vr,
              int ldvr, const hsr_options *opt, hsr_column_info *info) {
    g_launches = 0;
    g_timing.reset();
    if (tlsz == 0 && n > 0) tlsz = plain_tlsz_for(n);
    int rc = check_args(n, ldH, nrhs, tlsz, ldvr, H, wr, vr);
    if (rc) return rc;
    if (rhs_tlsz <= 0) return HSR_ERR_ARG;
    if (nrhs == 0) return HSR_OK;
    Workspace &w = ws();
    if (!w.stream) HSR_CK(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
    cudaStream_t st = w.stream;
    // Keep the caller's leading dimensions on the device when they allow it
    // (TMA needs an even pitch for H), so each transfer is one contiguous copy.
    const long long ldh = (ldH % 2 == 0) ? ldH : round_up(n, 32);
    const long long ldx = ldvr;
    HSR_CK(w.H.ensure((size_t)ldh * n * 8));
    HSR_CK(w.X.ensure((size_t)ldx * nrhs * 8));
    HSR_CK(w.wr.ensure((size_t)nrhs * 8));
    g_timing.begin(kcH2D, st);
    if (const void *Hm = mapped_view(H))
        HSR_CK(copy_cols(w.H.as<double>(), ldh, static_cast<const double *>(Hm), ldH, n, n, st));
    else if (ldh == ldH)
        HSR_CK(cudaMemcpyAsync(w.H.p, H, ((size_t)ldH * (n - 1) + n) * 8, cudaMemcpyHostToDevice, st));
    else
        HSR_CK(cudaMemcpy2DAsync(w.H.p, ldh * 8, H, (size_t)ldH * 8, (size_t)n * 8, n, cudaMemcpyHostToDevice, st));
    HSR_CK(cudaMemcpyAsync(w.wr.p, wr, (size_t)nrhs * 8, cudaMemcpyHostToDevice, st));
    g_timing.end(st);
    hsr_options o{};
    if (opt) o = *opt;
    if (o.user_rhs)
        HSR_CK(cudaMemcpyAsync(w.X.p, vr, ((size_t)ldvr * (nrhs - 1) + n) * 8, cudaMemcpyHostToDevice, st));
    std::vector<int> hs;
    std::vector<unsigned char> hp;
    std::vector<double> hsc, hn, hts;
    const bool want = info != nullptr;
    rc = solve_device(n, w.H.as<double>(), ldh, nrhs, w.wr.as<double>(), tlsz, w.X.as<double>(), ldx, &o, st,
                      nullptr, nullptr, want && info->status ? &hs : nullptr,
                      want && info->perturbed ? &hp : nullptr, want && info->scale ? &hsc : nullptr,
                      want && info->norm ? &hn : nullptr, want && info->tile_scales ? &hts : nullptr);
    if (rc < 0) return rc;
    g_timing.begin(kcD2H, st);
    if (void *Xm = mapped_view(vr))   // the caller's padding rows stay untouched
        HSR_CK(copy_cols(static_cast<double *>(Xm), ldvr, w.X.as<double>(), ldx, n, nrhs, st));
    else if (ldvr == n)   // no padding rows in the caller's block: one contiguous copy
        HSR_CK(cudaMemcpyAsync(vr, w.X.p, (size_t)n * nrhs * 8, cudaMemcpyDeviceToHost, st));
    else             // leave the caller's padding rows untouched
        HSR_CK(cudaMemcpy2DAsync(vr, (size_t)ldvr * 8, w.X.p, ldx * 8, (size_t)n * 8, nrhs,
                                 cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaMemcpyAsync(wr, w.wr.p, (size_t)nrhs * 8, cudaMemcpyDeviceToHost, st));
    g_timing.end(st);
    HSR_CK(cudaStreamSynchronize(st));
    g_timing.resolve();
    if (want) {
        if (info->status) memcpy(info->status, hs.data(), (size_t)nrhs * sizeof(int));
        if (info->perturbed) memcpy(info->perturbed, hp.data(), (size_t)nrhs);
        if (info->scale) memcpy(info->scale, hsc.data(), (size_t)nrhs * 8);
        if (info->norm) memcpy(info->norm, hn.data(), (size_t)nrhs * 8);
        if (info->tile_scales) memcpy(info->tile_scales, hts.data(), hts.size() * 8);
    }
    return rc;
}


// ------------------------------------------------------- complex shifts
// Pair p of a complex solve owns columns 2p (real part) and 2p+1 (imaginary
// part) of X and of every per-column workspace; the shifts are interleaved
// the same way.  A pass runs the same stage schedule as run_pass, with the
// complex kernels (hsr_cplx.cu) and the complex epilogue of the GEMM; off and
// cnt count columns and are even.
int run_pass_c(Solver &s, int mode, int its, int off, int cnt) {
    Workspace &w = *s.w;
    HSR_CK(w.ensure_side());
    cudaStream_t M = s.st, D = w.side;
    for (int c0 = 0; c0 < cnt; c0 += s.Scap) {
        const int cc = std::min(s.Scap, cnt - c0);
        const bool gvy = diag_vy_global((cc / 2 + 31) / 32, diag_c_ctas_per_sm(s.tlsz));
        double *gs = gvy ? w.gscratch.as<double>() : nullptr;
        DevProblem P0 = problem_for(s, off + c0, cc, 0);
        HSR_LAUNCH_C(kcSetup, M, launch_init_c(P0, mode, s.eps3_dev, its, M));
        {
            const int J = s.T - 1;
            DevProblem P = problem_for(s, off + c0, cc, J & 1);
            HSR_LAUNCH_C(kcDiag, M, launch_diag_c(P, J, s.fr[J + 1] - s.fr[J], gs, M));
        }
        for (int J = s.T - 1; J >= 1; --J) {
            const int bj = s.fr[J + 1] - s.fr[J];
            DevProblem P = problem_for(s, off + c0, cc, J & 1);
            DevProblem Pn = problem_for(s, off + c0, cc, (J - 1) & 1);
            HSR_LAUNCH_C(kcPart1, M, launch_part1_c(P, J, M));
            HSR_CK(cudaEventRecord(w.ev_top, M));
            HSR_CK(cudaStreamWaitEvent(D, w.ev_top, 0));
            HSR_LAUNCH_C(kcGemmTop, D,
                         launch_gemm_c(P, J, s.fr[J - 1], s.fr[J], s.tmH, s.tmW[J & 1], s.tmZ[J & 1], D));
            HSR_LAUNCH_C(kcDiag, D, launch_diag_c(Pn, J - 1, s.fr[J] - s.fr[J - 1], gs, D));
            HSR_CK(cudaEventRecord(w.ev_diag, D));
            if (s.fr[J - 1] > 0)
                HSR_LAUNCH_C(kcGemm, M,
                             launch_gemm_c(P, J, 0, s.fr[J - 1], s.tmH, s.tmW[J & 1], s.tmZ[J & 1], M));
            HSR_CK(cudaStreamWaitEvent(M, w.ev_diag, 0));
            if (g_timing.enabled) g_timing.gemm_fma[0] += (double)s.fr[J - 1] * (2.0 * bj - 1.0) * cc;
        }
        DevProblem P = problem_for(s, off + c0, cc, 0);
        HSR_LAUNCH_C(kcFinal, M, launch_finalize_c(P, s.d_colnorm + off + c0, s.d_status + off + c0,
                                                   s.d_scale ? s.d_scale + (off + c0) / 2 : nullptr, M));
        HSR_LAUNCH_C(kcFinal, M, launch_normalize(P, s.d_colnorm + off + c0, s.d_status + off + c0, M));
    }
    return HSR_OK;
}

// Complex solve on device data: H (ldh even, aligned), dwc [2*np] interleaved
// shifts (a workspace copy: permuted during restarts and restored before
// return), X n x 2np.  Pairs that do not converge are solved again with the
// restart vectors of successive rounds; their positions are unchanged on
// return.  Host outputs are per pair.
int solve_device_cplx(int n, const double *dH, long long ldh, int np, double *dwc, int tlsz, double *dX,
                      long long ldx, const hsr_options *opt, cudaStream_t st, int *d_status_pairs,
                      double *d_scale_pairs, std::vector<int> *h_status, std::vector<unsigned char> *h_pert,
                      std::vector<double> *h_scale, std::vector<double> *h_norm) {
    Workspace &w = ws();
    hsr_options o{};
    if (opt) o = *opt;
    Solver s{};
    s.n = n;
    s.tlsz = tlsz;
    s.T = (n + tlsz - 1) / tlsz;
    s.is = o.scaling == HSR_SCALING_DOUBLE ? 0 : 1;
    partition(n, s.T, tlsz, s.fr);
    s.H = dH;
    s.ldh = ldh;
    s.X = dX;
    s.ldx = ldx;
    s.wr = dwc;
    const int S = 2 * np;
    s.S = S;
    s.st = st;
    s.w = &w;
    {
        const double eps = DBL_EPSILON / 2;
        s.smlnum = std::fmax(2 * DBL_MIN, DBL_MIN * ((double)n / eps));
    }
    const int T = s.T;
    {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        double budget = o.hbm_budget_bytes > 0 ? o.hbm_budget_bytes : 0.6 * (double)free_b;
        const double per_col = 8.0 * (4.0 * round_up(n, 4) + 4.0 * tlsz + 2.0 * T + 16) + T + 2.0 * tlsz * 8;
        long long cap = (long long)(budget / per_col);
        cap = std::max<long long>(64, std::min<long long>(cap, S));
        cap = std::min<long long>(cap, 65534);
        s.Scap = (int)(cap & ~1LL);
    }
    s.Spad = (int)round_up(s.Scap, 64);
    const size_t Sp = (size_t)s.Spad;
    const size_t ldr = (size_t)round_up(n, 4);
    HSR_CK(w.R.ensure(ldr * Sp * 8));
    HSR_CK(w.Cr.ensure((size_t)n * Sp * 8));
    HSR_CK(w.Sr.ensure((size_t)n * Sp * 8));
    HSR_CK(w.beta.ensure((size_t)T * Sp * 8));
    HSR_CK(w.ynorm.ensure((size_t)T * Sp * 8));
    HSR_CK(w.W.ensure(2 * (size_t)tlsz * Sp * 8));
    HSR_CK(w.Zs.ensure(2 * (size_t)tlsz * Sp * 8));
    HSR_CK(w.vecs.ensure(2 * 4 * Sp * 8));
    HSR_CK(w.Zslow.ensure((size_t)T * tlsz * Sp * 8));
    HSR_CK(w.slow.ensure((size_t)T * Sp));
    HSR_CK(w.fr.ensure((size_t)(T + 1) * sizeof(int)));
    HSR_CK(w.bits.ensure((2 * (size_t)T * T + 2) * 8));
    HSR_CK(w.err.ensure(16));
    HSR_CK(w.colnorm.ensure((size_t)S * 8));
    HSR_CK(w.status.ensure((size_t)S * sizeof(int)));
    HSR_CK(w.pert.ensure((size_t)S));
    HSR_CK(w.scale.ensure((size_t)np * 8));
    {
        if (diag_vy_global((s.Scap / 2 + 31) / 32, diag_c_ctas_per_sm(tlsz))) HSR_CK(w.gscratch.ensure((size_t)((Sp / 2 + 31) / 32) * 4 * 32 * tlsz * 8));
    }
    HSR_CK(cudaMemsetAsync(w.W.p, 0, 2 * (size_t)tlsz * Sp * 8, st));
    HSR_CK(cudaMemsetAsync(w.Zs.p, 0, 2 * (size_t)tlsz * Sp * 8, st));
    HSR_CK(cudaMemsetAsync(w.err.p, 0, 16, st));
    HSR_CK(cudaMemcpyAsync(w.fr.p, s.fr.data(), (T + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    s.d_status = w.status.as<int>();
    s.d_colnorm = w.colnorm.as<double>();
    s.d_scale = w.scale.as<double>();
    s.d_pert = w.pert.as<unsigned char>();

    if (!make_map(&s.tmH, dH, (unsigned long long)n, (unsigned long long)n, (unsigned long long)ldh, kGemmBM,
                  kGemmKC) ||
        !make_map(&s.tmW[0], w.W.as<double>(), Sp, (unsigned long long)tlsz, Sp, kGemmBN, kGemmKC) ||
        !make_map(&s.tmW[1], w.W.as<double>() + (size_t)tlsz * Sp, Sp, (unsigned long long)tlsz, Sp, kGemmBN,
                  kGemmKC) ||
        !make_map(&s.tmZ[0], w.Zs.as<double>(), Sp, (unsigned long long)tlsz, Sp, kGemmBN, kGemmKC) ||
        !make_map(&s.tmZ[1], w.Zs.as<double>() + (size_t)tlsz * Sp, Sp, (unsigned long long)tlsz, Sp, kGemmBN,
                  kGemmKC))
        return HSR_ERR_CUDA;

    unsigned long long *bits = w.bits.as<unsigned long long>();
    HSR_CK(cudaMemsetAsync(bits, 0, (2 * (size_t)T * T + 2) * 8, st));
    {
        DevProblem P0 = problem_for(s, 0, std::min(S, s.Scap));
        HSR_LAUNCH_C(kcSetup, st, launch_norms(P0, bits, bits + (size_t)T * T, bits + 2 * (size_t)T * T,
                                               w.err.as<int>() + 1, st));
        ++g_launches;
    }
    double hinf = 0.0;
    HSR_CK(cudaMemcpyAsync(&hinf, bits + 2 * (size_t)T * T, 8, cudaMemcpyDeviceToHost, st));
    int nanflag[2] = {0, 0};
    HSR_CK(cudaMemcpyAsync(nanflag, w.err.as<int>(), 8, cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaStreamSynchronize(st));
    if (nanflag[1] & 1) hinf = NAN;
    const double eps3 = hinf * (DBL_EPSILON / 2);
    s.eps3_dev = reinterpret_cast<double *>(bits + 2 * (size_t)T * T + 1);
    HSR_CK(cudaMemcpyAsync(s.eps3_dev, &eps3, 8, cudaMemcpyHostToDevice, st));

    int rc = run_pass_c(s, 0, 0, 0, S);
    if (rc) return rc;

    // Restarts: stable partition of the pairs (converged first), tracked in
    // `order` so that the original positions are restored at the end.
    std::vector<int> order(np), st_h(S);
    for (int p = 0; p < np; ++p) order[p] = p;
    bool permuted = false;
    auto apply_perm = [&](int front, const std::vector<int> &perm) -> int {
        const int m = (int)perm.size();
        std::vector<int> cperm(2 * m);
        for (int q = 0; q < m; ++q) {
            cperm[2 * q] = 2 * perm[q];
            cperm[2 * q + 1] = 2 * perm[q] + 1;
        }
        HSR_CK(w.tmpX.ensure((size_t)n * 2 * m * 8));
        HSR_CK(w.perm.ensure((size_t)2 * m * sizeof(int)));
        HSR_CK(cudaMemcpyAsync(w.perm.p, cperm.data(), 2 * m * sizeof(int), cudaMemcpyHostToDevice, st));
        HSR_LAUNCH_C(kcOther, st, launch_gather_cols(w.tmpX.as<double>(), n, dX + (size_t)2 * front * ldx, ldx,
                                                     n, w.perm.as<int>(), 2 * m, st));
        HSR_CK(cudaMemcpy2DAsync(dX + (size_t)2 * front * ldx, ldx * 8, w.tmpX.p, (size_t)n * 8, (size_t)n * 8,
                                 2 * m, cudaMemcpyDeviceToDevice, st));
        auto permute = [&](void *dptr, size_t elem) -> int {
            std::vector<unsigned char> a((size_t)m * elem), b((size_t)m * elem);
            unsigned char *base = reinterpret_cast<unsigned char *>(dptr) + (size_t)front * elem;
            HSR_CK(cudaMemcpyAsync(a.data(), base, (size_t)m * elem, cudaMemcpyDeviceToHost, st));
            HSR_CK(cudaStreamSynchronize(st));
            for (int j = 0; j < m; ++j) memcpy(&b[(size_t)j * elem], &a[(size_t)perm[j] * elem], elem);
            HSR_CK(cudaMemcpyAsync(base, b.data(), (size_t)m * elem, cudaMemcpyHostToDevice, st));
            HSR_CK(cudaStreamSynchronize(st));
            return HSR_OK;
        };
        int r;
        if ((r = permute(dwc, 16))) return r;
        if ((r = permute(s.d_scale, 8))) return r;
        if ((r = permute(s.d_pert, 2))) return r;
        if ((r = permute(s.d_status, 2 * sizeof(int)))) return r;
        if ((r = permute(s.d_colnorm, 16))) return r;
        std::vector<int> no(order.begin() + front, order.begin() + front + m);
        for (int q = 0; q < m; ++q) order[front + q] = no[perm[q]];
        return HSR_OK;
    };
    int front = 0, its = 0;
    const int max_its = o.max_restarts < 0 ? n : std::min(o.max_restarts, n);
    while (np > 0) {
        HSR_CK(cudaMemcpyAsync(st_h.data() + 2 * front, s.d_status + 2 * front, (size_t)(S - 2 * front) * sizeof(int),
                               cudaMemcpyDeviceToHost, st));
        HSR_CK(cudaStreamSynchronize(st));
        int all = 1;
        for (int p = front; p < np; ++p)
            if (!st_h[2 * p]) all = 0;
        if (all || its >= max_its) break;
        const int m = np - front;
        std::vector<int> perm;
        perm.reserve(m);
        for (int q = 0; q < m; ++q)
            if (st_h[2 * (front + q)]) perm.push_back(q);
        const int nc = (int)perm.size();
        for (int q = 0; q < m; ++q)
            if (!st_h[2 * (front + q)]) perm.push_back(q);
        if ((rc = apply_perm(front, perm))) return rc;
        permuted = true;
        for (int q = 0; q < nc; ++q) st_h[2 * (front + q)] = st_h[2 * (front + q) + 1] = 1;
        front += nc;
        rc = run_pass_c(s, 1, its, 2 * front, 2 * (np - front));
        if (rc) return rc;
        ++its;
    }
    if (permuted) {
        HSR_CK(cudaMemcpyAsync(st_h.data(), s.d_status, (size_t)S * sizeof(int), cudaMemcpyDeviceToHost, st));
        HSR_CK(cudaStreamSynchronize(st));
        std::vector<int> inv(np);
        for (int q = 0; q < np; ++q) inv[order[q]] = q;
        std::vector<int> st2(S);
        for (int p = 0; p < np; ++p) st2[2 * p] = st2[2 * p + 1] = st_h[2 * inv[p]];
        if ((rc = apply_perm(0, inv))) return rc;
        st_h.swap(st2);
    }
    int nonconv = 0;
    for (int p = 0; p < np; ++p) nonconv += !st_h[2 * p];

    int errw = 0;
    HSR_CK(cudaMemcpyAsync(&errw, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaStreamSynchronize(st));
    g_timing.resolve();
    if (errw) return HSR_ERR_DEVICE;
    if (d_status_pairs)
        HSR_CK(cudaMemcpy2DAsync(d_status_pairs, sizeof(int), s.d_status, 2 * sizeof(int), sizeof(int), np,
                                 cudaMemcpyDeviceToDevice, st));
    if (d_scale_pairs)
        HSR_CK(cudaMemcpyAsync(d_scale_pairs, s.d_scale, (size_t)np * 8, cudaMemcpyDeviceToDevice, st));
    if (h_status) {
        h_status->resize(np);
        for (int p = 0; p < np; ++p) (*h_status)[p] = st_h[2 * p];
    }
    if (h_pert) {
        std::vector<unsigned char> t(S);
        HSR_CK(cudaMemcpy(t.data(), s.d_pert, S, cudaMemcpyDeviceToHost));
        h_pert->resize(np);
        for (int p = 0; p < np; ++p) (*h_pert)[p] = t[2 * p];
    }
    if (h_scale) {
        h_scale->resize(np);
        HSR_CK(cudaMemcpy(h_scale->data(), s.d_scale, (size_t)np * 8, cudaMemcpyDeviceToHost));
    }
    if (h_norm) {
        std::vector<double> t(S);
        HSR_CK(cudaMemcpy(t.data(), s.d_colnorm, (size_t)S * 8, cudaMemcpyDeviceToHost));
        h_norm->resize(np);
        for (int p = 0; p < np; ++p) (*h_norm)[p] = t[2 * p];
    }
    if (d_status_pairs || d_scale_pairs) HSR_CK(cudaStreamSynchronize(st));
    return nonconv ? HSR_ERR_NOT_CONVERGED : HSR_OK;
}

int check_args_c(int n, int ldH, int np, int tlsz, int ldvr, const void *H, const void *wr, const void *wi,
                 const void *vr) {
    if (n <= 0 || ldH < n || np < 0 || tlsz <= 0 || (tlsz % 4) != 0 || ldvr < n || !H) return HSR_ERR_ARG;
    if (np > 0 && (!wr || !wi || !vr)) return HSR_ERR_ARG;
    return HSR_OK;
}

int host_call_c(int n, const double *H, int ldH, int np, const double *wr, const double *wi, int tlsz,
                int rhs_tlsz, double *vr, int ldvr, const hsr_options *opt, hsr_column_info *info) {
    g_launches = 0;
    g_timing.reset();
    int rc = check_args_c(n, ldH, np, tlsz, ldvr, H, wr, wi, vr);
    if (rc) return rc;
    if (rhs_tlsz <= 0) return HSR_ERR_ARG;
    if (opt && opt->user_rhs) return HSR_ERR_ARG;
    if (np == 0) return HSR_OK;
    Workspace &w = ws();
    if (!w.stream) HSR_CK(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
    cudaStream_t st = w.stream;
    const long long ldh = (ldH % 2 == 0) ? ldH : round_up(n, 32);
    const long long ldx = ldvr;
    HSR_CK(w.H.ensure((size_t)ldh * n * 8));
    HSR_CK(w.X.ensure((size_t)ldx * 2 * np * 8));
    HSR_CK(w.wr.ensure((size_t)2 * np * 8));
    std::vector<double> wc(2 * (size_t)np);
    for (int p = 0; p < np; ++p) {
        wc[2 * p] = wr[p];
        wc[2 * p + 1] = wi[p];
    }
    g_timing.begin(kcH2D, st);
    if (const void *Hm = mapped_view(H))
        HSR_CK(copy_cols(w.H.as<double>(), ldh, static_cast<const double *>(Hm), ldH, n, n, st));
    else if (ldh == ldH)
        HSR_CK(cudaMemcpyAsync(w.H.p, H, ((size_t)ldH * (n - 1) + n) * 8, cudaMemcpyHostToDevice, st));
    else
        HSR_CK(cudaMemcpy2DAsync(w.H.p, ldh * 8, H, (size_t)ldH * 8, (size_t)n * 8, n, cudaMemcpyHostToDevice, st));
    HSR_CK(cudaMemcpyAsync(w.wr.p, wc.data(), (size_t)2 * np * 8, cudaMemcpyHostToDevice, st));
    g_timing.end(st);
    std::vector<int> hs;
    std::vector<unsigned char> hp;
    std::vector<double> hsc, hn;
    const bool want = info != nullptr;
    rc = solve_device_cplx(n, w.H.as<double>(), ldh, np, w.wr.as<double>(), tlsz, w.X.as<double>(), ldx, opt, st,
                           nullptr, nullptr, want && info->status ? &hs : nullptr,
                           want && info->perturbed ? &hp : nullptr, want && info->scale ? &hsc : nullptr,
                           want && info->norm ? &hn : nullptr);
    if (rc < 0) return rc;
    g_timing.begin(kcD2H, st);
    if (void *Xm = mapped_view(vr))
        HSR_CK(copy_cols(static_cast<double *>(Xm), ldvr, w.X.as<double>(), ldx, n, 2 * np, st));
    else if (ldvr == n)
        HSR_CK(cudaMemcpyAsync(vr, w.X.p, (size_t)n * 2 * np * 8, cudaMemcpyDeviceToHost, st));
    else
        HSR_CK(cudaMemcpy2DAsync(vr, (size_t)ldvr * 8, w.X.p, ldx * 8, (size_t)n * 8, 2 * np,
                                 cudaMemcpyDeviceToHost, st));
    g_timing.end(st);
    HSR_CK(cudaStreamSynchronize(st));
    g_timing.resolve();
    if (want) {
        if (info->status) memcpy(info->status, hs.data(), (size_t)np * sizeof(int));
        if (info->perturbed) memcpy(info->perturbed, hp.data(), (size_t)np);
        if (info->scale) memcpy(info->scale, hsc.data(), (size_t)np * 8);
        if (info->norm) memcpy(info->norm, hn.data(), (size_t)np * 8);
    }
    return rc;
}

}  // namespace
}  // namespace hsr

using namespace hsr;

extern "C" {

int hsr_last_status(void) { return g_last_status; }

const char *hsr_status_string(int status) {
    switch (status) {
    case HSR_OK: return "ok";
    case HSR_ERR_ARG: return "invalid argument";
    case HSR_ERR_NOMEM: return "out of memory";
    case HSR_ERR_CUDA: return cudaGetErrorString(last_cuda_error());
    case HSR_ERR_DEVICE: return "device kernel reported an internal error";
    case HSR_ERR_NOT_CONVERGED: return "some columns did not converge";
    default: return "unknown status";
    }
}

void tiled_inverse_iteration(int n, const double *H, int ldH, int nrhs, double *wr, int tlsz, int rhs_tlsz,
                             double *vr, int ldvr) {
    g_last_status = host_call(n, H, ldH, nrhs, wr, tlsz, rhs_tlsz, vr, ldvr, nullptr, nullptr);
}

int hsr_inverse_iteration_ex(int n, const double *H, int ldH, int nrhs, double *wr, int tlsz, int rhs_tlsz,
                             double *vr, int ldvr, const hsr_options *opt, hsr_column_info *info) {
    g_last_status = host_call(n, H, ldH, nrhs, wr, tlsz, rhs_tlsz, vr, ldvr, opt, info);
    return g_last_status;
}

int hsr_inverse_iteration_device(int n, const double *dH, int lddH, int nrhs, double *dwr, int tlsz, double *dvr,
                                 int lddvr, const hsr_options *opt, void *stream, int *d_status, double *d_scale) {
    g_launches = 0;
    g_timing.reset();
    if (tlsz == 0 && n > 0) tlsz = plain_tlsz_for(n);
    int rc = check_args(n, lddH, nrhs, tlsz, lddvr, dH, dwr, dvr);
    if (rc) return g_last_status = rc;
    if (nrhs == 0) return g_last_status = HSR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double *Huse = dH;
    long long ldh = lddH;
    if ((lddH & 1) || (reinterpret_cast<uintptr_t>(dH) & 15)) {
        // TMA needs an even pitch and a 16-byte aligned base: use a padded copy.
        Workspace &w = ws();
        ldh = round_up(n, 32);
        cudaError_t e = w.H.ensure((size_t)ldh * n * 8);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(w.H.p, ldh * 8, dH, (size_t)lddH * 8, (size_t)n * 8, n, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            last_cuda_error() = e;
            return g_last_status = HSR_ERR_CUDA;
        }
        Huse = w.H.as<double>();
    }
    rc = solve_device(n, Huse, ldh, nrhs, dwr, tlsz, dvr, lddvr, opt, st, d_scale, d_status, nullptr, nullptr,
                      nullptr, nullptr, nullptr);
    return g_last_status = rc;
}

int hsr_inverse_iteration_cplx_ex(int n, const double *H, int ldH, int npairs, const double *wr, const double *wi,
                                  int tlsz, int rhs_tlsz, double *vr, int ldvr, const hsr_options *opt,
                                  hsr_column_info *info) {
    g_last_status = host_call_c(n, H, ldH, npairs, wr, wi, tlsz, rhs_tlsz, vr, ldvr, opt, info);
    return g_last_status;
}

int hsr_inverse_iteration_cplx_device(int n, const double *dH, int lddH, int npairs, const double *dwr,
                                      const double *dwi, int tlsz, double *dvr, int lddvr, const hsr_options *opt,
                                      void *stream, int *d_status, double *d_scale) {
    g_launches = 0;
    g_timing.reset();
    int rc = check_args_c(n, lddH, npairs, tlsz, lddvr, dH, dwr, dwi, dvr);
    if (rc) return g_last_status = rc;
    if (opt && opt->user_rhs) return g_last_status = HSR_ERR_ARG;
    if (npairs == 0) return g_last_status = HSR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Workspace &w = ws();
    const double *Huse = dH;
    long long ldh = lddH;
    cudaError_t e = cudaSuccess;
    if ((lddH & 1) || (reinterpret_cast<uintptr_t>(dH) & 15)) {
        ldh = round_up(n, 32);
        e = w.H.ensure((size_t)ldh * n * 8);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(w.H.p, ldh * 8, dH, (size_t)lddH * 8, (size_t)n * 8, n, cudaMemcpyDeviceToDevice, st);
        Huse = w.H.as<double>();
    }
    // Interleave the shifts (re, im) into the workspace copy.
    if (e == cudaSuccess) e = w.wr.ensure((size_t)2 * npairs * 8);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(w.wr.p, 16, dwr, 8, 8, npairs, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(w.wr.as<double>() + 1, 16, dwi, 8, 8, npairs, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        return g_last_status = HSR_ERR_CUDA;
    }
    rc = solve_device_cplx(n, Huse, ldh, npairs, w.wr.as<double>(), tlsz, dvr, lddvr, opt, st, d_status, d_scale,
                           nullptr, nullptr, nullptr, nullptr);
    return g_last_status = rc;
}

int hsr_inverse_iteration_mixed(int n, const double *H, int ldH, int m, double *wr, double *wi, int tlsz,
                                int rhs_tlsz, double *vr, int ldvr, const hsr_options *opt, int *status) {
    // Validate the layout: a conjugate pair is two consecutive entries
    // (wr, +wi), (wr, -wi) with wi > 0.
    if (n <= 0 || ldH < n || m < 0 || ldvr < n || !H || (m > 0 && (!wr || !wi || !vr)) || tlsz <= 0 ||
        tlsz % 4 != 0 || rhs_tlsz <= 0 || (opt && opt->user_rhs))
        return g_last_status = HSR_ERR_ARG;
    std::vector<int> real_pos, pair_pos;
    for (int k = 0; k < m;) {
        if (wi[k] == 0.0) {
            real_pos.push_back(k);
            k += 1;
        } else {
            if (!(wi[k] > 0.0) || k + 1 >= m || wr[k + 1] != wr[k] || wi[k + 1] != -wi[k])
                return g_last_status = HSR_ERR_ARG;
            pair_pos.push_back(k);
            k += 2;
        }
    }
    const int nr = (int)real_pos.size(), np = (int)pair_pos.size();
    int rc_r = HSR_OK, rc_c = HSR_OK;
    if (nr > 0) {
        std::vector<double> w(nr), x((size_t)n * nr);
        std::vector<int> st(nr);
        for (int q = 0; q < nr; ++q) w[q] = wr[real_pos[q]];
        hsr_column_info info{};
        info.status = st.data();
        rc_r = host_call(n, H, ldH, nr, w.data(), tlsz, rhs_tlsz, x.data(), n, opt, &info);
        if (rc_r < 0) return g_last_status = rc_r;
        // The real path may reorder its shifts (converged first); they stay
        // in the real positions, each with its own column.
        for (int q = 0; q < nr; ++q) {
            const int k = real_pos[q];
            wr[k] = w[q];
            memcpy(vr + (size_t)k * ldvr, x.data() + (size_t)q * n, (size_t)n * 8);
            if (status) status[k] = st[q];
        }
    }
    if (np > 0) {
        std::vector<double> a(np), b(np), x((size_t)n * 2 * np);
        std::vector<int> st(np);
        for (int q = 0; q < np; ++q) {
            a[q] = wr[pair_pos[q]];
            b[q] = wi[pair_pos[q]];
        }
        hsr_column_info info{};
        info.status = st.data();
        rc_c = host_call_c(n, H, ldH, np, a.data(), b.data(), tlsz, rhs_tlsz, x.data(), n, opt, &info);
        if (rc_c < 0) return g_last_status = rc_c;
        for (int q = 0; q < np; ++q) {
            const int k = pair_pos[q];
            memcpy(vr + (size_t)k * ldvr, x.data() + (size_t)(2 * q) * n, (size_t)n * 8);
            memcpy(vr + (size_t)(k + 1) * ldvr, x.data() + (size_t)(2 * q + 1) * n, (size_t)n * 8);
            if (status) status[k] = status[k + 1] = st[q];
        }
    }
    return g_last_status = (rc_r == HSR_ERR_NOT_CONVERGED || rc_c == HSR_ERR_NOT_CONVERGED) ? HSR_ERR_NOT_CONVERGED
                                                                                              : HSR_OK;
}

long hsr_last_launch_count(void) { return g_launches; }

void hsr_set_kernel_timing(int enable) { g_timing.enabled = enable != 0; }

int hsr_last_kernel_times(double *ms, long *launches, double *gemm_fma) {
    for (int i = 0; i < kcCount; ++i) {
        if (ms) ms[i] = g_timing.ms[i];
        if (launches) launches[i] = g_timing.launches[i];
    }
    if (gemm_fma) *gemm_fma = g_timing.gemm_fma[0];
    return kcCount;
}

void hsr_release_workspace(void) { ws().release(); }

int hsr_selftest_arith(long long per_thread, unsigned long long seed, long long counts[4]) {
    if (per_thread < 0 || !counts) return record_status(HSR_ERR_ARG, cudaSuccess);
    Workspace &w = ws();
    cudaError_t e = w.probe.ensure(64);
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(w.probe.p);
    if (e == cudaSuccess) e = cudaMemset(cnt, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = launch_selftest_arith((unsigned long long)per_thread, seed, cnt, sms * 4, 0);
    unsigned long long h[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return record_status(HSR_ERR_CUDA, e);
    for (int i = 0; i < 4; ++i) counts[i] = (long long)h[i];
    return record_status(HSR_OK, cudaSuccess);
}

int hsr_probe_fp64_peak(double ms_target, double *dfma_gflops, double *dmma_gflops) {
    Workspace &w = ws();
    if (w.probe.ensure(64) != cudaSuccess) return HSR_ERR_CUDA;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 4;
    // Size one launch to ~ms_target/4, warm up, then time four launches
    // back to back (clocks ramped), and report the throughput.
    auto measure = [&](bool dmma, double *out) -> int {
        int iters = 512;
        float ms = 0.f;
        auto launch = [&]() {
            return dmma ? launch_probe_dmma(w.probe.as<double>(), blocks, iters, 0)
                        : launch_probe_dfma(w.probe.as<double>(), blocks, iters, 0);
        };
        for (int rep = 0; rep < 12; ++rep) {
            cudaEventRecord(e0, 0);
            cudaError_t e = launch();
            cudaEventRecord(e1, 0);
            if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return HSR_ERR_CUDA;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms >= 0.25 * ms_target || iters >= (1 << 24)) break;
            iters = (int)std::min<double>((double)iters * 2.0, (double)(1 << 24));
        }
        for (int rep = 0; rep < 2; ++rep)
            if (launch() != cudaSuccess) return HSR_ERR_CUDA;
        cudaEventRecord(e0, 0);
        for (int rep = 0; rep < 4; ++rep)
            if (launch() != cudaSuccess) return HSR_ERR_CUDA;
        cudaEventRecord(e1, 0);
        if (cudaEventSynchronize(e1) != cudaSuccess) return HSR_ERR_CUDA;
        cudaEventElapsedTime(&ms, e0, e1);
        const double warps = (double)blocks * 8;
        const double flops = 4.0 * (dmma ? warps * iters * 4.0 * 2.0 * 256 : warps * 32 * iters * 8.0 * 2.0);
        *out = flops / (ms * 1e-3) / 1e9;
        return HSR_OK;
    };
    int rc = HSR_OK;
    if (dfma_gflops) rc |= measure(false, dfma_gflops);
    if (dmma_gflops) rc |= measure(true, dmma_gflops);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc ? HSR_ERR_CUDA : HSR_OK;
}

int hsr_selftest_bounded_wait(void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Workspace &w = ws();
    HSR_CK(w.err.ensure(16));
    HSR_CK(cudaMemsetAsync(w.err.p, 0, 16, st));
    HSR_CK(launch_wait_selftest(w.err.as<int>(), 1L << 14, st));
    int errw = 0;
    HSR_CK(cudaMemcpyAsync(&errw, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    HSR_CK(cudaStreamSynchronize(st));
    HSR_CK(cudaMemsetAsync(w.err.p, 0, 16, st));
    HSR_CK(cudaStreamSynchronize(st));
    return g_last_status = (errw & kErrWaitTimeout) ? HSR_ERR_DEVICE : HSR_OK;
}

int hsr_autotune_plain(int n, const double *dH, int lddH, int nrhs, double *dwr, double *dvr, int lddvr,
                       const int *cand, int ncand, double *ms_out, int *shifts_per_cta, double *spc_ms,
                       int *top_fused, double *fused_ms, void *stream) {
    if (n <= 0 || nrhs <= 0 || !cand || ncand <= 0 || !dH || !dwr || !dvr) return g_last_status = HSR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *wr0 = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto done = [&](int rc) {
        set_diag_shifts_trial(0);
        set_fused_top_trial(-1);
        if (wr0) cudaFree(wr0);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return g_last_status = rc;
    };
    if (cudaMalloc(&wr0, (size_t)nrhs * 8) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess ||
        cudaMemcpyAsync(wr0, dwr, (size_t)nrhs * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return done(HSR_ERR_CUDA);
    // Mean of two timed solves after one warm-up; 1e300 when the solve fails.
    auto time_one = [&](int tl, double *ms) -> int {
        double tot = 0.0;
        for (int rep = 0; rep < 3; ++rep) {
            if (cudaMemcpyAsync(dwr, wr0, (size_t)nrhs * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
                cudaEventRecord(e0, st) != cudaSuccess)
                return HSR_ERR_CUDA;
            const int rc = hsr_inverse_iteration_device(n, dH, lddH, nrhs, dwr, tl, dvr, lddvr, nullptr, stream,
                                                        nullptr, nullptr);
            if (rc < 0) {
                *ms = 1e300;
                return HSR_OK;
            }
            float t = 0.f;
            if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&t, e0, e1) != cudaSuccess)
                return HSR_ERR_CUDA;
            if (rep > 0) tot += t;      // the first run warms the workspace
        }
        *ms = tot / 2;
        return HSR_OK;
    };
    int best = 0;
    double best_ms = 1e300;
    for (int c = 0; c < ncand; ++c) {
        double ms = 1e300;
        if (cand[c] > 0 && cand[c] % 4 == 0 && time_one(cand[c], &ms) != HSR_OK) return done(HSR_ERR_CUDA);
        if (ms_out) ms_out[c] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = cand[c];
        }
    }
    if (best <= 0) return done(HSR_ERR_ARG);
    // Shifts per diagonal CTA (8, 16, 32) at the chosen tile size.
    int best_sc = 0;
    double best_sc_ms = 1e300;
    const int scs[3] = {8, 16, 32};
    for (int i = 0; i < 3; ++i) {
        set_diag_shifts_trial(scs[i]);
        double ms = 1e300;
        if (time_one(best, &ms) != HSR_OK) return done(HSR_ERR_CUDA);
        if (spc_ms) spc_ms[i] = ms;
        if (ms < best_sc_ms) {
            best_sc_ms = ms;
            best_sc = scs[i];
        }
    }
    // With narrow diagonal CTAs: the top GEMM of each tile's rows inside
    // them or as its own launch ([separate, fused]); -1 where it does not
    // apply (32 shifts per CTA).
    int fused = 0;
    double fms[2] = {-1.0, -1.0};
    if (best_sc && best_sc < 32) {
        set_diag_shifts_trial(best_sc);
        for (int on = 0; on < 2; ++on) {
            set_fused_top_trial(on);
            if (time_one(best, &fms[on]) != HSR_OK) return done(HSR_ERR_CUDA);
        }
        fused = fms[1] <= fms[0] ? 1 : 0;
    }
    set_diag_shifts_trial(0);
    set_fused_top_trial(-1);
    if (cudaMemcpyAsync(dwr, wr0, (size_t)nrhs * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return done(HSR_ERR_CUDA);
    {
        std::lock_guard<std::mutex> g(g_plain_tune_mu);
        g_plain_tune[n] = best;
    }
    if (best_sc) record_diag_shifts(nrhs, best_sc);
    if (best_sc && best_sc < 32) record_fused_top(nrhs, fused != 0);
    if (shifts_per_cta) *shifts_per_cta = best_sc;
    if (top_fused) *top_fused = fused;
    if (fused_ms) {
        fused_ms[0] = fms[0];
        fused_ms[1] = fms[1];
    }
    done(HSR_OK);
    return best;
}

int hsr_autotune_plain_tlsz(int n) { return n > 0 ? plain_tlsz_for(n) : HSR_ERR_ARG; }

const char *hsr_version(void) { return "hsrq3in_gb300 0.1 (sm_103a, FP64 DFMA)"; }

}  // extern "C"

bool hsr::kernel_timing_enabled() { return g_timing.enabled; }

int hsr::record_status(int status, cudaError_t cuda_error) {
    if (cuda_error != cudaSuccess) last_cuda_error() = cuda_error;
    return g_last_status = status;
}
