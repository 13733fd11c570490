// hsr_noalloc.cu -- inverse iteration for callers that cannot allocate device
// memory.
//
// Some callers of this library may not call cudaMalloc once they are running:
// a serving process whose device memory is owned up front by a caching
// allocator or a fixed pool (a cudaMalloc there either fails because the pool
// already holds the memory, or synchronises the device and stalls every other
// stream), or a plug-in host that hands out device buffers but forbids its
// plug-ins from allocating their own.  hsr_inverse_iteration_noalloc serves
// them: the caller passes the inputs and outputs, and every other buffer the
// solve needs is carved out of one file-scope __device__ array of
// kNoallocScratchBytes that each GPU loading the library holds until the
// process exits.  Nothing is allocated on the device or the host heap, no
// stream or event is created, and all work is enqueued on the caller's stream.
//
// The array is shared by every call: calls whose work overlaps on the GPU
// (different streams, different host threads) race on it and must be
// serialised by the caller.  It keeps the previous call's contents; each call
// clears what has to start at zero (the norm accumulators and the error word)
// and writes everything else before reading it.  The first call on a device
// resolves the array's device address (cudaGetSymbolAddress, with that device
// current) and caches it, so that first call should come before any stream
// capture.  Under CUDA's default lazy module loading that first call also
// loads the library's kernels on the device and commits the array's device
// memory -- an allocation made by the driver on the caller's behalf -- so a
// caller whose pool takes the free memory later should make its first call
// before that (or load modules eagerly, CUDA_MODULE_LOADING=EAGER).
//
// The call returns only after the solve has finished: it synchronises the
// stream to read the norm of H, the convergence status of each restart round
// and the error word.  On a failure after work was enqueued it also waits
// for that work before returning, so a following call (on any stream) does
// not race with the failed one.
#include "hsr_common.h"
#include "hsr_kernels.h"
#include "../../include/hsrq3in_gb300.h"

#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace hsr {
namespace {

constexpr size_t kNoallocScratchBytes = (size_t)HSR_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::atomic<unsigned char *> g_scratch_ptr[kMaxDevices];

// Device address of the scratch array on the current device (set-up once).
cudaError_t scratch_base(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    unsigned char *p = g_scratch_ptr[dev].load();
    if (!p) {
        e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev].store(p);
    }
    *out = p;
    return cudaSuccess;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool encode_map(CUtensorMap *m, const double *base, unsigned long long inner, unsigned long long outer,
                unsigned long long ld, unsigned bx, unsigned by) {
    // Looked up once; a function-local static's initialiser runs exactly once
    // even when several host threads make their first call together.
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {ld * sizeof(double)};
    cuuint32_t box[2] = {bx, by};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline size_t up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carve {
    unsigned char *base;
    size_t off = 0;
    template <class T> T *take(size_t count) {
        off = up(off, 256);
        T *p = reinterpret_cast<T *>(base + off);
        off += count * sizeof(T);
        return p;
    }
};

// The CUDA error behind the last HSR_ERR_CUDA of this thread's call.
thread_local cudaError_t t_na_error = cudaSuccess;

#define NA_CK(x)                                 \
    do {                                         \
        const cudaError_t e_ = (x);              \
        if (e_ != cudaSuccess) {                 \
            t_na_error = e_;                     \
            return HSR_ERR_CUDA;                 \
        }                                        \
    } while (0)

struct NoallocSolve {
    int n, T, tlsz, S, Spad, is;
    int fr[HSR_NOALLOC_MAX_N / 4 + 2];
    const double *H;
    long long ldh;
    double *X;
    long long ldx;
    double *wr;
    cudaStream_t st;
    CUtensorMap tmH, tmW, tmZ;
    DevProblem base;    // pointers into the scratch array
    double *eps3_dev, *colnorm, *scale;
    int *status;
    double *tmpX;
    int *perm;
};

// One pass over columns [off, off+cnt): the tile sweep, finalize, normalize,
// sequentially on the caller's stream.
int noalloc_pass(NoallocSolve &s, int mode, int its, int off, int cnt) {
    DevProblem P = s.base;
    P.S = cnt;
    P.wr = s.wr + off;
    P.X = s.X + (size_t)off * s.ldx;
    P.pert = s.base.pert + off;
    NA_CK(launch_init(P, mode, s.eps3_dev, its, s.st));
    for (int J = s.T - 1; J >= 0; --J) {
        NA_CK(launch_diag(P, J, s.fr[J + 1] - s.fr[J], nullptr, s.st));
        if (J == 0) break;
        NA_CK(launch_part1(P, J, s.st));
        NA_CK(launch_gemm(P, J, 0, s.fr[J], s.tmH, s.tmW, s.tmZ, s.st));
    }
    NA_CK(launch_finalize(P, s.colnorm + off, s.status + off, s.scale + off, s.st));
    NA_CK(launch_normalize(P, s.colnorm + off, s.status + off, s.st));
    return HSR_OK;
}

}  // namespace
}  // namespace hsr

using namespace hsr;

namespace {

int noalloc_solve(int n, const double *dH, int lddH, int nrhs, double *dwr, int tlsz, double *dvr, int lddvr,
                  int scaling, cudaStream_t st_caller, int *status, bool *enqueued) {
    if (n <= 0 || lddH < n || nrhs < 0 || tlsz <= 0 || (tlsz % 4) != 0 || lddvr < n || !dH) return HSR_ERR_ARG;
    if (nrhs > 0 && (!dwr || !dvr)) return HSR_ERR_ARG;
    if (n > HSR_NOALLOC_MAX_N || nrhs > HSR_NOALLOC_MAX_NRHS) return HSR_ERR_ARG;
    if (nrhs == 0) return HSR_OK;
    unsigned char *base = nullptr;
    NA_CK(scratch_base(&base));

    NoallocSolve s;
    s.n = n;
    s.tlsz = tlsz;
    s.T = (n + tlsz - 1) / tlsz;
    s.S = nrhs;
    s.Spad = (int)up((size_t)nrhs, 64);
    s.is = scaling == HSR_SCALING_DOUBLE ? 0 : 1;
    s.st = st_caller;
    s.X = dvr;
    s.ldx = lddvr;
    s.wr = dwr;
    const int T = s.T;
    for (int i = 1; i < T; ++i) s.fr[i] = n - (T - i) * tlsz;   // partition.c:7-17
    s.fr[0] = 0;
    s.fr[T] = n;
    int bmax = 0;
    for (int I = 0; I < T; ++I) bmax = s.fr[I + 1] - s.fr[I] > bmax ? s.fr[I + 1] - s.fr[I] : bmax;
    if (diag_smem_bytes(bmax) < (size_t)64 * bmax * sizeof(double)) return HSR_ERR_ARG;

    // Carve every workspace out of the scratch array; reject what does not fit.
    const size_t Sp = (size_t)s.Spad;
    const size_t ldr = up((size_t)n, 4);
    const size_t wrows = T > 1 ? (size_t)tlsz : 1;
    const size_t zrows = (size_t)(T - 1) * tlsz + bmax;
    const bool copyH = (lddH & 1) || (reinterpret_cast<uintptr_t>(dH) & 15);
    const long long ldh_pad = (long long)up((size_t)n, 32);
    Carve cv{base};
    int *d_fr = cv.take<int>(T + 1);
    unsigned long long *bits = cv.take<unsigned long long>(2 * (size_t)T * T + 2);
    int *err = cv.take<int>(4);
    DevProblem &P = s.base;
    P = DevProblem{};
    P.n = n;
    P.T = T;
    P.Spad = s.Spad;
    P.tlsz = tlsz;
    P.fr = d_fr;
    P.R = cv.take<double>(ldr * Sp);
    P.ldr = (long long)ldr;
    P.Cr = cv.take<double>((size_t)n * Sp);
    P.Sr = cv.take<double>((size_t)n * Sp);
    P.beta = cv.take<double>((size_t)T * Sp);
    P.ynorm = cv.take<double>((size_t)T * Sp);
    P.Hn = reinterpret_cast<const double *>(bits);
    P.hn = reinterpret_cast<const double *>(bits + (size_t)T * T);
    P.W = cv.take<double>(wrows * Sp);
    P.Zs = cv.take<double>(wrows * Sp);
    double *v = cv.take<double>(4 * Sp);
    P.pi = v;
    P.ytil = v + Sp;
    P.z2n = v + 2 * Sp;
    P.zlast = v + 3 * Sp;
    P.Zslow = cv.take<double>(zrows * Sp);
    P.slow = cv.take<unsigned char>((size_t)T * Sp);
    P.pert = cv.take<unsigned char>(Sp);
    P.is = s.is;
    P.err = err;
    P.ldx = lddvr;
    s.colnorm = cv.take<double>(Sp);
    s.scale = cv.take<double>(Sp);
    s.status = cv.take<int>(Sp);
    s.tmpX = cv.take<double>((size_t)n * nrhs);
    s.perm = cv.take<int>(Sp);
    double *Hpad = copyH ? cv.take<double>((size_t)ldh_pad * n) : nullptr;
    if (cv.off > kNoallocScratchBytes) return HSR_ERR_ARG;
    {
        const double eps = DBL_EPSILON / 2;
        P.smlnum = std::fmax(2 * DBL_MIN, DBL_MIN * ((double)n / eps));
    }
    cudaStream_t st = s.st;
    *enqueued = true;

    if (copyH) {
        NA_CK(cudaMemcpy2DAsync(Hpad, (size_t)ldh_pad * 8, dH, (size_t)lddH * 8, (size_t)n * 8, n,
                                cudaMemcpyDeviceToDevice, st));
        s.H = Hpad;
        s.ldh = ldh_pad;
    } else {
        s.H = dH;
        s.ldh = lddH;
    }
    P.H = s.H;
    P.ldh = s.ldh;
    if (!encode_map(&s.tmH, s.H, (unsigned long long)n, (unsigned long long)n, (unsigned long long)s.ldh,
                    kGemmBM, kGemmKC) ||
        !encode_map(&s.tmW, P.W, Sp, wrows, Sp, kGemmBN, kGemmKC) ||
        !encode_map(&s.tmZ, P.Zs, Sp, wrows, Sp, kGemmBN, kGemmKC))
        return HSR_ERR_CUDA;

    // What must start at zero: norm accumulators, error word; W/Zs for a
    // deterministic padding region.
    NA_CK(cudaMemsetAsync(bits, 0, (2 * (size_t)T * T + 2) * 8, st));
    NA_CK(cudaMemsetAsync(err, 0, 4 * sizeof(int), st));
    NA_CK(cudaMemsetAsync(P.W, 0, wrows * Sp * 8, st));
    NA_CK(cudaMemsetAsync(P.Zs, 0, wrows * Sp * 8, st));
    NA_CK(cudaMemcpyAsync(d_fr, s.fr, (T + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    {
        DevProblem P0 = P;
        P0.S = nrhs;
        NA_CK(launch_norms(P0, bits, bits + (size_t)T * T, bits + 2 * (size_t)T * T, err + 1, st));
    }
    double hinf = 0.0;
    int flags[2] = {0, 0};
    NA_CK(cudaMemcpyAsync(&hinf, bits + 2 * (size_t)T * T, 8, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(flags, err, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (flags[1] & 1) hinf = NAN;
    const double eps3 = hinf * (DBL_EPSILON / 2);
    s.eps3_dev = reinterpret_cast<double *>(bits + 2 * (size_t)T * T + 1);
    NA_CK(cudaMemcpyAsync(s.eps3_dev, &eps3, 8, cudaMemcpyHostToDevice, st));

    int rc = noalloc_pass(s, 0, 0, 0, nrhs);
    if (rc) return rc;

    // Restarts with the same semantics as the allocating entry points:
    // converged columns move to the front (stable), the rest get the
    // dlaein-style start vector of round `its`.
    int st_h[HSR_NOALLOC_MAX_NRHS];
    int perm_h[HSR_NOALLOC_MAX_NRHS];
    unsigned char tmp_a[HSR_NOALLOC_MAX_NRHS * 8], tmp_b[HSR_NOALLOC_MAX_NRHS * 8];
    int front = 0, its = 0;
    while (true) {
        NA_CK(cudaMemcpyAsync(st_h + front, s.status + front, (nrhs - front) * sizeof(int), cudaMemcpyDeviceToHost,
                              st));
        NA_CK(cudaStreamSynchronize(st));
        bool all = true;
        for (int k = front; k < nrhs; ++k)
            if (!st_h[k]) all = false;
        if (all || its >= n) break;
        const int m = nrhs - front;
        int q = 0;
        for (int k = 0; k < m; ++k)
            if (st_h[front + k]) perm_h[q++] = k;
        const int nc = q;
        for (int k = 0; k < m; ++k)
            if (!st_h[front + k]) perm_h[q++] = k;
        NA_CK(cudaMemcpyAsync(s.perm, perm_h, m * sizeof(int), cudaMemcpyHostToDevice, st));
        NA_CK(launch_gather_cols(s.tmpX, n, dvr + (size_t)front * lddvr, lddvr, n, s.perm, m, st));
        NA_CK(cudaMemcpy2DAsync(dvr + (size_t)front * lddvr, (size_t)lddvr * 8, s.tmpX, (size_t)n * 8,
                                (size_t)n * 8, m, cudaMemcpyDeviceToDevice, st));
        auto permute = [&](void *dptr, size_t elem) -> int {
            unsigned char *d = static_cast<unsigned char *>(dptr) + (size_t)front * elem;
            NA_CK(cudaMemcpyAsync(tmp_a, d, (size_t)m * elem, cudaMemcpyDeviceToHost, st));
            NA_CK(cudaStreamSynchronize(st));
            for (int j = 0; j < m; ++j) memcpy(tmp_b + (size_t)j * elem, tmp_a + (size_t)perm_h[j] * elem, elem);
            NA_CK(cudaMemcpyAsync(d, tmp_b, (size_t)m * elem, cudaMemcpyHostToDevice, st));
            NA_CK(cudaStreamSynchronize(st));
            return HSR_OK;
        };
        if ((rc = permute(dwr, 8))) return rc;
        if ((rc = permute(s.scale, 8))) return rc;
        if ((rc = permute(P.pert, 1))) return rc;
        if ((rc = permute(s.status, sizeof(int)))) return rc;
        if ((rc = permute(s.colnorm, 8))) return rc;
        for (int j = 0; j < nc; ++j) st_h[front + j] = 1;
        front += nc;
        if ((rc = noalloc_pass(s, 1, its, front, nrhs - front))) return rc;
        ++its;
    }
    int errw = 0;
    NA_CK(cudaMemcpyAsync(&errw, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (errw) return HSR_ERR_DEVICE;
    int nonconv = 0;
    for (int k = 0; k < nrhs; ++k) {
        if (status) status[k] = st_h[k];
        nonconv += !st_h[k];
    }
    return nonconv ? HSR_ERR_NOT_CONVERGED : HSR_OK;
}

}  // namespace

extern "C" int hsr_inverse_iteration_noalloc(int n, const double *dH, int lddH, int nrhs, double *dwr, int tlsz,
                                             double *dvr, int lddvr, int scaling, void *stream, int *status) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    bool enqueued = false;
    t_na_error = cudaSuccess;
    const int rc = noalloc_solve(n, dH, lddH, nrhs, dwr, tlsz, dvr, lddvr, scaling, st, status, &enqueued);
    // After a failure, wait for whatever this call already enqueued: it
    // writes the shared scratch array and dvr, and the caller's next call
    // must not overlap with it.  Its own result does not change the status.
    if (rc < 0 && enqueued) (void)cudaStreamSynchronize(st);
    return record_status(rc, rc == HSR_ERR_CUDA ? t_na_error : cudaSuccess);
}
