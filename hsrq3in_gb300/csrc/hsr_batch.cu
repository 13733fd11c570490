// hsr_batch.cu -- batched and served solves: many problems, one tick at a time.
//
// A problem with T row tiles needs T stages (J = T-1 .. 0).  Problems start
// at their own tick and each tick advances every active problem by one stage,
// with the single-problem look-ahead: part 1 of stage J, then on a
// high-priority side stream the GEMM rows of tile J-1 followed by the
// diagonal solve of tile J-1, while the GEMM rows above tile J-1 run on the
// main stream.  One batched launch per
// phase covers the work items of all problems, so thousands of small
// problems fill the GPU together.  Each work item runs the single-problem
// kernel body, so every column computes exactly what it computes when its
// problem is solved alone with the same tile size.
//
//   batched (hsr_batch_plan_*): all problems start at tick 0; the whole tick
//     sequence, with its work lists already on the device, is captured once
//     into a CUDA graph and replayed by each execute.
//   served (hsr_server_*): a request loop admits requests in arrival order
//     while their footprint fits a device pool (HBM budget), copies them in,
//     runs ticks over the admitted set, and copies finished results out;
//     requests arriving while others run join at the next tick.
#include "hsr_common.h"
#include "hsr_kernels.h"
#include "../../include/hsrq3in_gb300.h"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace hsr {
namespace {

inline size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ------------------------------------------------------------- layout
// Device workspace of one problem.  Offsets are relative to the problem's
// base; every piece starts on a 256-byte boundary.  The pieces that must
// start at zero (norm accumulators, NaN flags) come first so that one memset
// clears them.
struct Layout {
    int n = 0, S = 0, T = 0, b = 0, Spad = 0;
    long long ldr = 0;
    size_t zero_bytes = 0;   // [0, zero_bytes) must be zeroed before setup
    size_t nbits, nan, fr, R, Cr, Sr, beta, ynorm, W, Zs, vecs, Zslow, slow, pert, colnorm, status, scale;
    size_t total = 0;
    void compute(int n_, int S_, int b_) {
        n = n_;
        S = S_;
        b = b_;
        T = (n + b - 1) / b;
        Spad = (int)up((size_t)S, 8);
        ldr = (long long)up((size_t)n, 4);
        size_t o = 0;
        auto take = [&](size_t bytes) {
            o = up(o, 256);
            const size_t at = o;
            o += bytes;
            return at;
        };
        const size_t Sp = (size_t)Spad;
        nbits = take((2 * (size_t)T * T + 2) * 8);
        nan = take(4 * sizeof(int));
        zero_bytes = up(o, 256);
        fr = take((size_t)(T + 1) * sizeof(int));
        R = take((size_t)ldr * S * 8);
        Cr = take((size_t)n * Sp * 8);
        Sr = take((size_t)n * Sp * 8);
        beta = take((size_t)T * Sp * 8);
        ynorm = take((size_t)T * Sp * 8);
        // Stage operands, two copies (even and odd tiles): the diagonal solve
        // of tile J-1 writes one while the GEMM of stage J reads the other.
        W = take(2 * (size_t)b * Sp * 8);
        Zs = take(2 * (size_t)b * Sp * 8);
        vecs = take(2 * 4 * Sp * 8);
        Zslow = take((size_t)T * b * Sp * 8);
        slow = take((size_t)T * Sp);
        pert = take(Sp);
        colnorm = take(Sp * 8);
        status = take(Sp * sizeof(int));
        scale = take(Sp * 8);
        total = up(o, 256);
    }
};

void partition_rows(int n, int T, int b, std::vector<int> &fr) {
    fr.assign(T + 1, 0);
    for (int i = 1; i < T; ++i) fr[i] = n - (T - i) * b;   // partition.c:7-17
    fr[0] = 0;
    fr[T] = n;
}

double smlnum_for(int n) {
    const double eps = DBL_EPSILON / 2;
    return std::fmax(2 * DBL_MIN, DBL_MIN * ((double)n / eps));
}

// DevProblem of one problem whose workspace starts at `base`, with the stage
// operands of tiles of the given parity.
DevProblem make_problem(const Layout &L, char *base, const double *H, long long ldh, double *wr, double *X,
                        long long ldx, int is, int *err, int parity) {
    const size_t stage = (size_t)L.b * L.Spad;
    DevProblem P{};
    P.n = L.n;
    P.T = L.T;
    P.S = L.S;
    P.Spad = L.Spad;
    P.tlsz = L.b;
    P.fr = reinterpret_cast<const int *>(base + L.fr);
    P.H = H;
    P.ldh = ldh;
    P.wr = wr;
    P.X = X;
    P.ldx = ldx;
    P.R = reinterpret_cast<double *>(base + L.R);
    P.ldr = L.ldr;
    P.Cr = reinterpret_cast<double *>(base + L.Cr);
    P.Sr = reinterpret_cast<double *>(base + L.Sr);
    P.beta = reinterpret_cast<double *>(base + L.beta);
    P.ynorm = reinterpret_cast<double *>(base + L.ynorm);
    P.nbits = reinterpret_cast<unsigned long long *>(base + L.nbits);
    P.Hn = reinterpret_cast<const double *>(P.nbits);
    P.hn = reinterpret_cast<const double *>(P.nbits + (size_t)L.T * L.T);
    P.W = reinterpret_cast<double *>(base + L.W) + parity * stage;
    P.Zs = reinterpret_cast<double *>(base + L.Zs) + parity * stage;
    double *v = reinterpret_cast<double *>(base + L.vecs) + parity * 4 * (size_t)L.Spad;
    P.pi = v;
    P.ytil = v + L.Spad;
    P.z2n = v + 2 * (size_t)L.Spad;
    P.zlast = v + 3 * (size_t)L.Spad;
    P.Zslow = reinterpret_cast<double *>(base + L.Zslow);
    P.slow = reinterpret_cast<unsigned char *>(base + L.slow);
    P.pert = reinterpret_cast<unsigned char *>(base + L.pert);
    P.smlnum = smlnum_for(L.n);
    P.is = is;
    P.err = err;
    P.colnorm = reinterpret_cast<double *>(base + L.colnorm);
    P.status = reinterpret_cast<int *>(base + L.status);
    P.scale = reinterpret_cast<double *>(base + L.scale);
    P.nanflag = reinterpret_cast<int *>(base + L.nan);
    return P;
}

bool make_maps(CUtensorMap *m, const Layout &L, const double *H, long long ldh, char *base, int parity) {
    const size_t stage = (size_t)L.b * L.Spad;
    return encode_tensor_map(&m[0], H, (unsigned long long)L.n, (unsigned long long)L.n,
                             (unsigned long long)ldh, kGemmBM, kGemmKC) &&
           encode_tensor_map(&m[1], reinterpret_cast<const double *>(base + L.W) + parity * stage,
                             (unsigned long long)L.Spad, (unsigned long long)L.b, (unsigned long long)L.Spad,
                             kGemmBN, kGemmKC) &&
           encode_tensor_map(&m[2], reinterpret_cast<const double *>(base + L.Zs) + parity * stage,
                             (unsigned long long)L.Spad,
                             (unsigned long long)L.b, (unsigned long long)L.Spad, kGemmBN, kGemmKC);
}

// ----------------------------------------------------------- work lists
// Phases of a tick in launch order.  phGemmTop and then phDiagNext run on the
// side stream, concurrently with phGemmRest.
enum Phase {
    phNorms = 0, phInit, phDiagFirst, phPart1, phGemmTop, phDiagNext, phGemmRest, phFinal, phNormalize, phCount
};

// Descriptor of a problem slot for the stage operands of tiles of parity J.
inline int desc(int slot, int J) { return 2 * slot + (J & 1); }

struct TickLists {
    std::vector<BatchItem> v[phCount];
    void clear() {
        for (auto &x : v) x.clear();
    }
    size_t size() const {
        size_t s = 0;
        for (auto &x : v) s += x.size();
        return s;
    }
};

// Setup of a new problem: norms, start vectors, diagonal solve of tile T-1.
void add_setup(TickLists &tl, int slot, const Layout &L) {
    const int rb = (L.n + kNormRows - 1) / kNormRows;
    for (int r = 0; r < rb; ++r) tl.v[phNorms].push_back(make_int4(desc(slot, 0), 0, r, 0));
    for (int k = 0; k < L.S; ++k) tl.v[phInit].push_back(make_int4(desc(slot, 0), 0, k, 0));
    const int J = L.T - 1, sb32 = (L.S + 31) / 32;
    for (int x = 0; x < sb32; ++x) tl.v[phDiagFirst].push_back(make_int4(desc(slot, J), J, x, 0));
}

// One tick of a problem whose diagonal tile J is solved: part 1 and the GEMM
// of stage J, the diagonal solve of tile J-1, and at the end finalize and
// normalize.  Returns true when the problem finishes in this tick.
bool add_stage(TickLists &tl, int slot, const Layout &L, const std::vector<int> &fr, int J) {
    const int sb32 = (L.S + 31) / 32;
    if (J >= 1) {
        const int p = desc(slot, J), pn = desc(slot, J - 1);
        const int sbp = (L.S + kPart1Shifts - 1) / kPart1Shifts;
        for (int x = 0; x < sbp; ++x) tl.v[phPart1].push_back(make_int4(p, J, x, 0));
        const int cbs = (L.S + kGemmBN - 1) / kGemmBN;
        const int top = (fr[J] - (fr[J - 1] & ~7) + kGemmBM - 1) / kGemmBM;
        for (int r = 0; r < top; ++r)
            for (int c = 0; c < cbs; ++c) tl.v[phGemmTop].push_back(make_int4(p, J, r | kGemmTopFlag, c));
        for (int x = 0; x < sb32; ++x) tl.v[phDiagNext].push_back(make_int4(pn, J - 1, x, 0));
        const int rest = (fr[J - 1] + kGemmBM - 1) / kGemmBM;
        for (int r = 0; r < rest; ++r)
            for (int c = 0; c < cbs; ++c) tl.v[phGemmRest].push_back(make_int4(p, J, r, c));
    }
    if (J > 1) return false;
    for (int x = 0; x < sb32; ++x) tl.v[phFinal].push_back(make_int4(desc(slot, 0), 0, x, 0));
    const int cb = (L.S + kNormalizeCols - 1) / kNormalizeCols;
    for (int x = 0; x < cb; ++x) tl.v[phNormalize].push_back(make_int4(desc(slot, 0), 0, x, 0));
    return true;
}

cudaError_t launch_phase(int ph, const DevProblem *probs, const BatchItem *items, int count, int bmax,
                         const CUtensorMap *maps, cudaStream_t st) {
    switch (ph) {
    case phNorms: return launch_norms_b(probs, items, count, st);
    case phInit: return launch_init_b(probs, items, count, st);
    case phDiagFirst:
    case phDiagNext: return launch_diag_b(probs, items, count, bmax, st);
    case phPart1: return launch_part1_b(probs, items, count, st);
    case phGemmTop:
    case phGemmRest: return launch_gemm_b(probs, items, count, maps, st);
    case phFinal: return launch_finalize_b(probs, items, count, st);
    case phNormalize: return launch_normalize_b(probs, items, count, st);
    }
    return cudaErrorInvalidValue;
}

// Items of one tick, by phase: [off, off + cnt) of the item array.
struct PhaseSpan {
    size_t off = 0;
    int cnt = 0;
};

// Copies a tick's lists into `dst` (phase order) and records their spans.
void pack_tick(const TickLists &tl, BatchItem *dst, size_t base, PhaseSpan *sp) {
    size_t off = 0;
    for (int ph = 0; ph < phCount; ++ph) {
        sp[ph].off = base + off;
        sp[ph].cnt = (int)tl.v[ph].size();
        if (!tl.v[ph].empty()) memcpy(dst + off, tl.v[ph].data(), sizeof(BatchItem) * tl.v[ph].size());
        off += tl.v[ph].size();
    }
}

// Optional device timing of the phases: an event pair around every launch.
struct PhaseTimer {
    std::vector<cudaEvent_t> ev;
    std::vector<std::pair<int, size_t>> starts;   // (phase, index of its start event)
    size_t record(cudaStream_t st) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        ev.push_back(e);
        return ev.size() - 1;
    }
    void add_to(double *ms) const {
        for (auto &x : starts) {
            float t = 0.f;
            if (x.second + 1 < ev.size() && cudaEventElapsedTime(&t, ev[x.second], ev[x.second + 1]) == cudaSuccess)
                ms[x.first] += t;
        }
    }
    ~PhaseTimer() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
};

// Launches one tick: main stream M, side stream D joined back into M.
cudaError_t launch_tick(const PhaseSpan *sp, const DevProblem *probs, const BatchItem *items, int bmax,
                        const CUtensorMap *maps, cudaStream_t M, cudaStream_t D, cudaEvent_t fork,
                        cudaEvent_t join, long &launches, PhaseTimer *tm) {
    auto run = [&](int ph, cudaStream_t st) -> cudaError_t {
        if (sp[ph].cnt == 0) return cudaSuccess;
        if (tm) tm->starts.push_back({ph, tm->record(st)});
        const cudaError_t e = launch_phase(ph, probs, items + sp[ph].off, sp[ph].cnt, bmax, maps, st);
        if (tm) tm->record(st);
        ++launches;
        return e;
    };
    cudaError_t e = cudaSuccess;
    for (int ph : {phNorms, phInit, phDiagFirst, phPart1})
        if ((e = run(ph, M)) != cudaSuccess) return e;
    const bool side = sp[phGemmTop].cnt > 0 || sp[phDiagNext].cnt > 0;
    if (side) {
        if ((e = cudaEventRecord(fork, M)) != cudaSuccess || (e = cudaStreamWaitEvent(D, fork, 0)) != cudaSuccess ||
            (e = run(phGemmTop, D)) != cudaSuccess || (e = run(phDiagNext, D)) != cudaSuccess ||
            (e = cudaEventRecord(join, D)) != cudaSuccess)
            return e;
    }
    if ((e = run(phGemmRest, M)) != cudaSuccess) return e;
    if (side && (e = cudaStreamWaitEvent(M, join, 0)) != cudaSuccess) return e;
    for (int ph : {phFinal, phNormalize})
        if ((e = run(ph, M)) != cudaSuccess) return e;
    return cudaSuccess;
}

int validate(const hsr_batch_problem &p, int b) {
    if (p.n <= 0 || p.lddH < p.n || p.nrhs < 0 || p.lddvr < p.n || !p.dH) return HSR_ERR_ARG;
    if (p.nrhs > 0 && (!p.dwr || !p.dvr)) return HSR_ERR_ARG;
    if ((p.lddH & 1) || (reinterpret_cast<uintptr_t>(p.dH) & 15)) return HSR_ERR_ARG;   // TMA source
    if (b <= 0 || (b % 4) != 0 || b > 384) return HSR_ERR_ARG;
    return HSR_OK;
}

// --------------------------------------------------------- autotune table
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tune;   // [n_lo, n_hi] -> tlsz

int default_tlsz(int n_hi) { return n_hi <= 256 ? 32 : 64; }

}  // namespace
}  // namespace hsr

using namespace hsr;

// ====================================================================== plan
struct hsr_batch_plan {
    int nprob = 0, b = 0, is = 1, ticks = 0;
    long launches = 0;
    std::vector<hsr_batch_problem> specs;
    std::vector<Layout> layouts;
    std::vector<size_t> offsets;
    char *pool = nullptr;
    size_t pool_bytes = 0, zero_bytes = 0;   // problem zero regions are laid out first
    DevProblem *d_probs = nullptr;
    CUtensorMap *d_maps = nullptr;
    BatchItem *d_items = nullptr;
    int *d_err = nullptr;
    int *d_status = nullptr;                  // statuses of all problems, contiguous
    std::vector<size_t> status_off;           // first column of each problem in d_status
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // Persistent-queue engine (built on first use).
    int engine = HSR_BATCH_ENGINE_TICKS;
    std::vector<std::vector<int>> frs;
    QueueItem *d_qitems = nullptr;
    int n_qitems = 0;
    int *d_ctr = nullptr;      // counters, then the ticket
    size_t n_ctr = 0;
    int qgrid = 0, qdiag_warps = 0;
    bool qdirect = false;      // the cooperative launch could not be captured
    cudaGraph_t qgraph = nullptr;
    cudaGraphExec_t qexec = nullptr;
    ~hsr_batch_plan() {
        if (qexec) cudaGraphExecDestroy(qexec);
        if (qgraph) cudaGraphDestroy(qgraph);
        if (d_qitems) cudaFree(d_qitems);
        if (d_ctr) cudaFree(d_ctr);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (pool) cudaFree(pool);
        if (d_probs) cudaFree(d_probs);
        if (d_maps) cudaFree(d_maps);
        if (d_items) cudaFree(d_items);
        if (d_err) cudaFree(d_err);
        if (d_status) cudaFree(d_status);
    }
};

namespace {
#define BP_CK(x)                            \
    do {                                    \
        if ((x) != cudaSuccess) {           \
            delete pl;                      \
            return HSR_ERR_CUDA;            \
        }                                   \
    } while (0)
}  // namespace

// The tuned entry whose order range overlaps [n_lo, n_hi] the most (a
// sample rarely spans the extremes of the batch it was drawn from); the
// default when none overlaps.
extern "C" int hsr_autotune_tlsz(int n_lo, int n_hi) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    long best_overlap = 0;
    int best = 0;
    for (auto &kv : g_tune) {
        const long ov = (long)std::min(n_hi, kv.first.second) - std::max(n_lo, kv.first.first) + 1;
        if (ov > best_overlap) {
            best_overlap = ov;
            best = kv.second;
        }
    }
    return best > 0 ? best : default_tlsz(n_hi);
}

extern "C" int hsr_batch_plan_create(hsr_batch_plan **out, int nprob, const hsr_batch_problem *probs, int tlsz,
                                     const hsr_options *opt, void *stream) {
    if (!out || nprob < 0 || (nprob > 0 && !probs)) return HSR_ERR_ARG;
    *out = nullptr;
    int n_lo = 1 << 30, n_hi = 0;
    for (int i = 0; i < nprob; ++i) {
        n_lo = std::min(n_lo, probs[i].n);
        n_hi = std::max(n_hi, probs[i].n);
    }
    const int b = tlsz > 0 ? tlsz : hsr_autotune_tlsz(n_lo, n_hi);
    for (int i = 0; i < nprob; ++i) {
        const int rc = validate(probs[i], b);
        if (rc) return rc;
    }
    hsr_batch_plan *pl = new hsr_batch_plan();
    pl->nprob = nprob;
    pl->b = b;
    pl->is = (opt && opt->scaling == HSR_SCALING_DOUBLE) ? 0 : 1;
    pl->specs.assign(probs, probs + nprob);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Layout: every problem's zero region first, then the workspaces.
    pl->layouts.resize(nprob);
    pl->offsets.resize(nprob);
    size_t zero_total = 0, ws_total = 0;
    std::vector<size_t> zoff(nprob);
    for (int i = 0; i < nprob; ++i) {
        Layout &L = pl->layouts[i];
        L.compute(probs[i].n, probs[i].nrhs, b);
        zoff[i] = zero_total;
        zero_total += L.zero_bytes;
        ws_total += L.total - L.zero_bytes;
    }
    pl->zero_bytes = zero_total;
    pl->pool_bytes = zero_total + ws_total + 256;
    BP_CK(cudaMalloc(&pl->pool, pl->pool_bytes));
    BP_CK(cudaMalloc(&pl->d_err, 16));
    size_t ncols = 0;
    for (int i = 0; i < nprob; ++i) ncols += (size_t)probs[i].nrhs;
    BP_CK(cudaMalloc(&pl->d_status, sizeof(int) * std::max<size_t>(ncols, 1)));
    ncols = 0;
    // Each problem gets a contiguous Layout whose zero region is elsewhere:
    // carve a virtual base so that base + L.nbits lands in the zero area and
    // base + L.fr ... in the workspace area.  Easiest: give every problem its
    // own full Layout in the workspace area and point nbits/nan at the zero
    // area explicitly.
    std::vector<DevProblem> hp(2 * (size_t)nprob);   // two descriptors per problem (tile parity)
    std::vector<CUtensorMap> hm(6 * (size_t)nprob);
    size_t ws = zero_total;
    std::vector<std::vector<int>> frs(nprob);
    for (int i = 0; i < nprob; ++i) {
        Layout &L = pl->layouts[i];
        char *base = pl->pool + ws - L.zero_bytes;   // workspace pieces start at L.zero_bytes
        pl->offsets[i] = ws - L.zero_bytes;
        ws += L.total - L.zero_bytes;
        char *zbase = pl->pool + zoff[i];
        for (int par = 0; par < 2; ++par) {
            DevProblem P = make_problem(L, base, probs[i].dH, probs[i].lddH, probs[i].dwr, probs[i].dvr,
                                        probs[i].lddvr, pl->is, pl->d_err, par);
            P.nbits = reinterpret_cast<unsigned long long *>(zbase + L.nbits);
            P.Hn = reinterpret_cast<const double *>(P.nbits);
            P.hn = reinterpret_cast<const double *>(P.nbits + (size_t)L.T * L.T);
            P.nanflag = reinterpret_cast<int *>(zbase + L.nan);
            P.status = pl->d_status + ncols;
            hp[desc(i, par)] = P;
            if (!make_maps(&hm[3 * (size_t)desc(i, par)], L, probs[i].dH, probs[i].lddH, base, par)) {
                delete pl;
                return HSR_ERR_CUDA;
            }
        }
        partition_rows(L.n, L.T, b, frs[i]);
        pl->frs.push_back(frs[i]);
        BP_CK(cudaMemcpyAsync(base + L.fr, frs[i].data(), (L.T + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
        pl->status_off.push_back(ncols);
        ncols += (size_t)probs[i].nrhs;
    }
    BP_CK(cudaMalloc(&pl->d_probs, sizeof(DevProblem) * std::max<size_t>(hp.size(), 1)));
    BP_CK(cudaMalloc(&pl->d_maps, sizeof(CUtensorMap) * std::max<size_t>(hm.size(), 1)));
    if (nprob) {
        BP_CK(cudaMemcpyAsync(pl->d_probs, hp.data(), sizeof(DevProblem) * hp.size(), cudaMemcpyHostToDevice, st));
        BP_CK(cudaMemcpyAsync(pl->d_maps, hm.data(), sizeof(CUtensorMap) * hm.size(), cudaMemcpyHostToDevice, st));
    }

    // Schedule: every problem is set up in tick 0; problem i runs the stage
    // of tile T_i - 1 - t in tick t.
    std::vector<BatchItem> all;
    std::vector<std::vector<PhaseSpan>> ticks;
    TickLists tl;
    std::vector<int> stage(nprob, -1);
    int live = 0;
    for (int i = 0; i < nprob; ++i)
        if (pl->layouts[i].S > 0) {
            add_setup(tl, i, pl->layouts[i]);
            stage[i] = pl->layouts[i].T - 1;
            ++live;
        }
    while (live > 0) {
        for (int i = 0; i < nprob; ++i) {
            if (stage[i] < 0) continue;
            if (add_stage(tl, i, pl->layouts[i], frs[i], stage[i])) {
                stage[i] = -1;
                --live;
            } else {
                --stage[i];
            }
        }
        ticks.emplace_back(phCount);
        const size_t at = all.size();
        all.resize(at + tl.size());
        pack_tick(tl, all.data() + at, at, ticks.back().data());
        tl.clear();
    }
    pl->ticks = (int)ticks.size();
    BP_CK(cudaMalloc(&pl->d_items, sizeof(BatchItem) * std::max<size_t>(all.size(), 1)));
    if (!all.empty())
        BP_CK(cudaMemcpyAsync(pl->d_items, all.data(), sizeof(BatchItem) * all.size(), cudaMemcpyHostToDevice, st));
    BP_CK(cudaStreamSynchronize(st));

    // Capture: zero the accumulators, then every tick, the diagonal solves of
    // the next tiles on a forked high-priority stream.
    cudaStream_t cap = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    bool ok = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi_prio) == cudaSuccess &&
              cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&join, cudaEventDisableTiming) == cudaSuccess;
    // First use sets the kernels' shared-memory attributes outside capture.
    if (ok) ok = launch_diag_b(pl->d_probs, pl->d_items, 0, b, cap) == cudaSuccess &&
                 launch_gemm_b(pl->d_probs, pl->d_items, 0, pl->d_maps, cap) == cudaSuccess;
    if (ok) ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    bool capturing = ok;
    if (ok) ok = cudaMemsetAsync(pl->pool, 0, std::max<size_t>(zero_total, 1), cap) == cudaSuccess;
    if (ok) ok = cudaMemsetAsync(pl->d_err, 0, 16, cap) == cudaSuccess;
    for (auto &t : ticks) {
        if (!ok) break;
        ok = launch_tick(t.data(), pl->d_probs, pl->d_items, b, pl->d_maps, cap, side, fork, join, pl->launches,
                         nullptr) == cudaSuccess;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = capturing ? cudaStreamEndCapture(cap, &g) : cudaErrorInvalidValue;
    if (cap) cudaStreamDestroy(cap);
    if (side) cudaStreamDestroy(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (!ok || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        delete pl;
        return HSR_ERR_CUDA;
    }
    pl->graph = g;
    if (cudaGraphInstantiateWithFlags(&pl->exec, g, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess) {
        delete pl;
        return HSR_ERR_CUDA;
    }
    *out = pl;
    return HSR_OK;
}

static cudaError_t queue_direct(hsr_batch_plan *pl, cudaStream_t st);

extern "C" int hsr_batch_plan_execute(hsr_batch_plan *pl, void *stream) {
    if (!pl) return HSR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (pl->engine == HSR_BATCH_ENGINE_QUEUE) {
        const cudaError_t e = pl->qdirect ? queue_direct(pl, st) : cudaGraphLaunch(pl->qexec, st);
        if (e != cudaSuccess) return record_status(HSR_ERR_CUDA, e);
    } else if (cudaGraphLaunch(pl->exec, st) != cudaSuccess) {
        return HSR_ERR_CUDA;
    }
    // Convergence: status of every column of every problem.
    int result = HSR_OK;
    int errw = 0;
    if (cudaMemcpyAsync(&errw, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return HSR_ERR_CUDA;
    size_t ncols = 0;
    for (int i = 0; i < pl->nprob; ++i) ncols += (size_t)pl->specs[i].nrhs;
    std::vector<int> stv(std::max<size_t>(ncols, 1));
    if (cudaStreamSynchronize(st) != cudaSuccess) return HSR_ERR_CUDA;
    if (ncols && cudaMemcpy(stv.data(), pl->d_status, ncols * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return HSR_ERR_CUDA;
    if (errw) return HSR_ERR_DEVICE;
    // Problems with columns that did not converge: solved again alone, which
    // runs the same first pass and then the restart rounds.
    for (int i = 0; i < pl->nprob; ++i) {
        bool all = true;
        for (int k = 0; k < pl->specs[i].nrhs; ++k) all = all && stv[pl->status_off[i] + (size_t)k];
        if (all) continue;
        const hsr_batch_problem &p = pl->specs[i];
        hsr_options o{};
        o.scaling = pl->is ? HSR_SCALING_POW2 : HSR_SCALING_DOUBLE;
        o.max_restarts = -1;
        const int rc = hsr_inverse_iteration_device(p.n, p.dH, p.lddH, p.nrhs, p.dwr, pl->b, p.dvr, p.lddvr, &o,
                                                    stream, nullptr, nullptr);
        if (rc < 0) return rc;
        if (rc == HSR_ERR_NOT_CONVERGED) result = HSR_ERR_NOT_CONVERGED;
    }
    return result;
}

// ------------------------------------------------------- queue engine
namespace {

// Counters of problem i start at base[i]: four fixed ones (norms, init,
// finalize, normalize), then four per stage J (diagonal solve of tile J,
// part 1, GEMM over the rows of tile J-1, GEMM over the rows above).
enum { qcNorms = 0, qcInit, qcFinal, qcNormalize, qcFixed };
inline int qc_stage(int J, int which) { return qcFixed + 4 * J + which; }
enum { qsDiag = 0, qsPart1, qsTop, qsRest };

// The work list of the queue engine: the ticks of the graph engine, in the
// order the graph launches them, with every item's dependencies on the
// counters of its own problem.  Initial vectors, diagonal solves and
// finalisation are grouped (a warp per column or 32-shift block) so that an
// item uses the CTA.
void build_queue(const hsr_batch_plan *pl, int dw, std::vector<QueueItem> &out, std::vector<int> &base,
                 size_t &n_ctr) {
    const int nprob = pl->nprob;
    base.assign(nprob, 0);
    n_ctr = 0;
    for (int i = 0; i < nprob; ++i) {
        base[i] = (int)n_ctr;
        n_ctr += qcFixed + 4 * (size_t)pl->layouts[i].T;
    }
    auto item = [](int x, int y, int z, int w, int kind, int ctr, int d0, int t0, int d1 = -1, int t1 = 0) {
        QueueItem q{};
        q.it = make_int4(x, y, z, w);
        q.kind = kind;
        q.ctr = ctr;
        q.dep0 = d0;
        q.tgt0 = t0;
        q.dep1 = d1;
        q.tgt1 = t1;
        return q;
    };
    struct Counts {
        int norms, init, diag, part1, fin, cbs;
    };
    std::vector<Counts> cnt(nprob);
    auto top_rows = [&](int i, int J) {
        const std::vector<int> &fr = pl->frs[i];
        return (fr[J] - (fr[J - 1] & ~7) + kGemmBM - 1) / kGemmBM;
    };
    auto rest_rows = [&](int i, int J) { return (pl->frs[i][J - 1] + kGemmBM - 1) / kGemmBM; };
    for (int i = 0; i < nprob; ++i) {
        const Layout &L = pl->layouts[i];
        const int sb32 = (L.S + 31) / 32;
        cnt[i] = Counts{(L.n + kNormRows - 1) / kNormRows, (L.S + kQueueInitCols - 1) / kQueueInitCols,
                        (sb32 + dw - 1) / dw, (L.S + kPart1Shifts - 1) / kPart1Shifts,
                        (sb32 + kQueueFinalBlocks - 1) / kQueueFinalBlocks, (L.S + kGemmBN - 1) / kGemmBN};
    }
    std::vector<QueueItem> ph[phCount];
    auto flush = [&]() {
        for (auto &v : ph) {
            out.insert(out.end(), v.begin(), v.end());
            v.clear();
        }
    };
    std::vector<int> stage(nprob, -1);
    int live = 0;
    for (int i = 0; i < nprob; ++i) {
        const Layout &L = pl->layouts[i];
        if (L.S == 0) continue;
        const int b0 = base[i], J = L.T - 1;
        for (int r = 0; r < cnt[i].norms; ++r)
            ph[phNorms].push_back(item(desc(i, 0), 0, r, 0, qkNorms, b0 + qcNorms, -1, 0));
        for (int g = 0; g < cnt[i].init; ++g)
            ph[phInit].push_back(item(desc(i, 0), 0, g, 0, qkInit, b0 + qcInit, b0 + qcNorms, cnt[i].norms));
        for (int g = 0; g < cnt[i].diag; ++g)
            ph[phDiagFirst].push_back(item(desc(i, J), J, g, 0, qkDiag, b0 + qc_stage(J, qsDiag), b0 + qcInit,
                                           cnt[i].init));
        stage[i] = J;
        ++live;
    }
    while (live > 0) {
        for (int i = 0; i < nprob; ++i) {
            const int J = stage[i];
            if (J < 0) continue;
            const Layout &L = pl->layouts[i];
            const int b0 = base[i];
            const Counts &c = cnt[i];
            if (J >= 1) {
                const int p = desc(i, J), pn = desc(i, J - 1);
                const int ntop = top_rows(i, J) * c.cbs;
                const int nrest = rest_rows(i, J) * c.cbs;
                const int prev_rest = J + 1 <= L.T - 1 ? rest_rows(i, J + 1) * c.cbs : 0;
                for (int x = 0; x < c.part1; ++x)
                    ph[phPart1].push_back(item(p, J, x, 0, qkPart1, b0 + qc_stage(J, qsPart1),
                                               b0 + qc_stage(J, qsDiag), c.diag,
                                               prev_rest > 0 ? b0 + qc_stage(J + 1, qsRest) : -1, prev_rest));
                for (int r = 0; r < top_rows(i, J); ++r)
                    for (int cb = 0; cb < c.cbs; ++cb)
                        ph[phGemmTop].push_back(item(p, J, r | kGemmTopFlag, cb, qkGemm, b0 + qc_stage(J, qsTop),
                                                     b0 + qc_stage(J, qsPart1), c.part1));
                for (int g = 0; g < c.diag; ++g)
                    ph[phDiagNext].push_back(item(pn, J - 1, g, 0, qkDiag, b0 + qc_stage(J - 1, qsDiag),
                                                  b0 + qc_stage(J, qsTop), ntop));
                for (int r = 0; r < rest_rows(i, J); ++r)
                    for (int cb = 0; cb < c.cbs; ++cb)
                        ph[phGemmRest].push_back(item(p, J, r, cb, qkGemm, b0 + qc_stage(J, qsRest),
                                                      b0 + qc_stage(J, qsPart1), c.part1));
                (void)nrest;
            }
            if (J <= 1) {
                for (int g = 0; g < c.fin; ++g)
                    ph[phFinal].push_back(item(desc(i, 0), 0, g, 0, qkFinal, b0 + qcFinal, b0 + qc_stage(0, qsDiag),
                                               c.diag));
                const int nn = (L.S + kNormalizeCols - 1) / kNormalizeCols;
                for (int x = 0; x < nn; ++x)
                    ph[phNormalize].push_back(item(desc(i, 0), 0, x, 0, qkNormalize, b0 + qcNormalize,
                                                   b0 + qcFinal, c.fin));
                stage[i] = -1;
                --live;
            } else {
                stage[i] = J - 1;
            }
        }
        flush();
    }
    flush();
}

}  // namespace

// Builds the queue engine's work list, counters and graph (once per plan).
static int build_queue_engine(hsr_batch_plan *pl, cudaStream_t st) {
    if (pl->qexec || pl->qdirect) return HSR_OK;
    const int dw = queue_diag_warps(pl->b);
    std::vector<QueueItem> items;
    std::vector<int> base;
    size_t n_ctr = 0;
    build_queue(pl, dw, items, base, n_ctr);
    const int grid = queue_max_grid(pl->b);
    if (grid <= 0) return HSR_ERR_CUDA;
    if (cudaMalloc(&pl->d_qitems, sizeof(QueueItem) * std::max<size_t>(items.size(), 1)) != cudaSuccess ||
        cudaMalloc(&pl->d_ctr, sizeof(int) * (n_ctr + 32)) != cudaSuccess)
        return HSR_ERR_NOMEM;
    if (!items.empty() &&
        cudaMemcpyAsync(pl->d_qitems, items.data(), sizeof(QueueItem) * items.size(), cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
        return HSR_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return HSR_ERR_CUDA;
    pl->n_qitems = (int)items.size();
    pl->n_ctr = n_ctr;
    pl->qgrid = grid;
    pl->qdiag_warps = dw;
    int *ticket = pl->d_ctr + n_ctr;
    // One graph: zero the accumulators, counters, ticket and error word, then
    // the single persistent launch.
    cudaStream_t cap = nullptr;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return HSR_ERR_CUDA;
    bool ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    const bool capturing = ok;
    if (ok) ok = cudaMemsetAsync(pl->pool, 0, std::max<size_t>(pl->zero_bytes, 1), cap) == cudaSuccess;
    if (ok) ok = cudaMemsetAsync(pl->d_err, 0, 16, cap) == cudaSuccess;
    if (ok) ok = cudaMemsetAsync(pl->d_ctr, 0, sizeof(int) * (n_ctr + 32), cap) == cudaSuccess;
    if (ok)
        ok = launch_queue(pl->d_probs, pl->d_qitems, pl->n_qitems, pl->d_maps, pl->d_ctr, ticket, pl->d_err, pl->b,
                          grid, cap) == cudaSuccess;
    cudaGraph_t g = nullptr;
    const cudaError_t ce = capturing ? cudaStreamEndCapture(cap, &g) : cudaErrorInvalidValue;
    cudaStreamDestroy(cap);
    if (ok && ce == cudaSuccess && cudaGraphInstantiate(&pl->qexec, g, 0) == cudaSuccess) {
        pl->qgraph = g;
        return HSR_OK;
    }
    // A runtime that cannot capture the cooperative launch: the same memsets
    // and launch are issued directly by every execute.
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    pl->qexec = nullptr;
    pl->qdirect = true;
    return HSR_OK;
}

static cudaError_t queue_direct(hsr_batch_plan *pl, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(pl->pool, 0, std::max<size_t>(pl->zero_bytes, 1), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(pl->d_err, 0, 16, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(pl->d_ctr, 0, sizeof(int) * (pl->n_ctr + 32), st)) != cudaSuccess)
        return e;
    return launch_queue(pl->d_probs, pl->d_qitems, pl->n_qitems, pl->d_maps, pl->d_ctr, pl->d_ctr + pl->n_ctr,
                        pl->d_err, pl->b, pl->qgrid, st);
}

extern "C" int hsr_batch_plan_set_engine(hsr_batch_plan *pl, int engine, void *stream) {
    if (!pl || (engine != HSR_BATCH_ENGINE_TICKS && engine != HSR_BATCH_ENGINE_QUEUE)) return HSR_ERR_ARG;
    if (engine == HSR_BATCH_ENGINE_QUEUE) {
        const int rc = build_queue_engine(pl, static_cast<cudaStream_t>(stream));
        if (rc) return rc;
    }
    pl->engine = engine;
    return HSR_OK;
}

extern "C" int hsr_batch_plan_queue_info(const hsr_batch_plan *pl, int *engine, long *items, int *grid,
                                         int *diag_warps, int *in_graph) {
    if (!pl) return HSR_ERR_ARG;
    if (in_graph) *in_graph = pl->qexec != nullptr;
    if (engine) *engine = pl->engine;
    if (items) *items = pl->n_qitems;
    if (grid) *grid = pl->qgrid;
    if (diag_warps) *diag_warps = pl->qdiag_warps;
    return HSR_OK;
}

extern "C" int hsr_batch_plan_info(const hsr_batch_plan *pl, int *tlsz, int *ticks, long *launches) {
    if (!pl) return HSR_ERR_ARG;
    if (tlsz) *tlsz = pl->b;
    if (ticks) *ticks = pl->ticks;
    if (launches) *launches = pl->launches;
    return HSR_OK;
}

extern "C" void hsr_batch_plan_destroy(hsr_batch_plan *pl) { delete pl; }

extern "C" int hsr_autotune_batch(int nprob, const hsr_batch_problem *probs, const int *cand, int ncand,
                                  double *ms_out, void *stream) {
    if (nprob <= 0 || !probs || !cand || ncand <= 0) return HSR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int n_lo = 1 << 30, n_hi = 0;
    for (int i = 0; i < nprob; ++i) {
        n_lo = std::min(n_lo, probs[i].n);
        n_hi = std::max(n_hi, probs[i].n);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = -1;
    double best_ms = 1e300;
    for (int c = 0; c < ncand; ++c) {
        hsr_batch_plan *pl = nullptr;
        double ms = 1e300;
        if (hsr_batch_plan_create(&pl, nprob, probs, cand[c], nullptr, stream) == HSR_OK) {
            hsr_batch_plan_execute(pl, stream);   // warm-up
            cudaEventRecord(e0, st);
            const int reps = 2;
            for (int r = 0; r < reps; ++r) cudaGraphLaunch(pl->exec, st);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms = t / reps;
            hsr_batch_plan_destroy(pl);
        }
        if (ms_out) ms_out[c] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = cand[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best > 0) {
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune[{n_lo, n_hi}] = best;
    }
    return best > 0 ? best : HSR_ERR_CUDA;
}

// ==================================================================== server
namespace hsr {
namespace {

// First-fit allocator over one device pool, with coalescing frees.
struct PoolAlloc {
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;   // offset -> size
    void reset(size_t c) {
        cap = c;
        used = peak = 0;
        free_.clear();
        free_[0] = c;
    }
    bool alloc(size_t bytes, size_t &off) {
        bytes = up(bytes, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                used += bytes;
                peak = std::max(peak, used);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = up(bytes, 256);
        used -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct ActiveReq {
    int req = -1, slot = -1;
    size_t off = 0, bytes = 0;
    Layout L;
    std::vector<int> fr;
    long long ldh = 0, ldx = 0;
    int stage = 0;            // diagonal tile solved last; its stage runs next
    bool finishing = false;   // the current tick completes the request
    bool retiring = false;    // results are on their way to the host
    cudaEvent_t done = nullptr;
    int *h_status = nullptr;  // pinned, [nrhs]
};

}  // namespace
}  // namespace hsr

struct hsr_server {
    hsr_server_config cfg{};
    int b = 64, is = 1, max_slots = 4096;
    cudaStream_t st = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    char *pool = nullptr;
    size_t pool_bytes = 0;
    PoolAlloc alloc;
    DevProblem *d_probs = nullptr;
    CUtensorMap *d_maps = nullptr;
    int *d_err = nullptr;
    BatchItem *d_items[2] = {nullptr, nullptr};
    BatchItem *h_items[2] = {nullptr, nullptr};
    size_t items_cap[2] = {0, 0};
    DevProblem *h_prob_stage = nullptr;   // pinned staging for slot descriptors
    CUtensorMap *h_map_stage = nullptr;
    cudaEvent_t tick_ev[2] = {nullptr, nullptr};
    std::vector<int> free_slots;
    ~hsr_server() {
        if (st) cudaStreamSynchronize(st);
        if (side) cudaStreamDestroy(side);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        for (int i = 0; i < 2; ++i) {
            if (d_items[i]) cudaFree(d_items[i]);
            if (h_items[i]) cudaFreeHost(h_items[i]);
            if (tick_ev[i]) cudaEventDestroy(tick_ev[i]);
        }
        if (h_prob_stage) cudaFreeHost(h_prob_stage);
        if (h_map_stage) cudaFreeHost(h_map_stage);
        if (d_probs) cudaFree(d_probs);
        if (d_maps) cudaFree(d_maps);
        if (d_err) cudaFree(d_err);
        if (pool) cudaFree(pool);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {
size_t request_bytes(const Layout &L, long long ldh, long long ldx) {
    return L.total + up((size_t)ldh * L.n * 8, 256) + up((size_t)L.S * 8, 256) + up((size_t)ldx * L.S * 8, 256);
}
}  // namespace

extern "C" int hsr_server_create(hsr_server **out, const hsr_server_config *cfg) {
    if (!out) return HSR_ERR_ARG;
    *out = nullptr;
    hsr_server *s = new hsr_server();
    if (cfg) s->cfg = *cfg;
    s->b = s->cfg.tlsz > 0 ? s->cfg.tlsz : hsr_autotune_tlsz(64, 4096);
    if (s->b % 4 || s->b > 384) {
        delete s;
        return HSR_ERR_ARG;
    }
    s->is = s->cfg.scaling == HSR_SCALING_DOUBLE ? 0 : 1;
    s->max_slots = s->cfg.max_active > 0 ? s->cfg.max_active : 4096;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    s->pool_bytes = (size_t)(s->cfg.hbm_budget_bytes > 0 ? s->cfg.hbm_budget_bytes : 0.4 * (double)fr);
    s->pool_bytes = up(s->pool_bytes, 256);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    const size_t ndesc = 2 * (size_t)s->max_slots;   // two descriptors per slot (tile parity)
    bool ok = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, hi_prio) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&s->pool, s->pool_bytes) == cudaSuccess &&
              cudaMalloc(&s->d_probs, sizeof(DevProblem) * ndesc) == cudaSuccess &&
              cudaMalloc(&s->d_maps, sizeof(CUtensorMap) * 3 * ndesc) == cudaSuccess &&
              cudaMalloc(&s->d_err, 16) == cudaSuccess &&
              cudaMallocHost(&s->h_prob_stage, sizeof(DevProblem) * ndesc) == cudaSuccess &&
              cudaMallocHost(&s->h_map_stage, sizeof(CUtensorMap) * 3 * ndesc) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->tick_ev[0], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->tick_ev[1], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        delete s;
        return HSR_ERR_NOMEM;
    }
    cudaMemset(s->d_err, 0, 16);
    s->alloc.reset(s->pool_bytes);
    *out = s;
    return HSR_OK;
}

extern "C" void hsr_server_destroy(hsr_server *s) { delete s; }

extern "C" int hsr_server_replay(hsr_server *s, int nreq, hsr_request *reqs, double *latency, int *status_out,
                                 hsr_server_stats *stats) {
    if (!s || nreq < 0 || (nreq > 0 && !reqs)) return HSR_ERR_ARG;
    using clock = std::chrono::steady_clock;
    const auto t0 = clock::now();
    auto elapsed = [&]() { return std::chrono::duration<double>(clock::now() - t0).count(); };
    cudaStream_t st = s->st;
    const int b = s->b;

    std::vector<int> order(nreq);
    for (int i = 0; i < nreq; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return reqs[a].arrival_s < reqs[c].arrival_s; });
    for (int i = 0; i < nreq; ++i) {
        const hsr_request &r = reqs[i];
        if (r.n <= 0 || r.ldH < r.n || r.nrhs < 0 || r.ldvr < r.n || !r.H || (r.nrhs && (!r.wr || !r.vr)))
            return HSR_ERR_ARG;
        if (status_out) status_out[i] = HSR_OK;
        if (latency) latency[i] = -1.0;
    }
    s->free_slots.clear();
    for (int i = s->max_slots - 1; i >= 0; --i) s->free_slots.push_back(i);
    std::deque<int> queue;
    std::vector<ActiveReq> active;
    size_t next = 0;
    int completed = 0, max_active = 0, parity = 0;
    long ticks = 0, launches = 0;
    bool tick_used[2] = {false, false};
    TickLists tl;
    PhaseSpan spans[phCount];
    int result = HSR_OK;
    double flops = 0.0, wait_s = 0.0;
    // Optional device timing of the phases (hsr_set_kernel_timing).
    PhaseTimer timer;
    PhaseTimer *tm = stats && kernel_timing_enabled() ? &timer : nullptr;
    // Convergence flags come back through one pinned array (a slice per request).
    struct PinnedInts {
        int *p = nullptr;
        ~PinnedInts() {
            if (p) cudaFreeHost(p);
        }
    } h_status;
    std::vector<size_t> status_at(nreq);
    size_t total_cols = 0;
    for (int i = 0; i < nreq; ++i) {
        status_at[i] = total_cols;
        total_cols += (size_t)reqs[i].nrhs;
    }
    if (cudaMallocHost(&h_status.p, sizeof(int) * std::max<size_t>(total_cols, 1)) != cudaSuccess)
        return HSR_ERR_NOMEM;
    // A failed CUDA call ends the replay: the work already enqueued is
    // waited for, every request that has not completed reports
    // HSR_ERR_CUDA, and so does the call.
    std::vector<char> finished(nreq, 0);
    auto fail = [&](cudaError_t e) -> int {
        (void)cudaStreamSynchronize(st);
        (void)cudaStreamSynchronize(s->side);
        for (auto &a : active)
            if (a.done) cudaEventDestroy(a.done);
        for (int i = 0; i < nreq; ++i)
            if (!finished[i] && status_out) status_out[i] = HSR_ERR_CUDA;
        return record_status(HSR_ERR_CUDA, e);
    };
#define SRV_CK(x)                              \
    do {                                       \
        const cudaError_t e_ = (x);            \
        if (e_ != cudaSuccess) return fail(e_); \
    } while (0)

    while (completed < nreq) {
        const double now = elapsed();
        while (next < (size_t)nreq && reqs[order[next]].arrival_s <= now) queue.push_back(order[next++]);

        // Retire requests whose results reached the host.
        for (size_t i = 0; i < active.size();) {
            ActiveReq &a = active[i];
            const cudaError_t q = a.retiring ? cudaEventQuery(a.done) : cudaErrorNotReady;
            if (q != cudaSuccess && q != cudaErrorNotReady) return fail(q);
            if (q == cudaSuccess) {
                const hsr_request &r = reqs[a.req];
                bool all = true;
                for (int k = 0; k < r.nrhs; ++k) all = all && a.h_status[k];
                int rc = HSR_OK;
                if (!all) {
                    // Restart rounds: solved again on the plain path.
                    hsr_options o{};
                    o.scaling = s->is ? HSR_SCALING_POW2 : HSR_SCALING_DOUBLE;
                    o.max_restarts = -1;
                    rc = hsr_inverse_iteration_ex(r.n, r.H, r.ldH, r.nrhs, r.wr, b, 64, r.vr, r.ldvr, &o, nullptr);
                    if (rc < 0) result = rc;
                }
                if (status_out) status_out[a.req] = rc;
                if (latency) latency[a.req] = elapsed() - r.arrival_s;
                finished[a.req] = 1;
                cudaEventDestroy(a.done);
                a.done = nullptr;
                s->alloc.release(a.off, a.bytes);
                s->free_slots.push_back(a.slot);
                active[i] = std::move(active.back());
                active.pop_back();
                ++completed;
                continue;
            }
            ++i;
        }

        // Admit in arrival order while the pool and slots allow.
        tl.clear();
        std::vector<int> admitted;
        while (!queue.empty() && !s->free_slots.empty()) {
            const int ri = queue.front();
            const hsr_request &r = reqs[ri];
            if (r.nrhs == 0) {
                queue.pop_front();
                if (latency) latency[ri] = elapsed() - r.arrival_s;
                finished[ri] = 1;
                ++completed;
                continue;
            }
            ActiveReq a;
            a.req = ri;
            a.L.compute(r.n, r.nrhs, b);
            a.ldh = round_up_ll(r.n, 32);
            a.ldx = round_up_ll(r.n, 4);
            a.bytes = request_bytes(a.L, a.ldh, a.ldx);
            if (a.bytes > s->pool_bytes) {   // can never fit
                queue.pop_front();
                if (status_out) status_out[ri] = HSR_ERR_NOMEM;
                result = HSR_ERR_NOMEM;
                finished[ri] = 1;
                ++completed;
                continue;
            }
            if (!s->alloc.alloc(a.bytes, a.off)) break;   // head of line waits for memory
            queue.pop_front();
            a.slot = s->free_slots.back();
            s->free_slots.pop_back();
            char *base = s->pool + a.off;
            double *dH = reinterpret_cast<double *>(base + a.L.total);
            double *dwr = reinterpret_cast<double *>(base + a.L.total + up((size_t)a.ldh * r.n * 8, 256));
            double *dX = reinterpret_cast<double *>(reinterpret_cast<char *>(dwr) + up((size_t)r.nrhs * 8, 256));
            partition_rows(r.n, a.L.T, b, a.fr);
            a.h_status = h_status.p + status_at[ri];
            // A page-locked request block moves by SM loads through its mapped
            // pointer, like the drop-in call's; other buffers by copy engine.
            if (const void *Hm = mapped_view(r.H)) {
                ++launches;
                SRV_CK(copy_cols(dH, a.ldh, static_cast<const double *>(Hm), r.ldH, r.n, r.n, st));
            } else {
                SRV_CK(cudaMemcpy2DAsync(dH, a.ldh * 8, r.H, (size_t)r.ldH * 8, (size_t)r.n * 8, r.n,
                                         cudaMemcpyHostToDevice, st));
            }
            SRV_CK(cudaMemcpyAsync(dwr, r.wr, (size_t)r.nrhs * 8, cudaMemcpyHostToDevice, st));
            SRV_CK(cudaMemcpyAsync(base + a.L.fr, a.fr.data(), (a.L.T + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                   st));
            SRV_CK(cudaMemsetAsync(base, 0, a.L.zero_bytes, st));
            const int d0 = desc(a.slot, 0);
            for (int par = 0; par < 2; ++par) {
                s->h_prob_stage[d0 + par] = make_problem(a.L, base, dH, a.ldh, dwr, dX, a.ldx, s->is, s->d_err, par);
                make_maps(&s->h_map_stage[3 * (size_t)(d0 + par)], a.L, dH, a.ldh, base, par);
            }
            SRV_CK(cudaMemcpyAsync(s->d_probs + d0, s->h_prob_stage + d0, 2 * sizeof(DevProblem),
                                   cudaMemcpyHostToDevice, st));
            SRV_CK(cudaMemcpyAsync(s->d_maps + 3 * (size_t)d0, s->h_map_stage + 3 * (size_t)d0,
                                   6 * sizeof(CUtensorMap), cudaMemcpyHostToDevice, st));
            add_setup(tl, a.slot, a.L);
            flops += 2.0 * (double)r.n * r.n * r.nrhs;
            a.stage = a.L.T - 1;
            active.push_back(std::move(a));
        }
        int running = 0;
        for (auto &a : active)
            if (!a.retiring) ++running;
        max_active = std::max(max_active, (int)active.size());
        if (running == 0) {
            if (completed >= nreq) break;
            // Idle: wait for an arrival or a completion.
            bool pending_done = false;
            for (auto &a : active) pending_done = pending_done || a.retiring;
            if (!pending_done && next < (size_t)nreq && queue.empty()) {
                const double wait = reqs[order[next]].arrival_s - elapsed();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            } else {
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            }
            continue;
        }

        // Build this tick: each running request runs its next stage.
        for (auto &a : active) {
            if (a.retiring) continue;
            a.finishing = add_stage(tl, a.slot, a.L, a.fr, a.stage);
        }
        const size_t count = tl.size();
        // The item buffer of this parity was last used two ticks ago.
        if (tick_used[parity]) {
            const double w0 = elapsed();
            SRV_CK(cudaEventSynchronize(s->tick_ev[parity]));
            wait_s += elapsed() - w0;
        }
        if (count > s->items_cap[parity]) {
            if (s->d_items[parity]) cudaFree(s->d_items[parity]);
            if (s->h_items[parity]) cudaFreeHost(s->h_items[parity]);
            s->items_cap[parity] = std::max<size_t>(count * 2, 4096);
            if (cudaMalloc(&s->d_items[parity], sizeof(BatchItem) * s->items_cap[parity]) != cudaSuccess ||
                cudaMallocHost(&s->h_items[parity], sizeof(BatchItem) * s->items_cap[parity]) != cudaSuccess) {
                s->d_items[parity] = nullptr;
                s->h_items[parity] = nullptr;
                s->items_cap[parity] = 0;
                (void)fail(cudaErrorMemoryAllocation);
                return record_status(HSR_ERR_NOMEM, cudaSuccess);
            }
        }
        pack_tick(tl, s->h_items[parity], 0, spans);
        SRV_CK(cudaMemcpyAsync(s->d_items[parity], s->h_items[parity], sizeof(BatchItem) * count,
                               cudaMemcpyHostToDevice, st));
        SRV_CK(launch_tick(spans, s->d_probs, s->d_items[parity], b, s->d_maps, st, s->side, s->fork, s->join,
                           launches, tm));
        // Requests that finished this tick: copy results to the host.
        for (auto &a : active) {
            if (a.retiring) continue;
            if (a.finishing) {
                const hsr_request &r = reqs[a.req];
                char *base = s->pool + a.off;
                double *dwr = reinterpret_cast<double *>(base + a.L.total + up((size_t)a.ldh * r.n * 8, 256));
                double *dX = reinterpret_cast<double *>(reinterpret_cast<char *>(dwr) + up((size_t)r.nrhs * 8, 256));
                if (void *Xm = mapped_view(r.vr)) {   // the caller's padding rows stay untouched
                    ++launches;
                    SRV_CK(copy_cols(static_cast<double *>(Xm), r.ldvr, dX, a.ldx, r.n, r.nrhs, st));
                } else {
                    SRV_CK(cudaMemcpy2DAsync(r.vr, (size_t)r.ldvr * 8, dX, a.ldx * 8, (size_t)r.n * 8, r.nrhs,
                                             cudaMemcpyDeviceToHost, st));
                }
                SRV_CK(cudaMemcpyAsync(a.h_status, base + a.L.status, r.nrhs * sizeof(int), cudaMemcpyDeviceToHost,
                                       st));
                SRV_CK(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
                SRV_CK(cudaEventRecord(a.done, st));
                a.retiring = true;
            } else {
                --a.stage;
            }
        }
        SRV_CK(cudaEventRecord(s->tick_ev[parity], st));
        tick_used[parity] = true;
        parity ^= 1;
        ++ticks;
    }
    SRV_CK(cudaStreamSynchronize(st));
    int errw = 0;
    SRV_CK(cudaMemcpy(&errw, s->d_err, sizeof(int), cudaMemcpyDeviceToHost));
#undef SRV_CK
    if (errw) result = HSR_ERR_DEVICE;
    if (stats) {
        stats->wall_s = elapsed();
        stats->ticks = ticks;
        stats->launches = launches;
        stats->max_active = max_active;
        stats->peak_bytes = (double)s->alloc.peak;
        stats->flops = flops;
        stats->host_wait_s = wait_s;
        for (int ph = 0; ph < phCount; ++ph) stats->phase_ms[ph] = 0.0;
        timer.add_to(stats->phase_ms);
    }
    return record_status(result, cudaSuccess);
}
