// batch.cu -- kernel-shape tuning and uneven batches over several contexts (C ABI, include/uepm_gb300.h).
//
// No reference counterpart: the reference solves one material at a time with an OpenMP loop over
// k-points (BandStructure::Compute_parallel, src/EPP/BandStructure.cpp:162-201).
//
// Tuning. A context's kernel-shape choices (uepm_tuning) are threaded into its launches. The
// autotuner times candidate shapes on a seeded sample of first-zone k-points with CUDA events and
// keeps the fastest, one field at a time (coordinate descent from the automatic choices); the result
// is cached per (device, n, real/complex, precision, nb, vectors).
//
// Batches. Groups of (context, k-points, outputs) are enqueued together: each distinct context on
// its own stream, forked from and joined back to the caller's stream, so the per-context pipelines
// (persistent-grid reductions, one-CTA-per-matrix kernels) overlap and fill the GPU together. The
// first run is eager (it warms the kernels' one-time set-up); the second captures the whole
// fork/join pipeline into a CUDA graph, and later runs replay it with a single graph launch while
// the groups and the contexts' workspaces are unchanged.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "ctx_internal.h"
#include "uepm_kernels.h"

using namespace uepm;

namespace {

#define UEPM_CK(call)                                                                  \
    do {                                                                               \
        cudaError_t err_ = (call);                                                     \
        if (err_ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(err_));           \
            return UEPM_ERR_CUDA;                                                      \
        }                                                                              \
    } while (0)

using TuneKey = std::tuple<int, int, int, int, int, int>;  // device, n, real, precision, nb, vectors
std::mutex                         g_tune_mu;
std::map<TuneKey, uepm_tuning>     g_tune_cache;

TuneKey tune_key(const uepm_ctx* ctx, int nb, uint32_t want) {
    const int vec = (want & (UEPM_WANT_VECTORS | UEPM_WANT_GRADIENT)) != 0;
    return TuneKey{ctx->device, ctx->n, ctx->real ? 1 : 0, ctx->precision, nb, vec};
}

bool valid_tuning(const uepm_ctx* ctx, const uepm_tuning& t) {
    if (t.reduction < 0 || t.reduction > 6) return false;
    if (t.ctas_per_sm < 0 || t.ctas_per_sm > 8) return false;
    if (t.cluster != 0 && t.cluster != 2 && t.cluster != 4 && t.cluster != 8 && t.cluster != 16) return false;
    if (t.vector_lanes != 0 && t.vector_lanes != 8 && t.vector_lanes != 16 && t.vector_lanes != 32) return false;
    if (t.chunk != 0 && (t.chunk < 64 || t.chunk > 32768)) return false;
    if (t.max_iter < 0 || t.max_iter > 1000) return false;
    if (t.tensor_cores < 0 || t.tensor_cores > 1) return false;
    if (t.streams < 0 || t.streams > 2) return false;
    (void)ctx;
    return true;
}

// Seeded uniform k-points in the first Brillouin zone (truncated octahedron: |k_i| <= 1 and
// |kx| + |ky| + |kz| <= 3/2), by rejection from [-1, 1]^3.
std::vector<double> sample_bz(size_t nk, uint64_t seed) {
    std::mt19937_64                        rng(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::vector<double>                    k;
    k.reserve(3 * nk);
    while (k.size() < 3 * nk) {
        const double x = u(rng), y = u(rng), z = u(rng);
        if (std::fabs(x) + std::fabs(y) + std::fabs(z) <= 1.5) {
            k.push_back(x);
            k.push_back(y);
            k.push_back(z);
        }
    }
    return k;
}

struct DeviceBuf {
    void* p = nullptr;
    ~DeviceBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace

extern "C" {

int uepm_ctx_get_tuning(const uepm_ctx* ctx, uepm_tuning* out) {
    if (!ctx || !out) {
        set_error("uepm_ctx_get_tuning: null argument");
        return UEPM_ERR_INVALID;
    }
    *out = ctx->tune;
    return UEPM_OK;
}

int uepm_ctx_set_tuning(uepm_ctx* ctx, const uepm_tuning* t) {
    if (!ctx || !t) {
        set_error("uepm_ctx_set_tuning: null argument");
        return UEPM_ERR_INVALID;
    }
    if (!valid_tuning(ctx, *t)) {
        set_error("uepm_ctx_set_tuning: a field is out of range");
        return UEPM_ERR_OUT_OF_RANGE;
    }
    ctx->tune = *t;
    return UEPM_OK;
}

int uepm_ctx_autotune(uepm_ctx* ctx, int nb, uint32_t want, size_t sample_k, void* stream) {
    if (!ctx) {
        set_error("uepm_ctx_autotune: null context");
        return UEPM_ERR_INVALID;
    }
    if (sample_k == 0) sample_k = 4096;
    const TuneKey key = tune_key(ctx, nb, want);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto                        it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const int32_t cap = ctx->tune.max_iter;
            ctx->tune          = it->second;
            ctx->tune.max_iter = cap;
            return UEPM_OK;
        }
    }
    SolvePlan sp;
    int       rc = plan_solve(ctx, 1, nb, want, &sp);
    if (rc) return rc;
    const bool   wv = (want & UEPM_WANT_VECTORS) != 0, wg = (want & UEPM_WANT_GRADIENT) != 0;
    const size_t n  = (size_t)ctx->n;
    if (wv) sample_k = std::max<size_t>(64, std::min(sample_k, ((size_t)512 << 20) / (16 * n * (size_t)nb)));
    cudaStream_t s = (cudaStream_t)stream;
    DeviceBuf    bk, bE, bX, bg, bs;
    const auto   hk = sample_bz(sample_k, 0x5eed0123ULL);
    UEPM_CK(cudaMalloc(&bk.p, sizeof(double) * 3 * sample_k));
    UEPM_CK(cudaMalloc(&bE.p, sizeof(double) * sample_k * nb));
    UEPM_CK(cudaMalloc(&bs.p, sizeof(int32_t) * sample_k));
    if (wv) UEPM_CK(cudaMalloc(&bX.p, 16 * n * nb * sample_k));
    if (wg) UEPM_CK(cudaMalloc(&bg.p, sizeof(double) * 3 * nb * sample_k));
    UEPM_CK(cudaMemcpyAsync(bk.p, hk.data(), sizeof(double) * 3 * sample_k, cudaMemcpyHostToDevice, s));
    cudaEvent_t a, b;
    UEPM_CK(cudaEventCreate(&a));
    UEPM_CK(cudaEventCreate(&b));
    const uepm_tuning saved = ctx->tune;
    const int         prof  = ctx->profiling;
    ctx->profiling          = 0;

    // milliseconds per solve of the sample with the context's current tuning (1 warm-up, 2 timed)
    auto timed = [&](double* ms) -> int {
        SolvePlan p;
        int       r = plan_solve(ctx, sample_k, nb, want, &p);
        if (!r) r = ensure_workspace(ctx, p.ws_bytes);
        if (r) return r;
        auto once = [&]() {
            return enqueue_solve(ctx, p, static_cast<double*>(bk.p), sample_k, nb, want, static_cast<double*>(bE.p),
                                 static_cast<double*>(bX.p), static_cast<double*>(bg.p), static_cast<int32_t*>(bs.p), s);
        };
        if ((r = once())) return r;
        if (cudaEventRecord(a, s) != cudaSuccess) return UEPM_ERR_CUDA;
        for (int q = 0; q < 2 && !r; ++q) r = once();
        if (r) return r;
        if (cudaEventRecord(b, s) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
            set_error("uepm_ctx_autotune: timing failed");
            return UEPM_ERR_CUDA;
        }
        float f = 0.f;
        cudaEventElapsedTime(&f, a, b);
        *ms = f / 2.0;
        return UEPM_OK;
    };

    uepm_tuning best = uepm_tuning{};
    best.max_iter    = saved.max_iter;  // not a shape: kept as the caller set it
    best.tensor_cores = saved.tensor_cores;
    best.streams      = saved.streams;
    ctx->tune        = best;
    double best_ms   = 0;
    rc               = timed(&best_ms);
    // candidates per field, tried one field at a time from the current best
    const bool mixed = ctx->precision == UEPM_PREC_MIXED;
    const int  tmax  = ctx->real ? 32 : 24;
    const bool regok = mixed && ctx->real && ctx->n <= tridiag_reg_max_n();
    const int  es    = mixed ? (ctx->real ? 4 : 8) : (ctx->real ? 8 : 16);  // bytes of a reduced element
    std::vector<int> chunks, reds, ctas, lanes, clusters;
    for (int c : {256, 512, 1024, 2048, 4096, 8192})
        if ((size_t)c < sample_k) chunks.push_back(c);
    reds = mixed ? std::vector<int>{2, 3, 4, 5, 6} : std::vector<int>{2, 3};  // 4, 5, 6: FP32 only
    ctas = {1, 2, 4, 6, 8};
    for (int c : {2, 4, 8, 16})
        if ((size_t)es * ctx->n * ((ctx->n + c - 1) / c) <= (200u << 10)) clusters.push_back(c);
    if (mixed || wv || wg)
        for (int l : {8, 16, 32})
            if ((ctx->n + l - 1) / l <= tmax) lanes.push_back(l);
    auto field_of = [](uepm_tuning& t, int f) -> int32_t& {
        return f == 0 ? t.chunk : f == 1 ? t.reduction : f == 2 ? t.ctas_per_sm : f == 3 ? t.cluster : t.vector_lanes;
    };
    for (int field = 0; field < 5 && !rc; ++field) {
        std::vector<int> cand = field == 0 ? chunks : field == 1 ? reds : field == 2 ? ctas : field == 3 ? clusters : lanes;
        // ctas_per_sm matters only for the global-memory kernel, cluster only for the cluster kernel
        if (field == 2 && best.reduction == 3) continue;
        if (field == 3 && best.reduction != 3 && !(best.reduction == 0 && !ctx->real)) continue;
        for (int v : cand) {
            uepm_tuning t    = best;
            field_of(t, field) = v;
            ctx->tune        = t;
            double ms        = 0;
            if ((rc = timed(&ms))) break;
            if (ms < best_ms * 0.99) {  // keep a change only for a clear gain
                best_ms = ms;
                best    = t;
            }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx->profiling = prof;
    if (rc) {
        ctx->tune = saved;
        return rc;
    }
    ctx->tune = best;
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = best;
    return UEPM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
struct uepm_batch {
    struct Group {
        uepm_ctx*     ctx;
        const double* k;
        size_t        nk;
        int           nb;
        uint32_t      want;
        double *      E, *X, *grad;
        int32_t*      st;
    };
    std::vector<Group>        groups;
    bool                      graphs = true;
    int                       runs   = 0;  // eager runs since the last change
    cudaGraphExec_t           exec   = nullptr;
    uint64_t                  kernels = 0;
    std::vector<uepm_ctx*>    ctxs;    // distinct contexts, in order of first appearance
    std::vector<void*>        ws_ptr;  // their workspaces when the graph was captured
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t>  joins;
    cudaEvent_t               fork = nullptr;
    // the batch runs on its own origin stream, ordered after the caller's stream on entry and before
    // it on exit (a graph cannot be captured on the legacy default stream)
    cudaStream_t origin = nullptr;
    cudaEvent_t  in = nullptr, out = nullptr;

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        runs = 0;
    }
};

extern "C" {

int uepm_batch_create(uepm_batch** out) {
    if (!out) {
        set_error("uepm_batch_create: null argument");
        return UEPM_ERR_INVALID;
    }
    *out = new uepm_batch();
    return UEPM_OK;
}

void uepm_batch_destroy(uepm_batch* b) {
    if (!b) return;
    b->drop_graph();
    for (auto s : b->streams) cudaStreamDestroy(s);
    for (auto e : b->joins) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->in) cudaEventDestroy(b->in);
    if (b->out) cudaEventDestroy(b->out);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

int uepm_batch_add(uepm_batch* b, uepm_ctx* ctx, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E,
                   double* d_X, double* d_grad, int32_t* d_status) {
    if (!b || !ctx || (nk && (!d_k || !d_E))) {
        set_error("uepm_batch_add: null argument");
        return UEPM_ERR_INVALID;
    }
    if ((want & UEPM_WANT_VECTORS) && !d_X) {
        set_error("uepm_batch_add: UEPM_WANT_VECTORS without an X buffer");
        return UEPM_ERR_INVALID;
    }
    if ((want & UEPM_WANT_GRADIENT) && !d_grad) {
        set_error("uepm_batch_add: UEPM_WANT_GRADIENT without a gradient buffer");
        return UEPM_ERR_INVALID;
    }
    SolvePlan sp;
    int       rc = plan_solve(ctx, std::max<size_t>(nk, 1), nb, want, &sp);
    if (rc) return rc;
    b->groups.push_back({ctx, d_k, nk, nb, want, d_E, d_X, d_grad, d_status});
    b->drop_graph();
    return UEPM_OK;
}

int uepm_batch_clear(uepm_batch* b) {
    if (!b) {
        set_error("uepm_batch_clear: null batch");
        return UEPM_ERR_INVALID;
    }
    b->groups.clear();
    b->drop_graph();
    return UEPM_OK;
}

int uepm_batch_set_graph(uepm_batch* b, int on) {
    if (!b) {
        set_error("uepm_batch_set_graph: null batch");
        return UEPM_ERR_INVALID;
    }
    b->graphs = on != 0;
    b->drop_graph();
    return UEPM_OK;
}

uint64_t uepm_batch_kernels_per_run(const uepm_batch* b) { return b ? b->kernels : 0; }

int uepm_batch_run(uepm_batch* b, void* stream) {
    if (!b) {
        set_error("uepm_batch_run: null batch");
        return UEPM_ERR_INVALID;
    }
    if (b->groups.empty()) return UEPM_OK;
    const cudaStream_t user = (cudaStream_t)stream;
    if (!b->origin) {
        UEPM_CK(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
        UEPM_CK(cudaEventCreateWithFlags(&b->in, cudaEventDisableTiming));
        UEPM_CK(cudaEventCreateWithFlags(&b->out, cudaEventDisableTiming));
    }
    const cudaStream_t s = b->origin;
    // leaves the origin stream ordered before the caller's stream
    auto to_user = [&]() -> int {
        UEPM_CK(cudaEventRecord(b->out, s));
        UEPM_CK(cudaStreamWaitEvent(user, b->out, 0));
        return UEPM_OK;
    };

    // distinct contexts and the workspace each needs (the largest plan of its groups)
    std::vector<uepm_ctx*> ctxs;
    std::vector<int>       gctx(b->groups.size());
    std::vector<SolvePlan> plans(b->groups.size());
    std::vector<size_t>    need;
    for (size_t g = 0; g < b->groups.size(); ++g) {
        const auto& gr = b->groups[g];
        auto        it = std::find(ctxs.begin(), ctxs.end(), gr.ctx);
        if (it == ctxs.end()) {
            ctxs.push_back(gr.ctx);
            need.push_back(0);
            it = ctxs.end() - 1;
        }
        gctx[g] = (int)(it - ctxs.begin());
        int rc  = plan_solve(gr.ctx, std::max<size_t>(gr.nk, 1), gr.nb, gr.want, &plans[g]);
        if (rc) return rc;
        need[gctx[g]] = std::max(need[gctx[g]], plans[g].ws_bytes);
    }
    for (size_t c = 0; c < ctxs.size(); ++c) {
        int rc = ensure_workspace(ctxs[c], need[c]);
        if (rc) return rc;
    }
    UEPM_CK(cudaEventRecord(b->in, user));
    UEPM_CK(cudaStreamWaitEvent(s, b->in, 0));
    // replay while nothing changed
    if (b->exec) {
        bool same = ctxs == b->ctxs;
        for (size_t c = 0; same && c < ctxs.size(); ++c) same = ctxs[c]->d_ws == b->ws_ptr[c];
        if (same) {
            UEPM_CK(cudaGraphLaunch(b->exec, s));
            count_launch((int)b->kernels);
            return to_user();
        }
        b->drop_graph();
    }
    while (b->streams.size() < ctxs.size()) {
        cudaStream_t st;
        cudaEvent_t  ev;
        UEPM_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        UEPM_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->streams.push_back(st);
        b->joins.push_back(ev);
    }
    if (!b->fork) UEPM_CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));

    const bool capture = b->graphs && b->runs >= 1;
    // per-kernel profiling records events that a graph cannot replay: off while capturing
    std::vector<int> prof(ctxs.size());
    for (size_t c = 0; c < ctxs.size(); ++c) {
        prof[c] = ctxs[c]->profiling;
        if (capture) ctxs[c]->profiling = 0;
    }
    auto restore = [&]() {
        for (size_t c = 0; c < ctxs.size(); ++c) ctxs[c]->profiling = prof[c];
    };
    if (capture && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        restore();
        set_error("uepm_batch_run: stream capture could not begin");
        return UEPM_ERR_CUDA;
    }
    const uint64_t l0 = launches_total();
    int            rc = UEPM_OK;
    if (cudaEventRecord(b->fork, s) != cudaSuccess) rc = UEPM_ERR_CUDA;
    for (size_t c = 0; !rc && c < ctxs.size(); ++c)
        if (cudaStreamWaitEvent(b->streams[c], b->fork, 0) != cudaSuccess) rc = UEPM_ERR_CUDA;
    // groups enqueued by estimated cost, largest first (the reduction's n^3 per k-point, 4x for
    // complex matrices), so that the longest pipelines start first and the cheap ones fill in behind
    // them (longest-processing-time order); each group's results do not depend on the order
    std::vector<size_t> order(b->groups.size());
    for (size_t g = 0; g < order.size(); ++g) order[g] = g;
    auto cost = [&](size_t g) {
        const auto&  gr = b->groups[g];
        const double n  = (double)gr.ctx->n;
        return n * n * n * (double)gr.nk * (gr.ctx->real ? 1.0 : 4.0);
    };
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost(x) > cost(y); });
    for (size_t q = 0; !rc && q < order.size(); ++q) {
        const size_t g  = order[q];
        const auto&  gr = b->groups[g];
        rc = enqueue_solve(gr.ctx, plans[g], gr.k, gr.nk, gr.nb, gr.want, gr.E, gr.X, gr.grad, gr.st, b->streams[gctx[g]]);
    }
    for (size_t c = 0; !rc && c < ctxs.size(); ++c) {
        if (cudaEventRecord(b->joins[c], b->streams[c]) != cudaSuccess || cudaStreamWaitEvent(s, b->joins[c], 0) != cudaSuccess)
            rc = UEPM_ERR_CUDA;
    }
    const uint64_t enq = launches_total() - l0;
    if (!capture) {
        restore();
        if (rc == UEPM_ERR_CUDA) set_error("uepm_batch_run: fork/join on the batch streams failed");
        if (!rc) {
            b->kernels = enq;
            b->runs += 1;
        }
        const int rj = to_user();
        return rc ? rc : rj;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &graph);
    restore();
    uncount_launches(enq);  // captured, not launched
    if (rc || ec != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (!rc) set_error(std::string("uepm_batch_run: capture failed: ") + cudaGetErrorString(ec));
        return rc ? rc : UEPM_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        b->exec = nullptr;
        set_error(std::string("uepm_batch_run: graph instantiation failed: ") + cudaGetErrorString(ei));
        return UEPM_ERR_CUDA;
    }
    b->kernels = enq;
    b->ctxs    = ctxs;
    b->ws_ptr.clear();
    for (auto c : ctxs) b->ws_ptr.push_back(c->d_ws);
    UEPM_CK(cudaGraphLaunch(b->exec, s));
    count_launch((int)b->kernels);
    return to_user();
}

}  // extern "C"
