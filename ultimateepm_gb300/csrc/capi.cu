// capi.cu -- the C ABI (include/uepm_gb300.h): context set-up, device workspace and the batched
// solve pipeline over chunks of k-points.
//
// Pipeline per chunk (all on one stream, no host round trips; in a two-lane solve consecutive chunks
// alternate between the caller's stream and the context's second stream):
//   FP64  k_rows -> k_assemble -> k_tridiag<double> -> k_bisect<double> (writes E in place)
//         [-> k_invit<double> -> k_backtransform<double> (X, gradient)]
//   MIXED k_rows -> k_assemble (FP64 + FP32 copy) -> k_tridiag<float> -> k_bisect<float>
//         -> k_invit<float> -> k_backtransform<float> -> k_refine (FP64 Rayleigh-Ritz: E, X, gradient)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "ctx_internal.h"
#include "ctx_view.h"
#include "uepm_common.cuh"
#include "uepm_gb300.h"
#include "uepm_kernels.h"

namespace uepm {

static thread_local std::string g_last_error;
static std::atomic<uint64_t>    g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }
void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
uint64_t launches_total() { return g_launches.load(); }
void     uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

// src/Common/physical_constants.hpp:18-44
namespace pc {
constexpr double h           = 6.62607015e-34;
constexpr double q_e         = 1.602176634e-19;
constexpr double pi          = 3.141592653589793238462643383279502884;
constexpr double h_bar       = h / (2.0 * pi);
constexpr double m_e         = 9.1093837015e-31;
constexpr double bohr_radius = 5.29177210903e-11;
}  // namespace pc

constexpr int kMaxOrder   = 512;  // largest matrix order n the kernels are instantiated for
constexpr int kGuardBands = 4;    // extra FP32 bands kept in the mixed-precision subspace
constexpr size_t kMaxChunk = 32768;  // k-points per launch: the assembly grid's z extent is <= 65535

}  // namespace uepm

using namespace uepm;

namespace uepm {
bool ctx_tables(const uepm_ctx* ctx, CtxTables* out) {
    if (!ctx || !out) return false;
    out->P    = ctx->P;
    out->d_G  = ctx->d_G;
    out->Vloc = ctx->d_Vloc;
    out->phNL = ctx->d_phNL;
    out->phSO = ctx->d_phSO;
    out->N    = ctx->N;
    out->n    = ctx->n;
    return true;
}
}  // namespace uepm

namespace {

enum KernelKind {
    KK_ROWS = 0,
    KK_ASSEMBLE,
    KK_TRIDIAG64,
    KK_TRIDIAG32,
    KK_BISECT,
    KK_INVIT,
    KK_BACKTRANSFORM,
    KK_REFINE_PROJECT,
    KK_SMALL_EIGH,
    KK_REFINE_VECTORS
};
const char* kKernelNames[UEPM_KERNEL_KINDS] = {"rows",   "assemble",      "tridiag_fp64",   "tridiag_fp32", "bisect",
                                               "invit",  "backtransform", "refine_project", "small_eigh",   "refine_vectors"};

cudaEvent_t take_event(uepm_ctx* ctx) {
    if (!ctx->pool.empty()) {
        cudaEvent_t e = ctx->pool.back();
        ctx->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets the kernels launched in its scope with events on `s` when profiling is on, tagged with
// the context's current pass (prof_group).
struct ProfScope {
    uepm_ctx*    ctx;
    cudaStream_t s;
    int          kind;
    unsigned     group;
    cudaEvent_t  a = nullptr;
    ProfScope(uepm_ctx* c, cudaStream_t st, int k) : ctx(c), s(st), kind(k), group(c->prof_group) {
        if (ctx->profiling) {
            a = take_event(ctx);
            cudaEventRecord(a, s);
        }
    }
    ~ProfScope() {
        if (ctx->profiling && a) {
            cudaEvent_t b = take_event(ctx);
            cudaEventRecord(b, s);
            ctx->pending.push_back({kind, group, a, b});
        }
    }
};

}  // namespace

#define UEPM_CUDA(call)                                                                                   \
    do {                                                                                                  \
        cudaError_t err_ = (call);                                                                        \
        if (err_ != cudaSuccess) {                                                                        \
            set_error(std::string(#call) + ": " + cudaGetErrorString(err_));                              \
            return UEPM_ERR_CUDA;                                                                         \
        }                                                                                                 \
    } while (0)

namespace {

// Pseudopotential::GetValue (src/EPP/Pseudopotential.cpp:24-56), same operand order, glibc cos/sin.
void pp_value(const uepm_material& m, int gx, int gy, int gz, double tau, double a, double* re, double* im) {
    const int    G2   = gx * gx + gy * gy + gz * gz;
    const double kfac = 2.0 * pc::pi / a;
    const double Gtau = kfac * (tau * gx + tau * gy + tau * gz);
    double       VS = 0.0, VA = 0.0;
    switch (G2) {
        case 3: VS = m.V3S; VA = m.V3A; break;
        case 4: VS = m.V4S; VA = m.V4A; break;
        case 8: VS = m.V8S; VA = m.V8A; break;
        case 11: VS = m.V11S; VA = m.V11A; break;
        default: break;
    }
    *re = VS * std::cos(Gtau);
    *im = VA * std::sin(Gtau);
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

struct Layout {
    size_t rows, rows32, H, H32, d, e, tq, ev, work, z, X32, refine, small, total;
};

// Bytes of workspace one chunk of `c` matrices needs, with the offset of every region.
Layout plan(const uepm_ctx* ctx, int nb, uint32_t want, size_t c) {
    const size_t n = ctx->n, N = ctx->N;
    const bool   mixed = ctx->precision == UEPM_PREC_MIXED;
    const bool   vecs  = (want & (UEPM_WANT_VECTORS | UEPM_WANT_GRADIENT)) != 0;
    const size_t m     = mixed ? std::min<size_t>(n, (size_t)nb + kGuardBands) : (size_t)nb;
    const size_t es    = ctx->real ? sizeof(double) : sizeof(cx<double>);  // FP64 matrix scalar
    const size_t es32  = ctx->real ? sizeof(float) : sizeof(cx<float>);   // FP32 matrix scalar
    const size_t rs    = mixed ? sizeof(float) : sizeof(double);           // real type of the reduction
    Layout       L{};
    size_t       off = 0;
    auto         take = [&](size_t bytes) {
        const size_t o = off;
        off            = align_up(off + bytes);
        return o;
    };
    L.rows   = take(c * N * ROW_STRIDE * sizeof(double));
    L.rows32 = (mixed && (ctx->ds_nl || ctx->ds_soc)) ? take(c * N * ROW_STRIDE * sizeof(float2)) : 0;
    L.H    = take(mixed && ctx->sparse_local ? 0 : c * n * n * es);  // the sparse path never forms it
    L.H32  = mixed ? take(c * n * n * es32) : 0;
    L.d    = take(c * n * rs);
    L.e    = take(c * n * rs);
    L.tq   = take(c * n * (mixed ? es32 : es));
    L.ev   = mixed ? take(c * m * rs) : 0;
    if (mixed || vecs) {
        L.work = take(c * invit_work_elems<double>((int)n) * rs);
        L.z    = take(c * m * n * rs);
    }
    if (mixed) {
        L.X32    = take(c * m * n * sizeof(cx<float>));
        L.refine = take(c * refine_work_elems((int)n, (int)m) * es);
        L.small  = take(c * refine_small_elems((int)m, nb) * es);
    }
    L.total = off;
    return L;
}

int ensure_ws(uepm_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->ws_bytes) return UEPM_OK;
    if (ctx->d_ws) cudaFree(ctx->d_ws);
    ctx->d_ws     = nullptr;
    ctx->ws_bytes = 0;
    if (cudaMalloc(&ctx->d_ws, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("device workspace allocation of " + std::to_string(bytes) + " bytes failed");
        return UEPM_ERR_NOMEM;
    }
    ctx->ws_bytes = bytes;
    return UEPM_OK;
}

int check_launch() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("kernel launch failed: ") + cudaGetErrorString(e));
        return UEPM_ERR_CUDA;
    }
    return UEPM_OK;
}


// One chunk of c k-points through the pipeline, FP64 (S = double for real H, cx<double> otherwise)
// or mixed precision (FP32 reduction in Lower<S>, FP64 Rayleigh-Ritz in S).
template <typename S>
void run_chunk(uepm_ctx* ctx, const Layout& L, char* ws, const double* kk, int c, int nb, int m, bool vec, double* E,
               cx<double>* Xo, double* gr, int* st, cudaStream_t s) {
    using S32            = typename Lower<S>::type;
    const int    n       = ctx->n;
    const size_t mstride = (size_t)n * n;
    auto*        rows    = reinterpret_cast<double*>(ws + L.rows);
    auto*        H       = reinterpret_cast<S*>(ws + L.H);
    const bool   ds_asm  = ctx->precision == UEPM_PREC_MIXED && (ctx->ds_nl || ctx->ds_soc);
    auto*        rows32  = ds_asm ? reinterpret_cast<float2*>(ws + L.rows32) : nullptr;
    {
        ProfScope p(ctx, s, KK_ROWS);
        launch_rows(ctx->P, kk, ctx->d_G, rows, c, s, rows32);
    }
    if (ctx->precision != UEPM_PREC_MIXED) {
        {
            ProfScope p(ctx, s, KK_ASSEMBLE);
            launch_assemble<S>(ctx->P, ctx->d_Vloc, ctx->d_phNL, ctx->d_phSO, rows, H, n, mstride, nullptr, 0, c, s);
        }
        auto* d  = reinterpret_cast<double*>(ws + L.d);
        auto* e  = reinterpret_cast<double*>(ws + L.e);
        auto* tq = reinterpret_cast<S*>(ws + L.tq);
        {
            ProfScope p(ctx, s, KK_TRIDIAG64);
            launch_tridiag<S>(H, n, n, mstride, d, e, tq, st, c, s, ctx->tune.reduction, ctx->tune.ctas_per_sm,
                              ctx->tune.cluster);
        }
        {
            ProfScope p(ctx, s, KK_BISECT);
            launch_bisect<double>(d, e, n, nb, E, nb, c, s, ctx->tune.max_iter, st);
        }
        if (vec) {
            auto* work = reinterpret_cast<double*>(ws + L.work);
            auto* z    = reinterpret_cast<double*>(ws + L.z);
            {
                ProfScope p(ctx, s, KK_INVIT);
                launch_invit<double>(d, e, E, nb, n, nb, work, z, st, c, s, ctx->tune.max_iter);
            }
            ProfScope p(ctx, s, KK_BACKTRANSFORM);
            launch_backtransform<S>(H, n, n, mstride, tq, z, nb, Xo, ctx->P, kk, ctx->d_G, gr, c, s, ctx->tune.vector_lanes);
        }
        return;
    }
    using SP  = typename Split<S>::type;
    auto* H32 = reinterpret_cast<S32*>(ws + L.H32);
    auto* Hs  = reinterpret_cast<SP*>(ws + L.H);
    // Real local-potential matrices reduced in registers: the reduction forms H(k) itself from the
    // resident V and the kinetic diagonal (the same FP32 values), so nothing is assembled.
    constexpr bool kReal32 = std::is_same<S32, float>::value;
    const bool     reg_local = kReal32 && ctx->sparse_local && (ctx->tune.reduction == 0 || ctx->tune.reduction == 1) &&
                           n <= tridiag_reg_max_n();
    if (!reg_local) {
        ProfScope p(ctx, s, KK_ASSEMBLE);
        // the FP64 matrix is kept only for the Rayleigh-Ritz products: stored as FP32 pairs in place;
        // with a local potential only, those products use the resident sparse V instead
        if (ctx->sparse_local)
            launch_assemble<S32>(ctx->P, ctx->d_Vloc, ctx->d_phNL, ctx->d_phSO, rows, H32, n, mstride, nullptr, 0, c, s);
        else if (ds_asm && ctx->ds_soc) {
            if constexpr (std::is_same<SP, ds4>::value)
                launch_assemble_soc_ds<SP>(ctx->P, ctx->Q, ctx->d_Vloc32, ctx->d_phNL32, ctx->d_phSO32, rows32, ctx->d_Vloc,
                                           ctx->d_phNL, ctx->d_phSO, rows, Hs, n, mstride, H32, mstride, c, s);
        } else if (ds_asm)
            launch_assemble_ds<SP>(ctx->P, ctx->Q, ctx->d_Vloc32, ctx->d_phNL32, rows32, ctx->d_Vloc, ctx->d_phNL, rows, Hs, n,
                                   mstride, H32, mstride, c, s);
        else
            launch_assemble<SP>(ctx->P, ctx->d_Vloc, ctx->d_phNL, ctx->d_phSO, rows, Hs, n, mstride, H32, mstride, c, s);
    }
    auto* d     = reinterpret_cast<float*>(ws + L.d);
    auto* e     = reinterpret_cast<float*>(ws + L.e);
    auto* tq    = reinterpret_cast<S32*>(ws + L.tq);
    auto* ev    = reinterpret_cast<float*>(ws + L.ev);
    auto* work  = reinterpret_cast<float*>(ws + L.work);
    auto* z     = reinterpret_cast<float*>(ws + L.z);
    auto* X32   = reinterpret_cast<cx<float>*>(ws + L.X32);
    auto* rw    = reinterpret_cast<S*>(ws + L.refine);
    auto* small = reinterpret_cast<S*>(ws + L.small);
    {
        ProfScope p(ctx, s, KK_TRIDIAG32);
        if constexpr (kReal32) {
            if (reg_local)
                launch_tridiag_reg_local(ctx->d_V32, ctx->d_Vloc, rows, H32, n, n, mstride, d, e, tq, st, c, s);
            else
                launch_tridiag<S32>(H32, n, n, mstride, d, e, tq, st, c, s, ctx->tune.reduction, ctx->tune.ctas_per_sm,
                                    ctx->tune.cluster);
        } else {
            launch_tridiag<S32>(H32, n, n, mstride, d, e, tq, st, c, s, ctx->tune.reduction, ctx->tune.ctas_per_sm,
                                ctx->tune.cluster, ctx->tune.tensor_cores == 0);
        }
    }
    {
        ProfScope p(ctx, s, KK_BISECT);
        launch_bisect<float>(d, e, n, m, ev, m, c, s, ctx->tune.max_iter, st);
    }
    {
        ProfScope p(ctx, s, KK_INVIT);
        launch_invit<float>(d, e, ev, m, n, m, work, z, st, c, s, ctx->tune.max_iter);
    }
    {
        ProfScope p(ctx, s, KK_BACKTRANSFORM);
        launch_backtransform<S32>(H32, n, n, mstride, tq, z, m, X32, ctx->P, kk, ctx->d_G, nullptr, c, s,
                                  ctx->tune.vector_lanes);
    }
    {
        ProfScope p(ctx, s, KK_REFINE_PROJECT);
        const SparseV sv{ctx->sparse_local, ctx->ell_w,  ctx->d_ell_col, ctx->d_ell_re,
                         ctx->d_ell_im,       ctx->d_Vloc, rows,            ctx->N};
        launch_refine_project<S>(Hs, n, n, mstride, X32, m, rw, small, c, s, sv, st, ctx->tune.tensor_cores == 0);
    }
    S* W = small + (size_t)2 * m * m;  // W block of the first matrix; matrices are refine_small_elems apart
    {
        ProfScope p(ctx, s, KK_SMALL_EIGH);
        launch_small_eigh<S>(small, m, nb, E, vec ? W : nullptr, st, c, s, ctx->tune.max_iter);
    }
    if (vec) {
        ProfScope p(ctx, s, KK_REFINE_VECTORS);
        launch_refine_vectors<S>(n, m, nb, X32, W, Xo, gr, ctx->P, kk, ctx->d_G, c, s);
    }
}

}  // namespace

namespace uepm {

int ensure_workspace(uepm_ctx* ctx, size_t bytes) { return ensure_ws(ctx, bytes); }

// Two lanes: a mixed solve's reduction holds the SMs' registers or shared memory, and the kernels
// after it (bisection, inverse iteration, the Rayleigh-Ritz products and the small solves) are bound
// by the latency of short per-matrix chains. Splitting the batch over two streams lets one half's
// later kernels run beside the other half's reduction. Per solve, one lane against two: Si local
// n = 137 (register-resident reduction), 2000 k, 16 bands: 2.00 -> 1.89 ms (three and four lanes no
// faster); 12 bands, Si nonlocal n = 137, 65536 k: 100.8 -> 100.0 ms; InP n = 113 complex: 158.5 ->
// 155.9; Ge n = 181 real, 32768 k: 151.2 -> 149.2; Ge SOC n = 362, 16 bands, 4000 k: 113.7 -> 111.0
// (each half in one pass of its own). Results are the same bits (every k-point is solved on its own).
// FP64 solves keep one stream: two measured 12.5 -> 12.9 ms (Si local, 2000 k), 601.7 -> 604.4 (Ge
// SOC, 2000 k) and 138.5 -> 131.4 (Ge n = 181 real, 8000 k), no gain overall.
constexpr size_t kLaneMinK = 1024;
static bool lanes_pay(const uepm_ctx* ctx, size_t nk) { return ctx->precision == UEPM_PREC_MIXED && nk >= kLaneMinK; }

int plan_solve(uepm_ctx* ctx, size_t nk, int nb, uint32_t want, SolvePlan* out, bool two_lanes) {
    if (nb < 1 || nb > ctx->n) {
        set_error("nb must be in [1, n]");
        return UEPM_ERR_OUT_OF_RANGE;
    }
    const bool mixed = ctx->precision == UEPM_PREC_MIXED;
    const int  n     = ctx->n;
    const int  m     = mixed ? std::min(n, nb + kGuardBands) : nb;
    if (mixed && m > kRefineMaxSubspace) {
        set_error("mixed precision supports at most " + std::to_string(kRefineMaxSubspace - kGuardBands) + " bands");
        return UEPM_ERR_INVALID;
    }
    // chunk size from the workspace budget and the tuning
    const size_t per    = plan(ctx, nb, want, 1).total;
    const size_t budget = std::max<size_t>(1, ctx->ws_limit / std::max<size_t>(per, 1));
    const size_t cap    = ctx->tune.chunk > 0 ? std::min<size_t>((size_t)ctx->tune.chunk, kMaxChunk) : kMaxChunk;
    size_t       chunk  = std::max<size_t>(1, std::min(std::min(budget, nk), cap));
    // automatic: two lanes where the batch fits one pass, whose halves then run side by side (a
    // batch of several passes keeps whole passes: halving them measured 1 % slower on 500 000 and
    // 1 000 000 k, Si nonlocal n = 137 and Ge SOC n = 362)
    const int want_l = ctx->tune.streams;  // 0 automatic, 1 or 2
    out->lanes = two_lanes && (want_l == 2 ? nk >= 2 : want_l == 0 && lanes_pay(ctx, nk) && nk <= chunk) ? 2 : 1;
    // two lanes: each lane's chunk within half the workspace budget, the tuned chunk, and half the
    // batch (so that both lanes have work)
    if (out->lanes == 2) chunk = std::max<size_t>(1, std::min(std::min(budget / 2, cap), (nk + 1) / 2));
    out->chunk    = chunk;
    out->m        = m;
    out->ws_bytes = out->lanes * plan(ctx, nb, want, chunk).total;
    return UEPM_OK;
}

int enqueue_solve(uepm_ctx* ctx, const SolvePlan& sp, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E,
                  double* d_X, double* d_grad, int32_t* d_status, cudaStream_t s, void* ws_ext, size_t ws_ext_bytes) {
    if (nk == 0) return UEPM_OK;
    if ((ws_ext ? ws_ext_bytes : ctx->ws_bytes) < sp.ws_bytes) {
        set_error("enqueue_solve: workspace smaller than the plan");
        return UEPM_ERR_RUNTIME;
    }
    const int    n     = ctx->n;
    const size_t chunk = sp.chunk;
    const Layout L     = plan(ctx, nb, want, chunk);
    char*        ws    = static_cast<char*>(ws_ext ? ws_ext : ctx->d_ws);
    if (d_status) UEPM_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int32_t) * nk, s));
    const bool   want_vec  = (want & UEPM_WANT_VECTORS) != 0;
    const bool   want_grad = (want & UEPM_WANT_GRADIENT) != 0;
    const int    lanes     = sp.lanes == 2 ? 2 : 1;
    cudaStream_t ls[2]     = {s, s};
    bool         forked    = false;
    if (lanes == 2) {  // fork: the second lane starts after everything enqueued on s so far
        if (!ctx->lane_stream) {
            // the stream and events are made outside stream capture only; a capture that meets
            // none runs both lanes' chunks in order on s (same workspace halves, same results)
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusActive;
            if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
                cudaGetLastError();
                cs = cudaStreamCaptureStatusActive;
            }
            if (cs == cudaStreamCaptureStatusNone) {
                UEPM_CUDA(cudaStreamCreateWithFlags(&ctx->lane_stream, cudaStreamNonBlocking));
                UEPM_CUDA(cudaEventCreateWithFlags(&ctx->lane_fork, cudaEventDisableTiming));
                UEPM_CUDA(cudaEventCreateWithFlags(&ctx->lane_join, cudaEventDisableTiming));
            }
        }
        if (ctx->lane_stream) {
            UEPM_CUDA(cudaEventRecord(ctx->lane_fork, s));
            UEPM_CUDA(cudaStreamWaitEvent(ctx->lane_stream, ctx->lane_fork, 0));
            ls[1] = ctx->lane_stream;
            forked = true;
        }
    }
    int rc = UEPM_OK;
    for (size_t off = 0, q = 0; off < nk; off += chunk, ++q) {
        const int          lane = (int)(q % lanes);
        const cudaStream_t sq   = ls[lane];
        char*              wsq  = ws + lane * L.total;
        if (lane == 0) ++ctx->prof_group;  // the chunks of both lanes of one pass share a group
        const int     c  = (int)std::min(chunk, nk - off);
        const double* kk = d_k + 3 * off;
        int*          st = d_status ? d_status + off : nullptr;
        double*       E  = d_E + off * nb;
        cx<double>*   Xo = want_vec ? reinterpret_cast<cx<double>*>(d_X) + off * nb * n : nullptr;
        double*       gr = want_grad ? d_grad + off * nb * 3 : nullptr;
        if (ctx->real) run_chunk<double>(ctx, L, wsq, kk, c, nb, sp.m, want_vec || want_grad, E, Xo, gr, st, sq);
        else run_chunk<cx<double>>(ctx, L, wsq, kk, c, nb, sp.m, want_vec || want_grad, E, Xo, gr, st, sq);
        if ((rc = check_launch())) break;
    }
    if (forked) {  // join (also after a failed launch): work enqueued on s later waits for the second lane
        UEPM_CUDA(cudaEventRecord(ctx->lane_join, ctx->lane_stream));
        UEPM_CUDA(cudaStreamWaitEvent(s, ctx->lane_join, 0));
    }
    return rc;
}

}  // namespace uepm

extern "C" {

int uepm_version(void) { return 10000; }
const char* uepm_last_error(void) { return g_last_error.c_str(); }
uint64_t uepm_kernel_launches(void) { return g_launches.load(); }

int uepm_ctx_create(const uepm_material* mat, const int32_t* G, int N, uint32_t flags, uepm_ctx** out) {
    if (!mat || !G || !out || N <= 0) {
        set_error("uepm_ctx_create: null argument or empty basis");
        return UEPM_ERR_INVALID;
    }
    const bool soc = (flags & UEPM_SOC) != 0, nl = (flags & UEPM_NONLOCAL) != 0;
    const int  n   = soc ? 2 * N : N;
    if (n > kMaxOrder) {
        set_error("matrix order " + std::to_string(n) + " exceeds the supported maximum " + std::to_string(kMaxOrder));
        return UEPM_ERR_INVALID;
    }
    if (soc && (mat->period_cation < 2 || mat->period_cation > 4)) {
        set_error("SpinOrbitCorrection::compute_lambda_1: Unsupported period for cation.");
        return UEPM_ERR_RUNTIME;
    }
    if (soc && (mat->period_anion < 2 || mat->period_anion > 4)) {
        set_error("SpinOrbitCorrection::compute_lambda_2: Unsupported period for anion.");
        return UEPM_ERR_RUNTIME;
    }
    auto* ctx  = new uepm_ctx();
    ctx->mat   = *mat;
    ctx->N     = N;
    ctx->n     = n;
    ctx->flags = flags;
    ctx->G.assign(G, G + 3 * (size_t)N);
    // H(k) is exactly real when nothing contributes an imaginary part: no spin-orbit blocks, no
    // antisymmetric local form factors (VA * sin = 0), and a nonlocal term whose antisymmetric part
    // (V_anion - V_cation) / 2 vanishes identically because both atoms carry the same parameters.
    const bool same_nl = !nl || (mat->alpha0_anion == mat->alpha0_cation && mat->beta0_anion == mat->beta0_cation &&
                                 mat->A2_anion == mat->A2_cation && mat->R0_anion == mat->R0_cation &&
                                 mat->R2_anion == mat->R2_cation);
    ctx->real_h = !soc && mat->V3A == 0.0 && mat->V4A == 0.0 && mat->V8A == 0.0 && mat->V11A == 0.0 && same_nl;
    ctx->real   = ctx->real_h;
    cudaGetDevice(&ctx->device);

    // Derived constants, each with the reference's own expression.
    const double a             = 1.0e-10 * mat->lattice_constant;          // Material.h:108-111
    const double two_pi_over_a = 2.0 * M_PI / a;                           // Hamiltonian.cpp:56
    const double diag_factor   = (pc::h_bar * pc::h_bar) / (2.0 * pc::m_e * pc::q_e);
    DevParams&   P             = ctx->P;
    P.N            = N;
    P.n            = n;
    P.nl           = nl ? 1 : 0;
    P.soc          = soc ? 1 : 0;
    P.square       = (mat->nl_well == 1) ? 1 : 0;
    P.kin_pref     = two_pi_over_a * two_pi_over_a * diag_factor;
    P.grad_pref    = 2.0 * diag_factor * (two_pi_over_a * two_pi_over_a);  // Hamiltonian.cpp:167
    P.frac_to_phys = 1.0 / two_pi_over_a;
    const double volume = (1.0 / 8.0) * pow(a, 3.0);                     // Material.h:130
    const double kF     = pow(96 * M_PI * M_PI, 1.0 / 3.0) / a;           // Material.h:170
    P.ff      = 2.0 * M_PI / a;
    P.nl_df   = pow(pc::h_bar, 2) / (2.0 * pc::m_e * pc::q_e);
    P.Vpre    = 4.0 * M_PI / volume;
    P.kF2     = pow(kF, 2.0);
    P.alpha0a = mat->alpha0_anion;
    P.beta0a  = mat->beta0_anion;
    P.A2a     = mat->A2_anion;
    P.alpha0c = mat->alpha0_cation;
    P.beta0c  = mat->beta0_cation;
    P.A2c     = mat->A2_cation;
    P.R0a     = mat->R0_anion;
    P.R0c     = mat->R0_cation;
    P.R2a     = mat->R2_anion;
    P.R2c     = mat->R2_cation;
    P.has_R0a = (mat->R0_anion != 0.0);
    P.has_R0c = (mat->R0_cation != 0.0);
    P.has_A2a = (mat->A2_anion != 0.0);
    P.has_A2c = (mat->A2_cation != 0.0);
    P.same_nl = same_nl ? 1 : 0;
    P.R0a2 = pow(P.R0a, 2.0);
    P.R0c2 = pow(P.R0c, 2.0);
    P.R2a2 = pow(P.R2a, 2.0);
    P.R2c2 = pow(P.R2c, 2.0);
    P.R0a3h = pow(P.R0a, 3.0) / (2.0);
    P.R0c3h = pow(P.R0c, 3.0) / (2.0);
    P.R2a3h = pow(P.R2a, 3.0) / (2.0);
    P.R2c3h = pow(P.R2c, 3.0) / (2.0);
    P.R0a3t = pow(P.R0a, 3.0) / (3.0);
    P.R0c3t = pow(P.R0c, 3.0) / (3.0);
    P.gpre_a = 5.0 * pow(M_PI, 1.5) * (pow(P.R2a, 3.0) / volume);
    P.gpre_c = 5.0 * pow(M_PI, 1.5) * (pow(P.R2c, 3.0) / volume);
    P.pa        = mat->period_anion;
    P.pc        = mat->period_cation;
    P.ra        = mat->radial_extent_anion;
    P.rc        = mat->radial_extent_cation;
    P.alpha_soc = mat->alpha_soc;
    P.mu_soc    = mat->mu_soc;
    P.kfac      = (2.0 * M_PI) / a;
    P.bohr      = pc::bohr_radius;

    // k-independent tables: local form factors (SetConstantNonDiagonalMatrix, Hamiltonian.cpp:32-48)
    // and the structure phases of the nonlocal and spin-orbit terms.
    const double         tau = (1.0 / 8.0) * a;
    std::vector<double2> V((size_t)N * N), phNL, phSO;
    if (nl) phNL.resize((size_t)N * N);
    if (soc) phSO.resize((size_t)N * N);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const int dx = G[3 * i] - G[3 * j], dy = G[3 * i + 1] - G[3 * j + 1], dz = G[3 * i + 2] - G[3 * j + 2];
            double    re, im;
            pp_value(*mat, dx, dy, dz, tau, a, &re, &im);
            V[(size_t)j * N + i] = make_double2(re, im);
            if (nl) {
                // Material.cpp:202-205: 2 pi (tau / a).(G_i - G_j), with tau / a = 1/8 exactly
                const double ta = tau / a;
                const double Gt = ta * (double)dx + ta * (double)dy + ta * (double)dz;
                phNL[(size_t)j * N + i] = make_double2(cos(2.0 * M_PI * Gt), sin(2.0 * M_PI * Gt));
            }
            if (soc) {
                // SpinOrbitFunctional.cpp:132: kfac * (tau . (G - G'))
                const double g = P.kfac * (tau * (double)dx + tau * (double)dy + tau * (double)dz);
                phSO[(size_t)j * N + i] = make_double2(std::cos(g), std::sin(g));
            }
        }
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        uepm_ctx_destroy(ctx);
        return UEPM_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&ctx->d_G, sizeof(int) * 3 * N)) != cudaSuccess) return fail(e, "cudaMalloc(G)");
    if ((e = cudaMemcpy(ctx->d_G, G, sizeof(int) * 3 * N, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "copy G");
    if ((e = cudaMalloc(&ctx->d_Vloc, sizeof(double2) * V.size())) != cudaSuccess) return fail(e, "cudaMalloc(V)");
    if ((e = cudaMemcpy(ctx->d_Vloc, V.data(), sizeof(double2) * V.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "copy V");
    if (nl) {
        if ((e = cudaMalloc(&ctx->d_phNL, sizeof(double2) * phNL.size())) != cudaSuccess) return fail(e, "cudaMalloc(phNL)");
        if ((e = cudaMemcpy(ctx->d_phNL, phNL.data(), sizeof(double2) * phNL.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "copy phNL");
    }
    ctx->ds_nl  = nl && !soc && (P.has_R0a || P.has_R0c || P.has_A2a || P.has_A2c);
    ctx->ds_soc = soc;
    if (ctx->ds_nl || ctx->ds_soc) {
        // the nonlocal constants and the k-independent tables as FP32 pairs; products the FP64
        // element forms first are formed here in FP64, in the same order
        DevParamsDS& Q = ctx->Q;
        Q.has_R0a      = P.has_R0a;
        Q.has_R0c      = P.has_R0c;
        Q.has_A2a      = P.has_A2a;
        Q.has_A2c      = P.has_A2c;
        Q.same_nl      = P.same_nl;
        Q.kF2          = ds_of_double(P.kF2);
        Q.alpha0a      = ds_of_double(P.alpha0a);
        Q.nl_df_beta0a = ds_of_double(P.nl_df * P.beta0a);
        Q.alpha0c      = ds_of_double(P.alpha0c);
        Q.beta0c_nl_df = ds_of_double(P.beta0c * P.nl_df);
        Q.A2a_5        = ds_of_double(P.A2a * 5);
        Q.A2c_5        = ds_of_double(P.A2c * 5);
        Q.VR0a2s       = ds_of_double(P.Vpre * P.R0a2 / P.ff);
        Q.VR0c2s       = ds_of_double(P.Vpre * P.R0c2 / P.ff);
        Q.VR2a2s       = ds_of_double(P.Vpre * P.R2a2 / P.ff);
        Q.VR2c2s       = ds_of_double(P.Vpre * P.R2c2 / P.ff);
        Q.VR0a3h       = ds_of_double(P.Vpre * P.R0a3h);
        Q.VR0c3h       = ds_of_double(P.Vpre * P.R0c3h);
        Q.VR2a3h       = ds_of_double(P.Vpre * P.R2a3h);
        Q.VR2c3h       = ds_of_double(P.Vpre * P.R2c3h);
        Q.VR0a3t       = ds_of_double(P.Vpre * P.R0a3t);
        Q.VR0c3t       = ds_of_double(P.Vpre * P.R0c3t);
        Q.square       = P.square;
        Q.gA2a         = ds_of_double(P.gpre_a * P.A2a);
        Q.gA2c         = ds_of_double(P.gpre_c * P.A2c);
        Q.R2a2h        = ds_of_double(0.5 * (P.R2a * P.R2a));
        Q.R2c2h        = ds_of_double(0.5 * (P.R2c * P.R2c));
        Q.mu_soc       = ds_of_double(P.mu_soc);
        Q.alpha_mu_soc = ds_of_double(P.alpha_soc * P.mu_soc);
        auto pairs4 = [](const std::vector<double2>& src) {
            std::vector<float4> out(src.size());
            for (size_t q = 0; q < src.size(); ++q) {
                const ds a = ds_of_double(src[q].x), b = ds_of_double(src[q].y);
                out[q]     = make_float4(a.h, a.l, b.h, b.l);
            }
            return out;
        };
        auto upload = [&](float4** dst, const std::vector<float4>& v, const char* what) -> cudaError_t {
            cudaError_t r = cudaMalloc(dst, sizeof(float4) * v.size());
            if (r == cudaSuccess) r = cudaMemcpy(*dst, v.data(), sizeof(float4) * v.size(), cudaMemcpyHostToDevice);
            if (r != cudaSuccess) set_error(std::string(what) + ": " + cudaGetErrorString(r));
            return r;
        };
        if ((e = upload(&ctx->d_Vloc32, pairs4(V), "V32")) != cudaSuccess) return fail(e, "upload(V32)");
        if (nl && (e = upload(&ctx->d_phNL32, pairs4(phNL), "phNL32")) != cudaSuccess) return fail(e, "upload(phNL32)");
        if (soc && (e = upload(&ctx->d_phSO32, pairs4(phSO), "phSO32")) != cudaSuccess) return fail(e, "upload(phSO32)");
    }
    if (soc) {
        if ((e = cudaMalloc(&ctx->d_phSO, sizeof(double2) * phSO.size())) != cudaSuccess) return fail(e, "cudaMalloc(phSO)");
        if ((e = cudaMemcpy(ctx->d_phSO, phSO.data(), sizeof(double2) * phSO.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "copy phSO");
    }
    if (!nl && !soc) {
        // V off the diagonal in transposed ELL form (slot e of row i at [e][i], columns ascending
        // within a row, short rows padded with zero values at column i); values split into FP32
        // pairs (round to nearest, as on the device). The diagonal gets the kinetic term per k on
        // the device.
        std::vector<std::vector<int>> nz(N);
        int                           W = 0;
        for (int i = 0; i < N; ++i) {
            for (int j = 0; j < N; ++j) {
                const double2 v = V[(size_t)j * N + i];
                if (j != i && (v.x != 0.0 || v.y != 0.0)) nz[i].push_back(j);
            }
            W = std::max(W, (int)nz[i].size());
        }
        const size_t        cnt = std::max<size_t>(1, (size_t)W * N);
        std::vector<int>    col(cnt, 0);
        std::vector<float2> re(cnt, float2{0.f, 0.f}), im(cnt, float2{0.f, 0.f});
        auto                split = [](double v) {
            const float hi = (float)v;
            return float2{hi, (float)(v - (double)hi)};
        };
        for (int i = 0; i < N; ++i) {
            for (int e = 0; e < W; ++e) {
                const size_t o = (size_t)e * N + i;
                if (e < (int)nz[i].size()) {
                    const int     j = nz[i][e];
                    const double2 v = V[(size_t)j * N + i];
                    col[o]          = j;
                    re[o]           = split(v.x);
                    im[o]           = split(v.y);
                } else {
                    col[o] = i;
                }
            }
        }
        ctx->ell_w = W;
        if ((e = cudaMalloc(&ctx->d_ell_col, sizeof(int) * cnt)) != cudaSuccess) return fail(e, "cudaMalloc(ell)");
        if ((e = cudaMalloc(&ctx->d_ell_re, sizeof(float2) * cnt)) != cudaSuccess) return fail(e, "cudaMalloc(ell)");
        if ((e = cudaMalloc(&ctx->d_ell_im, sizeof(float2) * cnt)) != cudaSuccess) return fail(e, "cudaMalloc(ell)");
        if ((e = cudaMemcpy(ctx->d_ell_col, col.data(), sizeof(int) * cnt, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(ctx->d_ell_re, re.data(), sizeof(float2) * cnt, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(ctx->d_ell_im, im.data(), sizeof(float2) * cnt, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "copy ell");
        // the FP32 off-diagonal of a real local H is k-independent: the register reduction reads it
        // from this table (rounded as the assembly's FP32 copy rounds it) instead of an assembled copy
        std::vector<float> v32((size_t)N * N);
        for (size_t q = 0; q < v32.size(); ++q) v32[q] = (float)V[q].x;
        if ((e = cudaMalloc(&ctx->d_V32, sizeof(float) * v32.size())) != cudaSuccess) return fail(e, "cudaMalloc(V32)");
        if ((e = cudaMemcpy(ctx->d_V32, v32.data(), sizeof(float) * v32.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "copy V32");
        ctx->sparse_local = true;
    }
    *out = ctx;
    return UEPM_OK;
}

int uepm_ctx_destroy(uepm_ctx* ctx) {
    if (!ctx) return UEPM_OK;
    if (ctx->d_G) cudaFree(ctx->d_G);
    if (ctx->d_Vloc) cudaFree(ctx->d_Vloc);
    if (ctx->d_phNL) cudaFree(ctx->d_phNL);
    if (ctx->d_phSO) cudaFree(ctx->d_phSO);
    if (ctx->d_Vloc32) cudaFree(ctx->d_Vloc32);
    if (ctx->d_phNL32) cudaFree(ctx->d_phNL32);
    if (ctx->d_phSO32) cudaFree(ctx->d_phSO32);
    if (ctx->d_ell_col) cudaFree(ctx->d_ell_col);
    if (ctx->d_ell_re) cudaFree(ctx->d_ell_re);
    if (ctx->d_ell_im) cudaFree(ctx->d_ell_im);
    if (ctx->d_V32) cudaFree(ctx->d_V32);
    if (ctx->d_ws) cudaFree(ctx->d_ws);
    if (ctx->d_io) cudaFree(ctx->d_io);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->lane_stream) cudaStreamDestroy(ctx->lane_stream);
    if (ctx->lane_fork) cudaEventDestroy(ctx->lane_fork);
    if (ctx->lane_join) cudaEventDestroy(ctx->lane_join);
    for (auto& r : ctx->pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : ctx->pool) cudaEventDestroy(e);
    delete ctx;
    return UEPM_OK;
}

int uepm_ctx_set_precision(uepm_ctx* ctx, int precision) {
    if (!ctx || (precision != UEPM_PREC_FP64 && precision != UEPM_PREC_MIXED)) {
        set_error("uepm_ctx_set_precision: bad context or precision");
        return UEPM_ERR_INVALID;
    }
    ctx->precision = precision;
    return UEPM_OK;
}

int uepm_ctx_order(const uepm_ctx* ctx) { return ctx ? ctx->n : UEPM_ERR_INVALID; }

int uepm_ctx_force_complex(uepm_ctx* ctx, int on) {
    if (!ctx) return UEPM_ERR_INVALID;
    ctx->force_cx = on != 0;
    ctx->real     = ctx->real_h && !ctx->force_cx;
    return ctx->real ? 1 : 0;
}

int uepm_ctx_set_workspace_limit(uepm_ctx* ctx, size_t bytes) {
    if (!ctx || bytes == 0) return UEPM_ERR_INVALID;
    ctx->ws_limit = bytes;
    return UEPM_OK;
}

int uepm_solve_device(uepm_ctx* ctx, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E, double* d_X,
                      double* d_grad, int32_t* d_status, void* stream) {
    if (!ctx || (!d_k && nk) || (!d_E && nk)) {
        set_error("uepm_solve_device: null argument");
        return UEPM_ERR_INVALID;
    }
    if ((want & UEPM_WANT_VECTORS) && !d_X) {
        set_error("uepm_solve_device: UEPM_WANT_VECTORS without an X buffer");
        return UEPM_ERR_INVALID;
    }
    if ((want & UEPM_WANT_GRADIENT) && !d_grad) {
        set_error("uepm_solve_device: UEPM_WANT_GRADIENT without a gradient buffer");
        return UEPM_ERR_INVALID;
    }
    SolvePlan plan;
    int       rc = plan_solve(ctx, nk, nb, want, &plan, true);
    if (rc || nk == 0) return rc;
    if ((rc = ensure_workspace(ctx, plan.ws_bytes))) return rc;
    return enqueue_solve(ctx, plan, d_k, nk, nb, want, d_E, d_X, d_grad, d_status, (cudaStream_t)stream);
}

int uepm_assemble_device(uepm_ctx* ctx, const double* d_k, size_t nk, double* d_H, void* stream) {
    if (!ctx || (nk && (!d_k || !d_H))) {
        set_error("uepm_assemble_device: null argument");
        return UEPM_ERR_INVALID;
    }
    if (nk == 0) return UEPM_OK;
    cudaStream_t s   = (cudaStream_t)stream;
    const int    n   = ctx->n;
    const size_t per = (size_t)ctx->N * ROW_STRIDE * sizeof(double);
    size_t       chunk = std::min(std::min<size_t>(nk, std::max<size_t>(1, ctx->ws_limit / per)), kMaxChunk);
    int          rc    = ensure_ws(ctx, align_up(chunk * per));
    if (rc) return rc;
    const size_t mstride = (size_t)n * n;
    for (size_t off = 0; off < nk; off += chunk) {
        const int c    = (int)std::min(chunk, nk - off);
        auto*     rows = reinterpret_cast<double*>(ctx->d_ws);
        auto*     H    = reinterpret_cast<cx<double>*>(d_H) + off * mstride;
        launch_rows(ctx->P, d_k + 3 * off, ctx->d_G, rows, c, s);
        launch_assemble<cx<double>>(ctx->P, ctx->d_Vloc, ctx->d_phNL, ctx->d_phSO, rows, H, n, mstride, nullptr, 0, c, s);
        if ((rc = check_launch())) return rc;
    }
    return UEPM_OK;
}

int uepm_ctx_set_profiling(uepm_ctx* ctx, int on) {
    if (!ctx) return UEPM_ERR_INVALID;
    ctx->profiling = on ? 1 : 0;
    for (int q = 0; q < UEPM_KERNEL_KINDS; ++q) {
        ctx->prof_ms[q] = 0.0;
        ctx->prof_n[q]  = 0;
    }
    return UEPM_OK;
}

int uepm_ctx_read_profile(uepm_ctx* ctx, double* ms, uint64_t* launches, int capacity) {
    if (!ctx) return UEPM_ERR_INVALID;
    // One launch per kind and pass: where the two lanes of a pass both ran a kind, it counts once,
    // from the earlier start to the later end (times relative to the first record's start).
    struct Span {
        int         kind;
        cudaEvent_t ref;
        float       lo, hi;
    };
    std::map<std::pair<unsigned, int>, Span> spans;
    for (auto& r : ctx->pending) {
        UEPM_CUDA(cudaEventSynchronize(r.b));
        auto it = spans.find({r.group, r.kind});
        if (it == spans.end()) {
            float t = 0.f;
            UEPM_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
            spans[{r.group, r.kind}] = Span{r.kind, r.a, 0.f, t};
        } else {
            float ta = 0.f, tb = 0.f;
            UEPM_CUDA(cudaEventElapsedTime(&ta, it->second.ref, r.a));
            UEPM_CUDA(cudaEventElapsedTime(&tb, it->second.ref, r.b));
            it->second.lo = std::min(it->second.lo, ta);
            it->second.hi = std::max(it->second.hi, tb);
        }
    }
    for (const auto& kv : spans) {
        ctx->prof_ms[kv.second.kind] += kv.second.hi - kv.second.lo;
        ctx->prof_n[kv.second.kind] += 1;
    }
    for (auto& r : ctx->pending) {
        ctx->pool.push_back(r.a);
        ctx->pool.push_back(r.b);
    }
    ctx->pending.clear();
    for (int q = 0; q < capacity && q < UEPM_KERNEL_KINDS; ++q) {
        if (ms) ms[q] = ctx->prof_ms[q];
        if (launches) launches[q] = ctx->prof_n[q];
    }
    return UEPM_KERNEL_KINDS;
}

const char* uepm_kernel_name(int kind) { return (kind >= 0 && kind < UEPM_KERNEL_KINDS) ? kKernelNames[kind] : ""; }

int uepm_solve(uepm_ctx* ctx, const double* k, size_t nk, int nb, uint32_t want, double* E, double* X, double* grad,
               int32_t* status) {
    if (!ctx || (nk && (!k || !E))) {
        set_error("uepm_solve: null argument");
        return UEPM_ERR_INVALID;
    }
    if (nb < 1 || nb > ctx->n) {
        set_error("uepm_solve: nb must be in [1, n]");
        return UEPM_ERR_OUT_OF_RANGE;
    }
    if (nk == 0) return UEPM_OK;
    if ((want & UEPM_WANT_VECTORS) && !X) {
        set_error("uepm_solve: UEPM_WANT_VECTORS without an X buffer");
        return UEPM_ERR_INVALID;
    }
    if ((want & UEPM_WANT_GRADIENT) && !grad) {
        set_error("uepm_solve: UEPM_WANT_GRADIENT without a gradient buffer");
        return UEPM_ERR_INVALID;
    }
    if (!ctx->stream) UEPM_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    const bool   wv = (want & UEPM_WANT_VECTORS) != 0, wg = (want & UEPM_WANT_GRADIENT) != 0;
    const size_t bk = align_up(sizeof(double) * 3 * nk), bE = align_up(sizeof(double) * nk * nb);
    const size_t bX = wv ? align_up(sizeof(double) * 2 * nk * nb * ctx->n) : 0;
    const size_t bg = wg ? align_up(sizeof(double) * 3 * nk * nb) : 0;
    const size_t bs = align_up(sizeof(int32_t) * nk);
    const size_t need = bk + bE + bX + bg + bs;
    if (need > ctx->io_bytes) {
        if (ctx->d_io) cudaFree(ctx->d_io);
        ctx->d_io     = nullptr;
        ctx->io_bytes = 0;
        if (cudaMalloc(&ctx->d_io, need) != cudaSuccess) {
            cudaGetLastError();
            set_error("uepm_solve: device I/O allocation failed");
            return UEPM_ERR_NOMEM;
        }
        ctx->io_bytes = need;
    }
    char*   io  = static_cast<char*>(ctx->d_io);
    double* dk  = reinterpret_cast<double*>(io);
    double* dE  = reinterpret_cast<double*>(io + bk);
    double* dX  = wv ? reinterpret_cast<double*>(io + bk + bE) : nullptr;
    double* dg  = wg ? reinterpret_cast<double*>(io + bk + bE + bX) : nullptr;
    auto*   dst = reinterpret_cast<int32_t*>(io + bk + bE + bX + bg);
    cudaStream_t s = ctx->stream;
    UEPM_CUDA(cudaMemcpyAsync(dk, k, sizeof(double) * 3 * nk, cudaMemcpyHostToDevice, s));
    int rc = uepm_solve_device(ctx, dk, nk, nb, want, dE, dX, dg, dst, s);
    if (rc) return rc;
    UEPM_CUDA(cudaMemcpyAsync(E, dE, sizeof(double) * nk * nb, cudaMemcpyDeviceToHost, s));
    if (wv) UEPM_CUDA(cudaMemcpyAsync(X, dX, sizeof(double) * 2 * nk * nb * ctx->n, cudaMemcpyDeviceToHost, s));
    if (wg) UEPM_CUDA(cudaMemcpyAsync(grad, dg, sizeof(double) * 3 * nk * nb, cudaMemcpyDeviceToHost, s));
    std::vector<int32_t> hs;
    int32_t*             so = status;
    if (!so) {
        hs.resize(nk);
        so = hs.data();
    }
    UEPM_CUDA(cudaMemcpyAsync(so, dst, sizeof(int32_t) * nk, cudaMemcpyDeviceToHost, s));
    UEPM_CUDA(cudaStreamSynchronize(s));
    for (size_t q = 0; q < nk; ++q)
        if (so[q] != 0) {
            set_error("uepm_solve: k-point " + std::to_string(q) + " reported status " + std::to_string(so[q]));
            return UEPM_ERR_NOT_CONVERGED;
        }
    return UEPM_OK;
}

}  // extern "C"
