// server.cu -- a band / group-velocity query server over resident contexts (C ABI, include/uepm_gb300.h).
//
// No reference counterpart: the reference has no serving loop; its full-band Monte Carlo looks bands
// up by interpolation on a mesh (src/FBMC/particle.cpp:52-63). Here queries of any size arrive at any
// time and are answered from the device:
//
//   * resident state: the contexts (form factors, G-vector sets, tuning) stay on the device; every
//     work item runs in a sub-range of one device arena allocated at creation, so nothing is
//     allocated while serving;
//   * work items: a request is cut into items of at most max_chunk k-points, in arrival order; a
//     velocity request expands each k-point into 7 (k and k +- h along each axis, central
//     differences), all solved as one batch;
//   * admission by HBM footprint: an item is started only when a slot is free and the arena has a
//     free range for its footprint (workspace of its solve plan + its inputs and outputs); an item
//     that cannot fit even in an empty arena fails its request;
//   * continuous batching: the slots are streams; a scheduler thread admits items whenever a slot
//     and memory free up, so items of requests that arrive while others are on the GPU run
//     concurrently with them, and a large request never holds the device for more than one item at
//     a time per slot;
//   * each item's results are copied back through pinned staging and scattered into the request's
//     host buffers; a request completes when its last item does, and its latency (submission to
//     completion) feeds the p50 / p99 statistics.
// Every k-point is solved by the same kernels with the same per-matrix arithmetic whether it runs
// alone or in the mix, so results are identical either way.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ctx_internal.h"

using namespace uepm;

namespace {

constexpr double kQe   = 1.602176634e-19;                              // C
constexpr double kHbar = 6.62607015e-34 / (2.0 * 3.141592653589793238462643383279502884);  // J s

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// First-fit allocator over the device arena (offsets only; the arena is one cudaMalloc).
class Arena {
public:
    void reset(size_t bytes) {
        size_ = bytes;
        free_.clear();
        free_[0] = bytes;
    }
    bool alloc(size_t bytes, size_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= bytes) {
                *off              = it->first;
                const size_t rest = it->second - bytes;
                const size_t next = it->first + bytes;
                free_.erase(it);
                if (rest) free_[next] = rest;
                return true;
            }
        return false;
    }
    void release(size_t off, size_t bytes) {
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

private:
    size_t                   size_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
};

struct Request {
    int64_t              id;
    int                  ctx;
    std::vector<double>  k;  // copied at submission
    size_t               nk;
    int                  nb;
    bool                 vel;
    double               h;
    double*              E;
    double*              V;
    int32_t*             st;
    size_t               items_left = 0;
    double               t_submit = 0, t_done = 0;
    bool                 done = false;
    int                  err  = UEPM_OK;
    std::string          msg;
};

struct Item {
    std::shared_ptr<Request> req;
    size_t                   off, cnt;  // user k-points [off, off + cnt)
};

struct Slot {
    cudaStream_t s    = nullptr;
    cudaEvent_t  done = nullptr;
    char*        pin  = nullptr;  // pinned staging: k in, then E and status out
    size_t       pin_bytes = 0;
    bool         busy = false;
    Item         item;
    size_t       arena_off = 0, arena_bytes = 0;
    size_t       ne = 0;  // expanded k-points of the item
    double*      dE = nullptr;
    int32_t*     dst = nullptr;
};

}  // namespace

struct uepm_server {
    std::vector<uepm_ctx*> ctxs;
    int                    device = 0;
    size_t                 max_chunk = 2048;
    int                    max_nb    = 64;
    char*                  d_arena = nullptr;
    Arena                  arena;
    std::vector<Slot>      slots;

    std::mutex                                    mu;
    std::condition_variable                       cv_work, cv_done;
    std::deque<Item>                              pending;
    std::map<int64_t, std::shared_ptr<Request>>   reqs;
    int64_t                                       next_id = 0;
    bool                                          stop    = false;
    std::thread                                   worker;
    std::vector<double>                           lat_ms;
    uint64_t                                      kpts_done = 0, items_done = 0;
    double                                        t_first = 0, t_last = 0;
    std::string                                   fatal;

    void run();
    bool admit(Slot& sl, Item& it);
    void finish(Slot& sl);
};

namespace {

// footprint of an item: workspace of its solve plus device k, E and status
bool item_plan(uepm_ctx* ctx, size_t ne, int nb, SolvePlan* sp, size_t* bytes) {
    if (plan_solve(ctx, ne, nb, UEPM_WANT_VALUES, sp) != UEPM_OK) return false;
    *bytes = align256(sp->ws_bytes) + align256(sizeof(double) * 3 * ne) + align256(sizeof(double) * ne * nb) +
             align256(sizeof(int32_t) * ne);
    return true;
}

}  // namespace

bool uepm_server::admit(Slot& sl, Item& it) {
    Request&  r   = *it.req;
    uepm_ctx* ctx = ctxs[r.ctx];
    const int mult = r.vel ? 7 : 1;
    const size_t ne = it.cnt * mult;
    SolvePlan sp;
    size_t    bytes = 0;
    if (!item_plan(ctx, ne, r.nb, &sp, &bytes)) {
        r.err = UEPM_ERR_INVALID;
        r.msg = "request: " + std::string(uepm_last_error());
        return true;  // consumed (failed)
    }
    size_t off = 0;
    if (!arena.alloc(bytes, &off)) {
        bool idle = true;
        for (auto& q : slots) idle &= !q.busy;
        if (idle) {  // cannot fit even alone
            r.err = UEPM_ERR_NOMEM;
            r.msg = "request: a work item needs " + std::to_string(bytes) + " bytes, more than the server's HBM budget";
            return true;
        }
        return false;  // wait for memory
    }
    char*    base = d_arena + off;
    char*    ws   = base;
    double*  dk   = reinterpret_cast<double*>(base + align256(sp.ws_bytes));
    double*  dE   = reinterpret_cast<double*>(reinterpret_cast<char*>(dk) + align256(sizeof(double) * 3 * ne));
    int32_t* dst  = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(dE) + align256(sizeof(double) * ne * r.nb));
    // expanded k-points into the pinned staging, then to the device
    double* hk = reinterpret_cast<double*>(sl.pin);
    for (size_t q = 0; q < it.cnt; ++q) {
        const double* k0 = &r.k[3 * (it.off + q)];
        double*       o  = hk + 3 * mult * q;
        o[0] = k0[0], o[1] = k0[1], o[2] = k0[2];
        if (r.vel)
            for (int ax = 0; ax < 3; ++ax)
                for (int sg = 0; sg < 2; ++sg) {
                    double* p = o + 3 * (1 + 2 * ax + sg);
                    p[0] = k0[0], p[1] = k0[1], p[2] = k0[2];
                    p[ax] += sg ? -r.h : r.h;
                }
    }
    int rc = UEPM_OK;
    if (cudaMemcpyAsync(dk, hk, sizeof(double) * 3 * ne, cudaMemcpyHostToDevice, sl.s) != cudaSuccess) rc = UEPM_ERR_CUDA;
    if (!rc)
        rc = enqueue_solve(ctx, sp, dk, ne, r.nb, UEPM_WANT_VALUES, dE, nullptr, nullptr, dst, sl.s, ws, sp.ws_bytes);
    double*  hE  = reinterpret_cast<double*>(sl.pin + align256(sizeof(double) * 3 * ne));
    int32_t* hst = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(hE) + align256(sizeof(double) * ne * r.nb));
    if (!rc && (cudaMemcpyAsync(hE, dE, sizeof(double) * ne * r.nb, cudaMemcpyDeviceToHost, sl.s) != cudaSuccess ||
                cudaMemcpyAsync(hst, dst, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost, sl.s) != cudaSuccess ||
                cudaEventRecord(sl.done, sl.s) != cudaSuccess))
        rc = UEPM_ERR_CUDA;
    if (rc) {
        arena.release(off, bytes);
        r.err = rc;
        r.msg = std::string("request: ") + uepm_last_error();
        return true;
    }
    sl.busy        = true;
    sl.item        = it;
    sl.arena_off   = off;
    sl.arena_bytes = bytes;
    sl.ne          = ne;
    return true;
}

void uepm_server::finish(Slot& sl) {
    Request&     r    = *sl.item.req;
    const int    mult = r.vel ? 7 : 1;
    const size_t ne   = sl.ne;
    const int    nb   = r.nb;
    const double* hE  = reinterpret_cast<const double*>(sl.pin + align256(sizeof(double) * 3 * ne));
    const int32_t* hst =
        reinterpret_cast<const int32_t*>(reinterpret_cast<const char*>(hE) + align256(sizeof(double) * ne * nb));
    // group velocity from central differences: dE/dk_reduced * (a / 2 pi) = grad_k E in eV m,
    // times q_e / hbar for m/s
    const double toV = ctxs[r.ctx]->P.frac_to_phys * kQe / kHbar / (2.0 * r.h);
    for (size_t q = 0; q < sl.item.cnt; ++q) {
        const size_t   u  = sl.item.off + q;
        const double*  e0 = hE + (size_t)mult * q * nb;
        int32_t        s  = 0;
        for (int p = 0; p < mult; ++p) s |= hst[mult * q + p];
        std::copy(e0, e0 + nb, r.E + u * nb);
        if (r.vel && r.V)
            for (int b = 0; b < nb; ++b)
                for (int ax = 0; ax < 3; ++ax)
                    r.V[(u * nb + b) * 3 + ax] = (e0[(1 + 2 * ax) * nb + b] - e0[(2 + 2 * ax) * nb + b]) * toV;
        if (r.st) r.st[u] = s;
    }
    arena.release(sl.arena_off, sl.arena_bytes);
    sl.busy = false;
    items_done += 1;
    if (--r.items_left == 0) {
        r.t_done = now_s();
        r.done   = true;
        lat_ms.push_back(1e3 * (r.t_done - r.t_submit));
        kpts_done += r.nk;
        t_last = r.t_done;
    }
}

void uepm_server::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        // completions
        bool progressed = false;
        for (auto& sl : slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                Request& r = *sl.item.req;
                r.err      = UEPM_ERR_CUDA;
                r.msg      = std::string("request: ") + cudaGetErrorString(q);
                cudaGetLastError();
            }
            finish(sl);
            progressed = true;
        }
        // admissions, in arrival order
        for (auto& sl : slots) {
            if (sl.busy || pending.empty()) continue;
            Item it = pending.front();
            if (it.req->err) {  // an earlier item of this request failed: drop the rest
                pending.pop_front();
                if (--it.req->items_left == 0) {
                    it.req->done   = true;
                    it.req->t_done = now_s();
                }
                progressed = true;
                continue;
            }
            if (!admit(sl, it)) break;  // no memory yet: keep the order
            pending.pop_front();
            progressed = true;
            if (it.req->err && !sl.busy && --it.req->items_left == 0) {
                it.req->done   = true;
                it.req->t_done = now_s();
            }
        }
        if (progressed) cv_done.notify_all();
        bool busy = false;
        for (auto& sl : slots) busy |= sl.busy;
        if (stop && !busy) break;
        if (!busy && pending.empty()) {
            cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        } else if (!progressed) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        }
    }
}

extern "C" {

int uepm_server_create(uepm_ctx* const* ctxs, int nctx, size_t hbm_budget, int slots, size_t max_chunk, int max_nb,
                       uepm_server** out) {
    if (!ctxs || nctx <= 0 || !out || slots <= 0 || max_chunk == 0 || max_nb <= 0) {
        set_error("uepm_server_create: bad argument");
        return UEPM_ERR_INVALID;
    }
    for (int c = 0; c < nctx; ++c)
        if (!ctxs[c]) {
            set_error("uepm_server_create: null context");
            return UEPM_ERR_INVALID;
        }
    auto sv       = std::make_unique<uepm_server>();
    sv->ctxs      = std::vector<uepm_ctx*>(ctxs, ctxs + nctx);
    sv->device    = ctxs[0]->device;
    sv->max_chunk = max_chunk;
    sv->max_nb    = max_nb;
    if (cudaSetDevice(sv->device) != cudaSuccess || cudaMalloc(&sv->d_arena, hbm_budget) != cudaSuccess) {
        cudaGetLastError();
        set_error("uepm_server_create: device arena of " + std::to_string(hbm_budget) + " bytes could not be allocated");
        return UEPM_ERR_NOMEM;
    }
    sv->arena.reset(hbm_budget);
    const size_t ne  = 7 * max_chunk;
    const size_t pin = align256(sizeof(double) * 3 * ne) + align256(sizeof(double) * ne * max_nb) + align256(sizeof(int32_t) * ne);
    sv->slots.resize(slots);
    for (auto& sl : sv->slots) {
        if (cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void**>(&sl.pin), pin) != cudaSuccess) {
            cudaGetLastError();
            set_error("uepm_server_create: stream, event or pinned staging could not be created");
            uepm_server_destroy(sv.release());
            return UEPM_ERR_NOMEM;
        }
        sl.pin_bytes = pin;
    }
    uepm_server* p = sv.release();
    p->worker      = std::thread([p] { p->run(); });
    *out           = p;
    return UEPM_OK;
}

int uepm_server_destroy(uepm_server* sv) {
    if (!sv) return UEPM_OK;
    if (sv->worker.joinable()) {
        {
            std::lock_guard<std::mutex> g(sv->mu);
            sv->stop = true;
        }
        sv->cv_work.notify_all();
        sv->worker.join();
    }
    for (auto& sl : sv->slots) {
        if (sl.s) cudaStreamSynchronize(sl.s);
        if (sl.s) cudaStreamDestroy(sl.s);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.pin) cudaFreeHost(sl.pin);
    }
    if (sv->d_arena) cudaFree(sv->d_arena);
    delete sv;
    return UEPM_OK;
}

int64_t uepm_server_submit(uepm_server* sv, int ctx_index, const double* k, size_t nk, int nb, uint32_t flags,
                           double fd_step, double* E, double* V, int32_t* status) {
    if (!sv || (nk && (!k || !E)) || ctx_index < 0 || ctx_index >= (int)sv->ctxs.size()) {
        set_error("uepm_server_submit: bad argument");
        return UEPM_ERR_INVALID;
    }
    const bool vel = (flags & UEPM_SERVE_VELOCITY) != 0;
    if (nb < 1 || nb > sv->max_nb || nb > sv->ctxs[ctx_index]->n) {
        set_error("uepm_server_submit: nb outside [1, min(n, max_nb)]");
        return UEPM_ERR_OUT_OF_RANGE;
    }
    if (vel && (!V || !(fd_step > 0.0))) {
        set_error("uepm_server_submit: a velocity request needs a V buffer and a positive step");
        return UEPM_ERR_INVALID;
    }
    auto r = std::make_shared<Request>();
    r->ctx = ctx_index;
    r->k.assign(k, k + 3 * nk);
    r->nk  = nk;
    r->nb  = nb;
    r->vel = vel;
    r->h   = fd_step;
    r->E   = E;
    r->V   = V;
    r->st  = status;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        r->id       = sv->next_id++;
        r->t_submit = now_s();
        if (sv->t_first == 0) sv->t_first = r->t_submit;
        if (nk == 0) {
            r->done   = true;
            r->t_done = r->t_submit;
        }
        for (size_t off = 0; off < nk; off += sv->max_chunk) {
            sv->pending.push_back({r, off, std::min(sv->max_chunk, nk - off)});
            r->items_left += 1;
        }
        sv->reqs[r->id] = r;
    }
    sv->cv_work.notify_all();
    return r->id;
}

int uepm_server_wait(uepm_server* sv, int64_t id, double timeout_s) {
    if (!sv) {
        set_error("uepm_server_wait: null server");
        return UEPM_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lk(sv->mu);
    auto                         it = sv->reqs.find(id);
    if (it == sv->reqs.end()) {
        set_error("uepm_server_wait: unknown request " + std::to_string(id));
        return UEPM_ERR_INVALID;
    }
    auto r    = it->second;
    auto pred = [&] { return r->done; };
    if (timeout_s < 0) sv->cv_done.wait(lk, pred);
    else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return 1;  // still running
    sv->reqs.erase(id);
    if (r->err) {
        set_error(r->msg);
        return r->err;
    }
    return UEPM_OK;
}

int uepm_server_stats(uepm_server* sv, double* p50_ms, double* p99_ms, uint64_t* completed, uint64_t* kpoints,
                      double* span_s) {
    if (!sv) {
        set_error("uepm_server_stats: null server");
        return UEPM_ERR_INVALID;
    }
    std::lock_guard<std::mutex> g(sv->mu);
    std::vector<double>         v = sv->lat_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        if (v.empty()) return 0.0;
        const size_t i = (size_t)std::ceil(p * (double)v.size()) - 1;
        return v[std::min(i, v.size() - 1)];
    };
    if (p50_ms) *p50_ms = pct(0.50);
    if (p99_ms) *p99_ms = pct(0.99);
    if (completed) *completed = v.size();
    if (kpoints) *kpoints = sv->kpts_done;
    if (span_s) *span_s = sv->t_last > sv->t_first ? sv->t_last - sv->t_first : 0.0;
    return UEPM_OK;
}

int uepm_server_reset_stats(uepm_server* sv) {
    if (!sv) {
        set_error("uepm_server_reset_stats: null server");
        return UEPM_ERR_INVALID;
    }
    std::lock_guard<std::mutex> g(sv->mu);
    sv->lat_ms.clear();
    sv->kpts_done = 0;
    sv->t_first = sv->t_last = 0;
    return UEPM_OK;
}

}  // extern "C"
