// ctx_internal.h -- the context behind the C ABI handle, and the solve entry points shared by the
// C ABI (capi.cu) and the batch / autotuning runtime (batch.cu). Not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "uepm_common.cuh"
#include "uepm_gb300.h"

struct uepm_ctx {
    int           device    = 0;
    uepm_material mat{};
    uepm::DevParams P{};
    int           N = 0, n = 0;
    uint32_t      flags     = 0;
    int           precision = UEPM_PREC_FP64;
    bool          real_h    = false;  // H(k) is exactly real for this material and flags
    bool          force_cx  = false;  // run the complex kernels even when H(k) is real
    bool          real      = false;  // real_h && !force_cx
    size_t        ws_limit  = (size_t)8 << 30;
    uepm_tuning   tune{};  // kernel-shape choices (0: automatic)
    int*          d_G       = nullptr;
    uepm::cx<double>* d_Vloc    = nullptr;
    double2*      d_phNL    = nullptr;
    double2*      d_phSO    = nullptr;
    // square nonlocal wells without spin-orbit: the mixed path forms H(k) in double-single
    // arithmetic from V and the nonlocal phase in FP32 pairs (re hi, re lo, im hi, im lo)
    bool              ds_nl     = false;
    uepm::DevParamsDS Q{};
    float4*           d_Vloc32  = nullptr;
    float4*           d_phNL32  = nullptr;
    bool              ds_soc    = false;  // spin-orbit: the same, with the spin-orbit phase in pairs
    float4*           d_phSO32  = nullptr;
    // local potential only (no nonlocal, no spin-orbit): H(k) = V + diag(kinetic(k)) with V the
    // k-independent local form-factor matrix, sparse (|G_i - G_j|^2 in {3, 4, 8, 11}); its rows as
    // CSR (every row also lists its diagonal) with values as FP32 pairs, for the mixed path's H X
    bool          sparse_local = false;
    int           ell_w     = 0;        // off-diagonal slots per row of V (transposed ELL)
    int*          d_ell_col = nullptr;  // [ell_w][N]
    float2*       d_ell_re  = nullptr;  // [ell_w][N] FP32 pairs of Re V
    float2*       d_ell_im  = nullptr;  // [ell_w][N] FP32 pairs of Im V
    float*        d_V32     = nullptr;  // [N][N] Re V rounded to FP32 (the diagonal is formed per k)
    void*         d_ws      = nullptr;
    size_t        ws_bytes  = 0;
    // second lane of a two-lane solve (created on first use) and its fork / join events
    cudaStream_t  lane_stream = nullptr;
    cudaEvent_t   lane_fork   = nullptr;
    cudaEvent_t   lane_join   = nullptr;
    // buffers of the host-pointer entry point
    cudaStream_t  stream    = nullptr;
    void*         d_io      = nullptr;
    size_t        io_bytes  = 0;
    std::vector<int32_t> G;
    // per-kernel timing (uepm_ctx_set_profiling)
    struct Rec {
        int         kind;
        unsigned    group;  // the pass (both lanes of a two-lane pass share it)
        cudaEvent_t a, b;
    };
    int                      profiling = 0;
    unsigned                 prof_group = 0;
    std::vector<Rec>         pending;
    std::vector<cudaEvent_t> pool;
    double                   prof_ms[UEPM_KERNEL_KINDS] = {0};
    uint64_t                 prof_n[UEPM_KERNEL_KINDS]  = {0};
};

namespace uepm {

void set_error(const std::string& msg);

// Workspace plan of one pipeline pass: chunk (k-points per pass) and the bytes it needs.
// lanes = 2: consecutive chunks alternate between the caller's stream and the context's second
// stream, each lane with its own workspace half (ws_bytes covers both).
struct SolvePlan {
    size_t chunk = 0, ws_bytes = 0;
    int    m     = 0;
    int    lanes = 1;
};
// Validates nb / want against the context and plans the passes of an nk-point solve (no allocation).
// two_lanes lets the plan take two lanes where they pay (mixed-precision solves of 1024 k-points or
// more that fit one pass) or where uepm_tuning.streams = 2 asks for them.
int plan_solve(uepm_ctx* ctx, size_t nk, int nb, uint32_t want, SolvePlan* out, bool two_lanes = false);
// Grows the context's device workspace to at least `bytes` (allocates: not while capturing).
int ensure_workspace(uepm_ctx* ctx, size_t bytes);
// Enqueues the solve on s; the workspace (the context's own, or ws / ws_bytes when given, so that
// several solves of one context can be in flight at once) must hold plan.ws_bytes. No allocation,
// no host sync.
int enqueue_solve(uepm_ctx* ctx, const SolvePlan& plan, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E,
                  double* d_X, double* d_grad, int32_t* d_status, cudaStream_t s, void* ws = nullptr,
                  size_t ws_bytes = 0);
uint64_t launches_total();
void     uncount_launches(uint64_t n);

}  // namespace uepm
