// noalloc.cu -- H(k) assembly for callers that must not allocate device memory when they call.
//
// Some callers of this library cannot call cudaMalloc at the moment they need H(k): a real-time
// or serving loop whose memory was reserved once at start-up and where a device allocation would
// stall the device (cudaMalloc synchronises), a host application whose device memory is owned by its
// own allocator or pool, or code that runs while other work is being captured or replayed. The regular
// uepm_assemble_device grows a per-context device workspace on demand (for the per-plane-wave row
// table), which may allocate. uepm_assemble_device_noalloc computes the same H(k) with that row table
// in a fixed-size, file-scope device array instead, so the call itself allocates nothing.
//
// The array (UEPM_NOALLOC_SCRATCH_BYTES = 16 MiB) exists on every GPU that loads this library, for as
// long as the library stays loaded. Its device address is looked up once per device, with that device
// current, by the first call on that device (cudaGetSymbolAddress); make that first call before any
// stream capture. The address is kept for the life of the process: after cudaDeviceReset (or any
// other teardown of the device's primary context) it is stale, so the entry point must not be used
// on that device again. Every call shares the array and it keeps the last call's contents: each call
// rewrites every entry it reads, so nothing has to start at zero, but two calls whose work overlaps on
// the GPU (different streams, or different host threads) race on it. One call takes at most
// kMaxNoallocK = 32768 k-points (the assembly grid's extent) and at most the scratch's worth.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ctx_view.h"
#include "uepm_common.cuh"
#include "uepm_gb300.h"
#include "uepm_kernels.h"

namespace uepm {
void set_error(const std::string& msg);
}  // namespace uepm

using namespace uepm;

namespace {

constexpr size_t kScratchDoubles = UEPM_NOALLOC_SCRATCH_BYTES / sizeof(double);
constexpr size_t kMaxNoallocK    = 32768;  // k-points per launch: the assembly grid's z extent is <= 65535

// The scratch row table. In host code this name is only a host-side stand-in for the device
// object: its device address comes from cudaGetSymbolAddress (scratch_on_current_device).
static __device__ __align__(256) double g_noalloc_rows[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex    g_mu;
double*       g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
int scratch_on_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error(std::string("uepm_assemble_device_noalloc: no usable current device: ") + cudaGetErrorString(e));
        return UEPM_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e       = cudaGetSymbolAddress(&p, g_noalloc_rows);
        if (e != cudaSuccess || !p) {
            set_error(std::string("uepm_assemble_device_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
            return UEPM_ERR_CUDA;
        }
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return UEPM_OK;
}

}  // namespace

extern "C" int uepm_assemble_device_noalloc(uepm_ctx* ctx, const double* d_k, size_t nk, double* d_H, void* stream) {
    CtxTables t;
    if (!ctx_tables(ctx, &t) || (nk && (!d_k || !d_H))) {
        set_error("uepm_assemble_device_noalloc: null argument");
        return UEPM_ERR_INVALID;
    }
    if (nk == 0) return UEPM_OK;
    if (nk > kMaxNoallocK) {
        set_error("uepm_assemble_device_noalloc: " + std::to_string(nk) + " k-points in one call; the limit is " +
                  std::to_string(kMaxNoallocK) + " per call");
        return UEPM_ERR_INVALID;
    }
    const size_t need = nk * (size_t)t.N * ROW_STRIDE;
    if (need > kScratchDoubles) {
        set_error("uepm_assemble_device_noalloc: " + std::to_string(nk) + " k-points with basis " + std::to_string(t.N) +
                  " need " + std::to_string(need * sizeof(double)) + " bytes of scratch; the limit is " +
                  std::to_string(UEPM_NOALLOC_SCRATCH_BYTES) + " bytes, i.e. at most " +
                  std::to_string(kScratchDoubles / ((size_t)t.N * ROW_STRIDE)) + " k-points per call");
        return UEPM_ERR_INVALID;
    }
    double* rows = nullptr;
    int     rc   = scratch_on_current_device(&rows);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    launch_rows(t.P, d_k, t.d_G, rows, (int)nk, s);
    launch_assemble<cx<double>>(t.P, t.Vloc, t.phNL, t.phSO, rows, reinterpret_cast<cx<double>*>(d_H), t.n,
                                (size_t)t.n * t.n, nullptr, 0, (int)nk, s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("uepm_assemble_device_noalloc: kernel launch failed: ") + cudaGetErrorString(e));
        return UEPM_ERR_CUDA;
    }
    return UEPM_OK;
}
