// star.cu -- irreducible wedge -> full Brillouin zone: energies and gradients of every mesh vertex
// from the solved wedge vertices, as MeshBZ::distribute_energies_from_iw_wedge_to_full_bz does
// (src/BZ_MESH/bz_mesh.cpp:1383-1414), as one device gather after the solve.
//
// Each full-zone vertex v has a source wedge vertex src[v] and the signed permutation that maps the
// wedge k-point onto it; its energies are the source's, and its gradient is the source gradient g
// taken through the same operation: grad_v[j] = sign[j] * g[perm[j]]. The operation is the one
// apply_same_symmetry_operation (bz_mesh.cpp:1312-1381) finds, computed on the host once per mesh.
#include <cuda_runtime.h>

#include <string>

#include "ctx_internal.h"
#include "uepm_kernels.h"

namespace uepm {
namespace {

// op: perm[0..2] in bits 0-5 (2 bits each), sign bits 6-8 (1 = negative)
__global__ void k_star_expand(const double* __restrict__ E_iw, const double* __restrict__ g_iw, const int64_t* __restrict__ src,
                              const uint16_t* __restrict__ op, size_t n_full, int nb, double* __restrict__ E_full,
                              double* __restrict__ g_full) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_full * (size_t)nb) return;
    const size_t v = idx / nb;
    const int    b = (int)(idx - v * nb);
    const size_t s = (size_t)src[v];
    E_full[idx]    = E_iw[s * nb + b];
    if (g_iw && g_full) {
        const unsigned o = op[v];
        const double*  g = g_iw + (s * nb + b) * 3;
        double*        h = g_full + idx * 3;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int    p = (o >> (2 * j)) & 3;
            const double x = g[p];
            h[j]           = ((o >> (6 + j)) & 1) ? -x : x;
        }
    }
}

}  // namespace
}  // namespace uepm

using namespace uepm;

extern "C" int uepm_star_expand_device(const double* d_E_iw, const double* d_grad_iw, const int64_t* d_src,
                                       const uint16_t* d_op, size_t n_full, int nb, double* d_E_full, double* d_grad_full,
                                       void* stream) {
    if ((n_full && (!d_E_iw || !d_src || !d_E_full)) || nb <= 0 || ((d_grad_iw != nullptr) != (d_grad_full != nullptr)) ||
        (d_grad_iw && !d_op)) {
        set_error("uepm_star_expand_device: bad argument");
        return UEPM_ERR_INVALID;
    }
    if (n_full == 0) return UEPM_OK;
    const size_t total = n_full * (size_t)nb;
    const int    blk   = 256;
    k_star_expand<<<(unsigned)((total + blk - 1) / blk), blk, 0, (cudaStream_t)stream>>>(d_E_iw, d_grad_iw, d_src, d_op, n_full,
                                                                                       nb, d_E_full, d_grad_full);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("uepm_star_expand_device: ") + cudaGetErrorString(e));
        return UEPM_ERR_CUDA;
    }
    return UEPM_OK;
}
