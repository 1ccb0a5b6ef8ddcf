// dielectric.cu -- the eigenvector consumer of the dielectric function: squared overlaps between
// conduction states at k + q and valence states at k, summed against the smeared pair of the
// energy grid, on the device after the solves at k and k + q.
//
// Replaces the per-q body of DielectricFunction::compute_dielectric_function
// (src/EPP/DielectricFunction.cpp:92-150) and the per-vertex sums of
// BZ_States::compute_dielectric_function (src/BZ_MESH/bz_states.cpp:101-140, where each vertex
// enters with the volume / 4 of every tetrahedron that holds it: a per-k weight here):
//   for each k:  O_cv = |sum_i u_c(k+q)_i u_v(k)_i|^2,  dE_cv = E_c(k+q) - E_v(k)   (c >= first_cond > v)
//   s_k(w) = sum_{c, v} O_cv [ (dE_cv - w) / ((dE_cv - w)^2 + eta^2) + (dE_cv + w) / ((dE_cv + w)^2 + eta^2) ]
//   sums(w) += weight_k s_k(w)
// in FP64, pairs in the reference's order (conduction outer, valence inner), each pair's two
// fractions over one denominator (rounding-level differences from the reference's two divisions).
// The overlap is the reference's Eigen expression col(c).adjoint().dot(col(v)): dot() conjugates
// its first operand, which is already the adjoint, so no factor is conjugated. For a real H (the
// elemental crystals the reference's epsilon driver runs) this equals |<u_c|u_v>|^2; it is kept as
// written so that complex H gives the reference's numbers too.
//
// Layout. A persistent grid of CTAs takes k-points b, b + grid, ...: the CTA stages the valence rows
// of X(k) and the conduction rows of X(k+q) in shared memory (coalesced), one warp per overlap
// forms the n-term dot with a shuffle reduction, and then every thread runs its energies of the
// grid over the P pairs (the pair table is a shared-memory broadcast). Each CTA keeps its energy
// sums in registers and writes them once; a second kernel adds the CTAs' partial sums in a fixed
// order, so results do not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "ctx_internal.h"
#include "uepm_kernels.h"

namespace uepm {
namespace {

constexpr int kDfThreads = 256;
constexpr int kDfWarps   = kDfThreads / 32;
constexpr int kDfMaxE    = 16;  // energies per thread: ne <= kDfMaxE * kDfThreads

__global__ void __launch_bounds__(kDfThreads) k_dielectric_sums(const double2* __restrict__ Xk, const double2* __restrict__ Xkq,
                                                              const double* __restrict__ Ek, const double* __restrict__ Ekq,
                                                              size_t nk, int nb, int n, int fc, const double* __restrict__ en,
                                                              int ne, double eta, const double* __restrict__ wk,
                                                              double* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smraw[];
    double2*  sx  = reinterpret_cast<double2*>(smraw);         // [nb][n]: valence rows of X(k), conduction of X(k+q)
    const int P   = (nb - fc) * fc;
    double*   so  = reinterpret_cast<double*>(sx + (size_t)nb * n);  // [P] squared overlaps
    double*   sd  = so + P;                                           // [P] energy differences
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double eta2 = eta * eta;
    double       acc[kDfMaxE];
#pragma unroll
    for (int t = 0; t < kDfMaxE; ++t) acc[t] = 0.0;
    for (size_t b = blockIdx.x; b < nk; b += gridDim.x) {
        __syncthreads();  // the previous k-point's tables are consumed
        for (int r = warp; r < nb; r += kDfWarps) {
            const double2* src = (r < fc ? Xk : Xkq) + ((size_t)b * nb + r) * n;
            for (int i = lane; i < n; i += 32) sx[(size_t)r * n + i] = src[i];
        }
        __syncthreads();
        for (int p = warp; p < P; p += kDfWarps) {
            const int      c = fc + p / fc, v = p - (p / fc) * fc;
            const double2* xc = sx + (size_t)c * n;
            const double2* xv = sx + (size_t)v * n;
            double         re = 0.0, im = 0.0;  // sum_i x_c[i] x_v[i] (the reference's expression)
            for (int i = lane; i < n; i += 32) {
                const double2 a = xc[i], u = xv[i];
                re = fma(a.x, u.x, fma(-a.y, u.y, re));
                im = fma(a.x, u.y, fma(a.y, u.x, im));
            }
            re = warp_sum(re);
            im = warp_sum(im);
            if (lane == 0) {
                so[p] = re * re + im * im;
                sd[p] = Ekq[b * nb + c] - Ek[b * nb + v];
            }
        }
        __syncthreads();
        const double w = wk ? wk[b] : 1.0;
#pragma unroll
        for (int t = 0; t < kDfMaxE; ++t) {
            const int e = tid + kDfThreads * t;
            if (e < ne) {  // uniform per t except in the last partial group
                const double om = en[e];
                double       s  = 0.0;
                for (int p = 0; p < P; ++p) {
                    // the pair over one denominator (one FP64 division instead of two):
                    // a / (a^2 + eta^2) + b / (b^2 + eta^2) = (a B + b A) / (A B)
                    const double d = sd[p], a = d - om, b = d + om;
                    const double A = fma(a, a, eta2), B = fma(b, b, eta2);
                    s += so[p] * (fma(a, B, b * A) / (A * B));
                }
                acc[t] += w * s;
            }
        }
    }
#pragma unroll
    for (int t = 0; t < kDfMaxE; ++t) {
        const int e = tid + kDfThreads * t;
        if (e < ne) part[(size_t)blockIdx.x * ne + e] = acc[t];
    }
}

// sums[e] += sum over the grid's partial sums, in CTA order
__global__ void k_dielectric_reduce(const double* __restrict__ part, int grid, int ne, double* __restrict__ sums) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double s = 0.0;
    for (int g = 0; g < grid; ++g) s += part[(size_t)g * ne + e];
    sums[e] += s;
}

}  // namespace
}  // namespace uepm

using namespace uepm;

extern "C" int uepm_dielectric_sums_device(const double* d_Xk, const double* d_Xkq, const double* d_Ek, const double* d_Ekq,
                                           size_t nk, int nb, int n, int first_cond, const double* d_energies, int ne,
                                           double eta, const double* d_weights, double* d_sums, void* stream) {
    if (nb <= 0 || n <= 0 || first_cond <= 0 || first_cond >= nb || ne <= 0 || ne > kDfMaxE * kDfThreads || !d_energies ||
        !d_sums || (nk && (!d_Xk || !d_Xkq || !d_Ek || !d_Ekq))) {
        set_error("uepm_dielectric_sums_device: bad argument");
        return UEPM_ERR_INVALID;
    }
    if (nk == 0) return UEPM_OK;
    cudaStream_t s    = (cudaStream_t)stream;
    const size_t smem = sizeof(double2) * (size_t)nb * n + sizeof(double) * 2 * (size_t)(nb - first_cond) * first_cond;
    if (smem > 200 * 1024) {
        set_error("uepm_dielectric_sums_device: nb x n too large for one CTA's shared memory");
        return UEPM_ERR_INVALID;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<size_t>(nk, (size_t)std::max(1, sms) * 2);
    double*   part = nullptr;
    cudaError_t e  = cudaMallocAsync(&part, sizeof(double) * (size_t)grid * ne, s);
    if (e != cudaSuccess) {
        set_error(std::string("uepm_dielectric_sums_device: ") + cudaGetErrorString(e));
        return UEPM_ERR_NOMEM;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_dielectric_sums, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_dielectric_sums<<<grid, kDfThreads, smem, s>>>(reinterpret_cast<const double2*>(d_Xk), reinterpret_cast<const double2*>(d_Xkq),
                                                      d_Ek, d_Ekq, nk, nb, n, first_cond, d_energies, ne, eta, d_weights, part);
    k_dielectric_reduce<<<(ne + 127) / 128, 128, 0, s>>>(part, grid, ne, d_sums);
    count_launch(2);
    cudaFreeAsync(part, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("uepm_dielectric_sums_device: ") + cudaGetErrorString(e));
        return UEPM_ERR_CUDA;
    }
    return UEPM_OK;
}
