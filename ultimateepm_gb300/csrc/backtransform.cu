// backtransform.cu -- eigenvectors of H from those of T (x = Q z, Q = H_0 H_1 ... H_{n-2}) and the
// Hellmann-Feynman kinetic gradient of each band (Hamiltonian::compute_gradient_at_level,
// src/EPP/Hamiltonian.cpp:146-194).
//
// One CTA per matrix; each warp carries whole eigenvectors in registers (lane owns rows
// r = lane + 32 t) through all n-1 reflectors, so warps never synchronise with each other.
// Per reflector and vector: v^H z (4 FMA per row) and z -= (tau v^H z) v (4 FMA per row), i.e. the
// 8 n^2 nb algorithmic flops of the back-transformation.
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

template <typename T, int NT, int MAXT>
__global__ void __launch_bounds__(NT) k_backtransform(const cx<T>* __restrict__ H, int n, int ld, size_t mstride,
                                                      const cx<T>* __restrict__ tq, const T* __restrict__ z, int nb,
                                                      cx<T>* __restrict__ Xout, const DevParams P, const double* __restrict__ kpts,
                                                      const int* __restrict__ G, double* __restrict__ grad, int batch) {
    constexpr int NW = NT / 32;
    const int     b  = blockIdx.x;
    if (b >= batch) return;
    const int    lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const cx<T>* A    = H + (size_t)b * mstride;
    const cx<T>* tb   = tq + (size_t)b * n;
    for (int j = warp; j < nb; j += NW) {
        cx<T> zr[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) {
            const int r = lane + 32 * t;
            zr[t]       = mk<T>(r < n ? z[((size_t)b * nb + j) * n + r] : T(0), T(0));
        }
        for (int i = n - 2; i >= 0; --i) {
            const cx<T> tau = tb[i];
            if (tau.x == T(0) && tau.y == T(0)) continue;
            const cx<T>* vc = A + (size_t)i * ld;
            cx<T>        vr[MAXT];
            cx<T>        dot = mk<T>(0, 0);
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int r = lane + 32 * t;
                vr[t]       = mk<T>(0, 0);
                if (r > i && r < n) {
                    vr[t] = (r == i + 1) ? mk<T>(1, 0) : ldc(vc + r);
                    dot   = cfmac(vr[t], zr[t], dot);
                }
            }
            dot           = warp_sum(dot);
            const cx<T> s = cmul(tau, dot);
#pragma unroll
            for (int t = 0; t < MAXT; ++t) zr[t] = cfma(mk<T>(-vr[t].x, -vr[t].y), s, zr[t]);
        }
        if (Xout) {
            cx<T>* xo = Xout + ((size_t)b * nb + j) * n;
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int r = lane + 32 * t;
                if (r < n) stc(xo + r, zr[t]);
            }
        }
        if (grad) {
            const double* k  = kpts + 3 * (size_t)b;
            double        sx = 0, sy = 0, sz = 0;
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int r = lane + 32 * t;
                if (r < n) {
                    const int    bi = (r < P.N) ? r : r - P.N;
                    const double w  = (double)zr[t].x * (double)zr[t].x + (double)zr[t].y * (double)zr[t].y;
                    sx += (k[0] + G[3 * bi]) * w;
                    sy += (k[1] + G[3 * bi + 1]) * w;
                    sz += (k[2] + G[3 * bi + 2]) * w;
                }
            }
            sx = warp_sum(sx);
            sy = warp_sum(sy);
            sz = warp_sum(sz);
            if (lane == 0) {
                double* go = grad + ((size_t)b * nb + j) * 3;
                go[0]      = (sx * P.grad_pref) * P.frac_to_phys;
                go[1]      = (sy * P.grad_pref) * P.frac_to_phys;
                go[2]      = (sz * P.grad_pref) * P.frac_to_phys;
            }
        }
    }
}

template <typename T, int MAXT>
static void bt_launch(const cx<T>* H, int n, int ld, size_t mstride, const cx<T>* tq, const T* z, int nb, cx<T>* Xout,
                      const DevParams& P, const double* d_k, const int* d_G, double* grad, int batch, cudaStream_t s) {
    constexpr int NT = 256;
    k_backtransform<T, NT, MAXT><<<batch, NT, 0, s>>>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch);
    count_launch();
}

template <typename T>
void launch_backtransform(const cx<T>* H, int n, int ld, size_t mstride, const cx<T>* tq, const T* z, int nb, cx<T>* Xout,
                          const DevParams& P, const double* d_k, const int* d_G, double* grad, const T*, double*, int batch,
                          cudaStream_t s) {
    if (n <= 128) bt_launch<T, 4>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 160) bt_launch<T, 5>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 256) bt_launch<T, 8>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 384) bt_launch<T, 12>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else bt_launch<T, 16>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
}

template void launch_backtransform<double>(const cx<double>*, int, int, size_t, const cx<double>*, const double*, int,
                                           cx<double>*, const DevParams&, const double*, const int*, double*, const double*,
                                           double*, int, cudaStream_t);
template void launch_backtransform<float>(const cx<float>*, int, int, size_t, const cx<float>*, const float*, int, cx<float>*,
                                          const DevParams&, const double*, const int*, double*, const float*, double*, int,
                                          cudaStream_t);

}  // namespace uepm
