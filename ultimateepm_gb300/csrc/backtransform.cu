// backtransform.cu -- eigenvectors of H from those of T (x = Q z, Q = H_0 H_1 ... H_{n-2}) and the
// Hellmann-Feynman kinetic gradient of each band (Hamiltonian::compute_gradient_at_level,
// src/EPP/Hamiltonian.cpp:146-194).
//
// One CTA per matrix; each warp carries whole eigenvectors in registers (lane owns rows
// r = lane + 32 t) through all n-1 reflectors, so warps never synchronise with each other.
// Per reflector and vector: v^H z and z -= (tau v^H z) v over the reflector's rows, i.e. the
// 8 n^2 nb algorithmic flops of the back-transformation (2 n^2 nb for real symmetric matrices).
// Output vectors are complex (the C ABI layout) whatever the arithmetic.
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

template <typename S, int NT, int MAXT, int VPW>
__global__ void __launch_bounds__(NT) k_backtransform(const S* __restrict__ H, int n, int ld, size_t mstride,
                                                      const S* __restrict__ tq, const typename ST<S>::R* __restrict__ z, int nb,
                                                      cx<typename ST<S>::R>* __restrict__ Xout, const DevParams P,
                                                      const double* __restrict__ kpts, const int* __restrict__ G,
                                                      double* __restrict__ grad, int batch) {
    using R          = typename ST<S>::R;
    constexpr int NW = NT / 32;
    const int     b  = blockIdx.x;
    if (b >= batch) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const S*  A    = H + (size_t)b * mstride;
    const S*  tb   = tq + (size_t)b * n;
    const int tn   = (n + 31) >> 5;
    // each warp carries VPW vectors at once: one reflector load serves all of them
    for (int j0 = warp * VPW; j0 < nb; j0 += NW * VPW) {
        S zr[VPW][MAXT];
#pragma unroll
        for (int q = 0; q < VPW; ++q)
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int r = lane + 32 * t;
                zr[q][t]    = ST<S>::make((r < n && j0 + q < nb) ? z[((size_t)b * nb + j0 + q) * n + r] : R(0), R(0));
            }
        for (int i = n - 2; i >= 0; --i) {
            const S tau = tb[i];
            if (ST<S>::re(tau) == R(0) && ST<S>::im(tau) == R(0)) continue;
            const S*  vc = A + (size_t)i * ld;
            const int t0 = (i + 1) >> 5;  // first chunk holding a row > i (warp-uniform)
            S         vr[MAXT];
            S         dot[VPW];
#pragma unroll
            for (int q = 0; q < VPW; ++q) dot[q] = ST<S>::zero();
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                vr[t] = ST<S>::zero();
                if (t >= t0 && t < tn) {
                    const int r = lane + 32 * t;
                    if (r > i && r < n) vr[t] = (r == i + 1) ? ST<S>::one() : ldc(vc + r);
#pragma unroll
                    for (int q = 0; q < VPW; ++q) dot[q] = cfmac(vr[t], zr[q][t], dot[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < VPW; ++q) dot[q] = warp_sum(dot[q]);
#pragma unroll
            for (int q = 0; q < VPW; ++q) {
                const S sdt = ST<S>::neg(cmul(tau, dot[q]));
#pragma unroll
                for (int t = 0; t < MAXT; ++t)
                    if (t >= t0 && t < tn) zr[q][t] = cfma(vr[t], sdt, zr[q][t]);
            }
        }
#pragma unroll
        for (int q = 0; q < VPW; ++q) {
            const int j = j0 + q;
            if (j >= nb) break;
            if (Xout) {
                cx<R>* xo = Xout + ((size_t)b * nb + j) * n;
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {
                    const int r = lane + 32 * t;
                    if (r < n) stc(xo + r, mk<R>(ST<S>::re(zr[q][t]), ST<S>::im(zr[q][t])));
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
                        const double w  = (double)ST<S>::norm(zr[q][t]);
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
}

template <typename S, int MAXT>
static void bt_launch(const S* H, int n, int ld, size_t mstride, const S* tq, const typename ST<S>::R* z, int nb,
                      cx<typename ST<S>::R>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                      int batch, cudaStream_t s) {
    constexpr int NT    = 128;
    constexpr int words = (int)(sizeof(S) / 4);
    // vectors per warp: as many as keep the carried registers near 24 words per lane
    constexpr int VPW = (MAXT * words * 4 <= 24) ? 4 : (MAXT * words * 2 <= 24) ? 2 : 1;
    k_backtransform<S, NT, MAXT, VPW><<<batch, NT, 0, s>>>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch);
    count_launch();
}

template <typename S>
void launch_backtransform(const S* H, int n, int ld, size_t mstride, const S* tq, const typename ST<S>::R* z, int nb,
                          cx<typename ST<S>::R>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                          int batch, cudaStream_t s) {
    if (n <= 128) bt_launch<S, 4>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 160) bt_launch<S, 5>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 256) bt_launch<S, 8>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else if (n <= 384) bt_launch<S, 12>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
    else bt_launch<S, 16>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s);
}

#define UEPM_BT_INST(S)                                                                                          \
    template void launch_backtransform<S>(const S*, int, int, size_t, const S*, const ST<S>::R*, int, cx<ST<S>::R>*, \
                                          const DevParams&, const double*, const int*, double*, int, cudaStream_t);
UEPM_BT_INST(double)
UEPM_BT_INST(float)
UEPM_BT_INST(cx<double>)
UEPM_BT_INST(cx<float>)
#undef UEPM_BT_INST

}  // namespace uepm
