// backtransform.cu -- eigenvectors of H from those of T (x = Q z, Q = H_0 H_1 ... H_{n-2}) and the
// Hellmann-Feynman kinetic gradient of each band (Hamiltonian::compute_gradient_at_level,
// src/EPP/Hamiltonian.cpp:146-194).
//
// One CTA per matrix. The reflectors are staged in shared memory in blocks of KB (coalesced copies
// of the reflector columns, the implicit unit element written out), so each is read from memory
// once however many vectors it is applied to. Each vector belongs to a group of LPV lanes (lane gl
// owns rows gl + LPV t, t < T) and stays in registers through all n-1 reflectors: per reflector and
// vector, v^H z over the group (a log2(LPV)-level butterfly) and z -= (tau v^H z) v, i.e. the
// 8 n^2 nb algorithmic flops of the back-transformation (2 n^2 nb for real symmetric matrices).
// Rows at or above the reflector's first row are skipped in whole chunks (t < (i + 1) / LPV).
// Output vectors are complex (the C ABI layout) whatever the arithmetic.
#include <algorithm>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kBtMaxWarps = 8;


// Start of reflector i in the packed staging of reflectors 0, 1, ...: reflector i' keeps the rows
// LPV floor((i' + 1) / LPV) .. ldv - 1, so the first i rows sum to
// i ldv - LPV sum_{q=1..i} floor(q / LPV) = i ldv - LPV (LPV c (c - 1) / 2 + c (i - c LPV + 1)), c = floor(i / LPV).
template <int LPV>
__host__ __device__ __forceinline__ int packed_off(int i, int ldv) {
    const int c = i / LPV;
    return i * ldv - LPV * (LPV * c * (c - 1) / 2 + c * (i - c * LPV + 1));
}
constexpr int kBtStageBytes = 48 << 10;

template <typename S, int LPV, int T>
__global__ void __launch_bounds__(32 * kBtMaxWarps) k_backtransform(const S* __restrict__ H, int n, int ld, size_t mstride,
                                                                   const S* __restrict__ tq,
                                                                   const typename ST<S>::R* __restrict__ z, int nb, int cap,
                                                                   cx<typename ST<S>::R>* __restrict__ Xout,
                                                                   const DevParams P, const double* __restrict__ kpts,
                                                                   const int* __restrict__ G, double* __restrict__ grad,
                                                                   int batch) {
    using R          = typename ST<S>::R;
    const int     b  = blockIdx.x;
    if (b >= batch) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    // Reflector i is zero on rows <= i, i.e. on the row chunks t < tc(i) = (i + 1) / LPV of every
    // lane, so it is staged packed: rows LPV tc(i) .. ldv - 1 only (ldv = LPV T, the rows from n on
    // zero, so that every chunk t < T is valid and no per-chunk bound is needed), at
    // packed_off(i) - packed_off(i0) in a block [i0, i1] of reflectors whose packed rows fit `cap`
    // elements. At basis 137 (FP32, T = 18) all 136 reflectors take 43 KB: one block, one wait.
    const int ldv  = LPV * T;
    S*        Vs   = reinterpret_cast<S*>(smraw);  // [cap] packed reflector rows
    S*        taus = Vs + cap;                     // [n]
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, gl = lane & (LPV - 1);
    const int warp = tid >> 5, nwarp = nthr >> 5;
    const int grp = tid / LPV, ngrp = nthr / LPV;
    const S*  A   = H + (size_t)b * mstride;
    const S*  tb  = tq + (size_t)b * n;
    const int nch = (nb + ngrp - 1) / ngrp;  // vector chunks (uniform over the CTA)
    for (int ch = 0; ch < nch; ++ch) {
        const int  j   = ch * ngrp + grp;
        const bool has = j < nb;
        S          zr[T];
        int        i0 = 0;
        if (n < 2) {  // no reflectors: the vectors are those of T
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const int r = gl + LPV * t;
                zr[t]       = ST<S>::make((has && r < n) ? z[((size_t)b * nb + j) * n + r] : R(0), R(0));
            }
        }
        for (int i1 = n - 2; i1 >= 0; i1 = i0 - 1) {
            // smallest i0 whose block [i0, i1] fits (one reflector always does: cap >= ldv)
            const int end = packed_off<LPV>(i1 + 1, ldv);
            int       lo = 0, hi = i1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (end - packed_off<LPV>(mid, ldv) <= cap) hi = mid;
                else lo = mid + 1;
            }
            i0             = lo;
            const int off0 = packed_off<LPV>(i0, ldv);
            __syncthreads();  // previous block consumed
            // asynchronous element copies: every load of the block is in flight at once, so the
            // memory latency is paid once per block rather than once per element of each thread
            for (int i = i0 + warp; i <= i1; i += nwarp) {
                const int r0 = LPV * ((i + 1) / LPV);
                const S*  ac = A + (size_t)i * ld;
                S*        vs = Vs + (packed_off<LPV>(i, ldv) - off0) - r0;
                for (int r = r0 + lane; r < ldv; r += 32) {
                    if (r > i + 1 && r < n) {
                        // per real component: each copy is then aligned to its own size
                        const R* src = reinterpret_cast<const R*>(ac + r);
                        R*       dst = reinterpret_cast<R*>(vs + r);
                        cp_async_elem<sizeof(R)>(dst, src);
                        if constexpr (sizeof(S) != sizeof(R)) cp_async_elem<sizeof(R)>(dst + 1, src + 1);
                    } else {
                        vs[r] = (r == i + 1) ? ST<S>::one() : ST<S>::zero();
                    }
                }
            }
            for (int i = i0 + tid; i <= i1; i += nthr) taus[i] = tb[i];
            if (i1 == n - 2) {  // first block: the vectors load while the reflectors are in flight
#pragma unroll
                for (int t = 0; t < T; ++t) {
                    const int r = gl + LPV * t;
                    zr[t]       = ST<S>::make((has && r < n) ? z[((size_t)b * nb + j) * n + r] : R(0), R(0));
                }
            }
            cp_async_wait_all();
            __syncthreads();
            // the reflectors in runs of equal tc; with the run loop unrolled tc is a constant, so
            // the dead chunks are not issued at all
#pragma unroll
            for (int tc = T - 1; tc >= 0; --tc) {
                const int ihi = min(i1, LPV * tc + LPV - 2), ilo = max(i0, LPV * tc - 1);
                if (ihi < ilo) continue;
                const int len  = ldv - LPV * tc;
                const S*  vrow = Vs + (packed_off<LPV>(ihi, ldv) - off0) - LPV * tc + gl;
                for (int i = ihi; i >= ilo; --i, vrow -= len) {
                    const S tau = taus[i];
                    if (ST<S>::re(tau) == R(0) && ST<S>::im(tau) == R(0)) continue;  // uniform
                    S dot0 = ST<S>::zero(), dot1 = ST<S>::zero();
#pragma unroll
                    for (int t = tc; t < T; ++t) {
                        if ((t - tc) & 1) dot1 = cfmac(vrow[LPV * t], zr[t], dot1);
                        else dot0 = cfmac(vrow[LPV * t], zr[t], dot0);
                    }
                    S dot = cadd(dot0, dot1);
#pragma unroll
                    for (int o = LPV / 2; o > 0; o >>= 1) {
                        if constexpr (sizeof(S) == sizeof(R)) {
                            dot += __shfl_xor_sync(0xffffffffu, dot, o);
                        } else {
                            dot = ST<S>::make(ST<S>::re(dot) + __shfl_xor_sync(0xffffffffu, ST<S>::re(dot), o),
                                              ST<S>::im(dot) + __shfl_xor_sync(0xffffffffu, ST<S>::im(dot), o));
                        }
                    }
                    const S sdt = ST<S>::neg(cmul(tau, dot));
#pragma unroll
                    for (int t = tc; t < T; ++t) zr[t] = cfma(vrow[LPV * t], sdt, zr[t]);
                }
            }
        }
        if (Xout && has) {
            cx<R>* xo = Xout + ((size_t)b * nb + j) * n;
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const int r = gl + LPV * t;
                if (r < n) stc(xo + r, mk<R>(ST<S>::re(zr[t]), ST<S>::im(zr[t])));
            }
        }
        if (grad) {
            double sx = 0, sy = 0, sz = 0;
            if (has) {
                const double* k = kpts + 3 * (size_t)b;
#pragma unroll
                for (int t = 0; t < T; ++t) {
                    const int r = gl + LPV * t;
                    if (r < n) {
                        const int    bi = (r < P.N) ? r : r - P.N;
                        const double w  = (double)ST<S>::norm(zr[t]);
                        sx += (k[0] + G[3 * bi]) * w;
                        sy += (k[1] + G[3 * bi + 1]) * w;
                        sz += (k[2] + G[3 * bi + 2]) * w;
                    }
                }
            }
#pragma unroll
            for (int o = LPV / 2; o > 0; o >>= 1) {
                sx += __shfl_xor_sync(0xffffffffu, sx, o);
                sy += __shfl_xor_sync(0xffffffffu, sy, o);
                sz += __shfl_xor_sync(0xffffffffu, sz, o);
            }
            if (has && gl == 0) {
                double* go = grad + ((size_t)b * nb + j) * 3;
                go[0]      = (sx * P.grad_pref) * P.frac_to_phys;
                go[1]      = (sy * P.grad_pref) * P.frac_to_phys;
                go[2]      = (sz * P.grad_pref) * P.frac_to_phys;
            }
        }
    }
}

template <typename S, int LPV, int T>
static void bt_launch(const S* H, int n, int ld, size_t mstride, const S* tq, const typename ST<S>::R* z, int nb,
                      cx<typename ST<S>::R>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                      int batch, cudaStream_t s) {
    constexpr int GW    = 32 / LPV;
    const int     warps = std::min(kBtMaxWarps, (nb + GW - 1) / GW);
    const int     ldv   = LPV * T;
    const int     total = packed_off<LPV>(std::max(n - 1, 0), ldv);  // all n - 1 reflectors
    const int     cap   = std::max(ldv, std::min(total, (int)(kBtStageBytes / sizeof(S))));
    const size_t  smem  = sizeof(S) * ((size_t)cap + n);
    auto          kern  = k_backtransform<S, LPV, T>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<batch, 32 * warps, smem, s>>>(H, n, ld, mstride, tq, z, nb, cap, Xout, P, d_k, d_G, grad, batch);
    count_launch();
}

// (lanes per vector, rows per lane): automatic is 8 lanes while a lane's rows fit about 40 register
// words, then 16 and 32; a requested lane count is honoured where its rows fit that budget.
template <typename S>
void launch_backtransform(const S* H, int n, int ld, size_t mstride, const S* tq, const typename ST<S>::R* z, int nb,
                          cx<typename ST<S>::R>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                          int batch, cudaStream_t s, int lanes) {
    constexpr bool CX   = sizeof(S) == 2 * sizeof(typename ST<S>::R);
    const int      tmax = CX ? 24 : 32;  // rows per lane within the register budget
    if (lanes != 8 && lanes != 16 && lanes != 32) lanes = 0;
    if (lanes && (n + lanes - 1) / lanes > tmax) lanes = 0;
    if (!lanes) lanes = (n + 7) / 8 <= tmax ? 8 : (n + 15) / 16 <= tmax ? 16 : 32;
    const int t = (n + lanes - 1) / lanes;
#define UEPM_BT(L_, T_) bt_launch<S, L_, T_>(H, n, ld, mstride, tq, z, nb, Xout, P, d_k, d_G, grad, batch, s)
    if (lanes == 8) {
        if (t <= 12) UEPM_BT(8, 12);
        else if (t <= 18) UEPM_BT(8, 18);
        else if (t <= 24) UEPM_BT(8, 24);
        else UEPM_BT(8, 32);
    } else if (lanes == 16) {
        if (t <= 12) UEPM_BT(16, 12);
        else if (t <= 18) UEPM_BT(16, 18);
        else if (t <= 24) UEPM_BT(16, 24);
        else UEPM_BT(16, 32);
    } else {
        if (t <= 12) UEPM_BT(32, 12);
        else UEPM_BT(32, 18);
    }
#undef UEPM_BT
}

#define UEPM_BT_INST(S)                                                                                          \
    template void launch_backtransform<S>(const S*, int, int, size_t, const S*, const ST<S>::R*, int, cx<ST<S>::R>*, \
                                          const DevParams&, const double*, const int*, double*, int, cudaStream_t, int);
UEPM_BT_INST(double)
UEPM_BT_INST(float)
UEPM_BT_INST(cx<double>)
UEPM_BT_INST(cx<float>)
#undef UEPM_BT_INST

}  // namespace uepm
