// tridiag.cu -- batched Householder reduction of complex Hermitian matrices to real symmetric
// tridiagonal form, one CTA per matrix (the first half of Eigen's SelfAdjointEigenSolver, called by
// Hamiltonian::Diagonalize, src/EPP/Hamiltonian.cpp:125-134).
//
// Algorithm (LAPACK zhetd2 / Eigen tridiagonalization_inplace, lower storage): for i = 0..n-2
//   v = house(A[i+1:, i])               beta real, tau = (beta - alpha) / beta
//   p = tau * A22 v                     Hermitian product from the lower triangle
//   w = p - (tau/2)(p^H v) v
//   A22 -= v w^H + w v^H                lower triangle only
// so that A = Q T Q^H with Q = H_0 ... H_{n-2}, H_i = I - tau_i v_i v_i^H. The reflector tails stay
// in A below the subdiagonal and the tau_i go to `tq`, for the back-transformation.
//
// GB300 mapping. The matrix lives in a per-k HBM workspace (L2-resident while the CTA works on
// it). Each step streams the trailing triangle twice (product, then rank-2 update). Warps own
// columns round-robin, lanes own rows r = lane + 32 t (fixed alignment), so the Hermitian product
// keeps per-lane row accumulators in registers and needs one cross-warp sum in shared memory per
// step. Each stored element costs exactly 8 FMAs in the product and 8 in the update, which is the
// 16/3 n^3 algorithmic flop count; in FP64 this kernel is bound by GB300's FP64 pipe.
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

template <typename T, int NT, int MAXT>
__global__ void __launch_bounds__(NT) k_tridiag(cx<T>* __restrict__ H, int n, int ld, size_t mstride, T* __restrict__ dOut,
                                                T* __restrict__ eOut, cx<T>* __restrict__ tqOut, int* __restrict__ status,
                                                int batch) {
    constexpr int NW = NT / 32;
    const int     b  = blockIdx.x;
    if (b >= batch) return;
    cx<T>* A = H + (size_t)b * mstride;
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T>*    v    = reinterpret_cast<cx<T>*>(smraw);  // n
    cx<T>*    w    = v + n;                            // n
    cx<T>*    pdot = w + n;                            // n
    cx<T>*    pacc = pdot + n;                         // NW * n
    T*        red  = reinterpret_cast<T*>(pacc + NW * n);  // 3 * NW
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    bool      bad = false;

    for (int i = 0; i < n - 1; ++i) {
        const int o = i + 1, m = n - o;
        cx<T>*    col = A + (size_t)i * ld + o;

        // ---- Householder vector of A[o:, i] -------------------------------------------------
        T part = 0;
        for (int r = 1 + tid; r < m; r += NT) {
            const cx<T> x = ldc(col + r);
            part          = fma(x.x, x.x, fma(x.y, x.y, part));
        }
        part = warp_sum(part);
        if (lane == 0) red[warp] = part;
        const cx<T> c0 = ldc(col);
        __syncthreads();
        T tail2 = 0;
#pragma unroll
        for (int q = 0; q < NW; ++q) tail2 += red[q];
        T     beta;
        cx<T> th, sc;
        if (tail2 <= num<T>::tiny() && c0.y * c0.y <= num<T>::tiny()) {
            th   = mk<T>(0, 0);
            sc   = mk<T>(0, 0);
            beta = c0.x;
        } else {
            beta = sqrt(fma(c0.x, c0.x, fma(c0.y, c0.y, tail2)));
            if (c0.x >= 0) beta = -beta;
            const T ib = T(1) / beta;
            th         = mk<T>((beta - c0.x) * ib, -c0.y * ib);
            // sc = 1 / (c0 - beta)
            const T ar = c0.x - beta, ai = c0.y;
            const T den = T(1) / fma(ar, ar, ai * ai);
            sc          = mk<T>(ar * den, -ai * den);
        }
        const bool skip = (th.x == T(0) && th.y == T(0));
        for (int r = tid; r < m; r += NT) {
            cx<T> vr;
            if (r == 0) {
                vr = mk<T>(1, 0);
            } else {
                vr = cmul(ldc(col + r), sc);
                stc(col + r, vr);
            }
            v[r] = vr;
        }
        if (tid == 0) {
            const T di = A[(size_t)i * ld + i].x;
            dOut[(size_t)b * n + i]  = di;
            eOut[(size_t)b * n + i]  = beta;
            tqOut[(size_t)b * n + i] = th;
            stc(col, mk<T>(beta, 0));
            if (!isfinite(beta) || !isfinite(di)) bad = true;
        }
        __syncthreads();
        if (skip) continue;

        // ---- p = A22 v (Hermitian, lower storage) ---------------------------------------------
        cx<T> acc[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) acc[t] = mk<T>(0, 0);
        for (int c = warp; c < m; c += NW) {
            const cx<T>* ac  = A + (size_t)(o + c) * ld + o;
            const cx<T>  vc  = v[c];
            cx<T>        dot = mk<T>(0, 0);
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int r = lane + 32 * t;
                if (r > c && r < m) {
                    const cx<T> a = ldc(ac + r);
                    acc[t]        = cfma(a, vc, acc[t]);
                    dot           = cfmac(a, v[r], dot);
                }
            }
            dot = warp_sum(dot);
            if (lane == 0) {
                const T acc_d = ac[c].x;
                pdot[c]       = mk<T>(fma(acc_d, vc.x, dot.x), fma(acc_d, vc.y, dot.y));
            }
        }
#pragma unroll
        for (int t = 0; t < MAXT; ++t) {
            const int r = lane + 32 * t;
            if (r < m) pacc[warp * n + r] = acc[t];
        }
        __syncthreads();

        // ---- w = tau p; alpha = -tau/2 (w^H v) -------------------------------------------------
        cx<T> part2 = mk<T>(0, 0);
        for (int r = tid; r < m; r += NT) {
            cx<T> p = pdot[r];
#pragma unroll
            for (int q = 0; q < NW; ++q) p = cadd(p, pacc[q * n + r]);
            const cx<T> wr = cmul(th, p);
            w[r]           = wr;
            part2          = cfmac(wr, v[r], part2);
        }
        part2 = warp_sum(part2);
        if (lane == 0) {
            red[NW + warp]     = part2.x;
            red[2 * NW + warp] = part2.y;
        }
        __syncthreads();
        cx<T> wv = mk<T>(0, 0);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            wv.x += red[NW + q];
            wv.y += red[2 * NW + q];
        }
        const cx<T> alpha = cscale(cmul(th, wv), T(-0.5));
        for (int r = tid; r < m; r += NT) w[r] = cfma(alpha, v[r], w[r]);
        __syncthreads();

        // ---- A22 -= v w^H + w v^H (lower) ------------------------------------------------------
        for (int c = warp; c < m; c += NW) {
            cx<T>*      ac = A + (size_t)(o + c) * ld + o;
            const cx<T> vc = v[c], wc = w[c];
            for (int r = c + lane; r < m; r += 32) {
                cx<T> a = ldc(ac + r);
                a       = cfms_conjb(v[r], wc, a);
                a       = cfms_conjb(w[r], vc, a);
                stc(ac + r, a);
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        const T dl = A[(size_t)(n - 1) * ld + (n - 1)].x;
        dOut[(size_t)b * n + n - 1] = dl;
        eOut[(size_t)b * n + n - 1] = T(0);
        tqOut[(size_t)b * n + n - 1] = mk<T>(0, 0);
        if (!isfinite(dl)) bad = true;
        if (bad && status) status[b] |= 2;  // UEPM_K_NONFINITE
    }
}

template <typename T, int NT, int MAXT>
static void tridiag_launch_t(cx<T>* H, int n, int ld, size_t mstride, T* d, T* e, cx<T>* tq, int* status, int batch,
                             cudaStream_t s) {
    const size_t smem = sizeof(cx<T>) * (size_t)(3 + NT / 32) * n + sizeof(T) * 3 * (NT / 32);
    auto         kern = k_tridiag<T, NT, MAXT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<batch, NT, smem, s>>>(H, n, ld, mstride, d, e, tq, status, batch);
    count_launch();
}

template <typename T>
void launch_tridiag(cx<T>* H, int n, int ld, size_t mstride, T* d, T* e, cx<T>* tq, int* status, int batch, cudaStream_t s) {
    // rows of the trailing matrix are at most n - 1 = 32 * MAXT
    if (n <= 129) tridiag_launch_t<T, 256, 4>(H, n, ld, mstride, d, e, tq, status, batch, s);
    else if (n <= 161) tridiag_launch_t<T, 256, 5>(H, n, ld, mstride, d, e, tq, status, batch, s);
    else if (n <= 257) tridiag_launch_t<T, 256, 8>(H, n, ld, mstride, d, e, tq, status, batch, s);
    else if (n <= 385) tridiag_launch_t<T, 256, 12>(H, n, ld, mstride, d, e, tq, status, batch, s);
    else tridiag_launch_t<T, 256, 16>(H, n, ld, mstride, d, e, tq, status, batch, s);
}

template void launch_tridiag<double>(cx<double>*, int, int, size_t, double*, double*, cx<double>*, int*, int, cudaStream_t);
template void launch_tridiag<float>(cx<float>*, int, int, size_t, float*, float*, cx<float>*, int*, int, cudaStream_t);

}  // namespace uepm
