// tridiag_cluster.cu -- Householder reduction to tridiagonal form of matrices too large for one SM,
// one thread-block cluster of C CTAs (2..16) per matrix, the matrix held in the cluster's shared
// memory. Same algorithm and outputs as k_tridiag (tridiag.cu): d, e, tau per step and the
// reflector tails in column i of H, so the eigenvalue / eigenvector kernels are shared (the first
// half of Eigen's SelfAdjointEigenSolver behind Hamiltonian::Diagonalize,
// src/EPP/Hamiltonian.cpp:125-134).
//
// Layout: column j of the (full-storage, Hermitian) matrix lives, all n rows, in the shared memory of
// CTA j mod C, as its local column j / C. Step i (trailing block i+1..n-1):
//   cluster barrier: the owner of column i has published v (and tau, in v's unused slot i)
//   every CTA: copies v from the owner (distributed shared memory); partial product
//              p_q = A[:, own columns] v[own columns] into its own shared memory
//   cluster barrier
//   every CTA: p = sum over the C partials (distributed shared memory); w = tau p;
//              alpha = -tau/2 (w^H v); w += alpha v (each CTA holds the full w)
//   every CTA: A[:, own columns] -= v w^H + w v^H (rows and columns > i)
//   owner of column i+1: its Householder vector for the next step
// Two cluster barriers per step. Control flow is uniform over the cluster (every CTA reads the same
// tau), so all CTAs reach the same barriers; a CTA's shared memory is read by the others only
// between barriers that it also passes, and a final barrier precedes its exit.
#include <cooperative_groups.h>

#include <algorithm>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace cg = cooperative_groups;

namespace uepm {
namespace {

constexpr int kClNT = 256;
constexpr int kClNW = kClNT / 32;

// Block-wide sum (all threads get the result); red holds 2 * kClNW values.
template <typename R>
__device__ __forceinline__ R block_sum(R x, R* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    x = warp_sum(x);
    if (lane == 0) red[warp] = x;
    __syncthreads();
    R s = 0;
#pragma unroll
    for (int q = 0; q < kClNW; ++q) s += red[q];
    __syncthreads();
    return s;
}

// Householder vector of local column lc (global column j) into vb (slot j holds tau), plus the
// outputs d[j], e[j], tau[j] and the reflector tail of column j of the global matrix.
template <typename S>
__device__ void house(const S* __restrict__ Aloc, int n, int lc, int j, S* __restrict__ vb, S* __restrict__ Ag, int ld,
                      typename ST<S>::R* __restrict__ dOut, typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut,
                      typename ST<S>::R* red, bool& bad) {
    using R         = typename ST<S>::R;
    const S*  col   = Aloc + (size_t)lc * n;
    R         part  = 0;
    for (int r = j + 2 + threadIdx.x; r < n; r += kClNT) part += ST<S>::norm(col[r]);
    const R tail2 = block_sum(part, red);
    const S c0    = col[j + 1];
    const R c0r = ST<S>::re(c0), c0i = ST<S>::im(c0);
    R       beta;
    S       th, sc;
    if (tail2 <= num<R>::tiny() && c0i * c0i <= num<R>::tiny()) {
        th   = ST<S>::zero();
        sc   = ST<S>::zero();
        beta = c0r;
    } else {
        beta = sqrt(fma(c0r, c0r, fma(c0i, c0i, tail2)));
        if (c0r >= 0) beta = -beta;
        const R ib = R(1) / beta;
        th         = ST<S>::make((beta - c0r) * ib, -c0i * ib);
        const R ar = c0r - beta, ai = c0i;
        const R den = R(1) / fma(ar, ar, ai * ai);
        sc          = ST<S>::make(ar * den, -ai * den);
    }
    S* cg_ = Ag + (size_t)j * ld;
    for (int r = j + 1 + threadIdx.x; r < n; r += kClNT) {
        const S v = (r == j + 1) ? ST<S>::one() : cmul(col[r], sc);
        vb[r]     = v;
        if (r > j + 1) stc(cg_ + r, v);
    }
    if (threadIdx.x == 0) {
        vb[j]       = th;  // tau, in the slot v does not use
        const R dj  = ST<S>::re(col[j]);
        dOut[j]     = dj;
        eOut[j]     = beta;
        tqOut[j]    = th;
        stc(cg_ + j + 1, ST<S>::make(beta, R(0)));
        if (!isfinite(beta) || !isfinite(dj)) bad = true;
    }
}

template <typename S>
__global__ void __launch_bounds__(kClNT) k_tridiag_cluster(S* __restrict__ H, int n, int ld, size_t mstride,
                                                           typename ST<S>::R* __restrict__ dOut,
                                                           typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut,
                                                           int* __restrict__ status, int batch, int ncol) {
    using R            = typename ST<S>::R;
    cg::cluster_group cl = cg::this_cluster();
    const int         C  = (int)cl.num_blocks();
    const int         q  = (int)cl.block_rank();
    const int         nclusters = gridDim.x / C;
    const int         cid       = blockIdx.x / C;
    const int         tid       = threadIdx.x;
    extern __shared__ __align__(16) unsigned char smraw[];
    S* Aloc = reinterpret_cast<S*>(smraw);  // [ncol][n]
    S* vbuf = Aloc + (size_t)ncol * n;      // [2][n], published Householder vectors
    S* v    = vbuf + 2 * (size_t)n;         // [n] local copy of the current v
    S* pp   = v + n;                        // [n] this CTA's partial product
    S* w    = pp + n;                       // [n] full w
    R* red  = reinterpret_cast<R*>(w + n);  // [2 * kClNW]
    const int myc = (n - q + C - 1) / C;    // columns owned: q, q + C, ...

    for (int b = cid; b < batch; b += nclusters) {  // uniform over the cluster
        S*   Ag  = H + (size_t)b * mstride;
        bool bad = false;
        for (int idx = tid; idx < myc * n; idx += kClNT) {
            const int lc = idx / n, r = idx - lc * n;
            Aloc[(size_t)lc * n + r] = Ag[(size_t)(q + C * lc) * ld + r];
        }
        __syncthreads();
        if (q == 0 && n > 1) house(Aloc, n, 0, 0, vbuf, Ag, ld, dOut + (size_t)b * n, eOut + (size_t)b * n, tqOut + (size_t)b * n, red, bad);
        for (int i = 0; i < n - 1; ++i) {
            cl.sync();  // v of step i published; every CTA is done with step i - 1
            const int own  = i % C;
            const S*  vsrc = cl.map_shared_rank(vbuf + (size_t)(i & 1) * n, own);
            const S   tau  = vsrc[i];
            for (int r = tid; r < n; r += kClNT) v[r] = (r > i) ? vsrc[r] : ST<S>::zero();
            const bool skip = ST<S>::re(tau) == R(0) && ST<S>::im(tau) == R(0);  // same in every CTA
            __syncthreads();
            if (!skip) {
                // partial product over own columns c > i, rows r > i
                const int lc0 = (i + 1 - q + C - 1) / C;  // first own local column with c > i
                for (int r = i + 1 + tid; r < n; r += kClNT) {
                    S acc = ST<S>::zero();
                    for (int lc = lc0; lc < myc; ++lc) acc = cfma(Aloc[(size_t)lc * n + r], v[q + C * lc], acc);
                    pp[r] = acc;
                }
                cl.sync();  // partials published
                S dloc = ST<S>::zero();
                for (int r = i + 1 + tid; r < n; r += kClNT) {
                    S p = ST<S>::zero();
                    for (int qq = 0; qq < C; ++qq) p = cadd(p, cl.map_shared_rank(pp, qq)[r]);
                    const S wr = cmul(tau, p);
                    w[r]       = wr;
                    dloc       = cfmac(wr, v[r], dloc);
                }
                const R wvr = block_sum(ST<S>::re(dloc), red);
                const R wvi = block_sum(ST<S>::im(dloc), red);
                const S alpha = cscale(cmul(tau, ST<S>::make(wvr, wvi)), R(-0.5));
                for (int r = i + 1 + tid; r < n; r += kClNT) w[r] = cfma(alpha, v[r], w[r]);
                __syncthreads();
                // rank-2 update of own columns c > i, rows r > i
                for (int lc = lc0; lc < myc; ++lc) {
                    const int c  = q + C * lc;
                    const S   vc = v[c], wc = w[c];
                    S*        ac = Aloc + (size_t)lc * n;
                    for (int r = i + 1 + tid; r < n; r += kClNT) {
                        S a = ac[r];
                        a   = cfms_conjb(v[r], wc, a);
                        a   = cfms_conjb(w[r], vc, a);
                        if (r == c) a = ST<S>::make(ST<S>::re(a), R(0));
                        ac[r] = a;
                    }
                }
                __syncthreads();
            }
            // the owner of column i + 1 forms the next Householder vector
            if (i + 1 < n - 1 && q == (i + 1) % C)
                house(Aloc, n, (i + 1) / C, i + 1, vbuf + (size_t)((i + 1) & 1) * n, Ag, ld, dOut + (size_t)b * n,
                      eOut + (size_t)b * n, tqOut + (size_t)b * n, red, bad);
        }
        if (q == (n - 1) % C && tid == 0) {
            const R dl = ST<S>::re(Aloc[(size_t)((n - 1) / C) * n + n - 1]);
            dOut[(size_t)b * n + n - 1]  = dl;
            eOut[(size_t)b * n + n - 1]  = R(0);
            tqOut[(size_t)b * n + n - 1] = ST<S>::zero();
            if (!isfinite(dl)) bad = true;
        }
        if (tid == 0 && bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
        cl.sync();  // no CTA reuses or releases shared memory another may still read
    }
}

template <typename S>
size_t cluster_smem(int n, int C) {
    const int ncol = (n + C - 1) / C;
    return sizeof(S) * ((size_t)ncol * n + 5 * (size_t)n) + sizeof(typename ST<S>::R) * 2 * kClNW;
}

}  // namespace

template <typename S>
int tridiag_cluster_size(int n, int want) {
    // smallest cluster whose share of the matrix leaves room for two CTAs per SM, else one
    const int sizes[4] = {2, 4, 8, 16};
    if (want) {
        for (int C : sizes)
            if (C == want) return cluster_smem<S>(n, C) <= (220u << 10) ? C : 0;
        return 0;
    }
    for (int C : sizes)
        if (cluster_smem<S>(n, C) <= (110u << 10)) return C;
    for (int C : sizes)
        if (cluster_smem<S>(n, C) <= (220u << 10)) return C;
    return 0;
}

template <typename S>
bool launch_tridiag_cluster(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                            int* status, int batch, cudaStream_t s, int want_c) {
    const int C = tridiag_cluster_size<S>(n, want_c);
    if (!C || batch <= 0) return false;
    const size_t smem = cluster_smem<S>(n, C);
    auto         kern = k_tridiag_cluster<S>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
    if (C > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id               = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.blockDim           = dim3(kClNT);
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = s;
    cfg.attrs              = at;
    cfg.numAttrs           = 1;
    int maxc               = 0;
    cfg.gridDim            = dim3(C * std::min(batch, 1024));
    if (cudaOccupancyMaxActiveClusters(&maxc, kern, &cfg) != cudaSuccess || maxc <= 0) {
        cudaGetLastError();
        return false;
    }
    cfg.gridDim = dim3(C * std::min(batch, maxc));
    const int ncol = (n + C - 1) / C;
    if (cudaLaunchKernelEx(&cfg, kern, H, n, ld, mstride, d, e, tq, status, batch, ncol) != cudaSuccess) return false;
    count_launch();
    return true;
}

#define UEPM_TC_INST(S)                                                                                             \
    template int  tridiag_cluster_size<S>(int, int);                                                                \
    template bool launch_tridiag_cluster<S>(S*, int, int, size_t, typename ST<S>::R*, typename ST<S>::R*, S*, int*, int, \
                                            cudaStream_t, int);
UEPM_TC_INST(float)
UEPM_TC_INST(double)
UEPM_TC_INST(cx<float>)
UEPM_TC_INST(cx<double>)
#undef UEPM_TC_INST

}  // namespace uepm
