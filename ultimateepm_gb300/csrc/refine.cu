// refine.cu -- FP64 Rayleigh-Ritz refinement of FP32 eigenvectors (mixed-precision path).
//
// No reference counterpart: the reference only has the FP64 Eigen solve. Given FP32 approximations
// X (n x m, m = nb + guard bands) to the lowest eigenvectors of the FP64 Hermitian H, this computes
// in FP64
//   k_refine_project   Y = H X, S = X^H X, A = X^H Y            (one CTA per matrix)
//   k_small_eigh       the m x m pencil A c = lambda S c: Cholesky S = L L^H, C = L^-1 A L^-H,
//                      parallel cyclic Jacobi on C (m/2 disjoint rotations at a time), ascending
//                      sort, W = L^-H V   (one warp per matrix, all in shared memory)
//   k_refine_vectors   Ritz vectors X W and their Hellmann-Feynman gradients (on request)
// Ritz values err by about ||H x - lambda x||^2 / gap, where the gap is to the first eigenvalue
// outside the subspace; the guard bands keep that gap open.
//
// FP64 work per matrix (complex): 4 n^2 m FMA for Y, 4 n m(m+1) for S and A, O(m^3) for the small
// solve, 4 n m nb for the refined vectors. Real symmetric matrices need a quarter of that.
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kProjNT = 256;


template <typename S>
__global__ void __launch_bounds__(kProjNT) k_refine_project(const S* __restrict__ H, int n, int ld, size_t mstride,
                                                            const cx<float>* __restrict__ X32, int m, S* __restrict__ work,
                                                            S* __restrict__ small, int batch) {
    const int b = blockIdx.x;
    if (b >= batch) return;
    const int tid = threadIdx.x;
    const S*  A   = H + (size_t)b * mstride;
    S*        X   = work + (size_t)b * refine_work_elems(n, m);  // [r][j]
    S*        Y   = X + (size_t)n * m;                             // [r][j]
    for (int q = tid; q < n * m; q += kProjNT) {
        const int       j = q / n, r = q - j * n;
        const cx<float> x = X32[((size_t)b * m + j) * n + r];
        X[(size_t)r * m + j] = ST<S>::make((double)x.x, (double)x.y);
    }
    __syncthreads();
    // Y = H X (H in full storage): item = (block of 4 vectors, row r); H(r, c) coalesced over r
    const int nblk = (m + 3) / 4;
    for (int item = tid; item < nblk * n; item += kProjNT) {
        const int jb = item / n, r = item - jb * n;
        const int j0 = jb * 4;
        S         acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = ST<S>::zero();
        if (j0 + 4 <= m) {
            for (int c = 0; c < n; ++c) {
                const S  h  = ldc(A + (size_t)c * ld + r);
                const S* xr = X + (size_t)c * m + j0;
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[q] = cfma(h, xr[q], acc[q]);
            }
        } else {
            for (int c = 0; c < n; ++c) {
                const S  h  = ldc(A + (size_t)c * ld + r);
                const S* xr = X + (size_t)c * m + j0;
                for (int q = 0; q < m - j0; ++q) acc[q] = cfma(h, xr[q], acc[q]);
            }
        }
        for (int q = 0; q < 4 && j0 + q < m; ++q) Y[(size_t)r * m + j0 + q] = acc[q];
    }
    __syncthreads();
    // S = X^H X and A = X^H Y, upper triangles (p <= q) only
    S*        Sg = small + (size_t)b * refine_small_elems(m, 0);
    S*        Ag = Sg + (size_t)m * m;
    const int np = m * (m + 1) / 2;
    for (int k = tid; k < np; k += kProjNT) {
        int p = 0, rest = k;
        while (rest >= m - p) {
            rest -= m - p;
            ++p;
        }
        const int q = p + rest;
        S         s = ST<S>::zero(), a = ST<S>::zero();
        for (int r = 0; r < n; ++r) {
            const S xp = X[(size_t)r * m + p];
            s          = cfmac(xp, X[(size_t)r * m + q], s);
            a          = cfmac(xp, Y[(size_t)r * m + q], a);
        }
        Sg[p * m + q] = s;
        Ag[p * m + q] = a;
        Sg[q * m + p] = ST<S>::conj(s);
        Ag[q * m + p] = ST<S>::conj(a);
    }
}

// One WARP per matrix; L, C and V live in shared memory. small = [S | A | W] per matrix, contiguous.
// The Jacobi sweeps rotate m/2 disjoint pairs at once (round-robin tournament order), the lanes of
// the warp computing the pairs' rotations and then sharing the row/column updates, so FP64
// instructions are issued with most lanes busy.
constexpr int kSmallWarps = 2;

// shared memory of one warp's matrix: L, C, V (m x (m+1) scalars each) and 4 rotation arrays
template <typename S>
__host__ __device__ inline size_t small_eigh_warp_bytes(int m) {
    const int me = (m + 1) & ~1;
    return (sizeof(S) * 3 * (size_t)m * (m + 1) + sizeof(double) * 4 * (size_t)me + 15) & ~(size_t)15;
}

template <typename S>
__global__ void __launch_bounds__(32 * kSmallWarps) k_small_eigh(S* __restrict__ small, int m, int nb, double* __restrict__ Eout,
                                                                 int want_w, int* __restrict__ status, int batch) {
    using R         = double;
    const int warp  = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b     = blockIdx.x * kSmallWarps + warp;
    const int mp    = m + 1;                       // padded row length
    const int me    = (m + 1) & ~1;                // m rounded up to even (tournament size)
    extern __shared__ __align__(16) unsigned char smraw[];
    S*  L    = reinterpret_cast<S*>(smraw + (size_t)warp * small_eigh_warp_bytes<S>(m));
    S*  Cm   = L + (size_t)m * mp;
    S*  V    = Cm + (size_t)m * mp;
    R*  rc   = reinterpret_cast<R*>(V + (size_t)m * mp);  // per pair: cosine
    R*  rs   = rc + me;                                   // sine
    R*  rex  = rs + me;                                   // unit phase e of the off-diagonal (re, im)
    R*  rey  = rex + me;
    if (b >= batch) return;
    S*       Sg  = small + (size_t)b * refine_small_elems(m, nb);
    const S* Ag  = Sg + (size_t)m * m;
    S*       Wg  = Sg + (size_t)2 * m * m;
    bool     bad = false;
#define LL(i, j) L[(size_t)(i) * mp + (j)]
#define CC(i, j) Cm[(size_t)(i) * mp + (j)]
#define VV(i, j) V[(size_t)(i) * mp + (j)]
    for (int q = lane; q < m * m; q += 32) {
        const int i = q / m, j = q - i * m;
        LL(i, j)    = Sg[q];
        VV(i, j)    = Ag[q];  // A, overwritten below
    }
    __syncwarp();
    // FP32 eigenvectors are orthonormal to ~1e-6, so S = I + E with a small E and, to first order,
    // S^-1/2 = I - E/2 (Loewdin): C = A - (E A + A E)/2 and W = (I - E/2) V, with an O(|E|^2 |A|)
    // error (~1e-11 eV at |E| = 1e-6). When some |E_ij| exceeds 1e-4 the Cholesky route runs instead.
    R emax = 0;
    for (int q = lane; q < m * m; q += 32) {
        const int i = q / m, j = q - i * m;
        const S   e = (i == j) ? ST<S>::make(ST<S>::re(LL(i, j)) - 1.0, ST<S>::im(LL(i, j))) : LL(i, j);
        emax        = fmax(emax, sqrt(ST<S>::norm(e)));
    }
    emax             = warp_max(emax);
    const bool lowdin = emax <= 1e-4;
    if (lowdin) {
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            S         acc = ST<S>::zero();
            for (int j = 0; j < m; ++j) {
                const S eij = (i == j) ? ST<S>::make(ST<S>::re(LL(i, j)) - 1.0, ST<S>::im(LL(i, j))) : LL(i, j);
                const S ejc = (j == c) ? ST<S>::make(ST<S>::re(LL(j, c)) - 1.0, ST<S>::im(LL(j, c))) : LL(j, c);
                acc         = cfma(eij, VV(j, c), acc);
                acc         = cfma(VV(i, j), ejc, acc);
            }
            CC(i, c) = cfma(acc, ST<S>::make(-0.5, 0.0), VV(i, c));
        }
        __syncwarp();
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            VV(i, c)    = CC(i, c);
        }
        __syncwarp();
    }
    // Cholesky S = L L^H (lanes over rows)
    for (int k = 0; k < m && !lowdin; ++k) {
        R dkk = ST<S>::re(LL(k, k));
        for (int j = 0; j < k; ++j) dkk -= ST<S>::norm(LL(k, j));
        if (!(dkk > 0.0)) {
            bad = true;
            dkk = 1.0;
        }
        const R lkk = sqrt(dkk), il = 1.0 / lkk;
        __syncwarp();
        for (int i = k + 1 + lane; i < m; i += 32) {
            S s = LL(i, k);
            for (int j = 0; j < k; ++j) s = cfms_conjb(LL(i, j), LL(k, j), s);
            LL(i, k) = cscale(s, il);
        }
        __syncwarp();
        if (lane == 0) LL(k, k) = ST<S>::make(lkk, 0.0);
        __syncwarp();
    }
    // M = L^-1 A into C (lanes over columns), then L^-1 M^H into V; symmetrised into C below.
    if (!lowdin) {
        for (int c = lane; c < m; c += 32)
            for (int i = 0; i < m; ++i) {
                S s = VV(i, c);
                for (int j = 0; j < i; ++j) s = cfma(ST<S>::neg(LL(i, j)), CC(j, c), s);
                CC(i, c) = cscale(s, 1.0 / ST<S>::re(LL(i, i)));
            }
        __syncwarp();
        for (int c = lane; c < m; c += 32)
            for (int i = 0; i < m; ++i) {
                S s = ST<S>::conj(CC(c, i));
                for (int j = 0; j < i; ++j) s = cfma(ST<S>::neg(LL(i, j)), VV(j, c), s);
                VV(i, c) = cscale(s, 1.0 / ST<S>::re(LL(i, i)));
            }
        __syncwarp();
    }
    // C = (V + V^H) / 2, V = I
    for (int q = lane; q < m * m; q += 32) {
        const int i = q / m, c = q - i * m;
        if (i <= c) {
            const S u = VV(i, c), l = VV(c, i);
            const S h = ST<S>::make(0.5 * (ST<S>::re(u) + ST<S>::re(l)), i == c ? 0.0 : 0.5 * (ST<S>::im(u) - ST<S>::im(l)));
            CC(i, c)  = h;
            CC(c, i)  = ST<S>::conj(h);
        }
    }
    __syncwarp();
    for (int q = lane; q < m * m; q += 32) {
        const int i = q / m, c = q - i * m;
        VV(i, c)    = (i == c) ? ST<S>::one() : ST<S>::zero();
    }
    __syncwarp();
    // parallel cyclic Jacobi: me - 1 rounds of me / 2 disjoint pairs per sweep
    const int npair = me / 2;
    for (int sweep = 0; sweep < 10; ++sweep) {
        R off = 0, dia = 0;
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            if (i < c) off = fmax(off, sqrt(ST<S>::norm(CC(i, c))));
            if (i == c) dia = fmax(dia, fabs(ST<S>::re(CC(i, i))));
        }
        off = warp_max(off);
        dia = warp_max(dia);
        // remaining off-diagonals move the Ritz values by at most ~off (degenerate pairs) or
        // off^2 / gap: 1e-10 of the largest diagonal is ~2e-9 eV here
        if (off <= 1e-10 * dia || off == 0.0) break;
        for (int round = 0; round < me - 1; ++round) {
            // tournament pairing: slot 0 fixed, slots 1..me-1 rotate
            if (lane < npair) {
                const int a0 = (lane == 0) ? 0 : ((lane - 1 + round) % (me - 1)) + 1;
                const int a1 = ((me - 2 - lane + round) % (me - 1)) + 1;
                const int p = min(a0, a1), q = max(a0, a1);
                R         cc = 1.0, ss = 0.0, ex = 1.0, ey = 0.0;
                if (q < m) {
                    const S bpq = CC(p, q);
                    const R ab  = sqrt(ST<S>::norm(bpq));
                    const R a = ST<S>::re(CC(p, p)), d = ST<S>::re(CC(q, q));
                    if (ab > 1e-18 * (fabs(a) + fabs(d)) && ab != 0.0) {
                        const R tau = (d - a) / (2.0 * ab);
                        const R t   = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        cc          = 1.0 / sqrt(1.0 + t * t);
                        ss          = t * cc;
                        ex          = ST<S>::re(bpq) / ab;
                        ey          = ST<S>::im(bpq) / ab;
                    }
                }
                rc[lane]  = cc;
                rs[lane]  = ss;
                rex[lane] = ex;
                rey[lane] = ey;
            }
            __syncwarp();
            // columns: C <- C J, V <- V J  (work items: pair x row)
            for (int it = lane; it < npair * m; it += 32) {
                const int k = it / m, r = it - k * m;
                const int a0 = (k == 0) ? 0 : ((k - 1 + round) % (me - 1)) + 1;
                const int a1 = ((me - 2 - k + round) % (me - 1)) + 1;
                const int p = min(a0, a1), q = max(a0, a1);
                if (q >= m) continue;
                const R c = rc[k], s = rs[k];
                if (s == 0.0 && c == 1.0) continue;
                const R ex = rex[k], ey = rey[k];
                const S jqp = ST<S>::make(-s * ex, s * ey);
                const S jqq = ST<S>::make(c * ex, -c * ey);
                const S cp = CC(r, p), cq = CC(r, q);
                CC(r, p) = cfma(cq, jqp, cscale(cp, c));
                CC(r, q) = cfma(cq, jqq, cscale(cp, s));
                const S vp = VV(r, p), vq = VV(r, q);
                VV(r, p) = cfma(vq, jqp, cscale(vp, c));
                VV(r, q) = cfma(vq, jqq, cscale(vp, s));
            }
            __syncwarp();
            // rows: C <- J^H C
            for (int it = lane; it < npair * m; it += 32) {
                const int k = it / m, r = it - k * m;
                const int a0 = (k == 0) ? 0 : ((k - 1 + round) % (me - 1)) + 1;
                const int a1 = ((me - 2 - k + round) % (me - 1)) + 1;
                const int p = min(a0, a1), q = max(a0, a1);
                if (q >= m) continue;
                const R c = rc[k], s = rs[k];
                if (s == 0.0 && c == 1.0) continue;
                const R ex = rex[k], ey = rey[k];
                const S jqp = ST<S>::make(-s * ex, s * ey);
                const S jqq = ST<S>::make(c * ex, -c * ey);
                const S cp = CC(p, r), cq = CC(q, r);
                CC(p, r) = cfma(ST<S>::conj(jqp), cq, cscale(cp, c));
                CC(q, r) = cfma(ST<S>::conj(jqq), cq, cscale(cp, s));
            }
            __syncwarp();
            if (lane < npair) {
                const int a0 = (lane == 0) ? 0 : ((lane - 1 + round) % (me - 1)) + 1;
                const int a1 = ((me - 2 - lane + round) % (me - 1)) + 1;
                const int p = min(a0, a1), q = max(a0, a1);
                if (q < m && !(rs[lane] == 0.0 && rc[lane] == 1.0)) {
                    CC(p, q) = ST<S>::zero();
                    CC(q, p) = ST<S>::zero();
                    CC(p, p) = ST<S>::make(ST<S>::re(CC(p, p)), 0.0);
                    CC(q, q) = ST<S>::make(ST<S>::re(CC(q, q)), 0.0);
                }
            }
            __syncwarp();
        }
    }
    // ascending order of the Ritz values (lane 0), nb smallest out
    int* ord = reinterpret_cast<int*>(rc);  // reuse: 4 me doubles hold m ints
    if (lane == 0) {
        for (int i = 0; i < m; ++i) ord[i] = i;
        for (int i = 1; i < m; ++i) {
            const int o = ord[i];
            const R   ev = ST<S>::re(CC(o, o));
            int       k  = i - 1;
            while (k >= 0 && ST<S>::re(CC(ord[k], ord[k])) > ev) {
                ord[k + 1] = ord[k];
                --k;
            }
            ord[k + 1] = o;
        }
    }
    __syncwarp();
    for (int j = lane; j < nb; j += 32) {
        const R ev = ST<S>::re(CC(ord[j], ord[j]));
        Eout[(size_t)b * nb + j] = ev;
        if (!isfinite(ev)) bad = true;
    }
    // W = (I - E/2) V[:, ord[:nb]] (Loewdin) or L^-H V[:, ord[:nb]] (Cholesky)
    if (want_w && lowdin) {
        for (int q = lane; q < m * nb; q += 32) {
            const int i = q / nb, c = q - i * nb;
            const int oc = ord[c];
            S         acc = ST<S>::zero();
            for (int j = 0; j < m; ++j) {
                const S eij = (i == j) ? ST<S>::make(ST<S>::re(LL(i, j)) - 1.0, ST<S>::im(LL(i, j))) : LL(i, j);
                acc         = cfma(eij, VV(j, oc), acc);
            }
            Wg[(size_t)i * nb + c] = cfma(acc, ST<S>::make(-0.5, 0.0), VV(i, oc));
        }
    }
    if (want_w && !lowdin) {
        for (int c = lane; c < nb; c += 32) {
            const int oc = ord[c];
            for (int i = m - 1; i >= 0; --i) {
                S s = VV(i, oc);
                for (int j = i + 1; j < m; ++j) s = cfms_conjb(Wg[(size_t)j * nb + c], LL(j, i), s);
                Wg[(size_t)i * nb + c] = cscale(s, 1.0 / ST<S>::re(LL(i, i)));
            }
        }
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad && lane == 0 && status) atomicOr(status + b, 2);
#undef LL
#undef CC
#undef VV
}

// Ritz vectors x_j = X W[:, j] and gradients; one CTA per matrix, one warp per band.
template <typename S>
__global__ void k_refine_vectors(int n, int m, int nb, const S* __restrict__ work, const S* __restrict__ Wg,
                                 cx<double>* __restrict__ Xout, double* __restrict__ grad, const DevParams P,
                                 const double* __restrict__ kpts, const int* __restrict__ G, int batch) {
    const int b = blockIdx.x;
    if (b >= batch) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const S*  X    = work + (size_t)b * refine_work_elems(n, m);
    const S*  Wb   = Wg + (size_t)b * refine_small_elems(m, nb);
    for (int j = warp; j < nb; j += nw) {
        double sx = 0, sy = 0, sz = 0;
        for (int r = lane; r < n; r += 32) {
            S x = ST<S>::zero();
            for (int q = 0; q < m; ++q) x = cfma(X[(size_t)r * m + q], Wb[(size_t)q * nb + j], x);
            if (Xout) stc(Xout + ((size_t)b * nb + j) * n + r, mk<double>(ST<S>::re(x), ST<S>::im(x)));
            if (grad) {
                const double* k  = kpts + 3 * (size_t)b;
                const int     bi = (r < P.N) ? r : r - P.N;
                const double  w  = ST<S>::norm(x);
                sx += (k[0] + G[3 * bi]) * w;
                sy += (k[1] + G[3 * bi + 1]) * w;
                sz += (k[2] + G[3 * bi + 2]) * w;
            }
        }
        if (grad) {
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

template <typename S>
void launch_refine_project(const S* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, S* work, S* small,
                           int batch, cudaStream_t s) {
    k_refine_project<S><<<batch, kProjNT, 0, s>>>(H, n, ld, mstride, X32, m, work, small, batch);
    count_launch();
}

template <typename S>
void launch_small_eigh(S* small, int m, int nb, double* Eout, S* W, int* status, int batch, cudaStream_t s) {
    const size_t smem = small_eigh_warp_bytes<S>(m) * kSmallWarps;
    auto         kern = k_small_eigh<S>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<(batch + kSmallWarps - 1) / kSmallWarps, 32 * kSmallWarps, smem, s>>>(small, m, nb, Eout, W != nullptr, status,
                                                                              batch);
    count_launch();
}

template <typename S>
void launch_refine_vectors(int n, int m, int nb, const S* work, const S* W, cx<double>* Xout, double* grad,
                           const DevParams& P, const double* d_k, const int* d_G, int batch, cudaStream_t s) {
    k_refine_vectors<S><<<batch, 256, 0, s>>>(n, m, nb, work, W, Xout, grad, P, d_k, d_G, batch);
    count_launch();
}

#define UEPM_RF_INST(S)                                                                                             \
    template void launch_refine_project<S>(const S*, int, int, size_t, const cx<float>*, int, S*, S*, int, cudaStream_t); \
    template void launch_small_eigh<S>(S*, int, int, double*, S*, int*, int, cudaStream_t);                        \
    template void launch_refine_vectors<S>(int, int, int, const S*, const S*, cx<double>*, double*, const DevParams&,   \
                                           const double*, const int*, int, cudaStream_t);
UEPM_RF_INST(double)
UEPM_RF_INST(cx<double>)
#undef UEPM_RF_INST

}  // namespace uepm
