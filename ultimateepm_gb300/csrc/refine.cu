// refine.cu -- FP64 Rayleigh-Ritz refinement of FP32 eigenvectors (mixed-precision path).
//
// No reference counterpart: the reference only has the FP64 Eigen solve. Given FP32 approximations
// X (n x m, m = nb + guard bands) to the lowest eigenvectors of the FP64 Hermitian H, this computes
// in FP64
//   k_refine_project   Y = H X, S = X^H X, A = X^H Y            (one CTA per matrix)
//   k_small_eigh       the m x m pencil A c = lambda S c: Cholesky S = L L^H, C = L^-1 A L^-H,
//                      cyclic Jacobi on C, ascending sort, W = L^-H V   (one THREAD per matrix:
//                      GB300's FP64 pipe costs the same per warp instruction whatever the lane mask,
//                      so the small dense solve runs 32 matrices per warp instead of one matrix per
//                      warp)
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

// interleaved small-matrix storage: element e of matrix b at base[e * batch + b]
#define SM(base, e) (base)[(size_t)(e) * batch + b]

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
    S*        Sg = small;
    S*        Ag = small + (size_t)m * m * batch;
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
        SM(Sg, p * m + q) = s;
        SM(Ag, p * m + q) = a;
        SM(Sg, q * m + p) = ST<S>::conj(s);
        SM(Ag, q * m + p) = ST<S>::conj(a);
    }
}

// One thread per matrix. small = [S | A | M | C] (m x m each, interleaved), W = m x nb (interleaved).
template <typename S>
__global__ void k_small_eigh(S* __restrict__ small, int m, int nb, double* __restrict__ Eout, S* __restrict__ Wout,
                             int* __restrict__ status, int batch) {
    using R     = double;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    S*   Sg  = small;                              // S, then L (lower)
    S*   Ag  = small + (size_t)m * m * batch;      // A, then the Jacobi matrix C
    S*   Mg  = small + (size_t)2 * m * m * batch;  // M = L^-1 A, then V
    S*   Cg  = small + (size_t)3 * m * m * batch;  // C before symmetrisation
    bool bad = false;
    // Cholesky S = L L^H
    for (int k = 0; k < m; ++k) {
        R dkk = ST<S>::re(SM(Sg, k * m + k));
        for (int j = 0; j < k; ++j) dkk -= ST<S>::norm(SM(Sg, k * m + j));
        if (!(dkk > 0.0)) {
            bad = true;
            dkk = 1.0;
        }
        const R lkk = sqrt(dkk), il = 1.0 / lkk;
        SM(Sg, k * m + k) = ST<S>::make(lkk, 0.0);
        for (int i = k + 1; i < m; ++i) {
            S s = SM(Sg, i * m + k);
            for (int j = 0; j < k; ++j) s = cfms_conjb(SM(Sg, i * m + j), SM(Sg, k * m + j), s);
            SM(Sg, i * m + k) = cscale(s, il);
        }
    }
    // M = L^-1 A
    for (int c = 0; c < m; ++c)
        for (int i = 0; i < m; ++i) {
            S s = SM(Ag, i * m + c);
            for (int j = 0; j < i; ++j) s = cfma(ST<S>::neg(SM(Sg, i * m + j)), SM(Mg, j * m + c), s);
            SM(Mg, i * m + c) = cscale(s, 1.0 / ST<S>::re(SM(Sg, i * m + i)));
        }
    // C = L^-1 M^H (Hermitian)
    for (int c = 0; c < m; ++c)
        for (int i = 0; i < m; ++i) {
            S s = ST<S>::conj(SM(Mg, c * m + i));
            for (int j = 0; j < i; ++j) s = cfma(ST<S>::neg(SM(Sg, i * m + j)), SM(Cg, j * m + c), s);
            SM(Cg, i * m + c) = cscale(s, 1.0 / ST<S>::re(SM(Sg, i * m + i)));
        }
    // symmetrise C into Ag; V = I into Mg
    for (int i = 0; i < m; ++i)
        for (int c = 0; c < m; ++c) {
            if (i < c) {
                const S u = SM(Cg, i * m + c), l = SM(Cg, c * m + i);
                const S h = ST<S>::make(0.5 * (ST<S>::re(u) + ST<S>::re(l)), 0.5 * (ST<S>::im(u) - ST<S>::im(l)));
                SM(Ag, i * m + c) = h;
                SM(Ag, c * m + i) = ST<S>::conj(h);
            } else if (i == c) {
                SM(Ag, i * m + i) = ST<S>::make(ST<S>::re(SM(Cg, i * m + i)), 0.0);
            }
            SM(Mg, i * m + c) = (i == c) ? ST<S>::one() : ST<S>::zero();
        }
    // cyclic Jacobi; a sweep without any rotation ends it (at most 12 sweeps)
    for (int sweep = 0; sweep < 12; ++sweep) {
        int rot = 0;
        for (int p = 0; p < m - 1; ++p)
            for (int q = p + 1; q < m; ++q) {
                const S bpq = SM(Ag, p * m + q);
                const R a = ST<S>::re(SM(Ag, p * m + p)), d = ST<S>::re(SM(Ag, q * m + q));
                const R ab = sqrt(ST<S>::norm(bpq));
                if (ab <= 1e-18 * (fabs(a) + fabs(d)) || ab == 0.0) continue;
                ++rot;
                const R tau = (d - a) / (2.0 * ab);
                const R t   = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const R c   = 1.0 / sqrt(1.0 + t * t), s = t * c;
                const R ex = ST<S>::re(bpq) / ab, ey = ST<S>::im(bpq) / ab;  // b = |b| e
                // J = [[c, s], [-s conj(e), c conj(e)]] on columns p, q: C <- J^H C J, V <- V J
                const S jqp = ST<S>::make(-s * ex, s * ey);
                const S jqq = ST<S>::make(c * ex, -c * ey);
                for (int r = 0; r < m; ++r) {
                    const S cp = SM(Ag, r * m + p), cq = SM(Ag, r * m + q);
                    SM(Ag, r * m + p) = cfma(cq, jqp, cscale(cp, c));
                    SM(Ag, r * m + q) = cfma(cq, jqq, cscale(cp, s));
                    const S vp = SM(Mg, r * m + p), vq = SM(Mg, r * m + q);
                    SM(Mg, r * m + p) = cfma(vq, jqp, cscale(vp, c));
                    SM(Mg, r * m + q) = cfma(vq, jqq, cscale(vp, s));
                }
                for (int r = 0; r < m; ++r) {
                    const S cp = SM(Ag, p * m + r), cq = SM(Ag, q * m + r);
                    SM(Ag, p * m + r) = cfma(ST<S>::conj(jqp), cq, cscale(cp, c));
                    SM(Ag, q * m + r) = cfma(ST<S>::conj(jqq), cq, cscale(cp, s));
                }
                SM(Ag, p * m + q) = ST<S>::zero();
                SM(Ag, q * m + p) = ST<S>::zero();
                SM(Ag, p * m + p) = ST<S>::make(ST<S>::re(SM(Ag, p * m + p)), 0.0);
                SM(Ag, q * m + q) = ST<S>::make(ST<S>::re(SM(Ag, q * m + q)), 0.0);
            }
        if (rot == 0) break;
    }
    // the nb smallest Ritz values in ascending order (selection), with their columns of V
    for (int j = 0; j < nb; ++j) {
        int kmin = j;
        R   emin = ST<S>::re(SM(Ag, j * m + j));
        for (int q = j + 1; q < m; ++q) {
            const R eq = ST<S>::re(SM(Ag, q * m + q));
            if (eq < emin) {
                emin = eq;
                kmin = q;
            }
        }
        if (kmin != j) {
            const S t = SM(Ag, j * m + j);
            SM(Ag, j * m + j) = SM(Ag, kmin * m + kmin);
            SM(Ag, kmin * m + kmin) = t;
            for (int r = 0; r < m; ++r) {
                const S v = SM(Mg, r * m + j);
                SM(Mg, r * m + j) = SM(Mg, r * m + kmin);
                SM(Mg, r * m + kmin) = v;
            }
        }
        Eout[(size_t)b * nb + j] = emin;
        if (!isfinite(emin)) bad = true;
    }
    // W = L^-H V[:, :nb] (back substitution with L^H)
    if (Wout) {
        for (int c = 0; c < nb; ++c)
            for (int i = m - 1; i >= 0; --i) {
                S s = SM(Mg, i * m + c);
                for (int j = i + 1; j < m; ++j) s = cfms_conjb(SM(Wout, j * nb + c), SM(Sg, j * m + i), s);
                SM(Wout, i * nb + c) = cscale(s, 1.0 / ST<S>::re(SM(Sg, i * m + i)));
            }
    }
    if (bad && status) atomicOr(status + b, 2);
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
    for (int j = warp; j < nb; j += nw) {
        double sx = 0, sy = 0, sz = 0;
        for (int r = lane; r < n; r += 32) {
            S x = ST<S>::zero();
            for (int q = 0; q < m; ++q) x = cfma(X[(size_t)r * m + q], SM(Wg, q * nb + j), x);
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
#undef SM

template <typename S>
void launch_refine_project(const S* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, S* work, S* small,
                           int batch, cudaStream_t s) {
    k_refine_project<S><<<batch, kProjNT, 0, s>>>(H, n, ld, mstride, X32, m, work, small, batch);
    count_launch();
}

template <typename S>
void launch_small_eigh(S* small, int m, int nb, double* Eout, S* W, int* status, int batch, cudaStream_t s) {
    k_small_eigh<S><<<(batch + 63) / 64, 64, 0, s>>>(small, m, nb, Eout, W, status, batch);
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
