// refine.cu -- FP64 Rayleigh-Ritz refinement of FP32 eigenvectors (mixed-precision path).
//
// No reference counterpart: the reference only has the FP64 Eigen solve. Given FP32 approximations
// X (n x m, m = nb + guard bands) to the lowest eigenvectors of the FP64 Hermitian H, this computes
// in FP64
//   Y = H X,  S = X^H X,  A = X^H Y,
// solves the m x m pencil A c = lambda S c (Cholesky S = L L^H, C = L^-1 A L^-H, cyclic complex
// Jacobi on C), and returns the nb lowest Ritz values (and, on request, the Ritz vectors X L^-H V and
// their Hellmann-Feynman gradients). Ritz values err by about ||H x - lambda x||^2 / gap, where the
// gap is to the first eigenvalue outside the subspace; the guard bands keep that gap open.
//
// One CTA per matrix. FP64 work per matrix: 4 n^2 m FMA for Y, 4 n m(m+1) for S and A, O(m^3) for the
// small solve (one warp), 4 n m nb for the refined vectors.
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kRefineNT  = 256;
constexpr int kRefineMax = 40;  // largest subspace (nb + guard) handled by the warp solver

__device__ __forceinline__ cx<double> cconj(cx<double> a) { return mk(a.x, -a.y); }

__global__ void __launch_bounds__(kRefineNT) k_refine(const cx<double>* __restrict__ H, int n, int ld, size_t mstride,
                                                      const cx<float>* __restrict__ X32, int m, int nb,
                                                      double* __restrict__ Eout, cx<double>* __restrict__ Xout,
                                                      double* __restrict__ grad, const DevParams P, const double* __restrict__ kpts,
                                                      const int* __restrict__ G, cx<double>* __restrict__ work,
                                                      int* __restrict__ status, int batch) {
    const int b = blockIdx.x;
    if (b >= batch) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const cx<double>* A  = H + (size_t)b * mstride;
    cx<double>*       X  = work + (size_t)b * refine_work_elems(n, m);  // [r][j]
    cx<double>*       Y  = X + (size_t)n * m;                             // [r][j]
    extern __shared__ __align__(16) unsigned char smraw[];
    const int   mp = m + 1;  // padded row length of the m x m scratch matrices
    cx<double>* sSb = reinterpret_cast<cx<double>*>(smraw);
    cx<double>* sAb = sSb + (size_t)m * mp;
    cx<double>* sVb = sAb + (size_t)m * mp;
    double*     sE  = reinterpret_cast<double*>(sVb + (size_t)m * mp);
    int*        sOrd = reinterpret_cast<int*>(sE + kRefineMax);
    __shared__ int sBad;
#define sS(i, j) sSb[(size_t)(i) * mp + (j)]
#define sA(i, j) sAb[(size_t)(i) * mp + (j)]
#define sV(i, j) sVb[(size_t)(i) * mp + (j)]
    if (tid == 0) sBad = 0;

    // X (FP32, [j][r]) -> FP64, [r][j]
    for (int q = tid; q < n * m; q += kRefineNT) {
        const int       j = q / n, r = q - j * n;
        const cx<float> x = X32[((size_t)b * m + j) * n + r];
        X[(size_t)r * m + j] = mk((double)x.x, (double)x.y);
    }
    __syncthreads();

    // Y = H X, H Hermitian from its lower triangle; item = (4-vector block, row r)
    const int nblk = (m + 3) / 4;
    for (int item = tid; item < nblk * n; item += kRefineNT) {
        const int  jb = item / n, r = item - jb * n;
        const int  j0 = jb * 4;
        cx<double> acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = mk(0.0, 0.0);
        for (int c = 0; c < n; ++c) {
            const cx<double>  h  = (c <= r) ? ldc(A + (size_t)c * ld + r) : cconj(ldc(A + (size_t)r * ld + c));
            const cx<double>* xr = X + (size_t)c * m + j0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j0 + q < m) acc[q] = cfma(h, xr[q], acc[q]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (j0 + q < m) Y[(size_t)r * m + j0 + q] = acc[q];
    }
    __syncthreads();

    // S = X^H X and A = X^H Y (upper triangles, p <= q), one (p, q) per thread
    for (int pq = tid; pq < m * m; pq += kRefineNT) {
        const int p = pq / m, q = pq - p * m;
        if (p > q) continue;
        cx<double> s = mk(0.0, 0.0), a = mk(0.0, 0.0);
        for (int r = 0; r < n; ++r) {
            const cx<double> xp = X[(size_t)r * m + p];
            s                   = cfmac(xp, X[(size_t)r * m + q], s);
            a                   = cfmac(xp, Y[(size_t)r * m + q], a);
        }
        sS(p, q) = s;
        sA(p, q) = a;
        sS(q, p) = cconj(s);
        sA(q, p) = cconj(a);
    }
    __syncthreads();

    if (warp == 0) {
        // Cholesky S = L L^H, L stored in the lower triangle of sS (lanes over rows).
        for (int k = 0; k < m; ++k) {
            double dkk = sS(k, k).x;
            for (int j = 0; j < k; ++j) dkk -= sS(k, j).x * sS(k, j).x + sS(k, j).y * sS(k, j).y;
            if (!(dkk > 0.0)) {
                if (lane == 0) sBad = 1;
                dkk = 1.0;
            }
            const double lkk = sqrt(dkk);
            __syncwarp();
            for (int i = k + 1 + lane; i < m; i += 32) {
                cx<double> s = sS(i, k);
                for (int j = 0; j < k; ++j) s = cfms_conjb(sS(i, j), sS(k, j), s);
                sS(i, k) = cscale(s, 1.0 / lkk);
            }
            __syncwarp();
            if (lane == 0) sS(k, k) = mk(lkk, 0.0);
            __syncwarp();
        }
        // M = L^-1 A (column c per lane), stored in sV
        for (int c = lane; c < m; c += 32)
            for (int i = 0; i < m; ++i) {
                cx<double> s = sA(i, c);
                for (int j = 0; j < i; ++j) s = csub(s, cmul(sS(i, j), sV(j, c)));
                sV(i, c) = cscale(s, 1.0 / sS(i, i).x);
            }
        __syncwarp();
        // C = L^-1 M^H (C is Hermitian), stored in sA
        for (int c = lane; c < m; c += 32)
            for (int i = 0; i < m; ++i) {
                cx<double> s = cconj(sV(c, i));
                for (int j = 0; j < i; ++j) s = csub(s, cmul(sS(i, j), sA(j, c)));
                sA(i, c) = cscale(s, 1.0 / sS(i, i).x);
            }
        __syncwarp();
        // symmetrise, V = I
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            if (i < c) {
                const cx<double> u = sA(i, c), l = sA(c, i);
                const cx<double> h = mk(0.5 * (u.x + l.x), 0.5 * (u.y - l.y));
                sA(i, c)           = h;
                sA(c, i)           = cconj(h);
            } else if (i == c) {
                sA(i, i).y = 0.0;
            }
            sV(i, c) = mk(i == c ? 1.0 : 0.0, 0.0);
        }
        __syncwarp();
        // cyclic complex Jacobi: at most 12 sweeps, stop once every off-diagonal is negligible
        for (int sweep = 0; sweep < 12; ++sweep) {
            double off = 0.0, dia = 0.0;
            for (int q = lane; q < m * m; q += 32) {
                const int i = q / m, c = q - i * m;
                if (i < c) off = fmax(off, fabs(sA(i, c).x) + fabs(sA(i, c).y));
                if (i == c) dia = fmax(dia, fabs(sA(i, i).x));
            }
            off = warp_max(off);
            dia = warp_max(dia);
            if (off <= 1e-17 * dia || off == 0.0) break;
            for (int p = 0; p < m - 1; ++p)
                for (int q = p + 1; q < m; ++q) {
                    const cx<double> bpq = sA(p, q);
                    const double     ab  = sqrt(bpq.x * bpq.x + bpq.y * bpq.y);
                    if (ab <= 1e-300) continue;
                    const double     a = sA(p, p).x, d = sA(q, q).x;
                    const double     tau = (d - a) / (2.0 * ab);
                    const double     t   = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                    const double     c   = 1.0 / sqrt(1.0 + t * t), s = t * c;
                    const cx<double> e   = mk(bpq.x / ab, bpq.y / ab);  // b = |b| e
                    // J = [[c, s], [-s conj(e), c conj(e)]] on columns p, q; C <- J^H C J; V <- V J
                    const cx<double> jqp = mk(-s * e.x, s * e.y);   // -s conj(e)
                    const cx<double> jqq = mk(c * e.x, -c * e.y);   //  c conj(e)
                    for (int r = lane; r < m; r += 32) {
                        const cx<double> cp = sA(r, p), cq = sA(r, q);
                        sA(r, p) = cfma(cq, jqp, cscale(cp, c));
                        sA(r, q) = cfma(cq, jqq, cscale(cp, s));
                        const cx<double> vp = sV(r, p), vq = sV(r, q);
                        sV(r, p) = cfma(vq, jqp, cscale(vp, c));
                        sV(r, q) = cfma(vq, jqq, cscale(vp, s));
                    }
                    __syncwarp();
                    for (int r = lane; r < m; r += 32) {
                        // rows: (J^H C)_p = c C_p + conj(jqp) C_q ; (J^H C)_q = s C_p + conj(jqq) C_q
                        const cx<double> cp = sA(p, r), cq = sA(q, r);
                        sA(p, r) = cfma(cconj(jqp), cq, cscale(cp, c));
                        sA(q, r) = cfma(cconj(jqq), cq, cscale(cp, s));
                    }
                    __syncwarp();
                    if (lane == 0) {
                        sA(p, q)   = mk(0.0, 0.0);
                        sA(q, p)   = mk(0.0, 0.0);
                        sA(p, p).y = 0.0;
                        sA(q, q).y = 0.0;
                    }
                    __syncwarp();
                }
        }
        // ascending order of the Ritz values
        if (lane == 0) {
            for (int i = 0; i < m; ++i) {
                sE[i]   = sA(i, i).x;
                sOrd[i] = i;
            }
            for (int i = 1; i < m; ++i) {
                const double ev = sE[i];
                const int    o  = sOrd[i];
                int          k  = i - 1;
                while (k >= 0 && sE[k] > ev) {
                    sE[k + 1]   = sE[k];
                    sOrd[k + 1] = sOrd[k];
                    --k;
                }
                sE[k + 1]   = ev;
                sOrd[k + 1] = o;
            }
        }
        __syncwarp();
        for (int j = lane; j < nb; j += 32) {
            const double ev = sE[j];
            Eout[(size_t)b * nb + j] = ev;
            if (!isfinite(ev)) sBad = 1;
        }
        // W = L^-H V (back substitution with the upper factor L^H), into sA
        if (Xout || grad) {
            for (int c = lane; c < m; c += 32)
                for (int i = m - 1; i >= 0; --i) {
                    cx<double> s = sV(i, c);
                    for (int j = i + 1; j < m; ++j) s = cfms_conjb(sA(j, c), sS(j, i), s);
                    sA(i, c) = cscale(s, 1.0 / sS(i, i).x);
                }
        }
    }
    __syncthreads();
    if (tid == 0 && sBad && status) status[b] |= 2;
    if (!(Xout || grad)) return;

    // Ritz vectors x_j = X W[:, ord(j)] for the nb kept bands, one warp per band
    for (int j = warp; j < nb; j += kRefineNT / 32) {
        const int c  = sOrd[j];
        double    sx = 0, sy = 0, sz = 0;
        for (int r = lane; r < n; r += 32) {
            cx<double> x = mk(0.0, 0.0);
            for (int q = 0; q < m; ++q) x = cfma(X[(size_t)r * m + q], sA(q, c), x);
            if (Xout) stc(Xout + ((size_t)b * nb + j) * n + r, x);
            if (grad) {
                const double* k  = kpts + 3 * (size_t)b;
                const int     bi = (r < P.N) ? r : r - P.N;
                const double  w  = x.x * x.x + x.y * x.y;
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
#undef sS
#undef sA
#undef sV
}

void launch_refine(const cx<double>* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, int nb, double* Eout,
                   cx<double>* Xout, double* grad, const DevParams& P, const double* d_k, const int* d_G, cx<double>* work,
                   int* status, int batch, cudaStream_t s) {
    const size_t smem = sizeof(cx<double>) * 3 * (size_t)m * (m + 1) + sizeof(double) * kRefineMax + sizeof(int) * kRefineMax;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_refine<<<batch, kRefineNT, smem, s>>>(H, n, ld, mstride, X32, m, nb, Eout, Xout, grad, P, d_k, d_G, work, status, batch);
    count_launch();
}

}  // namespace uepm
