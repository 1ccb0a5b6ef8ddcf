// tridiag.cu -- batched Householder reduction of Hermitian (or real symmetric) matrices to real
// symmetric tridiagonal form, one CTA per matrix (the first half of Eigen's SelfAdjointEigenSolver,
// called by Hamiltonian::Diagonalize, src/EPP/Hamiltonian.cpp:125-134).
//
// Algorithm (LAPACK zhetd2 / Eigen tridiagonalization_inplace): for i = 0..n-2
//   v = house(A[i+1:, i])               beta real, tau = (beta - alpha) / beta
//   p = tau * A22 v
//   w = p - (tau/2)(p^H v) v
//   A22 -= v w^H + w v^H
// so that A = Q T Q^H with Q = H_0 ... H_{n-2}, H_i = I - tau_i v_i v_i^H. The reflector tails stay
// in column i below the subdiagonal and the tau_i go to `tq`, for the back-transformation.
//
// GB300 mapping. GB300's FP64 pipe issues one warp instruction per ~16 cycles per SM whatever the
// lane mask, so the kernel is organised to issue FP64 instructions only with full lanes and only for
// algorithmic work:
//   * the matrix is kept in FULL storage (both triangles): the rank-2 update computes the lower
//     triangle and mirrors each element into the upper one (a store, no arithmetic), so the product
//     p = A22 v is a plain row-by-lane product with per-lane accumulators and no cross-lane
//     reductions (4 FMA per element, complex);
//   * chunk loops have warp-uniform bounds, so fully masked chunks are skipped, not issued;
//   * the Householder scalars (sqrt, reciprocals) are computed once per CTA by one thread.
// Per step: 4 m^2 FMA for the product + 4 m^2 for the lower-triangle update (complex), i.e. the
// 16/3 n^3 algorithmic flops (4/3 n^3 for real symmetric matrices). The matrix lives in a per-k HBM
// workspace; the 129 MB L2 holds the working set of the resident CTAs.
#include <algorithm>
#include <type_traits>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kUpd = 4;  // elements per thread per round of the rank-2 update

// SMEM = true: the matrix is copied into shared memory (leading dimension n | 1, odd, so that the
// mirrored row-wise stores do not collide on banks), reduced there, and its reflector columns are
// written back. Used where n x n fits (the FP32 reductions of the mixed path), because those are
// bound by memory latency rather than by arithmetic.
// Global-memory variant: CTAs per SM that must fit the register file (the persistent grid relies on
// several to hide L2/DRAM latency): 5 for the real and complex-FP32 matrices up to n = 161, 4 above,
// fewer for complex FP64 with many row chunks (whose accumulators alone take 4 MAXT registers).
template <typename S, int MAXT>
constexpr int tridiag_min_blocks() {
    return sizeof(S) * MAXT <= 8 * 5 ? 5 : (sizeof(S) <= 8 || MAXT <= 5 ? 4 : (MAXT <= 8 ? 3 : 2));
}

template <typename S, int NT, int MAXT, bool SMEM>
__global__ void __launch_bounds__(NT, SMEM ? 1 : tridiag_min_blocks<S, MAXT>()) k_tridiag(S* __restrict__ H, int n, int ldg, size_t mstride,
                                                typename ST<S>::R* __restrict__ dOut, typename ST<S>::R* __restrict__ eOut,
                                                S* __restrict__ tqOut, int* __restrict__ status, int batch) {
    using R       = typename ST<S>::R;
    constexpr int NW = NT / 32;
    const int lds = n | 1;
    extern __shared__ __align__(16) unsigned char smraw[];
    S*        As   = reinterpret_cast<S*>(smraw);  // SMEM: n x lds
    S*        v    = SMEM ? As + (size_t)n * lds : As;  // n
    S*        w    = v + n;                        // n
    S*        pacc = w + n;                        // NW * n
    R*        red  = reinterpret_cast<R*>(pacc + NW * n);  // 3 * NW
    __shared__ S   s_th, s_sc;
    __shared__ int s_skip;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // The grid may be smaller than the batch: each CTA reduces matrices b, b + gridDim.x, ... so the
    // number of matrices in flight (and their L2 working set) is set by the launch, not the batch.
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    S*        Ag  = H + (size_t)b * mstride;
    bool      bad = false;
    S*        A   = SMEM ? As : Ag;
    const int ld  = SMEM ? lds : ldg;
    if (SMEM) {
        for (int q = tid; q < n * n; q += NT) {
            const int c = q / n, r = q - c * n;
            As[(size_t)c * lds + r] = Ag[(size_t)c * ldg + r];
        }
        __syncthreads();
    }

    for (int i = 0; i < n - 1; ++i) {
        const int o = i + 1, m = n - o;
        S*        col = A + (size_t)i * ld + o;

        // ---- Householder vector of A[o:, i] -------------------------------------------------
        R part = 0;
        for (int r = 1 + tid; r < m; r += NT) part += ST<S>::norm(ldc(col + r));
        part = warp_sum(part);
        if (lane == 0) red[warp] = part;
        __syncthreads();
        if (tid == 0) {
            R tail2 = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) tail2 += red[q];
            const S c0 = ldc(col);
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
                // sc = 1 / (c0 - beta)
                const R ar = c0r - beta, ai = c0i;
                const R den = R(1) / fma(ar, ar, ai * ai);
                sc          = ST<S>::make(ar * den, -ai * den);
            }
            s_th   = th;
            s_sc   = sc;
            s_skip = (ST<S>::re(th) == R(0) && ST<S>::im(th) == R(0));
            const R di = ST<S>::re(A[(size_t)i * ld + i]);
            dOut[(size_t)b * n + i]  = di;
            eOut[(size_t)b * n + i]  = beta;
            tqOut[(size_t)b * n + i] = th;
            stc(col, ST<S>::make(beta, R(0)));
            if (!isfinite(beta) || !isfinite(di)) bad = true;
        }
        __syncthreads();
        const S th = s_th, sc = s_sc;
        for (int r = tid; r < m; r += NT) {
            S vr;
            if (r == 0) {
                vr = ST<S>::one();
            } else {
                vr = cmul(ldc(col + r), sc);
                stc(col + r, vr);
            }
            v[r] = vr;
        }
        __syncthreads();
        if (s_skip) continue;

        // ---- p = A22 v (full storage): warps own columns, lanes own rows ----------------------
        S acc[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) acc[t] = ST<S>::zero();
        const int tn = (m + 31) >> 5;
        // FP32 matrices beyond the on-chip sizes reduce from L2/DRAM and wait on memory: there the
        // column's chunks are all loaded before the first FMA (Ge SOC n = 362: 242 -> 220 ms per
        // 2000 k). The FP64 kernel is FP64-pipe bound and keeps the interleaved form (11.2 vs
        // 12.0 ms at n = 137), as do the shapes where the extra registers would spill.
        constexpr bool kBatchLoads = sizeof(R) == 4 && MAXT <= 12;
        for (int c = warp; c < m; c += NW) {
            const S* ac = A + (size_t)(o + c) * ld + o;
            const S  vc = v[c];
            if constexpr (kBatchLoads) {
                S a[MAXT];
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {
                    const int r = lane + 32 * t;
                    a[t]        = (t < tn && r < m) ? ldc(ac + r) : ST<S>::zero();
                }
#pragma unroll
                for (int t = 0; t < MAXT; ++t)
                    if (t < tn) acc[t] = cfma(a[t], vc, acc[t]);  // warp-uniform
            } else {
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {
                    if (t < tn) {  // warp-uniform
                        const int r = lane + 32 * t;
                        const S   a = (r < m) ? ldc(ac + r) : ST<S>::zero();
                        acc[t]      = cfma(a, vc, acc[t]);
                    }
                }
            }
        }
#pragma unroll
        for (int t = 0; t < MAXT; ++t) {
            const int r = lane + 32 * t;
            if (t < tn && r < m) pacc[warp * n + r] = acc[t];
        }
        __syncthreads();

        // ---- w = tau p; alpha = -tau/2 (w^H v) -------------------------------------------------
        S part2 = ST<S>::zero();
        for (int r = tid; r < m; r += NT) {
            S p = pacc[r];
#pragma unroll
            for (int q = 1; q < NW; ++q) p = cadd(p, pacc[q * n + r]);
            const S wr = cmul(th, p);
            w[r]       = wr;
            part2      = cfmac(wr, v[r], part2);
        }
        part2 = warp_sum(part2);
        if (lane == 0) {
            red[NW + warp]     = ST<S>::re(part2);
            red[2 * NW + warp] = ST<S>::im(part2);
        }
        __syncthreads();
        R wvr = 0, wvi = 0;
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            wvr += red[NW + q];
            wvi += red[2 * NW + q];
        }
        const S alpha = cscale(cmul(th, ST<S>::make(wvr, wvi)), R(-0.5));
        for (int r = tid; r < m; r += NT) w[r] = cfma(alpha, v[r], w[r]);
        __syncthreads();

        // ---- A22 -= v w^H + w v^H: lower triangle computed, upper mirrored -------------------
        // The m (m + 1) / 2 lower elements in column-major order, element e to thread e mod NT:
        // consecutive threads take consecutive rows of a column (coalesced), and only the last
        // round has idle lanes (per-column 32-row chunks left ~16 idle lanes in every column).
        // Each thread takes its elements kUpd at a time, all loads first, so that kUpd loads per
        // thread are in flight (one at a time left every element waiting a full L2/DRAM latency).
        {
            const int tot = m * (m + 1) / 2;
            int       c = 0, r = tid;  // (column, row) of element tid
            while (r >= m && c < m) {
                r = r - m + c + 1;
                ++c;
            }
            for (int e0 = tid; e0 < tot; e0 += kUpd * NT) {
                int cq[kUpd], rq[kUpd];
                S   aq[kUpd];
#pragma unroll
                for (int q = 0; q < kUpd; ++q) {
                    cq[q] = c;
                    rq[q] = r;
                    r += NT;  // next element of this thread
                    while (r >= m && c < m) {
                        r = r - m + c + 1;
                        ++c;
                    }
                }
#pragma unroll
                for (int q = 0; q < kUpd; ++q)
                    if (e0 + q * NT < tot) aq[q] = ldc(A + (size_t)(o + cq[q]) * ld + o + rq[q]);
#pragma unroll
                for (int q = 0; q < kUpd; ++q) {
                    if (e0 + q * NT >= tot) break;
                    const int cc = cq[q], rr = rq[q];
                    S         a  = cfms_conjb(v[rr], w[cc], aq[q]);
                    a            = cfms_conjb(w[rr], v[cc], a);
                    if (rr == cc) {
                        a = ST<S>::make(ST<S>::re(a), R(0));
                    } else {
                        stc(A + (size_t)(o + rr) * ld + (o + cc), ST<S>::conj(a));
                    }
                    stc(A + (size_t)(o + cc) * ld + o + rr, a);
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        const R dl = ST<S>::re(A[(size_t)(n - 1) * ld + (n - 1)]);
        dOut[(size_t)b * n + n - 1] = dl;
        eOut[(size_t)b * n + n - 1] = R(0);
        tqOut[(size_t)b * n + n - 1] = ST<S>::zero();
        if (!isfinite(dl)) bad = true;
        if (bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
    }
    if (SMEM) {
        // reflector tails (column i, rows i+2..n-1) for the back-transformation
        __syncthreads();
        for (int q = tid; q < n * n; q += NT) {
            const int c = q / n, r = q - c * n;
            if (r > c + 1) Ag[(size_t)c * ldg + r] = As[(size_t)c * lds + r];
        }
    }
    __syncthreads();  // shared memory is reused by the CTA's next matrix
    }
}

// ------------------------------------------------------------------------------------------------
// Fused variant for FP32 matrices reduced from L2/DRAM (beyond the on-chip sizes), where every
// step streams the trailing matrix through memory. Step j (reflector v_j on rows/columns o = j+1..):
//   (a) p_j = A v_j from the previous pass's per-warp partials; w_j = tau p_j - (tau/2)(w^H v_j) v_j
//   (b) step j's update of column o alone, then the reflector of column o (d, e, tau, v_{j+1} and
//       its tail in H)
//   (c) ONE pass over the trailing block [o+1:, o+1:]: each element gets step j's update
//       a -= v w^H + w v^H (both triangles, no mirror store) and enters p_{j+1} = A v_{j+1}
//       before it is stored.
// One read and one write per element and step, where the unfused kernel reads the block for the
// product, reads and writes the lower triangle for the update, and scatters the mirror (32-byte
// sectors for 8-byte elements). The two triangles are updated with the same products, so they stay
// Hermitian to rounding; the diagonal is kept real.
template <typename S, int NT>
__device__ __forceinline__ void fused_reflector(const S (&colv)[2], S* __restrict__ A, int ld, int n, int col,
                                                typename ST<S>::R* dB, typename ST<S>::R* eB, S* tB, S* vnext,
                                                typename ST<S>::R* red, S* s_sc, S* s_th, S* s_alpha, bool& bad) {
    using R          = typename ST<S>::R;
    constexpr int NW = NT / 32;
    const int     tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, m = n - col;
    R             part = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int rr = threadIdx.x + NT * k;
        if (rr >= m) continue;
        if (rr >= 2) part += ST<S>::norm(colv[k]);
        if (rr == 1) *s_alpha = colv[k];
        if (rr == 0) {
            const R dv = ST<S>::re(colv[k]);
            dB[col]    = dv;
            if (!isfinite(dv)) bad = true;
        }
    }
    part = warp_sum(part);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (tid == 0) {
        S th = ST<S>::zero(), sc = ST<S>::zero();
        if (m >= 2) {
            R tail2 = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) tail2 += red[q];
            const S c0 = *s_alpha;
            const R c0r = ST<S>::re(c0), c0i = ST<S>::im(c0);
            R       beta;
            if (tail2 <= num<R>::tiny() && c0i * c0i <= num<R>::tiny()) {
                beta = c0r;
            } else {
                beta = sqrt(fma(c0r, c0r, fma(c0i, c0i, tail2)));
                if (c0r >= 0) beta = -beta;
                const R ib = R(1) / beta;
                th         = ST<S>::make((beta - c0r) * ib, -c0i * ib);
                const R ar = c0r - beta, ai = c0i;
                const R den = R(1) / fma(ar, ar, ai * ai);
                sc          = ST<S>::make(ar * den, -ai * den);  // 1 / (c0 - beta)
            }
            eB[col]                                = beta;
            A[(size_t)col * ld + col + 1]          = ST<S>::make(beta, R(0));
            if (!isfinite(beta)) bad = true;
        } else {
            eB[col] = R(0);
        }
        tB[col] = th;
        *s_th   = th;
        *s_sc   = sc;
    }
    __syncthreads();
    const S sc = *s_sc;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int rr = threadIdx.x + NT * k;
        if (rr < 1 || rr >= m) continue;
        if (rr == 1) {
            vnext[0] = ST<S>::one();
        } else {
            const S x     = cmul(colv[k], sc);
            vnext[rr - 1] = x;
            stc(A + (size_t)col * ld + col + rr, x);
        }
    }
    __syncthreads();
}

template <typename S, int NT, int MAXT>
__global__ void __launch_bounds__(NT, 4) k_tridiag_fused(S* __restrict__ H, int n, int ld, size_t mstride,
                                                        typename ST<S>::R* __restrict__ dOut,
                                                        typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut,
                                                        int* __restrict__ status, int batch) {
    using R          = typename ST<S>::R;
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smraw[];
    S*        vb   = reinterpret_cast<S*>(smraw);            // [2][n] reflectors, by step parity
    S*        w    = vb + 2 * (size_t)n;                      // [n]
    S*        pacc = w + n;                                   // [NW][n] per-warp partials of A v
    R*        red  = reinterpret_cast<R*>(pacc + (size_t)NW * n);  // [3 NW]: norms | dot re | dot im
    __shared__ S s_sc, s_th, s_alpha;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        __syncthreads();  // shared memory of the previous matrix consumed
        S*   A   = H + (size_t)b * mstride;
        R*   dB  = dOut + (size_t)b * n;
        R*   eB  = eOut + (size_t)b * n;
        S*   tB  = tqOut + (size_t)b * n;
        bool bad = false;
        // ---- the reflector of column 0, then p_0 = A[1:,1:] v_0 (pass without update) ----------
        S colv[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int rr = tid + NT * k;
            colv[k]      = rr < n ? ldc(A + rr) : ST<S>::zero();
        }
        fused_reflector<S, NT>(colv, A, ld, n, 0, dB, eB, tB, vb, red, &s_sc, &s_th, &s_alpha, bad);
        S th = s_th;
        for (int j = 0; j <= n - 1; ++j) {
            // pass over the block [o+1:, o+1:] (o = j for the prologue pass at j = 0, j + 1 after):
            // prologue: product with v_0 only; step j: update with (v_j, w_j), product with v_{j+1}
            const bool pro = j == 0;
            const int  o   = pro ? 0 : j;  // the block starts at row/column o + 1
            const int  mb  = n - 1 - o;
            if (!pro && mb < 0) break;
            const S* vcur = vb + (size_t)((j - 1) & 1) * n;  // v_{j-1}: offset rows o.. (step j-1's)
            const S* vnx  = vb + (size_t)(j & 1) * n;        // v_j on rows o + 1..
            if (mb >= 1) {
                S         acc[MAXT];
#pragma unroll
                for (int t = 0; t < MAXT; ++t) acc[t] = ST<S>::zero();
                const int tn = (mb + 31) >> 5;
                // a column's chunks in groups of GS: the group's loads are issued together, then
                // updated, stored and accumulated (smaller groups for the long columns, whose
                // loads would otherwise spill)
                constexpr int GS = MAXT > 12 ? 4 : (MAXT > 8 ? (MAXT + 1) / 2 : MAXT);
                for (int C = warp; C < mb; C += NW) {
                    S*      ac = A + (size_t)(o + 1 + C) * ld + o + 1;
                    const S vn = vnx[C];
                    const S wc = pro ? ST<S>::zero() : w[C + 1], vc = pro ? ST<S>::zero() : vcur[C + 1];
#pragma unroll
                    for (int g = 0; g < MAXT; g += GS) {
                        S a[GS];
#pragma unroll
                        for (int q = 0; q < GS; ++q) {
                            const int t = g + q, Rr = lane + 32 * t;
                            a[q]        = (t < MAXT && t < tn && Rr < mb) ? ldc(ac + Rr) : ST<S>::zero();
                        }
#pragma unroll
                        for (int q = 0; q < GS; ++q) {
                            const int t = g + q, Rr = lane + 32 * t;
                            if (t < MAXT && t < tn) {  // warp-uniform
                                if (!pro && Rr < mb) {
                                    S x = cfms_conjb(vcur[Rr + 1], wc, a[q]);
                                    x   = cfms_conjb(w[Rr + 1], vc, x);
                                    if (Rr == C) x = ST<S>::make(ST<S>::re(x), R(0));
                                    stc(ac + Rr, x);
                                    a[q] = x;
                                }
                                acc[t] = cfma(a[q], vn, acc[t]);
                            }
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {
                    const int Rr = lane + 32 * t;
                    if (t < tn && Rr < mb) pacc[(size_t)warp * n + Rr] = acc[t];
                }
            }
            __syncthreads();
            // ---- step j' = (pro ? 0 : j): p = A v_{j'} (rows o + 1..), w, then column o + 1 --------
            const int col = o + 1;  // the next column to reduce
            const int m   = n - col;
            if (m < 1) break;
            const S* v = vnx;  // v_{j'} on rows col..
            S        wown[2];
            S        dot = ST<S>::zero();
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int rr = tid + NT * k;
                wown[k]      = ST<S>::zero();
                if (rr < m) {
                    S p = pacc[rr];
#pragma unroll
                    for (int q = 1; q < NW; ++q) p = cadd(p, pacc[(size_t)q * n + rr]);
                    wown[k] = cmul(th, p);
                    dot     = cfmac(wown[k], v[rr], dot);
                }
            }
            dot = warp_sum(dot);
            if (lane == 0) {
                red[NW + warp]     = ST<S>::re(dot);
                red[2 * NW + warp] = ST<S>::im(dot);
            }
            __syncthreads();
            R dr = 0, di = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                dr += red[NW + q];
                di += red[2 * NW + q];
            }
            const S alpha = cscale(cmul(th, ST<S>::make(dr, di)), R(-0.5));
            S       p0    = pacc[0];
#pragma unroll
            for (int q = 1; q < NW; ++q) p0 = cadd(p0, pacc[(size_t)q * n]);
            const S w0 = cfma(alpha, v[0], cmul(th, p0));
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int rr = tid + NT * k;
                if (rr < m) {
                    wown[k] = cfma(alpha, v[rr], wown[k]);
                    w[rr]   = wown[k];
                    // column col after the step: a -= v_r conj(w_0) + w_r conj(v_0)
                    S x = ldc(A + (size_t)col * ld + col + rr);
                    x   = cfms_conjb(v[rr], w0, x);
                    x   = cfms_conjb(wown[k], v[0], x);
                    if (rr == 0) x = ST<S>::make(ST<S>::re(x), R(0));
                    colv[k] = x;
                } else {
                    colv[k] = ST<S>::zero();
                }
            }
            // (w is read by the next pass after the reflector's barriers)
            fused_reflector<S, NT>(colv, A, ld, n, col, dB, eB, tB, vb + (size_t)((j + 1) & 1) * n, red, &s_sc, &s_th,
                                   &s_alpha, bad);
            th = s_th;
        }
        bad = __syncthreads_or(bad);
        if (tid == 0 && bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
    }
}

// Deferred variant: every other rank-2 update is held back one step. The pass after an odd step j
// (reflector v_j formed from column j with both pending updates) is read-only: it accumulates
// S v_j from the stored matrix S, which still lacks update j-1, and the vector phase corrects it,
// p_j = S v_j - v_{j-1} (w_{j-1}^H v_j) - w_{j-1} (v_{j-1}^H v_j), with the two dots formed in the
// previous vector phase. The pass after an even step applies updates j-2 and j-1 together (rank 4)
// and accumulates the exact product. Per two steps the trailing matrix is read three times and
// written once instead of read and written twice.
template <typename S, int NT, int MAXT>
__global__ void __launch_bounds__(NT, 4)
    k_tridiag_fused_deferred(S* __restrict__ H, int n, int ld, size_t mstride, typename ST<S>::R* __restrict__ dOut,
                             typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut, int* __restrict__ status,
                             int batch) {
    using R          = typename ST<S>::R;
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smraw[];
    S*        vb   = reinterpret_cast<S*>(smraw);            // [3][n]: v_j in slot j % 3 (v_j[i] <-> row j + 1 + i)
    S*        wb   = vb + 3 * (size_t)n;                      // [2][n]: w_j in slot j % 2
    S*        pacc = wb + 2 * (size_t)n;                      // [NW][n] per-warp partials of S v
    R*        red  = reinterpret_cast<R*>(pacc + (size_t)NW * n);  // [3 NW]: norms | dot re | dot im
    R*        red2 = red + 3 * NW;                            // [4 NW]: w^H v' re, im | v^H v' re, im
    __shared__ S s_sc, s_th, s_alpha;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        __syncthreads();  // shared memory of the previous matrix consumed
        S*   A   = H + (size_t)b * mstride;
        R*   dB  = dOut + (size_t)b * n;
        R*   eB  = eOut + (size_t)b * n;
        S*   tB  = tqOut + (size_t)b * n;
        bool bad = false;
        S    colv[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int rr = tid + NT * k;
            colv[k]      = rr < n ? ldc(A + rr) : ST<S>::zero();
        }
        fused_reflector<S, NT>(colv, A, ld, n, 0, dB, eB, tB, vb, red, &s_sc, &s_th, &s_alpha, bad);
        S th = s_th;
        for (int j = 0; j <= n - 1; ++j) {
            const int  mb  = n - 1 - j;  // the block [j+1:, j+1:]
            const bool odd = (j & 1) != 0;
            const bool rw  = j >= 2 && !odd;  // apply updates j-2 and j-1
            const S*   vj  = vb + (size_t)(j % 3) * n;
            const S*   v1  = vb + (size_t)((j + 2) % 3) * n;  // v_{j-1}
            const S*   v2  = vb + (size_t)((j + 1) % 3) * n;  // v_{j-2}
            const S*   w1  = wb + (size_t)((j + 1) & 1) * n;  // w_{j-1}
            const S*   w2  = wb + (size_t)(j & 1) * n;        // w_{j-2}
            if (mb >= 1) {
                S         acc[MAXT];
#pragma unroll
                for (int t = 0; t < MAXT; ++t) acc[t] = ST<S>::zero();
                const int     tn = (mb + 31) >> 5;
                constexpr int GS = MAXT > 12 ? 4 : (MAXT > 8 ? (MAXT + 1) / 2 : MAXT);
                for (int C = warp; C < mb; C += NW) {
                    S*      ac = A + (size_t)(j + 1 + C) * ld + j + 1;
                    const S vn = vj[C];
                    S       c2w = ST<S>::zero(), c2v = ST<S>::zero(), c1w = ST<S>::zero(), c1v = ST<S>::zero();
                    if (rw) {
                        c2w = w2[C + 2];
                        c2v = v2[C + 2];
                        c1w = w1[C + 1];
                        c1v = v1[C + 1];
                    }
#pragma unroll
                    for (int g = 0; g < MAXT; g += GS) {
                        S a[GS];
#pragma unroll
                        for (int q = 0; q < GS; ++q) {
                            const int t = g + q, Rr = lane + 32 * t;
                            a[q]        = (t < MAXT && t < tn && Rr < mb) ? ldc(ac + Rr) : ST<S>::zero();
                        }
#pragma unroll
                        for (int q = 0; q < GS; ++q) {
                            const int t = g + q, Rr = lane + 32 * t;
                            if (t < MAXT && t < tn) {  // warp-uniform
                                if (rw && Rr < mb) {
                                    S x = cfms_conjb(v2[Rr + 2], c2w, a[q]);
                                    x   = cfms_conjb(w2[Rr + 2], c2v, x);
                                    x   = cfms_conjb(v1[Rr + 1], c1w, x);
                                    x   = cfms_conjb(w1[Rr + 1], c1v, x);
                                    if (Rr == C) x = ST<S>::make(ST<S>::re(x), R(0));
                                    stc(ac + Rr, x);
                                    a[q] = x;
                                }
                                acc[t] = cfma(a[q], vn, acc[t]);
                            }
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {
                    const int Rr = lane + 32 * t;
                    if (t < tn && Rr < mb) pacc[(size_t)warp * n + Rr] = acc[t];
                }
            }
            __syncthreads();
            const int col = j + 1, m = n - col;
            if (m < 1) break;
            // p_j (corrected for the held-back update j-1 after a read-only pass), w_j
            S d1 = ST<S>::zero(), d2 = ST<S>::zero();
            if (odd) {
                R a1 = 0, b1 = 0, a2 = 0, b2 = 0;
#pragma unroll
                for (int q = 0; q < NW; ++q) {
                    a1 += red2[q];
                    b1 += red2[NW + q];
                    a2 += red2[2 * NW + q];
                    b2 += red2[3 * NW + q];
                }
                d1 = ST<S>::make(a1, b1);
                d2 = ST<S>::make(a2, b2);
            }
            S wown[2];
            S dot = ST<S>::zero();
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int rr = tid + NT * k;
                wown[k]      = ST<S>::zero();
                if (rr < m) {
                    S p = pacc[rr];
#pragma unroll
                    for (int q = 1; q < NW; ++q) p = cadd(p, pacc[(size_t)q * n + rr]);
                    if (odd) {
                        p = cfma(ST<S>::neg(v1[rr + 1]), d1, p);
                        p = cfma(ST<S>::neg(w1[rr + 1]), d2, p);
                    }
                    wown[k] = cmul(th, p);
                    dot     = cfmac(wown[k], vj[rr], dot);
                }
            }
            dot = warp_sum(dot);
            if (lane == 0) {
                red[NW + warp]     = ST<S>::re(dot);
                red[2 * NW + warp] = ST<S>::im(dot);
            }
            __syncthreads();
            R dr = 0, di = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                dr += red[NW + q];
                di += red[2 * NW + q];
            }
            const S alpha = cscale(cmul(th, ST<S>::make(dr, di)), R(-0.5));
            S       p0    = pacc[0];
#pragma unroll
            for (int q = 1; q < NW; ++q) p0 = cadd(p0, pacc[(size_t)q * n]);
            if (odd) {
                p0 = cfma(ST<S>::neg(v1[1]), d1, p0);
                p0 = cfma(ST<S>::neg(w1[1]), d2, p0);
            }
            const S w0  = cfma(alpha, vj[0], cmul(th, p0));
            const S c1w = odd ? w1[1] : ST<S>::zero(), c1v = odd ? v1[1] : ST<S>::zero();
            S*      wj  = wb + (size_t)(j & 1) * n;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int rr = tid + NT * k;
                if (rr < m) {
                    wown[k] = cfma(alpha, vj[rr], wown[k]);
                    wj[rr]  = wown[k];
                    // column col: the held-back update j-1 (odd j), then update j
                    S x = ldc(A + (size_t)col * ld + col + rr);
                    if (odd) {
                        x = cfms_conjb(v1[rr + 1], c1w, x);
                        x = cfms_conjb(w1[rr + 1], c1v, x);
                    }
                    x = cfms_conjb(vj[rr], w0, x);
                    x = cfms_conjb(wown[k], vj[0], x);
                    if (rr == 0) x = ST<S>::make(ST<S>::re(x), R(0));
                    colv[k] = x;
                } else {
                    colv[k] = ST<S>::zero();
                }
            }
            S* vnext = vb + (size_t)((j + 1) % 3) * n;
            fused_reflector<S, NT>(colv, A, ld, n, col, dB, eB, tB, vnext, red, &s_sc, &s_th, &s_alpha, bad);
            th = s_th;
            if (!odd && m >= 2) {
                // the dots the next (odd) step corrects with: w_j^H v_{j+1} and v_j^H v_{j+1} over rows >= j + 2
                S e1 = ST<S>::zero(), e2 = ST<S>::zero();
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int rr = tid + NT * k;
                    if (rr >= 1 && rr < m) {
                        const S vn = vnext[rr - 1];
                        e1         = cfmac(wown[k], vn, e1);
                        e2         = cfmac(vj[rr], vn, e2);
                    }
                }
                e1 = warp_sum(e1);
                e2 = warp_sum(e2);
                if (lane == 0) {
                    red2[warp]          = ST<S>::re(e1);
                    red2[NW + warp]     = ST<S>::im(e1);
                    red2[2 * NW + warp] = ST<S>::re(e2);
                    red2[3 * NW + warp] = ST<S>::im(e2);
                }
            }
        }
        bad = __syncthreads_or(bad);
        if (tid == 0 && bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
    }
}

static int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

template <typename S, int NT, int MAXT, bool SMEM>
static void tridiag_launch_t(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                             int* status, int batch, cudaStream_t s, int ctas_per_sm) {
    using R           = typename ST<S>::R;
    const size_t smem = sizeof(S) * ((SMEM ? (size_t)n * (n | 1) : 0) + (size_t)(2 + NT / 32) * n) + sizeof(R) * 3 * (NT / 32);
    auto         kern = k_tridiag<S, NT, MAXT, SMEM>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int grid = batch;
    if (!SMEM) {
        // automatic: keep the matrices in flight within ~120 MB so that they stay in the 129 MB L2
        // (FP64 at n = 137: 5 per SM, 13.1 ms for 2000 matrices against 14.1 at 4 and 14.5 at 6), but
        // never below 4 CTAs per SM: for large (complex / spin-orbit) matrices, latency hiding wins
        // over L2 residency (measured 1.5-2x over 1 CTA per SM at n = 178..458, FP32)
        const size_t bytes  = sizeof(S) * (size_t)n * n;
        int          per_sm = (int)std::max<size_t>(4, std::min<size_t>(8, (120u << 20) / (bytes * (size_t)sm_count())));
        if (ctas_per_sm > 0) per_sm = std::min(ctas_per_sm, 8);
        int fit = 0;  // never more than are resident at once: the rest would wait as a tail
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, NT, smem) == cudaSuccess && fit > 0)
            per_sm = std::min(per_sm, fit);
        grid = std::min(batch, per_sm * sm_count());
    }
    kern<<<grid, NT, smem, s>>>(H, n, ld, mstride, d, e, tq, status, batch);
    count_launch();
}

template <typename S, int MAXT, bool DEFER = false>
static void fused_launch_t(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                           int* status, int batch, cudaStream_t s, int ctas_per_sm) {
    using R           = typename ST<S>::R;
    constexpr int NT  = 256;
    const size_t  smem = DEFER ? sizeof(S) * (size_t)(5 + NT / 32) * n + sizeof(R) * 7 * (NT / 32)
                               : sizeof(S) * (size_t)(3 + NT / 32) * n + sizeof(R) * 3 * (NT / 32);
    auto          kern = DEFER ? k_tridiag_fused_deferred<S, NT, MAXT> : k_tridiag_fused<S, NT, MAXT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // matrices in flight as for the unfused kernel (L2 budget, at least 4 per SM), capped at the
    // kernel's occupancy
    const size_t bytes  = sizeof(S) * (size_t)n * n;
    int          per_sm = (int)std::max<size_t>(4, std::min<size_t>(8, (120u << 20) / (bytes * (size_t)sm_count())));
    if (ctas_per_sm > 0) per_sm = std::min(ctas_per_sm, 8);
    int fit = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, NT, smem) == cudaSuccess && fit > 0)
        per_sm = std::min(per_sm, fit);
    const int grid = std::min(batch, per_sm * sm_count());
    kern<<<grid, NT, smem, s>>>(H, n, ld, mstride, d, e, tq, status, batch);
    count_launch();
}

// Shared-memory residency: FP32 matrices whose n x n copy (plus vectors) fits in 200 KB.
template <typename S>
static bool use_smem(int n) {
    using R = typename ST<S>::R;
    return sizeof(R) == 4 && sizeof(S) * ((size_t)n * (n | 1) + (size_t)10 * n) <= 200 * 1024;
}

template <typename S, int MAXT>
static void tridiag_pick(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                         int* status, int batch, cudaStream_t s, int ctas_per_sm) {
    if (use_smem<S>(n)) tridiag_launch_t<S, 256, MAXT, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
    else tridiag_launch_t<S, 256, MAXT, false>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
}

template <typename S>
void launch_tridiag(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq, int* status,
                    int batch, cudaStream_t s, int variant, int ctas_per_sm, int cluster, bool tensor_cores) {
    if constexpr (std::is_same<S, float>::value) {
        if ((variant == 0 || variant == 1) && n <= tridiag_reg_max_n()) {
            launch_tridiag_reg(H, n, ld, mstride, d, e, tq, status, batch, s);
            return;
        }
    }
    // the cluster reduction is a tuning choice: the fused kernel below beats it at every order it
    // was automatic for (complex FP32, 2000 k: n = 178 22.5 vs 30.4 ms, 229 50.2 vs 79.7, 274 64.3
    // vs 112.0)
    constexpr bool F32 = sizeof(typename ST<S>::R) == 4;
    if (variant == 3 && launch_tridiag_cluster<S>(H, n, ld, mstride, d, e, tq, status, batch, s, cluster)) return;
    // FP32 matrices reduced from L2/DRAM: the fused kernels (one pass per step, 4; every other
    // update deferred, 3 passes per two steps, 5 and automatic). Reduction time per 2000 k: Ge SOC
    // n = 362 222 ms unfused, 102.7 fused, 81.3 deferred; GaP SOC n = 458 230.6 -> 198.3 ms.
    if constexpr (F32) {
        // the blocked kernel (6) is automatic from order 200 (2000 k, mixed: Ge SOC n = 362 81.3 ->
        // 47.5 ms, Si SOC n = 338 67.1 -> 41.7, GaP SOC n = 458 198.3 -> 81.8; with its trailing updates
        // on the tensor cores, whole solves against the deferred kernel: Si SOC n = 274 33.4 against
        // 45.5 ms, InAs n = 229 27.2 against 27.7); below, the deferred kernel stays ahead (GaAs SOC
        // n = 178 16.5 against 19.3 ms per solve). Real matrices, whose updates stay on the FP32 pipe,
        // keep the order-300 switch (real Sn and Ge n = 229: deferred 16.3 and 17.4 ms per solve,
        // blocked 19.4 and 20.6).
        if ((variant == 6 || (variant == 0 && n >= (ST<S>::cplx ? 200 : 300))) &&
            launch_tridiag_blocked<S>(H, n, ld, mstride, d, e, tq, status, batch, s, tensor_cores))
            return;
        // automatic: the deferred kernel for every FP32 order beyond the register kernel, also where
        // the matrix would fit shared memory (2000 k: Ge nonlocal n = 181 real 5.85 ms against 14.3
        // for the shared-memory kernel; InP n = 113 complex 2.37 against 3.27; GaAs n = 89 complex
        // 1.45 against 1.70)
        const bool auto_fused = variant == 0;
        if (variant == 4 && n <= 512) {
            if (n <= 129) fused_launch_t<S, 4>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 161) fused_launch_t<S, 5>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 257) fused_launch_t<S, 8>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 385) fused_launch_t<S, 12>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else fused_launch_t<S, 16>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            return;
        }
        if ((variant == 5 || auto_fused) && n <= 512) {
            if (n <= 129) fused_launch_t<S, 4, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 161) fused_launch_t<S, 5, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 257) fused_launch_t<S, 8, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else if (n <= 385) fused_launch_t<S, 12, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            else fused_launch_t<S, 16, true>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
            return;
        }
    }
    // rows of the trailing matrix are at most n - 1 <= 32 * MAXT
    if (n <= 129) tridiag_pick<S, 4>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
    else if (n <= 161) tridiag_pick<S, 5>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
    else if (n <= 257) tridiag_pick<S, 8>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
    else if (n <= 385) tridiag_pick<S, 12>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
    else tridiag_pick<S, 16>(H, n, ld, mstride, d, e, tq, status, batch, s, ctas_per_sm);
}

template void launch_tridiag<cx<double>>(cx<double>*, int, int, size_t, double*, double*, cx<double>*, int*, int, cudaStream_t, int, int, int, bool);
template void launch_tridiag<cx<float>>(cx<float>*, int, int, size_t, float*, float*, cx<float>*, int*, int, cudaStream_t, int, int, int, bool);
template void launch_tridiag<double>(double*, int, int, size_t, double*, double*, double*, int*, int, cudaStream_t, int, int, int, bool);
template void launch_tridiag<float>(float*, int, int, size_t, float*, float*, float*, int*, int, cudaStream_t, int, int, int, bool);

}  // namespace uepm
