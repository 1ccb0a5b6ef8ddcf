// tridiag_blocked.cu -- blocked Householder reduction of FP32 Hermitian (or real symmetric) matrices
// to real symmetric tridiagonal form for the orders beyond one SM's shared memory (the mixed path's
// reduction of the spin-orbit matrices, n = 178..512): the first half of Eigen's
// SelfAdjointEigenSolver called by Hamiltonian::Diagonalize (src/EPP/Hamiltonian.cpp:125-134).
//
// Algorithm: LAPACK zhetrd with zlatrd panels (lower storage). For each panel of NB columns
// j0..j0+NB-1, column i of the panel is
//   (a) brought up to date with the panel's earlier reflectors,
//         A[i:, i] -= V[i:, :ii] W[i, :ii]^H + W[i:, :ii] V[i, :ii]^H,
//   (b) reduced by its reflector v (zlarfg: beta real, tau, tail scaled by 1 / (alpha - beta)),
//   (c) given w = tau (A22 v - V (W^H v) - W (V^H v)), w += -(tau / 2)(w^H v) v, where A22 is the
//       trailing matrix as it was at the start of the panel (the panel's updates are deferred);
// and after the panel the trailing matrix takes all NB updates at once,
//   A22 -= V W^H + W V^H                              (a rank-2 NB update, zher2k),
// so that A = Q T Q^H with Q = H_0 ... H_{n-2}, H_i = I - tau_i v_i v_i^H: the same reflectors,
// tails (column i, rows i+2..n-1) and tau as the unblocked kernels, for the back-transformation.
//
// GB300 mapping. One CTA per matrix, one matrix per SM at a time (a persistent grid over the batch):
// the matrix stays in global memory, but only its LOWER triangle is ever read or written, so the
// 152 matrices in flight (n = 362 complex: 0.52 MB each, 80 MB) stay resident in the 129 MB L2 and
// the per-column product A22 v streams from L2, not HBM. The Hermitian product takes each stored
// element once for both of its uses (y_r += a v_c and y_c += conj(a) v_r): a warp walks 8-column
// strips of the triangle in 64-row tiles (two adjacent rows per lane, one 16-byte load per column
// for complex), adds row sums to its partial vector and keeps the strip's column sums in registers
// across its consecutive tiles, reduced across lanes once per strip. The work is split evenly over
// the warps; the per-warp partial vectors are summed in a fixed order (deterministic results). The
// trailing update reads and writes the lower triangle once per panel instead of once per column.
// Shared memory holds the panel's V and W, the per-warp partial products and the current reflector.
#include <algorithm>
#include <type_traits>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

namespace {

constexpr int kBlkNT = 512;  // threads per CTA (16 warps)
constexpr int kBlkNW = kBlkNT / 32;
constexpr int kBlkNB = 16;   // panel width

template <typename S>
__device__ __forceinline__ S sh_xor(S v, int o);
template <>
__device__ __forceinline__ float sh_xor<float>(float v, int o) {
    return __shfl_xor_sync(0xffffffffu, v, o);
}
template <>
__device__ __forceinline__ cx<float> sh_xor<cx<float>>(cx<float> v, int o) {
    return mk(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

// tile index t of the lower triangle of nt x nt tiles -> (R, C), R >= C, t = R (R + 1) / 2 + C
__device__ __forceinline__ void tri_tile(int t, int& R, int& C) {
    int r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    while (r * (r + 1) / 2 > t) --r;
    R = r;
    C = t - r * (r + 1) / 2;
}

template <typename S>
struct BlkSmem {
    // bytes of dynamic shared memory for order n
    static __host__ __device__ size_t bytes(int n) {
        using R = typename ST<S>::R;
        return sizeof(S) * ((size_t)2 * kBlkNB * n + (size_t)kBlkNW * n + (n + 32) + 2 * kBlkNB) +
               sizeof(R) * 4 * kBlkNW + 64;
    }
};

template <typename S>
__global__ void __launch_bounds__(kBlkNT, 1)
    k_tridiag_blocked(S* __restrict__ H, int n, int ld, size_t mstride, typename ST<S>::R* __restrict__ dOut,
                      typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut, int* __restrict__ status, int batch) {
    using R = typename ST<S>::R;
    extern __shared__ __align__(16) unsigned char smraw[];
    S* Vp   = reinterpret_cast<S*>(smraw);              // [k][r], NB x n
    S* Wp   = Vp + (size_t)kBlkNB * n;                  // [k][r], NB x n
    S* yp   = Wp + (size_t)kBlkNB * n;                  // [warp][r], NW x n
    S* v    = yp + (size_t)kBlkNW * n;                  // n + 32 (zero padded past n)
    S* tdot = v + (n + 32);                             // t1 (W^H v) then t2 (V^H v), NB each
    R* red  = reinterpret_cast<R*>(tdot + 2 * kBlkNB);  // 4 x NW
    __shared__ S s_c0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // With an even order every column starts at an even element, so row pairs from an even row are
    // 16-byte (8-byte for real) aligned: the product's tiles then start at o rounded down to even.
    const bool vec = (n & 1) == 0 && (mstride & 1) == 0 && (ld & 1) == 0;

    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        S*   A   = H + (size_t)b * mstride;
        bool bad = false;
        for (int r = tid; r < n + 32; r += kBlkNT) v[r] = ST<S>::zero();

        for (int j0 = 0; j0 < n - 1; j0 += kBlkNB) {
            const int jb = min(kBlkNB, n - 1 - j0);
            for (int q = tid; q < kBlkNB * n; q += kBlkNT) {
                Vp[q] = ST<S>::zero();
                Wp[q] = ST<S>::zero();
            }
            __syncthreads();
            // the thread's element of the panel's next column, loaded one column ahead (the panel's
            // columns do not change until their turn)
            S anext = (j0 + tid < n) ? ldc(A + (size_t)j0 * ld + j0 + tid) : ST<S>::zero();

            for (int ii = 0; ii < jb; ++ii) {
                const int i = j0 + ii, o = i + 1, m = n - o;
                // ---- (a) column i brought up to date; its reflector -----------------------------
                const int r   = i + tid;  // one row per thread (n <= kBlkNT)
                S         a   = anext;
                R         nrm = R(0);
                if (r < n) {
                    for (int k = 0; k < ii; ++k) {
                        a = cfms_conjb(Vp[k * n + r], Wp[k * n + i], a);
                        a = cfms_conjb(Wp[k * n + r], Vp[k * n + i], a);
                    }
                    if (r == i) {
                        const R di              = ST<S>::re(a);
                        dOut[(size_t)b * n + i] = di;
                        if (!isfinite(di)) bad = true;
                    } else if (r == o) {
                        s_c0 = a;
                    } else {
                        nrm = ST<S>::norm(a);
                    }
                }
                nrm = warp_sum(nrm);
                if (lane == 0) red[warp] = nrm;
                __syncthreads();
                // Householder scalars, the same in every thread (zlarfg)
                R tail2 = 0;
#pragma unroll
                for (int q = 0; q < kBlkNW; ++q) tail2 += red[q];
                const S c0  = s_c0;
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
                    const R ib  = R(1) / beta;
                    th          = ST<S>::make((beta - c0r) * ib, -c0i * ib);
                    const R ar  = c0r - beta, ai = c0i;
                    const R den = R(1) / fma(ar, ar, ai * ai);
                    sc          = ST<S>::make(ar * den, -ai * den);
                }
                if (r < n && r > i) {
                    const S vr = (r == o) ? ST<S>::one() : cmul(a, sc);
                    stc(A + (size_t)i * ld + r, (r == o) ? ST<S>::make(beta, R(0)) : vr);
                    v[r]           = vr;
                    Vp[ii * n + r] = vr;
                }
                if (tid < o) v[tid] = ST<S>::zero();
                if (tid == 0) {
                    eOut[(size_t)b * n + i]  = beta;
                    tqOut[(size_t)b * n + i] = th;
                    if (!isfinite(beta)) bad = true;
                }
                if (ii + 1 < jb && r + 1 < n) anext = ldc(A + (size_t)o * ld + r + 1);
                __syncthreads();

                // ---- (c) y = A22 v over the lower triangle (rows, cols o..n-1); t1, t2 --------------
                // Work units: (8-column strip C, 64-row tile R) of the lower triangle in strip-major
                // order, split evenly over the warps in contiguous ranges. Each lane takes two adjacent
                // rows. Row sums go to the warp's partial vector; the strip's 8 column sums
                // (conj(a) v_r) accumulate in registers over the warp's consecutive tiles of the strip
                // and are reduced across lanes once per strip. Only the tile of each strip that meets
                // the diagonal (or the last row) needs masks. Tiles start at ro (o, or o - 1 for the
                // aligned pairs): row / column o - 1 contributes nothing (v is zero there, and its
                // column sum lands in the unused entry o - 1 of the partial vector).
                S* my = yp + (size_t)warp * n;
                for (int q = o + lane; q < n; q += 32) my[q] = ST<S>::zero();
                __syncwarp();
                const int ro = vec ? (o & ~1) : o;
                const int ml = n - ro;
                const int nr = (ml + 63) >> 6, nc = (ml + 7) >> 3;
                // strip C covers columns ro + 8C .. ro + 8C + 7 and row tiles C / 8 .. nr - 1
                int U = 0;
                for (int C = 0; C < nc; C += 8) U += min(8, nc - C) * (nr - (C >> 3));
                const int u0 = (int)(((long long)U * warp) / kBlkNW), u1 = (int)(((long long)U * (warp + 1)) / kBlkNW);
                if (u0 < u1) {
                    int C = 0, rem = u0;
                    while (rem >= nr - (C >> 3)) {
                        rem -= nr - (C >> 3);
                        ++C;
                    }
                    int R_ = (C >> 3) + rem;
                    S   vc[8], xc[8];
                    int u = u0;
                    while (u < u1) {
                        const int c0s = ro + 8 * C;  // first column of the strip
#pragma unroll
                        for (int cc = 0; cc < 8; ++cc) {
                            vc[cc] = v[c0s + cc];  // zero padded past n
                            xc[cc] = ST<S>::zero();
                        }
                        for (; u < u1 && R_ < nr; ++u, ++R_) {
                            const int r0   = ro + 64 * R_ + 2 * lane;  // this lane's rows r0, r0 + 1
                            const S*  base = A + (size_t)c0s * ld + r0;
                            S         x0[8], x1[8];
                            // interior: all 64 rows exist and lie below the strip's 8 columns
                            const bool full = (ro + 64 * R_ + 63 < n) && (64 * R_ > 8 * C + 7);
                            if (full) {
#pragma unroll
                                for (int cc = 0; cc < 8; ++cc) {
                                    const S* p = base + (size_t)cc * ld;
                                    if (vec) {  // aligned pair (uniform branch)
                                        if constexpr (ST<S>::cplx) {
                                            const float4 q = *reinterpret_cast<const float4*>(p);
                                            x0[cc]         = ST<S>::make(q.x, q.y);
                                            x1[cc]         = ST<S>::make(q.z, q.w);
                                        } else {
                                            const float2 q = *reinterpret_cast<const float2*>(p);
                                            x0[cc]         = ST<S>::make(q.x, 0.f);
                                            x1[cc]         = ST<S>::make(q.y, 0.f);
                                        }
                                    } else {
                                        x0[cc] = ldc(p);
                                        x1[cc] = ldc(p + 1);
                                    }
                                }
                                const S vr0 = v[r0], vr1 = v[r0 + 1];
                                S       y0 = ST<S>::zero(), y1 = ST<S>::zero();
#pragma unroll
                                for (int cc = 0; cc < 8; ++cc) {
                                    y0     = cfma(x0[cc], vc[cc], y0);
                                    y1     = cfma(x1[cc], vc[cc], y1);
                                    xc[cc] = cfmac(x0[cc], vr0, xc[cc]);
                                    xc[cc] = cfmac(x1[cc], vr1, xc[cc]);
                                }
                                my[r0]     = cadd(my[r0], y0);
                                my[r0 + 1] = cadd(my[r0 + 1], y1);
                            } else {
#pragma unroll
                                for (int cc = 0; cc < 8; ++cc) {
                                    const int c = c0s + cc;
                                    x0[cc] = (r0 < n && c < n && r0 >= c) ? ldc(base + (size_t)cc * ld) : ST<S>::zero();
                                    x1[cc] = (r0 + 1 < n && c < n && r0 + 1 >= c) ? ldc(base + (size_t)cc * ld + 1)
                                                                                  : ST<S>::zero();
                                }
                                const S vr0 = v[r0 < n ? r0 : n], vr1 = v[r0 + 1 < n ? r0 + 1 : n];
                                S       y0 = ST<S>::zero(), y1 = ST<S>::zero();
#pragma unroll
                                for (int cc = 0; cc < 8; ++cc) {
                                    y0 = cfma(x0[cc], vc[cc], y0);
                                    y1 = cfma(x1[cc], vc[cc], y1);
                                    // the diagonal element counts once (row product)
                                    xc[cc] = cfmac((r0 == c0s + cc) ? ST<S>::zero() : x0[cc], vr0, xc[cc]);
                                    xc[cc] = cfmac((r0 + 1 == c0s + cc) ? ST<S>::zero() : x1[cc], vr1, xc[cc]);
                                }
                                if (r0 < n) my[r0] = cadd(my[r0], y0);
                                if (r0 + 1 < n) my[r0 + 1] = cadd(my[r0 + 1], y1);
                            }
                        }
                        // column sums over the lanes: halving exchanges leave lane L with column L & 7
                        // summed over its group of 8 lanes, then the four groups are folded
#pragma unroll
                        for (int st = 0; st < 3; ++st) {
                            const int  sft = 4 >> st;
                            const bool up  = (lane & sft) != 0;
#pragma unroll
                            for (int j = 0; j < sft; ++j) {
                                const S send = up ? xc[j] : xc[j + sft];
                                const S keep = up ? xc[j + sft] : xc[j];
                                xc[j]        = cadd(keep, sh_xor(send, sft));
                            }
                        }
                        S ycol = cadd(xc[0], sh_xor(xc[0], 8));
                        ycol   = cadd(ycol, sh_xor(ycol, 16));
                        __syncwarp();
                        const int cl = c0s + lane;
                        if (lane < 8 && cl < n) my[cl] = cadd(my[cl], ycol);
                        __syncwarp();
                        ++C;  // next strip
                        R_ = C >> 3;
                    }
                }
                // t1_k = W_k^H v, t2_k = V_k^H v for the panel's earlier reflectors (k < ii)
                for (int q = warp; q < 2 * ii; q += kBlkNW) {
                    const S* col = (q < ii) ? Wp + (size_t)q * n : Vp + (size_t)(q - ii) * n;
                    S        s   = ST<S>::zero();
                    for (int rr = o + lane; rr < n; rr += 32) s = cfmac(col[rr], v[rr], s);
                    s = warp_sum(s);
                    if (lane == 0) tdot[(q < ii) ? q : kBlkNB + (q - ii)] = s;
                }
                __syncthreads();

                // ---- w = tau (y - V t1 - W t2); alpha = -tau/2 (w^H v); w += alpha v -----------------
                S wr = ST<S>::zero();
                S wv = ST<S>::zero();
                if (r < n && r > i) {
                    S part[kBlkNW];
#pragma unroll
                    for (int q = 0; q < kBlkNW; ++q) part[q] = yp[(size_t)q * n + r];
#pragma unroll
                    for (int h = kBlkNW / 2; h > 0; h >>= 1)
#pragma unroll
                        for (int q = 0; q < h; ++q) part[q] = cadd(part[q], part[q + h]);
                    S y1 = ST<S>::zero(), y2 = ST<S>::zero();
                    for (int k = 0; k < ii; ++k) {
                        y1 = cfma(Vp[k * n + r], tdot[k], y1);
                        y2 = cfma(Wp[k * n + r], tdot[kBlkNB + k], y2);
                    }
                    const S y = csub(part[0], cadd(y1, y2));
                    wr        = cmul(th, y);
                    wv        = cfmac(wr, v[r], wv);
                }
                wv = warp_sum(wv);
                if (lane == 0) {
                    red[kBlkNW + warp]     = ST<S>::re(wv);
                    red[2 * kBlkNW + warp] = ST<S>::im(wv);
                }
                __syncthreads();
                R wvr = 0, wvi = 0;
#pragma unroll
                for (int q = 0; q < kBlkNW; ++q) {
                    wvr += red[kBlkNW + q];
                    wvi += red[2 * kBlkNW + q];
                }
                const S alpha = cscale(cmul(th, ST<S>::make(wvr, wvi)), R(-0.5));
                if (r < n && r > i) Wp[ii * n + r] = cfma(alpha, v[r], wr);
                __syncthreads();
            }

            // ---- trailing update A22 -= V W^H + W V^H (lower triangle, rows/cols q0..n-1) -----------
            const int q0 = j0 + jb, mt = n - q0;
            if (mt > 0) {
                const int nt = (mt + 31) >> 5, T = nt * (nt + 1) / 2;
                for (int t = warp; t < T; t += kBlkNW) {
                    int R_, C_;
                    tri_tile(t, R_, C_);
                    const int  rr  = q0 + 32 * R_ + lane;
                    const int  c0c = q0 + 32 * C_;
                    const bool rv  = rr < n;
                    S          vr[kBlkNB], wr[kBlkNB];
#pragma unroll
                    for (int k = 0; k < kBlkNB; ++k) {
                        vr[k] = (rv && k < jb) ? Vp[k * n + rr] : ST<S>::zero();
                        wr[k] = (rv && k < jb) ? Wp[k * n + rr] : ST<S>::zero();
                    }
#pragma unroll 1
                    for (int cb = 0; cb < 32; cb += 8) {
                        S x[8];
#pragma unroll
                        for (int cc = 0; cc < 8; ++cc) {
                            const int  c  = c0c + cb + cc;
                            const bool ok = rv && c < n && (R_ > C_ || lane >= cb + cc);
                            x[cc]         = ok ? ldc(A + (size_t)c * ld + rr) : ST<S>::zero();
                        }
#pragma unroll
                        for (int cc = 0; cc < 8; ++cc) {
                            const int c  = c0c + cb + cc;
                            const int cs = c < n ? c : n - 1;
                            S         y  = x[cc];
#pragma unroll
                            for (int k = 0; k < kBlkNB; ++k) {
                                y = cfms_conjb(vr[k], Wp[k * n + cs], y);
                                y = cfms_conjb(wr[k], Vp[k * n + cs], y);
                            }
                            const bool ok = rv && c < n && (R_ > C_ || lane >= cb + cc);
                            if (ok) stc(A + (size_t)c * ld + rr, (rr == c) ? ST<S>::make(ST<S>::re(y), R(0)) : y);
                        }
                    }
                }
            }
            __syncthreads();
        }
        if (tid == 0) {
            const R dl                   = ST<S>::re(ldc(A + (size_t)(n - 1) * ld + (n - 1)));
            dOut[(size_t)b * n + n - 1]  = dl;
            eOut[(size_t)b * n + n - 1]  = R(0);
            tqOut[(size_t)b * n + n - 1] = ST<S>::zero();
            if (!isfinite(dl)) bad = true;
        }
        bad = __syncthreads_or(bad);
        if (tid == 0 && bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
    }
}

}  // namespace

int tridiag_blocked_max_n() { return kBlkNT; }

template <typename S>
bool launch_tridiag_blocked(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                            int* status, int batch, cudaStream_t s) {
    if (n < 2 || n > kBlkNT) return false;
    const size_t smem = BlkSmem<S>::bytes(n);
    if (smem > 227 * 1024) return false;
    auto kern = k_tridiag_blocked<S>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
    int dev = 0, sms = 0, fit = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, kBlkNT, smem) != cudaSuccess || fit < 1) fit = 1;
    const int grid = std::min(batch, std::max(1, sms) * fit);
    kern<<<grid, kBlkNT, smem, s>>>(H, n, ld, mstride, d, e, tq, status, batch);
    count_launch();
    return true;
}

template bool launch_tridiag_blocked<float>(float*, int, int, size_t, float*, float*, float*, int*, int, cudaStream_t);
template bool launch_tridiag_blocked<cx<float>>(cx<float>*, int, int, size_t, float*, float*, cx<float>*, int*, int,
                                                cudaStream_t);

}  // namespace uepm
