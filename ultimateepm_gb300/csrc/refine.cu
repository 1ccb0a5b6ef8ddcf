// refine.cu -- FP64-accurate Rayleigh-Ritz refinement of FP32 eigenvectors (mixed-precision path).
//
// No reference counterpart: the reference only has the FP64 Eigen solve. Given FP32 approximations
// X (n x m, m = nb + guard bands) to the lowest eigenvectors of the FP64 Hermitian H, this computes
//   k_refine_project   Y = H X, S = X^H X, A = X^H Y            (one CTA per matrix)
//   k_small_eigh       the m x m pencil A c = lambda S c: Cholesky S = L L^H, C = L^-1 A L^-H,
//                      parallel cyclic Jacobi on C (m/2 disjoint rotations at a time), ascending
//                      sort, W = L^-H V   (one warp per matrix, all in shared memory, FP64)
//   k_refine_vectors   Ritz vectors X W and their Hellmann-Feynman gradients (on request)
// Ritz values err by about ||H x - lambda x||^2 / gap, where the gap is to the first eigenvalue
// outside the subspace; the guard bands keep that gap open.
//
// The products of k_refine_project need FP64-level accuracy (an error dA moves the Ritz values by
// dA, and |H| reaches ~10^2 eV), but their operands are exact FP32 values (X) and FP64 values split
// into FP32 pairs (H, written that way by the assembly): they run in double-single arithmetic on the
// FP32 pipe (exact products, two-sum accumulation, ~48 significant bits), about 10 FP32 operations
// per real multiply-add instead of one FMA on GB300's ~60x slower FP64 pipe.
#include <type_traits>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kProjNT = 256;
constexpr int kProjVB = 4;                  // vectors per Y work item
constexpr size_t kProjStageBytes = 96 << 10;  // X staged in shared memory up to this size

template <typename S>
using XElem = std::conditional_t<std::is_same<S, double>::value, float, float2>;  // FP32 element of X
template <typename S>
using YElem = std::conditional_t<std::is_same<S, double>::value, float2, float4>;  // double-single Y

template <typename S>
__host__ __device__ inline int proj_mp(int m) {
    return (m + kProjVB - 1) / kProjVB * kProjVB;
}
template <typename S>
inline size_t proj_stage_bytes(int n, int m) {
    return sizeof(XElem<S>) * (size_t)n * proj_mp<S>(m);
}

// X(r, j) from the staged copy ([r][mp]) or from X32 ([j][n]); zero for the padding vectors j >= m.
template <typename S, bool STAGED>
__device__ __forceinline__ XElem<S> x_at(const XElem<S>* Xs, const cx<float>* Xg, int n, int m, int mp, int r, int j) {
    if (STAGED) return Xs[(size_t)r * mp + j];
    cx<float> v = j < m ? Xg[(size_t)j * n + r] : cx<float>{0.f, 0.f};
    if constexpr (std::is_same<S, double>::value) return v.x;
    else return make_float2(v.x, v.y);
}

// The diagonal of a local-potential H as stored pairs: V_rr + kinetic in FP64 (the sum the
// assembly forms) split into FP32 pairs.
__device__ __forceinline__ ds2 split_pair(double v) {
    const float hi = __double2float_rn(v);
    return ds2{hi, __double2float_rn(v - (double)hi)};
}
template <typename S>
__device__ __forceinline__ typename Split<S>::type sparse_diag(const SparseV& sv, int b, int r) {
    const cx<double> v  = sv.Vloc[(size_t)r * sv.N + r];
    const ds2        re = split_pair(v.x + sv.rows[((size_t)b * sv.N + r) * ROW_STRIDE + RF_KIN]);
    if constexpr (std::is_same<S, double>::value) {
        return re;
    } else {
        const ds2 im = split_pair(v.y);
        return ds4{re.hi, re.lo, im.hi, im.lo};
    }
}
template <typename S>
__device__ __forceinline__ typename Split<S>::type sparse_slot(const SparseV& sv, size_t o) {
    const float2 a = sv.re[o];
    if constexpr (std::is_same<S, double>::value) {
        return ds2{a.x, a.y};
    } else {
        const float2 c = sv.im[o];
        return ds4{a.x, a.y, c.x, c.y};
    }
}

// y[q] += h x(c, j0 + q), q < kProjVB
template <typename S, bool STAGED>
__device__ __forceinline__ void proj_accumulate(dsacc (&yr)[kProjVB], dsacc (&yi)[kProjVB], const typename Split<S>::type& h,
                                                const XElem<S>* Xs, const cx<float>* Xg, int n, int m, int mp, int c,
                                                int j0) {
#pragma unroll
    for (int q = 0; q < kProjVB; ++q) {
        const XElem<S> x = x_at<S, STAGED>(Xs, Xg, n, m, mp, c, j0 + q);
        if constexpr (!std::is_same<S, double>::value) {  // (hr + i hi)(xr + i xi)
            ds_add_prod(yr[q], h.rhi, h.rlo, x.x);
            ds_add_prod(yr[q], -h.ihi, -h.ilo, x.y);
            ds_add_prod(yi[q], h.rhi, h.rlo, x.y);
            ds_add_prod(yi[q], h.ihi, h.ilo, x.x);
        } else {
            ds_add_prod(yr[q], h.hi, h.lo, x);
        }
    }
}

template <typename S, bool STAGED, bool SPARSE, bool YDONE = false>
__global__ void __launch_bounds__(kProjNT) k_refine_project(const typename Split<S>::type* __restrict__ H, int n, int ld,
                                                            size_t mstride, const cx<float>* __restrict__ X32, int m,
                                                            void* __restrict__ work, S* __restrict__ small, int batch,
                                                            const SparseV sv) {
    constexpr bool CX = !std::is_same<S, double>::value;
    using SE          = typename Split<S>::type;
    using XT          = XElem<S>;
    using YT          = YElem<S>;
    const int b = blockIdx.x;
    if (b >= batch) return;
    const int        tid = threadIdx.x, mp = proj_mp<S>(m);
    const cx<float>* Xg  = X32 + (size_t)b * m * n;
    extern __shared__ __align__(16) unsigned char smraw[];
    XT* Xs = reinterpret_cast<XT*>(smraw);  // [r][mp]
    if (STAGED) {
        // asynchronous element copies (all in flight at once); the padding vectors j >= m are zero
        const int warp = tid >> 5, lane = tid & 31;
        for (int j = warp; j < mp; j += kProjNT / 32) {
            for (int r = lane; r < n; r += 32) {
                XT* dst = Xs + (size_t)r * mp + j;
                if (j < m) cp_async_elem<sizeof(XT)>(dst, Xg + (size_t)j * n + r);  // Re, or (Re, Im)
                else *dst = XT{};
            }
        }
        cp_async_wait_all();
        __syncthreads();
    }
    // ---- Y = H X: item (row r, block of kProjVB vectors), the vector block fastest, so that the
    // lanes sharing a row take H(r, c) in one request and each element of H leaves memory once;
    // H(r, c + 1) is fetched while the products of column c run --------------------------------------
    YT*       Y    = reinterpret_cast<YT*>(work) + (size_t)b * refine_work_elems(n, m) * sizeof(S) / sizeof(YT);  // [r][mp]
    const SE* A    = H + (size_t)b * mstride;
    const int nblk = mp / kProjVB;
    for (int item = tid; item < (YDONE ? 0 : nblk * n); item += kProjNT) {  // YDONE: Y came from the tensor cores
        const int r = item / nblk, jb = item - r * nblk, j0 = jb * kProjVB;
        dsacc     yr[kProjVB], yi[kProjVB];
#pragma unroll
        for (int q = 0; q < kProjVB; ++q) yr[q] = yi[q] = dsacc{0.f, 0.f};
        if constexpr (SPARSE) {
            // the diagonal, then the off-diagonal slots (coalesced over r)
            proj_accumulate<S, STAGED>(yr, yi, sparse_diag<S>(sv, b, r), Xs, Xg, n, m, mp, r, j0);
#pragma unroll 4
            for (int e = 0; e < sv.W; ++e) {
                const size_t o = (size_t)e * sv.N + r;
                proj_accumulate<S, STAGED>(yr, yi, sparse_slot<S>(sv, o), Xs, Xg, n, m, mp, sv.col[o], j0);
            }
        } else {
            SE h = A[r];
            for (int c = 0; c < n; ++c) {
                const SE hc = h;
                if (c + 1 < n) h = A[(size_t)(c + 1) * ld + r];
                proj_accumulate<S, STAGED>(yr, yi, hc, Xs, Xg, n, m, mp, c, j0);
            }
        }
#pragma unroll
        for (int q = 0; q < kProjVB; ++q) {
            if constexpr (CX) Y[(size_t)r * mp + j0 + q] = make_float4(yr[q].h, yr[q].l, yi[q].h, yi[q].l);
            else Y[(size_t)r * mp + j0 + q] = make_float2(yr[q].h, yr[q].l);
        }
    }
    __syncthreads();
    // ---- S = X^H X and A = X^H Y, upper triangles (p <= q) only, FP64 out ---------------------------
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
        dsacc     sr{0.f, 0.f}, si{0.f, 0.f}, ar{0.f, 0.f}, ai{0.f, 0.f};
        for (int r = 0; r < n; ++r) {
            const XT xp = x_at<S, STAGED>(Xs, Xg, n, m, mp, r, p);
            const XT xq = x_at<S, STAGED>(Xs, Xg, n, m, mp, r, q);
            const YT y  = Y[(size_t)r * mp + q];
            if constexpr (CX) {  // conj(xp) xq and conj(xp) y
                ds_add_prod(sr, xp.x, xq.x);
                ds_add_prod(sr, xp.y, xq.y);
                ds_add_prod(si, xp.x, xq.y);
                ds_add_prod(si, -xp.y, xq.x);
                ds_add_prod(ar, y.x, y.y, xp.x);
                ds_add_prod(ar, y.z, y.w, xp.y);
                ds_add_prod(ai, y.z, y.w, xp.x);
                ds_add_prod(ai, -y.x, -y.y, xp.y);
            } else {
                ds_add_prod(sr, xp, xq);
                ds_add_prod(ar, y.x, y.y, xp);
            }
        }
        const S s = ST<S>::make(ds_value(sr), ds_value(si)), a = ST<S>::make(ds_value(ar), ds_value(ai));
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

// shared memory of one warp's matrix: L, C, V (m x (m+1) scalars each), 4 rotation arrays, the
// round's pair table, then FP32 copies of E = S - I and A for the Loewdin correction
template <typename S>
__host__ __device__ inline size_t small_eigh_lowdin_offset(int m) {
    const int me = (m + 1) & ~1;
    return (sizeof(S) * 3 * (size_t)m * (m + 1) + (sizeof(double) + sizeof(S)) * 2 * (size_t)me + sizeof(int) * (size_t)me +
            15) &
           ~(size_t)15;
}
template <typename S>
__host__ __device__ inline size_t small_eigh_warp_bytes(int m) {
    return (small_eigh_lowdin_offset<S>(m) + sizeof(typename Lower<S>::type) * 3 * (size_t)m * m + 15) & ~(size_t)15;
}

__device__ __forceinline__ float to_lower(double v) { return (float)v; }
__device__ __forceinline__ cx<float> to_lower(cx<double> v) { return mk((float)v.x, (float)v.y); }
__device__ __forceinline__ double from_lower(float v) { return (double)v; }
__device__ __forceinline__ cx<double> from_lower(cx<float> v) { return mk((double)v.x, (double)v.y); }

// cap > 0 (UEPM tuning max_iter) bounds the Jacobi sweeps (automatic: 12); sweeps that end by the
// cap with couplings still above the stopping threshold set UEPM_K_NOCONVERGE.
template <typename S>
__global__ void __launch_bounds__(32 * kSmallWarps) k_small_eigh(S* __restrict__ small, int m, int nb, double* __restrict__ Eout,
                                                                 int want_w, int* __restrict__ status, int batch, int cap) {
    using R         = double;
    const int warp  = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b     = blockIdx.x * kSmallWarps + warp;
    const int mp    = m + 1;                       // padded row length
    const int me    = (m + 1) & ~1;                // m rounded up to even (tournament size)
    extern __shared__ __align__(16) unsigned char smraw[];
    S*  L    = reinterpret_cast<S*>(smraw + (size_t)warp * small_eigh_warp_bytes<S>(m));
    S*  Cm   = L + (size_t)m * mp;
    S*  V    = Cm + (size_t)m * mp;
    R*  rc   = reinterpret_cast<R*>(V + (size_t)m * mp);  // per pair: cosine c
    R*  rs   = rc + me;                                   // sine s
    S*  jp   = reinterpret_cast<S*>(rs + me);             // -s conj(e), e the unit phase of C_pq
    S*  jq   = jp + me;                                   // c conj(e)
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
    // FP32 eigenvectors are nearly orthonormal, so S = I + E with a small E (|E| up to ~1e-4 for
    // close eigenvalues just outside the inverse iteration's clusters) and, to second order,
    // S^-1/2 = I + F, F = -E/2 + 3E^2/8 (Loewdin):
    //   C = (I + F) A (I + F) = A - (G + G^H)/2 + 3/8 (P + P^H) + E G^H / 4 + O(|E|^3 |A|),
    //   G = E A, P = E G,     and W = (I + F) V,
    // an error of ~1e-11 eV at |E| = 1e-4 (the first-order form left ~|E|^2 |A| ~ 1e-7 eV). When some
    // |E_ij| exceeds 1e-4 the Cholesky route runs instead.
    using F = typename Lower<S>::type;
    F* Ef   = reinterpret_cast<F*>(smraw + (size_t)warp * small_eigh_warp_bytes<S>(m) + small_eigh_lowdin_offset<S>(m));
    F* Af   = Ef + (size_t)m * m;  // A, then P
    F* Gf   = Af + (size_t)m * m;  // G, then E V for the vectors
    R  emax2 = 0;
    for (int q = lane; q < m * m; q += 32) {
        const int i = q / m, j = q - i * m;
        const S   e = (i == j) ? ST<S>::make(ST<S>::re(LL(i, j)) - 1.0, ST<S>::im(LL(i, j))) : LL(i, j);
        emax2       = fmax(emax2, ST<S>::norm(e));
    }
    emax2             = warp_max(emax2);
    const bool lowdin = emax2 <= 1e-8;  // max |E_ij| <= 1e-4
    if (lowdin) {
        // the corrections are ~|E| |A| ~ 1e-3 eV and need ~1e-6 relative accuracy: FP32 products
        // (on copies converted once), added to A in FP64
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            const S   e = (i == c) ? ST<S>::make(ST<S>::re(LL(i, c)) - 1.0, ST<S>::im(LL(i, c))) : LL(i, c);
            Ef[q]       = to_lower(e);
            Af[q]       = to_lower(VV(i, c));
        }
        __syncwarp();
        for (int q = lane; q < m * m; q += 32) {  // G = E A
            const int i = q / m, c = q - i * m;
            F         acc = ST<F>::zero();
            for (int j = 0; j < m; ++j) acc = cfma(Ef[i * m + j], Af[j * m + c], acc);
            Gf[q] = acc;
        }
        __syncwarp();
        for (int q = lane; q < m * m; q += 32) {  // P = E G, over A
            const int i = q / m, c = q - i * m;
            F         acc = ST<F>::zero();
            for (int j = 0; j < m; ++j) acc = cfma(Ef[i * m + j], Gf[j * m + c], acc);
            Af[q] = acc;
        }
        __syncwarp();
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            F         egh = ST<F>::zero();  // (E G^H)_ic
            for (int j = 0; j < m; ++j) egh = cfma(Ef[i * m + j], ST<F>::conj(Gf[c * m + j]), egh);
            const F g1 = cadd(Gf[i * m + c], ST<F>::conj(Gf[c * m + i]));
            const F p2 = cadd(Af[i * m + c], ST<F>::conj(Af[c * m + i]));
            const F corr = cfma(g1, ST<F>::make(-0.5f, 0.f), cfma(p2, ST<F>::make(0.375f, 0.f), cscale(egh, 0.25f)));
            CC(i, c) = cadd(VV(i, c), from_lower(corr));
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
    // parallel cyclic Jacobi: me - 1 rounds of me / 2 disjoint pairs per sweep. The rotation angle
    // comes from FP32 arithmetic and (c, s) and the unit phase e are then renormalised in FP64 by the
    // series 1/sqrt(1 + x) = 1 - x/2 + 3x^2/8 (|x| ~ 1e-7), so every rotation is orthogonal to FP64
    // precision; an angle off by ~1e-7 leaves ~1e-7 of |C_pq| behind, which the next sweep removes.
    // Pairs below the stopping threshold are not rotated, and a round with no pair above it is
    // skipped: once the nearly diagonal C has converged, the final sweep costs only its checks.
    const int npair = me / 2;
    const int nblk  = npair * (npair + 1) / 2;           // 2 x 2 blocks (k, l), k <= l, of C
    int*      pp    = reinterpret_cast<int*>(jq + me);  // pair table of the round: p, q
    int*      pq    = pp + npair;
    // Without vectors only the near-degenerate pairs are rotated: a coupling b whose rotation angle
    // b / gap is at most 1e-4 moves the Ritz values by b^2 / gap, which is added after the sweeps
    // (second-order perturbation; the neglected third-order terms are ~b theta^2 < 1e-12 eV here).
    // With vectors every pair above the threshold is rotated.
    const R th0sq = want_w ? 0.0 : 1e-8;
    R       dia   = 0;
    for (int i = lane; i < m; i += 32) dia = fmax(dia, fabs(ST<S>::re(CC(i, i))));
    dia = warp_max(dia);
    // remaining off-diagonals move the Ritz values by at most ~off (degenerate pairs) or
    // off^2 / gap: 1e-10 of the largest diagonal is ~2e-9 eV here
    R          thr2      = (1e-10 * dia) * (1e-10 * dia);
    const int  sweeps    = cap > 0 ? cap : 12;
    bool       converged = false;
    for (int sweep = 0; sweep < sweeps; ++sweep) {
        if (want_w) {
            R off2 = 0;
            dia    = 0;
            for (int q = lane; q < m * m; q += 32) {
                const int i = q / m, c = q - i * m;
                if (i < c) off2 = fmax(off2, ST<S>::norm(CC(i, c)));
                if (i == c) dia = fmax(dia, fabs(ST<S>::re(CC(i, i))));
            }
            off2 = warp_max(off2);
            dia  = warp_max(dia);
            thr2 = (1e-10 * dia) * (1e-10 * dia);
            if (off2 <= thr2 || off2 == 0.0) {
                converged = true;
                break;
            }
        }
        bool rotated = false;
        for (int round = 0; round < me - 1; ++round) {
            // tournament pairing: slot 0 fixed, slots 1..me-1 rotate
            bool act = false;
            if (lane < npair) {
                const int a0 = (lane == 0) ? 0 : ((lane - 1 + round) % (me - 1)) + 1;
                const int a1 = ((me - 2 - lane + round) % (me - 1)) + 1;
                const int p = min(a0, a1), q = max(a0, a1);
                R         cc = 1.0, ss = 0.0, ex = 1.0, ey = 0.0;
                if (q < m) {
                    const S bpq = CC(p, q);
                    const R b2  = ST<S>::norm(bpq);
                    const R a = ST<S>::re(CC(p, p)), d = ST<S>::re(CC(q, q));
                    if (b2 > thr2 && b2 > th0sq * (d - a) * (d - a)) {
                        act               = true;
                        const float ib = rsqrtf((float)b2);  // 1 / |b|
                        const float t0 = 0.5f * (float)(d - a) * ib;
                        const float t  = copysignf(1.f, t0) / (fabsf(t0) + sqrtf(fmaf(t0, t0, 1.f)));
                        const float c0 = rsqrtf(fmaf(t, t, 1.f));
                        cc             = c0;
                        ss             = t * c0;
                        R x            = fma(cc, cc, ss * ss) - 1.0;
                        R f            = fma(fma(0.375, x, -0.5), x, 1.0);
                        cc *= f;
                        ss *= f;
                        if constexpr (std::is_same<S, double>::value) {
                            ex = ST<S>::re(bpq) >= 0.0 ? 1.0 : -1.0;
                        } else {
                            ex = ST<S>::re(bpq) * (R)ib;
                            ey = ST<S>::im(bpq) * (R)ib;
                            x  = fma(ex, ex, ey * ey) - 1.0;
                            f  = fma(fma(0.375, x, -0.5), x, 1.0);
                            ex *= f;
                            ey *= f;
                        }
                    }
                }
                pp[lane] = p;
                pq[lane] = q;
                rc[lane] = cc;
                rs[lane] = ss;
                jp[lane] = ST<S>::make(-ss * ex, ss * ey);
                jq[lane] = ST<S>::make(cc * ex, -cc * ey);
            }
            if (!__any_sync(0xffffffffu, act)) continue;  // warp-uniform: nothing to rotate
            rotated = true;
            __syncwarp();
            // V <- V J, the accumulated rotations (only needed for the Ritz vectors)
            if (want_w) {
                for (int it = lane; it < npair * m; it += 32) {
                    const int k = it / m, r = it - k * m;
                    const R   c = rc[k], sn = rs[k];
                    if (sn == 0.0) continue;
                    const int p = pp[k], q = pq[k];
                    const S   vp = VV(r, p), vq = VV(r, q);
                    VV(r, p) = cfma(vq, jp[k], cscale(vp, c));
                    VV(r, q) = cfma(vq, jq[k], cscale(vp, sn));
                }
            }
            // C <- J^H C J in 2 x 2 blocks: rows of pair k, columns of pair l, one block per lane,
            // k <= l computed and the block below the diagonal mirrored (C stays exactly Hermitian),
            // so each off-diagonal pair of entries costs one two-sided rotation
            for (int it = lane; it < nblk; it += 32) {
                int k = 0, rem = it;
                while (rem >= npair - k) {
                    rem -= npair - k;
                    ++k;
                }
                const int l = k + rem;
                if (rs[k] == 0.0 && rs[l] == 0.0) continue;  // both rotations are the identity
                const int  pk = pp[k], qk = pq[k], pl = pp[l], ql = pq[l];
                const bool hk = qk < m, hl = ql < m;  // q = m is the bye of an odd m
                const S    b00 = CC(pk, pl), b01 = hl ? CC(pk, ql) : ST<S>::zero();
                const S    b10 = hk ? CC(qk, pl) : ST<S>::zero(), b11 = (hk && hl) ? CC(qk, ql) : ST<S>::zero();
                const R    cl = rc[l], sl = rs[l], ck = rc[k], sk = rs[k];
                const S    jpl = jp[l], jql = jq[l], jpk = ST<S>::conj(jp[k]), jqk = ST<S>::conj(jq[k]);
                const S    t00 = cfma(b01, jpl, cscale(b00, cl)), t01 = cfma(b01, jql, cscale(b00, sl));
                const S    t10 = cfma(b11, jpl, cscale(b10, cl)), t11 = cfma(b11, jql, cscale(b10, sl));
                const S    n00 = cfma(jpk, t10, cscale(t00, ck)), n01 = cfma(jpk, t11, cscale(t01, ck));
                const S    n10 = cfma(jqk, t10, cscale(t00, sk)), n11 = cfma(jqk, t11, cscale(t01, sk));
                CC(pk, pl) = n00;
                if (hl) CC(pk, ql) = n01;
                if (hk) CC(qk, pl) = n10;
                if (hk && hl) CC(qk, ql) = n11;
                if (k != l) {
                    CC(pl, pk) = ST<S>::conj(n00);
                    if (hl) CC(ql, pk) = ST<S>::conj(n01);
                    if (hk) CC(pl, qk) = ST<S>::conj(n10);
                    if (hk && hl) CC(ql, qk) = ST<S>::conj(n11);
                }
            }
            __syncwarp();
            if (lane < npair && rs[lane] != 0.0) {  // Hermitian diagonal stays real
                const int p = pp[lane], q = pq[lane];
                CC(p, p)    = ST<S>::make(ST<S>::re(CC(p, p)), 0.0);
                CC(q, q)    = ST<S>::make(ST<S>::re(CC(q, q)), 0.0);
            }
            __syncwarp();
        }
        if (!want_w && !rotated) {
            converged = true;
            break;
        }
    }
    if (!converged && want_w) {  // the cap ended the sweeps: one last check of the couplings
        R off2 = 0;
        for (int q = lane; q < m * m; q += 32) {
            const int i = q / m, c = q - i * m;
            if (i < c) off2 = fmax(off2, ST<S>::norm(CC(i, c)));
        }
        off2      = warp_max(off2);
        converged = off2 <= thr2 || off2 == 0.0;
    }
    if (!want_w) {
        // lambda_p = C_pp + sum_q |C_pq|^2 / (C_pp - C_qq) over the couplings left above the
        // threshold (all with angles below 1e-4); the small terms in FP32, the sum in FP64
        R lam[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int p = lane + 32 * h;
            if (p >= m) continue;
            const R cpp = ST<S>::re(CC(p, p));
            float   cor = 0.f;
            for (int q = 0; q < m; ++q) {
                if (q == p) continue;
                const R b2 = ST<S>::norm(CC(p, q));
                const R g  = cpp - ST<S>::re(CC(q, q));
                if (b2 > thr2 && g != 0.0) cor += __fdividef((float)b2, (float)g);
            }
            lam[h] = cpp + (R)cor;
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int p = lane + 32 * h;
            if (p < m) CC(p, p) = ST<S>::make(lam[h], 0.0);
        }
        __syncwarp();
    }
    // ascending order of the Ritz values, nb smallest out: the rank of each value among all (ties
    // by index, i.e. a stable sort) from integer keys that order as the doubles do (-0 as +0)
    long long* key = reinterpret_cast<long long*>(rc);  // reuse: me doubles hold m keys
    int*       ord = reinterpret_cast<int*>(jp);
    for (int i = lane; i < m; i += 32) {
        const long long v = __double_as_longlong(ST<S>::re(CC(i, i)) + 0.0);
        key[i]            = v >= 0 ? v : v ^ 0x7fffffffffffffffLL;
    }
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
        const long long ki = key[i];
        int             rk = 0;
        for (int j = 0; j < m; ++j) {
            const long long kj = key[j];
            rk += (kj < ki) || (kj == ki && j < i);
        }
        ord[rk] = i;
    }
    __syncwarp();
    for (int j = lane; j < nb; j += 32) {
        const R ev = ST<S>::re(CC(ord[j], ord[j]));
        Eout[(size_t)b * nb + j] = ev;
        if (!isfinite(ev)) bad = true;
    }
    // W = (I - E/2) V[:, ord[:nb]] (Loewdin) or L^-H V[:, ord[:nb]] (Cholesky)
    if (want_w && lowdin) {
        // W = V - E V / 2 (FP64) + 3/8 E (E V) (FP32, ~|E|^2)
        for (int q = lane; q < m * nb; q += 32) {
            const int i = q / nb, c = q - i * nb;
            const int oc = ord[c];
            F         acc = ST<F>::zero();
            for (int j = 0; j < m; ++j) acc = cfma(Ef[i * m + j], to_lower(VV(j, oc)), acc);
            Gf[q] = acc;
        }
        __syncwarp();
        for (int q = lane; q < m * nb; q += 32) {
            const int i = q / nb, c = q - i * nb;
            const int oc = ord[c];
            S         acc = ST<S>::zero();
            F         ac2 = ST<F>::zero();
            for (int j = 0; j < m; ++j) {
                const S eij = (i == j) ? ST<S>::make(ST<S>::re(LL(i, j)) - 1.0, ST<S>::im(LL(i, j))) : LL(i, j);
                acc         = cfma(eij, VV(j, oc), acc);
                ac2         = cfma(Ef[i * m + j], Gf[j * nb + c], ac2);
            }
            Wg[(size_t)i * nb + c] = cadd(cfma(acc, ST<S>::make(-0.5, 0.0), VV(i, oc)), from_lower(cscale(ac2, 0.375f)));
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
    // converged is warp-uniform (warp reductions and warp-uniform branches); a NaN coupling never
    // compares below the threshold, so a non-finite matrix reports NONFINITE only
    if (lane == 0 && status && (bad || !converged)) atomicOr(status + b, bad ? 2 : 1);
#undef LL
#undef CC
#undef VV
}

// Ritz vectors x_j = X W[:, j] and gradients; one CTA per matrix, one warp per band.
template <typename S>
__global__ void k_refine_vectors(int n, int m, int nb, const cx<float>* __restrict__ X32, const S* __restrict__ Wg,
                                 cx<double>* __restrict__ Xout, double* __restrict__ grad, const DevParams P,
                                 const double* __restrict__ kpts, const int* __restrict__ G, int batch) {
    const int b = blockIdx.x;
    if (b >= batch) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const cx<float>* X = X32 + (size_t)b * m * n;  // [q][r]
    const S*  Wb   = Wg + (size_t)b * refine_small_elems(m, nb);
    for (int j = warp; j < nb; j += nw) {
        double sx = 0, sy = 0, sz = 0;
        for (int r = lane; r < n; r += 32) {
            S x = ST<S>::zero();
            for (int q = 0; q < m; ++q) {
                const cx<float> xv = X[(size_t)q * n + r];
                x                  = cfma(ST<S>::make((double)xv.x, (double)xv.y), Wb[(size_t)q * nb + j], x);
            }
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

template <typename S, bool SPARSE, bool YDONE>
static void refine_project_t(const typename Split<S>::type* H, int n, int ld, size_t mstride, const cx<float>* X32, int m,
                             S* work, S* small, int batch, cudaStream_t s, const SparseV& sv) {
    const size_t stage = proj_stage_bytes<S>(n, m);
    if (stage <= kProjStageBytes) {
        auto kern = k_refine_project<S, true, SPARSE, YDONE>;
        if (stage > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage);
        kern<<<batch, kProjNT, stage, s>>>(H, n, ld, mstride, X32, m, work, small, batch, sv);
    } else {
        k_refine_project<S, false, SPARSE, YDONE><<<batch, kProjNT, 0, s>>>(H, n, ld, mstride, X32, m, work, small, batch, sv);
    }
    count_launch();
}

template <typename S>
void launch_refine_project(const typename Split<S>::type* H, int n, int ld, size_t mstride, const cx<float>* X32, int m,
                           S* work, S* small, int batch, cudaStream_t s, const SparseV& sv, int* status, bool tensor_cores) {
    if (sv.on) {
        refine_project_t<S, true, false>(H, n, ld, mstride, X32, m, work, small, batch, s, sv);
        return;
    }
    if constexpr (!std::is_same<S, double>::value) {
        // complex dense H from order kRefineTcMinN: Y = H X on the tensor cores (Ozaki splitting,
        // refine_tc.cu), then S and A here. A real H stays on the FP32 pipe: with a quarter of the
        // complex multiply-adds per element there, the tensor-core form's slicing and second pass over
        // H do not pay (Ge nonlocal n = 181, 2000 k: 0.96 ms against 0.83)
        if (tensor_cores && n >= kRefineTcMinN &&
            launch_refine_y_tc(H, n, ld, mstride, X32, m, proj_mp<S>(m), work, refine_work_elems(n, m), status, batch, s)) {
            refine_project_t<S, false, true>(H, n, ld, mstride, X32, m, work, small, batch, s, sv);
            return;
        }
    }
    refine_project_t<S, false, false>(H, n, ld, mstride, X32, m, work, small, batch, s, sv);
}

template <typename S>
void launch_small_eigh(S* small, int m, int nb, double* Eout, S* W, int* status, int batch, cudaStream_t s, int cap) {
    const size_t smem = small_eigh_warp_bytes<S>(m) * kSmallWarps;
    auto         kern = k_small_eigh<S>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<(batch + kSmallWarps - 1) / kSmallWarps, 32 * kSmallWarps, smem, s>>>(small, m, nb, Eout, W != nullptr, status,
                                                                              batch, cap);
    count_launch();
}

template <typename S>
void launch_refine_vectors(int n, int m, int nb, const cx<float>* X32, const S* W, cx<double>* Xout, double* grad,
                           const DevParams& P, const double* d_k, const int* d_G, int batch, cudaStream_t s) {
    k_refine_vectors<S><<<batch, 256, 0, s>>>(n, m, nb, X32, W, Xout, grad, P, d_k, d_G, batch);
    count_launch();
}

#define UEPM_RF_INST(S)                                                                                             \
    template void launch_refine_project<S>(const typename Split<S>::type*, int, int, size_t, const cx<float>*, int, S*, S*, \
                                           int, cudaStream_t, const SparseV&, int*, bool);                        \
    template void launch_small_eigh<S>(S*, int, int, double*, S*, int*, int, cudaStream_t, int);                   \
    template void launch_refine_vectors<S>(int, int, int, const cx<float>*, const S*, cx<double>*, double*, const DevParams&, \
                                           const double*, const int*, int, cudaStream_t);
UEPM_RF_INST(double)
UEPM_RF_INST(cx<double>)
#undef UEPM_RF_INST

}  // namespace uepm
