// tridiag_eig.cu -- eigenvalues and eigenvectors of the real symmetric tridiagonal T from tridiag.cu.
//
// The reference computes ALL n eigenvalues with Eigen's implicit QR (Hamiltonian.cpp:125-134) and
// then keeps the first nb (BandStructure.cpp:183-184). Here only the nb lowest are computed:
//
//   k_bisect  Sturm-count bisection (one warp per matrix, one lane per eigenvalue index), with
//             LAPACK dstebz's pivot guard and absolute/relative stopping tolerances. Each value is
//             the j-th smallest eigenvalue of T to about eps * ||T||.
//   k_invit   inverse iteration (one warp per matrix, one lane per eigenvalue): LU with partial
//             pivoting of T - lambda I, three solves (FP64; two in FP32) from a deterministic
//             pseudo-random start, LAPACK dstein's shift perturbation for close eigenvalues and
//             modified Gram-Schmidt inside clusters (consecutive gaps <= 1e-3 ||T||_1), so
//             degenerate bands (Kramers pairs with SOC, the Gamma-point triplets) get an
//             orthonormal basis of their eigenspace. Groups that are degenerate to rounding
//             (consecutive gaps below 8 eps ||T||_1) share one shift placed just below the group
//             instead, and a Gram-Schmidt step that leaves little of a vector adds solves (see
//             k_invit). Iteration counts are bounded: nothing here can spin.
#include <algorithm>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

constexpr int kBisectWarpsPerBlock = 4;
constexpr int kInvitWarpsPerBlock  = 2;

// Reciprocal of a Sturm-count pivot: PTX's rcp.approx.ftz.f64 as the start value, refined by two
// Newton-Raphson steps for 1/q written with fused multiply-adds, e = 1 - q r, r <- r + r e (the
// relative error squares at every step; the fma form of P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34 (1990) 111-119). The pivots
// that reach it are normal numbers, |q| > pivmin >= DBL_MIN (the guard below replaces smaller ones);
// where 1/q itself would be subnormal (|q| > 2^1022) the approximation flushes it to zero, a
// perturbation of e^2 / q below 2^-1022. The GPU test of uepm_pivot_reciprocal_device bounds the
// result against the correctly rounded 1.0 / q over the whole pivot range.
__device__ __forceinline__ double sturm_rcp(double q) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(q));
    double er = fma(-q, r, 1.0);
    r         = fma(r, er, r);
    er        = fma(-q, r, 1.0);
    return fma(r, er, r);
}
// The pivot guard of the Sturm count (dstebz): a pivot within pivmin becomes -pivmin. It compares
// the high words (sign cleared), so it also catches pivots slightly above pivmin.
__device__ __forceinline__ double sturm_guard(double q, int piv_hi, double pivmin) {
    return ((__double2hiint(q) & 0x7fffffff) <= piv_hi) ? -pivmin : q;
}

// Sturm count: the number of eigenvalues of T below x, from the LDL^T pivots
// q_0 = d_0 - x, q_i = (d_i - x) - e_{i-1}^2 / q_{i-1} (pivots within pivmin replaced by -pivmin).
// FP64: 1 / q from sturm_rcp (a backward perturbation of e^2 far below the tolerance), and the
// pivot guard and sign test use integer compares on the high word, so a step issues 6 FP64
// instructions instead of a full IEEE division sequence.
__device__ __forceinline__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e2, int n, double x,
                                           double pivmin) {
    const int piv_hi = __double2hiint(pivmin);
    double    q      = sturm_guard(d[0] - x, piv_hi, pivmin);
    int       cnt    = (int)((unsigned)__double2hiint(q) >> 31);
    for (int i = 1; i < n; ++i) {
        const double r = sturm_rcp(q);
        q              = sturm_guard(fma(-e2[i - 1], r, d[i] - x), piv_hi, pivmin);
        cnt += (int)((unsigned)__double2hiint(q) >> 31);
    }
    return cnt;
}
__device__ __forceinline__ int sturm_count(const float* __restrict__ d, const float* __restrict__ e2, int n, float x,
                                           float pivmin) {
    float q = d[0] - x;
    if (fabsf(q) <= pivmin) q = -pivmin;
    int cnt = (q < 0.f);
    for (int i = 1; i < n; ++i) {
        q = (d[i] - x) - __fdividef(e2[i - 1], q);
        if (fabsf(q) <= pivmin) q = -pivmin;
        cnt += (q < 0.f);
    }
    return cnt;
}

// One group of LPM lanes per matrix (LPM = smallest power of two >= nb, at most 32), so a warp
// bisects 32 / LPM matrices at once and every lane carries an eigenvalue.
// Shared memory of one matrix in k_bisect: d and e^2 in T; for the FP64 kernel also their FP32
// rounding (hi) and remainders (lo), for the FP32 pre-bracketing and the double-single counts.
template <typename T>
__host__ __device__ inline size_t bisect_matrix_bytes(int n) {
    const size_t b = sizeof(T) * 2 * (size_t)n + (sizeof(T) == 8 ? sizeof(float) * 4 * (size_t)n : 0);
    return (b + 15) & ~(size_t)15;
}

// Double-single Sturm count: the same LDL^T recurrence with every quantity carried as an unevaluated
// FP32 pair (about 48 significant bits) on the FP32 pipe, ~30 FP32 instructions per step instead of
// 6 FP64 ones (64x wider pipe). Its backward error, a few 2^-48 ||T||, bounds how far the
// double-single phase of the bisection may go; the final bracket is confirmed and finished with
// FP64 counts. Two-sum (Knuth) and exact products (fmaf) with non-contracted operations.
struct dsf {
    float h, l;
};
__device__ __forceinline__ dsf ds_norm(float s, float e) {  // |s| >= |e|
    const float t = __fadd_rn(s, e);
    return dsf{t, __fsub_rn(e, __fsub_rn(t, s))};
}
__device__ __forceinline__ dsf ds_sub(dsf a, dsf b) {
    const float s  = __fsub_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    const float e  = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(__fsub_rn(0.f, b.h), bb));
    return ds_norm(s, __fadd_rn(e, __fsub_rn(a.l, b.l)));
}
__device__ __forceinline__ dsf ds_div(dsf a, dsf q) {
    const float rq = __frcp_rn(q.h);
    const float r1 = __fmul_rn(a.h, rq);
    const float p  = __fmul_rn(r1, q.h);
    const float pe = fmaf(r1, q.h, -p);
    float       t  = __fsub_rn(__fsub_rn(a.h, p), pe);
    t              = fmaf(-r1, q.l, __fadd_rn(t, a.l));
    return ds_norm(r1, __fmul_rn(t, rq));
}
__device__ __forceinline__ int sturm_count_ds(const float* dh, const float* dl, const float* e2h, const float* e2l, int n,
                                              dsf x, float pivmin) {
    dsf q = ds_sub(dsf{dh[0], dl[0]}, x);
    if (fabsf(q.h) <= pivmin) q = dsf{-pivmin, 0.f};
    int cnt = q.h < 0.f;
    for (int i = 1; i < n; ++i) {
        const dsf r = ds_div(dsf{e2h[i - 1], e2l[i - 1]}, q);
        q           = ds_sub(ds_sub(dsf{dh[i], dl[i]}, x), r);
        if (fabsf(q.h) <= pivmin) q = dsf{-pivmin, 0.f};
        cnt += q.h < 0.f;
    }
    return cnt;
}
__device__ __forceinline__ dsf ds_of(double v) {
    const float h = __double2float_rn(v);
    return dsf{h, __double2float_rn(v - (double)h)};
}

// Iterations per bisection phase: `cap` when positive (UEPM tuning max_iter), else 64 for the FP32
// and double-single pre-bracketing and 200 for the final phase (which needs ~60: the range over
// eps ||T||). An eigenvalue whose final bracket is still open when the cap ends it sets
// UEPM_K_NOCONVERGE in status; a non-finite bracket (NaN / Inf in T) sets UEPM_K_NONFINITE.
template <typename T>
__global__ void k_bisect(const T* __restrict__ dIn, const T* __restrict__ eIn, int n, int nb, int lpm, T* __restrict__ evOut,
                         int ev_ld, int batch, int cap, int* __restrict__ status) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mpw  = 32 / lpm;
    const int g    = lane / lpm, gl = lane - g * lpm;
    const int b    = (blockIdx.x * kBisectWarpsPerBlock + warp) * mpw + g;
    extern __shared__ __align__(16) unsigned char smraw[];
    unsigned char* mine = smraw + ((size_t)warp * mpw + g) * bisect_matrix_bytes<T>(n);
    T*             d    = reinterpret_cast<T*>(mine);
    T*             e2   = d + n;
    float*         df   = reinterpret_cast<float*>(e2 + n);  // FP64 kernel only: hi parts
    float*         e2f  = df + n;
    float*         dlo  = e2f + n;                           // lo parts
    float*         e2lo = dlo + n;
    const bool valid = b < batch;
    T          lo = T(3.0e38), hi = T(-3.0e38), emax2 = T(0);
    if (valid) {
        const T* dg = dIn + (size_t)b * n;
        const T* eg = eIn + (size_t)b * n;
        for (int i = gl; i < n; i += lpm) {
            const T di = dg[i];
            const T em = (i > 0) ? fabs(eg[i - 1]) : T(0);
            const T ep = (i < n - 1) ? fabs(eg[i]) : T(0);
            d[i]       = di;
            if (sizeof(T) == 8) {
                df[i]  = (float)di;
                dlo[i] = (float)((double)di - (double)df[i]);
            }
            if (i < n - 1) {
                e2[i] = eg[i] * eg[i];
                emax2 = max(emax2, e2[i]);
                if (sizeof(T) == 8) {
                    e2f[i]  = (float)e2[i];
                    e2lo[i] = (float)((double)e2[i] - (double)e2f[i]);
                }
            }
            lo = min(lo, di - em - ep);
            hi = max(hi, di + em + ep);
        }
    }
    // reductions within each lane group
    for (int o = lpm / 2; o > 0; o >>= 1) {
        lo    = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi    = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        emax2 = max(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
    }
    __syncwarp();
    if (!valid) return;
    const T eps    = num<T>::eps();
    const T pivmin = num<T>::tiny() * max(T(1), emax2);
    const T tnorm  = max(fabs(lo), fabs(hi));
    const T widen  = T(2) * eps * tnorm * T(n) + T(2) * pivmin;
    lo -= widen;
    hi += widen;
    const T   atol    = eps * tnorm;
    const int it_pre  = cap > 0 ? min(cap, 64) : 64;
    const int it_last = cap > 0 ? cap : 200;
    int       flags   = 0;
    for (int j = gl; j < nb; j += lpm) {
        T a = lo, c = hi;
        if (sizeof(T) == 8) {
            // FP32 pre-bracketing: bisect in FP32 (the FP32 pipe is 64x wider on GB300) to ~1e-6
            // relative, widen by 16 eps32 ||T|| (the backward error of an FP32 Sturm count is a few
            // eps32 ||T||) and keep the bracket only if two FP64 counts confirm it.
            const float pivf = FLT_MIN * fmaxf(1.f, (float)emax2);
            const float tolf = 4.f * FLT_EPSILON * (float)tnorm;
            float       af = (float)a, cf = (float)c;
            for (int it = 0; it < it_pre; ++it) {
                const float mf = 0.5f * (af + cf);
                if (cf - af <= tolf || mf <= af || mf >= cf) break;
                if (sturm_count(df, e2f, n, mf, pivf) > j) cf = mf;
                else af = mf;
            }
            const T w   = T(16) * T(FLT_EPSILON) * tnorm;
            const T lo2 = max(a, T(af) - w), hi2 = min(c, T(cf) + w);
            if (lo2 < hi2 && sturm_count(d, e2, n, lo2, pivmin) <= j && sturm_count(d, e2, n, hi2, pivmin) > j) {
                a = lo2;
                c = hi2;
                // double-single phase: bisect down to a few units of its backward error, widen by
                // that error and keep the bracket only if two FP64 counts confirm it
                const T ulp_ds = T(3.552713678800501e-15) * tnorm;  // 2^-48 ||T||
                T       ad = a, cd = c;
                for (int it = 0; it < it_pre; ++it) {
                    const T mid = T(0.5) * (ad + cd);
                    if (cd - ad <= T(64) * ulp_ds || mid <= ad || mid >= cd) break;
                    if (sturm_count_ds(df, dlo, e2f, e2lo, n, ds_of((double)mid), pivf) > j) cd = mid;
                    else ad = mid;
                }
                const T lo3 = max(a, ad - T(16) * ulp_ds), hi3 = min(c, cd + T(16) * ulp_ds);
                if (lo3 < hi3 && sturm_count(d, e2, n, lo3, pivmin) <= j && sturm_count(d, e2, n, hi3, pivmin) > j) {
                    a = lo3;
                    c = hi3;
                }
            }
        }
        // count(a) <= j < count(c) holds throughout; at most ~log2(range / atol) < 200 steps.
        bool done = false;
        for (int it = 0; it < it_last && !done; ++it) {
            const T mid = T(0.5) * (a + c);
            const T tol = max(atol, T(2) * eps * max(fabs(a), fabs(c)));
            done        = c - a <= tol || mid <= a || mid >= c;
            if (done) break;
            if (sturm_count(d, e2, n, mid, pivmin) > j) c = mid;
            else a = mid;
        }
        if (!done) {
            const T mid = T(0.5) * (a + c);
            done        = c - a <= max(atol, T(2) * eps * max(fabs(a), fabs(c))) || mid <= a || mid >= c;
        }
        if (!isfinite(a) || !isfinite(c)) flags |= 2;       // UEPM_K_NONFINITE
        else if (!done) flags |= 1;                         // UEPM_K_NOCONVERGE
        evOut[(size_t)b * ev_ld + j] = T(0.5) * (a + c);
    }
    if (flags && status) atomicOr(status + b, flags);
}

template <typename T>
void launch_bisect(const T* d, const T* e, int n, int nb, T* ev, int ev_ld, int batch, cudaStream_t s, int cap, int* status) {
    // lanes per matrix: >= nb (one lane per eigenvalue) and large enough that the d / e^2 copies
    // of the warp's matrices fit in 96 KB of shared memory per block
    const int max_mpw = (int)std::max<size_t>(1, (96 * 1024) / (bisect_matrix_bytes<T>(n) * kBisectWarpsPerBlock));
    int       lpm     = 1;
    while ((lpm < nb || 32 / lpm > max_mpw) && lpm < 32) lpm <<= 1;
    const int    mpw    = 32 / lpm;
    const int    warps  = (batch + mpw - 1) / mpw;
    const int    blocks = (warps + kBisectWarpsPerBlock - 1) / kBisectWarpsPerBlock;
    const size_t smem   = bisect_matrix_bytes<T>(n) * mpw * kBisectWarpsPerBlock;
    auto         kern   = k_bisect<T>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, 32 * kBisectWarpsPerBlock, smem, s>>>(d, e, n, nb, lpm, ev, ev_ld, batch, cap, status);
    count_launch();
}

// ------------------------------------------------------------------------------------------------
// Inverse iteration, one lane per eigenvalue (dstein's algorithm: LU of T - lam I with partial
// pivoting, solves from a deterministic start vector, Gram-Schmidt inside clusters of close
// eigenvalues). The per-lane arrays are interleaved by lane ([i][lane]) so that the lanes of a warp
// touch consecutive addresses at every step i (layout below).

__device__ __forceinline__ unsigned hash32(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Pivot reciprocal in the LU of T - lam I: the FP32 kernel uses the fast form (inverse iteration
// only needs a small backward error in its solves).
__device__ __forceinline__ float irecip(float b) { return __fdividef(1.f, b); }
__device__ __forceinline__ double irecip(double b) { return 1.0 / b; }
__device__ __forceinline__ float isqrt_inv(float a) { return rsqrtf(a); }
__device__ __forceinline__ double isqrt_inv(double a) { return 1.0 / sqrt(a); }

// Iterations per vector: the FP32 vectors of the mixed path only need their components outside the
// guard-banded subspace small (the FP64 Rayleigh-Ritz resolves mixing inside it), the FP64 vectors
// of the drop-in path are final.
template <typename T>
struct InvitIters {
    static constexpr int value = 3;
};
template <>
struct InvitIters<float> {
    static constexpr int value = 2;
};
constexpr double kGsKeep   = 0.02;  // Gram-Schmidt remainder below which two more solves follow
constexpr double kGsSettle = 0.5;   // remainder of the last step below which one more follows

// Work arrays per matrix, each n x LS interleaved by lane (LS = lanes in use, min(nb, 32)): U0, U1
// (the reciprocal diagonal and the first superdiagonal of U), Lm (the multipliers), Z (the vector; the forward sweep writes its
// right-hand side into it, Y[i] landing after Z[i] was consumed, and the back substitution
// overwrites it in place), then one word of row-interchange bits per 32 rows and lane (the third row
// of U is e[i+1] where rows were interchanged, else 0), then copies of d and e. SMEM: all in shared
// memory (one warp per CTA), else in the global workspace.
template <typename T>
__host__ __device__ inline size_t invit_smem_bytes(int n, int ls) {
    return sizeof(T) * (4 * (size_t)n * ls + 2 * (size_t)n) + sizeof(unsigned) * (size_t)((n + 31) / 32) * ls;
}

// cap > 0 (UEPM tuning max_iter) bounds the solves per vector; a vector that would need more than
// the cap (NIT, or the extra solves after a lossy Gram-Schmidt step) sets UEPM_K_NOCONVERGE.
template <typename T, bool SMEM>
__global__ void k_invit(const T* __restrict__ dIn, const T* __restrict__ eIn, const T* __restrict__ ev, int ev_ld, int n,
                        int nb, T* __restrict__ work, T* __restrict__ zOut, int* __restrict__ status, int batch, int cap) {
    constexpr int WPB  = SMEM ? 1 : kInvitWarpsPerBlock;
    constexpr int NIT  = InvitIters<T>::value;
    const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int     b    = blockIdx.x * WPB + warp;
    __shared__ T   s_lam[WPB][33];
    __shared__ int s_gs[WPB][33];
    extern __shared__ __align__(16) unsigned char smraw[];
    if (b >= batch) return;
    const int LS = min(nb, 32);
    const T*  d  = dIn + (size_t)b * n;
    const T*  e  = eIn + (size_t)b * n;
    T*        W  = SMEM ? reinterpret_cast<T*>(smraw) : work + (size_t)b * invit_work_elems<T>(n);
    T *U0 = W, *U1 = W + (size_t)n * LS, *Lm = W + (size_t)2 * n * LS, *Z = W + (size_t)3 * n * LS;
    if (SMEM) {  // the recurrences read d and e at every step: keep them next to the factors
        T* ds = W + (size_t)4 * n * LS;
        T* es = ds + n;
        for (int i = lane; i < n; i += 32) {
            ds[i] = d[i];
            es[i] = e[i];
        }
        __syncwarp();
        d = ds;
        e = es;
    }
    unsigned* SW = reinterpret_cast<unsigned*>(W + (size_t)4 * n * LS + (SMEM ? 2 * (size_t)n : 0));  // [n/32][LS]
    T*        zb = zOut + (size_t)b * nb * n;  // final vectors, [j][i]
#define AT(X, i) X[(size_t)(i) * LS + lane]

    // ||T||_1 for the cluster tolerance and the tiny-pivot replacement (dstein / dlagts).
    T onenrm = 0;
    for (int i = lane; i < n; i += 32) {
        const T r = fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : T(0)) + (i < n - 1 ? fabs(e[i]) : T(0));
        onenrm    = max(onenrm, r);
    }
    onenrm          = warp_max(onenrm);
    const T eps     = num<T>::eps();
    const T ortol   = T(1e-3) * onenrm;
    const T pivtiny = eps * onenrm;
    // Eigenvalues closer than ptight are one eigenvalue to the working precision (the two members
    // of a Kramers pair differ by rounding in T). dstein's shifts (the eigenvalue, then + 10 eps
    // |lambda|) would put every member's shift inside the rounding band of the factorisation, where
    // the solve returns one rounding-chosen direction of the eigenspace whatever the start vector;
    // the second member then differs from the first only by rounding and Gram-Schmidt keeps noise
    // (seen in FP32 as Ritz errors up to 1e-5 eV on the second band of a pair at about one k-point
    // in a thousand). Instead every member of such a group takes one shift p below the group,
    // p = max(8 eps ||T||_1, 2 x the group's spread) and at most half-way to the eigenvalue
    // below: the solve then stretches the group's eigenspace nearly evenly (by at most 1.5x
    // between members where the eigenvalue below does not cap the offset), the start vectors keep
    // their directions inside it, Gram-Schmidt keeps
    // them orthogonal, and the rest of the spectrum still shrinks by p / gap per solve. (Detecting
    // groups up to 64 eps ||T||_1 was tried: it also grouped the genuinely split pairs of
    // zinc-blende crystals with spin-orbit, whose larger shared offsets left up to 2e-8 eV.)
    const T ptight = T(8) * eps * onenrm;  // consecutive gaps below this form a group
    const T poff   = ptight;               // smallest offset of a group's shared shift
    // largest |z| for which sum z^2 stays finite
    const T   zsafe  = sizeof(T) == 4 ? T(1e17) : T(1e150);
    bool      bad    = false;
    bool      capped = false;  // warp-uniform: a vector wanted more solves than the cap allows
    const int maxit  = cap > 0 ? cap : NIT + 2;

    // carried across groups of 32: the previous shift, eigenvalue and cluster start
    T   prev_lam = T(0), prev_ev = T(0);
    int prev_gs  = 0;
    for (int g0 = 0; g0 < nb; g0 += 32) {
        const int gn = min(32, nb - g0);
        if (lane == 0) {
            T   pl = prev_lam, pe = prev_ev;
            int pg = prev_gs;
            for (int q = 0; q < gn; ++q) {
                const int  j     = g0 + q;
                const T    x     = ev[(size_t)b * ev_ld + j];
                const bool tprev = j > 0 && x - pe < ptight;
                const bool tnext = j + 1 < nb && ev[(size_t)b * ev_ld + j + 1] - x < ptight;
                T          xj    = x;
                if (tprev) {
                    xj = pl;  // a later member of a degenerate group: the group's shift and cluster
                } else {
                    if (tnext) {  // the first member: the group's spread, then its shift
                        int jl = j + 1;
                        while (jl + 1 < nb && ev[(size_t)b * ev_ld + jl + 1] - ev[(size_t)b * ev_ld + jl] < ptight) ++jl;
                        const T p = max(poff, T(2) * (ev[(size_t)b * ev_ld + jl] - x));
                        xj        = x - (j > 0 ? min(p, T(0.5) * (x - pe)) : p);
                    }
                    if (j > 0) {
                        const T pertol = T(10) * fabs(eps * xj);
                        if (xj - pl < pertol) xj = pl + pertol;
                        if (xj - pl > ortol) pg = j;
                    } else {
                        pg = 0;
                    }
                }
                s_lam[warp][q] = xj;
                s_gs[warp][q]  = pg;
                pl             = xj;
                pe             = x;
            }
            prev_lam = pl;
            prev_ev  = pe;
            prev_gs  = pg;
        }
        __syncwarp();
        prev_lam = __shfl_sync(0xffffffffu, prev_lam, 0);
        prev_ev  = __shfl_sync(0xffffffffu, prev_ev, 0);
        prev_gs  = __shfl_sync(0xffffffffu, prev_gs, 0);
        const bool active = lane < gn;
        const T    lam    = active ? s_lam[warp][lane] : T(0);
        const int  j      = g0 + lane;
        bool       clus   = false;  // any vector of this group orthogonalised against earlier ones
        for (int q = 0; q < gn; ++q) clus |= s_gs[warp][q] < g0 + q;

        // deterministic start vector in (-1, 1)
        if (active)
            for (int i = 0; i < n; ++i) {
                const unsigned h = hash32((unsigned)j * 0x9e3779b9U + (unsigned)i * 0x85ebca6bU + 0x27d4eb2fU);
                AT(Z, i)         = T(2) * T(h & 0xffffff) / T(16777216) - T(1) + T(1e-3);
            }
        __syncwarp();

        T   sc   = T(1);              // pending scale of Z
        int need = min(NIT, maxit);   // solves to run (raised after a Gram-Schmidt step that kept little)
        capped |= NIT > maxit;
        for (int it = 0; it < need; ++it) {
            if (active) {
                T rp = AT(Z, 0) * sc;
                if (it == 0) {
                    // LU with partial pivoting of T - lam I (factors kept), applied to Z -> Y. The
                    // interchange is a select, not a branch (lanes pivot differently), and U0 holds
                    // the reciprocal of the pivot (tiny pivots replaced by +-pivtiny, as dlagtf
                    // perturbs them), so both solves multiply.
                    T        p0 = d[0] - lam, p1 = (n > 1) ? e[0] : T(0);
                    unsigned bits = 0;
                    for (int i = 0; i < n - 1; ++i) {
                        const T    s0 = e[i], s1 = d[i + 1] - lam, s2 = (i + 1 < n - 1) ? e[i + 1] : T(0);
                        const T    rs = AT(Z, i + 1) * sc;
                        const bool sw = fabs(p0) < fabs(s0);
                        T          den = sw ? s0 : p0;
                        if (fabs(den) < pivtiny) den = (den < T(0)) ? -pivtiny : pivtiny;
                        const T rd = irecip(den);
                        const T l  = (sw ? p0 : s0) * rd;
                        const T u1 = sw ? s1 : p1, zi = sw ? rs : rp;
                        AT(U0, i)  = rd;
                        AT(U1, i)  = u1;
                        AT(Z, i)   = zi;
                        AT(Lm, i)  = l;
                        p0         = fma(-l, u1, sw ? p1 : s1);
                        p1         = sw ? -l * s2 : s2;
                        rp         = fma(-l, zi, sw ? rp : rs);
                        bits |= (unsigned)sw << (i & 31);
                        if ((i & 31) == 31) {
                            AT(SW, i >> 5) = bits;
                            bits           = 0;
                        }
                    }
                    if (((n - 1) & 31) != 0) AT(SW, (n - 2) >> 5) = bits;
                    if (fabs(p0) < pivtiny) p0 = (p0 < T(0)) ? -pivtiny : pivtiny;
                    AT(U0, n - 1) = irecip(p0);
                } else {
                    // the same elimination on the new right-hand side
                    for (int i = 0; i < n - 1; ++i) {
                        const T    rs = AT(Z, i + 1) * sc;
                        const T    l  = AT(Lm, i);
                        const bool sw = (AT(SW, i >> 5) >> (i & 31)) & 1u;
                        const T    zi = sw ? rs : rp;
                        AT(Z, i)      = zi;
                        rp            = fma(-l, zi, sw ? rp : rs);
                    }
                }
                // back substitution into Z with the 2-norm and the largest entry
                T z2 = T(0), z1 = rp * AT(U0, n - 1);
                AT(Z, n - 1) = z1;
                T ss = z1 * z1, zmax = fabs(z1);
                for (int i = n - 2; i >= 0; --i) {
                    const bool sw = (AT(SW, i >> 5) >> (i & 31)) & 1u;
                    const T    u2 = (sw && i + 1 < n - 1) ? e[i + 1] : T(0);
                    const T    zi = (AT(Z, i) - AT(U1, i) * z1 - u2 * z2) * AT(U0, i);
                    AT(Z, i)      = zi;
                    ss            = fma(zi, zi, ss);
                    zmax          = max(zmax, fabs(zi));
                    z2            = z1;
                    z1            = zi;
                }
                if (!(zmax > T(0)) || !isfinite(zmax)) {
                    bad = true;
                    sc  = T(0);
                } else if (zmax <= zsafe) {
                    sc = isqrt_inv(ss);
                } else {  // rescale by the largest entry before squaring
                    const T inv = T(1) / zmax;
                    ss          = T(0);
                    for (int i = 0; i < n; ++i) {
                        const T zi = AT(Z, i) * inv;
                        AT(Z, i)   = zi;
                        ss         = fma(zi, zi, ss);
                    }
                    sc = isqrt_inv(ss);
                }
            }
            if (clus) {
                // modified Gram-Schmidt inside clusters, in index order (warp-cooperative), on
                // normalised vectors
                if (active)
                    for (int i = 0; i < n; ++i) AT(Z, i) *= sc;
                sc = T(1);
                __syncwarp();
                T kept2 = T(1);  // smallest squared norm left by the projections (unit vectors in)
                for (int q = 0; q < gn; ++q) {
                    const int jq = g0 + q;
                    const int gs = s_gs[warp][q];
                    if (gs >= jq) continue;
                    for (int p = gs; p < jq; ++p) {
                        // previous vector: this group's Z column, or an earlier group's final output
                        T dot = T(0);
                        for (int i = lane; i < n; i += 32) {
                            const T zp = (p >= g0) ? Z[(size_t)i * LS + (p - g0)] : zb[(size_t)p * n + i];
                            dot        = fma(zp, Z[(size_t)i * LS + q], dot);
                        }
                        dot = warp_sum(dot);
                        for (int i = lane; i < n; i += 32) {
                            const T zp = (p >= g0) ? Z[(size_t)i * LS + (p - g0)] : zb[(size_t)p * n + i];
                            Z[(size_t)i * LS + q] -= dot * zp;
                        }
                        __syncwarp();
                    }
                    T ss = T(0);
                    for (int i = lane; i < n; i += 32) ss = fma(Z[(size_t)i * LS + q], Z[(size_t)i * LS + q], ss);
                    ss        = warp_sum(ss);
                    kept2     = min(kept2, ss);
                    const T r = (ss > T(0)) ? T(1) / sqrt(ss) : T(0);
                    for (int i = lane; i < n; i += 32) Z[(size_t)i * LS + q] *= r;
                    __syncwarp();
                }
                // A vector that came out of its solve nearly parallel to an earlier one (the start
                // vectors' components in a degenerate eigenspace can nearly coincide) keeps only a
                // small remainder, in which rounding and the components outside the eigenspace are
                // magnified by 1 / remainder: give it two more solves. A last step that still
                // removes most of a vector (close groups still turning into each other) gets one
                // more. At most NIT + 2 solves in all; kept2 is warp-uniform (warp sums), so the
                // trip count stays uniform.
                int want_n = need;
                if (kept2 < T(kGsKeep * kGsKeep)) want_n = min(NIT + 2, max(need, it + 3));
                else if (it == need - 1 && kept2 < T(kGsSettle * kGsSettle)) want_n = min(NIT + 2, it + 2);
                capped |= want_n > maxit;
                need = min(want_n, maxit);
            }
        }
        // write this group's vectors ([j][i], coalesced over i), with the pending scale
        const T scq = sc;
        __syncwarp();
        for (int q = 0; q < gn; ++q) {
            const T s = __shfl_sync(0xffffffffu, scq, q);
            for (int i = lane; i < n; i += 32) zb[(size_t)(g0 + q) * n + i] = Z[(size_t)i * LS + q] * s;
        }
        __syncwarp();
    }
#undef AT
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0 && status && (bad || capped)) status[b] |= (bad ? 2 : 0) | (capped ? 1 : 0);  // NONFINITE, NOCONVERGE
}

template <typename T>
void launch_invit(const T* d, const T* e, const T* ev, int ev_ld, int n, int nb, T* work, T* z, int* status, int batch,
                  cudaStream_t s, int cap) {
    const size_t smem = invit_smem_bytes<T>(n, std::min(nb, 32));
    // shared memory where at least four warps fit per SM; beyond that the latency-bound recurrences
    // run better from the L1/L2-cached workspace at higher occupancy (FP32, 2000 k: Ge SOC n = 362
    // 1.9 -> 1.6 ms, one warp per SM in shared memory; Si n = 137 0.13 ms in shared memory against
    // 0.18 from the workspace)
    if (smem <= 56 * 1024 || (sizeof(T) == 8 && smem <= 200 * 1024)) {
        auto kern = k_invit<T, true>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<batch, 32, smem, s>>>(d, e, ev, ev_ld, n, nb, work, z, status, batch, cap);
    } else {
        const int blocks = (batch + kInvitWarpsPerBlock - 1) / kInvitWarpsPerBlock;
        k_invit<T, false><<<blocks, 32 * kInvitWarpsPerBlock, 0, s>>>(d, e, ev, ev_ld, n, nb, work, z, status, batch, cap);
    }
    count_launch();
}

template void launch_bisect<double>(const double*, const double*, int, int, double*, int, int, cudaStream_t, int, int*);
template void launch_bisect<float>(const float*, const float*, int, int, float*, int, int, cudaStream_t, int, int*);
template void launch_invit<double>(const double*, const double*, const double*, int, int, int, double*, double*, int*, int,
                                   cudaStream_t, int);
template void launch_invit<float>(const float*, const float*, const float*, int, int, int, float*, float*, int*, int,
                                  cudaStream_t, int);

}  // namespace uepm

// ------------------------------------------------------------------------------------------------
namespace {
__global__ void k_pivot_reciprocal(const double* __restrict__ q, double pivmin, size_t n, double* __restrict__ r) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) r[t] = uepm::sturm_rcp(uepm::sturm_guard(q[t], __double2hiint(pivmin), pivmin));
}
}  // namespace

extern "C" int uepm_pivot_reciprocal_device(const double* d_q, double pivmin, size_t n, double* d_r, void* stream) {
    if (n == 0) return 0;
    if (!d_q || !d_r || !(pivmin > 0.0)) return -1;  // UEPM_ERR_INVALID
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_pivot_reciprocal<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_q, pivmin, n, d_r);
    uepm::count_launch();
    return cudaGetLastError() == cudaSuccess ? 0 : -4;  // UEPM_ERR_CUDA
}
