// refine_tc.cu -- Y = H X of the Rayleigh-Ritz refinement (mixed path, complex H) on the tensor
// cores, to double-single accuracy.
//
// No reference counterpart (the reference only has the FP64 Eigen solve). The double-single form of
// this product (refine.cu) costs about ten FP32 operations per real multiply-add. Here both operands
// are split into small integers instead (the error-free splitting of Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012): with a power-of-two scale per
// row of H (2^E_r above twice the row's largest |Re|, |Im|) and per vector of X (2^F_j likewise),
//   H(r, c) = 2^(E_r - 6) sum_s alpha_s 2^(-6 s),   X(c, j) = 2^(F_j - 6) sum_t gamma_t 2^(-6 t),
// with integers |alpha|, |gamma| <= 32 (7 slices each: 42 bits below the scale; H is taken from its
// FP32 pair hi + lo exactly, X from FP32). Every slice product alpha gamma is an integer of at most
// 2^10, so the sum over the K = 2n real terms of the pairs (s, t) with the same weight w = s + t
// (at most 7 pairs, s, t < 7, w <= 7) stays below 7 2^10 2n <= 2^24 for n <= 1170: an FP32
// accumulation of exact BF16 products is exact. The 36 pairs run as BF16 tcgen05.mma (kind::f16)
// into 8 TMEM accumulators D_w, one per weight, and
//   Y(r, j) = 2^(E_r + F_j - 12) sum_w D_w 2^(-6 w)
// is summed in double-single. Dropped terms (weights 8 and beyond, the slices' remainders) are below
// about 2^-43 of 2^(E_r + F_j) per real term.
//
// Real form of the complex product (K = 2n): A = [Re H | Im H] (rows r), B rows j' = j: [Re X_j |
// -Im X_j], rows j' = mp + j: [Im X_j | Re X_j], so that D(r, j) = Re Y(r, j), D(r, mp + j) =
// Im Y(r, j). K is walked in chunks of 16 complex columns (K 32: their Re parts, then their Im
// parts).
//
// One CTA (512 threads) per 128-row tile of one matrix: a pass over the tile's rows for their
// scales (and over X for the vectors'), then the chunks pipelined over two operand buffers: warps
// 1..15 slice chunk q into buffer q & 1 (after the MMAs of chunk q - 2 released it) and signal an
// mbarrier, thread 0 issues the chunk's 72 MMAs and commits them to the buffer's mbarrier; at the
// end every warp reads its TMEM lane quarter and writes Y. All waits are bounded; a wait that gives
// up marks the matrix UEPM_K_NOCONVERGE.
#include <cuda_bf16.h>

#include "tcgen05.cuh"
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

namespace {

constexpr int       kYtNT     = 512;
constexpr int       kYtM      = 128;  // rows of H per CTA, one TMEM lane each
constexpr int       kYtC      = 16;   // complex columns per K chunk
constexpr int       kYtK      = 2 * kYtC;
constexpr int       kYtNmax   = 64;   // D columns: Re Y of the mp vectors, then Im Y, padded to 16
constexpr int       kYtSl     = 7;    // slices per operand
constexpr int       kYtW      = 8;    // weights w = s + t <= 7, one TMEM accumulator of 64 columns each
constexpr uint32_t  kYtCols   = 512;
constexpr size_t    kYtASlice = (size_t)kYtM * kYtK * 2;      // bytes of one BF16 slice of the row operand
constexpr size_t    kYtBSlice = (size_t)kYtNmax * kYtK * 2;   // of the column operand
constexpr size_t    kYtStage  = kYtSl * (kYtASlice + kYtBSlice);  // 84 KB
constexpr size_t    kYtSmem   = 2 * kYtStage;
constexpr long long kYtWaitCycles = 2000000000ll;  // ~1 s at the SM clock

// Bounded wait (~1 s) for the phase of the given parity; a wait that gives up sets the CTA's fail
// flag, and every later wait of the CTA returns at once (so a failed CTA ends in about a second).
__device__ __forceinline__ bool yt_wait(uint64_t* bar, uint32_t parity, volatile int* fail) {
    const long long t0 = clock64();
    while (!tc::mbar_try_wait(bar, parity)) {
        if (*fail) return false;
        if (clock64() - t0 > kYtWaitCycles) {
            *fail = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void two_sum(float& a, float& b) {  // (a, b) <- (fl(a + b), the rounding error)
    const float s  = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    b              = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    a              = s;
}

// the 7 slices of p + q (|p + q| < 32, |q| <= ulp(p) / 2), 8 values -> 7 x (8 BF16 = 16 bytes)
__device__ __forceinline__ void slice8(float (&p)[8], float (&q)[8], uint4 (&out)[kYtSl]) {
#pragma unroll
    for (int s = 0; s < kYtSl; ++s) {
        float a[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (s) two_sum(p[i], q[i]);
            a[i] = rintf(p[i]);
            p[i] = __fmul_rn(__fsub_rn(p[i], a[i]), 64.f);  // exact: |p - a| <= 1/2 and a multiple of ulp(p)
            q[i] = __fmul_rn(q[i], 64.f);
        }
        __nv_bfloat162 b0 = __floats2bfloat162_rn(a[0], a[1]), b1 = __floats2bfloat162_rn(a[2], a[3]);
        __nv_bfloat162 b2 = __floats2bfloat162_rn(a[4], a[5]), b3 = __floats2bfloat162_rn(a[6], a[7]);
        out[s] = make_uint4(*reinterpret_cast<uint32_t*>(&b0), *reinterpret_cast<uint32_t*>(&b1),
                            *reinterpret_cast<uint32_t*>(&b2), *reinterpret_cast<uint32_t*>(&b3));
    }
}

// 2^E with x < 2^(E - 1) for the largest |component| x of a row or vector (E = 0 for x = 0):
// returns 2^(6 - E), the multiplier that puts the values below 32 in magnitude
__device__ __forceinline__ void scale_of(float x, float& mul, int& E) {
    int e = 0;
    frexpf(x, &e);  // x = m 2^e, m in [1/2, 1)
    E   = x > 0.f ? e + 1 : 0;
    mul = ldexpf(1.f, 6 - E);
}

__global__ void __launch_bounds__(kYtNT, 1)
    k_refine_y_tc(const ds4* __restrict__ H, int n, int ld, size_t mstride, const cx<float>* __restrict__ X32, int m,
                  int mp, int N, float4* __restrict__ Yw, size_t ystride, int* __restrict__ status, int ntile) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ float    s_rmax[kYtM], s_rmul[kYtM], s_cmax[kYtNmax / 2], s_cmul[kYtNmax / 2];
    __shared__ int      s_rE[kYtM], s_cE[kYtNmax / 2];
    __shared__ uint64_t s_staged[2], s_done[2];
    __shared__ uint32_t s_tmem;
    __shared__ int      s_fail;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int b = blockIdx.x / ntile, r0 = (blockIdx.x - b * ntile) * kYtM;
    const ds4*       A  = H + (size_t)b * mstride;
    const cx<float>* Xg = X32 + (size_t)b * m * n;

    // ---- scales: rows of this tile, vectors of X; TMEM and the mbarriers ---------------------------
    if (tid < kYtM) s_rmax[tid] = 0.f;
    if (tid < kYtNmax / 2) s_cmax[tid] = 0.f;
    if (tid == 0) {
        s_fail = 0;
        tc::mbar_init(&s_staged[0], kYtNT - 32);
        tc::mbar_init(&s_staged[1], kYtNT - 32);
        tc::mbar_init(&s_done[0], 1);
        tc::mbar_init(&s_done[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(&s_tmem, kYtCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = s_tmem;
    {
        // rows: 4 threads per row, each with kYtPass loads in flight (the pass is bound by load latency)
        constexpr int kStep = kYtNT / kYtM, kYtPass = 8;
        const int     rl = tid & (kYtM - 1), part = tid >> 7, r = r0 + rl;
        const float4* Af = reinterpret_cast<const float4*>(A);  // (rhi, rlo, ihi, ilo)
        float         mx = 0.f;
        if (r < n) {
            int c = part;
            for (; c + (kYtPass - 1) * kStep < n; c += kYtPass * kStep) {
                float4 v[kYtPass];
#pragma unroll
                for (int u = 0; u < kYtPass; ++u) v[u] = __ldg(Af + (size_t)(c + u * kStep) * ld + r);
#pragma unroll
                for (int u = 0; u < kYtPass; ++u) mx = fmaxf(mx, fmaxf(fabsf(v[u].x), fabsf(v[u].z)));
            }
            for (; c < n; c += kStep) {
                const float4 v = __ldg(Af + (size_t)c * ld + r);
                mx             = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.z)));
            }
        }
        atomicMax(reinterpret_cast<int*>(&s_rmax[rl]), __float_as_int(mx));  // non-negative: int order
        // vectors: one warp per vector, reduced by shuffles (one store per vector)
        for (int j = warp; j < m; j += kYtNT / 32) {
            float xm = 0.f;
            for (int c = lane; c < n; c += 32) {
                const cx<float> x = Xg[(size_t)j * n + c];
                xm                = fmaxf(xm, fmaxf(fabsf(x.x), fabsf(x.y)));
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
            if (lane == 0) s_cmax[j] = xm;
        }
    }
    __syncthreads();
    if (tid < kYtM) scale_of(s_rmax[tid], s_rmul[tid], s_rE[tid]);
    if (tid < kYtNmax / 2) scale_of(s_cmax[tid], s_cmul[tid], s_cE[tid]);
    __syncthreads();

    // ---- chunks: warps 1..15 slice, thread 0 issues -----------------------------------------------
    const int nch = (n + kYtC - 1) / kYtC;
    bool      ok  = true;
    if (warp > 0) {
        const int wid = tid - 32;
        for (int q = 0; q < nch; ++q) {
            const int buf = q & 1;
            if (q >= 2) ok = yt_wait(&s_done[buf], ((q - 2) >> 1) & 1, &s_fail) && ok;  // the MMAs of chunk q - 2 read it
            unsigned char* st = smraw + (size_t)buf * kYtStage;
            unsigned char* sa = st;                                // slice s at s * kYtASlice
            unsigned char* sb = st + (size_t)kYtSl * kYtASlice;   // slice t at t * kYtBSlice
            const int      c0 = q * kYtC;
            for (int it = wid; it < 2 * kYtM + 4 * N; it += kYtNT - 32) {
                if (it < 2 * kYtM) {  // H: row rl, columns c0 + 8h .. + 7 -> K groups h (Re) and 2 + h (Im)
                    const int   rl = it & (kYtM - 1), h = it >> 7, r = r0 + rl;
                    const float mu = s_rmul[rl];
                    float       pr[8], qr[8], pi[8], qi[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int c = c0 + 8 * h + i;
                        const ds4 v = (r < n && c < n) ? A[(size_t)c * ld + r] : ds4{0.f, 0.f, 0.f, 0.f};
                        pr[i]       = v.rhi * mu;  // powers of two: exact
                        qr[i]       = v.rlo * mu;
                        pi[i]       = v.ihi * mu;
                        qi[i]       = v.ilo * mu;
                    }
                    uint4 o[kYtSl];
                    slice8(pr, qr, o);
#pragma unroll
                    for (int s = 0; s < kYtSl; ++s)
                        *reinterpret_cast<uint4*>(sa + s * kYtASlice + ((size_t)h * kYtM + rl) * 16) = o[s];
                    slice8(pi, qi, o);
#pragma unroll
                    for (int s = 0; s < kYtSl; ++s)
                        *reinterpret_cast<uint4*>(sa + s * kYtASlice + ((size_t)(2 + h) * kYtM + rl) * 16) = o[s];
                } else {  // X: row j' of the column operand, K group g
                    const int   u = it - 2 * kYtM, jr = u % N, g = u / N;
                    const bool  imr = jr >= mp;
                    const int   j = imr ? jr - mp : jr;
                    const bool  valid = jr < 2 * mp && j < m;
                    const float nu = valid ? s_cmul[j] : 0.f;
                    float       p[8], z[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int       c = c0 + 8 * (g & 1) + i;
                        const cx<float> x = (valid && c < n) ? Xg[(size_t)j * n + c] : cx<float>{0.f, 0.f};
                        // g 0, 1 pair with Re H: Re X (Re row) or Im X (Im row); g 2, 3 with Im H: -Im X or Re X
                        const float val = g < 2 ? (imr ? x.y : x.x) : (imr ? x.x : -x.y);
                        p[i]            = val * nu;
                        z[i]            = 0.f;
                    }
                    uint4 o[kYtSl];
                    slice8(p, z, o);
#pragma unroll
                    for (int t = 0; t < kYtSl; ++t)
                        *reinterpret_cast<uint4*>(sb + t * kYtBSlice + ((size_t)g * kYtNmax + jr) * 16) = o[t];
                }
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            tc::mbar_arrive(&s_staged[buf]);
        }
    } else if (lane == 0) {  // warp 0: thread 0 issues, its other lanes wait below
        const uint32_t idesc = tc::idesc_bf16(kYtM, N);
        const uint32_t base  = tc::smem_addr(smraw);
        for (int q = 0; q < nch; ++q) {
            const int buf = q & 1;
            if (!yt_wait(&s_staged[buf], (q >> 1) & 1, &s_fail)) {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            const uint32_t sa = base + (uint32_t)(buf * kYtStage), sb = sa + (uint32_t)(kYtSl * kYtASlice);
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {  // K steps of 16: groups 2 ks, 2 ks + 1
#pragma unroll
                for (int w = 0; w < kYtW; ++w) {
#pragma unroll
                    for (int s = (w > kYtSl - 1 ? w - (kYtSl - 1) : 0); s <= (w < kYtSl - 1 ? w : kYtSl - 1); ++s) {
                        const int      t     = w - s;
                        const uint64_t ad    = tc::smem_desc(sa + s * (uint32_t)kYtASlice + ks * 2 * kYtM * 16, kYtM * 16, 128);
                        const uint64_t bd    = tc::smem_desc(sb + t * (uint32_t)kYtBSlice + ks * 2 * kYtNmax * 16, kYtNmax * 16, 128);
                        const bool     first = q == 0 && ks == 0 && s == (w > kYtSl - 1 ? w - (kYtSl - 1) : 0);
                        tc::mma_f16(tbase + 64 * w, ad, bd, idesc, first ? 0u : 1u);
                    }
                }
            }
            tc::mma_commit(&s_done[buf]);
        }
    }
    if (warp == 0) __syncwarp();

    // ---- read back: D_w of this warp's lane quarter, 8-column units, summed in double-single -------
    {
        const int  last = nch - 1;
        const bool okw  = yt_wait(&s_done[last & 1], (last >> 1) & 1, &s_fail);  // the last commit covers all MMAs
        ok              = __syncthreads_and(ok && okw) != 0;
        tc::fence_after_sync();
        if (ok) {
            const int qd = warp & 3, wi = warp >> 2, r = r0 + 32 * qd + lane;
            for (int u = wi; u < N / 8; u += 4) {
                float h[8], l[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) h[i] = l[i] = 0.f;
#pragma unroll
                for (int w = kYtW - 1; w >= 0; --w) {  // smallest weight first
                    float d[8];
                    tc::tmem_ld8(tbase + ((uint32_t)(32 * qd) << 16) + 64 * w + 8 * u, d);
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        float x = ldexpf(d[i], -6 * w);  // exact: D_w is an integer below 2^24
                        two_sum(h[i], x);
                        l[i] = __fadd_rn(l[i], x);
                    }
                }
                if (r < n) {
                    float* Yr = reinterpret_cast<float*>(Yw + (size_t)b * ystride + (size_t)r * mp);
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int jr = 8 * u + i;
                        if (jr >= 2 * mp) continue;
                        const bool imr = jr >= mp;
                        const int  j   = imr ? jr - mp : jr;
                        const int  e   = s_rE[r - r0] + s_cE[j] - 12;
                        float      hh = h[i], ll = l[i];
                        two_sum(hh, ll);  // renormalised pair
                        Yr[(size_t)j * 4 + (imr ? 2 : 0)] = ldexpf(hh, e);
                        Yr[(size_t)j * 4 + (imr ? 3 : 1)] = ldexpf(ll, e);
                    }
                }
            }
        } else if (tid == 0 && status) {
            atomicOr(status + b, 1);  // UEPM_K_NOCONVERGE: a bounded wait gave up
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tbase, kYtCols);
    }
}

}  // namespace

bool launch_refine_y_tc(const ds4* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, int mp, void* work,
                        size_t ystride, int* status, int batch, cudaStream_t s) {
    const int N = (2 * mp + 15) / 16 * 16;
    if (n < 2 || n > 1024 || m > mp || N > kYtNmax || mp > kYtNmax / 2) return false;
    auto kern = k_refine_y_tc;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kYtSmem) != cudaSuccess) return false;
    const int ntile = (n + kYtM - 1) / kYtM;
    kern<<<batch * ntile, kYtNT, kYtSmem, s>>>(H, n, ld, mstride, X32, m, mp, N, reinterpret_cast<float4*>(work), ystride,
                                              status, ntile);
    count_launch();
    return true;
}

}  // namespace uepm
