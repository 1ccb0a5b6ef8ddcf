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

#include "tcgen05.cuh"
#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {

namespace {

constexpr int kBlkNT = 512;  // threads per CTA (16 warps)
constexpr int kBlkNW = kBlkNT / 32;
constexpr int kBlkNB = 16;   // panel width

// Tensor-core trailing update (complex matrices): tiles of 128 rows x NC columns (NC = 64, 48 or
// 32, the widest whose operand staging fits shared memory) of the trailing matrix, D = P_rows
// Q_cols^T in the real form with K = 64 (Re V, Im V, Re W, Im W of the panel's 16 reflectors), each
// operand split into TF32 hi + lo parts, both rounded to nearest, and all four products taken
// (about 2^-23 relative per product, the FP32 pipe's level: the spin-orbit matrices' Kramers pairs
// need it; hi hi + hi lo + lo hi with an unrounded lo left one pair in a few thousand split in the
// FP32 tridiagonal), accumulated in TMEM. The column operand and the accumulators are double-buffered, so that the MMAs of one tile run
// while the previous tile is read back and the next one staged.
constexpr int      kTcM       = 128;
constexpr int      kTcK       = 4 * kBlkNB;
constexpr int      kTcCols    = 512;  // TMEM columns: 2 buffers x (Re, Im+, Im-) x 64
constexpr int      kTcMinRows = 96;   // smaller trailing matrices take the SIMT update
__host__ __device__ constexpr size_t tc_stage_bytes(int nc) {  // A hi/lo, two B buffers hi/lo
    return (size_t)2 * (kTcM + 2 * nc) * kTcK * sizeof(float);
}
constexpr long long kTcWaitCycles = 2000000000ll;  // ~1 s at the SM clock: a bounded wait

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
    // with the tensor-core update: its operand staging overlays the per-warp partial vectors and
    // everything after them (dead during the trailing update; the zero padding of v is restored)
    static __host__ __device__ size_t bytes_tc(int n, int nc) {
        const size_t stage = sizeof(S) * (size_t)2 * kBlkNB * n + tc_stage_bytes(nc);
        const size_t base  = bytes(n);
        return stage > base ? stage : base;
    }
};

// Rows [r0, r0 + ROWS) of the panel in the real K-major form of the tensor-core operands: K index
// 0..15 Re V_k, 16..31 Im V_k, 32..47 Re W_k, 48..63 Im W_k; element (r, k) at float
// (k / 4) * ROWS * 4 + (r - r0) * 4 + k % 4, split into TF32 hi (rounded to nearest) and the
// remainder rounded to TF32 lo (x - hi - lo is below 2^-24 |x|). Rows past n are zero. Written by
// the worker warps (1..15).
template <int ROWS>
__device__ __forceinline__ void tc_stage(const cx<float>* Vp, const cx<float>* Wp, int n, int r0, float* hi, float* lo) {
    for (int it = threadIdx.x - 32; it < ROWS * 8; it += kBlkNT - 32) {
        const int rl = it % ROWS, gq = it / ROWS;  // consecutive threads: consecutive rows
        const int w = gq >> 2, g = gq & 3, r = r0 + rl;
        const cx<float>* src = (w ? Wp : Vp) + (size_t)(4 * g) * n + r;
        float re[4], im[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const cx<float> x = (r < n) ? src[(size_t)j * n] : cx<float>{0.f, 0.f};
            re[j]             = x.x;
            im[j]             = x.y;
        }
        const int gre = w * 8 + g, gim = gre + 4;  // 4-wide K groups of the Re and Im parts
        float4    h, l;
        h.x = tc::to_tf32(re[0]); h.y = tc::to_tf32(re[1]); h.z = tc::to_tf32(re[2]); h.w = tc::to_tf32(re[3]);
        l   = make_float4(tc::to_tf32(re[0] - h.x), tc::to_tf32(re[1] - h.y), tc::to_tf32(re[2] - h.z), tc::to_tf32(re[3] - h.w));
        *reinterpret_cast<float4*>(hi + ((size_t)gre * ROWS + rl) * 4) = h;
        *reinterpret_cast<float4*>(lo + ((size_t)gre * ROWS + rl) * 4) = l;
        h.x = tc::to_tf32(im[0]); h.y = tc::to_tf32(im[1]); h.z = tc::to_tf32(im[2]); h.w = tc::to_tf32(im[3]);
        l   = make_float4(tc::to_tf32(im[0] - h.x), tc::to_tf32(im[1] - h.y), tc::to_tf32(im[2] - h.z), tc::to_tf32(im[3] - h.w));
        *reinterpret_cast<float4*>(hi + ((size_t)gim * ROWS + rl) * 4) = h;
        *reinterpret_cast<float4*>(lo + ((size_t)gim * ROWS + rl) * 4) = l;
    }
}

// Waits (bounded, ~1 s) for the phase of the given parity of the mbarrier at bar. With a fail flag:
// a wait that gives up sets it, and every later wait of the CTA returns at once.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* fail = nullptr) {
    const long long t0 = clock64();
    while (!tc::mbar_try_wait(bar, parity)) {
        if (fail && *fail) return false;
        if (clock64() - t0 > kTcWaitCycles) {
            if (fail) *fail = 1;
            return false;
        }
    }
    return true;
}

// A tile of the tensor-core update: rows [rb, rb + 128) (stored: [rlo, rhi)), columns [cb, cb + NC)
// (stored: [clo, chi)); its sequence number (over the kernel) selects the buffer (seq & 1) and the
// mbarrier phase (seq >> 1).
struct TcTile {
    int      rb, rlo, rhi, cb, clo, chi;
    uint32_t seq;
};

// The issuer (one thread): waits for the workers' staging of tile t, issues its 64 MMAs (Re: 8 chunk
// pairs, Im+ and Im-: 4 each, 4 split products per pair) into TMEM buffer seq & 1 and commits them to
// that buffer's MMA mbarrier. False if the wait gave up (nothing issued).
template <int NC>
__device__ __forceinline__ bool tc_issue(const TcTile& t, const float* aH, const float* aL, const float* bH0,
                                         uint32_t tbase, uint64_t* staged, uint64_t* done, volatile int* fail) {
    const uint32_t buf = t.seq & 1u;
    if (!tc_wait(staged + buf, (t.seq >> 1) & 1u, fail)) return false;
    tc::fence_after_sync();
    constexpr uint32_t idesc = tc::idesc_tf32(kTcM, NC);
    const float*       bH    = bH0 + (size_t)buf * 2 * NC * kTcK;
    const float*       bL    = bH + (size_t)NC * kTcK;
    const uint64_t     ah0 = tc::smem_desc(tc::smem_addr(aH), kTcM * 16, 128);
    const uint64_t     al0 = tc::smem_desc(tc::smem_addr(aL), kTcM * 16, 128);
    const uint64_t     bh0 = tc::smem_desc(tc::smem_addr(bH), NC * 16, 128);
    const uint64_t     bl0 = tc::smem_desc(tc::smem_addr(bL), NC * 16, 128);
    // 8-wide K chunks: 0,1 Re V; 2,3 Im V; 4,5 Re W; 6,7 Im W. A chunk moves the start address
    // (descriptor bits 0-13, in 16-byte units) by 2 * rows core-matrix rows.
    constexpr int pa[16] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 4, 5, 2, 3, 6, 7};
    constexpr int pb[16] = {4, 5, 6, 7, 0, 1, 2, 3, 6, 7, 2, 3, 4, 5, 0, 1};
#pragma unroll
    for (int p = 0; p < 16; ++p) {
        const int      acc   = p < 8 ? 0 : p < 12 ? 1 : 2;  // Re, Im+, Im-
        const uint32_t d     = tbase + 192 * buf + 64 * acc;
        const uint64_t oa    = (uint64_t)(2 * pa[p] * kTcM), ob = (uint64_t)(2 * pb[p] * NC);
        const uint32_t accum = (p == 0 || p == 8 || p == 12) ? 0u : 1u;  // the first MMA of D overwrites it
        tc::mma_tf32(d, ah0 + oa, bh0 + ob, idesc, accum);
        tc::mma_tf32(d, ah0 + oa, bl0 + ob, idesc, 1u);
        tc::mma_tf32(d, al0 + oa, bh0 + ob, idesc, 1u);
        tc::mma_tf32(d, al0 + oa, bl0 + ob, idesc, 1u);
    }
    tc::mma_commit(done + buf);
    return true;
}

// A worker warp's share of tile t: its rows (its TMEM lane quarter; warp w has quarter w & 3, and
// quarter 0 has 3 worker warps, 4, 8 and 12, the others 4) and up to 3 of the tile's 8-column units
// (u = wi, wi + nw, ...): its elements are loaded (lower triangle, the tile's own rows and columns;
// zero elsewhere) before the wait for the tile's MMAs, then Re, Im+ and Im- are read from TMEM and
// A + (-Re, Im+ - Im-) stored. False if the wait gave up.
constexpr int kTcUnits = 3;  // at most ceil(64 / 8 / 3) units per worker warp
struct TcShare {
    int qd, nw, wi;
    __device__ TcShare() {
        const int warp = threadIdx.x >> 5;
        qd = warp & 3;
        nw = qd ? 4 : 3;
        wi = (warp >> 2) - (qd ? 0 : 1);
    }
};
template <int NC>
__device__ __forceinline__ bool tc_readback(const TcTile& t, cx<float>* A, int ld, uint32_t tbase, uint64_t* done,
                                            volatile int* fail) {
    const TcShare  sh;
    const int      r   = t.rb + 32 * sh.qd + (threadIdx.x & 31);
    const bool     rok = r >= t.rlo && r < t.rhi;
    const uint32_t buf = t.seq & 1u;
    cx<float>      z[kTcUnits][8];  // the share's elements, in flight during the wait
#pragma unroll
    for (int k = 0; k < kTcUnits; ++k) {
        const int u = sh.wi + k * sh.nw;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = t.cb + 8 * u + j;
            z[k][j] = (u < NC / 8 && rok && c >= t.clo && c < t.chi && c <= r) ? ldc(A + (size_t)c * ld + r)
                                                                               : cx<float>{0.f, 0.f};
        }
    }
    bool ok = tc_wait(done + buf, (t.seq >> 1) & 1u, fail);
    ok      = __all_sync(0xffffffffu, ok);
    tc::fence_after_sync();
    if (ok) {
#pragma unroll
        for (int k = 0; k < kTcUnits; ++k) {
            const int u = sh.wi + k * sh.nw;
            if (u >= NC / 8) break;
            const uint32_t tl = tbase + 192 * buf + ((uint32_t)(32 * sh.qd) << 16) + 8 * u;
            float          dre[8], dip[8], dim[8];
            tc::tmem_ld8x3(tl, tl + 64, tl + 128, dre, dip, dim);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int c = t.cb + 8 * u + j;
                if (rok && c >= t.clo && c < t.chi && c <= r)
                    stc(A + (size_t)c * ld + r, cx<float>{z[k][j].x - dre[j], (r == c) ? 0.f : z[k][j].y + dip[j] - dim[j]});
            }
        }
    }
    tc::fence_before_sync();
    return ok;
}

// A22 -= V W^H + W V^H on the tensor cores, lower triangle of rows / columns q0..n-1. Row blocks of
// 128 and column blocks of NC are laid from the end (n rounded up to 8) towards q0; a block clamped
// at q0 (rounded down to 8) overlaps its neighbour and stores only the rows / columns that are its
// own. Warp-specialised: thread 0 issues each tile's MMAs as soon as the tile is staged; warps 1..15
// stage tile t into buffer t & 1 (the row operand when the row block changes, after draining the tile
// in flight), signal it on the staged mbarrier, then read back tile t - 1 while tile t's MMAs run.
// Every wait is bounded. seq: the kernel's running tile count (buffer and phase parity). Returns
// false if a wait gave up (the update is then incomplete).
template <int NC>
__device__ bool tc_trailing_update(cx<float>* A, int n, int ld, int q0, const cx<float>* Vp, const cx<float>* Wp,
                                   float* stage, uint32_t tbase, uint64_t* staged, uint64_t* done, uint32_t& seq,
                                   volatile int* fail) {
    float*         aH = stage;
    float*         aL = aH + (size_t)kTcM * kTcK;
    float*         bH0 = aL + (size_t)kTcM * kTcK;  // buffer b: hi at bH0 + b * 2 NC K, lo NC K after it
    const int      base8 = q0 & ~7, n8 = (n + 7) & ~7;
    const bool     issuer = threadIdx.x == 0, worker = threadIdx.x >= 32;
    bool           ok = true, pending = false;
    TcTile         prev{};
    for (int rhi = n, rbe = n8; rhi > q0;) {
        const int rb = max(rbe - kTcM, base8), rlo = max(rb, q0);
        bool      first = true;
        for (int chi = n, cbe = n8; chi > q0;) {
            const int cb = max(cbe - NC, base8), clo = max(cb, q0);
            if (clo < rhi) {  // the tile holds elements on or below the diagonal
                const TcTile t{rb, rlo, rhi, cb, clo, chi, seq++};
                if (worker) {
                    if (first) {
                        if (pending) {  // the row operand is about to change: drain the tile in flight
                            ok      = tc_readback<NC>(prev, A, ld, tbase, done, fail) && ok;
                            pending = false;
                        }
                        tc_stage<kTcM>(Vp, Wp, n, rb, aH, aL);
                    }
                    float* bh = bH0 + (size_t)(t.seq & 1u) * 2 * NC * kTcK;
                    tc_stage<NC>(Vp, Wp, n, cb, bh, bh + (size_t)NC * kTcK);
                    tc::fence_async_smem();
                    tc::fence_before_sync();
                    tc::mbar_arrive(staged + (t.seq & 1u));
                    if (pending) ok = tc_readback<NC>(prev, A, ld, tbase, done, fail) && ok;
                    prev    = t;
                    pending = true;
                } else if (issuer) {
                    ok = tc_issue<NC>(t, aH, aL, bH0, tbase, staged, done, fail) && ok;
                }
                first = false;
            }
            chi = clo;
            cbe = cb;
        }
        rhi = rlo;
        rbe = rb;
    }
    if (worker && pending) ok = tc_readback<NC>(prev, A, ld, tbase, done, fail) && ok;
    return __syncthreads_and(ok) != 0;
}

template <typename S>
__global__ void __launch_bounds__(kBlkNT, 1)
    k_tridiag_blocked(S* __restrict__ H, int n, int ld, size_t mstride, typename ST<S>::R* __restrict__ dOut,
                      typename ST<S>::R* __restrict__ eOut, S* __restrict__ tqOut, int* __restrict__ status, int batch,
                      int use_tc) {
    using R = typename ST<S>::R;
    extern __shared__ __align__(16) unsigned char smraw[];
    S* Vp   = reinterpret_cast<S*>(smraw);              // [k][r], NB x n
    S* Wp   = Vp + (size_t)kBlkNB * n;                  // [k][r], NB x n
    S* yp   = Wp + (size_t)kBlkNB * n;                  // [warp][r], NW x n
    S* v    = yp + (size_t)kBlkNW * n;                  // n + 32 (zero padded past n)
    S* tdot = v + (n + 32);                             // t1 (W^H v) then t2 (V^H v), NB each
    R* red  = reinterpret_cast<R*>(tdot + 2 * kBlkNB);  // 4 x NW
    __shared__ S s_c0;
    __shared__ uint64_t s_staged[2];  // tensor-core update: tile staged (worker warps -> issuer), per buffer
    __shared__ uint64_t s_done[2];    // its MMAs complete (tcgen05.commit -> worker warps), per buffer
    __shared__ uint32_t s_tmem;       // TMEM base address
    __shared__ int      s_tcfail;     // a tensor-core wait gave up
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // With an even order every column starts at an even element, so row pairs from an even row are
    // 16-byte (8-byte for real) aligned: the product's tiles then start at o rounded down to even.
    const bool vec = (n & 1) == 0 && (mstride & 1) == 0 && (ld & 1) == 0;
    // the tensor-core update (complex only; use_tc = its column-block width, 0 off): TMEM for its
    // accumulators, an mbarrier per buffer for its MMAs
    constexpr bool TC = ST<S>::cplx;
    bool           tc_on = TC && use_tc != 0;
    uint32_t       tc_seq = 0, tbase = 0;  // tiles so far (buffer and mbarrier phase parity)
    if constexpr (TC) {
        if (tc_on) {
            if (tid == 0) {
                s_tcfail = 0;
                tc::mbar_init(&s_staged[0], kBlkNT - 32);
                tc::mbar_init(&s_staged[1], kBlkNT - 32);
                tc::mbar_init(&s_done[0], 1);
                tc::mbar_init(&s_done[1], 1);
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            }
            if (warp == 0) {
                tc::tmem_alloc(&s_tmem, kTcCols);
                tc::tmem_relinquish();
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            tbase = s_tmem;
        }
    }

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
            bool      simt = mt > 0;
            if constexpr (TC) {
                if (tc_on && mt >= kTcMinRows) {
                    simt = false;
                    float* stage = reinterpret_cast<float*>(yp);
                    const bool ok =
                        use_tc == 64   ? tc_trailing_update<64>(A, n, ld, q0, Vp, Wp, stage, tbase, s_staged, s_done, tc_seq, &s_tcfail)
                        : use_tc == 48 ? tc_trailing_update<48>(A, n, ld, q0, Vp, Wp, stage, tbase, s_staged, s_done, tc_seq, &s_tcfail)
                                       : tc_trailing_update<32>(A, n, ld, q0, Vp, Wp, stage, tbase, s_staged, s_done, tc_seq, &s_tcfail);
                    if (!ok) {
                        // a wait gave up: this matrix is incomplete, and the CTA keeps to the SIMT update
                        if (tid == 0 && status) atomicOr(status + b, 1);  // UEPM_K_NOCONVERGE
                        tc_on = false;
                    }
                    for (int q = n + tid; q < n + 32; q += kBlkNT) v[q] = ST<S>::zero();  // staging overlaid it
                }
            }
            if (simt) {
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
    if constexpr (TC) {
        if (use_tc) {
            if (!tc_on && tid == 0 && tc_seq > 0) {  // a wait gave up: the last tiles' MMAs get one more bounded wait
                tc_wait(&s_done[(tc_seq - 1) & 1u], ((tc_seq - 1) >> 1) & 1u);
                if (tc_seq > 1) tc_wait(&s_done[tc_seq & 1u], ((tc_seq - 2) >> 1) & 1u);
            }
            tc::fence_before_sync();
            __syncthreads();
            if (warp == 0) {
                tc::fence_after_sync();
                tc::tmem_dealloc(tbase, kTcCols);
            }
        }
    }
}

}  // namespace

int tridiag_blocked_max_n() { return kBlkNT; }

template <typename S>
bool launch_tridiag_blocked(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                            int* status, int batch, cudaStream_t s, bool tensor_cores) {
    if (n < 2 || n > kBlkNT) return false;
    // the tensor-core update with the widest column block whose staging fits
    int nc = 0;
    if (tensor_cores && ST<S>::cplx)
        for (int w : {64, 48, 32})
            if (!nc && BlkSmem<S>::bytes_tc(n, w) <= 227 * 1024) nc = w;
    const size_t smem = nc ? BlkSmem<S>::bytes_tc(n, nc) : BlkSmem<S>::bytes(n);
    if (smem > 227 * 1024) return false;
    auto kern = k_tridiag_blocked<S>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
    int dev = 0, sms = 0, fit = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, kBlkNT, smem) != cudaSuccess || fit < 1) fit = 1;
    const int grid = std::min(batch, std::max(1, sms) * fit);
    kern<<<grid, kBlkNT, smem, s>>>(H, n, ld, mstride, d, e, tq, status, batch, nc);
    count_launch();
    return true;
}

template bool launch_tridiag_blocked<float>(float*, int, int, size_t, float*, float*, float*, int*, int, cudaStream_t,
                                           bool);
template bool launch_tridiag_blocked<cx<float>>(cx<float>*, int, int, size_t, float*, float*, cx<float>*, int*, int,
                                                cudaStream_t, bool);

}  // namespace uepm
