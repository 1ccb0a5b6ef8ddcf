// tridiag_reg.cu -- register-resident Householder reduction of real symmetric FP32 matrices
// (n <= 176) to tridiagonal form, one CTA of 256 threads per matrix. Same algorithm and the same
// outputs as k_tridiag (tridiag.cu): d, e, tau per step and the reflector tails v[i+2:] in column i of
// H, so the bisection, inverse iteration and back-transformation kernels are shared. It replaces the
// shared-memory-resident FP32 reduction of the mixed path where the matrix fits the register file
// (the first half of Eigen's SelfAdjointEigenSolver behind Hamiltonian::Diagonalize,
// src/EPP/Hamiltonian.cpp:125-134).
//
// Layout. The 256 threads form a 16 x 16 grid; thread (r, c) owns A[r + 16t][c + 16u] for
// t, u < K = ceil(n / 16) in registers (2-D cyclic distribution: the trailing matrix of every step
// stays spread over all threads). Shared memory holds only the current column (double-buffered) and
// the product vector y, so each step is
//   (a) every thread computes the Householder scalars of column j from the shared column and the
//       norm partials published with it (identical arithmetic everywhere, no barrier); warp 0
//       writes d, e, tau and the reflector tail;
//   (b) p = A v: K x K FMAs per thread, a 16-lane butterfly per row, y and the warp partials of
//       v^T p to shared memory;                                             -- barrier
//   (c) w = tau p - (tau^2 / 2)(v^T p) v, A -= v w^T + w v^T on the registers; the owners of column
//       j + 1 publish it, with the partial sums of squares of its tail.     -- barrier
// (Working with the unnormalised reflector x - beta e_{j+1} and tau' = 1 / (beta (beta - alpha))
// saves the scaling of v but measured slower and less accurate on the 2000-point Si path.)
// Rows and columns that are already reduced (index <= j) are skipped at compile time: the steps are
// run in blocks of 16 with the first live local index S0 = floor((j + 1) / 16) as a template
// parameter, so the unrolled loops start at S0 and no register array is indexed at run time.
#include <algorithm>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {
namespace {

constexpr int kGrid = 16;               // thread grid kGrid x kGrid
constexpr int kThreads = kGrid * kGrid;  // 256
constexpr int kWarps = kThreads / 32;

template <int K>
struct RegShared {
    float               col[2][kGrid * K];  // column j (buffer j & 1), zero beyond n
    __align__(16) float nrm[2][kGrid];      // per-row-group partial sums of squares of col[j+2:]
    float               y[kGrid * K];       // p = A v of the current step, zero for rows <= j
    __align__(16) float red[kWarps];        // per-warp partials of v^T p
};

// Sum of 16 shared partials in a fixed order (identical in every thread).
__device__ __forceinline__ float sum16(const float* p) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    const float4 c = reinterpret_cast<const float4*>(p)[2], d = reinterpret_cast<const float4*>(p)[3];
    return (((a.x + a.y) + (a.z + a.w)) + ((b.x + b.y) + (b.z + b.w))) +
           (((c.x + c.y) + (c.z + c.w)) + ((d.x + d.y) + (d.z + d.w)));
}

// Householder vector element i of step j: v[j+1] = 1, v[i] = col[i] * sc below, 0 above.
__device__ __forceinline__ float house_v(const float* col, int i, int j, float sc) {
    return i > j + 1 ? col[i] * sc : (i == j + 1 ? 1.f : 0.f);
}

template <int K, int S0>
__device__ __forceinline__ void reduce_block(float (&a)[K][K], RegShared<K>& sh, float* __restrict__ Ag, int n, int ld,
                                             float* __restrict__ dOut, float* __restrict__ eOut,
                                             float* __restrict__ tqOut, bool& bad) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r = tid >> 4, c = tid & 15;
    const int jlo = max(kGrid * S0 - 1, 0), jhi = min(kGrid * S0 + kGrid - 2, n - 2);
    for (int j = jlo; j <= jhi; ++j) {
        const float* col = sh.col[j & 1];
        // ---- (a) Householder scalars of column j (every thread, same order of operations) ------
        // The column's owners published the partial sums of squares of its tail with it. The
        // divisions stay correctly rounded: with the approximate forms the biased tau of 136
        // successive reflectors lost enough orthogonality to move the refined eigenvalues of the
        // 2000-point Si path by 1e-5 eV.
        const float tail2 = sum16(sh.nrm[j & 1]);
        const float alpha = col[j + 1];
        float       beta = alpha, tau = 0.f, sc = 0.f;
        if (tail2 > num<float>::tiny()) {
            beta = sqrtf(fmaf(alpha, alpha, tail2));
            if (alpha >= 0.f) beta = -beta;
            tau = (beta - alpha) / beta;
            sc  = 1.f / (alpha - beta);
        }
        if (warp == 0) {
            float* cg = Ag + (size_t)j * ld;
            for (int i = j + 2 + lane; i < n; i += 32) cg[i] = col[i] * sc;
            if (lane == 0) {
                const float dj = col[j];
                dOut[j]   = dj;
                eOut[j]   = beta;
                tqOut[j]  = tau;
                cg[j + 1] = beta;
                if (!isfinite(beta) || !isfinite(dj)) bad = true;
            }
        }
        if (tau != 0.f) {  // uniform over the CTA
            float vc[K];
#pragma unroll
            for (int u = S0; u < K; ++u) vc[u] = house_v(col, c + kGrid * u, j, sc);
            // ---- (b) p = A v, reduced over the 16 column owners of each row ---------------------
            float p[K];
#pragma unroll
            for (int t = S0; t < K; ++t) {
                float s = 0.f;
#pragma unroll
                for (int u = S0; u < K; ++u) s = fmaf(a[t][u], vc[u], s);
                p[t] = s;
            }
#pragma unroll
            for (int off = 1; off < kGrid; off <<= 1) {
#pragma unroll
                for (int t = S0; t < K; ++t) p[t] += __shfl_xor_sync(0xffffffffu, p[t], off);
            }
            // every lane of the half-warp now holds p for rows r + 16t: v^T p over them (v is zero on
            // the reduced rows), both halves combined; lane c publishes row r + 16c
            float vtp = 0.f, mine = 0.f;
#pragma unroll
            for (int t = S0; t < K; ++t) {
                vtp = fmaf(house_v(col, r + kGrid * t, j, sc), p[t], vtp);
                if (c == t) mine = p[t];
            }
            vtp += __shfl_xor_sync(0xffffffffu, vtp, kGrid);
            const int im = r + kGrid * c;
            if (lane == 0) sh.red[warp] = vtp;
            if (c >= S0 && c < K) sh.y[im] = im > j ? mine : 0.f;
        }
        __syncthreads();
        if (tau != 0.f) {
            // ---- (c) rank-2 update on the registers ---------------------------------------------
            const float4 r0 = reinterpret_cast<const float4*>(sh.red)[0], r1 = reinterpret_cast<const float4*>(sh.red)[1];
            const float  vtp = ((r0.x + r0.y) + (r0.z + r0.w)) + ((r1.x + r1.y) + (r1.z + r1.w));
            const float  al  = -0.5f * tau * tau * vtp;
            float       vc[K], wc[K];
#pragma unroll
            for (int u = S0; u < K; ++u) {
                const int i = c + kGrid * u;
                vc[u]       = house_v(col, i, j, sc);
                wc[u]       = fmaf(tau, sh.y[i], al * vc[u]);
            }
#pragma unroll
            for (int t = S0; t < K; ++t) {
                const int   i  = r + kGrid * t;
                const float vr = house_v(col, i, j, sc);
                const float wr = fmaf(tau, sh.y[i], al * vr);
#pragma unroll
                for (int u = S0; u < K; ++u) a[t][u] = fmaf(-vr, wc[u], fmaf(-wr, vc[u], a[t][u]));
            }
        }
        // column j + 1 (local column S0 of the owners) for the next step, with the partial sums of
        // squares of its tail (rows >= j + 3)
        if (c == ((j + 1) & (kGrid - 1))) {
            float* nxt = sh.col[(j + 1) & 1];
            float  ss  = 0.f;
#pragma unroll
            for (int t = S0; t < K; ++t) {
                const float x = a[t][S0];
                nxt[r + kGrid * t] = x;
                if (r + kGrid * t >= j + 3) ss = fmaf(x, x, ss);
            }
            sh.nrm[(j + 1) & 1][r] = ss;
        }
        __syncthreads();
    }
    if constexpr (S0 + 1 < K) reduce_block<K, S0 + 1>(a, sh, Ag, n, ld, dOut, eOut, tqOut, bad);
}

template <int K>
__global__ void __launch_bounds__(kThreads, K <= 9 ? 2 : 1)
    k_tridiag_reg(float* __restrict__ H, int n, int ld, size_t mstride, float* __restrict__ dOut,
                  float* __restrict__ eOut, float* __restrict__ tqOut, int* __restrict__ status, int batch) {
    __shared__ RegShared<K> sh;
    const int tid = threadIdx.x, r = tid >> 4, c = tid & 15;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        float* Ag = H + (size_t)b * mstride;
        float  a[K][K];
        // a[t][u] = A[r+16t][c+16u], read as the (c+16u, r+16t) element of the column-major,
        // exactly symmetric matrix so that consecutive lanes read consecutive addresses
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int i = r + kGrid * t;
#pragma unroll
            for (int u = 0; u < K; ++u) {
                const int jj = c + kGrid * u;
                a[t][u]      = (i < n && jj < n) ? Ag[(size_t)i * ld + jj] : 0.f;
            }
        }
        for (int i = tid; i < kGrid * K; i += kThreads) {
            sh.col[0][i] = i < n ? Ag[i] : 0.f;
            sh.col[1][i] = 0.f;
        }
        if (c == 0) {  // owners of column 0: partial sums of squares of its tail (rows >= 2)
            float ss = 0.f;
#pragma unroll
            for (int t = 0; t < K; ++t)
                if (r + kGrid * t >= 2) ss = fmaf(a[t][0], a[t][0], ss);
            sh.nrm[0][r] = ss;
        }
        __syncthreads();
        bool bad = false;
        reduce_block<K, 0>(a, sh, Ag, n, ld, dOut + (size_t)b * n, eOut + (size_t)b * n, tqOut + (size_t)b * n, bad);
        if (tid == 0) {
            const float dl = sh.col[(n - 1) & 1][n - 1];
            dOut[(size_t)b * n + n - 1]  = dl;
            eOut[(size_t)b * n + n - 1]  = 0.f;
            tqOut[(size_t)b * n + n - 1] = 0.f;
            if (!isfinite(dl)) bad = true;
            if (bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
        }
        __syncthreads();  // shared memory is reused by the CTA's next matrix
    }
}

template <int K>
void launch_k(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
              cudaStream_t s) {
    static int grid_cap = 0;
    if (!grid_cap) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag_reg<K>, kThreads, 0);
        grid_cap = std::max(1, sms) * std::max(1, per_sm);
    }
    k_tridiag_reg<K><<<std::min(batch, grid_cap), kThreads, 0, s>>>(H, n, ld, mstride, d, e, tq, status, batch);
    count_launch();
}

}  // namespace

int tridiag_reg_max_n() { return kGrid * 11; }

void launch_tridiag_reg(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
                        cudaStream_t s) {
    switch ((n + kGrid - 1) / kGrid) {
        case 1: case 2: case 3: case 4: case 5:
        case 6: launch_k<6>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
        case 7: launch_k<7>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
        case 8: launch_k<8>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
        case 9: launch_k<9>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
        case 10: launch_k<10>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
        default: launch_k<11>(H, n, ld, mstride, d, e, tq, status, batch, s); break;
    }
}

}  // namespace uepm
