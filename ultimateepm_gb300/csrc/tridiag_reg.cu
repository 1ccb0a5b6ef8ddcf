// tridiag_reg.cu -- register-resident Householder reduction of real symmetric FP32 matrices
// (n <= 176) to tridiagonal form, one CTA of 256 threads per matrix. Same algorithm and the same
// outputs as k_tridiag (tridiag.cu): d, e, tau per step and the reflector tails v[i+2:] in column i of
// H, so the bisection, inverse iteration and back-transformation kernels are shared. It replaces the
// shared-memory-resident FP32 reduction of the mixed path where the matrix fits the register file
// (the first half of Eigen's SelfAdjointEigenSolver behind Hamiltonian::Diagonalize,
// src/EPP/Hamiltonian.cpp:125-134).
//
// Layout. The 256 threads form a 16 x 16 grid, thread (r, c) = (tid % 16, tid / 16), and own
// A[r + 16t][c + 16u] for t, u < K = ceil(n / 16) in registers (2-D cyclic distribution: the
// trailing matrix of every step stays spread over all threads). Rows are the fast index, so the 16
// owners of a column are one half-warp, and the 16 threads that share a column group reduce over
// rows within their half-warp. Shared memory holds the reflector v (double-buffered by step
// parity) and y = tau A v, both transposed ([q][t] = element q + 16t, so a thread's rows or
// columns are contiguous float4s), and a per-half-warp buffer for the column sums. Step j:
//   (a) product: y = tau A v as column sums (A is symmetric): each thread sums its rows for each of
//       its columns, the 16 partials of a column meet in the half-warp's buffer and lane u adds
//       those of column c + 16u; the warps' partials of v^T y go to shared memory.  -- barrier
//   (b) w = y - (tau/2)(v^T y) v and A -= v w^T + w v^T on the registers; the half-warp that owns
//       column j + 1 then forms its reflector (norm by shuffles, the Householder scalars, v scaled)
//       and publishes v, tau, d, e and the reflector tail.                         -- barrier
// Rows and columns that are already reduced (index <= j) are skipped at compile time: the steps run
// in blocks of 16 with the first live local index S0 = floor((j + 1) / 16) as a template parameter,
// so the unrolled loops start at S0 and no register array is indexed at run time.
#include <algorithm>

#include "uepm_common.cuh"
#include "uepm_kernels.h"

namespace uepm {
namespace {

constexpr int kGrid    = 16;              // thread grid kGrid x kGrid
constexpr int kThreads = kGrid * kGrid;   // 256
constexpr int kWarps   = kThreads / 32;
constexpr int kKP      = 12;              // row length of the transposed vectors (K <= 11; 48 B rows
                                          // keep 8 consecutive float4 rows on distinct banks)
constexpr int kPP      = 20;              // row pitch of the column-sum buffer (conflict-free float4 rows)
constexpr int kPartW   = kGrid * kPP + 16;  // per half-warp (the +16 puts the two halves of a warp on
                                            // different banks)

struct RegShared {
    __align__(16) float v[2][kGrid][kKP];  // v[b][q][t] = v_{q + 16t} of the step with parity b
    __align__(16) float y[kGrid][kKP];     // y[q][t] = (tau A v)_{q + 16t}, zero at reduced indices
    __align__(16) float part[kGrid][kPartW];  // [c][u * kPP + r]: row group r's sum for column c + 16u
    __align__(16) float red[kWarps];       // per-warp partials of v^T y
    float               tau[2];
};

// Loads row q, entries [S0, K), of a transposed vector (compile-time chunks of four).
template <int K, int S0>
__device__ __forceinline__ void load_row(const float (&src)[kKP], float (&dst)[K]) {
#pragma unroll
    for (int t4 = S0 / 4; t4 <= (K - 1) / 4; ++t4) {
        const float4 q = *reinterpret_cast<const float4*>(&src[4 * t4]);
        if (4 * t4 + 0 >= S0 && 4 * t4 + 0 < K) dst[4 * t4 + 0] = q.x;
        if (4 * t4 + 1 >= S0 && 4 * t4 + 1 < K) dst[4 * t4 + 1] = q.y;
        if (4 * t4 + 2 >= S0 && 4 * t4 + 2 < K) dst[4 * t4 + 2] = q.z;
        if (4 * t4 + 3 >= S0 && 4 * t4 + 3 < K) dst[4 * t4 + 3] = q.w;
    }
}

// The reflector of column jn (local column S0 of the half-warp c = jn % 16), from its registers:
// alpha = A[jn+1][jn], the tail A[jn+2:][jn]; v = (1, tail / (alpha - beta)) from row jn + 1 on.
// Runs in the whole warp that holds the owners (the shuffles use all 32 lanes; the other half-warp
// computes on its own column and stores nothing). For jn = n - 1 only d is written.
template <int K, int S0>
__device__ __forceinline__ void house_next(const float (&a)[K][K], RegShared& sh, int jn, int n, int r, int c,
                                           float* __restrict__ Ag, int ld, float* __restrict__ dOut,
                                           float* __restrict__ eOut, float* __restrict__ tqOut, bool& bad) {
    const bool own = c == (jn & (kGrid - 1));
    float      ss = 0.f, al = 0.f, dj = 0.f;
#pragma unroll
    for (int t = S0; t < K; ++t) {
        const int   row = r + kGrid * t;
        const float x   = a[t][S0];
        if (row >= jn + 2) ss = fmaf(x, x, ss);
        if (row == jn + 1) al = x;
        if (row == jn) dj = x;
    }
    if (own && r == (jn & (kGrid - 1))) {
        dOut[jn] = dj;
        if (!isfinite(dj)) bad = true;
    }
    if (jn >= n - 1) {
        if (own && r == 0) {
            eOut[jn]  = 0.f;
            tqOut[jn] = 0.f;
        }
        return;
    }
#pragma unroll
    for (int o = 1; o < kGrid; o <<= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const float alpha = __shfl_sync(0xffffffffu, al, (jn + 1) & (kGrid - 1), kGrid);
    // The divisions stay correctly rounded: with the approximate forms the biased tau of 136
    // successive reflectors lost enough orthogonality to move the refined eigenvalues of the
    // 2000-point Si path by 1e-5 eV.
    float beta = alpha, tau = 0.f, sc = 0.f;
    if (ss > num<float>::tiny()) {
        beta = sqrtf(fmaf(alpha, alpha, ss));
        if (alpha >= 0.f) beta = -beta;
        tau = (beta - alpha) / beta;
        sc  = 1.f / (alpha - beta);
    }
    if (!own) return;
    float* vq = sh.v[jn & 1][r];
    float* cg = Ag + (size_t)jn * ld;
#pragma unroll
    for (int t = S0; t < K; ++t) {
        const int   row = r + kGrid * t;
        const float x   = a[t][S0] * sc;
        vq[t]           = row > jn + 1 ? x : (row == jn + 1 ? 1.f : 0.f);
        if (row > jn + 1 && row < n) cg[row] = x;
    }
    if (r == ((jn + 1) & (kGrid - 1))) cg[jn + 1] = beta;
    if (r == 0) {
        eOut[jn]        = beta;
        tqOut[jn]       = tau;
        sh.tau[jn & 1]  = tau;
        if (!isfinite(beta)) bad = true;
    }
}

template <int K, int S0>
__device__ __forceinline__ void reduce_block(float (&a)[K][K], RegShared& sh, float* __restrict__ Ag, int n, int ld,
                                             float* __restrict__ dOut, float* __restrict__ eOut,
                                             float* __restrict__ tqOut, bool& bad) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r = tid & (kGrid - 1), c = tid >> 4;
    const int jlo = max(kGrid * S0 - 1, 0), jhi = min(kGrid * S0 + kGrid - 2, n - 2);
    for (int j = jlo; j <= jhi; ++j) {
        const int   b   = j & 1;
        const float tau = sh.tau[b];
        if (tau != 0.f) {  // uniform over the CTA
            // ---- (a) column sums of A v over this thread's rows -----------------------------------
            float vr[K], q[K];
            load_row<K, S0>(sh.v[b][r], vr);
#pragma unroll
            for (int u = S0; u < K; ++u) {
                float s = 0.f;
#pragma unroll
                for (int t = S0; t < K; ++t) s = fmaf(a[t][u], vr[t], s);
                q[u] = s;
            }
            // sum over the 16 row groups of the half-warp: lane u ends with column c + 16u
            float ysum = 0.f;
            if constexpr (K - S0 <= 3) {
#pragma unroll
                for (int o = 1; o < kGrid; o <<= 1) {
#pragma unroll
                    for (int u = S0; u < K; ++u) q[u] += __shfl_xor_sync(0xffffffffu, q[u], o);
                }
#pragma unroll
                for (int u = S0; u < K; ++u)
                    if (r == u) ysum = q[u];
            } else {
                float* pc = sh.part[c];
#pragma unroll
                for (int u = S0; u < K; ++u) pc[u * kPP + r] = q[u];
                __syncwarp();
                if (r >= S0 && r < K) {
                    const float4* pr = reinterpret_cast<const float4*>(pc + r * kPP);
                    const float4  p0 = pr[0], p1 = pr[1], p2 = pr[2], p3 = pr[3];
                    ysum = (((p0.x + p0.y) + (p0.z + p0.w)) + ((p1.x + p1.y) + (p1.z + p1.w))) +
                           (((p2.x + p2.y) + (p2.z + p2.w)) + ((p3.x + p3.y) + (p3.z + p3.w)));
                }
            }
            float vty = 0.f;
            if (r >= S0 && r < K) {
                const int   i  = c + kGrid * r;
                const float yv = i > j ? tau * ysum : 0.f;
                sh.y[c][r]     = yv;
                vty            = sh.v[b][c][r] * yv;
            }
            vty = warp_sum(vty);
            if (lane == 0) sh.red[warp] = vty;
        }
        __syncthreads();
        if (tau != 0.f) {
            // ---- (b) rank-2 update on the registers ---------------------------------------------
            const float4 r0 = reinterpret_cast<const float4*>(sh.red)[0], r1 = reinterpret_cast<const float4*>(sh.red)[1];
            const float  vty = ((r0.x + r0.y) + (r0.z + r0.w)) + ((r1.x + r1.y) + (r1.z + r1.w));
            const float  al  = -0.5f * tau * vty;
            float        vc[K], wc[K], vr[K], wr[K];
            load_row<K, S0>(sh.v[b][c], vc);
            load_row<K, S0>(sh.y[c], wc);
            load_row<K, S0>(sh.v[b][r], vr);
            load_row<K, S0>(sh.y[r], wr);
#pragma unroll
            for (int u = S0; u < K; ++u) wc[u] = fmaf(al, vc[u], wc[u]);
#pragma unroll
            for (int t = S0; t < K; ++t) {
                const float w = fmaf(al, vr[t], wr[t]);
#pragma unroll
                for (int u = S0; u < K; ++u) a[t][u] = fmaf(-vr[t], wc[u], fmaf(-w, vc[u], a[t][u]));
            }
        }
        // ---- the reflector of column j + 1 (local column S0 of its owners) ----------------------
        if (warp == (((j + 1) & (kGrid - 1)) >> 1)) house_next<K, S0>(a, sh, j + 1, n, r, c, Ag, ld, dOut, eOut, tqOut, bad);
        __syncthreads();
    }
    if constexpr (S0 + 1 < K) {
        if (kGrid * (S0 + 1) - 1 <= n - 2) reduce_block<K, S0 + 1>(a, sh, Ag, n, ld, dOut, eOut, tqOut, bad);
    }
}

// LOCAL: the matrix is not read from H but formed from the k-independent local potential: off the
// diagonal its FP32 rounding V32 ([N][N] column-major), on it the FP64 V (complex storage of a real
// matrix) plus the rows table's kinetic term, rounded once, exactly as the assembly's FP32 copy is;
// H then only receives the reflector tails. V32 (75 KB at N = 137) stays in L2 across the batch.
template <int K, bool LOCAL>
__global__ void __launch_bounds__(kThreads, K <= 9 ? 2 : 1)
    k_tridiag_reg(float* __restrict__ H, int n, int ld, size_t mstride, float* __restrict__ dOut,
                  float* __restrict__ eOut, float* __restrict__ tqOut, int* __restrict__ status, int batch,
                  const float* __restrict__ V32, const double* __restrict__ Vre, const double* __restrict__ rows) {
    __shared__ RegShared sh;
    const int tid = threadIdx.x, r = tid & (kGrid - 1), c = tid >> 4;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        float* Ag = H + (size_t)b * mstride;
        float  a[K][K];
        // a[t][u] = A[r+16t][c+16u] (column-major: consecutive lanes read consecutive rows)
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int i = r + kGrid * t;
#pragma unroll
            for (int u = 0; u < K; ++u) {
                const int jj = c + kGrid * u;
                if constexpr (LOCAL) {
                    float x = 0.f;
                    if (i < n && jj < n) {
                        if (i == jj)  // Re V[i][i] + kinetic, rounded once
                            x = __double2float_rn(Vre[2 * ((size_t)i * n + i)] +
                                                  rows[((size_t)b * n + i) * ROW_STRIDE + RF_KIN]);
                        else
                            x = V32[(size_t)jj * n + i];
                    }
                    a[t][u] = x;
                } else {
                    a[t][u] = (i < n && jj < n) ? Ag[(size_t)jj * ld + i] : 0.f;
                }
            }
        }
        bool   bad = false;
        float* dB  = dOut + (size_t)b * n;
        float* eB  = eOut + (size_t)b * n;
        float* tB  = tqOut + (size_t)b * n;
        if (tid < 32) house_next<K, 0>(a, sh, 0, n, r, c, Ag, ld, dB, eB, tB, bad);  // column 0: warp 0
        __syncthreads();
        if (n >= 2) reduce_block<K, 0>(a, sh, Ag, n, ld, dB, eB, tB, bad);
        bad = __syncthreads_or(bad);
        if (tid == 0 && bad && status) atomicOr(status + b, 2);  // UEPM_K_NONFINITE
    }
}

template <int K, bool LOCAL>
void launch_k(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
              cudaStream_t s, const float* V32, const double* Vre, const double* rows) {
    static int grid_cap = 0;
    if (!grid_cap) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag_reg<K, LOCAL>, kThreads, 0);
        grid_cap = std::max(1, sms) * std::max(1, per_sm);
    }
    k_tridiag_reg<K, LOCAL>
        <<<std::min(batch, grid_cap), kThreads, 0, s>>>(H, n, ld, mstride, d, e, tq, status, batch, V32, Vre, rows);
    count_launch();
}

template <bool LOCAL>
void launch_reg(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
                cudaStream_t s, const float* V32, const double* Vre, const double* rows) {
    switch ((n + kGrid - 1) / kGrid) {
        case 1: case 2: case 3: case 4: case 5:
        case 6: launch_k<6, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
        case 7: launch_k<7, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
        case 8: launch_k<8, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
        case 9: launch_k<9, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
        case 10: launch_k<10, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
        default: launch_k<11, LOCAL>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, Vre, rows); break;
    }
}

}  // namespace

int tridiag_reg_max_n() { return kGrid * 11; }

void launch_tridiag_reg(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
                        cudaStream_t s) {
    launch_reg<false>(H, n, ld, mstride, d, e, tq, status, batch, s, nullptr, nullptr, nullptr);
}

void launch_tridiag_reg_local(const float* V32, const cx<double>* Vloc, const double* rows, float* H, int n, int ld,
                              size_t mstride, float* d, float* e, float* tq, int* status, int batch, cudaStream_t s) {
    launch_reg<true>(H, n, ld, mstride, d, e, tq, status, batch, s, V32, reinterpret_cast<const double*>(Vloc), rows);
}

}  // namespace uepm
