// uepm_kernels.h -- host-side launch wrappers of the device kernels (one declaration per kernel).
// Scalar type S is double / float (real symmetric H) or cx<double> / cx<float> (complex Hermitian H).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "uepm_common.cuh"

namespace uepm {

void count_launch(int n = 1);

// assemble.cu: H(k) in FULL column-major storage (both triangles). SO = double (real H) or
// cx<double>; H32 (optional) receives the FP32 copy for the mixed path (float or cx<float>).
void launch_rows(const DevParams& P, const double* d_k, const int* d_G, double* d_rows, int batch, cudaStream_t s,
                 float2* d_rows32 = nullptr);
// Mixed path, no spin-orbit, square nonlocal wells: the assembly in double-single arithmetic on the
// FP32 pipe (SO = ds2 or ds4), from the k-independent tables in FP32 pairs and d_rows32 (written by
// launch_rows when given).
// The same with spin-orbit coupling (SO = ds4): the scalar part and the spin-orbit blocks in
// double-single, the FP64 element where the nonlocal part needs it.
template <typename SO>
void launch_assemble_soc_ds(const DevParams& P, const DevParamsDS& Q, const float4* Vloc32, const float4* phNL32,
                            const float4* phSO32, const float2* rows32, const cx<double>* Vloc, const double2* phNL,
                            const double2* phSO, const double* rows, SO* H, int ld, size_t mstride,
                            typename Lower<SO>::type* H32, size_t mstride32, int batch, cudaStream_t s);
template <typename SO>
void launch_assemble_ds(const DevParams& P, const DevParamsDS& Q, const float4* Vloc32, const float4* phNL32,
                        const float2* rows32, const cx<double>* Vloc, const double2* phNL, const double* rows, SO* H,
                        int ld, size_t mstride, typename Lower<SO>::type* H32, size_t mstride32, int batch,
                        cudaStream_t s);
template <typename SO>
void launch_assemble(const DevParams& P, const cx<double>* Vloc, const double2* phNL, const double2* phSO, const double* rows,
                     SO* H, int ld, size_t mstride, typename Lower<SO>::type* H32, size_t mstride32, int batch,
                     cudaStream_t s);

// tridiag.cu: Householder reduction in place. d, e: [batch][n]; tq: [batch][n] reflector scalars;
// status: [batch] (ORed with UEPM_K_NONFINITE on NaN/Inf).
// variant: 0 automatic, 1 register-resident (FP32 real, n <= tridiag_reg_max_n()), 2 one CTA per
// matrix (shared memory where the matrix fits, else global memory with a persistent grid), 3 one
// thread-block cluster per matrix (tridiag_cluster.cu), 4 one CTA per matrix in global memory with
// each step's update fused into the next step's product (FP32, n <= 512), 5 the same with every
// other update deferred to the next pass, 6 blocked (panels of 16 columns, lower triangle only, one
// matrix per SM, tridiag_blocked.cu; FP32, n <= 512). Automatic: 1 where it applies, 6 for FP32
// complex orders 200..512 and real orders 300..512, 5 for the other FP32 matrices, else 2.
// ctas_per_sm (0: automatic) caps the persistent grid of the global-memory kernels; cluster (0:
// automatic) is the cluster size of variant 3.
template <typename S>
void launch_tridiag(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq, int* status,
                    int batch, cudaStream_t s, int variant = 0, int ctas_per_sm = 0, int cluster = 0,
                    bool tensor_cores = true);
// tridiag_cluster.cu: cluster size for order n (want = 0: automatic; 0 returned when it cannot fit)
// and the launch (false when the cluster kernel cannot run this case).
template <typename S>
int tridiag_cluster_size(int n, int want);
template <typename S>
bool launch_tridiag_cluster(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                            int* status, int batch, cudaStream_t s, int want_c);
// tridiag_blocked.cu: the blocked reduction (false when it cannot run this order); tensor_cores puts
// the complex trailing updates on tcgen05 (where the operand staging fits shared memory).
int tridiag_blocked_max_n();
template <typename S>
bool launch_tridiag_blocked(S* H, int n, int ld, size_t mstride, typename ST<S>::R* d, typename ST<S>::R* e, S* tq,
                            int* status, int batch, cudaStream_t s, bool tensor_cores);
// tridiag_reg.cu: the same reduction for real FP32 matrices with n <= tridiag_reg_max_n(), held in
// registers (launch_tridiag<float> dispatches to it).
int  tridiag_reg_max_n();
void launch_tridiag_reg(float* H, int n, int ld, size_t mstride, float* d, float* e, float* tq, int* status, int batch,
                        cudaStream_t s);
// The same for real local-potential matrices formed in the kernel from the k-independent local V
// ([N][N], N = n: its FP32 rounding V32 off the diagonal, FP64 Vloc plus the rows table's kinetic term
// on it), bit-identical to reducing the assembly's FP32 copy; H receives only the reflector tails.
void launch_tridiag_reg_local(const float* V32, const cx<double>* Vloc, const double* rows, float* H, int n, int ld,
                              size_t mstride, float* d, float* e, float* tq, int* status, int batch, cudaStream_t s);

// tridiag_eig.cu
template <typename T>
void launch_bisect(const T* d, const T* e, int n, int nb, T* ev, int ev_ld, int batch, cudaStream_t s, int cap = 0,
                   int* status = nullptr);
template <typename T>
void launch_invit(const T* d, const T* e, const T* ev, int ev_ld, int n, int nb, T* work, T* z, int* status, int batch,
                  cudaStream_t s, int cap = 0);
// Inverse-iteration workspace per matrix (used where the arrays exceed shared memory): U0, U1, the
// multipliers and Z, each n x 32 interleaved by lane, and the row-interchange bits.
template <typename T>
__host__ __device__ inline size_t invit_work_elems(int n) {
    return (size_t)5 * n * 32;
}

// backtransform.cu: X = Q Z for nb real tridiagonal eigenvectors z ([batch][nb][n]); X is written as
// complex ([batch][nb][n]) when Xout is given; optional Hellmann-Feynman gradients ([batch][nb][3]).
template <typename S>
void launch_backtransform(const S* H, int n, int ld, size_t mstride, const S* tq, const typename ST<S>::R* z, int nb,
                          cx<typename ST<S>::R>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                          int batch, cudaStream_t s, int lanes = 0);

// refine.cu: FP64 Rayleigh-Ritz in the m-dimensional subspace of FP32 vectors X32 ([batch][m][n]);
// the nb lowest Ritz values go to Eout, optionally vectors / gradients.
constexpr int kRefineMaxSubspace = 40;
__host__ __device__ inline size_t refine_work_elems(int n, int m) { return (size_t)2 * n * m; }
// small-solve scratch per matrix, contiguous: S (m x m), A (m x m), then the m x nb (<= m x m) Ritz
// coefficients W at offset 2 m^2
__host__ __device__ inline size_t refine_small_elems(int m, int) { return (size_t)3 * m * m; }
// H is the FP32-pair copy the mixed-path assembly writes (Split<S>); work holds Y = H X. With a
// local potential only (sv.on), H is not formed: H X = V X + diag(kinetic) X from the resident CSR
// of V (every row lists its diagonal, whose FP64 value V_ii + kinetic is split per k as the
// assembly would), summed in the same column order, so Y is the same as from the dense pairs.
// V without its diagonal in transposed ELL form: slot e of row r at [e * N + r], padded with zero
// values (column r) to the widest row, so that threads on consecutive rows load consecutive words.
struct SparseV {
    bool              on;
    int               W;     // slots per row
    const int*        col;   // [W][N]
    const float2*     re;    // [W][N] (hi, lo) of Re V
    const float2*     im;    // [W][N] (hi, lo) of Im V
    const cx<double>* Vloc;  // N x N column-major, for the diagonal
    const double*     rows;  // [batch][N][ROW_STRIDE], for the kinetic term
    int               N;
};
// tensor_cores: a complex dense H of order >= kRefineTcMinN takes Y = H X on the tensor cores
// (refine_tc.cu); status gets UEPM_K_NOCONVERGE there if a bounded wait gives up.
constexpr int kRefineTcMinN = 150;
template <typename S>
void launch_refine_project(const typename Split<S>::type* H, int n, int ld, size_t mstride, const cx<float>* X32, int m,
                           S* work, S* small, int batch, cudaStream_t s, const SparseV& sv, int* status = nullptr,
                           bool tensor_cores = true);
// refine_tc.cu: Y (double-single, [r][mp] per matrix, ystride float4 apart) = H X for complex H on
// the tensor cores; false when it does not apply (nothing launched).
bool launch_refine_y_tc(const ds4* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, int mp, void* work,
                        size_t ystride, int* status, int batch, cudaStream_t s);
template <typename S>
void launch_small_eigh(S* small, int m, int nb, double* Eout, S* W, int* status, int batch, cudaStream_t s, int cap = 0);
template <typename S>
void launch_refine_vectors(int n, int m, int nb, const cx<float>* X32, const S* W, cx<double>* Xout, double* grad,
                           const DevParams& P, const double* d_k, const int* d_G, int batch, cudaStream_t s);

}  // namespace uepm
