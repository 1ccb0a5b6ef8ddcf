// uepm_kernels.h -- host-side launch wrappers of the device kernels (one declaration per kernel).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "uepm_common.cuh"

namespace uepm {

void count_launch(int n = 1);

// assemble.cu
void launch_rows(const DevParams& P, const double* d_k, const int* d_G, double* d_rows, int batch, cudaStream_t s);
void launch_assemble(const DevParams& P, const cx<double>* Vloc, const double2* phNL, const double2* phSO, const double* rows,
                     cx<double>* H, int ld, size_t mstride, cx<float>* H32, size_t mstride32, int batch, cudaStream_t s);
void launch_mirror_upper(cx<double>* H, int n, int ld, size_t mstride, int batch, cudaStream_t s);

// tridiag.cu: Householder reduction of the lower triangle, in place. d, e: [batch][n];
// tq: [batch][n] reflector scalars; status: [batch] (ORed with UEPM_K_NONFINITE on NaN/Inf).
template <typename T>
void launch_tridiag(cx<T>* H, int n, int ld, size_t mstride, T* d, T* e, cx<T>* tq, int* status, int batch, cudaStream_t s);

// tridiag_eig.cu
template <typename T>
void launch_bisect(const T* d, const T* e, int n, int nb, T* ev, int ev_ld, int batch, cudaStream_t s);
template <typename T>
void launch_invit(const T* d, const T* e, const T* ev, int ev_ld, int n, int nb, T* work, T* z, int* status, int batch,
                  cudaStream_t s);
// Inverse-iteration workspace per matrix: U0, U1, U2, Y, Z, each n x 32 interleaved by lane.
template <typename T>
__host__ __device__ inline size_t invit_work_elems(int n) {
    return (size_t)5 * n * 32;
}

// backtransform.cu: X = Q Z for the nb vectors, optional gradient and complex-vector output.
template <typename T>
void launch_backtransform(const cx<T>* H, int n, int ld, size_t mstride, const cx<T>* tq, const T* z, int nb,
                          cx<T>* Xout, const DevParams& P, const double* d_k, const int* d_G, double* grad,
                          const T* ev, double* Eout, int batch, cudaStream_t s);

// refine.cu: FP64 residual + Rayleigh-Ritz in the nb-dimensional subspace of FP32 vectors.
// X32 holds m >= nb FP32 vectors ([batch][m][n]); the nb lowest Ritz pairs are returned.
constexpr int kRefineMaxSubspace = 40;
void launch_refine(const cx<double>* H, int n, int ld, size_t mstride, const cx<float>* X32, int m, int nb, double* Eout,
                   cx<double>* Xout, double* grad, const DevParams& P, const double* d_k, const int* d_G, cx<double>* work,
                   int* status, int batch, cudaStream_t s);
__host__ __device__ inline size_t refine_work_elems(int n, int m) { return (size_t)2 * n * m; }

}  // namespace uepm
