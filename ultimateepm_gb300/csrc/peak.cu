// peak.cu -- calibration kernels: sustained FMA throughput of the FP64 and FP32 pipes on the current
// device, used as the roofline denominator for the compute-bound eigensolver kernels (the measured
// peaks file of this machine pool only carries HBM copy bandwidth and bf16 GEMM rates).
#include <cuda_runtime.h>

#include <string>

#include "uepm_gb300.h"

namespace uepm {
void set_error(const std::string& msg);
void count_launch(int n);
}  // namespace uepm

namespace {

template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, int iters, T b, T c) {
    T a[CHAINS];
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) a[q] = T(threadIdx.x + q) * T(1e-3);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < CHAINS; ++q) a[q] = fma(a[q], b, c);
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) s += a[q];
    if (s == T(-1)) out[threadIdx.x] = s;  // keeps the chains live; never true in practice
}

template <typename T, int CHAINS>
double run(int iters) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T*        out    = nullptr;
    if (cudaMalloc(&out, sizeof(T) * threads) != cudaSuccess) return -1.0;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fma_peak<T, CHAINS><<<blocks, threads>>>(out, iters / 4, T(0.999999), T(1e-7));  // warm-up
    cudaEventRecord(a);
    k_fma_peak<T, CHAINS><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(b);
    uepm::count_launch(2);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int uepm_measure_peak(int precision, double* tflops) {
    if (!tflops) return UEPM_ERR_INVALID;
    const double t = (precision == UEPM_PREC_FP64) ? run<double, 8>(4096) : run<float, 16>(16384);
    if (t <= 0.0) {
        uepm::set_error("peak measurement failed");
        return UEPM_ERR_CUDA;
    }
    *tflops = t;
    return UEPM_OK;
}
