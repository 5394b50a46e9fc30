// FP32 FMA issue rate of the device: the denominator of the FP32 FFT
// kernels' roofline (they are bound by FP32 issue, not by HBM).  A grid of
// two 512-thread CTAs per SM runs 16 independent FMA chains per thread, so
// every scheduler always has FMAs ready; timed with CUDA events.
#include <cuda_runtime.h>

#include <string>

#include "sdbe_internal.cuh"

namespace sdbe {
namespace {

constexpr int kPeakThreads = 512;
constexpr int kChains = 16;

__global__ void __launch_bounds__(kPeakThreads) k_fma_peak(float *out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) x[j] = static_cast<float>(threadIdx.x + j) * 1e-3f;
#pragma unroll 2
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += x[j];
    if (s == 12345.678f) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace
}  // namespace sdbe

using namespace sdbe;

extern "C" int sdbe_fp32_fma_rate(int32_t device, double *tflops, double *ms) {
    if (!tflops || !ms) return SDBE_ERR_ARG;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int iters = 1 << 18;
    const unsigned grid = static_cast<unsigned>(2 * sms);
    float t = 0.f;
    if (e == cudaSuccess) {
        k_fma_peak<<<grid, kPeakThreads>>>(out, iters / 8, 0.999f, 1e-3f);  // warm-up (clocks up)
        k_fma_peak<<<grid, kPeakThreads>>>(out, iters / 8, 0.999f, 1e-3f);
        e = cudaEventRecord(e0);
    }
    if (e == cudaSuccess) {
        k_fma_peak<<<grid, kPeakThreads>>>(out, iters, 0.999f, 1e-3f);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        set_thread_error(std::string("sdbe_fp32_fma_rate: ") + cudaGetErrorString(e));
        return SDBE_ERR_CUDA;
    }
    const double flops = 2.0 * kChains * static_cast<double>(iters) * grid * kPeakThreads;
    *ms = t;
    *tflops = flops / (static_cast<double>(t) * 1e-3) / 1e12;
    return SDBE_OK;
}
