// Summary statistics (mean, sample standard deviation) without any device
// allocation: a variant of sdbe_summary_stats for callers that cannot call
// cudaMalloc.  In APHIDS the GPU stage shares the device with the threads that
// copy packet groups in and payloads out; a cudaMalloc/cudaFree there can
// synchronize the whole device and stall those copies, and some callers run
// with a fixed, pre-reserved amount of device memory.  This entry point uses a fixed
// file-scope device array instead.
//
// The per-block partial sums of the existing kernel (k_stats_partial, one
// pair of FP64 sums per block, 256 threads x 64 samples per block) land in
// g_noalloc_scratch; a one-thread kernel in this file merges them in block
// order and leaves (mean, std) in the last two slots, which are copied to the
// caller's host memory.  The call waits for its stream before it returns.
#include <cuda_runtime.h>

#include <string>

#include "launchers.cuh"
#include "sdbe_internal.cuh"

namespace sdbe {

constexpr int kNoallocBlocks = 8192;          // partial pairs the array holds
constexpr int64_t kNoallocSamplesPerBlock = 256 * 64;

// 8192 partial pairs + (mean, std): 131,088 bytes on every device that loads
// the library, held until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[2 * kNoallocBlocks + 2];

// The partial sums are of x - in[0] (k_stats_partial), so the mean is in[0]
// plus their mean and no large offset cancels in the variance.
__global__ void k_noalloc_finalize(const float *in, int blocks, int64_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s1 = 0.0, s2 = 0.0;
    for (int b = 0; b < blocks; ++b) {
        s1 += g_noalloc_scratch[2 * b];
        s2 += g_noalloc_scratch[2 * b + 1];
    }
    const double nn = static_cast<double>(n);
    const double dmean = s1 / nn;
    g_noalloc_scratch[2 * kNoallocBlocks] = static_cast<double>(in[0]) + dmean;
    g_noalloc_scratch[2 * kNoallocBlocks + 1] = sqrt((s2 - s1 * dmean) / (nn - 1.0));
}

namespace {
// Device address of the array in the current device's context.  Looked up on
// every call (a host-side query that allocates nothing): an address kept from
// an earlier call would dangle once that context is torn down
// (cudaDeviceReset) and the module is loaded again.
cudaError_t noalloc_scratch(double **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    *out = static_cast<double *>(p);
    return e;
}
}  // namespace

}  // namespace sdbe

using namespace sdbe;

extern "C" int sdbe_summary_stats_noalloc(const float *in, int64_t n, double *out_host, void *stream) {
    if (!in || !out_host || n < 2) {
        set_thread_error("sdbe_summary_stats_noalloc: need n >= 2 and non-null pointers");
        return SDBE_ERR_ARG;
    }
    if (n > SDBE_NOALLOC_MAX_SAMPLES) {
        set_thread_error("sdbe_summary_stats_noalloc: n = " + std::to_string(n) + " exceeds the maximum of " +
                         std::to_string(static_cast<long long>(SDBE_NOALLOC_MAX_SAMPLES)) +
                         " samples (its fixed device array holds 8192 partial sums)");
        return SDBE_ERR_CAPACITY;
    }
    double *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int blocks = static_cast<int>((n + kNoallocSamplesPerBlock - 1) / kNoallocSamplesPerBlock);
    if (e == cudaSuccess) e = launch_stats_partial(in, n, scratch, blocks, st);
    if (e == cudaSuccess) {
        k_noalloc_finalize<<<1, 32, 0, st>>>(in, blocks, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out_host, scratch + 2 * kNoallocBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_thread_error(std::string("sdbe_summary_stats_noalloc: ") + cudaGetErrorString(e));
        return SDBE_ERR_CUDA;
    }
    return SDBE_OK;
}
