// Throughput probes for the roofline denominators of the CUDA-core and FP64
// kernels (no counterpart in the reference): FP32 FMA, FP64 FMA and FP64
// tensor-core (mma.sync m8n8k4 f64) rates of the current device, measured
// with CUDA events over a grid of several CTAs per SM.  Each thread runs
// independent dependency chains so that the pipes, not the latencies, bound
// the rate; the results feed the kernels' fraction-of-peak figures.

#include "../../include/spk_gpu.h"

#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int PROBE_ITERS = 4096;
constexpr int PROBE_CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_probe_fma(T* out, T seed) {
    T a[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) a[c] = seed + T(threadIdx.x + c);
    const T m = T(0.999999), k = T(1e-7);
    for (int it = 0; it < PROBE_ITERS; ++it) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) a[c] = a[c] * m + k;
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += a[c];
    if (s == T(-1)) out[blockIdx.x] = s;   // never true; keeps the chains alive
}

// One warp-wide m8n8k4 FP64 MMA per chain and iteration: 8 x 8 x 4 x 2 flops.
__global__ void __launch_bounds__(256) k_probe_dmma(double* out, double seed) {
    double acc[PROBE_CHAINS][2];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) { acc[c][0] = seed; acc[c][1] = seed + 1.0; }
    const double a = 1.0 + 1e-9 * threadIdx.x, b = 1.0 - 1e-9 * threadIdx.x;
    for (int it = 0; it < PROBE_ITERS / 4; ++it) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(acc[c][0]), "+d"(acc[c][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += acc[c][0] + acc[c][1];
    if (s == -1.0) out[blockIdx.x] = s;
}

template <typename K>
static double time_ms(K launch) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();   // warm-up
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

}  // namespace

extern "C" int spk_measure_peaks(double* fp32_tflops, double* fp64_tflops, double* dmma_tflops) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SPK_ECUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SPK_ECUDA;
    double* out = nullptr;
    const int grid = nsm * 8;
    if (cudaMalloc((void**)&out, sizeof(double) * grid) != cudaSuccess) return SPK_ENOMEM;
    const double threads = (double)grid * 256;
    double ms = time_ms([&] { k_probe_fma<float><<<grid, 256>>>((float*)out, 1.0f); });
    if (fp32_tflops) *fp32_tflops = threads * PROBE_ITERS * PROBE_CHAINS * 2.0 / (ms * 1e-3) / 1e12;
    ms = time_ms([&] { k_probe_fma<double><<<grid, 256>>>(out, 1.0); });
    if (fp64_tflops) *fp64_tflops = threads * PROBE_ITERS * PROBE_CHAINS * 2.0 / (ms * 1e-3) / 1e12;
    ms = time_ms([&] { k_probe_dmma<<<grid, 256>>>(out, 1.0); });
    if (dmma_tflops) *dmma_tflops = (threads / 32.0) * (PROBE_ITERS / 4) * PROBE_CHAINS * 512.0 / (ms * 1e-3) / 1e12;
    cudaError_t e = cudaGetLastError();
    cudaFree(out);
    return e == cudaSuccess ? SPK_OK : SPK_ECUDA;
}
