// Issue-rate microbenchmarks that measure the roofline of the direct summation on the GPU it
// runs on: MUFU (SFU) results per second, FP32 FMA results per second, and the SM clock seen
// while they run.  The field kernel's per-pair cost is quoted in these units (5 MUFU + 32 FP32
// operations per source-point evaluation), so evals/s peak = min(mufu/5, fp32/32).
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_gpu.h"
#include "afc_internal.h"

namespace afc {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;
constexpr int kCalThreads = 256;

// x <- 2^x - 1 keeps every chain in [-0.5, 0): one MUFU.EX2 and one FADD per step.
__global__ void __launch_bounds__(kCalThreads) mufu_rate_kernel(float* sink, float seed) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = -0.25f - 0.01f * c - seed * threadIdx.x;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) {
            float y;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            x[c] = y - 1.0f;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.f) sink[threadIdx.x] = s;  // keeps the chains alive
}

// x <- x * a + b, a contraction towards a fixed point: one FFMA per step.
__global__ void __launch_bounds__(kCalThreads) ffma_rate_kernel(float* sink, float seed) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.5f + 0.01f * c + seed * threadIdx.x;
    const float a = 0.999f, b = 0.0005f;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.f) sink[threadIdx.x] = s;
}

// SM clock: cycles counted by clock64 over a globaltimer interval, one thread.
__global__ void clock_kernel(unsigned long long* out, unsigned long long spin_ns) {
    unsigned long long t0, t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const long long c0 = clock64();
    unsigned long long guard = 0;
    do {
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    } while (t1 - t0 < spin_ns && ++guard < (1ull << 32));
    const long long c1 = clock64();
    out[0] = static_cast<unsigned long long>(c1 - c0);
    out[1] = t1 - t0;
}

}  // namespace
}  // namespace afc

extern "C" int32_t AFC_MeasureIssueRates(double* mufu_per_s, double* fp32_per_s,
                                         double* sm_clock_hz, int32_t* sm_count) {
    using namespace afc;
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return AFC_ERR_NO_DEVICE;
    if (sm_count) *sm_count = prop.multiProcessorCount;
    float* sink = nullptr;
    unsigned long long* clk = nullptr;
    if (cudaMalloc(&sink, sizeof(float) * kCalThreads) != cudaSuccess) return AFC_ERR_CUDA;
    if (cudaMalloc(&clk, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(sink);
        return AFC_ERR_CUDA;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = prop.multiProcessorCount * 8;
    const double ops = static_cast<double>(blocks) * kCalThreads * kChains * kIters;
    float ms = 0.f;
    double best_mufu = 0, best_ffma = 0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        mufu_rate_kernel<<<blocks, kCalThreads>>>(sink, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0) best_mufu = fmax(best_mufu, ops / (ms * 1e-3));
        cudaEventRecord(e0);
        ffma_rate_kernel<<<blocks, kCalThreads>>>(sink, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0) best_ffma = fmax(best_ffma, ops / (ms * 1e-3));
        count_launch(2);
    }
    clock_kernel<<<1, 1>>>(clk, 20000000ull);
    count_launch();
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, clk, sizeof(h), cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    cudaFree(clk);
    if (e != cudaSuccess) return AFC_ERR_CUDA;
    if (mufu_per_s) *mufu_per_s = best_mufu;
    if (fp32_per_s) *fp32_per_s = best_ffma;
    if (sm_clock_hz) *sm_clock_hz = h[1] ? static_cast<double>(h[0]) / (h[1] * 1e-9) : 0.0;
    return AFC_OK;
}
