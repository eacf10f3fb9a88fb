// Pipe-rate microbenchmarks that measure the roofline of the direct summation on the GPU it
// runs on: results per second of each MUFU (special-function unit) operation the summation
// uses (ex2, rsqrt, sqrt, sin, cos), FP32 FMA results per second, and the SM clock seen while
// they run.  The summation's canonical per-evaluation cost is one of each of those MUFU
// operations plus 32 FP32 operations, so evals/s peak = min(1 / sum_op(1 / rate_op),
// fp32 / 32).
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_gpu.h"
#include "afc_internal.h"

namespace afc {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;
constexpr int kCalThreads = 256;

// One MUFU operation per step on kChains independent chains.  Op 0: x <- 2^x - 1 (ex2, plus
// one FADD), 1: x <- rsqrt(x), 2: x <- sqrt(x), 3: x <- sin(x), 4: x <- cos(x); every chain
// stays bounded.
template <int OP>
__device__ __forceinline__ float mufu_step(float x) {
    float y;
    if constexpr (OP == 0) {
        asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        y -= 1.0f;
    } else if constexpr (OP == 1) {
        asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    } else if constexpr (OP == 2) {
        asm volatile("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    } else if constexpr (OP == 3) {
        asm volatile("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    } else {
        asm volatile("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    }
    return y;
}

template <int OP>
__global__ void __launch_bounds__(kCalThreads) mufu_rate_kernel(float* sink, float seed) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (OP == 0 ? -0.25f : 0.75f) - 0.01f * c - seed * threadIdx.x;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = mufu_step<OP>(x[c]);
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

namespace afc {
namespace {

template <int OP>
double time_mufu(int blocks, float* sink, cudaEvent_t e0, cudaEvent_t e1, double ops) {
    double best = 0;
    for (int rep = 0; rep < 3; ++rep) {
        float ms = 0.f;
        cudaEventRecord(e0);
        mufu_rate_kernel<OP><<<blocks, kCalThreads>>>(sink, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        count_launch();
        if (rep > 0 && ms > 0) best = fmax(best, ops / (ms * 1e-3));
    }
    return best;
}

}  // namespace
}  // namespace afc

// rates[0..4] = ex2, rsqrt, sqrt, sin, cos results/s; rates[5] = FP32 FMA results/s.
extern "C" int32_t AFC_MeasurePipeRates(double* rates, double* sm_clock_hz, int32_t* sm_count) {
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
    rates[0] = time_mufu<0>(blocks, sink, e0, e1, ops);
    rates[1] = time_mufu<1>(blocks, sink, e0, e1, ops);
    rates[2] = time_mufu<2>(blocks, sink, e0, e1, ops);
    rates[3] = time_mufu<3>(blocks, sink, e0, e1, ops);
    rates[4] = time_mufu<4>(blocks, sink, e0, e1, ops);
    double best_ffma = 0;
    for (int rep = 0; rep < 3; ++rep) {
        float ms = 0.f;
        cudaEventRecord(e0);
        ffma_rate_kernel<<<blocks, kCalThreads>>>(sink, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        count_launch();
        if (rep > 0 && ms > 0) best_ffma = fmax(best_ffma, ops / (ms * 1e-3));
    }
    rates[5] = best_ffma;
    clock_kernel<<<1, 1>>>(clk, 20000000ull);
    count_launch();
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, clk, sizeof(h), cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    cudaFree(clk);
    if (e != cudaSuccess) return AFC_ERR_CUDA;
    if (sm_clock_hz) *sm_clock_hz = h[1] ? static_cast<double>(h[0]) / (h[1] * 1e-9) : 0.0;
    return AFC_OK;
}
