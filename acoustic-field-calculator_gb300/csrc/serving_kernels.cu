// Small kernels of the serving engine: the packed sources of a request from its resident
// geometry plus the request's amplitudes and phases (given split, or interleaved as the
// solvers write them).  The folding matches pack_source: log2|A| in the exponent, the sign of
// A as +pi on the phase.
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"

namespace afc {
namespace {

__device__ __forceinline__ float4 fold(float a, float ph) {
    return make_float4(log2f(fabsf(a)), a < 0.f ? ph + 3.14159265358979323846f : ph, a, ph);
}

__global__ void repack_split_kernel(const PackedSource* __restrict__ geom,
                                    const float* __restrict__ amps,
                                    const float* __restrict__ phases, int64_t n,
                                    PackedSource* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p = geom[j];
    p.c = fold(amps[j], phases[j]);
    out[j] = p;
}

__global__ void repack_interleaved_kernel(const PackedSource* __restrict__ geom,
                                          const float* __restrict__ amp_phase, int64_t n,
                                          PackedSource* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p = geom[j];
    p.c = fold(amp_phase[2 * j], amp_phase[2 * j + 1]);
    out[j] = p;
}

}  // namespace

cudaError_t launch_repack(const PackedSource* geom, const float* amps, const float* phases,
                          const float* amp_phase, int64_t n, PackedSource* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
    if (amp_phase)
        repack_interleaved_kernel<<<blocks, 256, 0, s>>>(geom, amp_phase, n, out);
    else
        repack_split_kernel<<<blocks, 256, 0, s>>>(geom, amps, phases, n, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace afc
