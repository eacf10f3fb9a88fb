// Direct source->point summation on sm_103a.
//
// For every observation point x the kernels form
//     p(x) = sum_j A_j D(theta_j) exp(-alpha_j r_j) / r_j * exp(i (phi_j + k_j r_j))
// in FP32, sources in index order, which is the per-pair math of
// acoustic-field-calculator/src/system/uniform_medium.rs:111-120 summed as in :122-128, then
// apply the field transform of field_buffer/{pressure,power,complex_pressure}_field.rs:35-37.
//
// Layout and schedule
//   * Sources are packed once per call (PackedSource, 48 B) and streamed through shared memory
//     in tiles of kTile; every thread of a block reads the same source at the same time, so the
//     shared-memory reads are broadcasts.
//   * Each thread owns kPPT observation points spaced kThreads apart, so each of its kPPT
//     stores is part of one contiguous, coalesced warp store (4 B or 8 B per point).
//   * Grid points are generated from the grid description, never read from memory.
//
// Per pair: 3 sub, r^2, rsqrt (MUFU), cos(theta), acos, the directivity cubic (coefficients
// from a shared-memory table indexed by the 10-degree bin), ex2 (MUFU) for the attenuation,
// phase = phi + k r reduced to [-pi, pi] by a two-constant Cody-Waite step, then __sincosf
// (MUFU sin + cos) and two FMAs into the accumulators.
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"
#include "propagate.cuh"

namespace afc {

namespace {

constexpr int kThreads = 256;  // threads per block
constexpr int kPPT = 4;        // observation points per thread
constexpr int kTile = 256;     // sources per shared-memory tile

using dev::kLog2e;

__constant__ float4 c_dir_table[dev::kDirTableSize] = AFC_DIR_TABLE_INIT;

// Neumaier's compensated addition: sum + v with the lost low-order part added to comp.
__device__ __forceinline__ void neumaier_add(float& sum, float& comp, float v) {
    const float t = __fadd_rn(sum, v);
    if (fabsf(sum) >= fabsf(v)) {
        comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(sum, t), v));
    } else {
        comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(v, t), sum));
    }
    sum = t;
}

// Coordinates of grid point p, bit-identical to the reference's o + (n as f32 * res).
__device__ __forceinline__ void grid_point(const GridDev& g, int64_t p, float& x, float& y,
                                           float& z) {
    const int64_t i0 = p % g.count[0];
    const int64_t q = p / g.count[0];
    const int64_t i1 = q % g.count[1];
    const int64_t i2 = q / g.count[1];
    float v[3];
    v[0] = g.origin[0];
    v[1] = g.origin[1];
    v[2] = g.origin[2];
    const int64_t idx[3] = {i0, i1, i2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (g.count[k] > 1) {
            const int a = g.axis[k];
            const float o = a == 0 ? g.origin[0] : (a == 1 ? g.origin[1] : g.origin[2]);
            const float c = __fadd_rn(o, __fmul_rn(__ll2float_rn(idx[k]), g.res));
            if (a == 0) v[0] = c;
            else if (a == 1) v[1] = c;
            else v[2] = c;
        }
    }
    x = v[0];
    y = v[1];
    z = v[2];
}

template <int ST, int FT, int SUM, bool GRID>
__global__ void __launch_bounds__(kThreads, 2)
    field_direct_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                        const float* __restrict__ pts, int64_t m, void* __restrict__ out) {
    __shared__ float4 s_a[kTile];
    __shared__ float4 s_b[kTile];
    __shared__ float2 s_c[kTile];
    __shared__ float4 s_dir[dev::kDirTableSize];

    if (threadIdx.x < dev::kDirTableSize) s_dir[threadIdx.x] = c_dir_table[threadIdx.x];

    const int64_t base = static_cast<int64_t>(blockIdx.x) * (kThreads * kPPT) + threadIdx.x;
    float px[kPPT], py[kPPT], pz[kPPT];
    float re[kPPT], im[kPPT], cre[kPPT], cim[kPPT];
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        int64_t p = base + static_cast<int64_t>(k) * kThreads;
        if (p >= m) p = m - 1;  // computed but never stored
        if constexpr (GRID) {
            grid_point(g, p, px[k], py[k], pz[k]);
        } else {
            px[k] = __ldg(pts + 3 * p);
            py[k] = __ldg(pts + 3 * p + 1);
            pz[k] = __ldg(pts + 3 * p + 2);
        }
        re[k] = 0.f;
        im[k] = 0.f;
        cre[k] = 0.f;
        cim[k] = 0.f;
    }

    for (int64_t t0 = 0; t0 < n; t0 += kTile) {
        const int cnt = static_cast<int>((n - t0) < kTile ? (n - t0) : kTile);
        __syncthreads();
        for (int j = threadIdx.x; j < cnt; j += kThreads) {
            const PackedSource s = src[t0 + j];
            s_a[j] = s.a;
            s_b[j] = s.b;
            s_c[j] = make_float2(s.c.x, s.c.y);
        }
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < cnt; ++j) {
            const float4 a = s_a[j];
            const float4 b = s_b[j];
            const float2 c = s_c[j];
#pragma unroll
            for (int k = 0; k < kPPT; ++k) {
                float w, red;
                dev::pair_terms<ST>(a, b, c.x, c.y, s_dir, px[k], py[k], pz[k], w, red);
                float sn, cs;
                __sincosf(red, &sn, &cs);
                if constexpr (SUM == SUM_PLAIN) {
                    re[k] = fmaf(w, cs, re[k]);
                    im[k] = fmaf(w, sn, im[k]);
                } else {
                    neumaier_add(re[k], cre[k], w * cs);
                    neumaier_add(im[k], cim[k], w * sn);
                }
            }
        }
    }

#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        const int64_t p = base + static_cast<int64_t>(k) * kThreads;
        if (p >= m) break;
        float vr = re[k], vi = im[k];
        if constexpr (SUM == SUM_COMPENSATED) {
            vr = __fadd_rn(vr, cre[k]);
            vi = __fadd_rn(vi, cim[k]);
        }
        if constexpr (FT == FIELD_COMPLEX) {
            reinterpret_cast<float2*>(out)[p] = make_float2(vr, vi);
        } else {
            // norm_sqr = re*re + im*im without contraction (pressure_field.rs:35-37)
            const float ns = __fadd_rn(__fmul_rn(vr, vr), __fmul_rn(vi, vi));
            reinterpret_cast<float*>(out)[p] = (FT == FIELD_PRESSURE) ? __fsqrt_rn(ns) : ns;
        }
    }
}

__global__ void pack_sources_kernel(int st, const float* __restrict__ raw,
                                    const float* __restrict__ k, const float* __restrict__ atten,
                                    int64_t n, PackedSource* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p;
    if (st == SRC_T4010A1) {
        const float* s = raw + 9 * j;
        p.a = make_float4(s[0], s[1], s[2], k[j]);
        p.b = make_float4(s[3], s[4], s[5], -atten[j] * kLog2e);
        p.c = make_float4(s[6], s[7], 0.f, 0.f);
    } else {
        const float* s = raw + 6 * j;
        p.a = make_float4(s[0], s[1], s[2], k[j]);
        p.b = make_float4(0.f, 0.f, 0.f, -atten[j] * kLog2e);
        p.c = make_float4(s[3], s[4], 0.f, 0.f);
    }
    out[j] = p;
}

template <int ST, int FT, int SUM>
cudaError_t launch_typed(const PackedSource* src, int64_t n, const PointSet& ps, void* out,
                         cudaStream_t s) {
    const int64_t per_block = static_cast<int64_t>(kThreads) * kPPT;
    const int64_t blocks = (ps.m + per_block - 1) / per_block;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    if (ps.is_grid) {
        field_direct_kernel<ST, FT, SUM, true>
            <<<static_cast<unsigned>(blocks), kThreads, 0, s>>>(src, n, ps.grid, nullptr, ps.m, out);
    } else {
        field_direct_kernel<ST, FT, SUM, false>
            <<<static_cast<unsigned>(blocks), kThreads, 0, s>>>(src, n, ps.grid, ps.pts, ps.m, out);
    }
    count_launch();
    return cudaGetLastError();
}

template <int ST, int FT>
cudaError_t launch_sum(int sum_mode, const PackedSource* src, int64_t n, const PointSet& ps,
                       void* out, cudaStream_t s) {
    return sum_mode == SUM_COMPENSATED ? launch_typed<ST, FT, SUM_COMPENSATED>(src, n, ps, out, s)
                                       : launch_typed<ST, FT, SUM_PLAIN>(src, n, ps, out, s);
}

template <int ST>
cudaError_t launch_field_t(int field, int sum_mode, const PackedSource* src, int64_t n,
                           const PointSet& ps, void* out, cudaStream_t s) {
    switch (field) {
        case FIELD_PRESSURE: return launch_sum<ST, FIELD_PRESSURE>(sum_mode, src, n, ps, out, s);
        case FIELD_POWER: return launch_sum<ST, FIELD_POWER>(sum_mode, src, n, ps, out, s);
        case FIELD_COMPLEX: return launch_sum<ST, FIELD_COMPLEX>(sum_mode, src, n, ps, out, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

std::atomic<uint64_t> g_launches{0};

cudaError_t launch_pack_sources(int st, const float* raw, const float* k, const float* atten,
                                int64_t n, PackedSource* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    pack_sources_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(st, raw, k, atten, n, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_field(int st, int field, int sum_mode, const PackedSource* src, int64_t n,
                         const PointSet& ps, void* out, cudaStream_t s) {
    if (ps.m <= 0) return cudaSuccess;
    if (st == SRC_T4010A1) return launch_field_t<SRC_T4010A1>(field, sum_mode, src, n, ps, out, s);
    if (st == SRC_SPHERE) return launch_field_t<SRC_SPHERE>(field, sum_mode, src, n, ps, out, s);
    return cudaErrorInvalidValue;
}

}  // namespace afc
