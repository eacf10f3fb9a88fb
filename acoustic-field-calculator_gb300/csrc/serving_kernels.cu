// Kernels of the serving engine.
//   * The packed sources of a request from its resident geometry plus the request's amplitudes
//     and phases (given split, or interleaved as the solvers write them).  The folding matches
//     pack_source: log2|A| in the exponent, the sign of A as +pi on the phase.
//   * The request groups (serving_group.h): one packing launch for all jobs, two persistent
//     kernels over the (tile, source chunk) items -- the rows body for rows tiles, the general
//     body for the rest, each item one block, the same per-block code as the single-job kernels
//     (field_body.cuh, field_rows.cuh) -- and a combine launch that adds the chunked jobs'
//     partial sums in chunk order and applies the field transform.
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"
#include "field_body.cuh"
#include "field_rows.cuh"
#include "serving_group.h"

namespace afc {
namespace {

__device__ __forceinline__ float4 fold(float a, float ph) {
    return make_float4(log2f(fabsf(a)), a < 0.f ? ph + 3.14159265358979323846f : ph, a, ph);
}

__global__ void repack_split_kernel(const PackedSource* __restrict__ geom,
                                    const float* __restrict__ amps,
                                    const float* __restrict__ phases, int64_t n,
                                    PackedSource* __restrict__ out) {
    dev::pdl_release();  // the field launch after this one may fill its tables now
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p = geom[j];
    p.c = fold(amps[j], phases[j]);
    out[j] = p;
}

__global__ void repack_interleaved_kernel(const PackedSource* __restrict__ geom,
                                          const float* __restrict__ amp_phase, int64_t n,
                                          PackedSource* __restrict__ out) {
    dev::pdl_release();  // the field launch after this one may fill its tables now
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p = geom[j];
    p.c = fold(amp_phase[2 * j], amp_phase[2 * j + 1]);
    out[j] = p;
}

// ------------------------------------------------------------------ request groups

using namespace fb;
using serve::GItem;
using serve::GJob;
using serve::kGroupPairs;

__constant__ float4 c_dir_table_s[kDirTableSize] = AFC_DIR_TABLE_INIT;

__global__ void group_repack_kernel(const GJob* __restrict__ jobs) {
    const GJob& J = jobs[blockIdx.y];
    for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < J.n;
         j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        PackedSource p = J.geom[j];
        p.c = fold(J.amps[j], J.amps[J.n + j]);
        J.packed[j] = p;
    }
}

// The next item of a persistent block (every thread gets it; n_items or more: none left).
__device__ __forceinline__ long long group_next(unsigned long long* counter, long long& s_item) {
    __syncthreads();  // the previous item's readers of shared memory and s_item are done
    if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(counter, 1ull));
    __syncthreads();
    return s_item;
}

__device__ __forceinline__ void chunk_range(const GJob& J, int32_t chunk, int64_t& lo,
                                           int64_t& hi) {
    lo = static_cast<int64_t>(chunk) * J.chunk;
    if (lo > J.n) lo = J.n;
    hi = lo + J.chunk < J.n ? lo + J.chunk : J.n;
}

template <int ST>
__global__ void __launch_bounds__(kThreads, 2)
    group_rows_kernel(const GJob* __restrict__ jobs, const GItem* __restrict__ items,
                      int64_t n_items, unsigned long long* __restrict__ counter) {
    constexpr int P = kGroupPairs;
    constexpr int kPPT = 2 * P;
    __shared__ RowsSmem rs;
    __shared__ long long s_item;
    SmemTile& sm = rs.sm;
    RowsTable& rt = rs.rt;
    load_theta_table(sm, c_dir_table_s);
    load_rows_table(rt);
    for (;;) {
        const long long it = group_next(counter, s_item);
        if (it >= n_items) break;
        const GItem w = items[it];
        const GJob& J = jobs[w.job];
        int64_t lo, hi;
        chunk_range(J, w.chunk, lo, hi);
        float2 RE[P], IM[P], CRE[P], CIM[P];
        rows_accumulate<ST, SUM_PLAIN, P, true>(sm, rt, J.packed, J.n, lo, hi, J.g, J.tx_log2, J.tiles0,
                                          J.tiles1, w.tile, RE, IM, CRE, CIM);
        if (J.chunks == 1) {
            rows_store<SUM_PLAIN, P>(J.packed, J.n, J.g, J.tx_log2, J.tiles0, J.tiles1, w.tile,
                                     RE, IM, CRE, CIM, J.field, J.out);
            continue;
        }
        // the chunk's partial sums at the tile's points (indices as rows_store computes them)
        const int tx = threadIdx.x & ((1 << J.tx_log2) - 1);
        const int ty = threadIdx.x >> J.tx_log2;
        const int64_t t0 = w.tile % J.tiles0, rest = w.tile / J.tiles0;
        const int64_t t1 = rest % J.tiles1, i2 = rest / J.tiles1;
        const int64_t c0 = J.g.count[0], c1 = J.g.count[1];
        const int64_t i0 = (t0 << J.tx_log2) + tx;
        const int64_t i1b = (t1 * (kThreads >> J.tx_log2) + ty) * kPPT;
        if (i0 >= c0) continue;
        float2* part = J.partial + static_cast<int64_t>(w.chunk) * J.m;
#pragma unroll
        for (int k = 0; k < kPPT; ++k) {
            const int64_t i1 = i1b + k;
            if (i1 >= c1) break;
            part[(i2 * c1 + i1) * c0 + i0] =
                make_float2(lane_of(RE[k >> 1], k & 1), lane_of(IM[k >> 1], k & 1));
        }
    }
}

template <int ST>
__global__ void __launch_bounds__(kThreads, 2)
    group_flat_kernel(const GJob* __restrict__ jobs, const GItem* __restrict__ items,
                      int64_t n_items, unsigned long long* __restrict__ counter) {
    constexpr int P = kGroupPairs;
    constexpr int kPPT = 2 * P;
    __shared__ SmemTile sm;
    __shared__ long long s_item;
    extern __shared__ __align__(16) unsigned char group_dyn_smem[];
    GTable& gt = *reinterpret_cast<GTable*>(group_dyn_smem);
    load_theta_table(sm, c_dir_table_s);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    for (;;) {
        const long long it = group_next(counter, s_item);
        if (it >= n_items) break;
        const GItem w = items[it];
        const GJob& J = jobs[w.job];
        int64_t lo, hi;
        chunk_range(J, w.chunk, lo, hi);
        const int64_t first = w.tile * (kThreads * kPPT);
        float2 RE[P], IM[P], CRE[P], CIM[P];
        block_accumulate<ST, SUM_PLAIN, P, true>(sm, gt, J.packed, J.n, lo, hi, J.is_grid != 0, J.g,
                                           J.pts, J.m, first, RE, IM, CRE, CIM);
        if (J.chunks == 1) {
            block_store<SUM_PLAIN, P>(RE, IM, CRE, CIM, J.packed, J.n, J.is_grid != 0, J.g, J.pts,
                                      first, J.m, J.field, J.out);
            continue;
        }
        float2* part = J.partial + static_cast<int64_t>(w.chunk) * J.m;
#pragma unroll
        for (int k = 0; k < kPPT; ++k) {
            const int64_t p = first + threadIdx.x + static_cast<int64_t>(k) * kThreads;
            if (p >= J.m) break;
            part[p] = make_float2(lane_of(RE[k >> 1], k & 1), lane_of(IM[k >> 1], k & 1));
        }
    }
}

// The chunked jobs' fields: the partial sums added in chunk order, the field transform, and
// the coincident-source fix-up of the single-job kernels for NaN sums.
__global__ void group_combine_kernel(const GJob* __restrict__ jobs) {
    const GJob& J = jobs[blockIdx.y];
    if (J.chunks <= 1) return;
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < J.m;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float re = 0.f, im = 0.f;
        for (int32_t c = 0; c < J.chunks; ++c) {
            const float2 v = J.partial[static_cast<int64_t>(c) * J.m + p];
            re = __fadd_rn(re, v.x);
            im = __fadd_rn(im, v.y);
        }
        store_field(J.out, p, J.field, re, im);
        if (isnan(re) || isnan(im)) {
            float x, y, z;
            if (J.is_grid) {
                grid_point(J.g, p, x, y, z);
            } else {
                x = J.pts[3 * p];
                y = J.pts[3 * p + 1];
                z = J.pts[3 * p + 2];
            }
            fix_coincident(J.packed, J.n, x, y, z, p, J.field, J.out);
        }
    }
}

template <int ST>
constexpr int group_dyn_bytes() {
    return ST == SRC_T4010A1 ? kGTableBytes : 0;
}

template <auto Kernel>
int group_occupancy(int dyn) {
    int b = 0;
    if (allow_dynamic_smem<Kernel>(dyn) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, Kernel, kThreads, dyn) != cudaSuccess ||
        b < 1) {
        (void)cudaGetLastError();
        b = 1;
    }
    return b;
}

template <int ST>
cudaError_t launch_group_st(const GJob* d_jobs, int n_jobs, int64_t max_n, const GItem* d_rows,
                            int64_t n_rows, const GItem* d_flat, int64_t n_flat,
                            unsigned long long* d_counters, bool chunked, int rows_blocks,
                            int flat_blocks, cudaStream_t s, cudaStream_t s2, cudaEvent_t fork,
                            cudaEvent_t join) {
    cudaError_t e = cudaMemsetAsync(d_counters, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (max_n > 0) {
        const int64_t bx = (max_n + 255) / 256;
        group_repack_kernel<<<dim3(static_cast<unsigned>(bx < 64 ? bx : 64), n_jobs), 256, 0, s>>>(
            d_jobs);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    constexpr int kDyn = group_dyn_bytes<ST>();
    if ((e = allow_dynamic_smem<group_flat_kernel<ST>>(kDyn)) != cudaSuccess) return e;
    const bool both = n_rows > 0 && n_flat > 0;
    if (both) {
        if ((e = cudaEventRecord(fork, s)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s2, fork, 0)) != cudaSuccess)
            return e;
    }
    if (n_rows > 0) {
        group_rows_kernel<ST><<<rows_blocks, kThreads, 0, s>>>(d_jobs, d_rows, n_rows, d_counters);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (n_flat > 0) {
        group_flat_kernel<ST><<<flat_blocks, kThreads, kDyn, both ? s2 : s>>>(d_jobs, d_flat, n_flat,
                                                                            d_counters + 1);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (both) {
        if ((e = cudaEventRecord(join, s2)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s, join, 0)) != cudaSuccess)
            return e;
    }
    if (chunked) {
        group_combine_kernel<<<dim3(256, n_jobs), 256, 0, s>>>(d_jobs);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

int serve::group_rows_occupancy(int st) {
    return st == SRC_T4010A1 ? group_occupancy<group_rows_kernel<SRC_T4010A1>>(0)
                             : group_occupancy<group_rows_kernel<SRC_SPHERE>>(0);
}

int serve::group_flat_occupancy(int st) {
    return st == SRC_T4010A1
               ? group_occupancy<group_flat_kernel<SRC_T4010A1>>(group_dyn_bytes<SRC_T4010A1>())
               : group_occupancy<group_flat_kernel<SRC_SPHERE>>(group_dyn_bytes<SRC_SPHERE>());
}

cudaError_t serve::launch_group(int st, const GJob* d_jobs, int n_jobs, int64_t max_n,
                                const GItem* d_rows, int64_t n_rows, const GItem* d_flat,
                                int64_t n_flat, unsigned long long* d_counters, bool chunked,
                                int rows_blocks, int flat_blocks, cudaStream_t s, cudaStream_t s2,
                                cudaEvent_t fork, cudaEvent_t join) {
    if (n_jobs <= 0) return cudaSuccess;
    if (st == SRC_T4010A1)
        return launch_group_st<SRC_T4010A1>(d_jobs, n_jobs, max_n, d_rows, n_rows, d_flat, n_flat,
                                            d_counters, chunked, rows_blocks, flat_blocks, s, s2,
                                            fork, join);
    return launch_group_st<SRC_SPHERE>(d_jobs, n_jobs, max_n, d_rows, n_rows, d_flat, n_flat,
                                       d_counters, chunked, rows_blocks, flat_blocks, s, s2, fork,
                                       join);
}

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
