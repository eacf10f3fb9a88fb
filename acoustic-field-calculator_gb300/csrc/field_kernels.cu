// Direct source->point summation on sm_103a.
//
// For every observation point x the kernels form
//     p(x) = sum_j A_j D(theta_j) exp(-alpha_j r_j) / r_j * exp(i (phi_j + k_j r_j))
// in FP32, sources in index order, which is the per-pair math of
// acoustic-field-calculator/src/system/uniform_medium.rs:111-120 summed as in :122-128, then
// apply the field transform of field_buffer/{pressure,power,complex_pressure}_field.rs:35-37.
//
// Layout and schedule (the per-block body is in field_body.cuh)
//   * Sources are packed once per call (PackedSource, 48 B) and staged tile by tile into
//     shared memory with every per-source scalar stored twice ((v, v) pairs), so that one
//     LDS.128 yields two packed f32x2 broadcast operands.  All threads of a block read the
//     same source at the same time: shared-memory broadcasts.
//   * Each thread owns 2*PAIRS observation points spaced kThreads apart and processes them two
//     at a time with the sm_100 packed FP32 instructions (FFMA2 / FMUL2 / FADD2), which halves
//     the FP32 instructions issued; MUFU operations stay per point.  The PAIRS pairs of one
//     source are independent, so their instructions interleave; when any of a thread's
//     points has its theta next to a directivity bin edge (a single predicate), those points
//     are corrected after the source, off the interleaved path.
//   * On grids with more than one point along the second axis a thread's points are
//     consecutive along that axis (field_rows_kernel), so the offsets along the other two axes
//     are computed once per source and thread.  Both bodies take the directivity from a
//     cos(theta)-indexed table (no acos, no MUFU square root; propagate.cuh): the rows body
//     from the plain table, whose entries neighbouring grid points share, the general body from
//     a lane-replicated copy in dynamic shared memory that scattered points read without bank
//     conflicts.
//   * When every source of a tile points the same way as source 0 (a planar array), cos(theta)
//     comes from n.x - n.s with n.x precomputed per point and n.s per source: two FP32
//     operations per pair instead of four.  Each block decides this per tile.
//   * Each of the 2*PAIRS stores is one contiguous, coalesced warp store (4 B or 8 B a point).
//   * Grid points are generated from the grid description, never read from memory.
//   * Launches too small to give every SM two blocks split each point tile's sources over the
//     blocks of a thread-block cluster (field_split_kernel): rank r sums its share of the
//     sources, and rank 0 adds the others' partial sums, read from their shared memory, in
//     rank order -- deterministic, no workspace.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"
#include "field_body.cuh"
#include "field_rows.cuh"
#include "propagate.cuh"

namespace afc {

namespace {

using namespace fb;

__constant__ float4 c_dir_table[kDirTableSize] = AFC_DIR_TABLE_INIT;

// The general body's lane-replicated directivity table lives in dynamic shared memory
// (kGTableBytes for T4010A1 sources, none for sphere sources).
__device__ __forceinline__ GTable& dynamic_gtab() {
    extern __shared__ __align__(16) unsigned char afc_dyn_smem[];
    return *reinterpret_cast<GTable*>(afc_dyn_smem);
}

template <int ST, int SUM, bool GRID, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_direct_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                        const float* __restrict__ pts, int64_t m, int field,
                        void* __restrict__ out) {
    __shared__ SmemTile sm;
    GTable& gt = dynamic_gtab();
    load_theta_table(sm, c_dir_table);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    const int64_t first = static_cast<int64_t>(blockIdx.x) * (kThreads * 2 * PAIRS);
    block_points<ST, SUM, PAIRS>(sm, gt, src, n, GRID, g, pts, m, first, field, out);
}

// The partial sums of a cluster's blocks, combined into rank 0's: every rank writes its sums
// into its own staging arrays (free once its last tile is done), rank 0 adds ranks 1 .. S-1's
// (read from their shared memory through the cluster) in rank order.  Both cluster barriers
// are reached by every thread of every block; the second keeps the other ranks' shared memory
// alive until rank 0 has read it.
template <int SUM, int PAIRS>
__device__ __forceinline__ void cluster_combine(SmemTile& sm, float2 (&RE)[PAIRS],
                                                float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                                float2 (&CIM)[PAIRS]) {
    namespace cg = cooperative_groups;
    constexpr int kPPT = 2 * PAIRS;
    // partial sums (and compensations) of every thread, in the staging arrays once free
    static_assert(sizeof(float2) * (SUM == SUM_COMPENSATED ? 2 : 1) * kPPT * kThreads <=
                      4 * sizeof(sm.v0),
                  "partial sums must fit in the first four staging arrays");
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned S = cluster.num_blocks();
    const unsigned rank = cluster.block_rank();
    __syncthreads();  // the staging arrays are free
    float2* part = reinterpret_cast<float2*>(sm.v0);
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        part[k * kThreads + threadIdx.x] =
            make_float2(lane_of(RE[k >> 1], k & 1), lane_of(IM[k >> 1], k & 1));
        if constexpr (SUM == SUM_COMPENSATED)
            part[(kPPT + k) * kThreads + threadIdx.x] =
                make_float2(lane_of(CRE[k >> 1], k & 1), lane_of(CIM[k >> 1], k & 1));
    }
    cluster.sync();
    if (rank == 0) {
        for (unsigned q = 1; q < S; ++q) {
            const float2* rp = cluster.map_shared_rank(part, q);
#pragma unroll
            for (int k = 0; k < kPPT; ++k) {
                const float2 v = rp[k * kThreads + threadIdx.x];
                if constexpr (SUM == SUM_PLAIN) {
                    lane_of(RE[k >> 1], k & 1) += v.x;
                    lane_of(IM[k >> 1], k & 1) += v.y;
                } else {
                    const float2 c = rp[(kPPT + k) * kThreads + threadIdx.x];
                    neumaier_add(lane_of(RE[k >> 1], k & 1), lane_of(CRE[k >> 1], k & 1), v.x);
                    neumaier_add(lane_of(RE[k >> 1], k & 1), lane_of(CRE[k >> 1], k & 1), c.x);
                    neumaier_add(lane_of(IM[k >> 1], k & 1), lane_of(CIM[k >> 1], k & 1), v.y);
                    neumaier_add(lane_of(IM[k >> 1], k & 1), lane_of(CIM[k >> 1], k & 1), c.y);
                }
            }
        }
    }
    cluster.sync();
}

// Source range [r c, (r + 1) c) of rank r of S, c = ceil(n / S).
__device__ __forceinline__ void rank_sources(int64_t n, int64_t& s_lo, int64_t& s_hi) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int64_t S = cluster.num_blocks(), rank = cluster.block_rank();
    const int64_t chunk = (n + S - 1) / S;
    s_lo = rank * chunk < n ? rank * chunk : n;
    s_hi = s_lo + chunk < n ? s_lo + chunk : n;
}

// Small launches: a cluster of S blocks per point tile, block rank r summing its share of the
// sources (rank_sources); rank 0 combines the partial sums (cluster_combine) and stores.
template <int ST, int SUM, bool GRID, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_split_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                       const float* __restrict__ pts, int64_t m, int field,
                       void* __restrict__ out) {
    namespace cg = cooperative_groups;
    __shared__ SmemTile sm;
    constexpr int kPPT = 2 * PAIRS;
    GTable& gt = dynamic_gtab();
    load_theta_table(sm, c_dir_table);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    const unsigned S = cg::this_cluster().num_blocks();
    const int64_t first = static_cast<int64_t>(blockIdx.x / S) * (kThreads * kPPT);
    int64_t s_lo, s_hi;
    rank_sources(n, s_lo, s_hi);
    float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
    block_accumulate<ST, SUM, PAIRS>(sm, gt, src, n, s_lo, s_hi, GRID, g, pts, m, first, RE, IM,
                                     CRE, CIM);
    cluster_combine<SUM, PAIRS>(sm, RE, IM, CRE, CIM);
    if (cg::this_cluster().block_rank() == 0)
        block_store<SUM, PAIRS>(RE, IM, CRE, CIM, src, n, GRID, g, pts, first, m, field,
                                out);
}

// Mid-size grids: the rows tiling with every tile's sources split over a cluster of S blocks,
// S chosen so that the launch fills whole waves (split_width); rank 0 combines and stores.
template <int ST, int SUM, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_rows_split_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                            int tx_log2, int64_t tiles0, int64_t tiles1, int field,
                            void* __restrict__ out) {
    namespace cg = cooperative_groups;
    __shared__ RowsSmem rs;
    SmemTile& sm = rs.sm;
    RowsTable& rt = rs.rt;
    load_theta_table(sm, c_dir_table);
    load_rows_table(rt);
    const int64_t tile = blockIdx.x / cg::this_cluster().num_blocks();
    int64_t s_lo, s_hi;
    rank_sources(n, s_lo, s_hi);
    float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
    rows_accumulate<ST, SUM, PAIRS>(sm, rt, src, n, s_lo, s_hi, g, tx_log2, tiles0, tiles1, tile,
                                    RE, IM, CRE, CIM);
    cluster_combine<SUM, PAIRS>(sm, RE, IM, CRE, CIM);
    if (cg::this_cluster().block_rank() == 0)
        rows_store<SUM, PAIRS>(src, n, g, tx_log2, tiles0, tiles1, tile, RE, IM, CRE, CIM,
                               field, out);
}

// Grids with more than one point along their second axis: tiles of TX = 1 << tx_log2 first-axis
// indices by (kThreads / TX) * 2 * PAIRS second-axis indices, one plane each (field_rows.cuh).
template <int ST, int SUM, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_rows_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g, int tx_log2,
                      int64_t tiles0, int64_t tiles1, int field, void* __restrict__ out) {
    __shared__ RowsSmem rs;
    SmemTile& sm = rs.sm;
    RowsTable& rt = rs.rt;
    load_theta_table(sm, c_dir_table);
    load_rows_table(rt);
    block_rows<ST, SUM, PAIRS>(sm, rt, src, n, g, tx_log2, tiles0, tiles1, blockIdx.x, field, out);
}

__global__ void pack_sources_kernel(int st, const float* __restrict__ raw,
                                    const float* __restrict__ k, const float* __restrict__ atten,
                                    int64_t n, PackedSource* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    out[j] = pack_source(st, raw, k, atten, j);
}

// SM count per device (0: not queried yet); devices past the cache are queried every time.
constexpr int kSmCacheDevices = 64;
constexpr int kFallbackSms = 148;
std::atomic<int> g_num_sms[kSmCacheDevices] = {};

// Cluster split of small launches: at most the portable cluster size, each block summing at
// least kSplitMinSources sources.
constexpr int64_t kMaxClusterBlocks = 8;
constexpr int64_t kSplitMinSources = 64;

// Blocks of Kernel that can be resident at once: launched alone (S = 1) or in clusters of S
// blocks, where the occupancy calculator's count of co-resident clusters also sees how clusters
// pack into the GPCs (7-block clusters, for one, leave some slots of every GPC empty).  Cached
// per device and S; 2 blocks per SM if the query fails.
template <auto Kernel>
int64_t resident_blocks(int64_t S, int dyn) {
    static std::atomic<int> cache[kSmCacheDevices][kMaxClusterBlocks + 1];
    if (S < 1 || S > kMaxClusterBlocks) return 2LL * num_sms();
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = kSmCacheDevices;
    if (dev < kSmCacheDevices) {
        const int v = cache[dev][S].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int64_t v = 0;
    if (allow_dynamic_smem<Kernel>(dyn) == cudaSuccess) {
        if (S == 1) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, Kernel, kThreads, dyn) ==
                cudaSuccess)
                v = static_cast<int64_t>(b) * num_sms();
        } else {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(static_cast<unsigned>(S), 1, 1);
            cfg.blockDim = dim3(kThreads, 1, 1);
            cfg.dynamicSmemBytes = static_cast<size_t>(dyn);
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = static_cast<unsigned>(S);
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int c = 0;
            if (cudaOccupancyMaxActiveClusters(&c, Kernel, &cfg) == cudaSuccess)
                v = static_cast<int64_t>(c) * S;
        }
    }
    if (v <= 0) {
        (void)cudaGetLastError();  // a failed query must not surface as the next launch's error
        return 2LL * num_sms();
    }
    if (dev < kSmCacheDevices) cache[dev][S].store(static_cast<int>(v), std::memory_order_relaxed);
    return v;
}

// Cluster width for a launch of `blocks` point tiles over n sources, slots(S) being the blocks
// resident at once in clusters of S: 1 when the launch fills its last wave to 93 % or more
// (large launches), else the S <= 8 (each rank keeping >= kSplitMinSources sources) whose
// blocks * S best fill whole waves, each extra rank charged 1 % for its set-up and the combine.
template <class Slots>
int64_t split_width(int64_t blocks, int64_t n, Slots slots) {
    auto fill = [](int64_t b, int64_t sl) {
        const int64_t waves = (b + sl - 1) / sl;
        return static_cast<double>(b) / static_cast<double>(waves * sl);
    };
    if (blocks <= 0) return 1;
    double best_score = fill(blocks, slots(1));
    if (best_score >= 0.93) return 1;
    int64_t best = 1;
    for (int64_t S = 2; S <= kMaxClusterBlocks && n / S >= kSplitMinSources; ++S) {
        const double score = fill(blocks * S, slots(S)) - 0.01 * static_cast<double>(S - 1);
        if (score > best_score + 1e-9) {
            best = S;
            best_score = score;
        }
    }
    return best;
}

// Dynamic shared memory of a general-body kernel for source type ST.
template <int ST>
constexpr int gtab_bytes() {
    return ST == SRC_T4010A1 ? kGTableBytes : 0;
}

template <int ST, int SUM, int PAIRS>
cudaError_t launch_pairs(const PackedSource* src, int64_t n, const PointSet& ps, int field,
                         void* out, cudaStream_t s) {
    constexpr int kDyn = gtab_bytes<ST>();
    const int64_t per_block = static_cast<int64_t>(kThreads) * 2 * PAIRS;
    const int64_t flat_blocks = (ps.m + per_block - 1) / per_block;
    const RowsTiling rows = ps.is_grid ? rows_tiling(ps.grid, ps.m, PAIRS) : RowsTiling{};
    if (!rows.use) {
        // flat numbering whose blocks would leave the last wave short (or the GPU part empty):
        // split each tile's sources over a cluster
        const int64_t S = split_width(flat_blocks, n, [](int64_t w) {
            return w <= 1 ? resident_blocks<field_direct_kernel<ST, SUM, false, PAIRS>>(1, kDyn)
                          : resident_blocks<field_split_kernel<ST, SUM, false, PAIRS>>(w, kDyn);
        });
        if (S >= 2 && flat_blocks * S <= 0x7fffffffLL) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(static_cast<unsigned>(flat_blocks * S), 1, 1);
            cfg.blockDim = dim3(kThreads, 1, 1);
            cfg.dynamicSmemBytes = kDyn;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = static_cast<unsigned>(S);
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            cudaError_t e;
            if (ps.is_grid) {
                e = allow_dynamic_smem<field_split_kernel<ST, SUM, true, PAIRS>>(kDyn);
                if (e == cudaSuccess)
                    e = cudaLaunchKernelEx(&cfg, field_split_kernel<ST, SUM, true, PAIRS>, src, n,
                                           ps.grid, static_cast<const float*>(nullptr), ps.m,
                                           field, out);
            } else {
                e = allow_dynamic_smem<field_split_kernel<ST, SUM, false, PAIRS>>(kDyn);
                if (e == cudaSuccess)
                    e = cudaLaunchKernelEx(&cfg, field_split_kernel<ST, SUM, false, PAIRS>, src, n,
                                           ps.grid, ps.pts, ps.m, field, out);
            }
            count_launch();
            return e != cudaSuccess ? e : cudaGetLastError();
        }
    }
    if (ps.is_grid) {
        const RowsTiling& t = rows;
        if (t.use) {
            if (t.blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
            const int64_t S = split_width(t.blocks, n, [](int64_t w) {
                return w <= 1 ? resident_blocks<field_rows_kernel<ST, SUM, PAIRS>>(1, 0)
                              : resident_blocks<field_rows_split_kernel<ST, SUM, PAIRS>>(w, 0);
            });
            if (S >= 2 && t.blocks * S <= 0x7fffffffLL) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(static_cast<unsigned>(t.blocks * S), 1, 1);
                cfg.blockDim = dim3(kThreads, 1, 1);
                cfg.dynamicSmemBytes = 0;
                cfg.stream = s;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = static_cast<unsigned>(S);
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                const cudaError_t e =
                    cudaLaunchKernelEx(&cfg, field_rows_split_kernel<ST, SUM, PAIRS>, src, n,
                                       ps.grid, t.tx_log2, t.tiles0, t.tiles1, field, out);
                count_launch();
                return e != cudaSuccess ? e : cudaGetLastError();
            }
            field_rows_kernel<ST, SUM, PAIRS><<<static_cast<unsigned>(t.blocks), kThreads, 0, s>>>(
                src, n, ps.grid, t.tx_log2, t.tiles0, t.tiles1, field, out);
            count_launch();
            return cudaGetLastError();
        }
    }
    const int64_t blocks = flat_blocks;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    cudaError_t e;
    if (ps.is_grid) {
        if ((e = allow_dynamic_smem<field_direct_kernel<ST, SUM, true, PAIRS>>(kDyn)) != cudaSuccess)
            return e;
        field_direct_kernel<ST, SUM, true, PAIRS><<<static_cast<unsigned>(blocks), kThreads, kDyn, s>>>(
            src, n, ps.grid, nullptr, ps.m, field, out);
    } else {
        if ((e = allow_dynamic_smem<field_direct_kernel<ST, SUM, false, PAIRS>>(kDyn)) != cudaSuccess)
            return e;
        field_direct_kernel<ST, SUM, false, PAIRS><<<static_cast<unsigned>(blocks), kThreads, kDyn, s>>>(
            src, n, ps.grid, ps.pts, ps.m, field, out);
    }
    count_launch();
    return cudaGetLastError();
}

// Points per thread, the cluster split refilling the waves.  Grids with more than one point
// along their second axis, whose rows body shares two coordinates per thread: 4 point pairs
// from 131,072 points and 2 from 32,768 (40^3, 64^3 and 80^3 grids ran 4-9 % faster than with
// fewer pairs).  Scatter points and single-row grids: 4 point pairs from 32,768 points, one
// below (3,984 sources: 65,536 points ran 24 % and 262,144 points 2 % faster with 4 pairs
// than with one; 16,384 points ran 40 % slower with 2 pairs than with one, its 16 tiles too
// few even split 8 ways).
template <int ST>
cudaError_t launch_st(int sum_mode, const PackedSource* src, int64_t n, const PointSet& ps,
                      int field, void* out, cudaStream_t s) {
    if (sum_mode == SUM_COMPENSATED)
        return launch_pairs<ST, SUM_COMPENSATED, 2>(src, n, ps, field, out, s);
    const bool rows_grid = ps.is_grid && ps.grid.count[1] > 1;  // the rows body can take it
    const int64_t four_from = rows_grid ? 131072 : 32768;
    const int64_t two_from = rows_grid ? 32768 : INT64_MAX;
    if (ps.m >= four_from) return launch_pairs<ST, SUM_PLAIN, 4>(src, n, ps, field, out, s);
    if (ps.m >= two_from) return launch_pairs<ST, SUM_PLAIN, 2>(src, n, ps, field, out, s);
    return launch_pairs<ST, SUM_PLAIN, 1>(src, n, ps, field, out, s);
}

}  // namespace

std::atomic<uint64_t> g_launches{0};

RowsTiling rows_tiling(const GridDev& g, int64_t m, int pairs) {
    RowsTiling t{false, 5, 0, 0, 0, 0};
    if (g.count[1] <= 1 || m <= 0) return t;
    // first-axis tile: the smallest power of two >= count[0], between 32 and kThreads
    while (t.tx_log2 < 8 && (1LL << t.tx_log2) < g.count[0]) ++t.tx_log2;
    t.rows = (static_cast<int64_t>(kThreads) >> t.tx_log2) * 2 * pairs;
    t.tiles0 = (g.count[0] + (1LL << t.tx_log2) - 1) >> t.tx_log2;
    t.tiles1 = (g.count[1] + t.rows - 1) / t.rows;
    t.blocks = t.tiles0 * t.tiles1 * g.count[2];
    // the tiles leave the threads past the grid's edges idle: take them only while they keep
    // at least 90 % as many threads busy as the flat numbering does
    const int64_t per_block = static_cast<int64_t>(kThreads) * 2 * pairs;
    const int64_t flat_blocks = (m + per_block - 1) / per_block;
    t.use = 10 * flat_blocks >= 9 * t.blocks;
    return t;
}


int num_sms() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return kFallbackSms;
    if (dev < kSmCacheDevices) {
        v = g_num_sms[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
        return kFallbackSms;
    if (dev < kSmCacheDevices) g_num_sms[dev].store(v, std::memory_order_relaxed);
    return v;
}

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
    if (field < FIELD_PRESSURE || field > FIELD_COMPLEX) return cudaErrorInvalidValue;
    if (st == SRC_T4010A1) return launch_st<SRC_T4010A1>(sum_mode, src, n, ps, field, out, s);
    if (st == SRC_SPHERE) return launch_st<SRC_SPHERE>(sum_mode, src, n, ps, field, out, s);
    return cudaErrorInvalidValue;
}

}  // namespace afc
