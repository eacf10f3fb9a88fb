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
//   * Launches whose tiles would leave the last wave short either split each point tile's
//     sources over the blocks of a thread-block cluster (field_split_kernel,
//     field_rows_split_kernel): rank r sums its share of the sources, and rank 0 adds the
//     others' partial sums, read from their shared memory, in rank order -- deterministic, no
//     workspace; or, with scratch for partial sums, run the chunked launch (field_chunk_kernel,
//     field_rows_chunk_kernel): persistent blocks over contiguous ranges of the (tile, source)
//     pairs, whose partial sums a second launch adds in source order.  A cost model
//     (direct_cost, split_cost, chunk_cost) picks among the single pass, the split and the
//     chunked launch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

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

// The field kernels run as programmatic dependents of the launch before them on the stream (the
// source packing, normally): they fill their tables first and call pdl_wait before they read a
// source.

template <int ST, int SUM, bool GRID, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_direct_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                        const float* __restrict__ pts, int64_t m, int field,
                        void* __restrict__ out) {
    __shared__ SmemTile sm;
    GTable& gt = dynamic_gtab();
    load_theta_table(sm, c_dir_table);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    pdl_wait();
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
    pdl_wait();
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

// Work split of a chunked launch: `items` = tiles x chunks items in tile-major order (item
// t * chunks + c: point tile t against source chunk c); block b of G takes the contiguous items
// [start(b), start(b + 1)), `base` = items / G each and one more for the first `rem` blocks.
struct ChunkSplit {
    int64_t tiles, chunks, chunk;  // chunk: sources per chunk (the last one shorter)
    int64_t base, rem;
    // block that takes item i
    __device__ __forceinline__ int64_t block_of(int64_t i) const {
        const int64_t big = rem * (base + 1);
        return i < big ? i / (base + 1) : rem + (i - big) / base;
    }
    __device__ __forceinline__ int64_t start(int64_t b) const {
        return b * base + (b < rem ? b : rem);
    }
};

// The point tile of point q: blocks of tile_points consecutive points (flat numbering), or the
// rows tiling's tiles (tx_log2 > 0: 1 << tx_log2 first-axis indices by `rows` second-axis
// indices of one plane, numbered as rows_accumulate numbers them).
struct TileMap {
    int tx_log2;
    int64_t tile_points;
    int64_t rows, tiles0, tiles1, c0, c1;
    __device__ __forceinline__ int64_t tile_of(int64_t q) const {
        if (tx_log2 == 0) return q / tile_points;
        const int64_t i0 = q % c0, rest = q / c0;
        const int64_t i1 = rest % c1, i2 = rest / c1;
        return (i0 >> tx_log2) + tiles0 * (i1 / rows + tiles1 * i2);
    }
};

// Persistent chunked launch of the general body for launches whose point tiles alone would
// leave the last wave short.  A block's items of one tile are consecutive chunks, i.e. one
// source range: a segment, summed by one block_accumulate pass.  A tile's segments are
// numbered in chunk order (segment k of tile t begins where the k-th block after the tile's
// first item's block begins), and segment k writes its sums at the tile's points to
// partial[k * m + point]; field_chunk_combine_kernel adds them in that order.  The blocks'
// loads differ by one chunk at most.  Each block fills its directivity tables once.
template <int ST, bool GRID, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_chunk_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                       const float* __restrict__ pts, int64_t m, ChunkSplit cs,
                       float2* __restrict__ partial) {
    constexpr int kPPT = 2 * PAIRS;
    __shared__ SmemTile sm;
    GTable& gt = dynamic_gtab();
    load_theta_table(sm, c_dir_table);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    pdl_wait();
    pdl_release();  // the combine launch may be scheduled now; it waits for this grid's end
    const int64_t end = cs.start(blockIdx.x + 1);
    for (int64_t it = cs.start(blockIdx.x); it < end;) {
        const int64_t tile = it / cs.chunks;
        const int64_t tile_end = (tile + 1) * cs.chunks;
        const int64_t seg_end = end < tile_end ? end : tile_end;
        const int64_t c0 = it - tile * cs.chunks, c1 = seg_end - tile * cs.chunks;
        const int64_t lo = c0 * cs.chunk < n ? c0 * cs.chunk : n;
        const int64_t hi = c1 * cs.chunk < n ? c1 * cs.chunk : n;
        const int64_t k = cs.block_of(it) - cs.block_of(tile * cs.chunks);
        const int64_t first = tile * (kThreads * kPPT);
        float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
        block_accumulate<ST, SUM_PLAIN, PAIRS>(sm, gt, src, n, lo, hi, GRID, g, pts, m, first, RE,
                                               IM, CRE, CIM);
        float2* part = partial + k * m;
#pragma unroll
        for (int j = 0; j < kPPT; ++j) {
            const int64_t q = first + threadIdx.x + static_cast<int64_t>(j) * kThreads;
            if (q >= m) break;
            part[q] = make_float2(lane_of(RE[j >> 1], j & 1), lane_of(IM[j >> 1], j & 1));
        }
        it = seg_end;
    }
}

// The same over the rows tiling's tiles (rows_accumulate): a segment writes its sums at its
// tile's grid points.
template <int ST, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    field_rows_chunk_kernel(const PackedSource* __restrict__ src, int64_t n, GridDev g,
                            int tx_log2, int64_t tiles0, int64_t tiles1, int64_t m, ChunkSplit cs,
                            float2* __restrict__ partial) {
    constexpr int kPPT = 2 * PAIRS;
    __shared__ RowsSmem rs;
    SmemTile& sm = rs.sm;
    RowsTable& rt = rs.rt;
    load_theta_table(sm, c_dir_table);
    load_rows_table(rt);
    pdl_wait();
    pdl_release();
    const int tx = threadIdx.x & ((1 << tx_log2) - 1);
    const int ty = threadIdx.x >> tx_log2;
    const int64_t c0 = g.count[0], c1 = g.count[1];
    const int64_t end = cs.start(blockIdx.x + 1);
    for (int64_t it = cs.start(blockIdx.x); it < end;) {
        const int64_t tile = it / cs.chunks;
        const int64_t tile_end = (tile + 1) * cs.chunks;
        const int64_t seg_end = end < tile_end ? end : tile_end;
        const int64_t ca = it - tile * cs.chunks, cb = seg_end - tile * cs.chunks;
        const int64_t lo = ca * cs.chunk < n ? ca * cs.chunk : n;
        const int64_t hi = cb * cs.chunk < n ? cb * cs.chunk : n;
        const int64_t k = cs.block_of(it) - cs.block_of(tile * cs.chunks);
        float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
        rows_accumulate<ST, SUM_PLAIN, PAIRS>(sm, rt, src, n, lo, hi, g, tx_log2, tiles0, tiles1,
                                              tile, RE, IM, CRE, CIM);
        const int64_t t0 = tile % tiles0, rest = tile / tiles0;
        const int64_t t1 = rest % tiles1, i2 = rest / tiles1;
        const int64_t i0 = (t0 << tx_log2) + tx;
        const int64_t i1b = (t1 * (kThreads >> tx_log2) + ty) * kPPT;
        if (i0 < c0) {
            float2* part = partial + k * m;
#pragma unroll
            for (int j = 0; j < kPPT; ++j) {
                const int64_t i1 = i1b + j;
                if (i1 >= c1) break;
                part[(i2 * c1 + i1) * c0 + i0] =
                    make_float2(lane_of(RE[j >> 1], j & 1), lane_of(IM[j >> 1], j & 1));
            }
        }
        it = seg_end;
    }
}

// The fields of a chunked launch: each point's segment sums added in segment order, the field
// transform, and the coincident-source fix-up of the single-pass kernels for NaN sums.
template <bool GRID>
__global__ void __launch_bounds__(256)
    field_chunk_combine_kernel(const float2* __restrict__ partial, ChunkSplit cs, TileMap tm,
                               const PackedSource* __restrict__ src, int64_t n, GridDev g,
                               const float* __restrict__ pts, int64_t m, int field,
                               void* __restrict__ out) {
    // launched as a programmatic dependent of the chunk kernel: its partial sums are complete
    // and visible once this returns
    pdl_wait();
    for (int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < m;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t t0 = tm.tile_of(q) * cs.chunks;
        const int64_t segs = cs.block_of(t0 + cs.chunks - 1) - cs.block_of(t0) + 1;
        float re = 0.f, im = 0.f;
        for (int64_t k = 0; k < segs; ++k) {
            const float2 v = partial[k * m + q];
            re = __fadd_rn(re, v.x);
            im = __fadd_rn(im, v.y);
        }
        store_field(out, q, field, re, im);
        if (isnan(re) || isnan(im)) {
            float x, y, z;
            if (GRID) {
                grid_point(g, q, x, y, z);
            } else {
                x = pts[3 * q];
                y = pts[3 * q + 1];
                z = pts[3 * q + 2];
            }
            fix_coincident(src, n, x, y, z, q, field, out);
        }
    }
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
    pdl_wait();
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
    pdl_wait();
    block_rows<ST, SUM, PAIRS>(sm, rt, src, n, g, tx_log2, tiles0, tiles1, blockIdx.x, field, out);
}

__global__ void pack_sources_kernel(int st, const float* __restrict__ raw,
                                    const float* __restrict__ k, const float* __restrict__ atten,
                                    int64_t n, PackedSource* __restrict__ out) {
    // the launch after this one (a field kernel or the G build) may start its table fills now;
    // it waits for this grid before it reads a source
    pdl_release();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    out[j] = pack_source(st, raw, k, atten, j);
}

// SM count per device (0: not queried yet); devices past the cache are queried every time.
constexpr int kSmCacheDevices = 64;
constexpr int kFallbackSms = 148;
std::atomic<int> g_num_sms[kSmCacheDevices] = {};

// Cluster split of small launches: at most the portable cluster size, each block summing at
// least kSplitMinSources sources (the 249-source single focus on a 101 x 101 grid: 26 tiles
// split 7 ways, 21 us per launch, against 27 us at the 3 ways that 64 allowed).
constexpr int64_t kMaxClusterBlocks = 8;
constexpr int64_t kSplitMinSources = 32;

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

// Launches a field kernel on `grid` blocks of kThreads with `dyn` bytes of dynamic shared memory
// on s: in clusters of `cluster` blocks when that is above one, and with `pdl` as a programmatic
// dependent of the launch before it (the kernel fills its tables, then waits in pdl_wait).
template <typename... KArgs, typename... Args>
cudaError_t launch_field_kernel(void (*kernel)(KArgs...), int64_t grid, int dyn, cudaStream_t s,
                                unsigned cluster, bool pdl, Args... args) {
    cudaLaunchAttribute attr[2];
    unsigned na = 0;
    if (cluster > 1) {
        attr[na].id = cudaLaunchAttributeClusterDimension;
        attr[na].val.clusterDim.x = cluster;
        attr[na].val.clusterDim.y = 1;
        attr[na].val.clusterDim.z = 1;
        ++na;
    }
    if (pdl) {
        attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid), 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = static_cast<size_t>(dyn);
    cfg.stream = s;
    cfg.attrs = na ? attr : nullptr;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Chunked launches (field_chunk_kernel): chunks of kChunkSources sources (one: the blocks'
// loads differ by one source iteration at most; a block's consecutive chunks of a tile are one
// pass whatever their size), partial sums of at most kChunkMaxBytes.
constexpr int64_t kChunkSources = 1;
constexpr int64_t kChunkMaxBytes = 256LL << 20;

// Modelled time of a launch's options over `tiles` point tiles of n sources each, in source
// iterations of one block (about 0.67 us at 4 point pairs per thread on a GB300).  Calibrated on
// 3,984 sources and 65,536 to 4,194,304 scatter points: a pass of 2,048 points over 210 sources
// took 148.5 us against 140.6 us of source iterations, so the set-up of a pass over a source
// range (its points, their bounding box, the partial staging tile, the store) costs about 11
// iterations, and a chunked launch about 20 us more than its passes (the combine launch, the
// drain).
// Its source iterations ran 2.5 % slower than the single-pass kernel's at full waves (4,194,304
// points: 0.688 against 0.671 us; the 256^3 grid through the rows form: 66.2 against 64.6 ms).
// A single pass of several waves loses less to its short last wave than the wave count says
// (that wave's blocks share their SMs with fewer others and run faster: 4,194,304 scatter
// points in 6.7 waves took 3.5 % less than modelled), so against it the chunked launch must
// model kMultiWaveMargin cheaper.  The general body's cluster split gains the same way (a 96^3
// grid on the flat numbering: split in 2.8 waves 3.9 % faster than the chunked launch the model
// preferred by 2.7 %), the rows body's did not (128^3 in 6.7 split waves: split and chunked
// within 1 % of their modelled times, the chunked launch 2.7 % faster), so there the margin
// applies against the single pass only.
constexpr double kPassSetup = 11.0;
constexpr double kChunkFixedUs = 20.0;
constexpr double kChunkIterationUs = 0.688;
constexpr double kChunkSlowdown = 1.025;
constexpr double kMultiWaveMargin = 0.97;

// the cost the chunked launch must beat: `cost` of a launch of `blocks` blocks on `slots`
// resident ones, less kMultiWaveMargin when that launch runs two or more waves and `margin`
double chunk_bar(double cost, int64_t blocks, int64_t slots, bool margin) {
    return (margin && (blocks + slots - 1) / slots >= 2) ? kMultiWaveMargin * cost : cost;
}

// one pass per tile (field_direct_kernel) on `slots` resident blocks
double direct_cost(int64_t tiles, int64_t n, int64_t slots) {
    const int64_t waves = (tiles + slots - 1) / slots;
    return static_cast<double>(waves) * (static_cast<double>(n) + kPassSetup);
}

// S blocks per tile in clusters (field_split_kernel) on `slots` resident blocks of S-clusters
double split_cost(int64_t tiles, int64_t n, int64_t S, int64_t slots) {
    const int64_t waves = (tiles * S + slots - 1) / slots;
    return static_cast<double>(waves) *
           (static_cast<double>((n + S - 1) / S) + kPassSetup + 2.0);
}

// the chunked launch on `blocks` persistent blocks: the largest block's chunks, up to two
// passes, the fixed cost, at the chunked kernel's iteration rate
double chunk_cost(int64_t tiles, int64_t n, int64_t blocks) {
    const int64_t chunks = (n + kChunkSources - 1) / kChunkSources;
    const int64_t per = (tiles * chunks + blocks - 1) / blocks;
    return kChunkSlowdown * (static_cast<double>(per * kChunkSources) + 2.0 * kPassSetup) +
           kChunkFixedUs / kChunkIterationUs;
}

// The work split of a chunked launch of `tiles` tiles and n sources on `blocks` blocks, and the
// partial-sum slots it needs per point (the most segments any tile has).
ChunkSplit chunk_split(int64_t tiles, int64_t n, int64_t blocks, int64_t* slots_per_point) {
    ChunkSplit cs{};
    cs.tiles = tiles;
    cs.chunks = (n + kChunkSources - 1) / kChunkSources;
    cs.chunk = kChunkSources;
    const int64_t items = tiles * cs.chunks;
    if (blocks > items) blocks = items;
    cs.base = items / blocks;
    cs.rem = items % blocks;
    // a tile's chunks - 1 item boundaries after its first item start at most
    // ceil((chunks - 1) / base) more blocks
    *slots_per_point = cs.base > 0 ? (cs.chunks - 1 + cs.base - 1) / cs.base + 1 : cs.chunks;
    return cs;
}

// Per-device pool of the chunked launches' partial sums: stream-ordered allocations that keep
// up to kChunkMaxBytes after they are freed, so that repeated calls do not return memory to the
// driver and take it again.
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kSmCacheDevices] = {};

cudaError_t scratch_alloc(void** ptr, size_t bytes, cudaStream_t s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kSmCacheDevices) return cudaErrorMemoryAllocation;
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pool_mu);
        if (!g_pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
            uint64_t keep = static_cast<uint64_t>(kChunkMaxBytes);
            if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) !=
                cudaSuccess) {
                cudaMemPoolDestroy(pool);
                return e;
            }
            g_pools[dev] = pool;
        }
        pool = g_pools[dev];
    }
    return cudaMallocFromPoolAsync(ptr, bytes, pool, s);
}

// Dynamic shared memory of a general-body kernel for source type ST.
template <int ST>
constexpr int gtab_bytes() {
    return ST == SRC_T4010A1 ? kGTableBytes : 0;
}

// A chunked launch of the general body (field_chunk_kernel + field_chunk_combine_kernel) on
// `blocks` persistent blocks.  cudaErrorMemoryAllocation: no scratch for the partial sums
// (nothing was launched).
template <int ST, bool GRID, int PAIRS>
cudaError_t launch_chunked(const PackedSource* src, int64_t n, const PointSet& ps, int field,
                           void* out, cudaStream_t s, int64_t tiles, int64_t blocks, bool pdl,
                           const RowsTiling* rows = nullptr) {
    constexpr int kDyn = gtab_bytes<ST>();
    int64_t slots = 0;
    const ChunkSplit cs = chunk_split(tiles, n, blocks, &slots);
    const size_t bytes = sizeof(float2) * static_cast<size_t>(slots) * static_cast<size_t>(ps.m);
    if (static_cast<int64_t>(bytes) > kChunkMaxBytes) return cudaErrorMemoryAllocation;
    void* partial = nullptr;
    if (scratch_alloc(&partial, bytes, s) != cudaSuccess) {
        (void)cudaGetLastError();
        return cudaErrorMemoryAllocation;
    }
    const int64_t items = tiles * cs.chunks;
    const unsigned grid_blocks = static_cast<unsigned>(blocks < items ? blocks : items);
    TileMap tm{0, static_cast<int64_t>(kThreads) * 2 * PAIRS, 0, 0, 0, 0, 0};
    cudaError_t e = cudaSuccess;
    if (rows) {
        tm = TileMap{rows->tx_log2, 0, rows->rows, rows->tiles0, rows->tiles1,
                     static_cast<int64_t>(ps.grid.count[0]), static_cast<int64_t>(ps.grid.count[1])};
        e = launch_field_kernel(field_rows_chunk_kernel<ST, PAIRS>, grid_blocks, 0, s, 1, pdl, src, n,
                                ps.grid, rows->tx_log2, rows->tiles0, rows->tiles1, ps.m, cs,
                                static_cast<float2*>(partial));
        count_launch();
        if (e == cudaSuccess) e = cudaGetLastError();
    } else if ((e = allow_dynamic_smem<field_chunk_kernel<ST, GRID, PAIRS>>(kDyn)) == cudaSuccess) {
        e = launch_field_kernel(field_chunk_kernel<ST, GRID, PAIRS>, grid_blocks, kDyn, s, 1, pdl,
                                src, n, ps.grid, ps.pts, ps.m, cs, static_cast<float2*>(partial));
        count_launch();
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        // a programmatic dependent of the chunk kernel: its launch overlaps that grid's tail
        const int64_t want = (ps.m + 255) / 256, cap = 8LL * num_sms();
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(static_cast<unsigned>(want < cap ? want : cap));
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, field_chunk_combine_kernel<GRID>,
                               static_cast<const float2*>(partial), cs, tm, src, n, ps.grid,
                               ps.pts, ps.m, field, out);
        count_launch();
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(partial, s);
    return e != cudaSuccess ? e : ef;
}

// `capturing`: s is being captured into a graph, which takes neither the chunked launch nor
// programmatic dependences.
template <int ST, int SUM, int PAIRS>
cudaError_t launch_pairs(const PackedSource* src, int64_t n, const PointSet& ps, int field,
                         void* out, cudaStream_t s, bool scratch_ok, bool capturing) {
    constexpr int kDyn = gtab_bytes<ST>();
    const bool pdl = !capturing;
    const int64_t per_block = static_cast<int64_t>(kThreads) * 2 * PAIRS;
    const int64_t flat_blocks = (ps.m + per_block - 1) / per_block;
    const RowsTiling rows = ps.is_grid ? rows_tiling(ps.grid, ps.m, PAIRS) : RowsTiling{};
    // the chunked launch numbers tiles x sources work items in 64 bits: only below 2^62 of them
    const bool chunk_fits = n < (1LL << 31) && flat_blocks < (1LL << 31);
    if constexpr (PAIRS == 4 && SUM == SUM_PLAIN) if (!rows.use && scratch_ok && chunk_fits && n >= 2 * kChunkSources) {
        // chunked (not while the stream is being captured: the partial sums are allocated on
        // the stream) when the model puts it below the single pass and the cluster split
        if (!capturing) {
            const int64_t slots1 = resident_blocks<field_direct_kernel<ST, SUM, false, PAIRS>>(1, kDyn);
            double other = direct_cost(flat_blocks, n, slots1);
            double bar = chunk_bar(other, flat_blocks, slots1, true);
            for (int64_t S = 2; S <= kMaxClusterBlocks && n / S >= kSplitMinSources; ++S) {
                const int64_t slots = resident_blocks<field_split_kernel<ST, SUM, false, PAIRS>>(S, kDyn);
                const double c = split_cost(flat_blocks, n, S, slots);
                if (c < other) {
                    other = c;
                    bar = chunk_bar(c, flat_blocks * S, slots, true);
                }
            }
            const int64_t blocks =
                ps.is_grid ? resident_blocks<field_chunk_kernel<ST, true, PAIRS>>(1, kDyn)
                           : resident_blocks<field_chunk_kernel<ST, false, PAIRS>>(1, kDyn);
            if (chunk_cost(flat_blocks, n, blocks) < bar) {
                const cudaError_t e =
                    ps.is_grid ? launch_chunked<ST, true, PAIRS>(src, n, ps, field, out, s, flat_blocks, blocks, pdl)
                               : launch_chunked<ST, false, PAIRS>(src, n, ps, field, out, s, flat_blocks, blocks, pdl);
                if (e != cudaErrorMemoryAllocation) return e;
            }
        }
    }
    if (!rows.use) {
        // flat numbering whose blocks would leave the last wave short (or the GPU part empty):
        // split each tile's sources over a cluster
        const int64_t S = split_width(flat_blocks, n, [](int64_t w) {
            return w <= 1 ? resident_blocks<field_direct_kernel<ST, SUM, false, PAIRS>>(1, kDyn)
                          : resident_blocks<field_split_kernel<ST, SUM, false, PAIRS>>(w, kDyn);
        });
        if (S >= 2 && flat_blocks * S <= 0x7fffffffLL) {
            const unsigned cl = static_cast<unsigned>(S);
            cudaError_t e;
            if (ps.is_grid) {
                e = allow_dynamic_smem<field_split_kernel<ST, SUM, true, PAIRS>>(kDyn);
                if (e == cudaSuccess)
                    e = launch_field_kernel(field_split_kernel<ST, SUM, true, PAIRS>, flat_blocks * S,
                                            kDyn, s, cl, pdl, src, n, ps.grid,
                                            static_cast<const float*>(nullptr), ps.m, field, out);
            } else {
                e = allow_dynamic_smem<field_split_kernel<ST, SUM, false, PAIRS>>(kDyn);
                if (e == cudaSuccess)
                    e = launch_field_kernel(field_split_kernel<ST, SUM, false, PAIRS>, flat_blocks * S,
                                            kDyn, s, cl, pdl, src, n, ps.grid, ps.pts, ps.m, field,
                                            out);
            }
            count_launch();
            return e != cudaSuccess ? e : cudaGetLastError();
        }
    }
    if (ps.is_grid) {
        const RowsTiling& t = rows;
        if (t.use) {
            if (t.blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
            if constexpr (PAIRS == 4 && SUM == SUM_PLAIN) if (scratch_ok && chunk_fits && n >= 2 * kChunkSources) {
                // the chunked launch over the rows tiles, on the same terms as the flat one
                if (!capturing) {
                    const int64_t slots1 = resident_blocks<field_rows_kernel<ST, SUM, PAIRS>>(1, 0);
                    double other = direct_cost(t.blocks, n, slots1);
                    double bar = chunk_bar(other, t.blocks, slots1, true);
                    for (int64_t S = 2; S <= kMaxClusterBlocks && n / S >= kSplitMinSources; ++S) {
                        const int64_t slots = resident_blocks<field_rows_split_kernel<ST, SUM, PAIRS>>(S, 0);
                        const double c = split_cost(t.blocks, n, S, slots);
                        if (c < other) {
                            other = c;
                            bar = chunk_bar(c, t.blocks * S, slots, false);
                        }
                    }
                    const int64_t blocks = resident_blocks<field_rows_chunk_kernel<ST, PAIRS>>(1, 0);
                    if (chunk_cost(t.blocks, n, blocks) < bar) {
                        const cudaError_t e = launch_chunked<ST, true, PAIRS>(
                            src, n, ps, field, out, s, t.blocks, blocks, pdl, &t);
                        if (e != cudaErrorMemoryAllocation) return e;
                    }
                }
            }
            const int64_t S = split_width(t.blocks, n, [](int64_t w) {
                return w <= 1 ? resident_blocks<field_rows_kernel<ST, SUM, PAIRS>>(1, 0)
                              : resident_blocks<field_rows_split_kernel<ST, SUM, PAIRS>>(w, 0);
            });
            if (S >= 2 && t.blocks * S <= 0x7fffffffLL) {
                const cudaError_t e = launch_field_kernel(
                    field_rows_split_kernel<ST, SUM, PAIRS>, t.blocks * S, 0, s,
                    static_cast<unsigned>(S), pdl, src, n, ps.grid, t.tx_log2, t.tiles0, t.tiles1,
                    field, out);
                count_launch();
                return e != cudaSuccess ? e : cudaGetLastError();
            }
            const cudaError_t e = launch_field_kernel(field_rows_kernel<ST, SUM, PAIRS>, t.blocks, 0, s,
                                                      1, pdl, src, n, ps.grid, t.tx_log2, t.tiles0,
                                                      t.tiles1, field, out);
            count_launch();
            return e != cudaSuccess ? e : cudaGetLastError();
        }
    }
    const int64_t blocks = flat_blocks;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    cudaError_t e;
    if (ps.is_grid) {
        if ((e = allow_dynamic_smem<field_direct_kernel<ST, SUM, true, PAIRS>>(kDyn)) != cudaSuccess)
            return e;
        e = launch_field_kernel(field_direct_kernel<ST, SUM, true, PAIRS>, blocks, kDyn, s, 1, pdl,
                                src, n, ps.grid, static_cast<const float*>(nullptr), ps.m, field, out);
    } else {
        if ((e = allow_dynamic_smem<field_direct_kernel<ST, SUM, false, PAIRS>>(kDyn)) != cudaSuccess)
            return e;
        e = launch_field_kernel(field_direct_kernel<ST, SUM, false, PAIRS>, blocks, kDyn, s, 1, pdl,
                                src, n, ps.grid, ps.pts, ps.m, field, out);
    }
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

// Points per thread, the cluster split or the chunked launch refilling the waves.  Scatter
// points and single-row grids: 4 point pairs from 32,768 points, one below (3,984 sources:
// 65,536 points ran 24 % and 262,144 points 2 % faster with 4 pairs than with one; 16,384
// points ran 40 % slower with 2 pairs than with one, its 16 tiles too few even split 8 ways).
// Where the chunked launch is open, point sets from 2,048 points against at least 1,024
// sources (and 5e6 evaluations) take 4 point pairs too (below).
// Grids with more than one point along their second axis, whose rows body shares two
// coordinates per thread: 4 point pairs from 32,768 points where the chunked launch is open
// (scratch allowed, no stream capture; 3,984 sources: 40^3 and 48^3 grids ran 12 % and 6 %
// faster, 200^2, 256^2 and 360^2 slices 19-25 %), else from 131,072 points and 2 from 32,768
// (40^3, 64^3 and 80^3 grids ran 4-9 % faster than with fewer pairs under the cluster split).
template <int ST>
cudaError_t launch_st(int sum_mode, const PackedSource* src, int64_t n, const PointSet& ps,
                      int field, void* out, cudaStream_t s, bool scratch_ok) {
    const bool capturing = stream_capturing(s);
    if (sum_mode == SUM_COMPENSATED)
        return launch_pairs<ST, SUM_COMPENSATED, 2>(src, n, ps, field, out, s, false, capturing);
    const bool chunk_open = scratch_ok && !capturing;
    const bool rows_grid = ps.is_grid && ps.grid.count[1] > 1;  // the rows body can take it
    int64_t four_from = (rows_grid && !chunk_open) ? 131072 : 32768;
    // small point sets against many sources: the split's S <= 8 ranks leave most SMs idle, the
    // chunked launch spreads the sources over all of them (3,984 sources: 2,048 to 24,576
    // scatter points ran 1.2-2.4x faster, 100^2 and 150^2 slices 1.5x and 1.2x); below about
    // 5e6 evaluations its fixed cost outweighs that (249 sources on 101^2: 21 -> 35 us)
    if (chunk_open && n >= 1024 && static_cast<double>(n) * static_cast<double>(ps.m) >= 5e6)
        four_from = 2048;
    const int64_t two_from = rows_grid ? 32768 : INT64_MAX;
    if (ps.m >= four_from)
        return launch_pairs<ST, SUM_PLAIN, 4>(src, n, ps, field, out, s, scratch_ok, capturing);
    if (ps.m >= two_from)
        return launch_pairs<ST, SUM_PLAIN, 2>(src, n, ps, field, out, s, scratch_ok, capturing);
    return launch_pairs<ST, SUM_PLAIN, 1>(src, n, ps, field, out, s, scratch_ok, capturing);
}

}  // namespace

std::atomic<uint64_t> g_launches{0};

RowsTiling rows_tiling(const GridDev& g, int64_t m, int pairs) {
    RowsTiling t{false, 5, 0, 0, 0, 0};
    if (g.count[1] <= 1 || m <= 0) return t;
    // first-axis tile: the power of two between 32 and kThreads (at most the smallest one >=
    // count[0]) whose tiles leave the fewest threads past the grid's edges; on a tie the wider
    // (a 592 x 592 slice: 19 x 32 = 608 columns of 64-row tiles, where 256 would take 768)
    int top = 5;
    while (top < 8 && (1LL << top) < g.count[0]) ++top;
    for (int k = top; k >= 5; --k) {
        const int64_t rows = (static_cast<int64_t>(kThreads) >> k) * 2 * pairs;
        const int64_t tiles0 = (g.count[0] + (1LL << k) - 1) >> k;
        const int64_t tiles1 = (g.count[1] + rows - 1) / rows;
        const int64_t blocks = tiles0 * tiles1 * g.count[2];
        if (k == top || blocks < t.blocks) {
            t.tx_log2 = k;
            t.rows = rows;
            t.tiles0 = tiles0;
            t.tiles1 = tiles1;
            t.blocks = blocks;
        }
    }
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
                         const PointSet& ps, void* out, cudaStream_t s, bool scratch_ok) {
    if (ps.m <= 0) return cudaSuccess;
    if (field < FIELD_PRESSURE || field > FIELD_COMPLEX) return cudaErrorInvalidValue;
    if (st == SRC_T4010A1) return launch_st<SRC_T4010A1>(sum_mode, src, n, ps, field, out, s, scratch_ok);
    if (st == SRC_SPHERE) return launch_st<SRC_SPHERE>(sum_mode, src, n, ps, field, out, s, scratch_ok);
    return cudaErrorInvalidValue;
}

}  // namespace afc
