// Many phase patterns on one fixed geometry: the field becomes the dense complex contraction
//     P (m points x K patterns) = G (m x n) Q (n x K),
//     G_ij = D(theta_ij) exp(-alpha_j r_ij) / r_ij exp(i k_j r_ij)   (unit amplitude, zero phase)
//     Q_jk = A_jk exp(i phi_jk)
// so that P_ik is the field of pattern k at point i (the per-pair math of
// acoustic-field-calculator/src/system/uniform_medium.rs:111-128 with the source's amplitude
// and phase factored out).  This form has no reference counterpart; it is evaluated here on the
// sm_100 tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// The complex product runs as one real GEMM C = A B^T with K = 2n (padded to 64):
//   A row i = (Re G_i0, Im G_i0, Re G_i1, ...)              (G stored as interleaved complex)
//   B^T row 2k   = (Re Q_0k, -Im Q_0k, Re Q_1k, -Im Q_1k, ...)  -> C[i][2k]   = Re P_ik
//   B^T row 2k+1 = (Im Q_0k,  Re Q_0k, Im Q_1k,  Re Q_1k, ...)  -> C[i][2k+1] = Im P_ik
// so C is P as interleaved complex, row-major.
//
// Precisions
//   split BF16: A = Ah + Al, B = Bh + Bl (hi = bf16(x), lo = bf16(x - hi)); C = Ah Bh + Ah Bl +
//     Al Bh accumulated in FP32 (the three products interleaved in each K block of one
//     accumulation), ~16 significant bits.
//   FP16 row-scaled: each row of G scaled by a power of two so that its largest entry is ~1,
//     one FP16 GEMM, the scale undone in the epilogue (exact).
//
// GEMM kernel (persistent, CTA pairs: clusters of 2 CTAs, one CTA per SM, 192 threads each):
//   an output tile is 256 x 256; CTA rank r of the pair owns rows 128 r .. 128 r + 127 of the
//   tile, loads those 128 rows of A and rows 128 r .. 128 r + 127 of the tile's 256 B^T rows,
//   and holds its 128 rows x 256 columns of the accumulator in its own tensor memory.
//   warp 0 lane 0  TMA producer (both CTAs): per 64-wide K block its A plane(s) and B^T
//                  plane(s), 128 x 64 each, 128-byte swizzle, into a shared-memory ring
//                  (split BF16: A hi, A lo, B hi, B lo = 64 KB a stage, 3 stages; FP16:
//                  32 KB, 7 stages) that runs on across tiles.  Both CTAs' copies complete on
//                  the rank-0 CTA's stage barrier.
//   warp 1         allocates 512 TMEM columns in both CTAs (two 256-column accumulators); in
//                  the rank-0 CTA lane 0 issues tcgen05.mma.cta_group::2 (M = 256, N = 256,
//                  K = 16, FP32 accumulate) -- split BF16 interleaves hi*hi, hi*lo and lo*hi
//                  within each K block, so every operand plane is read once per tile -- and
//                  frees each stage in both CTAs with one multicast tcgen05.commit.
//   warps 2-5      epilogue (both CTAs): tcgen05.ld of their 32 TMEM lanes, FP32 stores of C,
//                  overlapping the next tile's MMAs in the other accumulator.
// Per SM and K block this moves 32 (FP16) or 64 KB (split BF16) for 4 or 12 MMA steps of
// 128 x 256 x 16, two thirds (FP16) or four ninths (split BF16) of the operand bytes a 128 x 256
// single-CTA tile reads for the same work.
// Every mbarrier wait is bounded by a second of the global timer; on time-out the CTA records an
// error code, lets its copies in flight land (bounded) and frees its tensor memory, together with
// its peer, before it returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "propagate.cuh"

namespace afc {
namespace mp {

constexpr int BM = 256;    // output tile rows (a CTA pair)
constexpr int BN = 256;    // output tile columns
constexpr int BK = 64;     // 64 x 2-byte elements = one 128-byte swizzle row
constexpr int HALF = 128;  // rows of A and of B^T that one CTA of the pair loads per tile
constexpr int OP_TILE = HALF * BK * 2;  // 16 KB: 128 rows of one K block of one operand plane
constexpr int GEMM_THREADS = 192;
constexpr int TMEM_COLS = 256;

// Shared-memory ring of the GEMM: per stage kPlanes A tiles then kPlanes B^T tiles.
template <bool BF16>
struct GemmCfg {
    static constexpr int kPlanes = BF16 ? 2 : 1;  // split BF16: hi and lo
    static constexpr int kStageBytes = 2 * kPlanes * OP_TILE;
    static constexpr int kStages = BF16 ? 3 : 7;
    static constexpr int kSmemBytes = kStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;
};
static_assert(GemmCfg<true>::kSmemBytes <= 227 * 1024 && GemmCfg<false>::kSmemBytes <= 227 * 1024,
              "GEMM ring exceeds the shared memory of a CTA");
static_assert((2 * GemmCfg<false>::kStages + 5) * 8 + 8 <= 256, "GEMM barriers exceed their area");
// Every mbarrier wait gives up after kWaitNs of the global timer (a second: far beyond any stage's
// or tile's wait in a run that works; a tile's MMAs take about 0.1 ms), so that a kernel whose
// pipeline stalled returns an error code instead of hanging.  kWaitPolls backs the timer up.
constexpr uint64_t kWaitNs = 1000000000ull;
constexpr uint32_t kWaitPolls = 1u << 30;

enum : unsigned { ERR_NONE = 0, ERR_TIMEOUT_PRODUCER = 1, ERR_TIMEOUT_MMA = 2, ERR_TIMEOUT_EPILOGUE = 3 };

__constant__ float4 c_dir_table_mp[dev::kDirTableSize] = AFC_DIR_TABLE_INIT;

// ------------------------------------------------------------------ PTX wrappers

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait until the phase with the given parity has completed; false once kWaitNs have passed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    if (mbar_try(addr, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < kWaitPolls; ++i) {
        if (mbar_try(addr, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

// Shared::cluster address of the same shared-memory object in the CTA of the given cluster rank.
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Every thread of both CTAs of the cluster; orders shared and global memory across them.
__device__ __forceinline__ void cluster_sync() {
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Arrive on an mbarrier given by its shared::cluster address (this CTA's or the peer's).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar)
                 : "memory");
}

// TMA 2-D tile load into this CTA's shared memory; the transaction bytes complete on the mbarrier
// at shared::cluster address `bar`, which may lie in the peer CTA of the pair.
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar,
                                                 int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major tile in the 128-byte swizzled layout: start
// address >> 4 (bits 0-13), leading byte offset (unused for this layout, 16 B) in bits 16-29,
// stride byte offset between 8-row groups (1024 B) in bits 32-45, descriptor version 1 in bits
// 46-47, base offset 0 (tile 1024-byte aligned), swizzle mode 2 (128 B) in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(16u >> 4) << 16;
    d |= static_cast<uint64_t>(1024u >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    d |= static_cast<uint64_t>(2) << 61;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// format (bits 7-9, 10-12: 0 = F16, 1 = BF16), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t mma_idesc(bool bf16) {
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) |
           (static_cast<uint32_t>(BN >> 3) << 17) | (static_cast<uint32_t>(BM >> 4) << 24);
}

// One M = 256 step over the CTA pair: A rows 0-127 and B^T rows 0-127 from this (rank-0) CTA's
// shared memory, rows 128-255 from the same offsets in the peer's; D rows 0-127 in this CTA's
// tensor memory, rows 128-255 at the same address in the peer's.
__device__ __forceinline__ void mma_f16_pair(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                             uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Arrive once on the mbarrier at this offset in both CTAs of the pair when every tcgen05
// operation this thread issued so far has completed.
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
        " [%0], %1;" ::"r"(smem_u32(bar)),
        "h"(static_cast<uint16_t>(3))
        : "memory");
}

__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------------ GEMM

struct GemmArgs {
    int k_blocks;        // BK-blocks of the contraction (kpad / BK)
    float* c;            // M x ldc floats
    int64_t ldc;         // row stride of C in floats
    int64_t m;           // rows of C
    int n_tiles;         // BN-wide column tiles of C
    int64_t tiles;       // output tiles in all (BM-row tiles x n_tiles)
    const float* row_scale;  // nullable: C row i multiplied by row_scale[i]
    unsigned* err;       // error code (first writer wins)
    int stall;           // testing: the producer arms no stage, so that every wait runs out
};

// Persistent: CTA pair p computes output tiles p, p + pairs, ... (tile t = row tile t / n_tiles,
// column tile t % n_tiles), so the pairs running at one time share their A row tiles and B
// through L2.  The producers stream every tile's K blocks through the ring without stopping
// between tiles; the rank-0 MMA issuer accumulates tile i into TMEM accumulator i % 2 of both
// CTAs; the epilogue warps drain accumulator i % 2 while the MMAs of tile i + 1 run in the other
// one, and hand it back through the rank-0 CTA's tmem_empty barrier.
template <bool BF16>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    cgemm_tcgen05_kernel(const __grid_constant__ CUtensorMap map_a0,
                         const __grid_constant__ CUtensorMap map_a1,
                         const __grid_constant__ CUtensorMap map_b0,
                         const __grid_constant__ CUtensorMap map_b1, GemmArgs args) {
    using Cfg = GemmCfg<BF16>;
    constexpr int S = Cfg::kStages;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * Cfg::kStageBytes);  // rank 0's count
    uint64_t* empty = full + S;            // per CTA, one multicast commit per round
    uint64_t* tmem_full = empty + S;       // [2] per CTA: accumulator ready for the epilogue
    uint64_t* tmem_empty = tmem_full + 2;  // [2] rank 0's count: drained by all 8 epilogue warps
    uint64_t* done = tmem_empty + 2;       // per CTA: every MMA of the pair has finished
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* issued_slot = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();  // 0 issues the MMAs of the pair
    const int64_t first = blockIdx.x >> 1, stride = gridDim.x >> 1;

    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tmem_full[i], 1);
            mbar_init(&tmem_empty[i], 8);  // 4 epilogue warps in each CTA
        }
        mbar_init(done, 1);
        *issued_slot = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        // both CTAs' warp 1: the same 512 columns in each CTA's tensor memory
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(2 * TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    cluster_sync();  // both CTAs' barriers are initialised before any remote arrival
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;     // K blocks over all of this CTA's tiles
            int armed = 0;  // of those, the ones whose copies were issued
            bool ok = true;
            for (int64_t t = first; ok && t < args.tiles; t += stride) {
                const int a_row = static_cast<int>(t / args.n_tiles) * BM + static_cast<int>(rank) * HALF;
                const int b_row = static_cast<int>(t % args.n_tiles) * BN + static_cast<int>(rank) * HALF;
                for (int kb = 0; kb < args.k_blocks; ++kb, ++it) {
                    const int s = it % S;
                    const uint32_t ph = (it / S) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u)) {
                        atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_PRODUCER);
                        ok = false;
                        break;
                    }
                    if (args.stall) continue;
                    uint8_t* st = smem + s * Cfg::kStageBytes;
                    const uint32_t bar = cluster_addr(&full[s], 0);
                    // rank 0 arms its barrier with the bytes of both CTAs' copies
                    if (rank == 0) mbar_arrive_expect_tx(&full[s], 2 * Cfg::kStageBytes);
                    const int k = kb * BK;
                    tma_load_2d_pair(st, &map_a0, bar, k, a_row);
                    if (BF16) tma_load_2d_pair(st + OP_TILE, &map_a1, bar, k, a_row);
                    tma_load_2d_pair(st + Cfg::kPlanes * OP_TILE, &map_b0, bar, k, b_row);
                    if (BF16) tma_load_2d_pair(st + 3 * OP_TILE, &map_b1, bar, k, b_row);
                    armed = it + 1;
                }
            }
            *issued_slot = armed;
        }
    } else if (warp == 1) {
        if (rank == 0 && lane == 0) {
            constexpr uint32_t idesc = mma_idesc(BF16);
            int it = 0;
            int i = 0;  // this pair's tile count
            bool ok = true;
            for (int64_t t = first; ok && t < args.tiles; t += stride, ++i) {
                const int acc = i & 1;
                const uint32_t use = static_cast<uint32_t>(i >> 1);
                // the accumulator's previous tile must have been drained by both epilogues
                if (!mbar_wait(&tmem_empty[acc], (use & 1u) ^ 1u)) {
                    atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_MMA);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + static_cast<uint32_t>(acc * TMEM_COLS);
                for (int kb = 0; kb < args.k_blocks; ++kb, ++it) {
                    const int s = it % S;
                    const uint32_t ph = (it / S) & 1u;
                    if (!mbar_wait(&full[s], ph)) {
                        atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_MMA);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + s * Cfg::kStageBytes);
                    const uint64_t a_hi = smem_desc_sw128(sa);
                    const uint64_t b_hi = smem_desc_sw128(sa + Cfg::kPlanes * OP_TILE);
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        // K step of 16 elements = 32 bytes = 2 in the descriptor's address field
                        mma_f16_pair(d, a_hi + 2u * k, b_hi + 2u * k, idesc, (kb | k) != 0);
                        if (BF16) {
                            const uint64_t a_lo = smem_desc_sw128(sa + OP_TILE);
                            const uint64_t b_lo = smem_desc_sw128(sa + 3 * OP_TILE);
                            mma_f16_pair(d, a_hi + 2u * k, b_lo + 2u * k, idesc, 1u);
                            mma_f16_pair(d, a_lo + 2u * k, b_hi + 2u * k, idesc, 1u);
                        }
                    }
                    mma_commit_pair(&empty[s]);  // stage s free in both CTAs once these finish
                }
                if (ok) mma_commit_pair(&tmem_full[acc]);  // the tile's accumulator is complete
            }
            mma_commit_pair(done);  // completes once every MMA issued above has finished
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, i.e. rows of this CTA's half tile
        const int q = warp & 3;
        const uint32_t drained0 = cluster_addr(&tmem_empty[0], 0);
        const uint32_t drained1 = cluster_addr(&tmem_empty[1], 0);
        int i = 0;
        for (int64_t t = first; t < args.tiles; t += stride, ++i) {
            const int acc = i & 1;
            const uint32_t use = static_cast<uint32_t>(i >> 1);
            const int n_tile = static_cast<int>(t % args.n_tiles);
            const int64_t row = (t / args.n_tiles) * BM + static_cast<int64_t>(rank) * HALF + q * 32 + lane;
            // one lane waits, the warp follows converged (tcgen05.ld is warp-synchronous)
            const int ok = __shfl_sync(0xffffffffu,
                                       lane == 0 ? (mbar_wait(&tmem_full[acc], use & 1u) ? 1 : 0) : 0, 0);
            __syncwarp();
            if (!ok) {
                atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_EPILOGUE);
                break;
            }
            tc_fence_after();
            const float scale = (args.row_scale && row < args.m) ? args.row_scale[row] : 1.0f;
            const uint32_t src = tmem + static_cast<uint32_t>(acc * TMEM_COLS) +
                                 (static_cast<uint32_t>(q * 32) << 16);
#pragma unroll 1
            for (int c = 0; c < BN / 32; ++c) {
                uint32_t v[32];
                tmem_ld_32cols(src + c * 32, v);
                if (row < args.m) {
                    float4* dst = reinterpret_cast<float4*>(args.c + row * args.ldc +
                                                            static_cast<int64_t>(n_tile) * BN + c * 32);
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        dst[u] = make_float4(__uint_as_float(v[4 * u]) * scale,
                                             __uint_as_float(v[4 * u + 1]) * scale,
                                             __uint_as_float(v[4 * u + 2]) * scale,
                                             __uint_as_float(v[4 * u + 3]) * scale);
                    }
                }
            }
            // the accumulator may take the tile after next
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive_cluster(acc ? drained1 : drained0);
        }
    }
    tc_fence_before();
    __syncthreads();
    cluster_sync();  // both CTAs have issued everything and stopped waiting; errors are visible
    if (threadIdx.x == 0) {
        if (*static_cast<volatile unsigned*>(args.err) != ERR_NONE) {
            // copies may still be in flight: rank 0 waits (bounded) for the last stages armed on
            // its barriers, both CTAs then give any remaining copy time to land
            if (rank == 0) {
                const int issued = *issued_slot;
                for (int it = (issued > S ? issued - S : 0); it < issued; ++it)
                    mbar_wait(&full[it % S], (it / S) & 1u);
            }
            for (int i = 0; i < 1000; ++i) __nanosleep(1000);
        }
        mbar_wait(done, 0);  // no MMA may still write the tensor memory freed below
    }
    __syncthreads();
    cluster_sync();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(2 * TMEM_COLS));
    }
    cluster_sync();  // neither CTA leaves while its peer still frees the pair's tensor memory
}

// ------------------------------------------------------------------ operand preparation

template <typename T>
__device__ __forceinline__ T to_elem(float x);
template <>
__device__ __forceinline__ __nv_bfloat16 to_elem<__nv_bfloat16>(float x) {
    return __float2bfloat16_rn(x);
}
template <>
__device__ __forceinline__ __half to_elem<__half>(float x) {
    return __float2half_rn(x);
}
__device__ __forceinline__ float from_elem(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float from_elem(__half x) { return __half2float(x); }

// G rows for a tile of kRows points x 256 sources; thread t owns source j0 + t and writes the
// (re, im) pair of columns 2j, 2j+1 of each row (zero for the padding j >= n).
constexpr int kGRows = 32;

template <int ST, typename T, bool SPLIT>
__global__ void __launch_bounds__(256) build_g_kernel(const PackedSource* __restrict__ src, int64_t n,
                                                      const float* __restrict__ pts, int64_t m,
                                                      int64_t kpad, const float* __restrict__ row_inv,
                                                      T* __restrict__ a_hi, T* __restrict__ a_lo) {
    __shared__ float4 s_dir[dev::kDirTableSize];
    __shared__ float s_pts[kGRows * 3];
    if (threadIdx.x < dev::kDirTableSize) s_dir[threadIdx.x] = c_dir_table_mp[threadIdx.x];
    const int64_t r0 = static_cast<int64_t>(blockIdx.y) * kGRows;
    if (threadIdx.x < kGRows * 3) {
        const int64_t idx = r0 * 3 + threadIdx.x;
        s_pts[threadIdx.x] = idx < m * 3 ? pts[idx] : 0.f;
    }
    __syncthreads();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (2 * j >= kpad) return;
    PackedSource s{};
    const bool live = j < n;
    if (live) s = src[j];
    for (int r = 0; r < kGRows; ++r) {
        const int64_t row = r0 + r;
        if (row >= m) break;
        float gr = 0.f, gi = 0.f;
        if (live) {
            float w, red;
            dev::pair_terms<ST>(s.a, s.b, 0.0f, 0.0f, s_dir, s_pts[3 * r], s_pts[3 * r + 1],
                                s_pts[3 * r + 2], w, red);
            if (row_inv) w *= row_inv[row];
            gr = w * dev::mufu_cos(red);
            gi = w * dev::mufu_sin(red);
        }
        const T hr = to_elem<T>(gr), hi = to_elem<T>(gi);
        const int64_t o = row * kpad + 2 * j;
        a_hi[o] = hr;
        a_hi[o + 1] = hi;
        if constexpr (SPLIT) {
            a_lo[o] = to_elem<T>(gr - from_elem(hr));
            a_lo[o + 1] = to_elem<T>(gi - from_elem(hi));
        }
    }
}

// Power-of-two scale per row for the FP16 form: row_inv[i] = 2^-e with 2^e >= max_j |G_ij|
// (|G_ij| = D exp(-alpha r) / r needs no sine or cosine); row_scale[i] = 2^e undoes it.
template <int ST>
__global__ void __launch_bounds__(256) row_scale_kernel(const PackedSource* __restrict__ src, int64_t n,
                                                        const float* __restrict__ pts, int64_t m,
                                                        float* __restrict__ row_inv,
                                                        float* __restrict__ row_scale) {
    __shared__ float4 s_dir[dev::kDirTableSize];
    __shared__ float s_max[8];
    if (threadIdx.x < dev::kDirTableSize) s_dir[threadIdx.x] = c_dir_table_mp[threadIdx.x];
    __syncthreads();
    const int64_t row = blockIdx.x;
    const float px = pts[3 * row], py = pts[3 * row + 1], pz = pts[3 * row + 2];
    float mx = 0.f;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const PackedSource s = src[j];
        float w, red;
        dev::pair_terms<ST>(s.a, s.b, 0.0f, 0.0f, s_dir, px, py, pz, w, red);
        mx = fmaxf(mx, fabsf(w));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) mx = fmaxf(mx, s_max[w]);
        int e = 0;
        if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);  // mx = f 2^e, f in [0.5, 1)
        row_inv[row] = ldexpf(1.0f, -e);
        row_scale[row] = ldexpf(1.0f, e);
    }
}

// B^T rows 2k, 2k+1 for pattern k from amplitudes and phases (K x n, pattern-major).
template <typename T, bool SPLIT>
__global__ void build_q_kernel(const float* __restrict__ amps, const float* __restrict__ phases,
                               int64_t n, int64_t K, int64_t kpad, T* __restrict__ b_hi,
                               T* __restrict__ b_lo) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t k = blockIdx.y;
    if (2 * j >= kpad || k >= K) return;
    float qr = 0.f, qi = 0.f;
    if (j < n) {
        float sn, cs;
        sincosf(phases[k * n + j], &sn, &cs);
        const float a = amps[k * n + j];
        qr = a * cs;
        qi = a * sn;
    }
    const float v[4] = {qr, -qi, qi, qr};
    const int64_t o0 = (2 * k) * kpad + 2 * j, o1 = (2 * k + 1) * kpad + 2 * j;
    const int64_t off[4] = {o0, o0 + 1, o1, o1 + 1};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const T h = to_elem<T>(v[t]);
        b_hi[off[t]] = h;
        if constexpr (SPLIT) b_lo[off[t]] = to_elem<T>(v[t] - from_elem(h));
    }
}

// ------------------------------------------------------------------ host side

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

cudaError_t get_encoder() {
    std::lock_guard<std::mutex> lock(g_encode_mu);
    if (g_encode) return cudaSuccess;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return cudaSuccess;
}

// 2-D row-major [rows x kpad] 2-byte matrix, box = BK x box_rows, 128-byte swizzle.
cudaError_t make_map(CUtensorMap* map, const void* base, bool bf16, int64_t rows, int64_t kpad,
                     int box_rows) {
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kpad), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kpad) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                          2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

size_t a256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

// Workspace layout for n sources, m points, K patterns.
struct Layout {
    int64_t kpad;   // 2n rounded up to BK
    int64_t npad;   // 2K rounded up to BN (columns of C)
    size_t packed, a_hi, a_lo, b_hi, b_lo, row_inv, row_scale, c_pad, err, total;
};

// Sizes the contraction accepts: n and m below 2^31 (m a launch's row tiles), K within one
// launch's column tiles, and a workspace whose size, recomputed in 128 bits, stays below 2^62
// (so that no byte count wraps and a workspace sized by AFC_MultiPatternWorkspaceBytes always
// covers what the kernels touch).
bool sizes_ok(uint64_t n, uint64_t m, uint64_t K) {
    if (n >= (1ull << 31) || m >= (1ull << 31) - BM || K >= (1ull << 26)) return false;
    using u128 = unsigned __int128;
    const u128 kpad = (2 * static_cast<u128>(n) + BK - 1) / BK * BK;
    const u128 npad = (2 * static_cast<u128>(K) + BN - 1) / BN * BN;
    if (npad / BN > 65535) return false;
    const u128 total = 48 * static_cast<u128>(n) + 4 * static_cast<u128>(m) * kpad +
                       4 * npad * kpad + 8 * static_cast<u128>(m) + 4 * static_cast<u128>(m) * npad +
                       8 * 256;
    return total < (static_cast<u128>(1) << 62);
}

Layout layout(int64_t n, int64_t m, int64_t K, int precision) {
    Layout L{};
    L.kpad = ((2 * n + BK - 1) / BK) * BK;
    L.npad = ((2 * K + BN - 1) / BN) * BN;
    const bool split = precision == AFC_PRECISION_BF16X3;
    size_t off = 0;
    L.packed = off;
    off += a256(sizeof(PackedSource) * n);
    L.a_hi = off;
    off += a256(static_cast<size_t>(m) * L.kpad * 2);
    L.a_lo = off;
    if (split) off += a256(static_cast<size_t>(m) * L.kpad * 2);
    L.b_hi = off;
    off += a256(static_cast<size_t>(L.npad) * L.kpad * 2);
    L.b_lo = off;
    if (split) off += a256(static_cast<size_t>(L.npad) * L.kpad * 2);
    L.row_inv = off;
    off += a256(sizeof(float) * m);
    L.row_scale = off;
    off += a256(sizeof(float) * m);
    L.c_pad = off;
    if (L.npad != 2 * K) off += a256(sizeof(float) * static_cast<size_t>(m) * L.npad);
    L.err = off;
    off += 256;
    L.total = off;
    return L;
}

__global__ void copy_cols_kernel(const float* __restrict__ c, int64_t ldc, float* __restrict__ out,
                                 int64_t m, int64_t cols) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m * cols) return;
    out[i] = c[(i / cols) * ldc + (i % cols)];
}

// Co-resident CTA pairs of the GEMM kernel on a device (one CTA per SM by its shared memory),
// cached per device and precision.
constexpr int kPairCacheDevices = 64;
std::atomic<int> g_gemm_pairs[kPairCacheDevices][2] = {};

template <bool BF16>
cudaError_t launch_gemm(const CUtensorMap& ma0, const CUtensorMap& ma1, const CUtensorMap& mb0,
                        const CUtensorMap& mb1, const GemmArgs& a, int dev, cudaStream_t s) {
    using Cfg = GemmCfg<BF16>;
    auto* kern = cgemm_tcgen05_kernel<BF16>;
    cudaError_t e = cudaSuccess;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(GEMM_THREADS);
    cfg.dynamicSmemBytes = Cfg::kSmemBytes;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int pairs = (dev >= 0 && dev < kPairCacheDevices)
                    ? g_gemm_pairs[dev][BF16 ? 1 : 0].load(std::memory_order_relaxed)
                    : 0;
    if (pairs <= 0) {
        // first call on this device: the shared-memory opt-in and the co-resident pairs (both
        // kept, so that later calls, also under stream capture, make neither query)
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Cfg::kSmemBytes)) != cudaSuccess)
            return e;
        cfg.gridDim = dim3(2 * static_cast<unsigned>(num_sms() / 2));
        if ((e = cudaOccupancyMaxActiveClusters(&pairs, kern, &cfg)) != cudaSuccess) return e;
        if (pairs < 1) return cudaErrorInvalidConfiguration;
        if (dev >= 0 && dev < kPairCacheDevices)
            g_gemm_pairs[dev][BF16 ? 1 : 0].store(pairs, std::memory_order_relaxed);
    }
    const int64_t use = a.tiles < pairs ? a.tiles : pairs;
    cfg.gridDim = dim3(2 * static_cast<unsigned>(use));
    return cudaLaunchKernelEx(&cfg, kern, ma0, ma1, mb0, mb1, a);
}

}  // namespace mp
}  // namespace afc

using namespace afc;
using namespace afc::mp;

extern "C" size_t AFC_MultiPatternWorkspaceBytes(uint64_t n, uint64_t m, uint64_t patterns,
                                                 int32_t precision) {
    if (precision != AFC_PRECISION_BF16X3 && precision != AFC_PRECISION_FP16) return 0;
    if (!sizes_ok(n, m, patterns)) return 0;
    return layout(static_cast<int64_t>(n), static_cast<int64_t>(m), static_cast<int64_t>(patterns),
                  precision)
        .total;
}

extern "C" int32_t AFC_MultiPatternBuildG(int32_t source_type, int32_t precision,
                                          const float* d_sources, const float* d_wavenums,
                                          const float* d_attens, uint64_t n, const float* d_points,
                                          uint64_t m, uint64_t patterns, void* d_ws,
                                          size_t ws_bytes, void* stream) {
    if ((precision != AFC_PRECISION_BF16X3 && precision != AFC_PRECISION_FP16) ||
        (source_type != SRC_SPHERE && source_type != SRC_T4010A1)) {
        set_error_message("AFC_MultiPatternBuildG: invalid precision or source type");
        return AFC_ERR_INVALID;
    }
    if (!sizes_ok(n, m, patterns)) {
        set_error_message("AFC_MultiPatternBuildG: problem too large");
        return AFC_ERR_TOO_LARGE;
    }
    const Layout L = layout(static_cast<int64_t>(n), static_cast<int64_t>(m),
                            static_cast<int64_t>(patterns), precision);
    if (!d_ws || ws_bytes < L.total || (reinterpret_cast<uintptr_t>(d_ws) & 255u) ||
        (n && (!d_sources || !d_wavenums || !d_attens)) || (m && !d_points)) {
        set_error_message("AFC_MultiPatternBuildG: bad pointer or workspace too small/unaligned");
        return AFC_ERR_INVALID;
    }
    if (n == 0 || m == 0) return AFC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;  // the stream's device while launching; the caller's again on return
    int dev = 0;
    cudaError_t e = stream_device(s, &dev);
    if (e == cudaSuccess) e = dg.set(dev);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    char* ws = static_cast<char*>(d_ws);
    auto* packed = reinterpret_cast<PackedSource*>(ws + L.packed);
    e = launch_pack_sources(source_type, d_sources, d_wavenums, d_attens,
                                        static_cast<int64_t>(n), packed, s);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    const dim3 grid(static_cast<unsigned>((L.kpad / 2 + 255) / 256),
                    static_cast<unsigned>((m + kGRows - 1) / kGRows));
    const int64_t mm = static_cast<int64_t>(m), nn = static_cast<int64_t>(n);
    if (precision == AFC_PRECISION_BF16X3) {
        auto* ah = reinterpret_cast<__nv_bfloat16*>(ws + L.a_hi);
        auto* al = reinterpret_cast<__nv_bfloat16*>(ws + L.a_lo);
        if (source_type == SRC_T4010A1)
            build_g_kernel<SRC_T4010A1, __nv_bfloat16, true><<<grid, 256, 0, s>>>(packed, nn, d_points, mm, L.kpad, nullptr, ah, al);
        else
            build_g_kernel<SRC_SPHERE, __nv_bfloat16, true><<<grid, 256, 0, s>>>(packed, nn, d_points, mm, L.kpad, nullptr, ah, al);
        count_launch();
    } else {
        auto* ri = reinterpret_cast<float*>(ws + L.row_inv);
        auto* rs = reinterpret_cast<float*>(ws + L.row_scale);
        auto* ah = reinterpret_cast<__half*>(ws + L.a_hi);
        if (source_type == SRC_T4010A1) {
            row_scale_kernel<SRC_T4010A1><<<static_cast<unsigned>(m), 256, 0, s>>>(packed, nn, d_points, mm, ri, rs);
            build_g_kernel<SRC_T4010A1, __half, false><<<grid, 256, 0, s>>>(packed, nn, d_points, mm, L.kpad, ri, ah, nullptr);
        } else {
            row_scale_kernel<SRC_SPHERE><<<static_cast<unsigned>(m), 256, 0, s>>>(packed, nn, d_points, mm, ri, rs);
            build_g_kernel<SRC_SPHERE, __half, false><<<grid, 256, 0, s>>>(packed, nn, d_points, mm, L.kpad, ri, ah, nullptr);
        }
        count_launch(2);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    return AFC_OK;
}

namespace {

int32_t multipattern_apply(int32_t precision, const float* d_amps, const float* d_phases,
                           uint64_t n, uint64_t m, uint64_t patterns, float* d_out, void* d_ws,
                           size_t ws_bytes, void* stream, int stall) {
    if (precision != AFC_PRECISION_BF16X3 && precision != AFC_PRECISION_FP16) {
        set_error_message("AFC_MultiPatternApply: invalid precision");
        return AFC_ERR_INVALID;
    }
    if (!sizes_ok(n, m, patterns)) {
        set_error_message("AFC_MultiPatternApply: problem too large");
        return AFC_ERR_TOO_LARGE;
    }
    const int64_t nn = static_cast<int64_t>(n), mm = static_cast<int64_t>(m),
                  K = static_cast<int64_t>(patterns);
    const Layout L = layout(nn, mm, K, precision);
    if (!d_ws || ws_bytes < L.total || (reinterpret_cast<uintptr_t>(d_ws) & 255u) || !d_out ||
        (n && K && (!d_amps || !d_phases)) || (reinterpret_cast<uintptr_t>(d_out) & 15u)) {
        set_error_message("AFC_MultiPatternApply: bad pointer or workspace too small/unaligned");
        return AFC_ERR_INVALID;
    }
    if (m == 0 || K == 0) return AFC_OK;
    if (mm > (1LL << 31) - BM || L.npad / BN > 65535 || (mm + BM - 1) / BM > 65535LL * 32768) {
        set_error_message("AFC_MultiPatternApply: problem too large for one launch");
        return AFC_ERR_TOO_LARGE;
    }
    cudaError_t e = get_encoder();
    if (e != cudaSuccess) {
        set_error_message("AFC_MultiPatternApply: cuTensorMapEncodeTiled unavailable");
        return AFC_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;  // the stream's device while launching; the caller's again on return
    int dev = 0;
    if ((e = stream_device(s, &dev)) != cudaSuccess || (e = dg.set(dev)) != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    char* ws = static_cast<char*>(d_ws);
    const bool split = precision == AFC_PRECISION_BF16X3;
    unsigned* err = reinterpret_cast<unsigned*>(ws + L.err);
    if ((e = cudaMemsetAsync(err, 0, sizeof(unsigned), s)) != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    // Q
    {
        const dim3 grid(static_cast<unsigned>((L.kpad / 2 + 255) / 256), static_cast<unsigned>(K));
        if (split)
            build_q_kernel<__nv_bfloat16, true><<<grid, 256, 0, s>>>(
                d_amps, d_phases, nn, K, L.kpad, reinterpret_cast<__nv_bfloat16*>(ws + L.b_hi),
                reinterpret_cast<__nv_bfloat16*>(ws + L.b_lo));
        else
            build_q_kernel<__half, false><<<grid, 256, 0, s>>>(
                d_amps, d_phases, nn, K, L.kpad, reinterpret_cast<__half*>(ws + L.b_hi), nullptr);
        count_launch();
        // B^T rows 2K .. npad-1 (padding) must be zero
        if (L.npad > 2 * K)
            e = cudaMemsetAsync(ws + L.b_hi + static_cast<size_t>(2 * K) * L.kpad * 2, 0,
                                static_cast<size_t>(L.npad - 2 * K) * L.kpad * 2, s);
        if (e == cudaSuccess && split && L.npad > 2 * K)
            e = cudaMemsetAsync(ws + L.b_lo + static_cast<size_t>(2 * K) * L.kpad * 2, 0,
                                static_cast<size_t>(L.npad - 2 * K) * L.kpad * 2, s);
        if (e != cudaSuccess) {
            set_error_message(cudaGetErrorString(e));
            return AFC_ERR_CUDA;
        }
    }
    CUtensorMap ma0, ma1, mb0, mb1;
    if ((e = make_map(&ma0, ws + L.a_hi, split, mm, L.kpad, HALF)) != cudaSuccess ||
        (e = make_map(&ma1, ws + (split ? L.a_lo : L.a_hi), split, mm, L.kpad, HALF)) != cudaSuccess ||
        (e = make_map(&mb0, ws + L.b_hi, split, L.npad, L.kpad, HALF)) != cudaSuccess ||
        (e = make_map(&mb1, ws + (split ? L.b_lo : L.b_hi), split, L.npad, L.kpad, HALF)) != cudaSuccess) {
        set_error_message("AFC_MultiPatternApply: tensor map encoding failed");
        return AFC_ERR_CUDA;
    }
    GemmArgs a{};
    a.k_blocks = static_cast<int>(L.kpad / BK);
    const bool direct = L.npad == 2 * K;
    a.c = direct ? d_out : reinterpret_cast<float*>(ws + L.c_pad);
    a.ldc = L.npad;
    a.m = mm;
    a.row_scale = split ? nullptr : reinterpret_cast<const float*>(ws + L.row_scale);
    a.err = err;
    a.n_tiles = static_cast<int>(L.npad / BN);
    a.tiles = static_cast<int64_t>(a.n_tiles) * ((mm + BM - 1) / BM);
    a.stall = stall;
    e = split ? launch_gemm<true>(ma0, ma1, mb0, mb1, a, dev, s)
              : launch_gemm<false>(ma0, ma1, mb0, mb1, a, dev, s);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    count_launch();
    if (!direct) {
        const int64_t total = mm * 2 * K;
        copy_cols_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, s>>>(
            a.c, L.npad, d_out, mm, 2 * K);
        count_launch();
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    return AFC_OK;
}

}  // namespace

extern "C" int32_t AFC_MultiPatternApply(int32_t precision, const float* d_amps,
                                         const float* d_phases, uint64_t n, uint64_t m,
                                         uint64_t patterns, float* d_out, void* d_ws,
                                         size_t ws_bytes, void* stream) {
    return multipattern_apply(precision, d_amps, d_phases, n, m, patterns, d_out, d_ws, ws_bytes,
                              stream, 0);
}

// Testing: AFC_MultiPatternApply with the GEMM's producer arming no pipeline stage, so that every
// mbarrier wait of the kernel runs out (about a second) and the kernel returns through its error
// path.  The output is not computed.
extern "C" int32_t AFC_MultiPatternApplyWaitTest(int32_t precision, const float* d_amps,
                                                 const float* d_phases, uint64_t n, uint64_t m,
                                                 uint64_t patterns, float* d_out, void* d_ws,
                                                 size_t ws_bytes, void* stream) {
    return multipattern_apply(precision, d_amps, d_phases, n, m, patterns, d_out, d_ws, ws_bytes,
                              stream, 1);
}

// Error code left by the last AFC_MultiPatternApply in this workspace (0: none, 1-3: an
// mbarrier wait of the producer / MMA issuer / epilogue timed out).  Synchronises the stream.
extern "C" int32_t AFC_MultiPatternStatus(int32_t precision, uint64_t n, uint64_t m,
                                          uint64_t patterns, void* d_ws, void* stream) {
    const Layout L = layout(static_cast<int64_t>(n), static_cast<int64_t>(m),
                            static_cast<int64_t>(patterns), precision);
    unsigned h = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;
    int dev = 0;
    if (stream_device(s, &dev) != cudaSuccess || dg.set(dev) != cudaSuccess) return AFC_ERR_CUDA;
    if (cudaMemcpyAsync(&h, static_cast<char*>(d_ws) + L.err, sizeof(h), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return AFC_ERR_CUDA;
    return static_cast<int32_t>(h);
}

namespace afc {
namespace mp {

// PackedSource of pattern k: geometry from `geom`, amplitude and phase from the pattern arrays
// (same folding as pack_sources_kernel: log2|A| in the exponent, the sign of A as +pi).
__global__ void repack_pattern_kernel(const PackedSource* __restrict__ geom,
                                      const float* __restrict__ amps,
                                      const float* __restrict__ phases, int64_t n,
                                      PackedSource* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    PackedSource p = geom[j];
    const float a = amps[j], ph = phases[j];
    p.c = make_float4(log2f(fabsf(a)), a < 0.f ? ph + 3.14159265358979323846f : ph, a, ph);
    out[j] = p;
}

}  // namespace mp
}  // namespace afc

extern "C" int32_t AFC_MultiPatternDirect(int32_t source_type, const float* d_sources,
                                          const float* d_wavenums, const float* d_attens,
                                          uint64_t n, const float* d_points, uint64_t m,
                                          const float* d_amps, const float* d_phases,
                                          uint64_t patterns, float* d_out, void* d_ws,
                                          size_t ws_bytes, void* stream) {
    if (n >= (1ull << 40) || m >= (1ull << 62) / 8 || patterns >= (1ull << 62) / 8 ||
        (m && patterns > ((1ull << 62) / 8) / m)) {
        set_error_message("AFC_MultiPatternDirect: problem too large");
        return AFC_ERR_TOO_LARGE;
    }
    const size_t half = AFC_FieldWorkspaceBytes(n);
    if ((source_type != SRC_SPHERE && source_type != SRC_T4010A1) || !d_out ||
        (n && (!d_sources || !d_wavenums || !d_attens || !d_amps || !d_phases || !d_ws ||
               ws_bytes < 2 * half || (reinterpret_cast<uintptr_t>(d_ws) & 15u))) ||
        (m && !d_points)) {
        set_error_message("AFC_MultiPatternDirect: invalid argument or workspace too small");
        return AFC_ERR_INVALID;
    }
    if (m == 0 || patterns == 0) return AFC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;  // the stream's device while launching; the caller's again on return
    int dev = 0;
    cudaError_t e = stream_device(s, &dev);
    if (e == cudaSuccess) e = dg.set(dev);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    auto* geom = static_cast<PackedSource*>(d_ws);
    auto* pat = reinterpret_cast<PackedSource*>(static_cast<char*>(d_ws) + half);
    e = launch_pack_sources(source_type, d_sources, d_wavenums, d_attens,
                                        static_cast<int64_t>(n), geom, s);
    PointSet ps{};
    ps.is_grid = false;
    ps.pts = d_points;
    ps.m = static_cast<int64_t>(m);
    const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
    for (uint64_t k = 0; k < patterns && e == cudaSuccess; ++k) {
        if (n > 0) {
            repack_pattern_kernel<<<blocks, 256, 0, s>>>(geom, d_amps + k * n, d_phases + k * n,
                                                         static_cast<int64_t>(n), pat);
            count_launch();
        }
        e = launch_field(source_type, FIELD_COMPLEX, SUM_PLAIN, pat, static_cast<int64_t>(n), ps,
                         d_out + 2 * k * m, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return AFC_ERR_CUDA;
    }
    return AFC_OK;
}
