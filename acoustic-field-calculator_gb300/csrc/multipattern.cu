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
//     Al Bh accumulated in FP32 (three K-segments of one accumulation), ~16 significant bits.
//   FP16 row-scaled: each row of G scaled by a power of two so that its largest entry is ~1,
//     one FP16 GEMM, the scale undone in the epilogue (exact).
//
// GEMM kernel (one CTA per 128 x 256 output tile, 192 threads):
//   warp 0 lane 0  TMA producer: 128 x 64 A and 256 x 64 B tiles (128-byte swizzle) into a
//                  4-stage shared-memory ring, completion signalled on the stage's mbarrier.
//   warp 1         allocates 256 TMEM columns; lane 0 issues tcgen05.mma (M=128, N=256, K=16,
//                  FP32 accumulate in TMEM) and frees each stage with tcgen05.commit.
//   warps 2-5      epilogue: tcgen05.ld of their 32 TMEM lanes, FP32 stores of C.
// Every mbarrier wait is bounded; on time-out the CTA records an error code, drains its own
// copies (bounded) and frees its tensor memory before it returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "propagate.cuh"

namespace afc {
namespace mp {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BK = 64;  // 64 x 2-byte elements = one 128-byte swizzle row
constexpr int STAGES = 4;
constexpr int A_TILE = BM * BK * 2;
constexpr int B_TILE = BN * BK * 2;
constexpr int STAGE_BYTES = A_TILE + B_TILE;
constexpr int GEMM_THREADS = 192;
constexpr int TMEM_COLS = 256;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr uint32_t kWaitLimit = 1u << 24;

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

// Wait until the phase with the given parity has completed; false after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
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

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
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
    int k_blocks;        // BK-blocks per segment
    int nseg;            // 1 (FP16) or 3 (split BF16)
    int seg_a[3];        // which A map each segment reads (0 hi, 1 lo)
    int seg_b[3];        // which B map each segment reads
    float* c;            // M x ldc floats
    int64_t ldc;         // row stride of C in floats
    int64_t m;           // rows of C
    const float* row_scale;  // nullable: C row i multiplied by row_scale[i]
    unsigned* err;       // error code (first writer wins)
};

template <bool BF16>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    cgemm_tcgen05_kernel(const __grid_constant__ CUtensorMap map_a0,
                         const __grid_constant__ CUtensorMap map_a1,
                         const __grid_constant__ CUtensorMap map_b0,
                         const __grid_constant__ CUtensorMap map_b1, GemmArgs args) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* issued_slot = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x, m_tile = blockIdx.y;
    const int total = args.nseg * args.k_blocks;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *issued_slot = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            const CUtensorMap* ma[2] = {&map_a0, &map_a1};
            const CUtensorMap* mb[2] = {&map_b0, &map_b1};
            int it = 0;
            for (; it < total; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (it / STAGES) & 1u;
                if (!mbar_wait(&empty[s], ph ^ 1u)) {
                    atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_PRODUCER);
                    break;
                }
                const int seg = it / args.k_blocks, kb = it % args.k_blocks;
                uint8_t* sa = smem + s * STAGE_BYTES;
                mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                tma_load_2d(sa, ma[args.seg_a[seg]], &full[s], kb * BK, m_tile * BM);
                tma_load_2d(sa + A_TILE, mb[args.seg_b[seg]], &full[s], kb * BK, n_tile * BN);
            }
            *issued_slot = it;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = mma_idesc(BF16);
            int it = 0;
            for (; it < total; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (it / STAGES) & 1u;
                if (!mbar_wait(&full[s], ph)) {
                    atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_MMA);
                    break;
                }
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
                const uint64_t adesc = smem_desc_sw128(sa);
                const uint64_t bdesc = smem_desc_sw128(sa + A_TILE);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
                    // K step of 16 elements = 32 bytes = 2 in the descriptor's address field
                    mma_f16(tmem, adesc + 2u * k, bdesc + 2u * k, idesc, (it | k) != 0);
                }
                mma_commit(&empty[s]);
            }
            mma_commit(done);  // completes once every MMA issued above has finished
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, i.e. rows of the tile
        const int q = warp & 3;
        const int64_t row = static_cast<int64_t>(m_tile) * BM + q * 32 + lane;
        // one lane waits, the warp follows converged (tcgen05.ld is warp-synchronous)
        const int ok = __shfl_sync(0xffffffffu, lane == 0 ? (mbar_wait(done, 0) ? 1 : 0) : 0, 0);
        __syncwarp();
        if (!ok) {
            atomicCAS(args.err, ERR_NONE, ERR_TIMEOUT_EPILOGUE);
        } else {
            tc_fence_after();
            const float scale = (args.row_scale && row < args.m) ? args.row_scale[row] : 1.0f;
#pragma unroll 1
            for (int c = 0; c < BN / 32; ++c) {
                uint32_t v[32];
                tmem_ld_32cols(tmem + (static_cast<uint32_t>(q * 32) << 16) + c * 32, v);
                if (row < args.m) {
                    float4* dst = reinterpret_cast<float4*>(args.c + row * args.ldc +
                                                            static_cast<int64_t>(n_tile) * BN + c * 32);
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        dst[t] = make_float4(__uint_as_float(v[4 * t]) * scale,
                                             __uint_as_float(v[4 * t + 1]) * scale,
                                             __uint_as_float(v[4 * t + 2]) * scale,
                                             __uint_as_float(v[4 * t + 3]) * scale);
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *args.err != ERR_NONE) {
        // drain: wait (bounded) for every stage this CTA's producer armed to land
        const int issued = *issued_slot;
        for (int it = (issued > STAGES ? issued - STAGES : 0); it < issued; ++it)
            mbar_wait(&full[it % STAGES], (it / STAGES) & 1u);
        mbar_wait(done, 0);
    }
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    }
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

extern "C" int32_t AFC_MultiPatternApply(int32_t precision, const float* d_amps,
                                         const float* d_phases, uint64_t n, uint64_t m,
                                         uint64_t patterns, float* d_out, void* d_ws,
                                         size_t ws_bytes, void* stream) {
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
    if ((e = make_map(&ma0, ws + L.a_hi, split, mm, L.kpad, BM)) != cudaSuccess ||
        (e = make_map(&ma1, ws + (split ? L.a_lo : L.a_hi), split, mm, L.kpad, BM)) != cudaSuccess ||
        (e = make_map(&mb0, ws + L.b_hi, split, L.npad, L.kpad, BN)) != cudaSuccess ||
        (e = make_map(&mb1, ws + (split ? L.b_lo : L.b_hi), split, L.npad, L.kpad, BN)) != cudaSuccess) {
        set_error_message("AFC_MultiPatternApply: tensor map encoding failed");
        return AFC_ERR_CUDA;
    }
    GemmArgs a{};
    a.k_blocks = static_cast<int>(L.kpad / BK);
    if (split) {
        a.nseg = 3;  // hi*hi + hi*lo + lo*hi
        a.seg_a[0] = 0; a.seg_b[0] = 0;
        a.seg_a[1] = 0; a.seg_b[1] = 1;
        a.seg_a[2] = 1; a.seg_b[2] = 0;
    } else {
        a.nseg = 1;
        a.seg_a[0] = 0; a.seg_b[0] = 0;
    }
    const bool direct = L.npad == 2 * K;
    a.c = direct ? d_out : reinterpret_cast<float*>(ws + L.c_pad);
    a.ldc = L.npad;
    a.m = mm;
    a.row_scale = split ? nullptr : reinterpret_cast<const float*>(ws + L.row_scale);
    a.err = err;
    const dim3 grid(static_cast<unsigned>(L.npad / BN), static_cast<unsigned>((mm + BM - 1) / BM));
    if (split) {
        cudaFuncSetAttribute(cgemm_tcgen05_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cgemm_tcgen05_kernel<true><<<grid, GEMM_THREADS, SMEM_BYTES, s>>>(ma0, ma1, mb0, mb1, a);
    } else {
        cudaFuncSetAttribute(cgemm_tcgen05_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        cgemm_tcgen05_kernel<false><<<grid, GEMM_THREADS, SMEM_BYTES, s>>>(ma0, ma1, mb0, mb1, a);
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
