// Transfer matrix and multi-focus solvers on sm_103a.
//
//   build_g        G[i, j] = propagate(source j, focus i) with the sources' current amplitude
//                  and phase 0 (acoustic-field-optimizer/src/multiple_foci/macros.rs:32-53,
//                  called after the phases are zeroed, gs_pat.rs:38-45).  Row-major m x n.
//   GS-PAT         gs_pat.rs:47-80: den_j = sum_i |G_ij| (nalgebra row_sum = column sums),
//                  B = [conj(G_ij) / den_j^2]^T, R = G B (m x m), gamma = R p0, 100 times
//                  {p = gamma / |gamma| * p0; gamma = R p}, p = gamma / |gamma|^2 * p0^2,
//                  q = B p; amp_j = |q_j|, phase_j = arg q_j.  B is never materialised:
//                  R_ik = sum_j G_ij conj(G_kj) / den_j^2 and q_j = sum_i conj(G_ij) p_i / den_j^2.
//   GS             gs.rs:42-77: q = q0; 100 times {gamma = G q; p = gamma/|gamma| p0;
//                  xi = G^H p; q = xi/|xi| q0}.
//   Naive          naive.rs:37-49: q = G^H p0.
//
// Sizes are small (m <= 64 foci, n ~ 1e3 sources in the serving mix): G build is one thread per
// pair; R is one block per entry; the iterations run in a single block so that the 100
// dependent steps cost block barriers, not kernel launches (up to 64 foci with R in shared
// memory and every row of a product summed at once).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "afc_internal.h"
#include "afc_solvers.h"
#include "propagate.cuh"

namespace afc {

namespace {

__constant__ float4 c_dir_table_s[dev::kDirTableSize] = AFC_DIR_TABLE_INIT;

constexpr int kIterThreads = 1024;
constexpr float kPiF = 3.14159265358979323846f;  // f32 PI of the reference (core/mod.rs)

size_t align256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

struct SolverWs {
    PackedSource* packed;
    float2* g;
    float* inv_den2;
    float2* r;
    float2* p;
    float2* gamma;
    float2* q;
};

SolverWs carve(void* ws, int64_t n, int64_t m) {
    char* b = static_cast<char*>(ws);
    SolverWs w;
    w.packed = reinterpret_cast<PackedSource*>(b);
    b += align256(sizeof(PackedSource) * n);
    w.g = reinterpret_cast<float2*>(b);
    b += align256(sizeof(float2) * n * m);
    w.inv_den2 = reinterpret_cast<float*>(b);
    b += align256(sizeof(float) * n);
    w.r = reinterpret_cast<float2*>(b);
    b += align256(sizeof(float2) * m * m);
    w.p = reinterpret_cast<float2*>(b);
    b += align256(sizeof(float2) * m);
    w.gamma = reinterpret_cast<float2*>(b);
    b += align256(sizeof(float2) * m);
    w.q = reinterpret_cast<float2*>(b);
    return w;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// conj(a) * b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.x, b.y, -a.y * b.x));
}

__device__ __forceinline__ float2 warp_sum(float2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

template <int ST>
__global__ void build_g_kernel(const PackedSource* __restrict__ src, int64_t n,
                               const float* __restrict__ foci, int64_t m, float2* __restrict__ g) {
    __shared__ float4 s_dir[dev::kDirTableSize];
    if (threadIdx.x < dev::kDirTableSize) s_dir[threadIdx.x] = c_dir_table_s[threadIdx.x];
    dev::pdl_wait();  // the packed sources
    dev::pdl_release();
    __syncthreads();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t i = blockIdx.y;
    if (j >= n) return;
    const PackedSource s = src[j];
    float w, red;
    // the phases are zeroed before G is built (gs_pat.rs:39-41): phase' is pi for A < 0
    dev::pair_terms<ST>(s.a, s.b, s.c.x, s.c.z < 0.f ? 3.14159265358979323846f : 0.0f, s_dir,
                        foci[3 * i], foci[3 * i + 1], foci[3 * i + 2], w, red);
    g[i * n + j] = make_float2(w * dev::mufu_cos(red), w * dev::mufu_sin(red));
}

// inv_den2[j] = 1 / (sum_i |G_ij|)^2
__global__ void column_abs_sum_kernel(const float2* __restrict__ g, int64_t n, int64_t m,
                                      float* __restrict__ inv_den2) {
    dev::pdl_wait();
    dev::pdl_release();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float s = 0.f;
#pragma unroll 8
    for (int64_t i = 0; i < m; ++i) {
        const float2 v = g[i * n + j];
        s += hypotf(v.x, v.y);
    }
    inv_den2[j] = 1.0f / (s * s);
}

// R[i, k] = sum_j G_ij conj(G_kj) inv_den2_j, one block per entry.
__global__ void gspat_r_kernel(const float2* __restrict__ g, const float* __restrict__ inv_den2,
                               int64_t n, int64_t m, float2* __restrict__ r) {
    dev::pdl_wait();
    dev::pdl_release();
    const int64_t i = blockIdx.y, k = blockIdx.x;
    const float2* gi = g + i * n;
    const float2* gk = g + k * n;
    float2 acc = make_float2(0.f, 0.f);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const float2 t = cmulc(gk[j], gi[j]);  // G_ij conj(G_kj)
        const float s = inv_den2[j];
        acc.x = fmaf(t.x, s, acc.x);
        acc.y = fmaf(t.y, s, acc.y);
    }
    acc = warp_sum(acc);
    __shared__ float2 part[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = acc;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        float2 v = lane < nw ? part[lane] : make_float2(0.f, 0.f);
        v = warp_sum(v);
        if (lane == 0) r[i * m + k] = v;
    }
}

// gamma = M v for a row-major m x m matrix, one warp per row; v and gamma in global memory
// (visible block-wide after __syncthreads).
__device__ __forceinline__ void block_matvec(const float2* __restrict__ mat, const float2* v,
                                             float2* out, int64_t m) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t row = wid; row < m; row += nw) {
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t c = lane; c < m; c += 32) {
            const float2 t = cmul(mat[row * m + c], v[c]);
            acc.x += t.x;
            acc.y += t.y;
        }
        acc = warp_sum(acc);
        if (lane == 0) out[row] = acc;
    }
}

// The GS-PAT iteration (gs_pat.rs:54-71) in one block.
__global__ void __launch_bounds__(kIterThreads)
    gspat_iterate_kernel(const float2* __restrict__ r, const float* __restrict__ amps, int64_t m,
                         int repeat, float2* p, float2* gamma) {
    dev::pdl_wait();
    dev::pdl_release();
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) p[i] = make_float2(amps[i], 0.f);
    __syncthreads();
    for (int it = 0;; ++it) {
        block_matvec(r, p, gamma, m);
        __syncthreads();
        if (it == repeat) break;
        for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
            const float2 gv = gamma[i];
            const float s = amps[i] / hypotf(gv.x, gv.y);
            p[i] = make_float2(gv.x * s, gv.y * s);
        }
        __syncthreads();
    }
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        const float2 gv = gamma[i];
        const float a = hypotf(gv.x, gv.y);
        const float s = amps[i] * amps[i] / (a * a);
        p[i] = make_float2(gv.x * s, gv.y * s);
    }
}

// The same iteration for up to kGspatSmemFoci foci, R held in shared memory and every row of a
// product summed at once: kGspatRowThreads threads per row, thread `sub` summing columns sub,
// sub + 16, ... in order, then the 16 partial sums added by a butterfly within the half-warp.
// The row's first thread writes the row's new p into the other half of a double buffer, so one
// barrier per iteration separates an iteration's reads of p from the next one's writes.
constexpr int64_t kGspatSmemFoci = 64;
constexpr int kGspatRowThreads = 16;

__global__ void __launch_bounds__(kGspatSmemFoci * kGspatRowThreads, 1)
    gspat_iterate_smem_kernel(const float2* __restrict__ r, const float* __restrict__ amps,
                              int m, int repeat, float2* __restrict__ p_out) {
    __shared__ float2 s_r[kGspatSmemFoci * kGspatSmemFoci];
    __shared__ float2 s_p[2][kGspatSmemFoci];
    __shared__ float s_amp[kGspatSmemFoci];
    dev::pdl_wait();
    dev::pdl_release();
    for (int i = threadIdx.x; i < m * m; i += blockDim.x) s_r[i] = r[i];
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        s_amp[i] = amps[i];
        s_p[0][i] = make_float2(amps[i], 0.f);
    }
    __syncthreads();
    const int row = threadIdx.x / kGspatRowThreads, sub = threadIdx.x % kGspatRowThreads;
    const bool live = row < m;  // the block is whole warps: the last half-warp may have no row
    const float2* rr = s_r + (live ? row : 0) * m;
    int cur = 0;
    for (int it = 0;; ++it) {
        const float2* p = s_p[cur];
        float2 acc = make_float2(0.f, 0.f);
        if (live) {
            for (int c = sub; c < m; c += kGspatRowThreads) {
                const float2 t = cmul(rr[c], p[c]);
                acc.x += t.x;
                acc.y += t.y;
            }
        }
#pragma unroll
        for (int o = kGspatRowThreads / 2; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        }
        if (live && sub == 0) {
            if (it == repeat) {
                const float a = hypotf(acc.x, acc.y);
                const float s = s_amp[row] * s_amp[row] / (a * a);
                p_out[row] = make_float2(acc.x * s, acc.y * s);
            } else {
                const float s = s_amp[row] / hypotf(acc.x, acc.y);
                s_p[cur ^ 1][row] = make_float2(acc.x * s, acc.y * s);
            }
        }
        if (it == repeat) break;
        cur ^= 1;
        __syncthreads();
    }
}

// q_j = scale_j * sum_i conj(G_ij) p_i; writes (|q_j|, arg q_j).  scale = inv_den2 or 1.
__global__ void backpropagate_kernel(const float2* __restrict__ g, const float* __restrict__ scale,
                                     const float2* __restrict__ p, int64_t n, int64_t m,
                                     float* __restrict__ out) {
    dev::pdl_wait();
    dev::pdl_release();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 8
    for (int64_t i = 0; i < m; ++i) {
        const float2 t = cmulc(g[i * n + j], p[i]);
        acc.x += t.x;
        acc.y += t.y;
    }
    const float s = scale ? scale[j] : 1.0f;
    acc.x *= s;
    acc.y *= s;
    out[2 * j] = hypotf(acc.x, acc.y);
    out[2 * j + 1] = atan2f(acc.y, acc.x);
}

// Gerchberg-Saxton (gs.rs:42-77) in one block; q0 are the sources' amplitudes.
__global__ void __launch_bounds__(kIterThreads)
    gs_iterate_kernel(const float2* __restrict__ g, const PackedSource* __restrict__ src,
                      const float* __restrict__ amps, int64_t n, int64_t m, int repeat, float2* q,
                      float2* p, float* __restrict__ out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) q[j] = make_float2(src[j].c.z, 0.f);
    __syncthreads();
    for (int it = 0; it < repeat; ++it) {
        // gamma = G q, p = gamma / |gamma| * p0
        for (int64_t row = wid; row < m; row += nw) {
            float2 acc = make_float2(0.f, 0.f);
            for (int64_t j = lane; j < n; j += 32) {
                const float2 t = cmul(g[row * n + j], q[j]);
                acc.x += t.x;
                acc.y += t.y;
            }
            acc = warp_sum(acc);
            if (lane == 0) {
                const float s = amps[row] / hypotf(acc.x, acc.y);
                p[row] = make_float2(acc.x * s, acc.y * s);
            }
        }
        __syncthreads();
        // xi = G^H p, q = xi / |xi| * q0
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            float2 acc = make_float2(0.f, 0.f);
            for (int64_t i = 0; i < m; ++i) {
                const float2 t = cmulc(g[i * n + j], p[i]);
                acc.x += t.x;
                acc.y += t.y;
            }
            const float s = src[j].c.z / hypotf(acc.x, acc.y);
            q[j] = make_float2(acc.x * s, acc.y * s);
        }
        __syncthreads();
    }
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const float2 v = q[j];
        out[2 * j] = hypotf(v.x, v.y);
        out[2 * j + 1] = atan2f(v.y, v.x);
    }
}

// Greedy (greedy.rs:39-83) in one block.  Source i (in order) tries every candidate phasor
// c_k: thread k sums |amp_j - |G_ji c_k + cache_j|| over the foci j in order (f32, no
// contraction, as the reference); the first minimum wins; cache_j += G_ji c_best.
__global__ void __launch_bounds__(kIterThreads)
    greedy_kernel(const float2* __restrict__ g, const PackedSource* __restrict__ src, int64_t n,
                  int64_t m, const float* __restrict__ amps, const float2* __restrict__ cand,
                  const float* __restrict__ cand_arg, int div, float2* cache,
                  float* __restrict__ out) {
    __shared__ float s_v[kGreedyMaxDiv];
    __shared__ int s_best;
    for (int64_t j = threadIdx.x; j < m; j += blockDim.x) cache[j] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int64_t i = 0; i < n; ++i) {
        if (threadIdx.x < div) {
            const float2 c = cand[threadIdx.x];
            float v = 0.f;
            for (int64_t j = 0; j < m; ++j) {
                const float2 a = g[j * n + i];
                const float2 t = make_float2(__fsub_rn(__fmul_rn(a.x, c.x), __fmul_rn(a.y, c.y)),
                                             __fadd_rn(__fmul_rn(a.x, c.y), __fmul_rn(a.y, c.x)));
                const float2 q = cache[j];
                const float re = __fadd_rn(t.x, q.x), im = __fadd_rn(t.y, q.y);
                v = __fadd_rn(v, fabsf(__fsub_rn(amps[j], hypotf(re, im))));
            }
            s_v[threadIdx.x] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int best = 0;
            float min_v = __int_as_float(0x7f800000);  // +inf
            for (int k = 0; k < div; ++k) {
                if (s_v[k] < min_v) {
                    min_v = s_v[k];
                    best = k;
                }
            }
            s_best = best;
            out[2 * i] = src[i].c.z;
            out[2 * i + 1] = cand_arg[best];
        }
        __syncthreads();
        const float2 c = cand[s_best];
        for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
            const float2 a = g[j * n + i];
            const float2 t = make_float2(__fsub_rn(__fmul_rn(a.x, c.x), __fmul_rn(a.y, c.y)),
                                         __fadd_rn(__fmul_rn(a.x, c.y), __fmul_rn(a.y, c.x)));
            cache[j] = make_float2(__fadd_rn(cache[j].x, t.x), __fadd_rn(cache[j].y, t.y));
        }
        __syncthreads();
    }
}

__global__ void real_to_complex_kernel(const float* __restrict__ v, int64_t m,
                                       float2* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < m) out[i] = make_float2(v[i], 0.f);
}

__global__ void fill_amp_phase_kernel(float* out, int64_t n, float amp, float phase) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    out[2 * j] = amp;
    out[2 * j + 1] = phase;
}

unsigned blocks_for(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

size_t solver_workspace_bytes(int64_t n, int64_t m) {
    return align256(sizeof(PackedSource) * n) + align256(sizeof(float2) * n * m) +
           align256(sizeof(float) * n) + align256(sizeof(float2) * m * m) +
           2 * align256(sizeof(float2) * m) + align256(sizeof(float2) * n);
}

cudaError_t launch_build_g(int st, const float* d_raw, const float* d_k, const float* d_atten,
                           int64_t n, const float* d_foci, int64_t m, float2* d_g,
                           void* ws_packed, cudaStream_t s) {
    if (n <= 0 || m <= 0) return cudaSuccess;
    if (m > 65535) return cudaErrorInvalidValue;
    PackedSource* packed = static_cast<PackedSource*>(ws_packed);
    cudaError_t e = launch_pack_sources(st, d_raw, d_k, d_atten, n, packed, s);
    if (e != cudaSuccess) return e;
    const dim3 grid(blocks_for(n, 128), static_cast<unsigned>(m));
    const bool pdl = !stream_capturing(s);
    e = st == SRC_T4010A1
            ? launch_after(build_g_kernel<SRC_T4010A1>, grid, dim3(128), 0, s, pdl, packed, n,
                           d_foci, m, d_g)
            : launch_after(build_g_kernel<SRC_SPHERE>, grid, dim3(128), 0, s, pdl, packed, n,
                           d_foci, m, d_g);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_greedy(int st, const float* d_raw, const float* d_k, const float* d_atten,
                          int64_t n, const float* d_foci, const float* d_amps, int64_t m,
                          const float2* d_cand, const float* d_cand_arg, int div, float* d_out,
                          void* ws, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (m > kSolverMaxFoci || div < 1 || div > kGreedyMaxDiv) return cudaErrorInvalidValue;
    SolverWs w = carve(ws, n, m);
    cudaError_t e = launch_build_g(st, d_raw, d_k, d_atten, n, d_foci, m, w.g, w.packed, s);
    if (e != cudaSuccess) return e;
    if (m == 0) {
        // no foci: launch_build_g did nothing; the packed sources still carry the amplitudes
        if ((e = launch_pack_sources(st, d_raw, d_k, d_atten, n, w.packed, s)) != cudaSuccess)
            return e;
    }
    greedy_kernel<<<1, kIterThreads, 0, s>>>(w.g, w.packed, n, m, d_amps, d_cand, d_cand_arg, div,
                                             w.p, d_out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_solver(int kind, int st, const float* d_raw, const float* d_k,
                          const float* d_atten, int64_t n, const float* d_foci,
                          const float* d_amps, int64_t m, int repeat, float* d_out, void* ws,
                          cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (m > kSolverMaxFoci || repeat < 0) return cudaErrorInvalidValue;
    SolverWs w = carve(ws, n, m);
    if (m == 0) {
        // An empty focus list leaves q = 0 (GS-PAT, naive) or q = NaN (GS, normalising zero).
        const float v = kind == SOLVER_GS ? __builtin_nanf("") : 0.f;
        fill_amp_phase_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d_out, n, v, v);
        count_launch();
        return cudaGetLastError();
    }
    cudaError_t e = launch_build_g(st, d_raw, d_k, d_atten, n, d_foci, m, w.g, w.packed, s);
    if (e != cudaSuccess) return e;
    if (kind == SOLVER_GSPAT) {
        // each launch a programmatic dependent of the one before (the kernels wait first)
        const bool pdl = !stream_capturing(s);
        if ((e = launch_after(column_abs_sum_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, s, pdl,
                              static_cast<const float2*>(w.g), n, m, w.inv_den2)) != cudaSuccess)
            return e;
        if ((e = launch_after(gspat_r_kernel, dim3(static_cast<unsigned>(m), static_cast<unsigned>(m)),
                              dim3(128), 0, s, pdl, static_cast<const float2*>(w.g),
                              static_cast<const float*>(w.inv_den2), n, m, w.r)) != cudaSuccess)
            return e;
        if (m <= kGspatSmemFoci) {
            const unsigned threads = static_cast<unsigned>((m * kGspatRowThreads + 31) / 32 * 32);
            e = launch_after(gspat_iterate_smem_kernel, dim3(1), dim3(threads), 0, s, pdl,
                             static_cast<const float2*>(w.r), d_amps, static_cast<int>(m), repeat,
                             w.p);
        } else {
            e = launch_after(gspat_iterate_kernel, dim3(1), dim3(kIterThreads), 0, s, pdl,
                             static_cast<const float2*>(w.r), d_amps, m, repeat, w.p, w.gamma);
        }
        if (e != cudaSuccess) return e;
        if ((e = launch_after(backpropagate_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, s, pdl,
                              static_cast<const float2*>(w.g),
                              static_cast<const float*>(w.inv_den2),
                              static_cast<const float2*>(w.p), n, m, d_out)) != cudaSuccess)
            return e;
        count_launch(4);
    } else if (kind == SOLVER_NAIVE) {
        real_to_complex_kernel<<<blocks_for(m, 256), 256, 0, s>>>(d_amps, m, w.p);
        backpropagate_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w.g, nullptr, w.p, n, m, d_out);
        count_launch(2);
    } else if (kind == SOLVER_GS) {
        gs_iterate_kernel<<<1, kIterThreads, 0, s>>>(w.g, w.packed, d_amps, n, m, repeat, w.q, w.p,
                                                     d_out);
        count_launch();
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

namespace {

// Host-level solver state: one stream and grow-only buffers shared by all systems.
struct SolverCtx {
    std::mutex mu;
    int device = -1;
    cudaStream_t stream = nullptr;
    void* d_in = nullptr;
    size_t d_in_cap = 0;
    void* d_ws = nullptr;
    size_t d_ws_cap = 0;
    float* h_io = nullptr;
    size_t h_io_cap = 0;
};

SolverCtx g_solver;

cudaError_t grow_dev(void** p, size_t* cap, size_t bytes) {
    if (bytes <= *cap) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) *cap = bytes;
    return e;
}

}  // namespace

int solve_multi_focus(int kind, int st, float* src, const float* k, const float* atten,
                      int64_t n, const float* foci, const float* amps, int64_t m,
                      std::string* err, int phase_div) {
    if (m > kSolverMaxFoci) {
        *err = "too many foci (" + std::to_string(m) + " > " + std::to_string(kSolverMaxFoci) + ")";
        return -1;
    }
    const bool greedy = kind == SOLVER_GREEDY;
    if (greedy && (phase_div < 1 || phase_div > kGreedyMaxDiv)) {
        *err = "phase_div must be 1.." + std::to_string(kGreedyMaxDiv);
        return -1;
    }
    if (n == 0) return 0;
    std::lock_guard<std::mutex> lock(g_solver.mu);
    SolverCtx& c = g_solver;
    cudaError_t e;
    auto fail = [&](const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return -1;
    };
    if (!c.stream) {
        int count = 0;
        e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            *err = "no CUDA device available; this library has no CPU path";
            return -1;
        }
        if ((e = cudaGetDevice(&c.device)) != cudaSuccess) return fail("cudaGetDevice");
        if ((e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) != cudaSuccess) {
            c.stream = nullptr;
            return fail("cudaStreamCreate");
        }
    }
    DeviceGuard dg;  // the solver's device while it runs; the caller's again on return
    if ((e = dg.set(c.device)) != cudaSuccess) return fail("cudaSetDevice");
    const int stride = source_stride(st);
    // input block: raw | k | atten | foci | amps [| candidate phasors | their arguments, from a
    // 16-byte boundary] ; output: 2n floats
    const size_t base_floats = static_cast<size_t>(n) * (stride + 2) + 4 * static_cast<size_t>(m);
    const size_t cand_off = (base_floats + 3) & ~static_cast<size_t>(3);
    const size_t in_floats = greedy ? cand_off + 3 * static_cast<size_t>(phase_div) : base_floats;
    const size_t io_floats = in_floats > static_cast<size_t>(2 * n) ? in_floats : 2 * n;
    if (io_floats * sizeof(float) > c.h_io_cap) {
        if (c.h_io) cudaFreeHost(c.h_io);
        c.h_io = nullptr;
        c.h_io_cap = 0;
        if ((e = cudaHostAlloc(&c.h_io, io_floats * sizeof(float), cudaHostAllocDefault)) !=
            cudaSuccess)
            return fail("cudaHostAlloc");
        c.h_io_cap = io_floats * sizeof(float);
    }
    float* h = c.h_io;
    memcpy(h, src, sizeof(float) * n * stride);
    memcpy(h + n * stride, k, sizeof(float) * n);
    memcpy(h + n * (stride + 1), atten, sizeof(float) * n);
    memcpy(h + n * (stride + 2), foci, sizeof(float) * 3 * m);
    memcpy(h + n * (stride + 2) + 3 * m, amps, sizeof(float) * m);
    if (greedy) {
        // greedy.rs:21-27: exp(i 2 pi k / phase_div) in f32 (num-complex exp = from_polar(e^0, a))
        // and, for set_phase, their arguments (greedy.rs:79)
        float* hc = h + cand_off;
        for (int q = 0; q < phase_div; ++q) {
            const float a = 2.0f * kPiF * static_cast<float>(q) / static_cast<float>(phase_div);
            hc[2 * q] = 1.0f * cosf(a);
            hc[2 * q + 1] = 1.0f * sinf(a);
            hc[2 * phase_div + q] = atan2f(hc[2 * q + 1], hc[2 * q]);
        }
    }
    const size_t in_bytes = align256(in_floats * sizeof(float)) + align256(2 * n * sizeof(float));
    if ((e = grow_dev(&c.d_in, &c.d_in_cap, in_bytes)) != cudaSuccess) return fail("cudaMalloc");
    if ((e = grow_dev(&c.d_ws, &c.d_ws_cap, solver_workspace_bytes(n, m))) != cudaSuccess)
        return fail("cudaMalloc");
    float* d = static_cast<float*>(c.d_in);
    float* d_out = reinterpret_cast<float*>(static_cast<char*>(c.d_in) +
                                            align256(in_floats * sizeof(float)));
    if ((e = cudaMemcpyAsync(d, h, in_floats * sizeof(float), cudaMemcpyHostToDevice, c.stream)) !=
        cudaSuccess)
        return fail("cudaMemcpyAsync");
    if (greedy)
        e = launch_greedy(st, d, d + n * stride, d + n * (stride + 1), n, d + n * (stride + 2),
                          d + n * (stride + 2) + 3 * m, m,
                          reinterpret_cast<const float2*>(d + cand_off),
                          d + cand_off + 2 * phase_div, phase_div, d_out, c.d_ws, c.stream);
    else
        e = launch_solver(kind, st, d, d + n * stride, d + n * (stride + 1), n,
                          d + n * (stride + 2), d + n * (stride + 2) + 3 * m, m, kSolverRepeat,
                          d_out, c.d_ws, c.stream);
    if (e != cudaSuccess) return fail("solver launch");
    if ((e = cudaMemcpyAsync(h, d_out, 2 * n * sizeof(float), cudaMemcpyDeviceToHost, c.stream)) !=
        cudaSuccess)
        return fail("cudaMemcpyAsync");
    if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return fail("solver");
    const int iamp = st == SRC_T4010A1 ? 6 : 3;
    const int iphase = st == SRC_T4010A1 ? 7 : 4;
    for (int64_t j = 0; j < n; ++j) {
        src[j * stride + iamp] = h[2 * j];
        src[j * stride + iphase] = h[2 * j + 1];
    }
    return 0;
}

}  // namespace afc
