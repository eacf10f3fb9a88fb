// Grid field evaluation tiled by rows: the per-block body of field_rows_kernel.
//
// A block covers TX consecutive indices along the grid's first axis times TY consecutive
// indices along its second axis, in one plane of the third.  Each thread owns one first-axis
// index and 2*PAIRS consecutive second-axis indices, so its points share two of their three
// coordinates.  Sources are staged with their coordinates and directions permuted into the
// grid's axis order; per source and thread, the offsets along the first and third axes, the
// sum of their squares and (for tiles of unequal directions) their part of n.d are computed
// once, and each point pair only adds the offset along the second axis: three fewer packed
// FP32 instructions per pair than the general body (field_body.cuh), whose math this is.  The
// directivity comes from the cos(theta)-indexed table (directivity2_ctab), and a thread keeps
// the smallest |c - L| of its points for the exact edge path.  Points and the order of the sum
// over sources are the reference's (observe_area/grid/grid_area.rs:59-229,
// system/uniform_medium.rs:111-128).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"
#include "field_body.cuh"
#include "propagate.cuh"

namespace afc {
namespace fb {

__device__ __forceinline__ float pick3(float x, float y, float z, int a) {
    return a == 0 ? x : (a == 1 ? y : z);
}

// Per thread and source: offsets along the grid's first (v) and third (w) axes, v^2 + w^2,
// and n_v v + n_w w; for the far tiles also qb, qc with which the reference's
// (dx dx + dy dy) + dz dz is (du du + qb) + qc in the same rounding (see row_q2_parts).
struct RowShared {
    float dv, dw, vw2, nvw, qb, qc;
};

// The reference sums the squared offsets in x, y, z order (uniform_medium.rs:111-113); the rows
// body has the second grid axis's (u) per pair and the others' per source.  With a1 the xyz
// index of u and a0 that of v: u = z gives (du du + (sx + sy)) + 0, u = x gives
// (du du + sy) + sz and u = y gives (du du + sx) + sz, each rounding as the reference's sum
// (an addition commutes exactly, and adding +0 to a non-negative sum changes nothing).
__device__ __forceinline__ void row_q2_parts(float dv, float dw, int a0, int a1, float& qb,
                                             float& qc) {
    const float sv = __fmul_rn(dv, dv), sw = __fmul_rn(dw, dw);
    if (a1 == 2) {
        qb = __fadd_rn(sv, sw);
        qc = 0.f;
    } else {
        qb = a1 == 0 ? (a0 == 1 ? sv : sw) : (a0 == 0 ? sv : sw);  // y for u = x, x for u = y
        qc = a0 == 2 ? sv : sw;                                      // z
    }
}

// Point pair q of a thread against the staged source: offset along the second axis, r^2, 1/r,
// the numerator of cos(theta) and cos(theta), with the same operations on the hot loop and on
// its edge path.
template <bool UD>
struct RowGeom {
    float2 du, r2, rinv, cn, ct;
    __device__ __forceinline__ RowGeom(float2 u, float2 np, const RowShared& sh, float4 v0,
                                       float4 v2, float2 ns) {
        du = add2(u, hi2(v0));
        r2 = fma2(du, du, f2(sh.vw2));
        rinv = make_float2(mufu_rsqrt(r2.x), mufu_rsqrt(r2.y));
        if constexpr (UD) cn = add2(np, ns);
        else cn = fma2(hi2(v2), du, f2(sh.nvw));
        ct = mul2(cn, rinv);
    }
};

// Edge correction for one point of the rows body (see edge_correction): the pair is
// recomputed from the offsets as the hot loop computed it; the reference's bin needs the
// offsets and the direction back in x, y, z order (a0, a1, a2: the xyz index of each grid
// axis).
static __device__ __noinline__ float2 edge_correction_rows(const float4* __restrict__ tab,
                                                           const float* __restrict__ cneg,
                                                           const float4* __restrict__ ccoef,
                                                           float du, float dv, float dw, float vw2,
                                                           float cn, float n_a0, float n_a1,
                                                           float n_a2, int a0, int a1, float k,
                                                           float phase, float a2c, float la) {
    const float r2 = fmaf(du, du, vw2);
    const float rinv = mufu_rsqrt(r2);
    const float ct = cn * rinv;
    float2 t;
    const float d_fast = directivity2_ctab(cneg, ccoef, make_float2(ct, ct), t).x;
    const float thc = theta2_centred(make_float2(ct, ct)).x;
    // back to x, y, z: the first grid axis carries v, the second u, the third w
    const float dx = a0 == 0 ? dv : (a1 == 0 ? du : dw);
    const float dy = a0 == 1 ? dv : (a1 == 1 ? du : dw);
    const float dz = a0 == 2 ? dv : (a1 == 2 ? du : dw);
    const float nx = a0 == 0 ? n_a0 : (a1 == 0 ? n_a1 : n_a2);
    const float ny = a0 == 1 ? n_a0 : (a1 == 1 ? n_a1 : n_a2);
    const float nz = a0 == 2 ? n_a0 : (a1 == 2 ? n_a1 : n_a2);
    const int i_exact = exact_bin(dx, dy, dz, nx, ny, nz);
    float2 r;
    const float red =
        ref_phase2(ref_dist2(f2(dx), f2(dy), f2(dz)), f2(rinv), f2(k), f2(phase), r).x;
    const float w0 = rinv * mufu_ex2(fmaf(a2c, r.x, la));
    const float corr = w0 * (dir_in_bin(tab, thc, i_exact) - d_fast);
    return make_float2(corr * mufu_cos(red), corr * mufu_sin(red));
}

// The PAIRS point pairs of one thread against shared-memory source j (staged in grid axis
// order: v0 = (-s_a0, -s_a0, -s_a1, -s_a1), v1 = (-s_a2, -s_a2, k, k), v2 = (n_a0, n_a0, n_a1,
// n_a1), v3 = (n_a2, n_a2, a2, a2)).  p0, p2: the thread's coordinates along the first and
// third grid axes; U: its points' coordinates along the second; n0a: the shared direction (of
// source 0) in grid axis order, which every source of a UD tile has.
template <int ST, int SUM, int PAIRS, bool UD, int PH>
__device__ __forceinline__ void accumulate_rows(const SmemTile& sm, const RowsTable& rt, int j,
                                                float p0, float p2,
                                                int a0, int a1, float3 n0a, float2 (&U)[PAIRS],
                                                float2 (&NP)[PAIRS], float2 (&RE)[PAIRS],
                                                float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                                float2 (&CIM)[PAIRS]) {
    const float4 v0 = sm.v0[j], v1 = sm.v1[j], v3 = sm.v3[j], v4 = sm.v4[j];
    float4 v2 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 ns = f2(0.f);
    if constexpr (ST == SRC_T4010A1) {
        if constexpr (UD) ns = sm.ns[j];
        else v2 = sm.v2[j];
    }
    RowShared sh;
    sh.dv = p0 + v0.x;
    sh.dw = p2 + v1.x;
    sh.vw2 = fmaf(sh.dw, sh.dw, sh.dv * sh.dv);
    sh.nvw = 0.f;
    if constexpr (ST == SRC_T4010A1 && !UD) sh.nvw = fmaf(v3.x, sh.dw, v2.x * sh.dv);
    sh.qb = sh.qc = 0.f;
    if constexpr (PH == kPhaseRef) row_q2_parts(sh.dv, sh.dw, a0, a1, sh.qb, sh.qc);
    float near_min = kCTabMargin;  // smallest |c - L| of the thread's points (the edge test)
#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        const RowGeom<UD> p(U[q], NP[q], sh, v0, v2, ns);
        float2 r = mul2(p.r2, p.rinv);
        float2 red;
        if constexpr (PH == kPhaseRef) {
            const float2 q2 =
                make_float2(__fadd_rn(__fadd_rn(__fmul_rn(p.du.x, p.du.x), sh.qb), sh.qc),
                            __fadd_rn(__fadd_rn(__fmul_rn(p.du.y, p.du.y), sh.qb), sh.qc));
            red = ref_phase2(q2, p.rinv, hi2(v1), hi2(v4), r);
        } else if constexpr (PH == kPhaseMid) {
            red = mid_phase2(p.r2, p.rinv, hi2(v1), hi2(v4), r);
        } else {
            red = fma2(hi2(v1), r, hi2(v4));
        }
        const float2 ea = fma2(hi2(v3), r, lo2(v4));
        float2 w = mul2(p.rinv, make_float2(mufu_ex2(ea.x), mufu_ex2(ea.y)));
        if constexpr (ST == SRC_T4010A1) {
            float2 t;
            w = mul2(w, directivity2_ctab(rt.cneg, rt.ccoef, p.ct, t));
            near_min = fminf(near_min, fminf(fabsf(t.x), fabsf(t.y)));
        }
        const float2 sn = make_float2(mufu_sin(red.x), mufu_sin(red.y));
        const float2 cs = make_float2(mufu_cos(red.x), mufu_cos(red.y));
        if constexpr (SUM == SUM_PLAIN) {
            RE[q] = fma2(w, cs, RE[q]);
            IM[q] = fma2(w, sn, IM[q]);
        } else {
            const float2 tr = mul2(w, cs), ti = mul2(w, sn);
            neumaier_add(RE[q].x, CRE[q].x, tr.x);
            neumaier_add(RE[q].y, CRE[q].y, tr.y);
            neumaier_add(IM[q].x, CIM[q].x, ti.x);
            neumaier_add(IM[q].y, CIM[q].y, ti.y);
        }
    }
    if constexpr (ST == SRC_T4010A1) {
        if (near_min < kCTabMargin) {
            const float n_a0 = UD ? n0a.x : v2.x, n_a1 = UD ? n0a.y : v2.z,
                        n_a2 = UD ? n0a.z : v3.x;
#pragma unroll
            for (int q = 0; q < PAIRS; ++q) {
                const RowGeom<UD> p(U[q], NP[q], sh, v0, v2, ns);
                float2 t;
                directivity2_ctab(rt.cneg, rt.ccoef, p.ct, t);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (!near_edge_c(lane_of(t, h))) continue;
                    const float2 c = edge_correction_rows(
                        sm.dir, rt.cneg, rt.ccoef, lane_of(p.du, h), sh.dv, sh.dw, sh.vw2, lane_of(p.cn, h), n_a0,
                        n_a1, n_a2, a0, a1, v1.z, v4.z, v3.z, v4.x);
                    if constexpr (SUM == SUM_PLAIN) {
                        lane_of(RE[q], h) += c.x;
                        lane_of(IM[q], h) += c.y;
                    } else {
                        neumaier_add(lane_of(RE[q], h), lane_of(CRE[q], h), c.x);
                        neumaier_add(lane_of(IM[q], h), lane_of(CIM[q], h), c.y);
                    }
                }
            }
        }
    }
}

// Sources 0 .. cnt - 1 of the staged tile against the thread's points (accumulate_rows), with
// the tile's phase variant (MID: whether the mid tier is compiled in; without it, mid tiles take
// the careful variant).
template <int ST, int SUM, int PAIRS, bool UD, bool MID>
__device__ __forceinline__ void rows_source_loop(int ph, int cnt, const SmemTile& sm,
                                                 const RowsTable& rt, float p0, float p2, int a0,
                                                 int a1, float3 n0a, float2 (&U)[PAIRS],
                                                 float2 (&NP)[PAIRS], float2 (&RE)[PAIRS],
                                                 float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                                 float2 (&CIM)[PAIRS]) {
    if (ph == kPhaseFast) {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_rows<ST, SUM, PAIRS, UD, kPhaseFast>(sm, rt, j, p0, p2, a0, a1, n0a, U, NP,
                                                            RE, IM, CRE, CIM);
    } else if (MID && ph == kPhaseMid) {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_rows<ST, SUM, PAIRS, UD, kPhaseMid>(sm, rt, j, p0, p2, a0, a1, n0a, U, NP,
                                                           RE, IM, CRE, CIM);
    } else {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_rows<ST, SUM, PAIRS, UD, kPhaseRef>(sm, rt, j, p0, p2, a0, a1, n0a, U, NP,
                                                           RE, IM, CRE, CIM);
    }
}

// Coordinate of index i along grid axis k (xyz index a), bit-identical to the reference's
// o + (i as f32 * res); a fixed axis (count 1) stays at its origin.
__device__ __forceinline__ float axis_coord(const GridDev& g, int k, int a, int64_t i) {
    const float o = pick3(g.origin[0], g.origin[1], g.origin[2], a);
    return g.count[k] > 1 ? __fadd_rn(o, __fmul_rn(__ll2float_rn(i), g.res)) : o;
}

// One tile of the rows tiling (tile index -> (t0, t1) of plane i2; TX = 1 << tx_log2): the sums
// of sources s_lo .. s_hi - 1 at the thread's points, in RE, IM (CRE, CIM: compensations).
// Source 0's direction is the shared direction of the fast cos(theta) whatever the range.
template <int ST, int SUM, int PAIRS, bool MID = false>
__device__ __forceinline__ void rows_accumulate(SmemTile& sm, const RowsTable& rt,
                                                const PackedSource* __restrict__ src,
                                                int64_t n, int64_t s_lo, int64_t s_hi,
                                                const GridDev& g, int tx_log2, int64_t tiles0,
                                                int64_t tiles1, int64_t tile, float2 (&RE)[PAIRS],
                                                float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                                float2 (&CIM)[PAIRS]) {
    constexpr int kPPT = 2 * PAIRS;
    const int tx = threadIdx.x & ((1 << tx_log2) - 1);
    const int ty = threadIdx.x >> tx_log2;
    const int64_t t0 = tile % tiles0, rest = tile / tiles0;
    const int64_t t1 = rest % tiles1, i2 = rest / tiles1;
    const int64_t c0 = g.count[0], c1 = g.count[1];
    const int64_t i0 = (t0 << tx_log2) + tx;
    const int64_t i1b = (t1 * (kThreads >> tx_log2) + ty) * kPPT;
    const int a0 = g.axis[0], a1 = g.axis[1], a2 = g.axis[2];
    const float p0 = axis_coord(g, 0, a0, i0 < c0 ? i0 : c0 - 1);
    const float p2 = axis_coord(g, 2, a2, i2);

    float2 U[PAIRS], NP[PAIRS];
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        const int64_t i1 = i1b + k < c1 ? i1b + k : c1 - 1;  // computed but never stored
        lane_of(U[k >> 1], k & 1) = axis_coord(g, 1, a1, i1);
    }
    // direction of source 0: the reference direction of the shared-direction path
    float3 n0 = make_float3(0.f, 0.f, 0.f);
    if (ST == SRC_T4010A1 && n > 0) {
        const float4 b0 = src[0].b;
        n0 = make_float3(b0.x, b0.y, b0.z);
    }
    const float n0_a0 = pick3(n0.x, n0.y, n0.z, a0), n0_a1 = pick3(n0.x, n0.y, n0.z, a1),
                n0_a2 = pick3(n0.x, n0.y, n0.z, a2);
    const float npc = fmaf(n0_a2, p2, n0_a0 * p0);
    const float3 n0a = make_float3(n0_a0, n0_a1, n0_a2);
#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        NP[q] = fma2(f2(n0_a1), U[q], f2(npc));
        RE[q] = f2(0.f);
        IM[q] = f2(0.f);
        CRE[q] = f2(0.f);
        CIM[q] = f2(0.f);
    }

    // bounding box of the block's points in x, y, z (for the phase bound of each source tile)
    {
        float umin = U[0].x, umax = U[0].x;
#pragma unroll
        for (int k = 1; k < kPPT; ++k) {
            umin = fminf(umin, lane_of(U[k >> 1], k & 1));
            umax = fmaxf(umax, lane_of(U[k >> 1], k & 1));
        }
        float lo[3], hi[3];
        lo[0] = p0, hi[0] = p0, lo[1] = umin, hi[1] = umax, lo[2] = p2, hi[2] = p2;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
                hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
            }
        }
        if ((threadIdx.x & 31) == 0) {
            // grid-axis order (0: first, 1: second, 2: third) -> x, y, z slots
            const int ax[3] = {a0, a1, a2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sm.box[threadIdx.x >> 5][ax[c]] = lo[c];
                sm.box[threadIdx.x >> 5][3 + ax[c]] = hi[c];
            }
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            const int a = threadIdx.x;
            float v = sm.box[0][a];
#pragma unroll
            for (int w = 1; w < kThreads / 32; ++w)
                v = a < 3 ? fminf(v, sm.box[w][a]) : fmaxf(v, sm.box[w][a]);
            sm.bbox[a] = v;
        }
        __syncthreads();
    }

    for (int64_t s0 = s_lo; s0 < s_hi; s0 += kTile) {
        const int cnt = static_cast<int>((s_hi - s0) < kTile ? (s_hi - s0) : kTile);
        __syncthreads();
        bool same_dir = true, small_phase = true, mid_phase = true;
        for (int j = threadIdx.x; j < cnt; j += kThreads) {
            const PackedSource s = src[s0 + j];
            const float fx = fmaxf(fabsf(sm.bbox[0] - s.a.x), fabsf(sm.bbox[3] - s.a.x));
            const float fy = fmaxf(fabsf(sm.bbox[1] - s.a.y), fabsf(sm.bbox[4] - s.a.y));
            const float fz = fmaxf(fabsf(sm.bbox[2] - s.a.z), fabsf(sm.bbox[5] - s.a.z));
            const float rmax = sqrtf(fmaf(fz, fz, fmaf(fy, fy, fx * fx)));
            const float bound = fmaf(fabsf(s.a.w), rmax, fabsf(s.c.y));
            small_phase = small_phase && bound <= kUnreducedPhaseMax;
            mid_phase = mid_phase && bound <= kMidPhaseMax;
            const float s0_ = pick3(s.a.x, s.a.y, s.a.z, a0), s1_ = pick3(s.a.x, s.a.y, s.a.z, a1),
                        s2_ = pick3(s.a.x, s.a.y, s.a.z, a2);
            const float m0 = pick3(s.b.x, s.b.y, s.b.z, a0), m1 = pick3(s.b.x, s.b.y, s.b.z, a1),
                        m2 = pick3(s.b.x, s.b.y, s.b.z, a2);
            sm.v0[j] = make_float4(-s0_, -s0_, -s1_, -s1_);
            sm.v1[j] = make_float4(-s2_, -s2_, s.a.w, s.a.w);
            sm.v2[j] = make_float4(m0, m0, m1, m1);
            sm.v3[j] = make_float4(m2, m2, s.b.w, s.b.w);
            sm.v4[j] = make_float4(s.c.x, s.c.x, s.c.y, s.c.y);
            const float ns = fmaf(n0_a2, s2_, fmaf(n0_a1, s1_, n0_a0 * s0_));
            sm.ns[j] = f2(-ns);
            same_dir = same_dir && s.b.x == n0.x && s.b.y == n0.y && s.b.z == n0.z;
        }
        const bool tile_same_dir = __syncthreads_and(same_dir);
        const bool tile_small = __syncthreads_and(small_phase);
        const bool tile_mid = __syncthreads_and(mid_phase);
        const int tile_ph = tile_small ? kPhaseFast : ((MID && tile_mid) ? kPhaseMid : kPhaseRef);
        if (ST == SRC_T4010A1 && tile_same_dir)
            rows_source_loop<ST, SUM, PAIRS, true, MID>(tile_ph, cnt, sm, rt, p0, p2, a0, a1, n0a, U,
                                                        NP, RE, IM, CRE, CIM);
        else
            rows_source_loop<ST, SUM, PAIRS, false, MID>(tile_ph, cnt, sm, rt, p0, p2, a0, a1, n0a, U,
                                                         NP, RE, IM, CRE, CIM);
    }

}

// Store the thread's sums of one tile of the rows tiling (field transform applied); points
// whose sum is NaN are then passed to fix_coincident with the n sources src.
template <int SUM, int PAIRS>
__device__ __forceinline__ void rows_store(const PackedSource* __restrict__ src, int64_t n,
                                           const GridDev& g, int tx_log2, int64_t tiles0,
                                           int64_t tiles1, int64_t tile, float2 (&RE)[PAIRS],
                                           float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                           float2 (&CIM)[PAIRS], int field,
                                           void* __restrict__ out) {
    constexpr int kPPT = 2 * PAIRS;
    const int tx = threadIdx.x & ((1 << tx_log2) - 1);
    const int ty = threadIdx.x >> tx_log2;
    const int64_t t0 = tile % tiles0, rest = tile / tiles0;
    const int64_t t1 = rest % tiles1, i2 = rest / tiles1;
    const int64_t c0 = g.count[0], c1 = g.count[1];
    const int64_t i0 = (t0 << tx_log2) + tx;
    const int64_t i1b = (t1 * (kThreads >> tx_log2) + ty) * kPPT;
    if (i0 >= c0) return;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        const int64_t i1 = i1b + k;
        if (i1 >= c1) break;
        const int64_t p = (i2 * c1 + i1) * c0 + i0;
        float vr = lane_of(RE[k >> 1], k & 1);
        float vi = lane_of(IM[k >> 1], k & 1);
        if constexpr (SUM == SUM_COMPENSATED) {
            vr = __fadd_rn(vr, lane_of(CRE[k >> 1], k & 1));
            vi = __fadd_rn(vi, lane_of(CIM[k >> 1], k & 1));
        }
        bad |= isnan(vr) || isnan(vi);
        store_field(out, p, field, vr, vi);
    }
    if (bad) {
#pragma unroll 1
        for (int k = 0; k < kPPT; ++k) {
            const int64_t i1 = i1b + k;
            if (i1 >= c1) break;
            const int64_t p = (i2 * c1 + i1) * c0 + i0;
            float x, y, z;
            grid_point(g, p, x, y, z);
            fix_coincident(src, n, x, y, z, p, field, out);
        }
    }
}

// One tile of the rows tiling, all n sources, stored.
template <int ST, int SUM, int PAIRS, bool MID = false>
__device__ __forceinline__ void block_rows(SmemTile& sm, const RowsTable& rt,
                                           const PackedSource* __restrict__ src, int64_t n,
                                           const GridDev& g, int tx_log2, int64_t tiles0,
                                           int64_t tiles1, int64_t tile, int field,
                                           void* __restrict__ out) {
    float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
    rows_accumulate<ST, SUM, PAIRS, MID>(sm, rt, src, n, 0, n, g, tx_log2, tiles0, tiles1, tile, RE,
                                    IM, CRE, CIM);
    rows_store<SUM, PAIRS>(src, n, g, tx_log2, tiles0, tiles1, tile, RE, IM, CRE, CIM, field,
                           out);
}

}  // namespace fb
}  // namespace afc
