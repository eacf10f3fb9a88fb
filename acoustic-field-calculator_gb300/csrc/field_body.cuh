// Per-block body of the direct summation, shared by the single-job kernel
// (field_kernels.cu) and the persistent batched kernel (batch.cu): shared-memory source tiles,
// packed point pairs, the near-bin-edge correction, and the field-transform epilogue.  See
// field_kernels.cu for the schedule and propagate.cuh for the per-pair math.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "afc_internal.h"
#include "propagate.cuh"

namespace afc {
namespace fb {

using namespace dev;

constexpr int kThreads = 256;  // threads per block
constexpr int kTile = 256;     // sources per shared-memory tile

// PackedSource j from the ABI records (T4010A1: 9 floats, sphere: 6), wavenumbers and
// attenuations; the amplitude goes into the exponent as log2|A| and its sign into the phase.
__device__ __forceinline__ PackedSource pack_source(int st, const float* __restrict__ raw,
                                                   const float* __restrict__ k,
                                                   const float* __restrict__ atten, int64_t j) {
    PackedSource p;
    float amp, phase;
    if (st == SRC_T4010A1) {
        const float* s = raw + 9 * j;
        p.a = make_float4(s[0], s[1], s[2], k[j]);
        p.b = make_float4(s[3], s[4], s[5], -atten[j] * kLog2e);
        amp = s[6];
        phase = s[7];
    } else {
        const float* s = raw + 6 * j;
        p.a = make_float4(s[0], s[1], s[2], k[j]);
        p.b = make_float4(0.f, 0.f, 0.f, -atten[j] * kLog2e);
        amp = s[3];
        phase = s[4];
    }
    const float ph = amp < 0.f ? phase + 3.14159265358979323846f : phase;
    p.c = make_float4(log2f(fabsf(amp)), ph, amp, phase);
    return p;
}

// Shared-memory image of one source: five float4 of duplicated scalars and -n0.s.
//   v0 = (-x, -x, -y, -y)   v1 = (-z, -z, k, k)   v2 = (nx, nx, ny, ny)
//   v3 = (nz, nz, a2, a2)   v4 = (la, la, ph, ph)   ns = (-n0.s, -n0.s)
// a2 = -alpha log2(e), la = log2|A|, ph = phase (+ pi for A < 0), n0 = direction of source 0.
struct SmemTile {
    float4 v0[kTile], v1[kTile], v2[kTile], v3[kTile], v4[kTile];
    float2 ns[kTile];
    float4 dir[kDirTableSize];    // theta-binned cubics (the exact edge paths)
    float box[kThreads / 32][6];  // per-warp bounds of the block's points (min xyz, max xyz)
    float bbox[6];                // the block's bounds
};

// The rows body's cos(theta)-indexed table in shared memory.
struct RowsTable {
    float cneg[kCTabSize];        // -L per interval
    float4 ccoef[2 * kCTabSize];  // the cubic of each side
};

// Shared memory of the rows kernels: the staging tile and the rows table in one object (the
// layout the kernels' register allocation was tuned on; as two separate objects the 256^3
// launch ran 2 % slower).
struct RowsSmem {
    SmemTile sm;
    RowsTable rt;
};

// The cos(theta)-indexed directivity table in global memory (one copy per translation unit).
static __device__ const float g_ctab_negedge[kCTabSize] = AFC_CTAB_NEGEDGE_INIT;
static __device__ const float4 g_ctab_coef[2 * kCTabSize] = AFC_CTAB_COEF_INIT;

// Bytes of dynamic shared memory a general-body kernel needs for its GTable.
constexpr int kGTableBytes = static_cast<int>(sizeof(GTable));

// Dynamic shared memory beyond the default 48 KB per block needs an opt-in per kernel and per
// device; it is made once per device (one bit per device of the first 64) before a launch.
template <auto Kernel>
cudaError_t allow_dynamic_smem(int bytes) {
    static std::atomic<uint64_t> done{0};
    if (bytes <= 0) return cudaSuccess;
    int dev = 0;
    const cudaError_t ge = cudaGetDevice(&dev);
    if (ge != cudaSuccess) return ge;
    const uint64_t bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    const cudaError_t e =
        cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
    return e;
}

// Fill the block's theta-binned table (a __syncthreads must follow before its first use).
__device__ __forceinline__ void load_theta_table(SmemTile& sm, const float4* __restrict__ dir) {
    if (threadIdx.x < kDirTableSize) sm.dir[threadIdx.x] = dir[threadIdx.x];
}

// Fill the rows body's table (a __syncthreads must follow before its first use).
__device__ __forceinline__ void load_rows_table(RowsTable& rt) {
    for (int i = threadIdx.x; i < kCTabSize; i += blockDim.x) rt.cneg[i] = g_ctab_negedge[i];
    for (int i = threadIdx.x; i < 2 * kCTabSize; i += blockDim.x) rt.ccoef[i] = g_ctab_coef[i];
}

// Fill the general body's lane-replicated table from the rows table's intervals (entry u is
// interval u + BIAS - 1 there) and the clamp entry (edge at c = 1/2, D = 1 above, 0 below); a
// __syncthreads must follow before its first use.  Blocks of kThreads threads: each thread
// issues all its global loads before its first store, so the fill costs one load latency, not
// one per element (as a strided loop it took a sizeable part of a short block).
__device__ __forceinline__ void load_gtab(GTable& g) {
    constexpr int kFirst = AFC_CTAB_BIAS - 1;
    constexpr int kNeg = kGTabEntries * kGTabNegCopies;
    constexpr int kCoef = kGTabEntries * 2 * kGTabCoefCopies;
    constexpr int kNegIt = (kNeg + kThreads - 1) / kThreads;
    constexpr int kCoefIt = (kCoef + kThreads - 1) / kThreads;
    float nv[kNegIt];
    float4 cv[kCoefIt];
#pragma unroll
    for (int k = 0; k < kNegIt; ++k) {
        const int u = static_cast<int>(threadIdx.x + k * kThreads) / kGTabNegCopies;
        nv[k] = u < kGTabLast ? g_ctab_negedge[u + kFirst] : -0.5f;
    }
#pragma unroll
    for (int k = 0; k < kCoefIt; ++k) {
        const int e = static_cast<int>(threadIdx.x + k * kThreads) / kGTabCoefCopies;  // 2u + side
        const int u = e >> 1, side = e & 1;
        cv[k] = u < kGTabLast ? g_ctab_coef[2 * (u + kFirst) + side]
                              : make_float4(side ? 0.f : 1.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < kNegIt; ++k) {
        const int i = static_cast<int>(threadIdx.x + k * kThreads);
        if (i < kNeg) g.neg[i] = nv[k];
    }
#pragma unroll
    for (int k = 0; k < kCoefIt; ++k) {
        const int i = static_cast<int>(threadIdx.x + k * kThreads);
        if (i < kCoef) g.coef[i] = cv[k];
    }
}

// The phase phi + k r goes to sin/cos.approx unreduced when it is at most this large for every
// source of a tile and every point of the block: the approximations take their argument in
// turns after one FP32 multiply, whose rounding gives an absolute error of ~1.2e-7 |phase|
// (<= 8e-5 rad here, the order of the reference's own f32 rounding of phi + k r); larger
// phases are first reduced to [-pi, pi] (ref_phase2).
constexpr float kUnreducedPhaseMax = 640.0f;

// Tiles whose phase bound lies above kUnreducedPhaseMax but at most kMidPhaseMax, with every
// point in front of every source, take mid_phase2: r refined by a Newton step, phi fused,
// reduced to [-pi, pi].  It stays within about an ulp of phi (6.1e-5 rad below 1,024 rad) of the
// reference's rounding; larger phases take the reference's own rounding (ref_phase2).
constexpr float kMidPhaseMax = 1024.0f;

// Phase variants of the hot loops: unreduced (fast), Newton-refined and reduced (mid), or
// rounded as the reference rounds it and reduced (ref).
enum : int { kPhaseFast = 0, kPhaseMid = 1, kPhaseRef = 2 };

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
    float v[3] = {g.origin[0], g.origin[1], g.origin[2]};
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

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

__device__ __forceinline__ float& lane_of(float2& v, int hi) { return hi ? v.y : v.x; }
__device__ __forceinline__ float lane_of(const float2& v, int hi) { return hi ? v.y : v.x; }

// The far tiles' phase, rounded as the reference rounds it (uniform_medium.rs:111-120): from
// q2 = (dx dx + dy dy) + dz dz summed in x, y, z order without contraction, dist = sqrt(q2)
// rounded to nearest, phi = phase + k dist with the product and the sum rounded separately;
// then reduced to [-pi, pi] with 2 pi in two parts (Cody and Waite: n kTwoPiHi leaves the FMA
// unrounded and n kTwoPiLo corrects float(2 pi), whose error would add 1.7e-7 rad per turn).
// At distances of metres the reference's own f32 rounding of phi (1e-4 rad at 3 m) is as large
// as the field bar, so a phase rounded any other way would differ from its field by about that
// much.  A source with a negative amplitude carries phase + pi (PackedSource), whose rounding
// differs.
//
// dist (returned in r) is q2 rinv with one Newton step (refine_r), rinv ~ rsqrt(q2) (the pair's
// rsqrt.approx of its own r^2 is close enough): over 2e6 pairs at 1.5 to 6 m it equalled the
// IEEE square root every time.  sqrt.rn itself is not used because any call of it in these
// kernels, even on a path the launch never takes, cost the near-field loop 1-2 %.  The products
// and sums are the scalar __fmul_rn / __fadd_rn, which are never merged into an FMA.  A packed
// product feeding a packed sum is not safe from that: on 1M random inputs __fmul2_rn then
// __fadd2_rn, and equally mul.rn.f32x2 then add.rn.f32x2 written in PTX, gave the fused result
// wherever it differs (261,351 cases), and the far-field test measured the fused rounding of
// phase + k dist (1.3e-4 of the peak at 3 m, against 3e-6 for the reference's rounding).
__device__ __forceinline__ float2 ref_phase2(float2 q2, float2 rinv, float2 k, float2 phase,
                                             float2& r) {
    r = make_float2(refine_r(q2.x, rinv.x, q2.x * rinv.x), refine_r(q2.y, rinv.y, q2.y * rinv.y));
    const float2 ph = make_float2(__fadd_rn(phase.x, __fmul_rn(k.x, r.x)),
                                  __fadd_rn(phase.y, __fmul_rn(k.y, r.y)));
    const float2 nq = add2(fma2(ph, f2(kInv2Pi), f2(kRoundMagic)), f2(-kRoundMagic));
    return fma2(nq, f2(-kTwoPiLo), fma2(nq, f2(-kTwoPiHi), ph));
}

// The mid tiles' phase (kMidPhaseMax): r0 = r2 rinv (on entry in r) refined by one Newton step,
// r = r0 + (r2 - r0^2) rinv / 2 (refine_r, packed), then phi = phase + k r with one rounding,
// reduced to [-pi, pi] with 2 pi in two parts as ref_phase2 does.  The fused phi differs from
// the reference's separately rounded product and sum by at most about an ulp of phi.
__device__ __forceinline__ float2 mid_phase2(float2 r2, float2 rinv, float2 k, float2 phase,
                                             float2& r) {
    const float2 e = fma2(make_float2(-r.x, -r.y), r, r2);
    r = fma2(e, mul2(rinv, f2(0.5f)), r);
    const float2 ph = fma2(k, r, phase);
    const float2 nq = add2(fma2(ph, f2(kInv2Pi), f2(kRoundMagic)), f2(-kRoundMagic));
    return fma2(nq, f2(-kTwoPiLo), fma2(nq, f2(-kTwoPiHi), ph));
}

// (dx dx + dy dy) + dz dz rounded after every operation, for one point.
__device__ __forceinline__ float ref_dist2_1(float dx, float dy, float dz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
__device__ __forceinline__ float2 ref_dist2(float2 dx, float2 dy, float2 dz) {
    return make_float2(ref_dist2_1(dx.x, dy.x, dz.x), ref_dist2_1(dx.y, dy.y, dz.y));
}

// Correction for one point of a thread whose points include one next to a bin edge (or, in the
// careful variant, possibly on a source's back axis): recompute the pair with the hot loop's
// operations (UD: cos(theta) from the shared direction); if its fast cos(theta) is within
// kCTabMargin of the edge of its table interval, or below kBackAxisC, return w (D_exact -
// D_fast) (cos, sin), the amount to add to the point's accumulators, with D_exact the cubic of
// the reference's bin (exact_bin) at the fast theta; else zero.  Everything passes by value so
// that the caller's accumulators stay in registers.
template <bool UD>
__device__ __noinline__ float2 edge_correction(const float4* __restrict__ tab, GTableLane g,
                                               float4 v0, float4 v1, float4 v2, float4 v3,
                                               float4 v4, float2 ns, float3 n0, float np,
                                               float px, float py, float pz) {
    const float dx = px + v0.x, dy = py + v0.z, dz = pz + v1.x;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float rinv = mufu_rsqrt(r2);
    float ct, nx, ny, nz;
    if constexpr (UD) {
        ct = (np + ns.x) * rinv;
        nx = n0.x;
        ny = n0.y;
        nz = n0.z;
    } else {
        ct = fmaf(v3.x, dz, fmaf(v2.z, dy, v2.x * dx)) * rinv;
        nx = v2.x;
        ny = v2.z;
        nz = v3.x;
    }
    float2 t;
    const float d_fast = directivity2_gtab(g, make_float2(ct, ct), t).x;
    if (!near_edge_c(t.x) && !(ct < kBackAxisC)) return make_float2(0.f, 0.f);
    const float thc = theta2_centred(make_float2(ct, ct)).x;
    const int i_exact = exact_bin(dx, dy, dz, nx, ny, nz);
    float2 r;
    const float red =
        ref_phase2(ref_dist2(f2(dx), f2(dy), f2(dz)), f2(rinv), f2(v1.z), f2(v4.z), r).x;
    const float w0 = rinv * mufu_ex2(fmaf(v3.z, r.x, v4.x));
    const float corr = w0 * (dir_in_bin(tab, thc, i_exact) - d_fast);
    return make_float2(corr * mufu_cos(red), corr * mufu_sin(red));
}

// The geometry of point pair q against source (v0, v1, v2, v3, ns): d, r^2, 1/r, cos(theta),
// with the same operations on the hot loop and on its edge path.
template <bool UD>
struct PairGeom {
    float2 dx, dy, dz, r2, rinv, ct;
    __device__ __forceinline__ PairGeom(float2 px, float2 py, float2 pz, float2 np, float4 v0,
                                        float4 v1, float4 v2, float4 v3, float2 ns) {
        dx = add2(px, lo2(v0));
        dy = add2(py, hi2(v0));
        dz = add2(pz, lo2(v1));
        r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        rinv = make_float2(mufu_rsqrt(r2.x), mufu_rsqrt(r2.y));
        if constexpr (UD) ct = mul2(add2(np, ns), rinv);
        else ct = mul2(fma2(lo2(v3), dz, fma2(hi2(v2), dy, mul2(lo2(v2), dx))), rinv);
    }
};

// The PAIRS point pairs of one thread against shared-memory source j.  The hot loop only
// records the smallest distance of any of the thread's points to the bin edge of its table
// interval; that rare case recomputes the pairs' geometry to find which points, and corrects
// them one by one.  PH: the phase variant.  kPhaseRef is the careful variant, for tiles with a
// phase bound above kMidPhaseMax or with some point possibly behind a source: the phase is
// rounded as the reference rounds it and reduced before sin/cos (ref_phase2), and a cos(theta)
// next to -1 (kBackAxisC) also takes the exact path.  kPhaseMid: phases up to kMidPhaseMax,
// every point in front (mid_phase2).  The directivity comes straight from cos(theta), from the
// lane-replicated table (directivity2_gtab): no acos and no MUFU square root.
template <int ST, int SUM, int PAIRS, bool UD, int PH>
__device__ __forceinline__ void accumulate_source(const SmemTile& sm, const GTableLane& g, int j,
                                                  float3 n0, float2 (&PX)[PAIRS],
                                                  float2 (&PY)[PAIRS], float2 (&PZ)[PAIRS],
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
    float near_min = kCTabMargin;  // smallest |c - L| of the thread's points (the edge test)
    bool any_back = false;         // careful variant: some c next to -1
#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        const PairGeom<UD> p(PX[q], PY[q], PZ[q], NP[q], v0, v1, v2, v3, ns);
        float2 r = mul2(p.r2, p.rinv);
        float2 red;
        if constexpr (PH == kPhaseRef)
            red = ref_phase2(ref_dist2(p.dx, p.dy, p.dz), p.rinv, hi2(v1), hi2(v4), r);
        else if constexpr (PH == kPhaseMid)
            red = mid_phase2(p.r2, p.rinv, hi2(v1), hi2(v4), r);
        else red = fma2(hi2(v1), r, hi2(v4));
        const float2 ea = fma2(hi2(v3), r, lo2(v4));
        float2 w = mul2(p.rinv, make_float2(mufu_ex2(ea.x), mufu_ex2(ea.y)));
        if constexpr (ST == SRC_T4010A1) {
            float2 t;
            w = mul2(w, directivity2_gtab(g, p.ct, t));
            near_min = fminf(near_min, fminf(fabsf(t.x), fabsf(t.y)));
            if constexpr (PH == kPhaseRef) any_back |= (p.ct.x < kBackAxisC) | (p.ct.y < kBackAxisC);
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
        if (near_min < kCTabMargin || any_back) {
#pragma unroll
            for (int k = 0; k < 2 * PAIRS; ++k) {
                const int q = k >> 1, h = k & 1;
                const float2 c = edge_correction<UD>(sm.dir, g, v0, v1, v2, v3, v4, ns, n0,
                                                     lane_of(NP[q], h), lane_of(PX[q], h),
                                                     lane_of(PY[q], h), lane_of(PZ[q], h));
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

// Sources 0 .. cnt - 1 of the staged tile against the thread's points, with the tile's phase
// variant (MID: whether the mid tier is compiled in; without it, mid tiles take the careful
// variant).
template <int ST, int SUM, int PAIRS, bool UD, bool MID>
__device__ __forceinline__ void source_loop(int ph, int cnt, const SmemTile& sm, const GTableLane& gl,
                                            float3 n0, float2 (&PX)[PAIRS], float2 (&PY)[PAIRS],
                                            float2 (&PZ)[PAIRS], float2 (&NP)[PAIRS],
                                            float2 (&RE)[PAIRS], float2 (&IM)[PAIRS],
                                            float2 (&CRE)[PAIRS], float2 (&CIM)[PAIRS]) {
    if (ph == kPhaseFast) {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_source<ST, SUM, PAIRS, UD, kPhaseFast>(sm, gl, j, n0, PX, PY, PZ, NP, RE, IM,
                                                              CRE, CIM);
    } else if (MID && ph == kPhaseMid) {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_source<ST, SUM, PAIRS, UD, kPhaseMid>(sm, gl, j, n0, PX, PY, PZ, NP, RE, IM,
                                                             CRE, CIM);
    } else {
#pragma unroll 1
        for (int j = 0; j < cnt; ++j)
            accumulate_source<ST, SUM, PAIRS, UD, kPhaseRef>(sm, gl, j, n0, PX, PY, PZ, NP, RE, IM,
                                                             CRE, CIM);
    }
}

// One block of 2*PAIRS*kThreads observation points starting at point `first`: stage sources
// s_lo .. s_hi - 1 tile by tile into `sm` (its dir table must already be filled) and accumulate
// their fields into RE, IM (CRE, CIM: compensation terms).  `grid` selects generated grid
// points or explicit ones; source 0's direction is the shared direction of the fast cos(theta).
template <int ST, int SUM, int PAIRS, bool MID = false>
__device__ __forceinline__ void block_accumulate(SmemTile& sm, const GTable& gt,
                                                 const PackedSource* __restrict__ src,
                                                 int64_t n, int64_t s_lo, int64_t s_hi, bool grid,
                                                 const GridDev& g, const float* __restrict__ pts,
                                                 int64_t m, int64_t first, float2 (&RE)[PAIRS],
                                                 float2 (&IM)[PAIRS], float2 (&CRE)[PAIRS],
                                                 float2 (&CIM)[PAIRS]) {
    constexpr int kPPT = 2 * PAIRS;
    const GTableLane gl(gt);
    const int64_t base = first + threadIdx.x;
    float2 PX[PAIRS], PY[PAIRS], PZ[PAIRS], NP[PAIRS];
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        int64_t p = base + static_cast<int64_t>(k) * kThreads;
        if (p >= m) p = m - 1;  // computed but never stored
        float x, y, z;
        if (grid) {
            grid_point(g, p, x, y, z);
        } else {
            x = __ldg(pts + 3 * p);
            y = __ldg(pts + 3 * p + 1);
            z = __ldg(pts + 3 * p + 2);
        }
        lane_of(PX[k >> 1], k & 1) = x;
        lane_of(PY[k >> 1], k & 1) = y;
        lane_of(PZ[k >> 1], k & 1) = z;
    }
    // direction of source 0: the reference direction of the shared-direction path
    float3 n0 = make_float3(0.f, 0.f, 0.f);
    if (ST == SRC_T4010A1 && n > 0) {
        const float4 b0 = src[0].b;
        n0 = make_float3(b0.x, b0.y, b0.z);
    }
    // bounding box of the block's points (for the phase bound of each source tile)
    float bmin[3] = {PX[0].x, PY[0].x, PZ[0].x}, bmax[3] = {PX[0].x, PY[0].x, PZ[0].x};
#pragma unroll
    for (int k = 1; k < kPPT; ++k) {
        const float c[3] = {lane_of(PX[k >> 1], k & 1), lane_of(PY[k >> 1], k & 1),
                            lane_of(PZ[k >> 1], k & 1)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bmin[a] = fminf(bmin[a], c[a]);
            bmax[a] = fmaxf(bmax[a], c[a]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bmin[a] = fminf(bmin[a], __shfl_xor_sync(0xffffffffu, bmin[a], o));
            bmax[a] = fmaxf(bmax[a], __shfl_xor_sync(0xffffffffu, bmax[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            sm.box[threadIdx.x >> 5][a] = bmin[a];
            sm.box[threadIdx.x >> 5][3 + a] = bmax[a];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int a = threadIdx.x;
        float v = sm.box[0][a];
#pragma unroll
        for (int w = 1; w < kThreads / 32; ++w) v = a < 3 ? fminf(v, sm.box[w][a]) : fmaxf(v, sm.box[w][a]);
        sm.bbox[a] = v;
    }
    __syncthreads();  // sm.bbox is read while staging each tile below

#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        NP[q] = fma2(f2(n0.z), PZ[q], fma2(f2(n0.y), PY[q], mul2(f2(n0.x), PX[q])));
        RE[q] = f2(0.f);
        IM[q] = f2(0.f);
        CRE[q] = f2(0.f);
        CIM[q] = f2(0.f);
    }

    for (int64_t t0 = s_lo; t0 < s_hi; t0 += kTile) {
        const int cnt = static_cast<int>((s_hi - t0) < kTile ? (s_hi - t0) : kTile);
        __syncthreads();
        // plain: every phase of the tile bounded for the unreduced path and every point in front
        // of every source; mid: the same with the phases within kMidPhaseMax; otherwise the
        // tile takes the careful variant (kPhaseRef)
        bool same_dir = true, plain = true, mid = true;
        for (int j = threadIdx.x; j < cnt; j += kThreads) {
            const PackedSource s = src[t0 + j];
            // |phi' + k r| over the box: r is at most the distance to the farthest corner
            const float fx = fmaxf(fabsf(sm.bbox[0] - s.a.x), fabsf(sm.bbox[3] - s.a.x));
            const float fy = fmaxf(fabsf(sm.bbox[1] - s.a.y), fabsf(sm.bbox[4] - s.a.y));
            const float fz = fmaxf(fabsf(sm.bbox[2] - s.a.z), fabsf(sm.bbox[5] - s.a.z));
            const float rmax = sqrtf(fmaf(fz, fz, fmaf(fy, fy, fx * fx)));
            const float bound = fmaf(fabsf(s.a.w), rmax, fabsf(s.c.y));
            plain = plain && bound <= kUnreducedPhaseMax;
            mid = mid && bound <= kMidPhaseMax;
            if (ST == SRC_T4010A1) {
                // the box's lowest n.(x - s) (per axis the corner n points away from): when it is
                // not negative, every point is in front of the source, where cos(theta) >= 0
                const float lx = s.b.x >= 0.f ? sm.bbox[0] : sm.bbox[3];
                const float ly = s.b.y >= 0.f ? sm.bbox[1] : sm.bbox[4];
                const float lz = s.b.z >= 0.f ? sm.bbox[2] : sm.bbox[5];
                const float front = fmaf(s.b.z, lz - s.a.z, fmaf(s.b.y, ly - s.a.y, s.b.x * (lx - s.a.x)));
                plain = plain && front >= 0.f;
                mid = mid && front >= 0.f;
            }
            sm.v0[j] = make_float4(-s.a.x, -s.a.x, -s.a.y, -s.a.y);
            sm.v1[j] = make_float4(-s.a.z, -s.a.z, s.a.w, s.a.w);
            sm.v2[j] = make_float4(s.b.x, s.b.x, s.b.y, s.b.y);
            sm.v3[j] = make_float4(s.b.z, s.b.z, s.b.w, s.b.w);
            sm.v4[j] = make_float4(s.c.x, s.c.x, s.c.y, s.c.y);
            const float ns = fmaf(n0.z, s.a.z, fmaf(n0.y, s.a.y, n0.x * s.a.x));
            sm.ns[j] = f2(-ns);
            same_dir = same_dir && s.b.x == n0.x && s.b.y == n0.y && s.b.z == n0.z;
        }
        const bool tile_same_dir = __syncthreads_and(same_dir);
        const bool tile_plain = __syncthreads_and(plain);
        const bool tile_mid = __syncthreads_and(mid);
        const int tile_ph = tile_plain ? kPhaseFast : ((MID && tile_mid) ? kPhaseMid : kPhaseRef);
        if (ST == SRC_T4010A1 && tile_same_dir) {
            source_loop<ST, SUM, PAIRS, true, MID>(tile_ph, cnt, sm, gl, n0, PX, PY, PZ, NP, RE, IM, CRE, CIM);
        } else {
            source_loop<ST, SUM, PAIRS, false, MID>(tile_ph, cnt, sm, gl, n0, PX, PY, PZ, NP, RE, IM, CRE, CIM);
        }
    }
}

// Store the field of point p from its complex sum (vr, vi): the sum itself, its power
// norm_sqr = re*re + im*im without contraction, or the pressure sqrt(norm_sqr)
// (field_buffer/pressure_field.rs:35-37).
__device__ __forceinline__ void store_field(void* __restrict__ out, int64_t p, int field, float vr,
                                            float vi) {
    if (field == FIELD_COMPLEX) {
        reinterpret_cast<float2*>(out)[p] = make_float2(vr, vi);
    } else {
        const float ns = __fadd_rn(__fmul_rn(vr, vr), __fmul_rn(vi, vi));
        reinterpret_cast<float*>(out)[p] = (field == FIELD_PRESSURE) ? __fsqrt_rn(ns) : ns;
    }
}

// Point p at (px, py, pz), already stored by this thread: if its field is NaN and sources sit
// exactly on it, store the reference's field there.  At the reference's dist = 0
// (uniform_medium.rs:113-119) such a source gives amp * D * exp(-0 alpha) / 0 with D = 1 (acos
// of 0 / 0 is NaN: bin 0, t4010a1.rs:107-109), so from_polar gives components of +-inf, or NaN
// where the amplitude is 0 or sin(phase) is 0.  No finite term changes such a sum (nor does the
// Accurate tag's sorted sum), so the point's field is the sum of these terms alone.  The
// kernels' pair math gives 0 * inf = NaN there instead.  A NaN without a coincident source (a
// NaN coordinate or parameter) is left as stored.
static __device__ __noinline__ void fix_coincident(const PackedSource* __restrict__ src,
                                                   int64_t n, float px, float py, float pz,
                                                   int64_t p, int field, void* __restrict__ out) {
    const float v0 = field == FIELD_COMPLEX ? reinterpret_cast<const float2*>(out)[p].x
                                            : reinterpret_cast<const float*>(out)[p];
    const float v1 = field == FIELD_COMPLEX ? reinterpret_cast<const float2*>(out)[p].y : 0.f;
    if (!isnan(v0) && !isnan(v1)) return;
    float re = 0.f, im = 0.f;
    bool hit = false;
    for (int64_t j = 0; j < n; ++j) {
        const float4 a = src[j].a;
        if (ref_dist2_1(__fsub_rn(px, a.x), __fsub_rn(py, a.y), __fsub_rn(pz, a.z)) != 0.f)
            continue;
        const float4 b = src[j].b, c = src[j].c;
        // amp * exp(-dist alpha) / dist and phase + k dist at dist = 0
        const float w = __fdiv_rn(__fmul_rn(c.z, exp2f(__fmul_rn(0.f, b.w))), 0.f);
        const float phi = __fadd_rn(c.w, __fmul_rn(a.w, 0.f));
        re = __fadd_rn(re, __fmul_rn(w, cosf(phi)));
        im = __fadd_rn(im, __fmul_rn(w, sinf(phi)));
        hit = true;
    }
    if (hit) store_field(out, p, field, re, im);
}

// Apply the field transform to a block's sums (block_accumulate) and store them; points whose
// sum is NaN are then passed to fix_coincident.  `grid`, `g` and `pts` give the points as block_accumulate
// takes them.
template <int SUM, int PAIRS>
__device__ __forceinline__ void block_store(float2 (&RE)[PAIRS], float2 (&IM)[PAIRS],
                                            float2 (&CRE)[PAIRS], float2 (&CIM)[PAIRS],
                                            const PackedSource* __restrict__ src, int64_t n,
                                            bool grid, const GridDev& g,
                                            const float* __restrict__ pts, int64_t first,
                                            int64_t m, int field, void* __restrict__ out) {
    constexpr int kPPT = 2 * PAIRS;
    const int64_t base = first + threadIdx.x;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < kPPT; ++k) {
        const int64_t p = base + static_cast<int64_t>(k) * kThreads;
        if (p >= m) break;
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
            const int64_t p = base + static_cast<int64_t>(k) * kThreads;
            if (p >= m) break;
            float x, y, z;
            if (grid) {
                grid_point(g, p, x, y, z);
            } else {
                x = pts[3 * p];
                y = pts[3 * p + 1];
                z = pts[3 * p + 2];
            }
            fix_coincident(src, n, x, y, z, p, field, out);
        }
    }
}

// One block of 2*PAIRS*kThreads observation points starting at point `first`, all n sources:
// accumulate, apply the field transform and store.
template <int ST, int SUM, int PAIRS, bool MID = false>
__device__ __forceinline__ void block_points(SmemTile& sm, const GTable& gt,
                                             const PackedSource* __restrict__ src, int64_t n,
                                             bool grid, const GridDev& g,
                                             const float* __restrict__ pts, int64_t m,
                                             int64_t first, int field, void* __restrict__ out) {
    float2 RE[PAIRS], IM[PAIRS], CRE[PAIRS], CIM[PAIRS];
    block_accumulate<ST, SUM, PAIRS, MID>(sm, gt, src, n, 0, n, grid, g, pts, m, first, RE, IM, CRE,
                                     CIM);
    block_store<SUM, PAIRS>(RE, IM, CRE, CIM, src, n, grid, g, pts, first, m, field, out);
}

}  // namespace fb
}  // namespace afc
