// Per-pair propagation math shared by the field kernels and the solver kernels.
//
// One source j seen from one point x (acoustic-field-calculator/src/system/uniform_medium.rs:
// 111-120, identical to acoustic-field-optimizer/src/multiple_foci/macros.rs:17-30):
//     d = x - s_j, r = |d|, theta = acos(n_j . d / r), D = directivity(theta)
//     w = A_j D exp(-alpha_j r) / r,   phase = phi_j + k_j r
// and the contribution w * (cos phase, sin phase).
//
// Fast path (every pair): rsqrt / ex2 / sin / cos on the MUFU pipe (PTX .approx.ftz), the
// directivity from theta (an own-fit acos polynomial times a MUFU sqrt; the general body) or
// straight from cos(theta) (a cubic table; the rows body), everything else in FP32, two points
// at a time with the sm_100 packed f32x2 instructions where both points take the same
// operation.
//
// The T4010A1 directivity is piecewise in 10-degree bins and jumps at its edges (by up to
// 0.17).  A pair within rounding of a bin edge can land in a different bin than the
// reference's f32 arithmetic puts it, which changes that pair's term by up to 17 %.  Pairs
// next to an edge therefore take the exact bin: cos(theta) by the reference's f32 operations
// (no FMA, IEEE sqrt and division), then compared with the ten float thresholds kBinCos1..10
// at which the reference's bin ceil(acosf(c) / ANGLE_DIV) steps -- with acosf the one the
// reference calls, glibc's (Rust's f32::acos), whose last-ulp rounding near an edge decides
// the bin (derived and checked exhaustively around every edge in bin_edges.py).  The cubic of
// that bin is evaluated at the fast theta (within 3e-6 rad).  No double-precision operation
// is involved.
#pragma once

#include <cuda_runtime.h>

#include "afc_internal.h"

namespace afc {
namespace dev {

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kInv2Pi = 0.15915494309189535f;
// 2*pi split in two floats for the reduction phase - n*2pi: inside an FMA the product
// n*kTwoPiHi enters the subtraction unrounded, and kTwoPiLo = 2*pi - float(2*pi) corrects the
// remainder.
constexpr float kTwoPiHi = 6.28318548202514648f;     // float(2*pi)
constexpr float kTwoPiLo = -1.7484555314695172e-7f;  // 2*pi - float(2*pi)
// (u + 1.5 * 2^23) - 1.5 * 2^23 rounds |u| < 2^22 to the nearest integer with two FADDs.
constexpr float kRoundMagic = 12582912.0f;
// 2^23: for 0 <= q < 2^23, q + 2^23 rounded upward is 2^23 + ceil(q), whose low mantissa bits
// are ceil(q) as an integer (the bit pattern of 2^23 is 0x4B000000).
constexpr float kTwo23 = 8388608.0f;
// 2^23 - 1/2: for theta_c = theta + ANGLE_DIV / 2, theta_c / ANGLE_DIV + (2^23 - 1/2) rounded
// upward is 2^23 + ceil(theta / ANGLE_DIV) (to within the rounding of theta_c).
constexpr float kTwo23Half = 8388607.5f;
// 10-degree directivity bins: ANGLE_DIV = PI / 18 (t4010a1.rs:71) and its reciprocal.
constexpr float kAngleDiv = 3.14159265358979323846f / 18.0f;
constexpr float kInvAngleDiv = 18.0f / 3.14159265358979323846f;
constexpr float kHalfAngleDiv = 0.5f * kAngleDiv;
// A fast theta closer than this to a bin edge [rad] takes the exact path.  The fast theta is
// within ~3e-6 rad of the reference's (1.7e-6 from the polynomial, ~1e-6 from rsqrt and FMA
// rounding in cos(theta)), so 1e-5 leaves a factor of three.
constexpr float kEdgeMargin = 1.0e-5f;
constexpr float kEdgeBound = 0.5f * kAngleDiv - kEdgeMargin;

// bin(c) = #{b : c <= kBinCos_b} reproduces the reference's bin (0..10, NaN -> 0) for every
// float c = cos(theta) (bin_edges.py).
constexpr float kBinCos1 = 0x1.fffffep-1f;    // 0.99999994
constexpr float kBinCos2 = 0x1.f838b8p-1f;    // 0.98480773
constexpr float kBinCos3 = 0x1.e11f62p-1f;    // 0.939692557
constexpr float kBinCos4 = 0x1.bb67acp-1f;    // 0.866025329
constexpr float kBinCos5 = 0x1.8836f8p-1f;    // 0.766044378
constexpr float kBinCos6 = 0x1.491b72p-1f;    // 0.642787516
constexpr float kBinCos7 = 0x1.fffff8p-2f;    // 0.499999881
constexpr float kBinCos8 = 0x1.5e3a82p-2f;    // 0.342020065
constexpr float kBinCos9 = 0x1.63a196p-3f;    // 0.173648044
constexpr float kBinCos10 = -0x1.ddde9cp-23f;  // -2.2252536e-07

// acos(c) = sqrt(1 - c) * Q(c); Q of degree 5 fitted in fit_acos.py (float32 error <= 1.7e-6
// rad on [-0.03, 1]; for c in [-1, -0.02] it stays between 1.59 and 2.75 rad, i.e. beyond 90
// degrees where the directivity is 0, so cos(theta) needs no lower clamp).
constexpr float kAcos0 = 1.570797085762024f;
constexpr float kAcos1 = -0.21455863118171692f;
constexpr float kAcos2 = 0.08815829455852509f;
constexpr float kAcos3 = -0.04563731327652931f;
constexpr float kAcos4 = 0.020052572712302208f;
constexpr float kAcos5 = -0.0045999325811862946f;

// T4010A1 directivity (t4010a1.rs:18-69) as (A, B, C, D) per bin: the reference's cubic
// a + (b + (c + d x) x) x in x = theta - (i - 1) ANGLE_DIV re-expanded about the bin centre, in
// xc = x - ANGLE_DIV / 2 (derived and checked to 6e-8 against the reference's own f32
// evaluation in dir_table.py).  Entry 0 (theta == 0) evaluates to 1 like the reference's
// `0 => 1.0` arm, entries 1 and 2 are the constant-1 bins, entries 10..30 stand for every bin
// above 9 (0), and entry 31 (1) is where the rounded bin index wraps for theta within rounding
// of 0.
#define AFC_DIR_TABLE_INIT \
    { \
        {0x1.p+0f, 0.f, 0.f, 0.f},  \
        {0x1.p+0f, 0.f, 0.f, 0.f},  \
        {0x1.p+0f, 0.f, 0.f, 0.f},  \
        {0x1.ea25b8p-1f, -0x1.6dfba4p-1f, -0x1.4b12a6p+1f, 0x1.e10248p-11f},  \
        {0x1.9c91eep-1f, -0x1.113aaap+0f, -0x1.027ceep+0f, 0x1.6570fep-13f},  \
        {0x1.33e156p-1f, -0x1.37c58cp+0f, 0x1.b362dep-2f, 0x1.172b94p+2f},  \
        {0x1.a29d0ep-2f, -0x1.1721dep+0f, -0x1.1e0b46p-1f, -0x1.1e8668p+1f},  \
        {0x1.3096e8p-2f, -0x1.34f54ep-1f, 0x1.75296p-1f, 0x1.4657a2p+0f},  \
        {0x1.c19078p-3f, -0x1.26505cp-2f, 0x1.88e054p-1f, -0x1.20b0a8p+0f},  \
        {0x1.777e96p-3f, -0x1.965abp-3f, -0x1.d28ebp-3f, -0x1.cda5fap-1f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0.f, 0.f, 0.f, 0.f},  \
        {0x1.p+0f, 0.f, 0.f, 0.f} \
    }
// The fast path indexes the table with the low five bits of the rounded bin float (theta < 2.8
// rad, so the bin is at most 16, or wraps to 31 just below 0).
constexpr int kDirTableSize = 32;

// ------------------------------------------------------------------ launch ordering

// Programmatic dependent launch.  A kernel launched with the programmatic stream serialisation
// attribute may start before the launch ahead of it on its stream has ended: it calls pdl_wait
// before it reads anything that launch writes or writes anything that launch reads (the wait
// returns once that launch has completed and its writes are visible).  pdl_release lets the
// launch after this one be scheduled from here on.  Both are no-ops in a plain launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;"); }

// ------------------------------------------------------------------ MUFU operations

__device__ __forceinline__ float mufu_rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_sqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_sin(float x) {
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_cos(float x) {
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ------------------------------------------------------------------ packed f32x2 helpers

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// r = sqrt(r2) from r0 = r2 * rsqrt.approx(r2) and one Newton step, r0 + (r2 - r0^2) / (2 r0)
// with 1 / r0 ~ rinv: the approximation's relative error (~1.3e-7) would otherwise turn into a
// phase error k r 1.3e-7 that grows with distance (2e-4 rad at 3 m, 40 kHz).  Used by the
// transfer-matrix builds and by the field kernels' far tiles.
__device__ __forceinline__ float refine_r(float r2, float rinv, float r0) {
    return fmaf(0.5f * fmaf(-r0, r0, r2), rinv, r0);
}

// ------------------------------------------------------------------ directivity

// The reference's bin for one pair (uniform_medium.rs:113-116, t4010a1.rs:107-120): its f32
// cos(theta) = ((nx dx + ny dy) + nz dz) / sqrt((dx dx + dy dy) + dz dz) without contraction,
// IEEE sqrt and division, then the threshold count (a NaN or out-of-range c gives bin 0, as
// acosf's NaN does through Rust's `as usize`).
static __device__ __noinline__ int exact_bin(float dx, float dy, float dz, float nx, float ny,
                                             float nz) {
    const float dist = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(nx, dx), __fmul_rn(ny, dy)), __fmul_rn(nz, dz));
    const float c = __fdiv_rn(dot, dist);
    // acosf of a c rounded below -1 (a point on a tilted source's back axis) is NaN: bin 0
    if (c < -1.0f) return 0;
    return (c <= kBinCos1) + (c <= kBinCos2) + (c <= kBinCos3) + (c <= kBinCos4) +
           (c <= kBinCos5) + (c <= kBinCos6) + (c <= kBinCos7) + (c <= kBinCos8) +
           (c <= kBinCos9) + (c <= kBinCos10);
}

// Fast theta + ANGLE_DIV / 2 (the bin-centred angle the directivity is evaluated from) from
// cos(theta) for two points; the half bin rides on the final FMA for free.  A c rounded above
// 1 gives sqrt(|1 - c|), a theta of a few 1e-4 rad at most: bin 1, where the directivity is 1
// as at theta = 0.
__device__ __forceinline__ float2 theta2_centred(float2 ct) {
    const float2 c = ct;
    const float2 om = fma2(c, f2(-1.0f), f2(1.0f));  // 1 - c
    const float2 s = make_float2(mufu_sqrt(fabsf(om.x)), mufu_sqrt(fabsf(om.y)));
    float2 q = fma2(f2(kAcos5), c, f2(kAcos4));
    q = fma2(q, c, f2(kAcos3));
    q = fma2(q, c, f2(kAcos2));
    q = fma2(q, c, f2(kAcos1));
    q = fma2(q, c, f2(kAcos0));
    return fma2(s, q, f2(kHalfAngleDiv));
}

// The table entry the fast path takes for the centred angle thc (the packed form is in
// directivity2_fast): ceil(theta / ANGLE_DIV), 0..16, or 31 just below theta = 0.
__device__ __forceinline__ int fast_bin(float thc) {
    return __float_as_int(__fmaf_ru(thc, kInvAngleDiv, kTwo23Half)) & (kDirTableSize - 1);
}

// The cubic of table entry i at the centred angle thc.
__device__ __forceinline__ float dir_in_bin(const float4* __restrict__ tab, float thc, int i) {
    const float4 c = tab[i];
    const float xc = fmaf(static_cast<float>(i), -kAngleDiv, thc);
    return fmaf(fmaf(fmaf(c.w, xc, c.z), xc, c.y), xc, c.x);
}

// Directivity of one pair whose fast theta fell next to a bin edge: the exact bin's cubic at
// the fast centred angle thc.
__device__ __forceinline__ float directivity_exact(const float4* __restrict__ tab, float thc,
                                                   float dx, float dy, float dz, float nx,
                                                   float ny, float nz) {
    return dir_in_bin(tab, thc, exact_bin(dx, dy, dz, nx, ny, nz));
}

// Bin lookup and cubic for one point given 2^23 + ceil(theta / ANGLE_DIV) (whose low five bits
// are the table entry) and xc, theta's offset from the centre of that bin.
__device__ __forceinline__ float dir_cubic(const float4* __restrict__ tab, float fq_biased,
                                           float xc) {
    const float4 c = tab[__float_as_int(fq_biased) & (kDirTableSize - 1)];
    return fmaf(fmaf(fmaf(c.w, xc, c.z), xc, c.y), xc, c.x);
}

// Fast directivity of two points (packed) from their cos(theta).  `xc` receives each point's
// offset from the centre of its bin, the cubic's variable: |xc| > kEdgeBound marks a theta
// within kEdgeMargin of a bin edge, where the caller replaces the directivity by the exact
// bin's (testing every edge costs fewer instructions than selecting the four where the
// directivity jumps, and the exact bin gives the same D at the others).
__device__ __forceinline__ float2 directivity2_fast(const float4* __restrict__ tab, float2 ct,
                                                    float2& xc) {
    const float2 thc = theta2_centred(ct);                                 // theta + div / 2
    const float2 fq = __ffma2_ru(thc, f2(kInvAngleDiv), f2(kTwo23Half));  // 2^23 + ceil(q)
    const float2 fi = add2(fq, f2(-kTwo23));                               // ceil(q)
    xc = fma2(fi, f2(-kAngleDiv), thc);                                    // th - (fi - 1/2) div
    return make_float2(dir_cubic(tab, fq.x, xc.x), dir_cubic(tab, fq.y, xc.y));
}

__device__ __forceinline__ bool near_edge(float xc) { return fabsf(xc) > kEdgeBound; }

// A fast cos(theta) below this can belong to a point on the source's back axis whose
// reference cos(theta) rounds below -1, where acosf is NaN and the directivity 1 (bin 0); the
// acos polynomial is not fitted there (theta beyond 92 degrees only needs D = 0), so such pairs
// take the exact path.
constexpr float kBackAxisC = -1.0f + 4.0e-6f;

// ------------------------------------------------------------------ directivity from cos(theta)
//
// The hot loops take D as a function of c = cos(theta) directly, without theta = acos(c) and
// its MUFU square root: the c axis is cut into intervals of width 1/K, and interval
// i = floor(c K) + BIAS holds a cubic in x = c K - floor(c K) for each side of the bin edge it
// may contain (dir_ctable.py derives the table, within 1.3e-7 of D(acos c) in float32).  The
// side is the sign of c - L, L the edge's threshold on c; a pair within kCTabMargin of L (above
// the fast c's error, a few 1e-7) is recomputed by the kernels' exact edge path.  Intervals
// below -1/K give 0 (bin 10); c in [1, 3) (a unit cosine rounded up, or a direction longer than
// 1, where the reference's acos is NaN and its bin 0) gives 1.  The index is masked, so it
// stays inside the table for every c, NaN and infinities included; only a direction longer
// than 3 can land on a wrong entry.
#include "dir_ctable.inc"

constexpr int kCTabK = AFC_CTAB_K;
constexpr int kCTabSize = AFC_CTAB_SIZE;
// RD(c K + 2^23 + BIAS) = 2^23 + BIAS + floor(c K) for every c >= -BIAS / K (> -1)
constexpr float kCTabMagic = 8388608.0f + AFC_CTAB_BIAS;
constexpr float kCTabMargin = 4.0e-6f;
static_assert((kCTabSize & (kCTabSize - 1)) == 0 && kCTabSize >= AFC_CTAB_BIAS + 2 * kCTabK,
              "table index mask");

// D of two points from their fast cos(theta).  negedge[i] = -L of interval i (-1e30 without an
// edge), coef[2 i + side] the cubic of its side; t receives c - L.
__device__ __forceinline__ float2 directivity2_ctab(const float* __restrict__ negedge,
                                                    const float4* __restrict__ coef, float2 ct,
                                                    float2& t) {
    const float2 fq = __ffma2_rd(ct, f2(static_cast<float>(kCTabK)), f2(kCTabMagic));
    const float2 nfi = fma2(fq, f2(-1.0f), f2(kCTabMagic));          // -floor(c K)
    const float2 x = fma2(ct, f2(static_cast<float>(kCTabK)), nfi);  // c K - floor(c K), exact
    const int ix = __float_as_int(fq.x) & (kCTabSize - 1);
    const int iy = __float_as_int(fq.y) & (kCTabSize - 1);
    t = add2(ct, make_float2(negedge[ix], negedge[iy]));
    const float4 a = coef[(ix << 1) | static_cast<int>(__float_as_uint(t.x) >> 31)];
    const float4 b = coef[(iy << 1) | static_cast<int>(__float_as_uint(t.y) >> 31)];
    return make_float2(fmaf(fmaf(fmaf(a.w, x.x, a.z), x.x, a.y), x.x, a.x),
                       fmaf(fmaf(fmaf(b.w, x.y, b.z), x.y, b.y), x.y, b.x));
}

__device__ __forceinline__ bool near_edge_c(float t) { return fabsf(t) < kCTabMargin; }

// ------------------------------------------------------------------ the same, for scattered points
//
// The general body (scatter points, flat grids) takes D from the same cubics, laid out so that
// the 32 lanes of a warp never meet in a shared-memory bank, whatever intervals their points
// fall in.  The rows body's lanes hold neighbouring grid points and read a few neighbouring
// entries; a warp of scattered points reads up to 32 different ones, and in the plain table
// those collide in the banks (65,536- and 262,144-point launches ran 61 % and 54 % slower with
// it than with the theta path, whose 32-entry table they then kept, at one MUFU square root
// per pair).
//   * Entry u = floor(K c) + 1 for c in [-1/K, (kGTabLast - 1)/K) (interval u + BIAS - 1 of the
//     rows table), and u = kGTabClamp for every other c, taken with one unsigned minimum: c
//     below -1/K (beyond 90 degrees: D = 0), c from (kGTabLast - 1)/K = 0.9453 up (below 19
//     degrees, or a cosine rounded above 1: D = 1), and non-finite c.  The clamp entry's edge
//     sits at c = 1/2 with D = 0 below and 1 above, which gives both.  Interval 0 holds the
//     90-degree edge (its threshold is -2.2e-7) and interval kGTabLast - 1 the 20-degree one.
//   * Edge thresholds: kGTabNegCopies copies interleaved word by word, lane l reading copy l: a
//     warp's 32 four-byte loads fall in 32 different banks.
//   * Cubics: kGTabCoefCopies copies interleaved 16 bytes by 16 bytes, lane l reading copy
//     l mod 8: the 8 lanes of each phase of a 16-byte load fall in 8 different bank quads.
// Points on a tilted source's back axis (c rounded below -1, D = 1 in the reference) clamp to
// D = 0 here; the careful variant of the general body flags them (kBackAxisC) for the exact
// path, as before.
constexpr int kGTabLast = 122;               // entries 0 .. kGTabLast - 1 are table intervals
constexpr unsigned kGTabClamp = kGTabLast;   // every other c
constexpr int kGTabEntries = kGTabLast + 1;
constexpr int kGTabNegCopies = 32;
constexpr int kGTabCoefCopies = 8;
// RD(c K + 2^23 + 1) = 2^23 + 1 + floor(c K) for c >= -1/K; below, the sum falls under 2^23 and
// its bits under 0x4B000000, which the unsigned difference turns into a huge index.
constexpr float kGTabMagic = 8388609.0f;
constexpr unsigned kGTabBits = 0x4B000000u;

struct GTable {
    float neg[kGTabEntries * kGTabNegCopies];         // -L of entry u, copy l at u * 32 + l
    float4 coef[kGTabEntries * 2 * kGTabCoefCopies];  // side s of entry u, copy l at (2u + s) * 8 + l
};

// The lane's views of the table (its copies).
struct GTableLane {
    const float* neg;
    const float4* coef;
    __device__ __forceinline__ explicit GTableLane(const GTable& g) {
        const int lane = static_cast<int>(threadIdx.x & 31u);
        neg = g.neg + lane;
        coef = g.coef + (lane & (kGTabCoefCopies - 1));
    }
};

// D of two scattered points from their fast cos(theta); t receives c - L (|t| < kCTabMargin:
// next to a bin edge).  The same operations as directivity2_ctab on the table's intervals.
__device__ __forceinline__ float2 directivity2_gtab(const GTableLane& g, float2 ct, float2& t) {
    const float2 fq = __ffma2_rd(ct, f2(static_cast<float>(kCTabK)), f2(kGTabMagic));
    const float2 nfi = fma2(fq, f2(-1.0f), f2(kGTabMagic));          // -floor(c K)
    const float2 x = fma2(ct, f2(static_cast<float>(kCTabK)), nfi);  // c K - floor(c K)
    const unsigned ux = min(__float_as_uint(fq.x) - kGTabBits, kGTabClamp);
    const unsigned uy = min(__float_as_uint(fq.y) - kGTabBits, kGTabClamp);
    t = add2(ct, make_float2(g.neg[ux * kGTabNegCopies], g.neg[uy * kGTabNegCopies]));
    const float4 a = g.coef[((ux << 1) | (__float_as_uint(t.x) >> 31)) * kGTabCoefCopies];
    const float4 b = g.coef[((uy << 1) | (__float_as_uint(t.y) >> 31)) * kGTabCoefCopies];
    return make_float2(fmaf(fmaf(fmaf(a.w, x.x, a.z), x.x, a.y), x.x, a.x),
                       fmaf(fmaf(fmaf(b.w, x.y, b.z), x.y, b.y), x.y, b.x));
}

// Directivity of two points with the exact path applied in place (used where the pair is not
// on the hot loop).
__device__ __forceinline__ float2 directivity2(const float4* __restrict__ tab, float2 ct, float2 dx,
                                               float2 dy, float2 dz, float nx, float ny, float nz) {
    float2 xc;
    float2 d = directivity2_fast(tab, ct, xc);
    const bool ex = near_edge(xc.x) || ct.x < kBackAxisC, ey = near_edge(xc.y) || ct.y < kBackAxisC;
    if (ex | ey) {
        const float2 thc = theta2_centred(ct);
        if (ex) d.x = directivity_exact(tab, thc.x, dx.x, dy.x, dz.x, nx, ny, nz);
        if (ey) d.y = directivity_exact(tab, thc.y, dx.y, dy.y, dz.y, nx, ny, nz);
    }
    return d;
}

// ------------------------------------------------------------------ one pair, scalar

// Weight w and phase reduced to [-pi, pi] for source (a, b) with log2|amplitude| `la` and
// phase `phase` (sign of the amplitude folded in, layout of PackedSource) at point (px, py, pz).
template <int ST>
__device__ __forceinline__ void pair_terms(const float4& a, const float4& b, float la,
                                           float phase, const float4* __restrict__ tab, float px,
                                           float py, float pz, float& w, float& red) {
    const float dx = px - a.x;
    const float dy = py - a.y;
    const float dz = pz - a.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float rinv = mufu_rsqrt(r2);
    const float r = refine_r(r2, rinv, r2 * rinv);
    w = rinv * mufu_ex2(fmaf(b.w, r, la));
    if constexpr (ST == SRC_T4010A1) {
        const float ct = fmaf(b.z, dz, fmaf(b.y, dy, b.x * dx)) * rinv;
        const float2 d = directivity2(tab, make_float2(ct, ct), make_float2(dx, dx),
                                      make_float2(dy, dy), make_float2(dz, dz), b.x, b.y, b.z);
        w *= d.x;
    }
    const float ph = fmaf(a.w, r, phase);
    const float n = (ph * kInv2Pi + kRoundMagic) - kRoundMagic;
    red = fmaf(n, -kTwoPiLo, fmaf(n, -kTwoPiHi, ph));
}

}  // namespace dev
}  // namespace afc
