// Per-pair propagation math shared by the field kernels and the solver kernels.
//
// One source j seen from one point x (acoustic-field-calculator/src/system/uniform_medium.rs:
// 111-120, identical to acoustic-field-optimizer/src/multiple_foci/macros.rs:17-30):
//     d = x - s_j, r = |d|, theta = acos(n_j . d / r), D = directivity(theta)
//     w = A_j D exp(-alpha_j r) / r,   phase = phi_j + k_j r
// and the contribution w * (cos phase, sin phase).
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
// 10-degree directivity bins: ANGLE_DIV = PI / 18 (t4010a1.rs:71) and its reciprocal.
constexpr float kAngleDiv = 3.14159265358979323846f / 18.0f;
constexpr float kInvAngleDiv = 18.0f / 3.14159265358979323846f;

// T4010A1 directivity coefficients (t4010a1.rs:18-69) as (a, b, c, d) per bin.  Entry 0
// (theta == 0) evaluates to 1 like the reference's `0 => 1.0` arm, entries 1 and 2 are the
// constant-1 bins, and entry 10 stands for every bin above 9, which evaluates to 0.
#define AFC_DIR_TABLE_INIT                                                                      \
    {                                                                                           \
        {1.0f, 0.f, 0.f, 0.f}, {1.0f, 0.f, 0.f, 0.f}, {1.0f, 0.f, 0.f, 0.f},                    \
            {1.0f, -0.2633589359691162f, -2.586746661956269f, 0.0009174516976956062f},          \
            {0.891250938f, -0.8910683499820542f, -1.0097633564074366f, 0.0001704413361662757f}, \
            {0.707945784f, -1.1924098538381465f, -0.7167962799004945f, 4.362034715924911f},     \
            {0.501187234f, -1.0439934287916925f, 0.027352097655185065f, -2.238476800444034f},   \
            {0.354813389f, -0.7015151838490918f, 0.39509604454751995f, 1.274774620435337f},     \
            {0.251188643f, -0.4471050803642494f, 1.0625664749725618f, -1.1276955684895724f},    \
            {0.199526231f, -0.179254124486545f, 0.008242027161100222f, -0.9016569137759131f},   \
            {0.f, 0.f, 0.f, 0.f},                                                               \
    }
constexpr int kDirTableSize = 11;

// T4010A1::directivity (t4010a1.rs:107-120): bin i = ceil(theta / ANGLE_DIV),
// x = theta - (i - 1) * ANGLE_DIV, D = a + (b + (c + d x) x) x.  `tab` is the table above,
// normally staged in shared memory.
__device__ __forceinline__ float directivity(const float4* __restrict__ tab, float theta) {
    const float fi = ceilf(theta * kInvAngleDiv);
    int i = static_cast<int>(fi);  // NaN converts to 0, i.e. D = 1 as in the reference
    i = min(i, 10);
    const float4 c = tab[i];
    const float x = fmaf(-(fi - 1.0f), kAngleDiv, theta);
    return fmaf(fmaf(fmaf(c.w, x, c.z), x, c.y), x, c.x);
}

// Weight w and phase reduced to [-pi, pi] for source (a, b) with amplitude `amp` and phase
// `phase` (layout of PackedSource) at point (px, py, pz).
template <int ST>
__device__ __forceinline__ void pair_terms(const float4& a, const float4& b, float amp,
                                           float phase, const float4* __restrict__ tab, float px,
                                           float py, float pz, float& w, float& red) {
    const float dx = px - a.x;
    const float dy = py - a.y;
    const float dz = pz - a.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float rinv = rsqrtf(r2);
    const float r = r2 * rinv;
    w = amp * rinv * exp2f(b.w * r);
    if constexpr (ST == SRC_T4010A1) {
        const float ct = fmaf(b.z, dz, fmaf(b.y, dy, b.x * dx)) * rinv;
        w *= directivity(tab, acosf(ct));
    }
    const float ph = fmaf(a.w, r, phase);
    const float nq = rintf(ph * kInv2Pi);
    red = fmaf(nq, -kTwoPiLo, fmaf(nq, -kTwoPiHi, ph));
}

}  // namespace dev
}  // namespace afc
