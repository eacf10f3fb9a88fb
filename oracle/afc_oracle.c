/*
 * afc_oracle.c -- the ORACLE: a CPU restatement of the reference's acoustic-field
 * calculation path, used ONLY as test infrastructure.
 *
 *   Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load this
 *   library, and only as the checker or the timed CPU baseline.  The product
 *   (libafccapi.so) never links, loads or calls it.
 *
 *   PARITY UNPINNED.  The reference (shinolab/acoustic-field-calculator 0.6.1) is Rust;
 *   no Rust toolchain exists on these machines and the reference ships no golden vectors,
 *   known-answer tests or fixtures for this path (its only unit tests are in fmath and
 *   assert nothing about fields).  This file is therefore pinned only by the known-answer
 *   tests in tests/test_oracle_known_answers.py, which recompute the reference's formulas
 *   independently (numpy, float64) from the cited source lines.
 *
 * What it restates (file:line within the reference project):
 *   sound speed        acoustic-field-calculator/src/core/sound_speed.rs:22-24
 *   attenuation        acoustic-field-calculator/src/core/attenuation.rs:31-48
 *   k and alpha        acoustic-field-calculator/src/system/uniform_medium.rs:102-107
 *   directivity        acoustic-field-calculator/src/core/wave_sources/t4010a1.rs:18-71,107-120
 *   sphere source      acoustic-field-calculator/src/core/wave_sources/sphere_sources.rs:48-61
 *   propagate          acoustic-field-calculator/src/system/uniform_medium.rs:111-120
 *   propagate_all      acoustic-field-calculator/src/system/uniform_medium.rs:122-128
 *   CPU calculator     acoustic-field-calculator/src/calculator/cpu_calculator.rs:43-56
 *   accurate variant   acoustic-field-calculator/src/accurate/system_acc.rs:26-55
 *   field transforms   acoustic-field-calculator/src/field_buffer/{pressure,power,complex_pressure}_field.rs:35-37
 *   grid points        acoustic-field-calculator/src/observe_area/grid/builder.rs:144-209,
 *                      acoustic-field-calculator/src/observe_area/grid/grid_area.rs:59-229
 *   focal law          acoustic-field-optimizer/src/focal_point.rs:27-40
 *   G build            acoustic-field-optimizer/src/multiple_foci/macros.rs:17-53
 *   GS-PAT             acoustic-field-optimizer/src/multiple_foci/linear_synthesis/gs_pat.rs:35-81
 *                      (float64, and in f32 as the reference computes it)
 *   GS                 acoustic-field-optimizer/src/multiple_foci/linear_synthesis/gs.rs:33-78
 *   Naive              acoustic-field-optimizer/src/multiple_foci/linear_synthesis/naive.rs:29-51
 *
 * Float semantics.  The reference computes in f32 (Float = f32, core/mod.rs:100-105) with
 * libm acosf/expf/sinf/cosf/powf and no fused multiply-add (rustc does not contract).
 * This file must be compiled with -ffp-contract=off and without -ffast-math so that each
 * f32 operation rounds exactly where the reference's does; the float64 twins (suffix _f64)
 * evaluate the same formulas in double for error reports.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

/* std::f32::consts::PI */
#define ORC_PI_F 3.14159265358979323846f

/* Directivity coefficient tables of the T4010A1 model (t4010a1.rs:18-69).  The values are
 * the reference's data, written here as f32 literals exactly as the reference types them. */
static const float DIR_A[10] = {0.f, 1.0f, 1.0f, 1.0f, 0.891250938f, 0.707945784f,
                                0.501187234f, 0.354813389f, 0.251188643f, 0.199526231f};
static const float DIR_B[10] = {0.f, 0.f, 0.f, -0.2633589359691162f, -0.8910683499820542f,
                                -1.1924098538381465f, -1.0439934287916925f, -0.7015151838490918f,
                                -0.4471050803642494f, -0.179254124486545f};
static const float DIR_C[10] = {0.f, 0.f, 0.f, -2.586746661956269f, -1.0097633564074366f,
                                -0.7167962799004945f, 0.027352097655185065f, 0.39509604454751995f,
                                1.0625664749725618f, 0.008242027161100222f};
static const float DIR_D[10] = {0.f, 0.f, 0.f, 0.0009174516976956062f, 0.0001704413361662757f,
                                4.362034715924911f, -2.238476800444034f, 1.274774620435337f,
                                -1.1276955684895724f, -0.9016569137759131f};

/* ANGLE_DIV = PI / 18.0 in f32 (t4010a1.rs:71) */
static const float ANGLE_DIV_F = ORC_PI_F / 18.0f;

enum { ORC_SRC_SPHERE = 0, ORC_SRC_T4010A1 = 1 };
enum { ORC_FIELD_PRESSURE = 0, ORC_FIELD_POWER = 1, ORC_FIELD_COMPLEX = 2 };

/* Floats per source in the C-ABI layouts: SphereWaveSource {pos, amp, phase, freq}
 * (sphere_sources.rs:22-27) and T4010A1 {pos, dir, amp, phase, freq} (t4010a1.rs:76-82). */
static inline int src_stride(int st) { return st == ORC_SRC_T4010A1 ? 9 : 6; }

/* Rust `f as usize` for f32: NaN and negatives -> 0, saturating above. */
static inline size_t rust_f32_as_usize(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 18446744073709551616.0f) return SIZE_MAX;
    return (size_t)v;
}

/* ---------------------------------------------------------------- medium set-up */

/* sound_speed.rs:22-24: 331.3 * sqrt(t / 273.15) * 1000  [mm/s] */
ORC_EXPORT float oracle_sound_speed(float t) { return 331.3f * sqrtf(t / 273.15f) * 1000.0f; }

/* attenuation.rs:31-48 (Bass et al. 1995), returns Np/mm. */
ORC_EXPORT float oracle_attenuation_coef(float freq, float hr, float ps, float ps0, float t) {
    const float T0 = 293.15f, T01 = 273.16f, ten = 10.0f;
    float psat = ps0 * powf(ten, -6.8346f * powf(T01 / t, 1.261f) + 4.6151f);
    float h = ps0 * (hr / ps) * (psat / ps0);
    float f_ro = (24.f + 4.04e4f * h * (0.02f + h) / (0.391f + h)) / ps0;
    float f_rn = (1.f / ps0) * (9.f + 280.f * h * expf(-4.17f * (powf(T0 / t, 1.f / 3.f) - 1.f))) *
                 powf(T0 / t, 1.f / 2.f);
    float f = freq / ps;
    float alpha = (f * f) / ps0 * ps *
                  (1.84f * powf(t / T0, 1.f / 2.f) * 1e-11f +
                   powf(t / T0, -5.f / 2.f) *
                       (0.01278f * expf(-2239.1f / t) / (f_ro + f * f / f_ro) +
                        0.1068f * expf(-3352.f / t) / (f_rn + f * f / f_rn)));
    return alpha * 1e-3f;
}

/* uniform_medium.rs:102-107: k = 2*PI*f/c with c from the temperature, alpha at hr=30 %,
 * ps = ps0 = 1 atm. */
ORC_EXPORT void oracle_wavenum_atten(float temperature, float freq, float *k, float *alpha) {
    float c = oracle_sound_speed(temperature);
    *k = 2.0f * ORC_PI_F * freq / c;
    *alpha = oracle_attenuation_coef(freq, 30.f, 1.f, 1.f, temperature);
}

/* ---------------------------------------------------------------- directivity */

/* The bin index of t4010a1.rs:107-120: ceil(theta / ANGLE_DIV) as usize (NaN -> 0), clipped
 * to 10 (every index above 9 evaluates to 0). */
ORC_EXPORT int oracle_directivity_bin(float theta) {
    size_t i = rust_f32_as_usize(ceilf(theta / ANGLE_DIV_F));
    return i > 10 ? 10 : (int)i;
}

/* t4010a1.rs:107-120 in f32. */
ORC_EXPORT float oracle_directivity_t4010a1(float theta) {
    size_t i = rust_f32_as_usize(ceilf(theta / ANGLE_DIV_F));
    if (i == 0) return 1.0f;
    if (i > 9) return 0.0f;
    float a = DIR_A[i], b = DIR_B[i], c = DIR_C[i], d = DIR_D[i];
    float x = theta - ((float)i - 1.0f) * ANGLE_DIV_F;
    return a + (b + ((c + d * x) * x)) * x;
}

/* The same model evaluated in double (coefficients are the f32 table values). */
ORC_EXPORT double oracle_directivity_t4010a1_f64(double theta) {
    const double div = M_PI / 18.0;
    double q = ceil(theta / div);
    size_t i = (q > 0.0) ? (q >= 1e19 ? SIZE_MAX : (size_t)q) : 0;
    if (i == 0) return 1.0;
    if (i > 9) return 0.0;
    double a = DIR_A[i], b = DIR_B[i], c = DIR_C[i], d = DIR_D[i];
    double x = theta - ((double)i - 1.0) * div;
    return a + (b + ((c + d * x) * x)) * x;
}

/* ---------------------------------------------------------------- acos rounding */

/* The reference calls the platform libm's acosf.  glibc's acosf (2.39) is not correctly
 * rounded: it differs by one ulp from the correctly rounded value for a fair share of inputs,
 * and where theta lies within that ulp of a 10-degree directivity bin edge the bin -- and a
 * directivity jump of up to 0.164 -- depends on the libm.  Mode 0 (default) uses the
 * platform acosf like the reference; mode 1 uses acos correctly rounded to f32 (double acos,
 * then one rounding), which is what the GPU's exact near-edge path computes. */
static int g_acos_mode = 0;

ORC_EXPORT void oracle_set_acos_mode(int mode) { g_acos_mode = mode; }

static inline float ref_acosf(float c) {
    return g_acos_mode ? (float)acos((double)c) : acosf(c);
}

/* theta = acos(c) as the reference computes it (libm or correctly rounded, see
 * oracle_set_acos_mode). */
ORC_EXPORT float oracle_theta_of_cos(float c) { return ref_acosf(c); }

/* out[i] = the directivity bin of theta = acos(c[i]) (t4010a1.rs:107-120; clipped to 10). */
ORC_EXPORT void oracle_bins_of_cos(const float *c, int64_t n, int *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = oracle_directivity_bin(ref_acosf(c[i]));
}

/* ---------------------------------------------------------------- propagate */

/* uniform_medium.rs:111-120 (identical math in macros.rs:17-30), f32, no contraction. */
static inline void prop_f32(int st, const float *s, float k, float atten, float tx, float ty,
                            float tz, float *re, float *im) {
    float dx = tx - s[0], dy = ty - s[1], dz = tz - s[2];
    float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    float amp, phase, d;
    if (st == ORC_SRC_T4010A1) {
        float theta = ref_acosf((s[3] * dx + s[4] * dy + s[5] * dz) / dist);
        d = oracle_directivity_t4010a1(theta);
        amp = s[6];
        phase = s[7];
    } else {
        d = 1.0f; /* sphere_sources.rs:50-52 */
        amp = s[3];
        phase = s[4];
    }
    float r = amp * d * expf(-dist * atten) / dist;
    float phi = phase + k * dist;
    *re = r * cosf(phi);
    *im = r * sinf(phi);
}

static inline void prop_f64(int st, const float *s, float k, float atten, double tx, double ty,
                            double tz, double *re, double *im) {
    double dx = tx - (double)s[0], dy = ty - (double)s[1], dz = tz - (double)s[2];
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    double amp, phase, d;
    if (st == ORC_SRC_T4010A1) {
        double theta = acos(((double)s[3] * dx + (double)s[4] * dy + (double)s[5] * dz) / dist);
        d = oracle_directivity_t4010a1_f64(theta);
        amp = s[6];
        phase = s[7];
    } else {
        d = 1.0;
        amp = s[3];
        phase = s[4];
    }
    double r = amp * d * exp(-dist * (double)atten) / dist;
    double phi = phase + (double)k * dist;
    *re = r * cos(phi);
    *im = r * sin(phi);
}

static inline void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

ORC_EXPORT int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* One pair, f32 and f64, for unit tests. */
ORC_EXPORT void oracle_propagate(int st, const float *src, float k, float atten, float tx,
                                 float ty, float tz, float *out2) {
    prop_f32(st, src, k, atten, tx, ty, tz, &out2[0], &out2[1]);
}

/* cpu_calculator.rs:43-56 + uniform_medium.rs:122-128: for every point, the serial f32
 * complex sum over sources in index order, then the field transform.  `out` holds m floats
 * (pressure, power) or 2m floats (complex, interleaved re/im). */
ORC_EXPORT void oracle_field_f32(int st, const float *src, const float *k, const float *atten,
                                 int64_t n, const float *pts, int64_t m, int field, float *out,
                                 int nthreads) {
    const int stride = src_stride(st);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t p = 0; p < m; ++p) {
        const float tx = pts[3 * p], ty = pts[3 * p + 1], tz = pts[3 * p + 2];
        float cre = 0.0f, cim = 0.0f;
        for (int64_t j = 0; j < n; ++j) {
            float re, im;
            prop_f32(st, src + stride * j, k[j], atten[j], tx, ty, tz, &re, &im);
            cre += re;
            cim += im;
        }
        if (field == ORC_FIELD_PRESSURE) {
            out[p] = sqrtf(cre * cre + cim * cim);
        } else if (field == ORC_FIELD_POWER) {
            out[p] = cre * cre + cim * cim;
        } else {
            out[2 * p] = cre;
            out[2 * p + 1] = cim;
        }
    }
}

/* The float64 twin: same formulas in double; always writes the complex field (2m doubles). */
ORC_EXPORT void oracle_field_f64(int st, const float *src, const float *k, const float *atten,
                                 int64_t n, const float *pts, int64_t m, double *out,
                                 int nthreads) {
    const int stride = src_stride(st);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t p = 0; p < m; ++p) {
        const double tx = pts[3 * p], ty = pts[3 * p + 1], tz = pts[3 * p + 2];
        double cre = 0.0, cim = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            double re, im;
            prop_f64(st, src + stride * j, k[j], atten[j], tx, ty, tz, &re, &im);
            cre += re;
            cim += im;
        }
        out[2 * p] = cre;
        out[2 * p + 1] = cim;
    }
}

static int cmp_float(const void *a, const void *b) {
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

/* system_acc.rs:26-55: per point, the re and im terms are each summed in ascending order
 * (min-heap drained smallest first), starting from zero. */
ORC_EXPORT void oracle_field_accurate_f32(int st, const float *src, const float *k,
                                          const float *atten, int64_t n, const float *pts,
                                          int64_t m, int field, float *out, int nthreads) {
    const int stride = src_stride(st);
    set_threads(nthreads);
#pragma omp parallel
    {
        float *re_t = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
        float *im_t = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
#pragma omp for schedule(dynamic, 16)
        for (int64_t p = 0; p < m; ++p) {
            const float tx = pts[3 * p], ty = pts[3 * p + 1], tz = pts[3 * p + 2];
            for (int64_t j = 0; j < n; ++j)
                prop_f32(st, src + stride * j, k[j], atten[j], tx, ty, tz, &re_t[j], &im_t[j]);
            qsort(re_t, (size_t)n, sizeof(float), cmp_float);
            qsort(im_t, (size_t)n, sizeof(float), cmp_float);
            float cre = 0.0f, cim = 0.0f;
            for (int64_t j = 0; j < n; ++j) cre += re_t[j];
            for (int64_t j = 0; j < n; ++j) cim += im_t[j];
            if (field == ORC_FIELD_PRESSURE) {
                out[p] = sqrtf(cre * cre + cim * cim);
            } else if (field == ORC_FIELD_POWER) {
                out[p] = cre * cre + cim * cim;
            } else {
                out[2 * p] = cre;
                out[2 * p + 1] = cim;
            }
        }
        free(re_t);
        free(im_t);
    }
}

/* ---------------------------------------------------------------- grid areas */

/* builder.rs:150-152 (and :171-173, :198-200): n = ((max - min) / res) as usize + 1 in f32. */
ORC_EXPORT int64_t oracle_axis_count(float lo, float hi, float res) {
    return (int64_t)rust_f32_as_usize((hi - lo) / res) + 1;
}

/* Materialise the points of a grid area in the reference's order (grid_area.rs:59-229):
 * the first-specified axis varies fastest.  `axes` holds the axis codes (X=1, Y=2, Z=3) in
 * specification order; `dim` (1, 2 or 3) of them are ranged.  lo/hi are indexed by axis
 * (0 = x, 1 = y, 2 = z), for an `*_at` axis lo == hi.  Returns the point count; when `out`
 * is non-NULL it receives 3 floats per point.  Coordinates are o + (n as f32 * res). */
ORC_EXPORT int64_t oracle_grid_points(int dim, const float lo[3], const float hi[3], float res,
                                      const int axes[3], float *out) {
    int64_t cnt[3];
    for (int a = 0; a < 3; ++a) cnt[a] = oracle_axis_count(lo[a], hi[a], res);
    int order[3] = {axes[0] - 1, axes[1] - 1, axes[2] - 1};
    int64_t nf = dim >= 1 ? cnt[order[0]] : 1;
    int64_t ns = dim >= 2 ? cnt[order[1]] : 1;
    int64_t nt = dim >= 3 ? cnt[order[2]] : 1;
    int64_t total = nf * ns * nt;
    if (!out) return total;
    int64_t idx = 0;
    for (int64_t it = 0; it < nt; ++it)
        for (int64_t is = 0; is < ns; ++is)
            for (int64_t i0 = 0; i0 < nf; ++i0) {
                float p[3] = {lo[0], lo[1], lo[2]};
                p[order[0]] = lo[order[0]] + ((float)i0 * res);
                if (dim >= 2) p[order[1]] = lo[order[1]] + ((float)is * res);
                if (dim >= 3) p[order[2]] = lo[order[2]] + ((float)it * res);
                out[3 * idx] = p[0];
                out[3 * idx + 1] = p[1];
                out[3 * idx + 2] = p[2];
                ++idx;
            }
    return total;
}

/* ---------------------------------------------------------------- focal law */

/* focal_point.rs:27-40: phase = -2*PI * ((|pos - f| mod lambda) / lambda), lambda = c / freq. */
ORC_EXPORT void oracle_focal_point(int st, float *src, int64_t n, float sound_speed, float fx,
                                   float fy, float fz) {
    const int stride = src_stride(st);
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    const int ifreq = st == ORC_SRC_T4010A1 ? 8 : 5;
    for (int64_t j = 0; j < n; ++j) {
        float *s = src + stride * j;
        float dx = s[0] - fx, dy = s[1] - fy, dz = s[2] - fz;
        float d = sqrtf(dx * dx + dy * dy + dz * dz);
        float wave_length = sound_speed / s[ifreq];
        float phase = fmodf(d, wave_length) / wave_length;
        phase = -2.0f * ORC_PI_F * phase;
        s[iphase] = phase;
    }
}

/* bessel.rs:30-51: v = (dir.y, -dir.x, 0), theta_w = asin |v|; each source's offset
 * r = pos - point is rotated, r' = r cos(theta_w) + (r x v) sin(theta_w) + v (v.r)(1 - cos(theta_w)),
 * dist = sin(theta) |r'_xy| - cos(theta) r'_z, phase = -2 pi fmod(dist, lambda) / lambda.  f32 with
 * nalgebra's component orders: cross (a.y b.z - a.z b.y, a.z b.x - a.x b.z, a.x b.y - a.y b.x),
 * dot and norm^2 ((x x' + y y') + z z'). */
ORC_EXPORT void oracle_bessel_beam(int st, float *src, int64_t n, float sound_speed, float px,
                                   float py, float pz, float dx, float dy, float dz, float theta) {
    (void)dz;
    const int stride = src_stride(st);
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    const int ifreq = st == ORC_SRC_T4010A1 ? 8 : 5;
    float v[3] = {dy, -dx, 0.0f};
    float theta_w = asinf(sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]));
    for (int64_t j = 0; j < n; ++j) {
        float *s = src + stride * j;
        float r[3] = {s[0] - px, s[1] - py, s[2] - pz};
        float xr[3] = {r[1] * v[2] - r[2] * v[1], r[2] * v[0] - r[0] * v[2],
                       r[0] * v[1] - r[1] * v[0]};
        float vdr = (v[0] * r[0] + v[1] * r[1]) + v[2] * r[2];
        float scale = vdr * (1.0f - cosf(theta_w));
        float q[3];
        for (int c = 0; c < 3; ++c) {
            float a = r[c] * cosf(theta_w);
            float b = xr[c] * sinf(theta_w);
            q[c] = (a + b) + v[c] * scale;
        }
        float dist = sinf(theta) * sqrtf(q[0] * q[0] + q[1] * q[1]) - cosf(theta) * q[2];
        float wave_length = sound_speed / s[ifreq];
        float phase = fmodf(dist, wave_length) / wave_length;
        s[iphase] = -2.0f * ORC_PI_F * phase;
    }
}

/* ---------------------------------------------------------------- greedy
 * combination/greedy.rs:21-83 in f32: every phase set to 0; candidates exp(i 2 pi k / div)
 * (from_polar(e^0, a)); source by source, each candidate's sum over foci of
 * |amp_j - |propagate(i, focus_j) * c_k + cache_j|| (complex norm = hypot), the first minimum
 * kept, cache += its terms, phase_i = arg of the chosen candidate. */
ORC_EXPORT void oracle_greedy_f32(int st, float *src, const float *k, const float *atten, int64_t n,
                                  const float *foci, const float *amps, int64_t m, int div) {
    const int stride = src_stride(st);
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    float *cre = (float *)calloc((size_t)(m > 0 ? m : 1), sizeof(float));
    float *cim = (float *)calloc((size_t)(m > 0 ? m : 1), sizeof(float));
    float *pre = (float *)malloc(sizeof(float) * (size_t)div);
    float *pim = (float *)malloc(sizeof(float) * (size_t)div);
    float *tre = (float *)malloc(sizeof(float) * (size_t)(m > 0 ? m : 1) * (size_t)div);
    float *tim = (float *)malloc(sizeof(float) * (size_t)(m > 0 ? m : 1) * (size_t)div);
    for (int q = 0; q < div; ++q) {
        float a = 2.0f * ORC_PI_F * (float)q / (float)div;
        pre[q] = 1.0f * cosf(a);
        pim[q] = 1.0f * sinf(a);
    }
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = 0.0f;
    for (int64_t i = 0; i < n; ++i) {
        int best = 0;
        float min_v = INFINITY;
        for (int q = 0; q < div; ++q) {
            float v = 0.0f;
            for (int64_t j = 0; j < m; ++j) {
                float gr, gi;
                prop_f32(st, src + stride * i, k[i], atten[i], foci[3 * j], foci[3 * j + 1],
                         foci[3 * j + 2], &gr, &gi);
                float tr = gr * pre[q] - gi * pim[q];
                float ti = gr * pim[q] + gi * pre[q];
                tre[q * m + j] = tr;
                tim[q * m + j] = ti;
                v += fabsf(amps[j] - hypotf(tr + cre[j], ti + cim[j]));
            }
            if (v < min_v) {
                min_v = v;
                best = q;
            }
        }
        for (int64_t j = 0; j < m; ++j) {
            cre[j] += tre[best * m + j];
            cim[j] += tim[best * m + j];
        }
        src[stride * i + iphase] = atan2f(pim[best], pre[best]);
    }
    free(cre);
    free(cim);
    free(pre);
    free(pim);
    free(tre);
    free(tim);
}

/* ---------------------------------------------------------------- NLS phase retrieval
 * nls/macros.rs:16-58 and nls/{gradient_descent,gauss_newton,lm}.rs in float64, with the
 * reference's dense formulas taken literally: B = [G | -diag(amps)] (m x N, N = n + m, G with
 * every phase 0), BhB = B^H B (N x N), T = exp(-i x): JtJ = Re(BhB o T T^H), Jtf = column sums of
 * Im(BhB o T T^H); F(x) = Re(t^H BhB t), t = exp(i x).  Solves: (JtJ + mu I) by Cholesky (the
 * reference's QR gives the same solution), pinv(JtJ, 1e-3) by a Jacobi eigendecomposition
 * (JtJ is symmetric positive semi-definite, so its singular values are its eigenvalues).
 * kind: 0 gradient descent, 1 Gauss-Newton, 2 Levenberg-Marquardt.  Writes the phases. */
static void nls_jtj_jtf(const double *bre, const double *bim, int64_t N, const double *x,
                        double *A, double *g) {
    /* (BhB o T T^H)_ab = BhB_ab T_a conj(T_b), T = exp(-i x) */
    for (int64_t b = 0; b < N; ++b) g[b] = 0.0;
    for (int64_t a = 0; a < N; ++a)
        for (int64_t b = 0; b < N; ++b) {
            double hr = bre[a * N + b], hi = bim[a * N + b];
            double ph = -x[a] + x[b]; /* T_a conj(T_b) = exp(-i x_a + i x_b) */
            double cr = cos(ph), ci = sin(ph);
            double vr = hr * cr - hi * ci, vi = hr * ci + hi * cr;
            if (A) A[a * N + b] = vr;
            g[b] += vi;
        }
}

static double nls_fx(const double *bre, const double *bim, int64_t N, const double *x) {
    double f = 0.0; /* Re(t^H BhB t), t = exp(i x) */
    for (int64_t a = 0; a < N; ++a)
        for (int64_t b = 0; b < N; ++b) {
            double ph = -x[a] + x[b];
            f += bre[a * N + b] * cos(ph) - bim[a * N + b] * sin(ph);
        }
    return f;
}

static int chol_solve(double *a, double *b, int64_t k) {
    for (int64_t j = 0; j < k; ++j) {
        double d = a[j * k + j];
        for (int64_t p = 0; p < j; ++p) d -= a[j * k + p] * a[j * k + p];
        if (!(d > 0.0)) return 0;
        d = sqrt(d);
        a[j * k + j] = d;
        for (int64_t i = j + 1; i < k; ++i) {
            double t = a[i * k + j];
            for (int64_t p = 0; p < j; ++p) t -= a[i * k + p] * a[j * k + p];
            a[i * k + j] = t / d;
        }
    }
    for (int64_t i = 0; i < k; ++i) {
        double t = b[i];
        for (int64_t p = 0; p < i; ++p) t -= a[i * k + p] * b[p];
        b[i] = t / a[i * k + i];
    }
    for (int64_t i = k - 1; i >= 0; --i) {
        double t = b[i];
        for (int64_t p = i + 1; p < k; ++p) t -= a[p * k + i] * b[p];
        b[i] = t / a[i * k + i];
    }
    return 1;
}

/* Cyclic Jacobi: a (symmetric, destroyed) -> eigenvalues lam, eigenvectors in v's columns. */
static void jacobi(double *a, int64_t k, double *lam, double *v) {
    for (int64_t i = 0; i < k * k; ++i) v[i] = 0.0;
    for (int64_t i = 0; i < k; ++i) v[i * k + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int64_t i = 0; i < k * k; ++i) tot += a[i] * a[i];
        for (int64_t i = 0; i < k; ++i)
            for (int64_t j = 0; j < k; ++j)
                if (i != j) off += a[i * k + j] * a[i * k + j];
        if (off <= 1e-30 * tot) break;
        for (int64_t p = 0; p < k; ++p)
            for (int64_t q = p + 1; q < k; ++q) {
                double apq = a[p * k + q];
                if (apq == 0.0) continue;
                double th = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int64_t r = 0; r < k; ++r) {
                    double x1 = a[r * k + p], x2 = a[r * k + q];
                    a[r * k + p] = c * x1 - sn * x2;
                    a[r * k + q] = sn * x1 + c * x2;
                }
                for (int64_t r = 0; r < k; ++r) {
                    double x1 = a[p * k + r], x2 = a[q * k + r];
                    a[p * k + r] = c * x1 - sn * x2;
                    a[q * k + r] = sn * x1 + c * x2;
                }
                for (int64_t r = 0; r < k; ++r) {
                    double x1 = v[r * k + p], x2 = v[r * k + q];
                    v[r * k + p] = c * x1 - sn * x2;
                    v[r * k + q] = sn * x1 + c * x2;
                }
            }
    }
    for (int64_t i = 0; i < k; ++i) lam[i] = a[i * k + i];
}

static double vmax(const double *g, int64_t N) {
    double mx = -INFINITY;
    for (int64_t b = 0; b < N; ++b)
        if (g[b] > mx) mx = g[b];
    return mx;
}

static double vnorm(const double *v, int64_t N) {
    double s2 = 0.0;
    for (int64_t b = 0; b < N; ++b) s2 += v[b] * v[b];
    return sqrt(s2);
}

ORC_EXPORT void oracle_nls_f64(int kind, int st, float *src, const float *k, const float *atten,
                               int64_t n, const float *foci, const float *amps, int64_t m) {
    const int stride = src_stride(st);
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    const int64_t N = n + m;
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = 0.0f;
    double *bre = calloc((size_t)(m * N + 1), sizeof(double));
    double *bim = calloc((size_t)(m * N + 1), sizeof(double));
    for (int64_t i = 0; i < m; ++i) {
        for (int64_t j = 0; j < n; ++j)
            prop_f64(st, src + stride * j, k[j], atten[j], foci[3 * i], foci[3 * i + 1],
                     foci[3 * i + 2], &bre[i * N + j], &bim[i * N + j]);
        bre[i * N + n + i] = -(double)amps[i];
    }
    double *hre = calloc((size_t)(N * N + 1), sizeof(double));
    double *him = calloc((size_t)(N * N + 1), sizeof(double));
    for (int64_t a = 0; a < N; ++a)
        for (int64_t b = 0; b < N; ++b) {
            double sr = 0, si = 0; /* sum_i conj(B_ia) B_ib */
            for (int64_t i = 0; i < m; ++i) {
                sr += bre[i * N + a] * bre[i * N + b] + bim[i * N + a] * bim[i * N + b];
                si += bre[i * N + a] * bim[i * N + b] - bim[i * N + a] * bre[i * N + b];
            }
            hre[a * N + b] = sr;
            him[a * N + b] = si;
        }
    double *x = calloc((size_t)(N + 1), sizeof(double));
    double *g = calloc((size_t)(N + 1), sizeof(double));
    double *h = calloc((size_t)(N + 1), sizeof(double));
    double *xn = calloc((size_t)(N + 1), sizeof(double));
    double *A = calloc((size_t)(N * N + 1), sizeof(double));
    double *W = calloc((size_t)(N * N + 1), sizeof(double));
    double *V = calloc((size_t)(N * N + 1), sizeof(double));
    double *lam = calloc((size_t)(N + 1), sizeof(double));
    if (kind == 0) { /* gradient_descent.rs:44-52 */
        for (int it = 0; it < 10000; ++it) {
            nls_jtj_jtf(hre, him, N, x, NULL, g);
            if (vmax(g, N) <= 1e-6) break;
            for (int64_t b = 0; b < N; ++b) x[b] -= 0.1 * g[b];
        }
    } else if (kind == 1) { /* gauss_newton.rs:44-85 */
        nls_jtj_jtf(hre, him, N, x, A, g);
        int found = vmax(g, N) <= 1e-8;
        for (int it = 0; it < 200 && !found; ++it) {
            memcpy(W, A, sizeof(double) * (size_t)(N * N));
            jacobi(W, N, lam, V);
            for (int64_t b = 0; b < N; ++b) h[b] = 0.0;
            for (int64_t q = 0; q < N; ++q) {
                if (!(lam[q] > 1e-3)) continue;
                double proj = 0.0;
                for (int64_t b = 0; b < N; ++b) proj += V[b * N + q] * g[b];
                for (int64_t b = 0; b < N; ++b) h[b] -= V[b * N + q] * proj / lam[q];
            }
            if (vnorm(h, N) <= 1e-8 * (vnorm(x, N) + 1e-8)) {
                found = 1;
            } else {
                for (int64_t b = 0; b < N; ++b) x[b] += h[b];
                nls_jtj_jtf(hre, him, N, x, A, g);
                found = vmax(g, N) <= 1e-8;
            }
        }
    } else { /* lm.rs:44-100 */
        double nu = 2.0;
        nls_jtj_jtf(hre, him, N, x, A, g);
        double a_max = -INFINITY;
        for (int64_t b = 0; b < N; ++b)
            if (A[b * N + b] > a_max) a_max = A[b * N + b];
        double mu = 1e-3 * a_max;
        int found = vmax(g, N) <= 1e-8;
        double fx = nls_fx(hre, him, N, x);
        for (int it = 0; it < 200 && !found; ++it) {
            memcpy(W, A, sizeof(double) * (size_t)(N * N));
            for (int64_t b = 0; b < N; ++b) W[b * N + b] += mu;
            for (int64_t b = 0; b < N; ++b) h[b] = g[b];
            if (!chol_solve(W, h, N)) break;
            for (int64_t b = 0; b < N; ++b) h[b] = -h[b];
            if (vnorm(h, N) <= 1e-8 * (vnorm(x, N) + 1e-8)) {
                found = 1;
            } else {
                for (int64_t b = 0; b < N; ++b) xn[b] = x[b] + h[b];
                double fx_new = nls_fx(hre, him, N, xn);
                double l0 = 0.0;
                for (int64_t b = 0; b < N; ++b) l0 += h[b] * (mu * h[b] - g[b]);
                l0 *= 0.5;
                double rho = (fx - fx_new) / l0;
                fx = fx_new;
                if (rho > 0.0) {
                    memcpy(x, xn, sizeof(double) * (size_t)N);
                    nls_jtj_jtf(hre, him, N, x, A, g);
                    found = vmax(g, N) <= 1e-8;
                    double c = 2.0 * rho - 1.0;
                    double f = 1.0 - c * c * c;
                    mu *= f > 1.0 / 3.0 ? f : 1.0 / 3.0;
                    nu = 2.0;
                } else {
                    mu *= nu;
                    nu *= 2.0;
                }
            }
        }
    }
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = (float)x[j];
    free(bre);
    free(bim);
    free(hre);
    free(him);
    free(x);
    free(g);
    free(h);
    free(xn);
    free(A);
    free(W);
    free(V);
    free(lam);
}

/* ---------------------------------------------------------------- APO
 * nls/apo.rs:36-158 in float64, literally: explicit R_i = G^H D_i G (n x n each),
 * q0 = (G^H G + lambda I)^-1 G^H p (Cholesky; the reference's QR gives the same solution),
 * J(q) = sum_i |q^H R_i q - p_i^2|^2 + lambda |q.q| (nalgebra's dot: no conjugation),
 * grad J = sum_i R_i q (p_i^2 - |q^H R_i q|) + lambda q, the line search over a = i / 100,
 * and H += y y^T / (y.s) - (H s)(H s)^T / (s^T H s) (transposes, bilinear dots).  The output
 * amplitude is amp |q_j| / camax(q), camax being nalgebra 0.27.1's largest |re| + |im| of the
 * entries; the phase is arg q_j. */
#include <complex.h>

static double apo_J(const double complex *R, const double complex *q, const double *p2, int64_t n,
                    int64_t m, double lambda) {
    double v = 0.0;
    for (int64_t i = 0; i < m; ++i) {
        double complex qrq = 0.0;
        for (int64_t a = 0; a < n; ++a) {
            double complex rq = 0.0;
            for (int64_t b = 0; b < n; ++b) rq += R[(i * n + a) * n + b] * q[b];
            qrq += conj(q[a]) * rq;
        }
        double complex t = qrq - p2[i];
        v += creal(t) * creal(t) + cimag(t) * cimag(t);
    }
    double complex qq = 0.0;
    for (int64_t b = 0; b < n; ++b) qq += q[b] * q[b];
    return v + cabs(qq) * lambda;
}

static void apo_grad(const double complex *R, const double complex *q, const double *p2,
                     int64_t n, int64_t m, double lambda, double complex *g) {
    for (int64_t a = 0; a < n; ++a) g[a] = lambda * q[a];
    for (int64_t i = 0; i < m; ++i) {
        double complex qrq = 0.0;
        for (int64_t a = 0; a < n; ++a) {
            double complex rq = 0.0;
            for (int64_t b = 0; b < n; ++b) rq += R[(i * n + a) * n + b] * q[b];
            qrq += conj(q[a]) * rq;
        }
        double s = p2[i] - cabs(qrq);
        for (int64_t a = 0; a < n; ++a) {
            double complex rq = 0.0;
            for (int64_t b = 0; b < n; ++b) rq += R[(i * n + a) * n + b] * q[b];
            g[a] += rq * s;
        }
    }
}

ORC_EXPORT void oracle_apo_f64(int st, float *src, const float *k, const float *atten, int64_t n,
                               const float *foci, const float *amps, int64_t m, float lambda) {
    const int stride = src_stride(st);
    const int iamp = st == ORC_SRC_T4010A1 ? 6 : 3;
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = 0.0f;
    double complex *G = calloc((size_t)(m * n + 1), sizeof(double complex));
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j) {
            double re, im;
            prop_f64(st, src + stride * j, k[j], atten[j], foci[3 * i], foci[3 * i + 1],
                     foci[3 * i + 2], &re, &im);
            G[i * n + j] = re + I * im;
        }
    double *p2 = calloc((size_t)(m + 1), sizeof(double));
    for (int64_t i = 0; i < m; ++i) p2[i] = (double)amps[i] * (double)amps[i];
    /* q0: (G^H G + lambda I) q0 = G^H p, complex Cholesky */
    double complex *A = calloc((size_t)(n * n + 1), sizeof(double complex));
    double complex *q = calloc((size_t)(n + 1), sizeof(double complex));
    for (int64_t a = 0; a < n; ++a) {
        for (int64_t b = 0; b < n; ++b) {
            double complex v = 0.0;
            for (int64_t i = 0; i < m; ++i) v += conj(G[i * n + a]) * G[i * n + b];
            A[a * n + b] = v + (a == b ? (double)lambda : 0.0);
        }
        double complex v = 0.0;
        for (int64_t i = 0; i < m; ++i) v += conj(G[i * n + a]) * (double)amps[i];
        q[a] = v;
    }
    for (int64_t j = 0; j < n; ++j) { /* A = L L^H in place (lower) */
        double d = creal(A[j * n + j]);
        for (int64_t p = 0; p < j; ++p) d -= creal(A[j * n + p] * conj(A[j * n + p]));
        d = sqrt(d);
        A[j * n + j] = d;
        for (int64_t i = j + 1; i < n; ++i) {
            double complex t = A[i * n + j];
            for (int64_t p = 0; p < j; ++p) t -= A[i * n + p] * conj(A[j * n + p]);
            A[i * n + j] = t / d;
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        double complex t = q[i];
        for (int64_t p = 0; p < i; ++p) t -= A[i * n + p] * q[p];
        q[i] = t / creal(A[i * n + i]);
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        double complex t = q[i];
        for (int64_t p = i + 1; p < n; ++p) t -= conj(A[p * n + i]) * q[p];
        q[i] = t / creal(A[i * n + i]);
    }
    double complex *R = calloc((size_t)(m * n * n + 1), sizeof(double complex));
    for (int64_t i = 0; i < m; ++i)
        for (int64_t a = 0; a < n; ++a)
            for (int64_t b = 0; b < n; ++b) R[(i * n + a) * n + b] = conj(G[i * n + a]) * G[i * n + b];
    double complex *H = calloc((size_t)(n * n + 1), sizeof(double complex));
    for (int64_t a = 0; a < n; ++a) H[a * n + a] = 1.0;
    double complex *g = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *gn = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *d = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *qn = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *sv = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *u = calloc((size_t)(n + 1), sizeof(double complex));
    double complex *tmp = calloc((size_t)(n + 1), sizeof(double complex));
    apo_grad(R, q, p2, n, m, lambda, g);
    for (int it = 0; it < 200; ++it) {
        for (int64_t a = 0; a < n; ++a) {
            double complex v = 0.0;
            for (int64_t b = 0; b < n; ++b) v += H[a * n + b] * g[b];
            d[a] = -v;
        }
        double alpha = 0.0, best = INFINITY;
        for (int li = 0; li < 100; ++li) {
            double a = (double)((float)li / 100.0f);
            for (int64_t b = 0; b < n; ++b) tmp[b] = q[b] + d[b] * a;
            double v = apo_J(R, tmp, p2, n, m, lambda);
            if (v < best) {
                best = v;
                alpha = a;
            }
        }
        double dn = 0.0;
        for (int64_t b = 0; b < n; ++b) {
            d[b] *= alpha;
            dn += creal(d[b] * conj(d[b]));
        }
        if (sqrt(dn) < 1e-8) break;
        for (int64_t b = 0; b < n; ++b) qn[b] = q[b] + d[b];
        apo_grad(R, qn, p2, n, m, lambda, gn);
        for (int64_t b = 0; b < n; ++b) sv[b] = gn[b] - g[b];
        double complex ys = 0.0, su = 0.0;
        for (int64_t a = 0; a < n; ++a) {
            double complex v = 0.0;
            for (int64_t b = 0; b < n; ++b) v += H[a * n + b] * sv[b];
            u[a] = v;
        }
        for (int64_t b = 0; b < n; ++b) {
            ys += d[b] * sv[b];
            su += sv[b] * u[b];
        }
        for (int64_t a = 0; a < n; ++a)
            for (int64_t b = 0; b < n; ++b) H[a * n + b] += d[a] * d[b] / ys - u[a] * u[b] / su;
        memcpy(q, qn, sizeof(double complex) * (size_t)n);
        memcpy(g, gn, sizeof(double complex) * (size_t)n);
    }
    double mx = 0.0; /* nalgebra 0.27.1 camax: the largest |re| + |im| */
    for (int64_t b = 0; b < n; ++b)
        if (fabs(creal(q[b])) + fabs(cimag(q[b])) > mx) mx = fabs(creal(q[b])) + fabs(cimag(q[b]));
    for (int64_t b = 0; b < n; ++b) {
        src[stride * b + iamp] = (float)((double)src[stride * b + iamp] * cabs(q[b]) / mx);
        src[stride * b + iphase] = (float)carg(q[b]);
    }
    free(G); free(p2); free(A); free(q); free(R); free(H); free(g); free(gn); free(d); free(qn);
    free(sv); free(u); free(tmp);
}

/* ---------------------------------------------------------------- G and the solvers */

/* macros.rs:32-53: G[i, j] = propagate(source j, focus i) with the sources' current amp and
 * phase.  Written row-major here: G[2*(i*n + j)] = re, [+1] = im (the reference stores the
 * same m x n matrix column-major). */
ORC_EXPORT void oracle_build_g_f32(int st, const float *src, const float *k, const float *atten,
                                   int64_t n, const float *foci, int64_t m, float *g) {
    const int stride = src_stride(st);
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j)
            prop_f32(st, src + stride * j, k[j], atten[j], foci[3 * i], foci[3 * i + 1],
                     foci[3 * i + 2], &g[2 * (i * n + j)], &g[2 * (i * n + j) + 1]);
}

ORC_EXPORT void oracle_build_g_f64(int st, const float *src, const float *k, const float *atten,
                                   int64_t n, const float *foci, int64_t m, double *g,
                                   int nthreads) {
    const int stride = src_stride(st);
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j)
            prop_f64(st, src + stride * j, k[j], atten[j], foci[3 * i], foci[3 * i + 1],
                     foci[3 * i + 2], &g[2 * (i * n + j)], &g[2 * (i * n + j) + 1]);
}

typedef struct {
    double re, im;
} cplx;

static inline cplx cmul(cplx a, cplx b) {
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline double cabs_(cplx a) { return hypot(a.re, a.im); }

/* Zero the phases (gs_pat.rs:38-41), build G (:45) in double. Returns malloc'd G (m x n). */
static cplx *gspat_build(int st, float *src, const float *k, const float *atten, int64_t n,
                         const float *foci, int64_t m) {
    const int stride = src_stride(st);
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = 0.0f;
    cplx *G = (cplx *)malloc(sizeof(cplx) * (size_t)(m * n));
    oracle_build_g_f64(st, src, k, atten, n, foci, m, (double *)G, 0);
    return G;
}

static void write_q(int st, float *src, int64_t n, const cplx *q, double *q_out) {
    const int stride = src_stride(st);
    const int iamp = st == ORC_SRC_T4010A1 ? 6 : 3;
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    for (int64_t j = 0; j < n; ++j) {
        src[stride * j + iamp] = (float)cabs_(q[j]);
        src[stride * j + iphase] = (float)atan2(q[j].im, q[j].re);
        if (q_out) {
            q_out[2 * j] = q[j].re;
            q_out[2 * j + 1] = q[j].im;
        }
    }
}

/* gs_pat.rs:35-81 in double.  Updates amp/phase of `src` in place like the reference and,
 * if q_out is non-NULL, stores the complex q (2n doubles). */
ORC_EXPORT void oracle_gspat_f64(int st, float *src, const float *k, const float *atten,
                                 int64_t n, const float *foci, const float *amps, int64_t m,
                                 int repeat, double *q_out) {
    cplx *G = gspat_build(st, src, k, atten, n, foci, m);
    double *den = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j) den[j] += cabs_(G[i * n + j]); /* row_sum: column sums */
    /* B = [conj(G_ij) / den_j^2]^T, n x m: B[j*m + i] */
    cplx *B = (cplx *)malloc(sizeof(cplx) * (size_t)(m * n));
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j) {
            double s = den[j] * den[j];
            cplx b = {G[i * n + j].re / s, -G[i * n + j].im / s};
            B[j * m + i] = b;
        }
    cplx *R = (cplx *)calloc((size_t)(m * m), sizeof(cplx));
    for (int64_t i = 0; i < m; ++i)
        for (int64_t c = 0; c < m; ++c) {
            cplx acc = {0, 0};
            for (int64_t j = 0; j < n; ++j) {
                cplx t = cmul(G[i * n + j], B[j * m + c]);
                acc.re += t.re;
                acc.im += t.im;
            }
            R[i * m + c] = acc;
        }
    cplx *p = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    cplx *gamma = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    for (int64_t i = 0; i < m; ++i) {
        p[i].re = amps[i];
        p[i].im = 0.0;
    }
    for (int it = 0; it <= repeat; ++it) {
        for (int64_t i = 0; i < m; ++i) {
            cplx acc = {0, 0};
            for (int64_t c = 0; c < m; ++c) {
                cplx t = cmul(R[i * m + c], p[c]);
                acc.re += t.re;
                acc.im += t.im;
            }
            gamma[i] = acc;
        }
        if (it == repeat) break;
        for (int64_t i = 0; i < m; ++i) {
            double a = cabs_(gamma[i]);
            p[i].re = gamma[i].re / a * amps[i];
            p[i].im = gamma[i].im / a * amps[i];
        }
    }
    for (int64_t i = 0; i < m; ++i) {
        double a = cabs_(gamma[i]);
        double s = (double)amps[i] * (double)amps[i] / (a * a);
        p[i].re = gamma[i].re * s;
        p[i].im = gamma[i].im * s;
    }
    cplx *q = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int64_t j = 0; j < n; ++j) {
        cplx acc = {0, 0};
        for (int64_t i = 0; i < m; ++i) {
            cplx t = cmul(B[j * m + i], p[i]);
            acc.re += t.re;
            acc.im += t.im;
        }
        q[j] = acc;
    }
    write_q(st, src, n, q, q_out);
    free(G);
    free(den);
    free(B);
    free(R);
    free(p);
    free(gamma);
    free(q);
}

typedef struct {
    float re, im;
} cplxf;

/* num-complex Complex<f32> arithmetic: (a re - b im, a im + b re) per product, hypotf modulus. */
static inline cplxf cmulf(cplxf a, cplxf b) {
    cplxf r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cplxf caddf(cplxf a, cplxf b) {
    cplxf r = {a.re + b.re, a.im + b.im};
    return r;
}

/* gs_pat.rs:38-81 in f32, as the reference computes it: G from the f32 propagate (phases
 * zeroed), den_j = sum_i |G_ij| (nalgebra row_sum, rows in order), B = (conj(G_ij) / (den_j
 * den_j))^T, R = G B and every matrix-vector product as nalgebra's gemv without BLAS (columns
 * accumulated in order: y = x_0 A_0, then y += x_c A_c), the 100 normalisations
 * gamma / |gamma| * p0, the final gamma / (|gamma| |gamma|) * p0 * p0, and q = B p, whose
 * modulus and argument (hypotf, atan2f) become each source's amp and phase.  Updates `src` in
 * place; q_out (2n doubles) receives q. */
ORC_EXPORT void oracle_gspat_f32(int st, float *src, const float *k, const float *atten,
                                 int64_t n, const float *foci, const float *amps, int64_t m,
                                 int repeat, double *q_out) {
    const int stride = src_stride(st);
    const int iamp = st == ORC_SRC_T4010A1 ? 6 : 3;
    const int iphase = st == ORC_SRC_T4010A1 ? 7 : 4;
    for (int64_t j = 0; j < n; ++j) src[stride * j + iphase] = 0.0f;
    cplxf *G = (cplxf *)malloc(sizeof(cplxf) * (size_t)(m * n)); /* G[i*n + j] */
    oracle_build_g_f32(st, src, k, atten, n, foci, m, (float *)G);
    float *den = (float *)calloc((size_t)n, sizeof(float));
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) den[j] += hypotf(G[i * n + j].re, G[i * n + j].im);
    cplxf *B = (cplxf *)malloc(sizeof(cplxf) * (size_t)(m * n)); /* B[j*m + i], n x m */
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j) {
            const float s = den[j] * den[j];
            cplxf b = {G[i * n + j].re / s, -G[i * n + j].im / s};
            B[j * m + i] = b;
        }
    /* R = G B (m x m): column c = sum_j B[j, c] G[:, j] */
    cplxf *R = (cplxf *)malloc(sizeof(cplxf) * (size_t)(m * m)); /* R[i*m + c] */
    for (int64_t c = 0; c < m; ++c)
        for (int64_t i = 0; i < m; ++i) {
            cplxf acc = cmulf(B[0 * m + c], G[i * n + 0]);
            for (int64_t j = 1; j < n; ++j) acc = caddf(cmulf(B[j * m + c], G[i * n + j]), acc);
            R[i * m + c] = acc;
        }
    cplxf *p = (cplxf *)malloc(sizeof(cplxf) * (size_t)m);
    cplxf *gamma = (cplxf *)malloc(sizeof(cplxf) * (size_t)m);
    for (int64_t i = 0; i < m; ++i) {
        p[i].re = amps[i];
        p[i].im = 0.0f;
    }
    for (int it = 0; it <= repeat; ++it) {
        /* gamma = R p: gamma_i = sum_c p_c R[i, c] */
        for (int64_t i = 0; i < m; ++i) {
            cplxf acc = cmulf(p[0], R[i * m + 0]);
            for (int64_t c = 1; c < m; ++c) acc = caddf(cmulf(p[c], R[i * m + c]), acc);
            gamma[i] = acc;
        }
        if (it == repeat) break;
        for (int64_t i = 0; i < m; ++i) {
            const float a = hypotf(gamma[i].re, gamma[i].im);
            const cplxf g = {gamma[i].re / a, gamma[i].im / a};
            const cplxf p0 = {amps[i], 0.0f};
            p[i] = cmulf(g, p0);
        }
    }
    for (int64_t i = 0; i < m; ++i) {
        const float a = hypotf(gamma[i].re, gamma[i].im);
        const float s = a * a;
        const cplxf g = {gamma[i].re / s, gamma[i].im / s};
        const cplxf p0 = {amps[i], 0.0f};
        p[i] = cmulf(cmulf(g, p0), p0);
    }
    /* q = B p: q_j = sum_i p_i B[j, i] */
    for (int64_t j = 0; j < n; ++j) {
        cplxf acc = cmulf(p[0], B[j * m + 0]);
        for (int64_t i = 1; i < m; ++i) acc = caddf(cmulf(p[i], B[j * m + i]), acc);
        src[stride * j + iamp] = hypotf(acc.re, acc.im);
        src[stride * j + iphase] = atan2f(acc.im, acc.re);
        if (q_out) {
            q_out[2 * j] = acc.re;
            q_out[2 * j + 1] = acc.im;
        }
    }
    free(G);
    free(den);
    free(B);
    free(R);
    free(p);
    free(gamma);
}

/* naive.rs:29-51 in double: q = G^H p. */
ORC_EXPORT void oracle_naive_f64(int st, float *src, const float *k, const float *atten,
                                 int64_t n, const float *foci, const float *amps, int64_t m,
                                 double *q_out) {
    cplx *G = gspat_build(st, src, k, atten, n, foci, m);
    cplx *q = (cplx *)calloc((size_t)n, sizeof(cplx));
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            q[j].re += G[i * n + j].re * amps[i];
            q[j].im -= G[i * n + j].im * amps[i];
        }
    write_q(st, src, n, q, q_out);
    free(G);
    free(q);
}

/* gs.rs:33-78 in double. */
ORC_EXPORT void oracle_gs_f64(int st, float *src, const float *k, const float *atten, int64_t n,
                              const float *foci, const float *amps, int64_t m, int repeat,
                              double *q_out) {
    const int stride = src_stride(st);
    const int iamp = st == ORC_SRC_T4010A1 ? 6 : 3;
    cplx *G = gspat_build(st, src, k, atten, n, foci, m);
    double *q0 = (double *)malloc(sizeof(double) * (size_t)n);
    cplx *q = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *p = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    for (int64_t j = 0; j < n; ++j) {
        q0[j] = src[stride * j + iamp];
        q[j].re = q0[j];
        q[j].im = 0.0;
    }
    for (int it = 0; it < repeat; ++it) {
        for (int64_t i = 0; i < m; ++i) {
            cplx g = {0, 0};
            for (int64_t j = 0; j < n; ++j) {
                cplx t = cmul(G[i * n + j], q[j]);
                g.re += t.re;
                g.im += t.im;
            }
            double a = cabs_(g);
            p[i].re = g.re / a * amps[i];
            p[i].im = g.im / a * amps[i];
        }
        for (int64_t j = 0; j < n; ++j) {
            cplx x = {0, 0};
            for (int64_t i = 0; i < m; ++i) {
                cplx gc = {G[i * n + j].re, -G[i * n + j].im};
                cplx t = cmul(gc, p[i]);
                x.re += t.re;
                x.im += t.im;
            }
            double a = cabs_(x);
            q[j].re = x.re / a * q0[j];
            q[j].im = x.im / a * q0[j];
        }
    }
    write_q(st, src, n, q, q_out);
    free(G);
    free(q0);
    free(q);
    free(p);
}
