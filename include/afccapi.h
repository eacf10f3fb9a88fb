/*
 * afccapi.h -- C ABI of libafccapi.so, the GB300 drop-in for the reference's `afccapi` cdylib
 * (shinolab/acoustic-field-calculator 0.6.1, capi/Cargo.toml:9-12).
 *
 * Every AFC_* / AFO_* function below keeps the reference's name, argument list, argument
 * meaning and return type; the comment on each cites the Rust export it replaces
 * (capi/src/<file>.rs:<lines>).  Handles are opaque `void*` created and freed by the matching
 * AFC_Create* / AFC_Free* calls; integer tags select the concrete type exactly as in
 * capi/src/type_inference_aux.rs:53-103:
 *   calculator  Cpu = 0, Accurate = 1, Gpu = 2
 *   source      SphereWaveSource = 0, T4010A1 = 1
 *   area        GridArea1D = 0, GridArea2D = 1, GridArea3D = 2, ScatterArea = 3
 *   field       Pressure = 0, Power = 1, ComplexPressure = 2
 *   axis        X = 1, Y = 2, Z = 3 (observe_area/grid/dimension.rs:23-39)
 * Lengths are millimetres, phases radians, frequencies hertz.
 *
 * Differences from the reference, all additive:
 *   - All three calculator tags compute on the GPU (no CPU path exists in this library):
 *     Cpu and Gpu run the FP32 direct-summation kernel, Accurate runs the same kernel with
 *     compensated (Neumaier) accumulation.  Without a usable CUDA device AFC_Calculate fails.
 *   - Where the reference panics (unknown tag, bad axis combination, no GPU), these functions
 *     return without effect (AFC_Calculate returns 0 and sets *out to NULL) and record a
 *     message that AFC_GetLastError() returns.
 *   - Extra exports, marked NEW below, have no counterpart in the reference ABI.
 */
#ifndef AFCCAPI_H
#define AFCCAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* nalgebra Vector3<f32>, passed by value (core/mod.rs:109-110). */
typedef struct AfcVector3 {
    float x, y, z;
} AfcVector3;

/* SphereWaveSource, repr(C) (core/wave_sources/sphere_sources.rs:22-27). */
typedef struct AfcSphereWaveSource {
    float x, y, z;
    float amp, phase, freq;
} AfcSphereWaveSource;

/* T4010A1, repr(C) (core/wave_sources/t4010a1.rs:76-82). */
typedef struct AfcT4010A1 {
    float x, y, z;
    float nx, ny, nz;
    float amp, phase, freq;
} AfcT4010A1;

/* ---------------------------------------------------------------- calculators */

/* capi/src/calculator.rs:20-36 */
void AFC_CreateCalculator(void **out, int32_t calc_type);
/* capi/src/calculator.rs:38-50 */
void AFC_FreeCalculator(void *handle, int32_t calc_type);
/* capi/src/calculator.rs:52-117.  Computes the field of `system` on `area` into `field` and
 * returns the number of elements (points; for the complex field, complex values).  *out
 * receives a pointer into the field buffer, valid until the next calculation into that buffer
 * or its free. */
uint64_t AFC_Calculate(void *calc_handle, void *system_handle, void *obs_handle,
                       void *field_handle, const void **out, int32_t calc_type,
                       int32_t source_type, int32_t obs_type, int32_t field_type);

/* ---------------------------------------------------------------- systems */

/* capi/src/system.rs:21-41 */
void AFC_CreateUniformSystem(void **out, float temperature, int32_t source_type);
/* capi/src/system.rs:43-55 */
void AFC_FreeUniformSystem(void *handle, int32_t source_type);
/* capi/src/system.rs:57-72: sound speed [mm/s] of the system's temperature */
float AFC_UniformSystemSoundSpeed(void *handle, int32_t source_type);
/* capi/src/system.rs:74-92.  The string is owned by the system handle and stays valid until
 * the next info call on it or its free (the reference leaks a CString instead). */
char *AFC_UniformSystemInfo(void *handle, int32_t source_type);
/* capi/src/system.rs:94-113 (same ownership as AFC_UniformSystemInfo) */
char *AFC_UniformSystemSourceInfo(void *handle, uint64_t source_idx, int32_t source_type);
/* capi/src/system.rs:115-121: k = 2 pi f / c(T), alpha = atmospheric attenuation at T */
void AFC_AddSphereWaveSource(void *handle, AfcSphereWaveSource source);
/* capi/src/system.rs:123-129 */
void AFC_AddT4010A1(void *handle, AfcT4010A1 source);
/* capi/src/system.rs:131-153: returns the source count and a MUTABLE pointer to the system's
 * source array; callers may rewrite amp/phase/pos through it, and every calculation reads the
 * array afresh. */
uint64_t AFC_GetWaveSources(void *handle, void **out, int32_t source_type);

/* NEW: add a source with an explicit wavenumber [rad/mm] and attenuation [Np/mm]; the Rust
 * API has this as UniformSystem::add_wave_source_with_wavenum_and_atten
 * (system/uniform_medium.rs:50-59), which the reference C ABI does not export. */
void AFC_AddSphereWaveSourceWithWavenumAtten(void *handle, AfcSphereWaveSource source,
                                            float wavenum, float atten);
void AFC_AddT4010A1WithWavenumAtten(void *handle, AfcT4010A1 source, float wavenum, float atten);

/* NEW, opt-in: skip the per-call source upload for callers that announce their edits.  The
 * reference's AFC_GetWaveSources hands out the source array for writing in place, so by default
 * every AFC_Calculate uploads and packs the system's sources again (capi/src/calculator.rs:
 * 52-117 reads them on every call).  With tracking on (enable != 0), a calculator reuses the
 * device copy it packed for this system in its previous calculation as long as the system's
 * sources have not changed since: changes made by this library (AFC_Add*, AFO_*, or a new
 * AFC_GetWaveSources pointer) are seen by themselves, while writes through a pointer obtained
 * earlier must be announced with AFC_UniformSystemSourcesChanged before the next calculation,
 * or that calculation uses the previous sources.  Turning tracking on or off also counts as
 * a change.  Returns 0, or a negative AFC_ERR_* code (afc_gpu.h) for an invalid handle or
 * tag. */
int32_t AFC_UniformSystemTrackSources(void *handle, int32_t source_type, int32_t enable);
/* NEW: announce that the system's sources were written through an AFC_GetWaveSources pointer
 * (needed only while tracking is on; harmless otherwise). */
int32_t AFC_UniformSystemSourcesChanged(void *handle, int32_t source_type);

/* ---------------------------------------------------------------- observation areas */

/* capi/src/observe_area.rs:20-27 */
void AFC_CreateScatterArea(void **out);
/* capi/src/observe_area.rs:29-35 */
void AFC_ScatterAddObservePoint(void *handle, AfcVector3 p);
/* capi/src/observe_area.rs:37-40 */
void AFC_FreeScatterArea(void *handle);
/* capi/src/observe_area.rs:42-84 */
void AFC_CreateGridArea1D(void **out, float first_start, float first_end, float second,
                          float third, float resolution, int32_t first_axis,
                          int32_t second_axis, int32_t third_axis);
/* capi/src/observe_area.rs:86-131 */
void AFC_CreateGridArea2D(void **out, float first_start, float first_end, float second_start,
                          float second_end, float third, float resolution, int32_t first_axis,
                          int32_t second_axis, int32_t third_axis);
/* capi/src/observe_area.rs:133-180 */
void AFC_CreateGridArea3D(void **out, float first_start, float first_end, float second_start,
                          float second_end, float third_start, float third_end,
                          float resolution, int32_t first_axis, int32_t second_axis,
                          int32_t third_axis);
/* capi/src/observe_area.rs:182-197: dimension is 1, 2 or 3 */
void AFC_FreeGridArea(void *handle, int32_t dimension);
/* capi/src/observe_area.rs:199-228: point counts along x, y, z (not specification order) */
void AFC_GetGridSize(void *handle, int32_t dimension, uint32_t *first, uint32_t *second,
                     uint32_t *third);

/* ---------------------------------------------------------------- field buffers */

/* capi/src/field_buffer.rs:19-49 */
void AFC_CreatePressureField(void **out);
void AFC_FreePressureField(void *handle);
void AFC_CreatePowerField(void **out);
void AFC_FreePowerField(void *handle);
void AFC_CreateComplexPressureField(void **out);
void AFC_FreeComplexPressureField(void *handle);

/* ---------------------------------------------------------------- optimizers */

/* capi/src/optimizer.rs:41-45: single-focus phases, focal_point.rs:27-40 */
void AFO_FocalPoint(void *handle, AfcVector3 point, int32_t source_type);
/* capi/src/optimizer.rs:79-95: GS-PAT (gs_pat.rs:35-81), computed on the GPU; writes amp and
 * phase of every source in place.  foci points to `size` AfcVector3. */
void AFO_GSPAT(void *handle, const void *foci, const float *amps, uint64_t size,
               int32_t source_type);
/* capi/src/optimizer.rs:97-109: Gerchberg-Saxton (gs.rs:33-78), on the GPU */
void AFO_GS(void *handle, const void *foci, const float *amps, uint64_t size,
            int32_t source_type);
/* capi/src/optimizer.rs:111-127: naive linear synthesis (naive.rs:29-51), on the GPU */
void AFO_Naive(void *handle, const void *foci, const float *amps, uint64_t size,
               int32_t source_type);

/* capi/src/optimizer.rs:47-58: Bessel beam phases (bessel.rs:30-51), host set-up */
void AFO_BesselBeam(void *handle, AfcVector3 point, AfcVector3 dir, float theta,
                    int32_t source_type);
/* capi/src/optimizer.rs:60-77: exported so that callers binding the whole reference ABI load
 * this library unchanged.  Its solver (fft/ifft.rs, an image file and an FFT) is outside this
 * library's scope: the call leaves the system unchanged and records an "unsupported" error for
 * AFC_GetLastError. */
void AFO_IFFT(void *handle, const char *path, AfcVector3 bottom_left, AfcVector3 top_left,
              AfcVector3 bottom_right, float spacing, float z, int32_t source_type);
/* capi/src/optimizer.rs:129-143: Horn (matrix/horn.rs), on the GPU; at most 256 foci.  Its
 * coordinate order comes from a fixed-seed generator (the reference's is unseeded). */
void AFO_Horn(void *handle, const void *foci, const float *amps, uint64_t size,
              int32_t source_type);
/* capi/src/optimizer.rs:145-159: Long (matrix/long.rs), on the GPU; at most 256 foci */
void AFO_Long(void *handle, const void *foci, const float *amps, uint64_t size,
              int32_t source_type);
/* capi/src/optimizer.rs:161-177: APO (nls/apo.rs), on the GPU */
void AFO_APO(void *handle, const void *foci, const float *amps, uint64_t size, float lambda,
             int32_t source_type);
/* capi/src/optimizer.rs:179-225: Gauss-Newton, gradient descent and Levenberg-Marquardt
 * (nls/{gauss_newton,gradient_descent,lm}.rs), on the GPU */
void AFO_GaussNewton(void *handle, const void *foci, const float *amps, uint64_t size,
                     int32_t source_type);
void AFO_GradientDescent(void *handle, const void *foci, const float *amps, uint64_t size,
                         int32_t source_type);
void AFO_LM(void *handle, const void *foci, const float *amps, uint64_t size,
            int32_t source_type);
/* capi/src/optimizer.rs:227-243: greedy phase choice (combination/greedy.rs), on the GPU */
void AFO_Greedy(void *handle, const void *foci, const float *amps, uint64_t size,
                uint64_t phase_div, int32_t source_type);

/* ---------------------------------------------------------------- errors (NEW) */

/* NEW: message of the last failed call on this thread ("" if none). */
const char *AFC_GetLastError(void);
/* NEW: clears the thread's last error. */
void AFC_ClearLastError(void);

#ifdef __cplusplus
}
#endif

#endif /* AFCCAPI_H */
