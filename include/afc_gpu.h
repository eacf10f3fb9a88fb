/*
 * afc_gpu.h -- device-pointer entry points of libafccapi.so (all NEW: the reference ABI has
 * no device-level calls).
 *
 * They run the same kernels as AFC_Calculate but take device buffers and a CUDA stream, so a
 * caller that keeps sources, points and results resident in GPU memory pays no host<->device
 * copies.  The work they replace is the reference's internal Vulkan dispatch
 * (acoustic-field-calculator/src/gpu/field_buffer/pressure_field.rs:48-255 and the shader
 * assets/shaders/cpressure_base.comp:43-71) and the CPU loop
 * (calculator/cpu_calculator.rs:43-56).
 *
 * Conventions: pointers named d_* are device pointers on the current CUDA device; `stream` is
 * a cudaStream_t (NULL = legacy default stream); calls are asynchronous with respect to the
 * host and return 0 on success or a negative AFC_ERR_* code (AFC_GetLastError has the text).
 * Source records use the AfcT4010A1 / AfcSphereWaveSource layouts of afccapi.h.
 */
#ifndef AFC_GPU_H
#define AFC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    AFC_OK = 0,
    AFC_ERR_INVALID = -1,   /* bad tag, size, pointer or alignment */
    AFC_ERR_CUDA = -2,      /* a CUDA call failed */
    AFC_ERR_NO_DEVICE = -3, /* no usable CUDA device */
    AFC_ERR_TOO_LARGE = -4, /* a size exceeds a documented maximum */
    AFC_ERR_UNSUPPORTED = -5
};

/* Accumulation of the per-point sum: plain FP32 in source order (the CPU / GPU calculators)
 * or compensated (the Accurate calculator). */
enum { AFC_SUM_PLAIN = 0, AFC_SUM_COMPENSATED = 1 };

/* A grid observation area.  Point p = i0 + count[0] * (i1 + count[1] * i2) lies at
 * origin[axis_k - 1] + (float)i_k * res along axis_k; the first specified axis varies fastest
 * (observe_area/grid/grid_area.rs:105-229). */
typedef struct AfcGridDesc {
    uint64_t count[3]; /* points along the 1st, 2nd, 3rd specified axis (1 for a fixed axis) */
    int32_t axis[3];   /* axis codes X = 1, Y = 2, Z = 3 in specification order */
    float origin[3];   /* x, y, z of point 0 */
    float res;         /* spacing [mm] */
} AfcGridDesc;

/* Describe a grid area handle (dimension 1, 2 or 3) for the device calls. */
int32_t AFC_GridDescFromArea(void *grid_handle, int32_t dimension, AfcGridDesc *out);

/* Bytes of device workspace the field calls need for n sources (16-byte aligned buffer); 0 for
 * n >= 2^40, which the field calls reject with AFC_ERR_TOO_LARGE.
 *
 * Besides that workspace, a field call on 32,768 points or more whose point tiles would leave
 * the GPU's last wave short (scatter sets and single-row grids of up to about half a million
 * points against thousands of sources) may take partial-sum scratch of a few bytes per point:
 * stream-ordered (cudaMallocFromPoolAsync, cudaFreeAsync on the call's stream) from a pool the
 * library keeps per device, which holds up to 256 MB between calls.  No scratch is taken while
 * the stream is being captured into a graph, by the compensated sum (sum_mode 1), by
 * AFC_FieldGridDeviceNoAlloc, or by the serving engine; those launches, and any call whose
 * scratch cannot be had, split the sources over thread-block clusters instead.  AFC_Calculate
 * behaves the same way. */
size_t AFC_FieldWorkspaceBytes(uint64_t n_sources);

/* Field of n sources on a grid.  d_out receives count[0]*count[1]*count[2] floats (pressure,
 * power) or float2 (complex). */
int32_t AFC_FieldGridDevice(int32_t source_type, int32_t field_type, int32_t sum_mode,
                            const float *d_sources, const float *d_wavenums,
                            const float *d_attens, uint64_t n, const AfcGridDesc *grid,
                            void *d_out, void *d_workspace, size_t workspace_bytes,
                            void *stream);

/* Field of n sources on m explicit points (3 floats each). */
int32_t AFC_FieldScatterDevice(int32_t source_type, int32_t field_type, int32_t sum_mode,
                               const float *d_sources, const float *d_wavenums,
                               const float *d_attens, uint64_t n, const float *d_points,
                               uint64_t m, void *d_out, void *d_workspace,
                               size_t workspace_bytes, void *stream);

/* ---- many phase patterns on one geometry (no counterpart in the reference: the reference
 * evaluates one pattern per AFC_Calculate) ----
 *
 * P (m points x K patterns, complex, row-major: P[i][k] at d_out[2 (i K + k)]) = G Q with
 * G_ij the field of source j at point i for unit amplitude and zero phase and
 * Q_jk = amps[k][j] exp(i phases[k][j]).  AFC_MultiPatternBuildG builds G once per geometry into
 * the workspace; AFC_MultiPatternApply evaluates any number of pattern sets against it on the
 * tensor cores.  Precision AFC_PRECISION_BF16X3: G and Q split into bf16 hi + lo parts,
 * hi*hi + hi*lo + lo*hi accumulated in FP32; AFC_PRECISION_FP16: one FP16 product with each
 * row of G scaled by a power of two. */
enum { AFC_PRECISION_BF16X3 = 1, AFC_PRECISION_FP16 = 2 };
/* Workspace bytes for BuildG / Apply; 0 for an unknown precision or a problem beyond the limits
 * (n, m < 2^31, patterns < 2^26, workspace < 2^62 bytes), which BuildG and Apply reject with
 * AFC_ERR_TOO_LARGE. */
size_t AFC_MultiPatternWorkspaceBytes(uint64_t n, uint64_t m, uint64_t patterns,
                                      int32_t precision);
int32_t AFC_MultiPatternBuildG(int32_t source_type, int32_t precision, const float *d_sources,
                               const float *d_wavenums, const float *d_attens, uint64_t n,
                               const float *d_points, uint64_t m, uint64_t patterns,
                               void *d_workspace, size_t workspace_bytes, void *stream);
int32_t AFC_MultiPatternApply(int32_t precision, const float *d_amps, const float *d_phases,
                              uint64_t n, uint64_t m, uint64_t patterns, float *d_out,
                              void *d_workspace, size_t workspace_bytes, void *stream);
/* 0 if the last AFC_MultiPatternApply in this workspace completed, else the code of the
 * tensor-core pipeline stage whose bounded wait (a second of the GPU's global timer) expired
 * first (1 loader, 2 MMA, 3 epilogue).  Synchronises the stream. */
int32_t AFC_MultiPatternStatus(int32_t precision, uint64_t n, uint64_t m, uint64_t patterns,
                               void *d_workspace, void *stream);
/* Testing the bounded waits: AFC_MultiPatternApply with the GEMM's loader arming no pipeline
 * stage, so that every wait of the kernel runs out and it returns through its error path (about
 * a second; the output is not computed).  AFC_MultiPatternStatus then reports a nonzero code,
 * and the workspace and context stay usable. */
int32_t AFC_MultiPatternApplyWaitTest(int32_t precision, const float *d_amps,
                                      const float *d_phases, uint64_t n, uint64_t m,
                                      uint64_t patterns, float *d_out, void *d_workspace,
                                      size_t workspace_bytes, void *stream);
/* The same P by FP32 direct summation, one field evaluation per pattern, written pattern-major
 * (P[i][k] at d_out[2 (k m + i)]); workspace of 2 * AFC_FieldWorkspaceBytes(n) bytes. */
int32_t AFC_MultiPatternDirect(int32_t source_type, const float *d_sources,
                               const float *d_wavenums, const float *d_attens, uint64_t n,
                               const float *d_points, uint64_t m, const float *d_amps,
                               const float *d_phases, uint64_t patterns, float *d_out,
                               void *d_workspace, size_t workspace_bytes, void *stream);

/* ---- many independent field jobs in one persistent launch (no counterpart in the
 * reference, which evaluates one AFC_Calculate at a time) ----
 *
 * A plan binds a list of jobs -- each one field evaluation of its own sources on its own grid
 * or points into its own output -- to a CUDA graph that packs every job's sources and runs two
 * persistent kernels over the (job, point tile) work items, longest first: one for the grid
 * jobs that take the rows tiling, one for the others.  The caller may rewrite the contents of
 * the source arrays between runs; the pointers and sizes are fixed at creation.  `tune` != 0
 * times, on the batch itself, each kernel's point tile (1, 2, 4 point pairs per thread) and
 * resident blocks per SM, and the plan with every grid job on the general kernel, and keeps
 * the fastest.  All jobs of a plan have the same source type. */
typedef struct AfcFieldJob {
    uint64_t n_sources;
    const float *d_sources; /* ABI records (AfcT4010A1 / AfcSphereWaveSource) */
    const float *d_wavenums;
    const float *d_attens;
    int32_t field_type; /* 0 pressure, 1 power, 2 complex */
    int32_t is_grid;    /* 1: `grid` gives the points; 0: d_points / n_points */
    AfcGridDesc grid;
    const float *d_points;
    uint64_t n_points;
    void *d_out;
} AfcFieldJob;

int32_t AFC_BatchCreate(int32_t source_type, const AfcFieldJob *jobs, uint64_t n_jobs,
                        int32_t tune, void **plan, void *stream);
/* Replays the plan's graph on `stream` (asynchronous). */
int32_t AFC_BatchRun(void *plan, void *stream);
/* The same jobs launched one at a time (pack + field kernel per job), for comparison. */
int32_t AFC_BatchRunOneByOne(void *plan, void *stream);
/* The general kernel's point pairs per thread and resident CTAs per SM, the work items of
 * both kernels, total evaluations. */
int32_t AFC_BatchDescribe(void *plan, int32_t *pairs, int32_t *blocks_per_sm, uint64_t *items,
                          double *evals);
/* Each kernel's point pairs per thread, resident CTAs per SM and work items (rows kernel: grid
 * jobs on the rows tiling; flat kernel: the others).  Any pointer may be NULL. */
int32_t AFC_BatchDescribeKernels(void *plan, int32_t *rows_pairs, int32_t *rows_blocks_per_sm,
                                 uint64_t *rows_items, int32_t *flat_pairs,
                                 int32_t *flat_blocks_per_sm, uint64_t *flat_items);
void AFC_BatchFree(void *plan);

/* ---- serving engine (no counterpart in the reference, whose calls block) ----
 *
 * Field-evaluation and GS-PAT hologram requests on resident geometries, admitted in arrival
 * order under a fixed HBM budget (a device arena of hbm_budget_bytes) and at most
 * max_inflight at a time, each on its own stream so that admitted requests overlap on the GPU
 * while later ones keep arriving.  Inputs are copied at submission (into a pinned host arena of
 * pinned_bytes; submission waits while it is full); results land in the caller's buffers before
 * AFC_ServeWait returns.  Latency is measured from submission until the request's last
 * device operation (the copy of its result to host memory) has completed. */
typedef struct AfcServeConfig {
    uint64_t hbm_budget_bytes;
    uint64_t pinned_bytes;
    int32_t max_inflight;
} AfcServeConfig;

typedef struct AfcServeStats {
    uint64_t completed;
    uint64_t failed;
    uint64_t queued;
    uint64_t peak_hbm_bytes;
    uint64_t hbm_budget_bytes;
    int32_t peak_inflight;
} AfcServeStats;

int32_t AFC_ServeCreate(const AfcServeConfig *config, void **engine);
/* Register sources (ABI records, wavenumbers, attenuations): packed once, resident. */
int32_t AFC_ServeAddGeometry(void *engine, int32_t source_type, const float *h_sources,
                             const float *h_wavenums, const float *h_attens, uint64_t n,
                             int32_t *geometry_id);
/* Field of the geometry with these amplitudes and phases on a grid (is_grid) or on n_points
 * explicit points; h_out receives floats (pressure, power) or float pairs (complex).
 * Returns the request id (> 0) or a negative AFC_ERR_* code. */
int64_t AFC_ServeSubmitField(void *engine, int32_t geometry, const float *h_amps,
                             const float *h_phases, int32_t field_type, int32_t is_grid,
                             const AfcGridDesc *grid, const float *h_points, uint64_t n_points,
                             float *h_out);
/* GS-PAT on the geometry (amplitudes as registered) for n_foci foci, then the pressure of
 * the solved drive on `slice`; h_amp_phase_out (optional) receives the drive (amp, phase). */
int64_t AFC_ServeSubmitGspat(void *engine, int32_t geometry, const float *h_foci,
                             const float *h_amps, uint64_t n_foci, const AfcGridDesc *slice,
                             float *h_slice_out, float *h_amp_phase_out);
/* Blocks until the request has finished; its latency and time spent queued [s].  Call it
 * exactly once per request (from any one thread): it releases the request's record. */
int32_t AFC_ServeWait(void *engine, int64_t request, double *latency_s, double *queue_s);
int32_t AFC_ServeStats(void *engine, AfcServeStats *stats);
/* Finishes queued and running requests, then frees the engine. */
void AFC_ServeDestroy(void *engine);

/* Measure, on the current device, with dependency-free microbenchmarks, the result rates
 * [operations/s] of rates[0..4] = MUFU ex2, rsqrt, sqrt, sin, cos and rates[5] = FP32 FMA,
 * the SM clock [Hz] while they run, and the SM count.  These are the denominators of the
 * direct summation's roofline. */
int32_t AFC_MeasurePipeRates(double rates[6], double *sm_clock_hz, int32_t *sm_count);

/* Select the device that calculators and solvers created afterwards on this thread use (the
 * reference's Vulkan calculator always takes the first device, gpu/gpu_calculator.rs:34-37;
 * the default here is also device 0).  The device-level calls follow their stream's device;
 * every call that launches on a device other than the thread's current one switches to it for
 * the call and back before returning, so no call changes the caller's current device. */
int32_t AFC_SetDevice(int32_t device);

/* Number of CUDA devices visible to this library (0 when none or the driver is unusable). */
int32_t AFC_CudaDeviceCount(void);

/* Allocation-free AFC_FieldGridDevice.  This entry point has no counterpart in the reference.
 *
 * For callers that cannot allocate GPU memory while they run: a real-time loop driving a
 * transducer array that must not block on the allocator or fail on memory mid-run, a host
 * that has handed the device's memory to its own pool, a plugin whose host forbids
 * allocation inside callbacks.  Instead of a caller-supplied workspace it uses a fixed
 * scratch array of AFC_NOALLOC_MAX_SOURCES packed sources (768 KiB) that the library
 * reserves on every GPU it is loaded on, for the life of the process; inputs and output are
 * the caller's, as for AFC_FieldGridDevice.  More sources than AFC_NOALLOC_MAX_SOURCES are
 * rejected with AFC_ERR_TOO_LARGE.  The first call on each device looks the scratch address
 * up (make it before capturing the stream into a graph) and keeps it for the life of the
 * process: use streams of the device's primary context and do not reset the device after that
 * first call.  All calls share the one scratch array, so calls whose GPU work overlaps
 * (unordered streams) race; order them on one stream.  It calls no allocator. */
#define AFC_NOALLOC_MAX_SOURCES 16384
int32_t AFC_FieldGridDeviceNoAlloc(int32_t source_type, int32_t field_type, int32_t sum_mode,
                                   const float *d_sources, const float *d_wavenums,
                                   const float *d_attens, uint64_t n, const AfcGridDesc *grid,
                                   void *d_out, void *stream);

/* Number of kernels this library has launched since it was loaded. */
uint64_t AFC_KernelLaunchCount(void);

#ifdef __cplusplus
}
#endif

#endif /* AFC_GPU_H */
