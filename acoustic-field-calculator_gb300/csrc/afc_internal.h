// Internal declarations shared by the CUDA kernels (.cu) and the C-ABI host layer (capi.cpp).
// Nothing here is part of the public ABI; the public declarations live in include/*.h.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>

namespace afc {

// Tags of the reference C ABI (capi/src/type_inference_aux.rs:53-103).
enum SourceType : int { SRC_SPHERE = 0, SRC_T4010A1 = 1 };
enum FieldType : int { FIELD_PRESSURE = 0, FIELD_POWER = 1, FIELD_COMPLEX = 2 };
enum CalcType : int { CALC_CPU = 0, CALC_ACCURATE = 1, CALC_GPU = 2 };
enum AreaType : int { AREA_GRID1D = 0, AREA_GRID2D = 1, AREA_GRID3D = 2, AREA_SCATTER = 3 };
// How the per-point sum over sources is accumulated.
enum SumMode : int { SUM_PLAIN = 0, SUM_COMPENSATED = 1 };

// Floats per source record in the reference ABI layout.
inline int source_stride(int st) { return st == SRC_T4010A1 ? 9 : 6; }

// One source as the field kernels read it (48 bytes, 16-byte aligned):
//   a = (x, y, z, k)              position [mm], wavenumber [rad/mm]
//   b = (nx, ny, nz, -alpha*log2e) direction, attenuation as a base-2 exponent per mm
//   c = (log2|amp|, phase', amp, phase)
// The kernels fold the amplitude into the attenuation exponent: A exp(-alpha r) =
// 2^(log2|A| - alpha log2e r), with the sign of A carried as phase' = phase + pi for A < 0.
struct __align__(16) PackedSource {
    float4 a, b, c;
};

// A grid area: the point with index p = i0 + c0 * (i1 + c1 * i2) (first specified axis fastest,
// observe_area/grid/grid_area.rs:105-229) has coordinate origin[ax_k] + (float)i_k * res along
// axis ax_k, computed with one f32 multiply and one f32 add as the reference does.
struct GridDev {
    int64_t count[3];  // points along the 1st/2nd/3rd specified axis (1 for a fixed axis)
    int axis[3];       // 0 = x, 1 = y, 2 = z, in specification order
    float origin[3];   // x, y, z
    float res;
};

// A set of observation points: a grid generated on the fly or explicit xyz triples.
struct PointSet {
    bool is_grid;
    GridDev grid;
    const float* pts;  // device, 3 floats per point (scatter)
    int64_t m;
};

cudaError_t launch_pack_sources(int st, const float* raw, const float* k, const float* atten,
                                int64_t n, PackedSource* out, cudaStream_t s);

// The field of n packed sources at ps into out on stream s.  scratch_ok: a launch whose point
// tiles would leave the last wave short may allocate partial sums (stream-ordered, from a
// per-device pool) and cut the sources into chunks; otherwise it splits them over clusters.
cudaError_t launch_field(int st, int field, int sum_mode, const PackedSource* src, int64_t n,
                         const PointSet& ps, void* out, cudaStream_t s, bool scratch_ok = true);

// The rows tiling of a grid for `pairs` point pairs per thread (blocks of 1 << tx_log2
// first-axis indices by (256 >> tx_log2) * 2 * pairs second-axis indices, one plane each), and
// whether to use it: grids with more than one point along their second axis whose tiles keep at
// least 90 % as many threads busy as the flat numbering.
struct RowsTiling {
    bool use;
    int tx_log2;
    int64_t rows;  // second-axis indices per tile
    int64_t tiles0, tiles1, blocks;
};
RowsTiling rows_tiling(const GridDev& g, int64_t m, int pairs);

// Packed sources of a request: geometry from `geom`, amplitude and phase from `amps` and
// `phases` or, when `amp_phase` is not NULL, from its interleaved (amp, phase) pairs.
cudaError_t launch_repack(const PackedSource* geom, const float* amps, const float* phases,
                          const float* amp_phase, int64_t n, PackedSource* out, cudaStream_t s);

// Streaming multiprocessors of the current device (cached per device after the first query).
int num_sms();

// Switches the calling thread's current device for the guard's lifetime and switches it back
// when the guard goes out of scope, so that an entry point that has to launch on its stream's
// (or handle's) device leaves the caller's current device as it found it.
class DeviceGuard {
   public:
    DeviceGuard() = default;
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
    // Make `dev` current; no call when it already is.
    cudaError_t set(int dev) {
        int cur = -1;
        cudaError_t e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return e;
        if (cur == dev) return cudaSuccess;
        if (!switched_) prev_ = cur;
        e = cudaSetDevice(dev);
        if (e == cudaSuccess) switched_ = true;
        return e;
    }
    ~DeviceGuard() {
        if (switched_) cudaSetDevice(prev_);
    }

   private:
    int prev_ = -1;
    bool switched_ = false;
};

// The device whose work `s` orders (the current device for the default stream, NULL).  While
// `s` is being captured into a graph cudaStreamGetDevice is refused (in the global and thread-
// local capture modes), so the current device is taken: a capture records work of the current
// device's context.
inline cudaError_t stream_device(cudaStream_t s, int* dev) {
    if (!s) return cudaGetDevice(dev);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return cudaGetDevice(dev);
    return cudaStreamGetDevice(s, dev);
}

// Whether `s` is being captured into a graph (captured work takes neither the chunked field
// launch's stream-ordered scratch nor programmatic dependences).  A failed query counts as a
// capture.
inline bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cst) != cudaSuccess) {
        (void)cudaGetLastError();
        return true;
    }
    return cst != cudaStreamCaptureStatusNone;
}

// Launches `kernel` on s, with `pdl` as a programmatic dependent of the launch before it (the
// kernel calls pdl_wait before touching that launch's data).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_after(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t dyn,
                                cudaStream_t s, bool pdl, Args... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = s;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Record `msg` as this thread's last error (read back by AFC_GetLastError).
void set_error_message(const char* msg);

// Kernels launched by this library since load (the bench reports the delta).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// Bytes written per point for a field type.
inline size_t field_elem_bytes(int field) { return field == FIELD_COMPLEX ? 8 : 4; }

}  // namespace afc
