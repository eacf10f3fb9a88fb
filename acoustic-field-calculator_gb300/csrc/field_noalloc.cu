// Allocation-free variant of AFC_FieldGridDevice.
//
// Who needs it: callers that must not allocate GPU memory at run time -- a real-time control
// loop driving a transducer array that may not block on the allocator or risk an
// out-of-memory failure mid-run, a host that has handed all device memory to its own pool,
// or a plugin whose host forbids allocation from inside a callback.  AFC_FieldGridDevice asks
// them for a workspace (the packed copy of the sources); this entry point instead uses a
// fixed scratch array that the library reserves when it is loaded.
//
// The scratch is a file-scope __device__ array of kNoAllocMaxSources packed sources
// (48 B each, 768 KiB in total); every GPU on which the library is loaded holds it until the
// process exits.  Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress (with that device
// current) and caches it; make that first call before capturing the stream into a graph.
// All calls share the one array: two calls whose work overlaps on the GPU (different streams,
// no ordering between them) race on it.  Every call rewrites the n entries it reads, so
// nothing has to be cleared between calls.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "afc_gpu.h"
#include "afc_internal.h"

namespace afc {
namespace {

constexpr uint64_t kNoAllocMaxSources = AFC_NOALLOC_MAX_SOURCES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) PackedSource g_noalloc_scratch[kNoAllocMaxSources];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on `dev` (looked up once per device, with it current).
cudaError_t scratch_on(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

// The message goes where AFC_GetLastError() reads it.
int32_t fail(int32_t code, const char* msg) {
    set_error_message(msg);
    return code;
}

}  // namespace
}  // namespace afc

extern "C" int32_t AFC_FieldGridDeviceNoAlloc(int32_t source_type, int32_t field_type,
                                              int32_t sum_mode, const float* d_sources,
                                              const float* d_wavenums, const float* d_attens,
                                              uint64_t n, const AfcGridDesc* grid, void* d_out,
                                              void* stream) {
    using namespace afc;
    if (n > kNoAllocMaxSources)
        return fail(AFC_ERR_TOO_LARGE,
                    "AFC_FieldGridDeviceNoAlloc: more sources than the 16384 its fixed scratch holds");
    if ((source_type != SRC_SPHERE && source_type != SRC_T4010A1) || field_type < FIELD_PRESSURE ||
        field_type > FIELD_COMPLEX || (sum_mode != AFC_SUM_PLAIN && sum_mode != AFC_SUM_COMPENSATED))
        return fail(AFC_ERR_INVALID, "AFC_FieldGridDeviceNoAlloc: invalid source/field/sum tag");
    if (!grid || !d_out || (n > 0 && (!d_sources || !d_wavenums || !d_attens)))
        return fail(AFC_ERR_INVALID, "AFC_FieldGridDeviceNoAlloc: NULL pointer");
    PointSet ps{};
    ps.is_grid = true;
    bool seen[3] = {false, false, false};
    for (int k = 0; k < 3; ++k) {
        const int a = grid->axis[k] - 1;
        if (a < 0 || a > 2 || seen[a] || grid->count[k] == 0)
            return fail(AFC_ERR_INVALID, "AFC_FieldGridDeviceNoAlloc: invalid grid description");
        seen[a] = true;
        ps.grid.axis[k] = a;
        ps.grid.count[k] = static_cast<int64_t>(grid->count[k]);
        ps.grid.origin[k] = grid->origin[k];
    }
    ps.grid.res = grid->res;
    // the point count must not wrap (counts that large would otherwise give a meaningless size)
    unsigned __int128 total = 1;
    for (int k = 0; k < 3; ++k) {
        total *= grid->count[k];
        if (total > (static_cast<unsigned __int128>(1) << 62))
            return fail(AFC_ERR_TOO_LARGE, "AFC_FieldGridDeviceNoAlloc: grid has too many points");
    }
    ps.m = static_cast<int64_t>(total);

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = -1;
    cudaError_t e = stream_device(s, &dev);
    if (e != cudaSuccess) return fail(AFC_ERR_CUDA, cudaGetErrorString(e));
    DeviceGuard dg;  // the stream's device while launching; the caller's again on return
    if ((e = dg.set(dev)) != cudaSuccess) return fail(AFC_ERR_CUDA, cudaGetErrorString(e));
    void* scratch = nullptr;
    if ((e = scratch_on(dev, &scratch)) != cudaSuccess)
        return fail(AFC_ERR_CUDA, cudaGetErrorString(e));
    PackedSource* packed = static_cast<PackedSource*>(scratch);
    if (n > 0) {
        e = launch_pack_sources(source_type, d_sources, d_wavenums, d_attens,
                                static_cast<int64_t>(n), packed, s);
        if (e != cudaSuccess) return fail(AFC_ERR_CUDA, cudaGetErrorString(e));
    }
    // no partial-sum scratch: this entry point allocates nothing
    e = launch_field(source_type, field_type, sum_mode, packed, static_cast<int64_t>(n), ps, d_out, s,
                     false);
    if (e != cudaSuccess) return fail(AFC_ERR_CUDA, cudaGetErrorString(e));
    return AFC_OK;
}
