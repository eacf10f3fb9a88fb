// Device work of the serving engine's request groups (serving_kernels.cu), shared with its host
// side (serving.cpp).  A group is a set of field requests of one source type that run as one set
// of persistent launches: every request is a job whose points are cut into tiles (the rows tiling
// for grids the single-job launch tiles by rows, blocks of kGroupTilePoints points otherwise) and
// whose sources are cut into `chunks` ranges; one work item is one (tile, chunk).  A job's cut
// depends on the job alone, so its field is the same whatever else runs in its group.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "afc_internal.h"

namespace afc {
namespace serve {

constexpr int kGroupPairs = 4;                            // point pairs per thread in a group
constexpr int64_t kGroupTilePoints = 256 * 2 * kGroupPairs;  // points of a flat tile
constexpr int64_t kMinChunkSources = 128;                 // sources of a chunk at least

struct GJob {
    const PackedSource* geom;  // resident geometry (amplitude and phase from the request)
    const float* amps;         // n amplitudes then n phases
    PackedSource* packed;      // the request's packed sources
    int64_t n;
    GridDev g;
    const float* pts;  // scatter points (device), or NULL for a grid
    int64_t m;
    void* out;
    float2* partial;  // chunks x m partial sums, chunk-major (chunks > 1)
    int32_t field;
    int32_t is_grid;
    int32_t chunks;
    int32_t rows;  // 1: tiles of the rows tiling
    int64_t chunk;  // sources per chunk (the last may be shorter)
    int32_t tx_log2;
    int32_t pad;
    int64_t tiles0, tiles1;
};

struct GItem {
    int32_t job;
    int32_t chunk;
    int64_t tile;
};

// Resident blocks per SM of the group's rows and flat kernels for source type st.
int group_rows_occupancy(int st);
int group_flat_occupancy(int st);

// One group on stream s: pack every job's sources, run the rows items on s and the flat items
// on s2 (forked and joined through the two events when both have work; the kernels take items
// from counters[0] and counters[1], which the launch resets), then add the chunked jobs'
// partial sums.  max_n: the most sources of a job; chunked: whether any job has chunks > 1.
cudaError_t launch_group(int st, const GJob* d_jobs, int n_jobs, int64_t max_n,
                         const GItem* d_rows, int64_t n_rows, const GItem* d_flat,
                         int64_t n_flat, unsigned long long* d_counters, bool chunked,
                         int rows_blocks, int flat_blocks, cudaStream_t s, cudaStream_t s2,
                         cudaEvent_t fork, cudaEvent_t join);

}  // namespace serve
}  // namespace afc
