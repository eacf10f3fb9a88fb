// Many independent field jobs of uneven size in one persistent launch, replayed from a CUDA
// graph.  No reference counterpart: the reference evaluates one AFC_Calculate at a time
// (calculator/cpu_calculator.rs:43-56); every job here computes exactly that field with the
// same per-block bodies as the single-job kernels (field_body.cuh, field_rows.cuh).
//
// Plan (AFC_BatchCreate):
//   * job table on the device: each job's source records, packed-arena offset, points (grid
//     description or explicit points), field type and output pointer;
//   * work items = (job, block of 2*PAIRS*256 points, or one tile of the rows tiling for the
//     grids the single-job launch tiles by rows), sorted by cost (sources x points) descending
//     so that the longest items start first and the short ones fill the tail;
//   * the autotuner (optional) runs the whole batch once per candidate point tile
//     (PAIRS = 1, 2, 4 point pairs per thread) and keeps the fastest;
//   * a CUDA graph is captured once: reset the work counter, pack every job's sources
//     (one block per job, re-reading the caller's source arrays so that edits between runs
//     are picked up), then the persistent kernel: (occupancy x SMs) CTAs that take items from
//     an atomic counter until none are left.
// AFC_BatchRun replays the graph; AFC_BatchRunOneByOne launches pack + field kernel per job on
// the stream (the comparison point).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <new>
#include <vector>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "field_body.cuh"
#include "field_rows.cuh"

namespace afc {
namespace batch {

using namespace fb;

__constant__ float4 c_dir_table_b[kDirTableSize] = AFC_DIR_TABLE_INIT;

struct JobDev {
    const float* raw;
    const float* k;
    const float* atten;
    int64_t n;
    int64_t src_off;  // first PackedSource of the job in the arena
    GridDev g;
    const float* pts;
    int64_t m;
    void* out;
    int field;
    int is_grid;
};

struct Item {
    int32_t job;
    int32_t block;  // flat block, or tile of the job's rows tiling
};

// How a job's points are split for the plan's point tile (rows_tiling).
struct JobTile {
    int32_t rows;  // 1: tiles of the rows tiling
    int32_t tx_log2;
    int64_t tiles0, tiles1;
};

__global__ void pack_all_kernel(int st, const JobDev* __restrict__ jobs,
                                PackedSource* __restrict__ arena) {
    const JobDev& J = jobs[blockIdx.x];
    for (int64_t j = threadIdx.x; j < J.n; j += blockDim.x)
        arena[J.src_off + j] = pack_source(st, J.raw, J.k, J.atten, j);
}

template <int ST, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    batch_kernel(const JobDev* __restrict__ jobs, const JobTile* __restrict__ tiles,
                 const Item* __restrict__ items, int64_t n_items,
                 unsigned long long* __restrict__ counter, const PackedSource* __restrict__ arena) {
    __shared__ SmemTile sm;
    __shared__ long long s_item;
    load_dir_tables(sm, c_dir_table_b);
    for (;;) {
        __syncthreads();  // the previous item's readers of sm and s_item are done
        if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(counter, 1ull));
        __syncthreads();
        const long long it = s_item;
        if (it >= n_items) break;
        const Item w = items[it];
        const JobDev J = jobs[w.job];
        const JobTile T = tiles[w.job];
        if (T.rows) {
            block_rows<ST, SUM_PLAIN, PAIRS>(sm, arena + J.src_off, J.n, J.g, T.tx_log2, T.tiles0,
                                             T.tiles1, w.block, J.field, J.out);
        } else {
            const int64_t first = static_cast<int64_t>(w.block) * (kThreads * 2 * PAIRS);
            block_points<ST, SUM_PLAIN, PAIRS>(sm, arena + J.src_off, J.n, J.is_grid != 0, J.g,
                                               J.pts, J.m, first, J.field, J.out);
        }
    }
}

struct Plan {
    int st = 1;
    int device = 0;
    int pairs = 4;
    int blocks_per_sm = 2;
    int64_t n_jobs = 0;
    int64_t total_sources = 0;
    double evals = 0;
    std::vector<JobDev> jobs;  // host copy
    JobDev* d_jobs = nullptr;
    JobTile* d_tiles = nullptr;  // per job, for the current point tile
    Item* d_items = nullptr;
    int64_t n_items = 0;
    unsigned long long* d_counter = nullptr;
    PackedSource* d_arena = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
};

template <int ST, int PAIRS>
cudaError_t launch_persistent(const Plan& p, int grid, cudaStream_t s) {
    batch_kernel<ST, PAIRS><<<grid, kThreads, 0, s>>>(p.d_jobs, p.d_tiles, p.d_items, p.n_items,
                                                       p.d_counter, p.d_arena);
    return cudaGetLastError();
}

template <int ST, int PAIRS>
int occupancy() {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batch_kernel<ST, PAIRS>, kThreads, 0) !=
            cudaSuccess ||
        b < 1)
        b = 1;
    return b;
}

int blocks_per_sm(int st, int pairs) {
    if (st == SRC_T4010A1)
        return pairs == 1 ? occupancy<SRC_T4010A1, 1>() : pairs == 2 ? occupancy<SRC_T4010A1, 2>() : occupancy<SRC_T4010A1, 4>();
    return pairs == 1 ? occupancy<SRC_SPHERE, 1>() : pairs == 2 ? occupancy<SRC_SPHERE, 2>() : occupancy<SRC_SPHERE, 4>();
}

cudaError_t launch_batch_kernel(const Plan& p, cudaStream_t s) {
    const int grid = num_sms() * p.blocks_per_sm;
    if (p.st == SRC_T4010A1) {
        if (p.pairs == 1) return launch_persistent<SRC_T4010A1, 1>(p, grid, s);
        if (p.pairs == 2) return launch_persistent<SRC_T4010A1, 2>(p, grid, s);
        return launch_persistent<SRC_T4010A1, 4>(p, grid, s);
    }
    if (p.pairs == 1) return launch_persistent<SRC_SPHERE, 1>(p, grid, s);
    if (p.pairs == 2) return launch_persistent<SRC_SPHERE, 2>(p, grid, s);
    return launch_persistent<SRC_SPHERE, 4>(p, grid, s);
}

// Items for the current point tile (2*pairs*256 points per block, or rows tiles for the
// grids the single-job launch tiles by rows), longest first.
cudaError_t build_items(Plan& p) {
    const int64_t per_block = static_cast<int64_t>(kThreads) * 2 * p.pairs;
    std::vector<std::pair<double, Item>> v;
    std::vector<JobTile> tiles(static_cast<size_t>(p.n_jobs));
    for (int64_t j = 0; j < p.n_jobs; ++j) {
        const JobDev& J = p.jobs[j];
        const double nsrc = static_cast<double>(J.n > 0 ? J.n : 1);
        const RowsTiling t = J.is_grid ? rows_tiling(J.g, J.m, p.pairs) : RowsTiling{};
        if (t.use) {
            if (t.blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
            tiles[j] = JobTile{1, t.tx_log2, t.tiles0, t.tiles1};
            const int64_t tx = 1LL << t.tx_log2;
            for (int64_t b = 0; b < t.blocks; ++b) {
                const int64_t t0 = b % t.tiles0, t1 = (b / t.tiles0) % t.tiles1;
                const int64_t pts = std::min(tx, J.g.count[0] - t0 * tx) *
                                    std::min(t.rows, J.g.count[1] - t1 * t.rows);
                v.push_back({static_cast<double>(pts) * nsrc,
                             Item{static_cast<int32_t>(j), static_cast<int32_t>(b)}});
            }
            continue;
        }
        tiles[j] = JobTile{0, 0, 0, 0};
        const int64_t blocks = (J.m + per_block - 1) / per_block;
        for (int64_t b = 0; b < blocks; ++b) {
            const int64_t pts = std::min(per_block, J.m - b * per_block);
            v.push_back({static_cast<double>(pts) * nsrc,
                         Item{static_cast<int32_t>(j), static_cast<int32_t>(b)}});
        }
    }
    if (p.n_jobs > 0) {
        if (!p.d_tiles) {
            const cudaError_t e = cudaMalloc(&p.d_tiles, sizeof(JobTile) * tiles.size());
            if (e != cudaSuccess) return e;
        }
        const cudaError_t e = cudaMemcpy(p.d_tiles, tiles.data(), sizeof(JobTile) * tiles.size(),
                                         cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    std::stable_sort(v.begin(), v.end(),
                     [](const std::pair<double, Item>& a, const std::pair<double, Item>& b) {
                         return a.first > b.first;
                     });
    std::vector<Item> items(v.size());
    for (size_t i = 0; i < v.size(); ++i) items[i] = v[i].second;
    if (p.d_items) cudaFree(p.d_items);
    p.d_items = nullptr;
    p.n_items = static_cast<int64_t>(items.size());
    if (items.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p.d_items, sizeof(Item) * items.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpy(p.d_items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice);
}

// The graph body: reset the counter, pack all sources, run the persistent kernel.
cudaError_t enqueue_batch(const Plan& p, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(p.d_counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (p.n_jobs > 0 && p.total_sources > 0) {
        pack_all_kernel<<<static_cast<unsigned>(p.n_jobs), 256, 0, s>>>(p.st, p.d_jobs, p.d_arena);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (p.n_items > 0) return launch_batch_kernel(p, s);
    return cudaSuccess;
}

cudaError_t capture(Plan& p) {
    if (p.exec) cudaGraphExecDestroy(p.exec);
    p.exec = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p.cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    e = enqueue_batch(p, p.cap);
    cudaError_t e2 = cudaStreamEndCapture(p.cap, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p.exec, g, 0);
    if (g) cudaGraphDestroy(g);
    return e;
}

void destroy(Plan* p) {
    if (!p) return;
    DeviceGuard dg;  // the plan's device while freeing; the caller's again on return
    dg.set(p->device);
    if (p->cap) cudaStreamSynchronize(p->cap);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->d_jobs) cudaFree(p->d_jobs);
    if (p->d_tiles) cudaFree(p->d_tiles);
    if (p->d_items) cudaFree(p->d_items);
    if (p->d_counter) cudaFree(p->d_counter);
    if (p->d_arena) cudaFree(p->d_arena);
    if (p->cap) cudaStreamDestroy(p->cap);
    delete p;
}

int32_t fail(int32_t code, const char* msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", msg, cudaGetErrorString(e));
        set_error_message(buf);
    } else {
        set_error_message(msg);
    }
    return code;
}

}  // namespace batch
}  // namespace afc

using namespace afc;
using namespace afc::batch;

extern "C" int32_t AFC_BatchCreate(int32_t source_type, const AfcFieldJob* jobs, uint64_t n_jobs,
                                   int32_t tune, void** plan_out, void* stream) {
    if (!plan_out) return fail(AFC_ERR_INVALID, "AFC_BatchCreate: plan_out is NULL");
    *plan_out = nullptr;
    if (source_type != SRC_SPHERE && source_type != SRC_T4010A1)
        return fail(AFC_ERR_INVALID, "AFC_BatchCreate: unknown source type");
    if (n_jobs > 0 && !jobs) return fail(AFC_ERR_INVALID, "AFC_BatchCreate: jobs is NULL");
    if (n_jobs > 0x7fffffffULL) return fail(AFC_ERR_TOO_LARGE, "AFC_BatchCreate: too many jobs");
    Plan* p = new (std::nothrow) Plan;
    if (!p) return fail(AFC_ERR_INVALID, "AFC_BatchCreate: out of host memory");
    p->st = source_type;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;  // the plan's device while it is built; the caller's again on return
    cudaError_t e = stream_device(s, &p->device);
    if (e == cudaSuccess) e = dg.set(p->device);
    if (e != cudaSuccess) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: stream device", e);
    }
    p->n_jobs = static_cast<int64_t>(n_jobs);
    p->jobs.resize(n_jobs);
    int64_t off = 0;
    for (uint64_t i = 0; i < n_jobs; ++i) {
        const AfcFieldJob& in = jobs[i];
        JobDev& J = p->jobs[i];
        if (in.n_sources >= (1ull << 40) || (!in.is_grid && in.n_points >= (1ull << 62))) {
            destroy(p);
            return fail(AFC_ERR_TOO_LARGE, "AFC_BatchCreate: a job has too many sources or points");
        }
        J.raw = in.d_sources;
        J.k = in.d_wavenums;
        J.atten = in.d_attens;
        J.n = static_cast<int64_t>(in.n_sources);
        J.src_off = off;
        off += J.n;
        if (off >= (1LL << 40)) {  // the packed-source arena holds 48 bytes per source
            destroy(p);
            return fail(AFC_ERR_TOO_LARGE, "AFC_BatchCreate: too many sources over all jobs");
        }
        J.field = in.field_type;
        J.is_grid = in.is_grid;
        J.out = in.d_out;
        J.pts = in.d_points;
        if (J.field < FIELD_PRESSURE || J.field > FIELD_COMPLEX || !J.out ||
            (J.n > 0 && (!J.raw || !J.k || !J.atten))) {
            destroy(p);
            return fail(AFC_ERR_INVALID, "AFC_BatchCreate: invalid job (field type or pointer)");
        }
        if (in.is_grid) {
            bool seen[3] = {false, false, false};
            for (int k = 0; k < 3; ++k) {
                const int a = in.grid.axis[k] - 1;
                if (a < 0 || a > 2 || seen[a] || in.grid.count[k] == 0) {
                    destroy(p);
                    return fail(AFC_ERR_INVALID, "AFC_BatchCreate: invalid grid description");
                }
                seen[a] = true;
                J.g.axis[k] = a;
                J.g.count[k] = static_cast<int64_t>(in.grid.count[k]);
                J.g.origin[k] = in.grid.origin[k];
            }
            J.g.res = in.grid.res;
            unsigned __int128 total = 1;  // checked after each factor: it must not wrap
            for (int k = 0; k < 3; ++k) {
                total *= in.grid.count[k];
                if (total > (static_cast<unsigned __int128>(1) << 62)) {
                    destroy(p);
                    return fail(AFC_ERR_TOO_LARGE,
                                "AFC_BatchCreate: a grid job has too many points");
                }
            }
            J.m = static_cast<int64_t>(total);
        } else {
            J.g = GridDev{};
            J.g.count[0] = J.g.count[1] = J.g.count[2] = 1;
            J.m = static_cast<int64_t>(in.n_points);
            if (J.m > 0 && !J.pts) {
                destroy(p);
                return fail(AFC_ERR_INVALID, "AFC_BatchCreate: scatter job without points");
            }
        }
        const int64_t max_blocks = (J.m + kThreads * 2 - 1) / (kThreads * 2);
        if (max_blocks > 0x7fffffffLL) {
            destroy(p);
            return fail(AFC_ERR_TOO_LARGE, "AFC_BatchCreate: a job has too many points");
        }
        p->evals += static_cast<double>(J.n) * static_cast<double>(J.m);
    }
    p->total_sources = off;
    if ((e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking)) != cudaSuccess) {
        p->cap = nullptr;
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: stream", e);
    }
    if ((e = cudaMalloc(&p->d_counter, sizeof(unsigned long long))) != cudaSuccess ||
        (n_jobs && (e = cudaMalloc(&p->d_jobs, sizeof(JobDev) * n_jobs)) != cudaSuccess) ||
        (off && (e = cudaMalloc(&p->d_arena, sizeof(PackedSource) * off)) != cudaSuccess)) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: device memory", e);
    }
    if (n_jobs && (e = cudaMemcpy(p->d_jobs, p->jobs.data(), sizeof(JobDev) * n_jobs,
                                  cudaMemcpyHostToDevice)) != cudaSuccess) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: job table", e);
    }
    // autotune the point tile on the batch itself
    int best = 4;
    if (tune) {
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int cand : {1, 2, 4}) {
            p->pairs = cand;
            p->blocks_per_sm = blocks_per_sm(p->st, cand);
            if ((e = build_items(*p)) != cudaSuccess) break;
            float ms = 0.f;
            for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // first run warms up
                cudaEventRecord(e0, p->cap);
                e = enqueue_batch(*p, p->cap);
                cudaEventRecord(e1, p->cap);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
            }
            count_launch(4);
            if (e != cudaSuccess) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e != cudaSuccess) {
            destroy(p);
            return fail(AFC_ERR_CUDA, "AFC_BatchCreate: autotuning", e);
        }
    }
    p->pairs = best;
    p->blocks_per_sm = blocks_per_sm(p->st, best);
    if ((e = build_items(*p)) != cudaSuccess || (e = capture(*p)) != cudaSuccess) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: work items / graph capture", e);
    }
    *plan_out = p;
    return AFC_OK;
}

extern "C" int32_t AFC_BatchRun(void* plan, void* stream) {
    Plan* p = static_cast<Plan*>(plan);
    if (!p || !p->exec) return fail(AFC_ERR_INVALID, "AFC_BatchRun: invalid plan");
    cudaError_t e = cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream));
    count_launch(p->n_items > 0 ? 2 : 1);
    if (e != cudaSuccess) return fail(AFC_ERR_CUDA, "AFC_BatchRun", e);
    return AFC_OK;
}

extern "C" int32_t AFC_BatchRunOneByOne(void* plan, void* stream) {
    Plan* p = static_cast<Plan*>(plan);
    if (!p) return fail(AFC_ERR_INVALID, "AFC_BatchRunOneByOne: invalid plan");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceGuard dg;  // the plan's device while launching; the caller's again on return
    const cudaError_t de = dg.set(p->device);
    if (de != cudaSuccess) return fail(AFC_ERR_CUDA, "AFC_BatchRunOneByOne: device", de);
    for (int64_t i = 0; i < p->n_jobs; ++i) {
        const JobDev& J = p->jobs[i];
        PackedSource* packed = p->d_arena + J.src_off;
        cudaError_t e = launch_pack_sources(p->st, J.raw, J.k, J.atten, J.n, packed, s);
        if (e == cudaSuccess) {
            PointSet ps{};
            ps.is_grid = J.is_grid != 0;
            ps.grid = J.g;
            ps.pts = J.pts;
            ps.m = J.m;
            e = launch_field(p->st, J.field, SUM_PLAIN, packed, J.n, ps, J.out, s);
        }
        if (e != cudaSuccess) return fail(AFC_ERR_CUDA, "AFC_BatchRunOneByOne", e);
    }
    return AFC_OK;
}

extern "C" int32_t AFC_BatchDescribe(void* plan, int32_t* pairs, int32_t* blocks_per_sm,
                                     uint64_t* items, double* evals) {
    Plan* p = static_cast<Plan*>(plan);
    if (!p) return fail(AFC_ERR_INVALID, "AFC_BatchDescribe: invalid plan");
    if (pairs) *pairs = p->pairs;
    if (blocks_per_sm) *blocks_per_sm = p->blocks_per_sm;
    if (items) *items = static_cast<uint64_t>(p->n_items);
    if (evals) *evals = p->evals;
    return AFC_OK;
}

extern "C" void AFC_BatchFree(void* plan) { destroy(static_cast<Plan*>(plan)); }
