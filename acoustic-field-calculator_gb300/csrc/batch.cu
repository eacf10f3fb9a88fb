// Many independent field jobs of uneven size in two persistent launches, replayed from a CUDA
// graph.  No reference counterpart: the reference evaluates one AFC_Calculate at a time
// (calculator/cpu_calculator.rs:43-56); every job here computes exactly that field with the
// same per-block bodies as the single-job kernels (field_body.cuh, field_rows.cuh).
//
// Plan (AFC_BatchCreate):
//   * job table on the device: each job's source records, packed-arena offset, points (grid
//     description or explicit points), field type and output pointer;
//   * two work lists, each sorted by cost (sources x points) descending so that the longest
//     items start first and the short ones fill the tail: tiles of the rows tiling for the grid
//     jobs the single-job launch tiles by rows (batch_rows_kernel, the rows body), and blocks
//     of 2*PAIRS*256 points for every other job (batch_flat_kernel, the general body).  One
//     kernel per body keeps each body's register allocation to itself (a single kernel holding
//     both ran at the register cap and spilled);
//   * the autotuner (optional) times the batch itself: the flat kernel's point pairs per thread
//     (1, 2, 4) and resident blocks per SM, then the rows kernel's, then the plan with every
//     grid job on the flat body, and keeps the fastest;
//   * a CUDA graph is captured once: reset both work counters, pack every job's sources (one
//     block per job, re-reading the caller's source arrays so that edits between runs are picked
//     up), then the two persistent kernels on forked streams (blocks per SM x SMs CTAs each,
//     taking items from their own atomic counter until none are left).  The second kernel's
//     blocks start as the first one's run out of work and exit, so the two overlap only at the
//     hand-over.
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

// How a grid job's points are tiled by the rows kernel.
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

// The next item of a persistent block (every thread gets it; n_items or more: none left).
__device__ __forceinline__ long long next_item(unsigned long long* counter, long long& s_item) {
    __syncthreads();  // the previous item's readers of shared memory and s_item are done
    if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(counter, 1ull));
    __syncthreads();
    return s_item;
}

template <int ST, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    batch_rows_kernel(const JobDev* __restrict__ jobs, const JobTile* __restrict__ tiles,
                      const Item* __restrict__ items, int64_t n_items,
                      unsigned long long* __restrict__ counter,
                      const PackedSource* __restrict__ arena) {
    __shared__ RowsSmem rs;
    __shared__ long long s_item;
    SmemTile& sm = rs.sm;
    RowsTable& rt = rs.rt;
    load_theta_table(sm, c_dir_table_b);
    load_rows_table(rt);
    for (;;) {
        const long long it = next_item(counter, s_item);
        if (it >= n_items) break;
        const Item w = items[it];
        const JobDev J = jobs[w.job];
        const JobTile T = tiles[w.job];
        block_rows<ST, SUM_PLAIN, PAIRS, true>(sm, rt, arena + J.src_off, J.n, J.g, T.tx_log2,
                                         T.tiles0, T.tiles1, w.block, J.field, J.out);
    }
}

template <int ST, int PAIRS>
__global__ void __launch_bounds__(kThreads, 2)
    batch_flat_kernel(const JobDev* __restrict__ jobs, const Item* __restrict__ items,
                      int64_t n_items, unsigned long long* __restrict__ counter,
                      const PackedSource* __restrict__ arena) {
    __shared__ SmemTile sm;
    __shared__ long long s_item;
    extern __shared__ __align__(16) unsigned char batch_dyn_smem[];
    GTable& gt = *reinterpret_cast<GTable*>(batch_dyn_smem);
    load_theta_table(sm, c_dir_table_b);
    if constexpr (ST == SRC_T4010A1) load_gtab(gt);
    for (;;) {
        const long long it = next_item(counter, s_item);
        if (it >= n_items) break;
        const Item w = items[it];
        const JobDev J = jobs[w.job];
        const int64_t first = static_cast<int64_t>(w.block) * (kThreads * 2 * PAIRS);
        block_points<ST, SUM_PLAIN, PAIRS, true>(sm, gt, arena + J.src_off, J.n, J.is_grid != 0, J.g,
                                           J.pts, J.m, first, J.field, J.out);
    }
}

// One of the two persistent kernels of a plan: its point tile, resident blocks per SM and work
// list.
struct Kern {
    int pairs = 4;
    int bps = 2;
    Item* d_items = nullptr;
    int64_t n_items = 0;
};

struct Plan {
    int st = 1;
    int device = 0;
    bool use_rows = true;  // grid jobs take the rows tiling where the single-job launch would
    int64_t n_jobs = 0;
    int64_t total_sources = 0;
    double evals = 0;
    std::vector<JobDev> jobs;  // host copy
    JobDev* d_jobs = nullptr;
    JobTile* d_tiles = nullptr;  // per job, for the rows kernel's point tile
    Kern rows, flat;
    unsigned long long* d_counters = nullptr;  // [0] rows, [1] flat
    PackedSource* d_arena = nullptr;
    cudaStream_t cap = nullptr, cap2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaGraphExec_t exec = nullptr;
};

template <int ST>
constexpr int flat_dyn_bytes() {
    return ST == SRC_T4010A1 ? kGTableBytes : 0;
}

template <int ST, int PAIRS>
cudaError_t launch_rows_t(const Plan& p, cudaStream_t s) {
    batch_rows_kernel<ST, PAIRS><<<num_sms() * p.rows.bps, kThreads, 0, s>>>(
        p.d_jobs, p.d_tiles, p.rows.d_items, p.rows.n_items, p.d_counters, p.d_arena);
    count_launch();
    return cudaGetLastError();
}

template <int ST, int PAIRS>
cudaError_t launch_flat_t(const Plan& p, cudaStream_t s) {
    const cudaError_t e = allow_dynamic_smem<batch_flat_kernel<ST, PAIRS>>(flat_dyn_bytes<ST>());
    if (e != cudaSuccess) return e;
    batch_flat_kernel<ST, PAIRS><<<num_sms() * p.flat.bps, kThreads, flat_dyn_bytes<ST>(), s>>>(
        p.d_jobs, p.flat.d_items, p.flat.n_items, p.d_counters + 1, p.d_arena);
    count_launch();
    return cudaGetLastError();
}

template <int ST>
cudaError_t launch_rows_st(const Plan& p, cudaStream_t s) {
    if (p.rows.pairs == 1) return launch_rows_t<ST, 1>(p, s);
    if (p.rows.pairs == 2) return launch_rows_t<ST, 2>(p, s);
    return launch_rows_t<ST, 4>(p, s);
}

template <int ST>
cudaError_t launch_flat_st(const Plan& p, cudaStream_t s) {
    if (p.flat.pairs == 1) return launch_flat_t<ST, 1>(p, s);
    if (p.flat.pairs == 2) return launch_flat_t<ST, 2>(p, s);
    return launch_flat_t<ST, 4>(p, s);
}

cudaError_t launch_rows(const Plan& p, cudaStream_t s) {
    return p.st == SRC_T4010A1 ? launch_rows_st<SRC_T4010A1>(p, s) : launch_rows_st<SRC_SPHERE>(p, s);
}

cudaError_t launch_flat(const Plan& p, cudaStream_t s) {
    return p.st == SRC_T4010A1 ? launch_flat_st<SRC_T4010A1>(p, s) : launch_flat_st<SRC_SPHERE>(p, s);
}

// Resident blocks per SM of a kernel (at least 1).
template <auto Kernel>
int occupancy(int dyn) {
    int b = 0;
    if (allow_dynamic_smem<Kernel>(dyn) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, Kernel, kThreads, dyn) != cudaSuccess ||
        b < 1) {
        (void)cudaGetLastError();
        b = 1;
    }
    return b;
}

template <int ST>
int rows_occupancy_st(int pairs) {
    if (pairs == 1) return occupancy<batch_rows_kernel<ST, 1>>(0);
    if (pairs == 2) return occupancy<batch_rows_kernel<ST, 2>>(0);
    return occupancy<batch_rows_kernel<ST, 4>>(0);
}

template <int ST>
int flat_occupancy_st(int pairs) {
    if (pairs == 1) return occupancy<batch_flat_kernel<ST, 1>>(flat_dyn_bytes<ST>());
    if (pairs == 2) return occupancy<batch_flat_kernel<ST, 2>>(flat_dyn_bytes<ST>());
    return occupancy<batch_flat_kernel<ST, 4>>(flat_dyn_bytes<ST>());
}

int rows_occupancy(int st, int pairs) {
    return st == SRC_T4010A1 ? rows_occupancy_st<SRC_T4010A1>(pairs) : rows_occupancy_st<SRC_SPHERE>(pairs);
}

int flat_occupancy(int st, int pairs) {
    return st == SRC_T4010A1 ? flat_occupancy_st<SRC_T4010A1>(pairs) : flat_occupancy_st<SRC_SPHERE>(pairs);
}

cudaError_t upload_items(std::vector<std::pair<double, Item>>& v, Kern& k) {
    std::stable_sort(v.begin(), v.end(),
                     [](const std::pair<double, Item>& a, const std::pair<double, Item>& b) {
                         return a.first > b.first;
                     });
    if (k.d_items) cudaFree(k.d_items);
    k.d_items = nullptr;
    k.n_items = static_cast<int64_t>(v.size());
    if (v.empty()) return cudaSuccess;
    std::vector<Item> items(v.size());
    for (size_t i = 0; i < v.size(); ++i) items[i] = v[i].second;
    cudaError_t e = cudaMalloc(&k.d_items, sizeof(Item) * items.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpy(k.d_items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice);
}

// The two work lists for the current point tiles: tiles of the rows tiling (rows.pairs) for
// the grid jobs the single-job launch tiles by rows (when use_rows), blocks of
// 2*flat.pairs*256 points for every other job; each longest first.
cudaError_t build_items(Plan& p) {
    const int64_t per_block = static_cast<int64_t>(kThreads) * 2 * p.flat.pairs;
    std::vector<std::pair<double, Item>> rv, fv;
    std::vector<JobTile> tiles(static_cast<size_t>(p.n_jobs));
    for (int64_t j = 0; j < p.n_jobs; ++j) {
        const JobDev& J = p.jobs[j];
        const double nsrc = static_cast<double>(J.n > 0 ? J.n : 1);
        const RowsTiling t =
            (p.use_rows && J.is_grid) ? rows_tiling(J.g, J.m, p.rows.pairs) : RowsTiling{};
        if (t.use) {
            if (t.blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
            tiles[j] = JobTile{1, t.tx_log2, t.tiles0, t.tiles1};
            const int64_t tx = 1LL << t.tx_log2;
            for (int64_t b = 0; b < t.blocks; ++b) {
                const int64_t t0 = b % t.tiles0, t1 = (b / t.tiles0) % t.tiles1;
                const int64_t pts = std::min(tx, J.g.count[0] - t0 * tx) *
                                    std::min(t.rows, J.g.count[1] - t1 * t.rows);
                rv.push_back({static_cast<double>(pts) * nsrc,
                              Item{static_cast<int32_t>(j), static_cast<int32_t>(b)}});
            }
            continue;
        }
        tiles[j] = JobTile{0, 0, 0, 0};
        const int64_t blocks = (J.m + per_block - 1) / per_block;
        for (int64_t b = 0; b < blocks; ++b) {
            const int64_t pts = std::min(per_block, J.m - b * per_block);
            fv.push_back({static_cast<double>(pts) * nsrc,
                          Item{static_cast<int32_t>(j), static_cast<int32_t>(b)}});
        }
    }
    cudaError_t e = cudaSuccess;
    if (p.n_jobs > 0) {
        if (!p.d_tiles && (e = cudaMalloc(&p.d_tiles, sizeof(JobTile) * tiles.size())) != cudaSuccess)
            return e;
        if ((e = cudaMemcpy(p.d_tiles, tiles.data(), sizeof(JobTile) * tiles.size(),
                            cudaMemcpyHostToDevice)) != cudaSuccess)
            return e;
    }
    if ((e = upload_items(rv, p.rows)) != cudaSuccess) return e;
    return upload_items(fv, p.flat);
}

// Which kernels a run enqueues (the autotuner times the flat kernel alone first).
enum Which { RUN_BOTH = 0, RUN_FLAT = 1 };

// The graph body: reset the counters, pack all sources, run the persistent kernels (forked
// onto s2 when both have work, joined back into s).
cudaError_t enqueue_batch(const Plan& p, cudaStream_t s, cudaStream_t s2, Which which = RUN_BOTH) {
    cudaError_t e = cudaMemsetAsync(p.d_counters, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (p.n_jobs > 0 && p.total_sources > 0) {
        pack_all_kernel<<<static_cast<unsigned>(p.n_jobs), 256, 0, s>>>(p.st, p.d_jobs, p.d_arena);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const bool rows = which == RUN_BOTH && p.rows.n_items > 0, flat = p.flat.n_items > 0;
    if (rows && flat) {
        if ((e = cudaEventRecord(p.fork, s)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s2, p.fork, 0)) != cudaSuccess ||
            (e = launch_rows(p, s)) != cudaSuccess || (e = launch_flat(p, s2)) != cudaSuccess ||
            (e = cudaEventRecord(p.join, s2)) != cudaSuccess)
            return e;
        return cudaStreamWaitEvent(s, p.join, 0);
    }
    if (rows) return launch_rows(p, s);
    if (flat) return launch_flat(p, s);
    return cudaSuccess;
}

cudaError_t capture(Plan& p) {
    if (p.exec) cudaGraphExecDestroy(p.exec);
    p.exec = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p.cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    e = enqueue_batch(p, p.cap, p.cap2);
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
    if (p->cap2) cudaStreamSynchronize(p->cap2);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->d_jobs) cudaFree(p->d_jobs);
    if (p->d_tiles) cudaFree(p->d_tiles);
    if (p->rows.d_items) cudaFree(p->rows.d_items);
    if (p->flat.d_items) cudaFree(p->flat.d_items);
    if (p->d_counters) cudaFree(p->d_counters);
    if (p->d_arena) cudaFree(p->d_arena);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->join) cudaEventDestroy(p->join);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->cap2) cudaStreamDestroy(p->cap2);
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

// Milliseconds of one run of the plan as it stands (`which` kernels), after one untimed run.
cudaError_t time_plan(Plan& p, Which which, float* ms) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = build_items(p);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
        if ((e = cudaEventRecord(e0, p.cap)) != cudaSuccess) break;
        if ((e = enqueue_batch(p, p.cap, p.cap2, which)) != cudaSuccess) break;
        if ((e = cudaEventRecord(e1, p.cap)) != cudaSuccess) break;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        e = cudaEventElapsedTime(ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return e;
}

// Point pairs and resident blocks per SM to try for a kernel of `occ(pairs)` blocks per SM.
template <class Occ>
std::vector<std::pair<int, int>> candidates(Occ occ) {
    std::vector<std::pair<int, int>> c;
    for (int pairs : {1, 2, 4}) {
        const int o = occ(pairs);
        c.push_back({pairs, o});
        if (o > 1) c.push_back({pairs, o - 1});
    }
    return c;
}

// The autotuner: the flat kernel alone over its point pairs and blocks per SM, then the rows
// kernel with it, then every grid job on the flat body; the fastest plan stays.
cudaError_t autotune(Plan& p) {
    float ms = 0.f, best = 1e30f;
    cudaError_t e = cudaSuccess;
    Kern best_flat = p.flat;
    for (const auto& c : candidates([&](int pr) { return flat_occupancy(p.st, pr); })) {
        p.flat.pairs = c.first;
        p.flat.bps = c.second;
        if ((e = time_plan(p, RUN_FLAT, &ms)) != cudaSuccess) return e;
        if (ms < best) {
            best = ms;
            best_flat = p.flat;
        }
    }
    p.flat.pairs = best_flat.pairs;
    p.flat.bps = best_flat.bps;
    best = 1e30f;
    Kern best_rows = p.rows;
    for (const auto& c : candidates([&](int pr) { return rows_occupancy(p.st, pr); })) {
        p.rows.pairs = c.first;
        p.rows.bps = c.second;
        if ((e = time_plan(p, RUN_BOTH, &ms)) != cudaSuccess) return e;
        if (ms < best) {
            best = ms;
            best_rows = p.rows;
        }
    }
    p.rows.pairs = best_rows.pairs;
    p.rows.bps = best_rows.bps;
    p.use_rows = false;
    if ((e = time_plan(p, RUN_BOTH, &ms)) != cudaSuccess) return e;
    p.use_rows = !(ms < best);  // keep the rows tiling unless every job on the flat body is faster
    return cudaSuccess;
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
    if ((e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&p->cap2, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming)) != cudaSuccess) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: streams / events", e);
    }
    if ((e = cudaMalloc(&p->d_counters, 2 * sizeof(unsigned long long))) != cudaSuccess ||
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
    // default tiles: 4 point pairs per thread, as many resident blocks as fit
    p->rows.pairs = p->flat.pairs = 4;
    p->rows.bps = rows_occupancy(p->st, 4);
    p->flat.bps = flat_occupancy(p->st, 4);
    if (tune && (e = autotune(*p)) != cudaSuccess) {
        destroy(p);
        return fail(AFC_ERR_CUDA, "AFC_BatchCreate: autotuning", e);
    }
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
    count_launch((p->total_sources > 0 ? 1 : 0) + (p->rows.n_items > 0 ? 1 : 0) +
                 (p->flat.n_items > 0 ? 1 : 0));
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
    if (pairs) *pairs = p->flat.pairs;
    if (blocks_per_sm) *blocks_per_sm = p->flat.bps;
    if (items) *items = static_cast<uint64_t>(p->rows.n_items + p->flat.n_items);
    if (evals) *evals = p->evals;
    return AFC_OK;
}

extern "C" int32_t AFC_BatchDescribeKernels(void* plan, int32_t* rows_pairs,
                                            int32_t* rows_blocks_per_sm, uint64_t* rows_items,
                                            int32_t* flat_pairs, int32_t* flat_blocks_per_sm,
                                            uint64_t* flat_items) {
    Plan* p = static_cast<Plan*>(plan);
    if (!p) return fail(AFC_ERR_INVALID, "AFC_BatchDescribeKernels: invalid plan");
    if (rows_pairs) *rows_pairs = p->rows.pairs;
    if (rows_blocks_per_sm) *rows_blocks_per_sm = p->rows.bps;
    if (rows_items) *rows_items = static_cast<uint64_t>(p->rows.n_items);
    if (flat_pairs) *flat_pairs = p->flat.pairs;
    if (flat_blocks_per_sm) *flat_blocks_per_sm = p->flat.bps;
    if (flat_items) *flat_items = static_cast<uint64_t>(p->flat.n_items);
    return AFC_OK;
}

extern "C" void AFC_BatchFree(void* plan) { destroy(static_cast<Plan*>(plan)); }
