// Serving engine: field-evaluation and GS-PAT hologram requests admitted under a fixed HBM
// budget, run concurrently on the GPU, with per-request latency.  No reference counterpart
// (the reference is a library of blocking calls); the work of each request is the reference's
// AFC_Calculate (calculator/cpu_calculator.rs:43-56) or AFO_GSPAT followed by a pressure slice
// (acoustic-field-optimizer/examples/foci.rs:151-153).
//
//   * Geometries (source positions, directions, wavenumbers, attenuations) are registered
//     once, packed on the device and stay resident; a request only uploads its amplitudes and
//     phases (field) or foci and target amplitudes (GS-PAT, whose transfer matrix G is built
//     on the device from the resident geometry and never leaves it).
//   * Submission copies the request's inputs into a pinned host arena and queues it.  A
//     scheduler thread admits queued requests in arrival order whenever a stream slot and
//     enough of the HBM budget (a first-fit device arena) are free, so requests that arrive while
//     others run join as soon as resources free up and their work overlaps on the device.
//   * Continuous batching: the field requests at the head of the queue are admitted together as
//     one group on one slot (up to kGroupMaxJobs requests of one source type, kGroupMaxItems
//     work items, kGroupMaxEvals evaluations) and run as one set of persistent launches
//     (serving_group.h) instead of one launch sequence each.  A request's work items (point
//     tiles times source chunks) depend on the request alone, so its result is the same alone
//     and in any group, bit for bit.  GS-PAT requests, and field requests too large for a
//     group's item table, run on a slot of their own.
//   * Each slot's work ends with a host callback (cudaLaunchHostFunc) that stamps the completion
//     time and wakes the scheduler, which frees the device ranges and hands the finished
//     requests to a pool of completer threads that copy results to the callers' buffers.
//   * Latency = submission to the completion of the request's last operation on the device
//     (the device-to-host copy of its result).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "afc_solvers.h"
#include "serving_group.h"

namespace afc {
namespace serve {

// Threads that copy finished results from pinned staging to the callers' buffers (a result
// is up to a few MB; one thread alone would cap throughput at high request rates).
constexpr int kCompleters = 4;
// Limits of one group: requests, work items (the slot's item table), evaluations (a group
// closes before it would exceed them, unless it is empty: a large request still runs).
constexpr int kGroupMaxJobs = 64;
constexpr int64_t kGroupMaxItems = 1 << 16;
constexpr double kGroupMaxEvals = 4.0e9;

constexpr size_t al256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

// A slot's group table: jobs, then items, then the two work counters.
constexpr size_t kGroupJobsBytes = al256(sizeof(GJob) * kGroupMaxJobs);
constexpr size_t kGroupItemsBytes = al256(sizeof(GItem) * kGroupMaxItems);
constexpr size_t kGroupTableBytes = kGroupJobsBytes + kGroupItemsBytes + 256;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// First-fit allocator of [0, capacity) with coalescing of freed ranges.
class RangeAllocator {
   public:
    explicit RangeAllocator(size_t cap = 0) : cap_(cap) {
        if (cap) free_[0] = cap;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = al256(bytes ? bytes : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, next = it->first + bytes;
                free_.erase(it);
                if (rest) free_[next] = rest;
                used_ += bytes;
                if (used_ > peak_) peak_ = used_;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = al256(bytes ? bytes : 1);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }

   private:
    size_t cap_;
    size_t used_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_;
};

struct Geometry {
    int st = 1;
    int64_t n = 0;
    float* d_raw = nullptr;  // ABI records | k | atten
    PackedSource* d_packed = nullptr;
};

enum Kind { KIND_FIELD = 0, KIND_GSPAT = 1 };
enum State { QUEUED = 0, RUNNING = 1, FINISHING = 2, DONE = 3, FAILED = 4 };

struct Request {
    int64_t id = 0;
    Kind kind = KIND_FIELD;
    int geom = 0;
    int st = 1;
    int field = 0;
    PointSet ps{};          // the points of a field request, or the slice of a GS-PAT request
    int64_t n_foci = 0;
    // pinned block: inputs then outputs
    size_t h_off = 0, h_bytes = 0, h_in = 0, h_out = 0, h_out2 = 0;
    size_t out_bytes = 0, out2_bytes = 0;
    float* user_out = nullptr;
    float* user_out2 = nullptr;
    // device block
    size_t d_off = 0, d_bytes = 0;
    // group layout of a field request (serving_group.h)
    bool grouped = false;
    bool rows = false;
    RowsTiling tiling{};
    int64_t tiles = 0, chunks = 1, chunk = 0, items = 0;
    size_t part_bytes = 0;
    double evals = 0;
    int slot = -1;
    State state = QUEUED;
    std::string error;
    double t_submit = 0, t_start = 0, t_done = 0;
};

class Engine;

// What a slot's completion callback needs.
struct SlotCtx {
    Engine* engine = nullptr;
    int slot = 0;
};

struct Slot {
    cudaStream_t stream = nullptr, stream2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    char* d_table = nullptr;  // group table (kGroupTableBytes), device
    char* h_table = nullptr;  // and its pinned staging
    std::vector<int64_t> reqs;
    bool busy = false, finished = false;
    double t_finished = 0;
    SlotCtx ctx;
};

// Device layout of a field request's block: drive, packed sources, points, result, partials.
struct FieldLayout {
    size_t ap, pk, pts, out, part;
};

FieldLayout field_layout(int64_t n, const Request& r) {
    FieldLayout L;
    L.ap = 0;
    L.pk = al256(8 * static_cast<size_t>(n));
    L.pts = L.pk + al256(48 * static_cast<size_t>(n));
    const size_t pts_bytes = r.ps.is_grid ? 0 : 12 * static_cast<size_t>(r.ps.m);
    L.out = L.pts + al256(pts_bytes);
    L.part = L.out + al256(r.out_bytes);
    return L;
}

// The group layout of a field request of n sources: point tiles (the rows tiling where the
// single-job launch would take it, else kGroupTilePoints-point blocks), cut into source chunks
// of at least kMinChunkSources sources until the request alone has about target items (so that
// a small request spreads over the GPU), and whether the request fits a group at all.
void group_layout(Request& r, int64_t n, int64_t target) {
    const RowsTiling t = r.ps.is_grid ? rows_tiling(r.ps.grid, r.ps.m, kGroupPairs) : RowsTiling{};
    r.rows = t.use;
    r.tiling = t;
    r.tiles = t.use ? t.blocks : (r.ps.m + kGroupTilePoints - 1) / kGroupTilePoints;
    int64_t chunks = 1;
    if (n > 0 && r.tiles > 0 && r.tiles < target) {
        chunks = (target + r.tiles - 1) / r.tiles;
        chunks = std::min(chunks, std::max<int64_t>(1, n / kMinChunkSources));
    }
    r.chunk = n > 0 ? (n + chunks - 1) / chunks : 0;
    r.chunks = n > 0 ? (n + r.chunk - 1) / r.chunk : 1;
    r.items = r.tiles * r.chunks;
    r.part_bytes = r.chunks > 1 ? 8 * static_cast<size_t>(r.chunks) * static_cast<size_t>(r.ps.m) : 0;
    r.evals = static_cast<double>(n) * static_cast<double>(r.ps.m);
    r.grouped = r.ps.m > 0 && r.items <= kGroupMaxItems;
}

class Engine {
   public:
    int device = 0;
    int64_t group_target = 304;  // work items a lone request is cut into (2 per SM)
    int occ_rows[2] = {1, 1}, occ_flat[2] = {1, 1};  // resident blocks per SM, per source type
    int sms = 1;
    char* d_arena = nullptr;
    char* h_arena = nullptr;
    // the pinned arena's address for kernels (under unified addressing every cudaHostAlloc
    // buffer is device-addressable): field kernels write results of up to kDirectOutBytes
    // straight into a request's host block, where a copy's fixed cost would dominate; larger
    // results (and all, when NULL) go through the device arena and the copy engine
    char* h_arena_dev = nullptr;
    static constexpr size_t kDirectOutBytes = 1u << 20;
    // where a request's field kernel writes its result: its host block, or NULL for its device
    // block
    char* direct_out(const Request& r) const {
        return (h_arena_dev && r.out_bytes <= kDirectOutBytes) ? h_arena_dev + r.h_off + r.h_out
                                                               : nullptr;
    }
    RangeAllocator dev_alloc, host_alloc;
    std::vector<Slot> slots;
    std::deque<Geometry> geoms;  // a deque: references stay valid while geometries are added

    std::mutex mu;
    std::condition_variable cv_sched, cv_done, cv_host;
    std::deque<int64_t> queue;
    std::deque<int64_t> finishing;
    std::unordered_map<int64_t, Request> reqs;
    int64_t next_id = 1;
    uint64_t wake = 0;  // bumped by submissions and completion callbacks
    std::atomic<bool> stop{false};
    std::thread sched;
    std::vector<std::thread> completers;  // copy results out of the pinned arena
    int inflight = 0, peak_inflight = 0;
    uint64_t completed = 0, failed = 0;

    ~Engine() { shutdown(); }

    void shutdown() {
        DeviceGuard dg;  // the engine's device while tearing down; the caller's again after
        dg.set(device);
        stop = true;
        {
            std::lock_guard<std::mutex> lk(mu);
            ++wake;
        }
        cv_sched.notify_all();
        cv_host.notify_all();
        if (sched.joinable()) sched.join();
        for (std::thread& t : completers)
            if (t.joinable()) t.join();
        for (Slot& s : slots) {
            if (s.stream) {
                cudaStreamSynchronize(s.stream);
                cudaStreamDestroy(s.stream);
            }
            if (s.stream2) {
                cudaStreamSynchronize(s.stream2);
                cudaStreamDestroy(s.stream2);
            }
            if (s.fork) cudaEventDestroy(s.fork);
            if (s.join) cudaEventDestroy(s.join);
            if (s.d_table) cudaFree(s.d_table);
            if (s.h_table) cudaFreeHost(s.h_table);
        }
        slots.clear();
        for (Geometry& g : geoms) {
            if (g.d_raw) cudaFree(g.d_raw);
            if (g.d_packed) cudaFree(g.d_packed);
        }
        geoms.clear();
        if (d_arena) cudaFree(d_arena);
        if (h_arena) cudaFreeHost(h_arena);
        d_arena = nullptr;
        h_arena = nullptr;
    }

    // Completion callback of slot i (runs on a CUDA driver thread: no CUDA calls here).
    void on_slot_done(int i) {
        const double t = now_s();
        {
            std::lock_guard<std::mutex> lk(mu);
            slots[i].finished = true;
            slots[i].t_finished = t;
            ++wake;
        }
        cv_sched.notify_all();
    }

    static void CUDART_CB slot_done(void* p) {
        SlotCtx* c = static_cast<SlotCtx*>(p);
        c->engine->on_slot_done(c->slot);
    }

    // Ends slot i's work with the completion callback; if that cannot be enqueued the slot is
    // marked finished at once (its requests carry the error).
    void close_slot(int i) {
        Slot& sl = slots[i];
        if (cudaLaunchHostFunc(sl.stream, slot_done, &sl.ctx) != cudaSuccess) {
            std::lock_guard<std::mutex> lk(mu);
            for (int64_t id : sl.reqs) {
                Request& r = reqs[id];
                if (r.error.empty()) r.error = "serving: completion callback could not be enqueued";
            }
            sl.finished = true;
            sl.t_finished = now_s();
            ++wake;
        }
    }

    // ---- work of one request on its own slot
    cudaError_t launch_single(Request& r, const Geometry& g) {
        Slot& sl = slots[r.slot];
        cudaStream_t s = sl.stream;
        char* d = d_arena + r.d_off;
        char* h = h_arena + r.h_off;
        cudaError_t e;
        const int64_t n = g.n;
        if (r.kind == KIND_FIELD) {
            const FieldLayout L = field_layout(n, r);
            const size_t in_pts_bytes = r.ps.is_grid ? 0 : 12 * static_cast<size_t>(r.ps.m);
            if (n && (e = cudaMemcpyAsync(d + L.ap, h + r.h_in, 8 * n, cudaMemcpyHostToDevice, s)) !=
                         cudaSuccess)
                return e;
            if (in_pts_bytes &&
                (e = cudaMemcpyAsync(d + L.pts, h + r.h_in + al256(8 * n), in_pts_bytes,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return e;
            float* amps = reinterpret_cast<float*>(d + L.ap);
            auto* packed = reinterpret_cast<PackedSource*>(d + L.pk);
            if ((e = launch_repack(g.d_packed, amps, amps + n, nullptr, n, packed, s)) != cudaSuccess)
                return e;
            PointSet ps = r.ps;
            if (!ps.is_grid) ps.pts = reinterpret_cast<const float*>(d + L.pts);
            // device memory only from the engine's budgeted arena: no partial-sum scratch
            char* direct = direct_out(r);
            if ((e = launch_field(g.st, r.field, SUM_PLAIN, packed, n, ps, direct ? direct : d + L.out,
                                  s, false)) != cudaSuccess)
                return e;
            if (!direct && r.out_bytes &&
                (e = cudaMemcpyAsync(h + r.h_out, d + L.out, r.out_bytes, cudaMemcpyDeviceToHost, s)) !=
                    cudaSuccess)
                return e;
        } else {
            // device: foci|amps (16 M), solver workspace, amp/phase (8n), packed (48n), slice out
            const int64_t M = r.n_foci;
            const size_t o_in = 0, o_ws = al256(16 * M), wsb = solver_workspace_bytes(n, M);
            const size_t o_ap = o_ws + al256(wsb), o_pk = o_ap + al256(8 * n);
            const size_t o_out = o_pk + al256(48 * n);
            if ((e = cudaMemcpyAsync(d + o_in, h + r.h_in, 16 * M, cudaMemcpyHostToDevice, s)) !=
                cudaSuccess)
                return e;
            const float* foci = reinterpret_cast<const float*>(d + o_in);
            const float* tamps = foci + 3 * M;
            float* ap = reinterpret_cast<float*>(d + o_ap);
            const int stride = source_stride(g.st);
            const float* raw = g.d_raw;
            if ((e = launch_solver(SOLVER_GSPAT, g.st, raw, raw + n * stride, raw + n * (stride + 1), n,
                                   foci, tamps, M, kSolverRepeat, ap, d + o_ws, s)) != cudaSuccess)
                return e;
            auto* packed = reinterpret_cast<PackedSource*>(d + o_pk);
            if ((e = launch_repack(g.d_packed, nullptr, nullptr, ap, n, packed, s)) != cudaSuccess)
                return e;
            char* direct = direct_out(r);
            if ((e = launch_field(g.st, FIELD_PRESSURE, SUM_PLAIN, packed, n, r.ps,
                                  direct ? direct : d + o_out, s, false)) != cudaSuccess)
                return e;
            if (!direct && r.out_bytes &&
                (e = cudaMemcpyAsync(h + r.h_out, d + o_out, r.out_bytes, cudaMemcpyDeviceToHost, s)) !=
                    cudaSuccess)
                return e;
            if ((e = cudaMemcpyAsync(h + r.h_out2, ap, r.out2_bytes, cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess)
                return e;
        }
        return cudaSuccess;
    }

    // ---- a group of field requests on slot i (rq: the requests, gs: their geometries)
    cudaError_t launch_group_slot(int i, const std::vector<Request*>& rq,
                                  const std::vector<const Geometry*>& gs) {
        Slot& sl = slots[i];
        cudaStream_t s = sl.stream;
        cudaError_t e;
        const int st = rq[0]->st;
        GJob* hj = reinterpret_cast<GJob*>(sl.h_table);
        GItem* hi = reinterpret_cast<GItem*>(sl.h_table + kGroupJobsBytes);
        std::vector<std::pair<double, GItem>> rows_items, flat_items;
        int64_t max_n = 0;
        bool chunked = false;
        for (size_t j = 0; j < rq.size(); ++j) {
            Request& r = *rq[j];
            const Geometry& g = *gs[j];
            const int64_t n = g.n;
            char* d = d_arena + r.d_off;
            char* h = h_arena + r.h_off;
            const FieldLayout L = field_layout(n, r);
            const size_t in_pts_bytes = r.ps.is_grid ? 0 : 12 * static_cast<size_t>(r.ps.m);
            if (n && (e = cudaMemcpyAsync(d + L.ap, h + r.h_in, 8 * n, cudaMemcpyHostToDevice, s)) !=
                         cudaSuccess)
                return e;
            if (in_pts_bytes &&
                (e = cudaMemcpyAsync(d + L.pts, h + r.h_in + al256(8 * n), in_pts_bytes,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return e;
            GJob& J = hj[j];
            J = GJob{};
            J.geom = g.d_packed;
            J.amps = reinterpret_cast<const float*>(d + L.ap);
            J.packed = reinterpret_cast<PackedSource*>(d + L.pk);
            J.n = n;
            J.g = r.ps.grid;
            J.pts = r.ps.is_grid ? nullptr : reinterpret_cast<const float*>(d + L.pts);
            J.m = r.ps.m;
            char* direct = direct_out(r);
            J.out = direct ? direct : d + L.out;
            J.partial = r.chunks > 1 ? reinterpret_cast<float2*>(d + L.part) : nullptr;
            J.field = r.field;
            J.is_grid = r.ps.is_grid ? 1 : 0;
            J.chunks = static_cast<int32_t>(r.chunks);
            J.chunk = r.chunk;
            J.rows = r.rows ? 1 : 0;
            J.tx_log2 = r.tiling.tx_log2;
            J.tiles0 = r.tiling.tiles0;
            J.tiles1 = r.tiling.tiles1;
            max_n = std::max(max_n, n);
            chunked = chunked || r.chunks > 1;
            // items: cost = points of the tile x sources of the chunk, longest first
            for (int64_t t = 0; t < r.tiles; ++t) {
                int64_t pts;
                if (r.rows) {
                    const int64_t tx = 1LL << r.tiling.tx_log2;
                    const int64_t t0 = t % r.tiling.tiles0, t1 = (t / r.tiling.tiles0) % r.tiling.tiles1;
                    pts = std::min(tx, r.ps.grid.count[0] - t0 * tx) *
                          std::min(r.tiling.rows, r.ps.grid.count[1] - t1 * r.tiling.rows);
                } else {
                    pts = std::min(kGroupTilePoints, r.ps.m - t * kGroupTilePoints);
                }
                for (int64_t c = 0; c < r.chunks; ++c) {
                    const int64_t lo = c * r.chunk, hi = std::min(n, lo + r.chunk);
                    const GItem it{static_cast<int32_t>(j), static_cast<int32_t>(c), t};
                    (r.rows ? rows_items : flat_items)
                        .push_back({static_cast<double>(pts) * static_cast<double>(hi - lo), it});
                }
            }
        }
        auto by_cost = [](const std::pair<double, GItem>& a, const std::pair<double, GItem>& b) {
            return a.first > b.first;
        };
        std::stable_sort(rows_items.begin(), rows_items.end(), by_cost);
        std::stable_sort(flat_items.begin(), flat_items.end(), by_cost);
        const int64_t n_rows = static_cast<int64_t>(rows_items.size());
        const int64_t n_flat = static_cast<int64_t>(flat_items.size());
        for (int64_t k = 0; k < n_rows; ++k) hi[k] = rows_items[k].second;
        for (int64_t k = 0; k < n_flat; ++k) hi[n_rows + k] = flat_items[k].second;
        const size_t used = kGroupJobsBytes + sizeof(GItem) * static_cast<size_t>(n_rows + n_flat);
        if ((e = cudaMemcpyAsync(sl.d_table, sl.h_table, used, cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
            return e;
        const GJob* dj = reinterpret_cast<const GJob*>(sl.d_table);
        const GItem* di = reinterpret_cast<const GItem*>(sl.d_table + kGroupJobsBytes);
        auto* counters =
            reinterpret_cast<unsigned long long*>(sl.d_table + kGroupJobsBytes + kGroupItemsBytes);
        const int sti = st == SRC_T4010A1 ? 1 : 0;
        if ((e = launch_group(st, dj, static_cast<int>(rq.size()), max_n, di, n_rows, di + n_rows,
                              n_flat, counters, chunked, occ_rows[sti] * sms,
                              occ_flat[sti] * sms, s, sl.stream2, sl.fork, sl.join)) != cudaSuccess)
            return e;
        for (size_t j = 0; j < rq.size(); ++j) {
            Request& r = *rq[j];
            const FieldLayout L = field_layout(gs[j]->n, r);
            if (r.out_bytes && !direct_out(r) &&
                (e = cudaMemcpyAsync(h_arena + r.h_off + r.h_out, d_arena + r.d_off + L.out,
                                     r.out_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
                return e;
        }
        return cudaSuccess;
    }

    int free_slot() const {
        for (size_t i = 0; i < slots.size(); ++i)
            if (!slots[i].busy) return static_cast<int>(i);
        return -1;
    }

    void start(Request& r, int slot) {
        r.slot = slot;
        r.state = RUNNING;
        r.t_start = now_s();
        ++inflight;
        if (inflight > peak_inflight) peak_inflight = inflight;
    }

    // Frees the device ranges of slot i's finished requests and queues them for the completers.
    void retire(int i) {
        Slot& sl = slots[i];
        for (int64_t id : sl.reqs) {
            Request& r = reqs[id];
            r.t_done = sl.t_finished;
            dev_alloc.release(r.d_off, r.d_bytes);
            --inflight;
            r.state = FINISHING;
            finishing.push_back(id);
        }
        sl.reqs.clear();
        sl.busy = false;
        sl.finished = false;
    }

    void scheduler_loop() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            bool retired = false;
            for (size_t i = 0; i < slots.size(); ++i) {
                if (slots[i].busy && slots[i].finished) {
                    retire(static_cast<int>(i));
                    retired = true;
                }
            }
            if (retired) cv_host.notify_all();
            if (stop && queue.empty() && inflight == 0) break;
            // admit in arrival order while a slot and the budget allow: the field requests at
            // the head of the queue as one group, anything else on a slot of its own
            std::vector<int> singles, groups;
            while (!queue.empty()) {
                const int fs = free_slot();
                if (fs < 0) break;
                Request& r = reqs[queue.front()];
                if (r.kind != KIND_FIELD || !r.grouped) {
                    if (!dev_alloc.alloc(r.d_bytes, &r.d_off)) break;
                    queue.pop_front();
                    start(r, fs);
                    slots[fs].busy = true;
                    slots[fs].reqs.assign(1, r.id);
                    singles.push_back(fs);
                    continue;
                }
                std::vector<int64_t> g;
                int64_t items = 0;
                double evals = 0;
                while (!queue.empty() && static_cast<int>(g.size()) < kGroupMaxJobs) {
                    Request& q = reqs[queue.front()];
                    if (q.kind != KIND_FIELD || !q.grouped || q.st != r.st) break;
                    if (!g.empty() &&
                        (items + q.items > kGroupMaxItems || evals + q.evals > kGroupMaxEvals))
                        break;
                    if (!dev_alloc.alloc(q.d_bytes, &q.d_off)) break;
                    queue.pop_front();
                    start(q, fs);
                    g.push_back(q.id);
                    items += q.items;
                    evals += q.evals;
                }
                if (g.empty()) break;  // the head request does not fit the budget yet
                slots[fs].busy = true;
                slots[fs].reqs = g;
                groups.push_back(fs);
            }
            if (!singles.empty() || !groups.empty()) {
                // the requests' and geometries' addresses, taken under the lock
                std::vector<std::pair<Request*, const Geometry*>> one;
                std::vector<std::vector<Request*>> grq;
                std::vector<std::vector<const Geometry*>> ggs;
                for (int fs : singles) {
                    Request* r = &reqs[slots[fs].reqs[0]];
                    one.push_back({r, &geoms[r->geom]});
                }
                for (int fs : groups) {
                    grq.emplace_back();
                    ggs.emplace_back();
                    for (int64_t id : slots[fs].reqs) {
                        Request* r = &reqs[id];
                        grq.back().push_back(r);
                        ggs.back().push_back(&geoms[r->geom]);
                    }
                }
                lk.unlock();
                for (size_t k = 0; k < singles.size(); ++k) {
                    const cudaError_t e = launch_single(*one[k].first, *one[k].second);
                    if (e != cudaSuccess) {
                        std::lock_guard<std::mutex> g2(mu);
                        one[k].first->error = cudaGetErrorString(e);
                    }
                    close_slot(singles[k]);
                }
                for (size_t k = 0; k < groups.size(); ++k) {
                    const cudaError_t e = launch_group_slot(groups[k], grq[k], ggs[k]);
                    if (e != cudaSuccess) {
                        std::lock_guard<std::mutex> g2(mu);
                        for (Request* r : grq[k]) r->error = cudaGetErrorString(e);
                    }
                    close_slot(groups[k]);
                }
                lk.lock();
                continue;
            }
            // nothing to admit or retire: sleep until a submission, a completion or stop
            const uint64_t seen = wake;
            if (!cv_sched.wait_for(lk, std::chrono::milliseconds(50),
                                   [&] { return wake != seen; }) &&
                inflight > 0) {
                // no callback for a while: a slot whose stream failed never calls back
                std::vector<std::pair<int, cudaStream_t>> busy;
                for (size_t i = 0; i < slots.size(); ++i)
                    if (slots[i].busy && !slots[i].finished)
                        busy.push_back({static_cast<int>(i), slots[i].stream});
                lk.unlock();
                std::vector<std::pair<int, cudaError_t>> bad;
                for (const auto& b : busy) {
                    const cudaError_t q = cudaStreamQuery(b.second);
                    if (q != cudaSuccess && q != cudaErrorNotReady) bad.push_back({b.first, q});
                }
                lk.lock();
                for (const auto& b : bad) {
                    Slot& sl = slots[b.first];
                    if (!sl.busy || sl.finished) continue;
                    for (int64_t id : sl.reqs) {
                        Request& r = reqs[id];
                        if (r.error.empty()) r.error = cudaGetErrorString(b.second);
                    }
                    sl.finished = true;
                    sl.t_finished = now_s();
                }
            }
        }
    }

    void completer_loop() {
        while (true) {
            int64_t id;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_host.wait_for(lk, std::chrono::milliseconds(1),
                                 [&] { return !finishing.empty() || stop; });
                if (finishing.empty()) {
                    if (stop && queue.empty() && inflight == 0) break;
                    continue;
                }
                id = finishing.front();
                finishing.pop_front();
            }
            Request* r;
            {
                std::lock_guard<std::mutex> lk(mu);
                r = &reqs[id];
            }
            if (r->error.empty()) {
                const char* block = h_arena + r->h_off;  // the request's staging block
                if (r->user_out && r->out_bytes) memcpy(r->user_out, block + r->h_out, r->out_bytes);
                if (r->user_out2 && r->out2_bytes)
                    memcpy(r->user_out2, block + r->h_out2, r->out2_bytes);
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                host_alloc.release(r->h_off, r->h_bytes);
                r->state = r->error.empty() ? DONE : FAILED;
                if (r->error.empty()) ++completed; else ++failed;
            }
            cv_done.notify_all();
            cv_host.notify_all();
        }
    }

    // Reserve pinned staging (waits for space), copy inputs, queue.
    int64_t submit(Request&& r, const void* in1, size_t b1, const void* in2, size_t b2) {
        r.h_in = 0;
        const size_t in_total = al256(b1) + al256(b2);
        r.h_out = in_total;
        r.h_out2 = in_total + al256(r.out_bytes);
        r.h_bytes = r.h_out2 + al256(r.out2_bytes);
        if (r.d_bytes > dev_alloc.capacity()) {
            set_error_message("serving: request needs more device memory than the whole HBM budget");
            return AFC_ERR_TOO_LARGE;
        }
        if (r.h_bytes > host_alloc.capacity()) {
            set_error_message("serving: request needs more pinned memory than the host arena");
            return AFC_ERR_TOO_LARGE;
        }
        std::unique_lock<std::mutex> lk(mu);
        cv_host.wait(lk, [&] { return stop || host_alloc.alloc(r.h_bytes, &r.h_off); });
        if (stop) return AFC_ERR_INVALID;
        lk.unlock();
        char* h = h_arena + r.h_off;
        if (b1) memcpy(h, in1, b1);
        if (b2) memcpy(h + al256(b1), in2, b2);
        lk.lock();
        r.id = next_id++;
        r.t_submit = now_s();
        r.state = QUEUED;
        const int64_t id = r.id;
        reqs.emplace(id, std::move(r));
        queue.push_back(id);
        ++wake;
        lk.unlock();
        cv_sched.notify_all();
        return id;
    }
};

// Points of one request at most: 2^40 points need terabytes, far beyond any HBM budget, and keep
// every byte count of the request far from wrapping.
constexpr int64_t kMaxRequestPoints = 1LL << 40;

bool valid_grid(const AfcGridDesc* g, GridDev* out) {
    if (!g) return false;
    bool seen[3] = {false, false, false};
    for (int k = 0; k < 3; ++k) {
        const int a = g->axis[k] - 1;
        if (a < 0 || a > 2 || seen[a] || g->count[k] == 0) return false;
        seen[a] = true;
        out->axis[k] = a;
        out->count[k] = static_cast<int64_t>(g->count[k]);
        out->origin[k] = g->origin[k];
    }
    out->res = g->res;
    // the point count must not wrap (a request that large could never be admitted anyway)
    unsigned __int128 total = 1;
    for (int k = 0; k < 3; ++k) {
        total *= g->count[k];
        if (total > (static_cast<unsigned __int128>(1) << 62)) return false;
    }
    return true;
}

}  // namespace serve
}  // namespace afc

using namespace afc;
using namespace afc::serve;

extern "C" int32_t AFC_ServeCreate(const AfcServeConfig* cfg, void** engine) {
    if (!engine || !cfg || cfg->hbm_budget_bytes == 0 || cfg->pinned_bytes == 0 ||
        cfg->max_inflight < 1) {
        set_error_message("AFC_ServeCreate: invalid configuration");
        return AFC_ERR_INVALID;
    }
    *engine = nullptr;
    Engine* e = new (std::nothrow) Engine;
    if (!e) return AFC_ERR_INVALID;
    cudaError_t ce = cudaGetDevice(&e->device);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_arena, cfg->hbm_budget_bytes);
    if (ce == cudaSuccess) ce = cudaHostAlloc(&e->h_arena, cfg->pinned_bytes, cudaHostAllocDefault);
    if (ce != cudaSuccess) {
        set_error_message(cudaGetErrorString(ce));
        delete e;
        return AFC_ERR_CUDA;
    }
    e->dev_alloc = RangeAllocator(cfg->hbm_budget_bytes);
    e->host_alloc = RangeAllocator(cfg->pinned_bytes);
    {
        void* hd = nullptr;
        if (cudaHostGetDevicePointer(&hd, e->h_arena, 0) == cudaSuccess && hd)
            e->h_arena_dev = static_cast<char*>(hd);
        else
            (void)cudaGetLastError();
    }
    e->sms = num_sms();
    e->group_target = 2LL * e->sms;
    for (int st = 0; st < 2; ++st) {
        e->occ_rows[st] = group_rows_occupancy(st);
        e->occ_flat[st] = group_flat_occupancy(st);
    }
    e->slots.resize(static_cast<size_t>(cfg->max_inflight));
    for (size_t i = 0; i < e->slots.size(); ++i) {
        Slot& s = e->slots[i];
        s.ctx.engine = e;
        s.ctx.slot = static_cast<int>(i);
        if ((ce = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (ce = cudaStreamCreateWithFlags(&s.stream2, cudaStreamNonBlocking)) != cudaSuccess ||
            (ce = cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming)) != cudaSuccess ||
            (ce = cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming)) != cudaSuccess ||
            (ce = cudaMalloc(&s.d_table, kGroupTableBytes)) != cudaSuccess ||
            (ce = cudaHostAlloc(&s.h_table, kGroupTableBytes, cudaHostAllocDefault)) != cudaSuccess) {
            set_error_message(cudaGetErrorString(ce));
            delete e;
            return AFC_ERR_CUDA;
        }
    }
    e->sched = std::thread([e] { e->scheduler_loop(); });
    for (int i = 0; i < kCompleters; ++i) e->completers.emplace_back([e] { e->completer_loop(); });
    *engine = e;
    return AFC_OK;
}

extern "C" int32_t AFC_ServeAddGeometry(void* engine, int32_t source_type, const float* h_sources,
                                        const float* h_wavenums, const float* h_attens, uint64_t n,
                                        int32_t* geometry_id) {
    Engine* e = static_cast<Engine*>(engine);
    if (!e || !geometry_id || (source_type != SRC_SPHERE && source_type != SRC_T4010A1) ||
        (n && (!h_sources || !h_wavenums || !h_attens))) {
        set_error_message("AFC_ServeAddGeometry: invalid argument");
        return AFC_ERR_INVALID;
    }
    Geometry g;
    g.st = source_type;
    g.n = static_cast<int64_t>(n);
    const int stride = source_stride(source_type);
    const size_t raw_floats = static_cast<size_t>(n) * (stride + 2);
    DeviceGuard dg;  // the engine's device while uploading; the caller's again on return
    cudaError_t ce = dg.set(e->device);
    if (ce == cudaSuccess) ce = cudaMalloc(&g.d_raw, sizeof(float) * (raw_floats ? raw_floats : 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&g.d_packed, sizeof(PackedSource) * (n ? n : 1));
    if (ce == cudaSuccess && n) {
        ce = cudaMemcpy(g.d_raw, h_sources, sizeof(float) * n * stride, cudaMemcpyHostToDevice);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(g.d_raw + n * stride, h_wavenums, sizeof(float) * n, cudaMemcpyHostToDevice);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(g.d_raw + n * (stride + 1), h_attens, sizeof(float) * n,
                            cudaMemcpyHostToDevice);
        if (ce == cudaSuccess)
            ce = launch_pack_sources(source_type, g.d_raw, g.d_raw + n * stride,
                                     g.d_raw + n * (stride + 1), g.n, g.d_packed, nullptr);
        if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    }
    if (ce != cudaSuccess) {
        if (g.d_raw) cudaFree(g.d_raw);
        if (g.d_packed) cudaFree(g.d_packed);
        set_error_message(cudaGetErrorString(ce));
        return AFC_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(e->mu);
    e->geoms.push_back(g);
    *geometry_id = static_cast<int32_t>(e->geoms.size() - 1);
    return AFC_OK;
}

extern "C" int64_t AFC_ServeSubmitField(void* engine, int32_t geometry, const float* h_amps,
                                        const float* h_phases, int32_t field_type, int32_t is_grid,
                                        const AfcGridDesc* grid, const float* h_points,
                                        uint64_t n_points, float* h_out) {
    Engine* e = static_cast<Engine*>(engine);
    int64_t gn = -1;  // the geometry's source count and type, read under the lock AddGeometry takes
    int gst = SRC_T4010A1;
    if (e && geometry >= 0) {
        std::lock_guard<std::mutex> lk(e->mu);
        if (geometry < static_cast<int32_t>(e->geoms.size())) {
            gn = e->geoms[geometry].n;
            gst = e->geoms[geometry].st;
        }
    }
    if (!e || gn < 0 || field_type < FIELD_PRESSURE || field_type > FIELD_COMPLEX || !h_out) {
        set_error_message("AFC_ServeSubmitField: invalid argument");
        return AFC_ERR_INVALID;
    }
    if (gn && (!h_amps || !h_phases)) {
        set_error_message("AFC_ServeSubmitField: amplitudes / phases are NULL");
        return AFC_ERR_INVALID;
    }
    Request r;
    r.kind = KIND_FIELD;
    r.geom = geometry;
    r.st = gst;
    r.field = field_type;
    r.ps.is_grid = is_grid != 0;
    if (is_grid) {
        if (!valid_grid(grid, &r.ps.grid)) {
            set_error_message("AFC_ServeSubmitField: invalid grid description");
            return AFC_ERR_INVALID;
        }
        r.ps.m = r.ps.grid.count[0] * r.ps.grid.count[1] * r.ps.grid.count[2];
    } else {
        if (n_points && !h_points) {
            set_error_message("AFC_ServeSubmitField: points are NULL");
            return AFC_ERR_INVALID;
        }
        r.ps.grid.count[0] = r.ps.grid.count[1] = r.ps.grid.count[2] = 1;
        r.ps.m = static_cast<int64_t>(n_points);
    }
    const int64_t n = gn, m = r.ps.m;
    if (m < 0 || m > kMaxRequestPoints) {  // byte counts must not wrap; no budget holds this
        set_error_message("AFC_ServeSubmitField: too many points");
        return AFC_ERR_TOO_LARGE;
    }
    r.out_bytes = field_elem_bytes(field_type) * static_cast<size_t>(m);
    r.user_out = h_out;
    const size_t pts_bytes = is_grid ? 0 : 12 * static_cast<size_t>(m);
    group_layout(r, n, e->group_target);
    r.d_bytes = al256(8 * n) + al256(48 * n) + al256(pts_bytes) + al256(r.out_bytes) +
                (r.grouped ? al256(r.part_bytes) : 0);
    // inputs: amps|phases contiguous, then points
    std::vector<float> ap(static_cast<size_t>(2 * n));
    if (n) {
        memcpy(ap.data(), h_amps, sizeof(float) * n);
        memcpy(ap.data() + n, h_phases, sizeof(float) * n);
    }
    return e->submit(std::move(r), ap.data(), sizeof(float) * 2 * n, h_points, pts_bytes);
}

extern "C" int64_t AFC_ServeSubmitGspat(void* engine, int32_t geometry, const float* h_foci,
                                        const float* h_amps, uint64_t n_foci,
                                        const AfcGridDesc* slice, float* h_slice_out,
                                        float* h_amp_phase_out) {
    Engine* e = static_cast<Engine*>(engine);
    int64_t gn = -1;  // the geometry's source count and type, read under the lock AddGeometry takes
    int gst = SRC_T4010A1;
    if (e && geometry >= 0) {
        std::lock_guard<std::mutex> lk(e->mu);
        if (geometry < static_cast<int32_t>(e->geoms.size())) {
            gn = e->geoms[geometry].n;
            gst = e->geoms[geometry].st;
        }
    }
    if (!e || gn < 0 || n_foci == 0 || !h_foci || !h_amps || !h_slice_out ||
        n_foci > static_cast<uint64_t>(kSolverMaxFoci)) {
        set_error_message("AFC_ServeSubmitGspat: invalid argument");
        return AFC_ERR_INVALID;
    }
    Request r;
    r.kind = KIND_GSPAT;
    r.geom = geometry;
    r.st = gst;
    r.n_foci = static_cast<int64_t>(n_foci);
    r.ps.is_grid = true;
    if (!valid_grid(slice, &r.ps.grid)) {
        set_error_message("AFC_ServeSubmitGspat: invalid slice description");
        return AFC_ERR_INVALID;
    }
    r.ps.m = r.ps.grid.count[0] * r.ps.grid.count[1] * r.ps.grid.count[2];
    const int64_t n = gn, M = r.n_foci;
    if (r.ps.m > kMaxRequestPoints) {  // byte counts below must not wrap
        set_error_message("AFC_ServeSubmitGspat: slice has too many points");
        return AFC_ERR_TOO_LARGE;
    }
    r.out_bytes = 4 * static_cast<size_t>(r.ps.m);
    r.out2_bytes = 8 * static_cast<size_t>(n);
    r.user_out = h_slice_out;
    r.user_out2 = h_amp_phase_out;
    r.d_bytes = al256(16 * M) + al256(solver_workspace_bytes(n, M)) + al256(8 * n) + al256(48 * n) +
                al256(r.out_bytes);
    std::vector<float> in(static_cast<size_t>(4 * M));
    memcpy(in.data(), h_foci, sizeof(float) * 3 * M);
    memcpy(in.data() + 3 * M, h_amps, sizeof(float) * M);
    return e->submit(std::move(r), in.data(), sizeof(float) * 4 * M, nullptr, 0);
}

extern "C" int32_t AFC_ServeWait(void* engine, int64_t request, double* latency_s,
                                 double* queue_s) {
    Engine* e = static_cast<Engine*>(engine);
    if (!e) return AFC_ERR_INVALID;
    std::unique_lock<std::mutex> lk(e->mu);
    auto it = e->reqs.find(request);
    if (it == e->reqs.end()) {
        set_error_message("AFC_ServeWait: unknown request");
        return AFC_ERR_INVALID;
    }
    // a reference, not the iterator: submissions may rehash the map while this thread waits
    Request& r = it->second;
    e->cv_done.wait(lk, [&] { return r.state == DONE || r.state == FAILED; });
    if (latency_s) *latency_s = r.t_done - r.t_submit;
    if (queue_s) *queue_s = r.t_start - r.t_submit;
    const bool ok = r.state == DONE;
    if (!ok) set_error_message(r.error.c_str());
    e->reqs.erase(request);
    return ok ? AFC_OK : AFC_ERR_CUDA;
}

extern "C" int32_t AFC_ServeStats(void* engine, AfcServeStats* out) {
    Engine* e = static_cast<Engine*>(engine);
    if (!e || !out) return AFC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(e->mu);
    out->completed = e->completed;
    out->failed = e->failed;
    out->peak_inflight = e->peak_inflight;
    out->peak_hbm_bytes = e->dev_alloc.peak();
    out->hbm_budget_bytes = e->dev_alloc.capacity();
    out->queued = e->queue.size();
    return AFC_OK;
}

extern "C" void AFC_ServeDestroy(void* engine) { delete static_cast<Engine*>(engine); }
