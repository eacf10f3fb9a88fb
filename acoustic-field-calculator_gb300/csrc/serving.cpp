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
//     enough of the HBM budget (a first-fit device arena) are free -- requests that arrive while
//     others run join as soon as resources free up, so their work overlaps on the device --
//     then polls the slots' completion events, frees their device memory and hands finished
//     requests to a pool of completer threads that copy results to the callers' buffers.
//   * Latency = submission to the moment the scheduler sees the request's last operation (the
//     device-to-host copy of its result) complete.
#include <cuda_runtime.h>

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
#include <vector>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "afc_solvers.h"

namespace afc {
namespace serve {

// Threads that copy finished results from pinned staging to the callers' buffers (a result
// is up to a few MB; one thread alone would cap throughput at high request rates).
constexpr int kCompleters = 4;

size_t al256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

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
    int slot = -1;
    State state = QUEUED;
    std::string error;
    double t_submit = 0, t_start = 0, t_done = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    int64_t req = -1;
};

class Engine {
   public:
    int device = 0;
    char* d_arena = nullptr;
    char* h_arena = nullptr;
    RangeAllocator dev_alloc, host_alloc;
    std::vector<Slot> slots;
    std::deque<Geometry> geoms;  // a deque: references stay valid while geometries are added

    std::mutex mu;
    std::condition_variable cv_sched, cv_done, cv_host;
    std::deque<int64_t> queue;
    std::deque<int64_t> finishing;
    std::unordered_map<int64_t, Request> reqs;
    int64_t next_id = 1;
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
            if (s.done) cudaEventDestroy(s.done);
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

    // ---- work of one request on its slot's stream
    // g: the request's geometry, looked up under `mu` (a deque element stays where it is while
    // geometries are added, but the lookup itself must not race with an addition).
    cudaError_t launch(Request& r, const Geometry& g) {
        Slot& sl = slots[r.slot];
        cudaStream_t s = sl.stream;
        char* d = d_arena + r.d_off;
        char* h = h_arena + r.h_off;
        cudaError_t e;
        const int64_t n = g.n;
        if (r.kind == KIND_FIELD) {
            // device: amps|phases (8n), packed (48n), points (12m, scatter), out
            const size_t o_ap = 0, o_pk = al256(8 * n), o_pts = o_pk + al256(48 * n);
            const size_t in_pts_bytes = r.ps.is_grid ? 0 : 12 * static_cast<size_t>(r.ps.m);
            const size_t o_out = o_pts + al256(in_pts_bytes);
            if (n && (e = cudaMemcpyAsync(d + o_ap, h + r.h_in, 8 * n, cudaMemcpyHostToDevice, s)) !=
                         cudaSuccess)
                return e;
            if (in_pts_bytes &&
                (e = cudaMemcpyAsync(d + o_pts, h + r.h_in + al256(8 * n), in_pts_bytes,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return e;
            float* amps = reinterpret_cast<float*>(d + o_ap);
            auto* packed = reinterpret_cast<PackedSource*>(d + o_pk);
            if ((e = launch_repack(g.d_packed, amps, amps + n, nullptr, n, packed, s)) != cudaSuccess)
                return e;
            PointSet ps = r.ps;
            if (!ps.is_grid) ps.pts = reinterpret_cast<const float*>(d + o_pts);
            if ((e = launch_field(g.st, r.field, SUM_PLAIN, packed, n, ps, d + o_out, s)) != cudaSuccess)
                return e;
            if (r.out_bytes &&
                (e = cudaMemcpyAsync(h + r.h_out, d + o_out, r.out_bytes, cudaMemcpyDeviceToHost, s)) !=
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
            if ((e = launch_field(g.st, FIELD_PRESSURE, SUM_PLAIN, packed, n, r.ps, d + o_out, s)) !=
                cudaSuccess)
                return e;
            if (r.out_bytes &&
                (e = cudaMemcpyAsync(h + r.h_out, d + o_out, r.out_bytes, cudaMemcpyDeviceToHost, s)) !=
                    cudaSuccess)
                return e;
            if ((e = cudaMemcpyAsync(h + r.h_out2, ap, r.out2_bytes, cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess)
                return e;
        }
        return cudaEventRecord(sl.done, s);
    }

    void scheduler_loop() {
        cudaSetDevice(device);
        while (true) {
            std::vector<int64_t> to_launch;
            bool work = false;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (stop && queue.empty() && inflight == 0) break;
                // admit in arrival order while a slot and the budget allow
                while (!queue.empty()) {
                    int free_slot = -1;
                    for (size_t i = 0; i < slots.size(); ++i)
                        if (slots[i].req < 0) {
                            free_slot = static_cast<int>(i);
                            break;
                        }
                    if (free_slot < 0) break;
                    Request& r = reqs[queue.front()];
                    if (!dev_alloc.alloc(r.d_bytes, &r.d_off)) break;
                    queue.pop_front();
                    r.slot = free_slot;
                    r.state = RUNNING;
                    r.t_start = now_s();
                    slots[free_slot].req = r.id;
                    ++inflight;
                    if (inflight > peak_inflight) peak_inflight = inflight;
                    to_launch.push_back(r.id);
                }
            }
            for (int64_t id : to_launch) {
                Request* r;
                const Geometry* g;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    r = &reqs[id];
                    g = &geoms[r->geom];
                }
                const cudaError_t e = launch(*r, *g);
                if (e != cudaSuccess) {
                    std::lock_guard<std::mutex> lk(mu);
                    r->error = cudaGetErrorString(e);
                    // the slot's event was not recorded: record it now so polling can retire it
                    cudaEventRecord(slots[r->slot].done, slots[r->slot].stream);
                }
                work = true;
            }
            // retire finished slots
            for (size_t i = 0; i < slots.size(); ++i) {
                int64_t id;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    id = slots[i].req;
                }
                if (id < 0) continue;
                const cudaError_t q = cudaEventQuery(slots[i].done);
                if (q == cudaErrorNotReady) continue;
                const double t = now_s();
                std::lock_guard<std::mutex> lk(mu);
                Request& r = reqs[id];
                if (q != cudaSuccess && r.error.empty()) r.error = cudaGetErrorString(q);
                r.t_done = t;
                dev_alloc.release(r.d_off, r.d_bytes);
                slots[i].req = -1;
                --inflight;
                r.state = FINISHING;
                finishing.push_back(id);
                work = true;
            }
            if (work) {
                cv_host.notify_all();
            } else {
                std::unique_lock<std::mutex> lk(mu);
                cv_sched.wait_for(lk, std::chrono::microseconds(inflight > 0 ? 10 : 500));
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
    e->slots.resize(static_cast<size_t>(cfg->max_inflight));
    for (Slot& s : e->slots) {
        if ((ce = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (ce = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming)) != cudaSuccess) {
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
    int64_t gn = -1;  // the geometry's source count, read under the lock AddGeometry takes
    if (e && geometry >= 0) {
        std::lock_guard<std::mutex> lk(e->mu);
        if (geometry < static_cast<int32_t>(e->geoms.size())) gn = e->geoms[geometry].n;
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
    r.d_bytes = al256(8 * n) + al256(48 * n) + al256(pts_bytes) + al256(r.out_bytes);
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
    int64_t gn = -1;  // the geometry's source count, read under the lock AddGeometry takes
    if (e && geometry >= 0) {
        std::lock_guard<std::mutex> lk(e->mu);
        if (geometry < static_cast<int32_t>(e->geoms.size())) gn = e->geoms[geometry].n;
    }
    if (!e || gn < 0 || n_foci == 0 || !h_foci || !h_amps || !h_slice_out ||
        n_foci > static_cast<uint64_t>(kSolverMaxFoci)) {
        set_error_message("AFC_ServeSubmitGspat: invalid argument");
        return AFC_ERR_INVALID;
    }
    Request r;
    r.kind = KIND_GSPAT;
    r.geom = geometry;
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
