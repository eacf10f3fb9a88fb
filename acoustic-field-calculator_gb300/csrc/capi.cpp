// C-ABI host layer of libafccapi.so: the handle objects of the reference's `afccapi`
// (capi/src/*.rs) re-implemented in C++, with every calculation dispatched to the CUDA
// kernels of this library.  There is no CPU compute path: without a CUDA device the
// calculation calls fail and record an error.
//
// Host-side f32 arithmetic (sound speed, k, alpha, grid counts, focal law) must round like
// the reference's Rust, which never fuses multiply-adds: this file is compiled with
// -ffp-contract=off.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "afc_gpu.h"
#include "afc_internal.h"
#include "afc_solvers.h"
#include "afccapi.h"

using namespace afc;

namespace {

// ------------------------------------------------------------------ errors

thread_local std::string t_last_error;

void set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
}

int32_t cuda_fail(cudaError_t e, const char* what) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return AFC_ERR_CUDA;
}

// ------------------------------------------------------------------ float formatting

// Rust's `{}` for f32: the shortest decimal that reads back as the same f32, written without
// an exponent (used by the info strings of system/uniform_medium.rs:73-90).
std::string rust_fmt_f32(float v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    if (v == 0.0f) return std::signbit(v) ? "-0" : "0";
    char buf[64];
    int prec = 1;
    for (; prec <= 9; ++prec) {
        snprintf(buf, sizeof(buf), "%.*e", prec - 1, static_cast<double>(v));
        if (strtof(buf, nullptr) == v) break;
    }
    // buf = [-]d.ddde[+-]xx
    std::string s(buf);
    bool neg = s[0] == '-';
    if (neg) s = s.substr(1);
    size_t epos = s.find('e');
    int exp10 = atoi(s.c_str() + epos + 1);
    std::string digits;
    for (size_t i = 0; i < epos; ++i)
        if (s[i] != '.') digits += s[i];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    std::string out;
    int point = exp10 + 1;  // digits before the decimal point
    if (point <= 0) {
        out = "0." + std::string(static_cast<size_t>(-point), '0') + digits;
    } else if (static_cast<size_t>(point) >= digits.size()) {
        out = digits + std::string(static_cast<size_t>(point) - digits.size(), '0');
    } else {
        out = digits.substr(0, static_cast<size_t>(point)) + "." +
              digits.substr(static_cast<size_t>(point));
    }
    return neg ? "-" + out : out;
}

// ------------------------------------------------------------------ physics set-up

constexpr float kPiF = 3.14159265358979323846f;  // std::f32::consts::PI

// core/sound_speed.rs:22-24 [mm/s]
float sound_speed(float t) { return 331.3f * sqrtf(t / 273.15f) * 1000.0f; }

// core/attenuation.rs:31-48, Np/mm
float attenuation_coef(float freq, float hr, float ps, float ps0, float t) {
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

// ------------------------------------------------------------------ handles

enum : uint32_t {
    MAGIC_SYSTEM = 0x41464353u,
    MAGIC_SCATTER = 0x41464341u,
    MAGIC_GRID = 0x41464347u,
    MAGIC_FIELD = 0x41464346u,
    MAGIC_CALC = 0x4146434Bu,
    MAGIC_DEAD = 0xDEADDEADu
};

// Systems get process-wide unique ids, so that a calculator's packed copy of one system's
// sources is never taken for another system created later at the same address.
std::atomic<uint64_t> g_system_uid{0};

// UniformSystem (system/uniform_medium.rs:21-27): AoS sources in the ABI layout plus SoA
// wavenumbers and attenuations.  `generation` counts the changes the library knows of (its own
// writes, handed-out pointers, announced edits); with `track` on, a calculator reuses its
// device copy of the sources while (uid, generation) are those it packed.
struct System {
    uint32_t magic = MAGIC_SYSTEM;
    int st;
    float temperature;
    float c;  // sound speed [mm/s]
    std::vector<float> src;
    std::vector<float> k, atten;
    std::string info, src_info;
    uint64_t uid = g_system_uid.fetch_add(1) + 1;
    uint64_t generation = 0;
    bool track = false;
    size_t count() const { return k.size(); }
};

// Scatter-area versions come from one process-wide counter, so that a (handle, version) pair
// never repeats: an area freed and another created at the same address get different
// versions, and a calculator's cached device copy of the old points is not reused.
std::atomic<uint64_t> g_scatter_version{0};
uint64_t next_scatter_version() { return g_scatter_version.fetch_add(1) + 1; }

struct Scatter {
    uint32_t magic = MAGIC_SCATTER;
    std::vector<float> pts;
    uint64_t version = next_scatter_version();  // renewed on every added point
};

struct Grid {
    uint32_t magic = MAGIC_GRID;
    int dim;
    int axes[3];   // axis codes 1..3 in specification order
    float lo[3];   // per axis x, y, z
    float hi[3];
    float res;
    uint64_t n[3];  // per axis x, y, z
    uint64_t points() const { return n[0] * n[1] * n[2]; }
};

struct Field {
    uint32_t magic = MAGIC_FIELD;
    int type;
    void* host = nullptr;  // pinned
    size_t cap = 0;
    uint64_t len = 0;
};

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct PinnedBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Per-calculator GPU state: a stream and grow-only buffers.  Scatter points stay resident
// while the same area handle at the same version is calculated again.
struct GpuCtx {
    int device = -1;
    cudaStream_t stream = nullptr;
    DevBuf src;     // raw sources | k | atten
    DevBuf packed;  // PackedSource[n]
    DevBuf pts;
    const void* pts_owner = nullptr;
    uint64_t pts_version = ~0ull;
    DevBuf out;
    PinnedBuf staging;
    // the system whose sources `packed` holds, at which generation (uid 0: none)
    uint64_t packed_uid = 0, packed_gen = 0;
    int64_t packed_n = -1;
    std::mutex mu;

    int32_t init() {
        if (stream) return AFC_OK;
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            set_error("no CUDA device available (%s); this library has no CPU path",
                      e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
            return AFC_ERR_NO_DEVICE;
        }
        e = cudaGetDevice(&device);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
        e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            stream = nullptr;
            return cuda_fail(e, "cudaStreamCreate");
        }
        return AFC_OK;
    }
    ~GpuCtx() {
        if (stream) {
            cudaStreamSynchronize(stream);
            src.release();
            packed.release();
            pts.release();
            out.release();
            staging.release();
            cudaStreamDestroy(stream);
        }
    }
};

struct Calculator {
    uint32_t magic = MAGIC_CALC;
    int type;
    GpuCtx gpu;
};

template <class T>
T* as(void* h, uint32_t magic, const char* what) {
    T* p = static_cast<T*>(h);
    if (!p || p->magic != magic) {
        set_error("invalid %s handle", what);
        return nullptr;
    }
    return p;
}

System* as_system(void* h, int st) {
    System* s = as<System>(h, MAGIC_SYSTEM, "system");
    if (s && s->st != st) {
        set_error("source type %d does not match the system (%d)", st, s->st);
        return nullptr;
    }
    return s;
}

// A system about to have its sources written (by this library, or through a pointer it hands
// out): its generation moves on, so no calculator reuses a copy packed before.
System* as_system_for_write(void* h, int st) {
    System* s = as_system(h, st);
    if (s) ++s->generation;
    return s;
}

bool valid_source_type(int st) { return st == SRC_SPHERE || st == SRC_T4010A1; }
bool valid_field_type(int f) { return f >= FIELD_PRESSURE && f <= FIELD_COMPLEX; }

// Rust `f as usize` for f32: NaN and negatives give 0.
uint64_t f32_as_usize(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 18446744073709551616.0f) return UINT64_MAX;
    return static_cast<uint64_t>(v);
}

// GridAreaBuilder::generate (observe_area/grid/builder.rs:144-209).
void* make_grid(int dim, const float first[2], const float second[2], const float third[2],
                float res, int a1, int a2, int a3) {
    const int axes[3] = {a1, a2, a3};
    bool seen[4] = {false, false, false, false};
    for (int a : axes) {
        if (a < 1 || a > 3 || seen[a]) {
            set_error("invalid axis combination (%d, %d, %d)", a1, a2, a3);
            return nullptr;
        }
        seen[a] = true;
    }
    Grid* g = new (std::nothrow) Grid;
    if (!g) {
        set_error("out of host memory");
        return nullptr;
    }
    g->dim = dim;
    g->res = res;
    const float* ranges[3] = {first, second, third};
    for (int k = 0; k < 3; ++k) {
        g->axes[k] = axes[k];
        g->lo[axes[k] - 1] = ranges[k][0];
        g->hi[axes[k] - 1] = ranges[k][1];
    }
    for (int a = 0; a < 3; ++a) g->n[a] = f32_as_usize((g->hi[a] - g->lo[a]) / res) + 1;
    return g;
}

// Points of a grid with per-axis counts c[0..2], false when the product does not fit in 62 bits
// (counts that large come only from a zero-like resolution or a wrapped count, and would
// otherwise be computed as a wrapped, meaningless size).
bool grid_points_checked(const uint64_t c[3], uint64_t* out) {
    unsigned __int128 p = 1;
    for (int k = 0; k < 3; ++k) {
        p *= c[k];
        if (p > (static_cast<unsigned __int128>(1) << 62)) return false;
    }
    *out = static_cast<uint64_t>(p);
    return true;
}

GridDev grid_dev(const Grid& g) {
    GridDev d;
    for (int k = 0; k < 3; ++k) {
        const int a = g.axes[k] - 1;
        d.axis[k] = a;
        d.count[k] = static_cast<int64_t>(k < g.dim ? g.n[a] : 1);
        d.origin[k] = g.lo[k];
    }
    d.res = g.res;
    return d;
}

int field_type_of(const Field* f) { return f->type; }

// Run one calculation on the calculator's stream: upload sources (and scatter points when they
// changed), pack, launch the field kernel, copy the result into the field's pinned buffer.
int32_t gpu_calculate(Calculator* calc, System* sys, void* area, int area_type, Field* field,
                      int sum_mode, uint64_t* out_len) {
    GpuCtx& g = calc->gpu;
    std::lock_guard<std::mutex> lock(g.mu);
    int32_t rc = g.init();
    if (rc != AFC_OK) return rc;
    DeviceGuard dg;  // the calculator's device while it runs; the caller's again on return
    cudaError_t e = dg.set(g.device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");

    PointSet ps{};
    if (area_type == AREA_SCATTER) {
        Scatter* sc = static_cast<Scatter*>(area);
        ps.is_grid = false;
        ps.m = static_cast<int64_t>(sc->pts.size() / 3);
        if (ps.m > 0 && (g.pts_owner != sc || g.pts_version != sc->version)) {
            const size_t bytes = sc->pts.size() * sizeof(float);
            if ((e = g.pts.ensure(bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(points)");
            if ((e = cudaMemcpyAsync(g.pts.p, sc->pts.data(), bytes, cudaMemcpyHostToDevice,
                                     g.stream)) != cudaSuccess)
                return cuda_fail(e, "cudaMemcpyAsync(points)");
            g.pts_owner = sc;
            g.pts_version = sc->version;
        }
        ps.pts = static_cast<const float*>(g.pts.p);
    } else {
        Grid* gr = static_cast<Grid*>(area);
        ps.is_grid = true;
        ps.grid = grid_dev(*gr);
        ps.m = static_cast<int64_t>(ps.grid.count[0] * ps.grid.count[1] * ps.grid.count[2]);
    }

    const int ft = field_type_of(field);
    const size_t out_bytes = static_cast<size_t>(ps.m) * field_elem_bytes(ft);
    {
        PinnedBuf hb{field->host, field->cap};
        if ((e = hb.ensure(out_bytes)) != cudaSuccess) return cuda_fail(e, "cudaHostAlloc(field)");
        field->host = hb.p;
        field->cap = hb.cap;
    }
    field->len = static_cast<uint64_t>(ps.m);
    if (ps.m == 0) {
        *out_len = 0;
        return AFC_OK;
    }

    const int64_t n = static_cast<int64_t>(sys->count());
    const int stride = source_stride(sys->st);
    const size_t raw_floats = static_cast<size_t>(n) * (stride + 2);
    // opted-in systems whose sources have not changed since this calculator packed them
    const bool reuse = sys->track && g.packed_uid == sys->uid && g.packed_gen == sys->generation &&
                       g.packed_n == n;
    g.packed_uid = 0;  // set again below once the packed copy is complete
    if (n > 0 && !reuse) {
        if ((e = g.staging.ensure(raw_floats * sizeof(float))) != cudaSuccess)
            return cuda_fail(e, "cudaHostAlloc(staging)");
        float* st = static_cast<float*>(g.staging.p);
        memcpy(st, sys->src.data(), sizeof(float) * n * stride);
        memcpy(st + n * stride, sys->k.data(), sizeof(float) * n);
        memcpy(st + n * (stride + 1), sys->atten.data(), sizeof(float) * n);
        if ((e = g.src.ensure(raw_floats * sizeof(float))) != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(sources)");
        if ((e = g.packed.ensure(sizeof(PackedSource) * n)) != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(packed)");
        if ((e = cudaMemcpyAsync(g.src.p, st, raw_floats * sizeof(float), cudaMemcpyHostToDevice,
                                 g.stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(sources)");
        const float* d = static_cast<const float*>(g.src.p);
        if ((e = launch_pack_sources(sys->st, d, d + n * stride, d + n * (stride + 1), n,
                                     static_cast<PackedSource*>(g.packed.p), g.stream)) !=
            cudaSuccess)
            return cuda_fail(e, "pack_sources");
    }
    // The kernels write the field straight into the pinned host buffer when the device can
    // address it (under unified addressing every cudaHostAlloc buffer is, at its host address):
    // no device-to-host copy after the launch.  Otherwise into device memory, then copied.
    void* dst = nullptr;
    const bool to_host = cudaHostGetDevicePointer(&dst, field->host, 0) == cudaSuccess && dst;
    if (!to_host) {
        (void)cudaGetLastError();
        if ((e = g.out.ensure(out_bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(field)");
        dst = g.out.p;
    }
    if ((e = launch_field(sys->st, ft, sum_mode, static_cast<const PackedSource*>(g.packed.p), n,
                          ps, dst, g.stream)) != cudaSuccess)
        return cuda_fail(e, "field kernel launch");
    if (!to_host &&
        (e = cudaMemcpyAsync(field->host, g.out.p, out_bytes, cudaMemcpyDeviceToHost, g.stream)) !=
            cudaSuccess)
        return cuda_fail(e, "cudaMemcpyAsync(field)");
    if ((e = cudaStreamSynchronize(g.stream)) != cudaSuccess)
        return cuda_fail(e, "field calculation");
    if (sys->track) {
        g.packed_uid = sys->uid;
        g.packed_gen = sys->generation;
        g.packed_n = n;
    }
    *out_len = static_cast<uint64_t>(ps.m);
    return AFC_OK;
}

void add_source(void* handle, int st, const float* rec, bool explicit_ka, float k, float a) {
    System* s = as_system_for_write(handle, st);
    if (!s) return;
    const int stride = source_stride(st);
    const float freq = rec[stride - 1];
    if (!explicit_ka) {
        // uniform_medium.rs:102-107
        const float c = sound_speed(s->temperature);
        k = 2.0f * kPiF * freq / c;
        a = attenuation_coef(freq, 30.f, 1.f, 1.f, s->temperature);
    }
    s->src.insert(s->src.end(), rec, rec + stride);
    s->k.push_back(k);
    s->atten.push_back(a);
}

// foci / amps of the multi-focus optimizers (capi/src/optimizer.rs:79-95).
bool unpack_foci(const void* foci, const float* amps, uint64_t size, std::vector<float>& f,
                 std::vector<float>& a) {
    if (size > 0 && (!foci || !amps)) {
        set_error("foci or amps is NULL");
        return false;
    }
    const float* fp = static_cast<const float*>(foci);
    f.assign(fp, fp + 3 * size);
    a.assign(amps, amps + size);
    return true;
}

void run_solver(int kind, void* handle, const void* foci, const float* amps, uint64_t size,
                int32_t st, int phase_div = 0) {
    if (!valid_source_type(st)) {
        set_error("unknown source type %d", st);
        return;
    }
    System* s = as_system_for_write(handle, st);
    if (!s) return;
    std::vector<float> f, a;
    if (!unpack_foci(foci, amps, size, f, a)) return;
    std::string err;
    const int rc = solve_multi_focus(kind, st, s->src.data(), s->k.data(), s->atten.data(),
                                     static_cast<int64_t>(s->count()), f.data(), a.data(),
                                     static_cast<int64_t>(size), &err, phase_div);
    if (rc != 0) set_error("%s", err.c_str());
}

void run_nls(int kind, void* handle, const void* foci, const float* amps, uint64_t size,
             int32_t st) {
    if (!valid_source_type(st)) {
        set_error("unknown source type %d", st);
        return;
    }
    System* s = as_system_for_write(handle, st);
    if (!s) return;
    std::vector<float> f, a;
    if (!unpack_foci(foci, amps, size, f, a)) return;
    std::string err;
    const int rc = solve_nls(kind, st, s->src.data(), s->k.data(), s->atten.data(),
                             static_cast<int64_t>(s->count()), f.data(), a.data(),
                             static_cast<int64_t>(size), &err);
    if (rc != 0) set_error("%s", err.c_str());
}

void run_matrix(int kind, void* handle, const void* foci, const float* amps, uint64_t size,
                int32_t st) {
    if (!valid_source_type(st)) {
        set_error("unknown source type %d", st);
        return;
    }
    System* s = as_system_for_write(handle, st);
    if (!s) return;
    std::vector<float> f, a;
    if (!unpack_foci(foci, amps, size, f, a)) return;
    std::string err;
    const int rc = solve_matrix(kind, st, s->src.data(), s->k.data(), s->atten.data(),
                                static_cast<int64_t>(s->count()), f.data(), a.data(),
                                static_cast<int64_t>(size), &err);
    if (rc != 0) set_error("%s", err.c_str());
}

void unsupported(const char* name) {
    set_error("%s: this solver is not provided by the GB300 library (system left unchanged)",
              name);
}

std::mutex g_dev_mu;

int32_t check_field_args(int32_t st, int32_t ft, int32_t sum, uint64_t n, const void* d_sources,
                         const void* d_k, const void* d_a, void* d_out, void* ws, size_t ws_bytes) {
    if (!valid_source_type(st) || !valid_field_type(ft) ||
        (sum != AFC_SUM_PLAIN && sum != AFC_SUM_COMPENSATED)) {
        set_error("invalid source/field/sum tag (%d, %d, %d)", st, ft, sum);
        return AFC_ERR_INVALID;
    }
    if (n >= (1ull << 40)) {
        set_error("too many sources (at most 2^40 per call)");
        return AFC_ERR_TOO_LARGE;
    }
    if (n > 0 && (!d_sources || !d_k || !d_a)) {
        set_error("source pointers are NULL");
        return AFC_ERR_INVALID;
    }
    if (!d_out) {
        set_error("output pointer is NULL");
        return AFC_ERR_INVALID;
    }
    if (n > 0 && (!ws || ws_bytes < AFC_FieldWorkspaceBytes(n) ||
                  (reinterpret_cast<uintptr_t>(ws) & 15u) != 0)) {
        set_error("workspace must be 16-byte aligned and at least %zu bytes",
                  AFC_FieldWorkspaceBytes(n));
        return AFC_ERR_INVALID;
    }
    return AFC_OK;
}

int32_t device_field(int32_t st, int32_t ft, int32_t sum, const float* d_sources,
                     const float* d_k, const float* d_a, uint64_t n, const PointSet& ps,
                     void* d_out, void* ws, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    // launch on the stream's device whatever device this thread last selected, and leave the
    // caller's current device as it was
    DeviceGuard dg;
    int sdev = -1;
    if ((e = stream_device(s, &sdev)) != cudaSuccess) return cuda_fail(e, "cudaStreamGetDevice");
    if ((e = dg.set(sdev)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    if (n > 0) {
        e = launch_pack_sources(st, d_sources, d_k, d_a, static_cast<int64_t>(n),
                                static_cast<PackedSource*>(ws), s);
        if (e != cudaSuccess) return cuda_fail(e, "pack_sources");
    }
    e = launch_field(st, ft, sum, static_cast<const PackedSource*>(ws), static_cast<int64_t>(n),
                     ps, d_out, s);
    if (e != cudaSuccess) return cuda_fail(e, "field kernel launch");
    return AFC_OK;
}

}  // namespace

void afc::set_error_message(const char* msg) { t_last_error = msg ? msg : ""; }

extern "C" {

// ------------------------------------------------------------------ errors

const char* AFC_GetLastError(void) { return t_last_error.c_str(); }
void AFC_ClearLastError(void) { t_last_error.clear(); }

// ------------------------------------------------------------------ calculators

void AFC_CreateCalculator(void** out, int32_t calc_type) {
    if (!out) return;
    *out = nullptr;
    if (calc_type < CALC_CPU || calc_type > CALC_GPU) {
        set_error("unknown calculator type %d", calc_type);
        return;
    }
    Calculator* c = new (std::nothrow) Calculator;
    if (!c) {
        set_error("out of host memory");
        return;
    }
    c->type = calc_type;
    *out = c;
}

void AFC_FreeCalculator(void* handle, int32_t calc_type) {
    Calculator* c = as<Calculator>(handle, MAGIC_CALC, "calculator");
    if (!c) return;
    if (c->type != calc_type) {
        set_error("calculator type %d does not match the handle (%d)", calc_type, c->type);
        return;
    }
    c->magic = MAGIC_DEAD;
    delete c;
}

uint64_t AFC_Calculate(void* calc_handle, void* system_handle, void* obs_handle,
                       void* field_handle, const void** out, int32_t calc_type,
                       int32_t source_type, int32_t obs_type, int32_t field_type) {
    if (out) *out = nullptr;
    if (!out) {
        set_error("out is NULL");
        return 0;
    }
    Calculator* calc = as<Calculator>(calc_handle, MAGIC_CALC, "calculator");
    if (!calc) return 0;
    if (calc->type != calc_type) {
        set_error("calculator type %d does not match the handle (%d)", calc_type, calc->type);
        return 0;
    }
    if (!valid_source_type(source_type)) {
        set_error("unknown source type %d", source_type);
        return 0;
    }
    System* sys = as_system(system_handle, source_type);
    if (!sys) return 0;
    void* area = nullptr;
    if (obs_type == AREA_SCATTER) {
        area = as<Scatter>(obs_handle, MAGIC_SCATTER, "scatter area");
    } else if (obs_type >= AREA_GRID1D && obs_type <= AREA_GRID3D) {
        Grid* g = as<Grid>(obs_handle, MAGIC_GRID, "grid area");
        if (g && g->dim != obs_type + 1) {
            set_error("area type %d does not match the %dD grid handle", obs_type, g->dim);
            g = nullptr;
        }
        if (g) {
            const GridDev d = grid_dev(*g);
            const uint64_t c[3] = {static_cast<uint64_t>(d.count[0]),
                                   static_cast<uint64_t>(d.count[1]),
                                   static_cast<uint64_t>(d.count[2])};
            uint64_t total = 0;
            if (!grid_points_checked(c, &total)) {
                set_error("grid has too many points (%llu x %llu x %llu)",
                          static_cast<unsigned long long>(c[0]),
                          static_cast<unsigned long long>(c[1]),
                          static_cast<unsigned long long>(c[2]));
                g = nullptr;
            }
        }
        area = g;
    } else {
        set_error("unknown observe area type %d", obs_type);
        return 0;
    }
    if (!area) return 0;
    if (!valid_field_type(field_type)) {
        set_error("unknown field type %d", field_type);
        return 0;
    }
    Field* field = as<Field>(field_handle, MAGIC_FIELD, "field buffer");
    if (!field) return 0;
    if (field->type != field_type) {
        set_error("field type %d does not match the buffer (%d)", field_type, field->type);
        return 0;
    }
    const int sum = calc_type == CALC_ACCURATE ? SUM_COMPENSATED : SUM_PLAIN;
    uint64_t len = 0;
    if (gpu_calculate(calc, sys, area, obs_type, field, sum, &len) != AFC_OK) return 0;
    *out = field->host;
    return len;
}

// ------------------------------------------------------------------ systems

void AFC_CreateUniformSystem(void** out, float temperature, int32_t source_type) {
    if (!out) return;
    *out = nullptr;
    if (!valid_source_type(source_type)) {
        set_error("unknown source type %d", source_type);
        return;
    }
    System* s = new (std::nothrow) System;
    if (!s) {
        set_error("out of host memory");
        return;
    }
    s->st = source_type;
    s->temperature = temperature;
    s->c = sound_speed(temperature);
    *out = s;
}

void AFC_FreeUniformSystem(void* handle, int32_t source_type) {
    System* s = as_system(handle, source_type);
    if (!s) return;
    s->magic = MAGIC_DEAD;
    delete s;
}

float AFC_UniformSystemSoundSpeed(void* handle, int32_t source_type) {
    System* s = as_system(handle, source_type);
    return s ? s->c : NAN;
}

char* AFC_UniformSystemInfo(void* handle, int32_t source_type) {
    System* s = as_system(handle, source_type);
    if (!s) return nullptr;
    // uniform_medium.rs:73-80
    s->info = "Uniform Medium:\n Temperature: " + rust_fmt_f32(s->temperature) + " K = " +
              rust_fmt_f32(s->temperature - 273.15f) + " ℃\n Sound Speed: " +
              rust_fmt_f32(sound_speed(s->temperature)) + " mm/s";
    return &s->info[0];
}

char* AFC_UniformSystemSourceInfo(void* handle, uint64_t idx, int32_t source_type) {
    System* s = as_system(handle, source_type);
    if (!s) return nullptr;
    if (idx >= s->count()) {
        set_error("source index %llu out of range (%zu sources)",
                  static_cast<unsigned long long>(idx), s->count());
        return nullptr;
    }
    // uniform_medium.rs:82-90
    const float k = s->k[idx];
    s->src_info = std::to_string(idx) + "-th wave source:\n Wavelength: " +
                  rust_fmt_f32(2.0f * kPiF / k) + " mm\n Wavenumber: " + rust_fmt_f32(k) +
                  " mm^-1\n Attenuation: " + rust_fmt_f32(s->atten[idx]) + " Np/mm";
    return &s->src_info[0];
}

void AFC_AddSphereWaveSource(void* handle, AfcSphereWaveSource source) {
    add_source(handle, SRC_SPHERE, &source.x, false, 0.f, 0.f);
}

void AFC_AddT4010A1(void* handle, AfcT4010A1 source) {
    add_source(handle, SRC_T4010A1, &source.x, false, 0.f, 0.f);
}

void AFC_AddSphereWaveSourceWithWavenumAtten(void* handle, AfcSphereWaveSource source,
                                            float wavenum, float atten) {
    add_source(handle, SRC_SPHERE, &source.x, true, wavenum, atten);
}

void AFC_AddT4010A1WithWavenumAtten(void* handle, AfcT4010A1 source, float wavenum,
                                    float atten) {
    add_source(handle, SRC_T4010A1, &source.x, true, wavenum, atten);
}

uint64_t AFC_GetWaveSources(void* handle, void** out, int32_t source_type) {
    if (out) *out = nullptr;
    if (!out) return 0;
    // the caller may write through the pointer: the next calculation uploads the sources again
    System* s = as_system_for_write(handle, source_type);
    if (!s) return 0;
    *out = s->src.data();
    return s->count();
}

int32_t AFC_UniformSystemTrackSources(void* handle, int32_t source_type, int32_t enable) {
    System* s = as_system_for_write(handle, source_type);
    if (!s) return AFC_ERR_INVALID;
    s->track = enable != 0;
    return AFC_OK;
}

int32_t AFC_UniformSystemSourcesChanged(void* handle, int32_t source_type) {
    return as_system_for_write(handle, source_type) ? AFC_OK : AFC_ERR_INVALID;
}

// ------------------------------------------------------------------ areas

void AFC_CreateScatterArea(void** out) {
    if (!out) return;
    *out = new (std::nothrow) Scatter;
    if (!*out) set_error("out of host memory");
}

void AFC_ScatterAddObservePoint(void* handle, AfcVector3 p) {
    Scatter* s = as<Scatter>(handle, MAGIC_SCATTER, "scatter area");
    if (!s) return;
    s->pts.push_back(p.x);
    s->pts.push_back(p.y);
    s->pts.push_back(p.z);
    s->version = next_scatter_version();
}

void AFC_FreeScatterArea(void* handle) {
    Scatter* s = as<Scatter>(handle, MAGIC_SCATTER, "scatter area");
    if (!s) return;
    s->magic = MAGIC_DEAD;
    delete s;
}

void AFC_CreateGridArea1D(void** out, float first_start, float first_end, float second,
                          float third, float resolution, int32_t first_axis,
                          int32_t second_axis, int32_t third_axis) {
    if (!out) return;
    const float f[2] = {first_start, first_end}, s[2] = {second, second}, t[2] = {third, third};
    *out = make_grid(1, f, s, t, resolution, first_axis, second_axis, third_axis);
}

void AFC_CreateGridArea2D(void** out, float first_start, float first_end, float second_start,
                          float second_end, float third, float resolution, int32_t first_axis,
                          int32_t second_axis, int32_t third_axis) {
    if (!out) return;
    const float f[2] = {first_start, first_end}, s[2] = {second_start, second_end},
                t[2] = {third, third};
    *out = make_grid(2, f, s, t, resolution, first_axis, second_axis, third_axis);
}

void AFC_CreateGridArea3D(void** out, float first_start, float first_end, float second_start,
                          float second_end, float third_start, float third_end,
                          float resolution, int32_t first_axis, int32_t second_axis,
                          int32_t third_axis) {
    if (!out) return;
    const float f[2] = {first_start, first_end}, s[2] = {second_start, second_end},
                t[2] = {third_start, third_end};
    *out = make_grid(3, f, s, t, resolution, first_axis, second_axis, third_axis);
}

void AFC_FreeGridArea(void* handle, int32_t dimension) {
    Grid* g = as<Grid>(handle, MAGIC_GRID, "grid area");
    if (!g) return;
    if (g->dim != dimension) {
        set_error("dimension %d does not match the %dD grid handle", dimension, g->dim);
        return;
    }
    g->magic = MAGIC_DEAD;
    delete g;
}

void AFC_GetGridSize(void* handle, int32_t dimension, uint32_t* first, uint32_t* second,
                     uint32_t* third) {
    Grid* g = as<Grid>(handle, MAGIC_GRID, "grid area");
    if (!g || !first || !second || !third) return;
    if (g->dim != dimension) {
        set_error("dimension %d does not match the %dD grid handle", dimension, g->dim);
        return;
    }
    *first = static_cast<uint32_t>(g->n[0]);
    *second = static_cast<uint32_t>(g->n[1]);
    *third = static_cast<uint32_t>(g->n[2]);
}

// ------------------------------------------------------------------ field buffers

#define AFC_FIELD_EXPORTS(CREATE, FREE, TYPE)                          \
    void CREATE(void** out) {                                          \
        if (!out) return;                                              \
        Field* f = new (std::nothrow) Field;                           \
        if (!f) {                                                      \
            set_error("out of host memory");                           \
            *out = nullptr;                                            \
            return;                                                    \
        }                                                              \
        f->type = TYPE;                                                \
        *out = f;                                                      \
    }                                                                  \
    void FREE(void* handle) {                                          \
        Field* f = as<Field>(handle, MAGIC_FIELD, "field buffer");     \
        if (!f) return;                                                \
        if (f->host) cudaFreeHost(f->host);                            \
        f->magic = MAGIC_DEAD;                                         \
        delete f;                                                      \
    }

AFC_FIELD_EXPORTS(AFC_CreatePressureField, AFC_FreePressureField, FIELD_PRESSURE)
AFC_FIELD_EXPORTS(AFC_CreatePowerField, AFC_FreePowerField, FIELD_POWER)
AFC_FIELD_EXPORTS(AFC_CreateComplexPressureField, AFC_FreeComplexPressureField, FIELD_COMPLEX)

// ------------------------------------------------------------------ optimizers

void AFO_FocalPoint(void* handle, AfcVector3 point, int32_t source_type) {
    if (!valid_source_type(source_type)) {
        set_error("unknown source type %d", source_type);
        return;
    }
    System* s = as_system_for_write(handle, source_type);
    if (!s) return;
    // focal_point.rs:28-39
    const int stride = source_stride(source_type);
    const int iphase = source_type == SRC_T4010A1 ? 7 : 4;
    for (size_t j = 0; j < s->count(); ++j) {
        float* r = s->src.data() + stride * j;
        const float dx = r[0] - point.x, dy = r[1] - point.y, dz = r[2] - point.z;
        const float d = sqrtf(dx * dx + dy * dy + dz * dz);
        const float wave_length = s->c / r[stride - 1];
        float phase = fmodf(d, wave_length) / wave_length;
        phase = -2.0f * kPiF * phase;
        r[iphase] = phase;
    }
}

void AFO_GSPAT(void* handle, const void* foci, const float* amps, uint64_t size,
               int32_t source_type) {
    run_solver(SOLVER_GSPAT, handle, foci, amps, size, source_type);
}

void AFO_GS(void* handle, const void* foci, const float* amps, uint64_t size,
            int32_t source_type) {
    run_solver(SOLVER_GS, handle, foci, amps, size, source_type);
}

void AFO_Naive(void* handle, const void* foci, const float* amps, uint64_t size,
               int32_t source_type) {
    run_solver(SOLVER_NAIVE, handle, foci, amps, size, source_type);
}

// bessel.rs:30-51 (Hasegawa et al. 2017): each source's phase from its offset to `point`,
// rotated by asin|v| about v = (dir.y, -dir.x, 0) (Rodrigues' formula with nalgebra's cross
// and dot orders), on a cone of half-angle theta: f32 host arithmetic, O(n) set-up.
void AFO_BesselBeam(void* handle, AfcVector3 point, AfcVector3 dir, float theta,
                    int32_t source_type) {
    if (!valid_source_type(source_type)) {
        set_error("unknown source type %d", source_type);
        return;
    }
    System* s = as_system_for_write(handle, source_type);
    if (!s) return;
    const float vx = dir.y, vy = -dir.x, vz = 0.0f;
    const float theta_w = asinf(sqrtf(vx * vx + vy * vy + vz * vz));
    const float cw = cosf(theta_w), sw = sinf(theta_w), omc = 1.0f - cosf(theta_w);
    const float st = sinf(theta), ct = cosf(theta);
    const int stride = source_stride(source_type);
    const int iphase = source_type == SRC_T4010A1 ? 7 : 4;
    for (size_t j = 0; j < s->count(); ++j) {
        float* rec = s->src.data() + stride * j;
        const float rx = rec[0] - point.x, ry = rec[1] - point.y, rz = rec[2] - point.z;
        // xr = r x v
        const float xx = ry * vz - rz * vy, xy = rz * vx - rx * vz, xz = rx * vy - ry * vx;
        const float vd = (vx * rx + vy * ry) + vz * rz;
        const float f = vd * omc;
        const float qx = (rx * cw + xx * sw) + vx * f;
        const float qy = (ry * cw + xy * sw) + vy * f;
        const float qz = (rz * cw + xz * sw) + vz * f;
        const float dist = st * sqrtf(qx * qx + qy * qy) - ct * qz;
        const float wave_length = s->c / rec[stride - 1];
        float phase = fmodf(dist, wave_length) / wave_length;
        phase = -2.0f * kPiF * phase;
        rec[iphase] = phase;
    }
}
void AFO_IFFT(void*, const char*, AfcVector3, AfcVector3, AfcVector3, float, float, int32_t) {
    unsupported("AFO_IFFT");
}
void AFO_Horn(void* handle, const void* foci, const float* amps, uint64_t size,
              int32_t source_type) {
    run_matrix(MATRIX_HORN, handle, foci, amps, size, source_type);
}
void AFO_Long(void* handle, const void* foci, const float* amps, uint64_t size,
              int32_t source_type) {
    run_matrix(MATRIX_LONG, handle, foci, amps, size, source_type);
}
void AFO_APO(void* handle, const void* foci, const float* amps, uint64_t size, float lambda,
             int32_t source_type) {
    if (!valid_source_type(source_type)) {
        set_error("unknown source type %d", source_type);
        return;
    }
    System* s = as_system_for_write(handle, source_type);
    if (!s) return;
    std::vector<float> f, a;
    if (!unpack_foci(foci, amps, size, f, a)) return;
    std::string err;
    const int rc = solve_apo(source_type, s->src.data(), s->k.data(), s->atten.data(),
                             static_cast<int64_t>(s->count()), f.data(), a.data(),
                             static_cast<int64_t>(size), lambda, &err);
    if (rc != 0) set_error("%s", err.c_str());
}
void AFO_GaussNewton(void* handle, const void* foci, const float* amps, uint64_t size,
                     int32_t source_type) {
    run_nls(NLS_GAUSS_NEWTON, handle, foci, amps, size, source_type);
}
void AFO_GradientDescent(void* handle, const void* foci, const float* amps, uint64_t size,
                         int32_t source_type) {
    run_nls(NLS_GRADIENT_DESCENT, handle, foci, amps, size, source_type);
}
void AFO_LM(void* handle, const void* foci, const float* amps, uint64_t size,
            int32_t source_type) {
    run_nls(NLS_LM, handle, foci, amps, size, source_type);
}
void AFO_Greedy(void* handle, const void* foci, const float* amps, uint64_t size,
                uint64_t phase_div, int32_t source_type) {
    if (phase_div < 1 || phase_div > static_cast<uint64_t>(kGreedyMaxDiv)) {
        set_error("AFO_Greedy: phase_div must be 1..%d", kGreedyMaxDiv);
        return;
    }
    run_solver(SOLVER_GREEDY, handle, foci, amps, size, source_type, static_cast<int>(phase_div));
}

// ------------------------------------------------------------------ device-level API

int32_t AFC_GridDescFromArea(void* grid_handle, int32_t dimension, AfcGridDesc* out) {
    Grid* g = as<Grid>(grid_handle, MAGIC_GRID, "grid area");
    if (!g || !out) return AFC_ERR_INVALID;
    if (g->dim != dimension) {
        set_error("dimension %d does not match the %dD grid handle", dimension, g->dim);
        return AFC_ERR_INVALID;
    }
    const GridDev d = grid_dev(*g);
    for (int k = 0; k < 3; ++k) {
        out->count[k] = static_cast<uint64_t>(d.count[k]);
        out->axis[k] = d.axis[k] + 1;
        out->origin[k] = d.origin[k];
    }
    out->res = d.res;
    return AFC_OK;
}

size_t AFC_FieldWorkspaceBytes(uint64_t n_sources) {
    if (n_sources >= (1ull << 40)) return 0;  // beyond what the field calls accept
    const size_t b = static_cast<size_t>(n_sources) * sizeof(PackedSource);
    return (b + 255) & ~static_cast<size_t>(255);
}

int32_t AFC_FieldGridDevice(int32_t st, int32_t ft, int32_t sum, const float* d_sources,
                            const float* d_k, const float* d_a, uint64_t n,
                            const AfcGridDesc* grid, void* d_out, void* ws, size_t ws_bytes,
                            void* stream) {
    int32_t rc = check_field_args(st, ft, sum, n, d_sources, d_k, d_a, d_out, ws, ws_bytes);
    if (rc != AFC_OK) return rc;
    if (!grid) {
        set_error("grid is NULL");
        return AFC_ERR_INVALID;
    }
    PointSet ps{};
    ps.is_grid = true;
    bool seen[3] = {false, false, false};
    for (int k = 0; k < 3; ++k) {
        const int a = grid->axis[k] - 1;
        if (a < 0 || a > 2 || seen[a] || grid->count[k] == 0) {
            set_error("invalid grid description");
            return AFC_ERR_INVALID;
        }
        seen[a] = true;
        ps.grid.axis[k] = a;
        ps.grid.count[k] = static_cast<int64_t>(grid->count[k]);
        ps.grid.origin[k] = grid->origin[k];
    }
    ps.grid.res = grid->res;
    uint64_t total = 0;
    if (!grid_points_checked(grid->count, &total)) {
        set_error("grid has too many points");
        return AFC_ERR_TOO_LARGE;
    }
    ps.m = static_cast<int64_t>(total);
    return device_field(st, ft, sum, d_sources, d_k, d_a, n, ps, d_out, ws, stream);
}

int32_t AFC_FieldScatterDevice(int32_t st, int32_t ft, int32_t sum, const float* d_sources,
                               const float* d_k, const float* d_a, uint64_t n,
                               const float* d_points, uint64_t m, void* d_out, void* ws,
                               size_t ws_bytes, void* stream) {
    int32_t rc = check_field_args(st, ft, sum, n, d_sources, d_k, d_a, d_out, ws, ws_bytes);
    if (rc != AFC_OK) return rc;
    if (m > 0 && !d_points) {
        set_error("points pointer is NULL");
        return AFC_ERR_INVALID;
    }
    if (m >= (1ull << 62)) {
        set_error("too many points");
        return AFC_ERR_TOO_LARGE;
    }
    PointSet ps{};
    ps.is_grid = false;
    ps.pts = d_points;
    ps.m = static_cast<int64_t>(m);
    return device_field(st, ft, sum, d_sources, d_k, d_a, n, ps, d_out, ws, stream);
}

uint64_t AFC_KernelLaunchCount(void) { return g_launches.load(); }

int32_t AFC_SetDevice(int32_t device) {
    cudaError_t e = cudaSetDevice(device);
    return e == cudaSuccess ? AFC_OK : cuda_fail(e, "cudaSetDevice");
}

int32_t AFC_CudaDeviceCount(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) return 0;
    return count;
}

}  // extern "C"
