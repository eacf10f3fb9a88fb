// Acoustic power optimization (acoustic-field-optimizer/src/multiple_foci/nls/apo.rs:98-158)
// on the device.
//
// The reference keeps m dense n x n matrices R_i = G^H D_i G, solves an n x n system for q0 and
// runs 200 quasi-Newton steps with a 100-point line search.  R_i = g_i^H g_i has rank one
// (g_i: row i of G), so with r = G q:
//     q^H R_i q = |r_i|^2,   grad J = G^H (s o r) + lambda q,  s_i = p2_i - |r_i|^2,
//     q0 = (G^H G + lambda I)^-1 G^H p = G^H (G G^H + lambda I)^-1 p       (an m x m solve),
// and J(q + a d) along the line needs only G q, G d and the three bilinear sums
// sum q_j^2, sum q_j d_j, sum d_j^2 (the reference's |q.q| term uses nalgebra's dot, which does
// not conjugate).  The n x n quasi-Newton matrix H stays dense: H grad, H s and its rank-two
// update run on the device; the m x m solve, the line search over a = 0, 0.01, .., 0.99 and the
// reference's control flow run on the host.  G is the float32 transfer matrix; everything the
// iteration carries (q, the gradients, d, H and the sums) is float64: the quasi-Newton update
// divides by y.s and s.H.s, which cancel badly, and in float32 the reference's own 18 x 14 foci
// example ends 10% away from the float64 iteration.  The kernels are memory-bound matrix-vector
// products and rank-two updates, so float64 costs bytes, not FP64 throughput.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "afc_internal.h"
#include "afc_solvers.h"
#include "dense_host.h"

namespace afc {
namespace {

constexpr int kApoThreads = 1024;
constexpr int kApoIterations = 200;  // apo.rs:19
constexpr int kApoLineSearch = 100;  // apo.rs:20
constexpr double kApoEps = 1e-8;     // apo.rs:18

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ double2 cmul(float2 a, double2 b) {
    return cmul(make_double2(a.x, a.y), b);
}

__device__ __forceinline__ double2 warp_sum2(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Block-wide complex sum (kApoThreads threads); `red` holds 32 double2.
__device__ double2 block_sum2(double2 v, double2* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum2(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    v = lane < (kApoThreads >> 5) ? red[lane] : make_double2(0.0, 0.0);
    return warp_sum2(v);
}

// r = G q (warp per row), then grad_j = sum_i conj(G_ij) s_i r_i + lambda q_j,
// s_i = p2_i - |r_i|^2.
__global__ void __launch_bounds__(kApoThreads)
    apo_grad_kernel(const float2* __restrict__ g, int64_t n, int64_t m,
                    const double* __restrict__ p2, const double2* __restrict__ q, double lambda,
                    double2* r, double2* grad) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t i = wid; i < m; i += nw) {
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t j = lane; j < n; j += 32) {
            const double2 v = cmul(g[i * n + j], q[j]);
            acc.x += v.x;
            acc.y += v.y;
        }
        acc = warp_sum2(acc);
        if (lane == 0) r[i] = acc;
    }
    __syncthreads();
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t i = 0; i < m; ++i) {
            const double2 ri = r[i];
            const float2 af = g[i * n + j];
            const double ax = af.x, ay = af.y;
            const double s = p2[i] - (ri.x * ri.x + ri.y * ri.y);
            // conj(a) s r_i
            acc.x += s * (ax * ri.x + ay * ri.y);
            acc.y += s * (ax * ri.y - ay * ri.x);
        }
        const double2 qj = q[j];
        grad[j] = make_double2(acc.x + lambda * qj.x, acc.y + lambda * qj.y);
    }
}

// out = sign * H v, H row-major n x n: warp per row.
__global__ void apo_hmv_kernel(const double2* __restrict__ h, int64_t n,
                               const double2* __restrict__ v, double sign,
                               double2* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t row = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t c = lane; c < n; c += 32) {
        const double2 t = cmul(h[row * n + c], v[c]);
        acc.x += t.x;
        acc.y += t.y;
    }
    acc = warp_sum2(acc);
    if (lane == 0) out[row] = make_double2(sign * acc.x, sign * acc.y);
}

// G d (m) and the bilinear sums sum q^2, sum q d, sum d^2 (into sums[0..2]).
__global__ void __launch_bounds__(kApoThreads)
    apo_line_kernel(const float2* __restrict__ g, int64_t n, int64_t m,
                    const double2* __restrict__ q, const double2* __restrict__ d, double2* gd,
                    double2* sums) {
    __shared__ double2 red[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t i = wid; i < m; i += nw) {
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t j = lane; j < n; j += 32) {
            const double2 v = cmul(g[i * n + j], d[j]);
            acc.x += v.x;
            acc.y += v.y;
        }
        acc = warp_sum2(acc);
        if (lane == 0) gd[i] = acc;
    }
    double2 sqq = make_double2(0.0, 0.0), sqd = sqq, sdd = sqq;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double2 a = q[j], b = d[j];
        const double2 aa = cmul(a, a), ab = cmul(a, b), bb = cmul(b, b);
        sqq.x += aa.x, sqq.y += aa.y;
        sqd.x += ab.x, sqd.y += ab.y;
        sdd.x += bb.x, sdd.y += bb.y;
    }
    sqq = block_sum2(sqq, red);
    sqd = block_sum2(sqd, red);
    sdd = block_sum2(sdd, red);
    if (threadIdx.x == 0) {
        sums[0] = sqq;
        sums[1] = sqd;
        sums[2] = sdd;
    }
}

// d <- alpha d, q_new = q + d, and |d|^2 into sums[3].x.
__global__ void __launch_bounds__(kApoThreads)
    apo_step_kernel(int64_t n, double alpha, double2* d, const double2* __restrict__ q,
                    double2* q_new, double2* sums) {
    __shared__ double2 red[32];
    double2 dd = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double2 v = make_double2(alpha * d[j].x, alpha * d[j].y);
        d[j] = v;
        q_new[j] = make_double2(q[j].x + v.x, q[j].y + v.y);
        dd.x += v.x * v.x + v.y * v.y;
    }
    dd = block_sum2(dd, red);
    if (threadIdx.x == 0) sums[3] = dd;
}

// s = grad_new - grad, and the bilinear sum y.s (y = d) into sums[4]; s.u (u = H s, computed
// between the two launches) into sums[5] by apo_su_kernel.
__global__ void __launch_bounds__(kApoThreads)
    apo_s_kernel(int64_t n, const double2* __restrict__ gn, const double2* __restrict__ go,
                 const double2* __restrict__ y, double2* s, double2* sums) {
    __shared__ double2 red[32];
    double2 ys = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double2 v = make_double2(gn[j].x - go[j].x, gn[j].y - go[j].y);
        s[j] = v;
        const double2 t = cmul(y[j], v);
        ys.x += t.x, ys.y += t.y;
    }
    ys = block_sum2(ys, red);
    if (threadIdx.x == 0) sums[4] = ys;
}

__global__ void __launch_bounds__(kApoThreads)
    apo_su_kernel(int64_t n, const double2* __restrict__ s, const double2* __restrict__ u,
                  double2* sums) {
    __shared__ double2 red[32];
    double2 su = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double2 t = cmul(s[j], u[j]);
        su.x += t.x, su.y += t.y;
    }
    su = block_sum2(su, red);
    if (threadIdx.x == 0) sums[5] = su;
}

// H += y y^T c1 - u u^T c2 (apo.rs:143-144 with transposes, not adjoints).
__global__ void apo_update_kernel(double2* h, int64_t n, const double2* __restrict__ y,
                                  const double2* __restrict__ u, double2 c1, double2 c2) {
    const int64_t r = blockIdx.y;
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n || c >= n) return;
    const double2 a = cmul(cmul(y[r], y[c]), c1), b = cmul(cmul(u[r], u[c]), c2);
    const double2 v = h[r * n + c];
    h[r * n + c] = make_double2(v.x + a.x - b.x, v.y + a.y - b.y);
}

__global__ void apo_identity_kernel(double2* h, int64_t n) {
    const int64_t r = blockIdx.y;
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n || c >= n) return;
    h[r * n + c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
}

unsigned blocks_for(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

std::mutex g_apo_mu;
cudaStream_t g_apo_stream = nullptr;
int g_apo_device = -1;

using cd = std::complex<double>;
using dense::hpd_solve;

}  // namespace

int solve_apo(int st, float* src, const float* k, const float* atten, int64_t n,
              const float* foci, const float* amps, int64_t m, float lambda, std::string* err) {
    if (m > kNlsMaxFoci) {
        *err = "too many foci for APO (" + std::to_string(m) + " > " + std::to_string(kNlsMaxFoci) +
               ")";
        return -1;
    }
    if (n == 0) return 0;
    if (n > 65535) {
        *err = "APO: at most 65535 sources (its n x n quasi-Newton matrix)";
        return -1;
    }
    const int stride = source_stride(st);
    const int iamp = st == SRC_T4010A1 ? 6 : 3;
    const int iphase = st == SRC_T4010A1 ? 7 : 4;
    std::lock_guard<std::mutex> lock(g_apo_mu);
    cudaError_t e;
    auto fail = [&](const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return -1;
    };
    if (!g_apo_stream) {
        int count = 0;
        e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            *err = "no CUDA device available; this library has no CPU path";
            return -1;
        }
        if ((e = cudaGetDevice(&g_apo_device)) != cudaSuccess) return fail("cudaGetDevice");
        if ((e = cudaStreamCreateWithFlags(&g_apo_stream, cudaStreamNonBlocking)) != cudaSuccess) {
            g_apo_stream = nullptr;
            return fail("cudaStreamCreate");
        }
    }
    DeviceGuard dg;  // the solver's device while it runs; the caller's again on return
    if ((e = dg.set(g_apo_device)) != cudaSuccess) return fail("cudaSetDevice");
    cudaStream_t s = g_apo_stream;
    std::vector<float> raw(src, src + n * stride);
    for (int64_t j = 0; j < n; ++j) raw[j * stride + iphase] = 0.f;  // apo.rs:101-103

    auto a256 = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += a256(bytes ? bytes : 1);
        return o;
    };
    const size_t o_raw = take(4 * n * stride), o_k = take(4 * n), o_at = take(4 * n),
                 o_foci = take(12 * m), o_p2 = take(8 * m), o_g = take(8 * m * n),
                 o_pk = take(48 * n), o_h = take(16 * n * n), o_q = take(16 * n),
                 o_qn = take(16 * n), o_gr = take(16 * n), o_gn = take(16 * n), o_d = take(16 * n),
                 o_sv = take(16 * n), o_u = take(16 * n), o_r = take(16 * m), o_gd = take(16 * m),
                 o_sums = take(128);
    char* d = nullptr;
    if ((e = cudaMalloc(&d, off)) != cudaSuccess) return fail("cudaMalloc");
    struct Free {
        char* p;
        ~Free() { cudaFree(p); }
    } free_d{d};
    auto F = [&](size_t o) { return reinterpret_cast<float*>(d + o); };
    auto F2 = [&](size_t o) { return reinterpret_cast<float2*>(d + o); };
    auto D = [&](size_t o) { return reinterpret_cast<double*>(d + o); };
    auto D2 = [&](size_t o) { return reinterpret_cast<double2*>(d + o); };
    std::vector<double> p2(static_cast<size_t>(m));
    for (int64_t i = 0; i < m; ++i)  // |p_i|^2, apo.rs:110
        p2[i] = static_cast<double>(amps[i]) * static_cast<double>(amps[i]);
    if ((e = cudaMemcpyAsync(d + o_raw, raw.data(), 4 * n * stride, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_k, k, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_at, atten, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (m && (e = cudaMemcpyAsync(d + o_foci, foci, 12 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (m && (e = cudaMemcpyAsync(d + o_p2, p2.data(), 8 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess))
        return fail("upload");
    if ((e = launch_build_g(st, F(o_raw), F(o_k), F(o_at), n, F(o_foci), m, F2(o_g), d + o_pk, s)) !=
        cudaSuccess)
        return fail("G");
    std::vector<float> gh(static_cast<size_t>(2 * m * n));
    if (m && ((e = cudaMemcpyAsync(gh.data(), d + o_g, 8 * m * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
              (e = cudaStreamSynchronize(s)) != cudaSuccess))
        return fail("G download");
    auto gel = [&](int64_t i, int64_t j) { return cd(gh[2 * (i * n + j)], gh[2 * (i * n + j) + 1]); };

    // q0 = G^H (G G^H + lambda I)^-1 p  (apo.rs:113-117)
    std::vector<cd> q0(static_cast<size_t>(n), cd(0.0));
    if (m > 0) {
        const int mm = static_cast<int>(m);
        std::vector<cd> kk(static_cast<size_t>(m * m)), c(static_cast<size_t>(m));
        for (int i = 0; i < mm; ++i) {
            for (int j = 0; j < mm; ++j) {
                cd acc = 0.0;
                for (int64_t b = 0; b < n; ++b) acc += gel(i, b) * std::conj(gel(j, b));
                kk[i * mm + j] = acc + (i == j ? cd(lambda) : cd(0.0));
            }
            c[i] = cd(amps[i], 0.0);
        }
        if (!hpd_solve(kk, c, mm)) {
            *err = "APO: G G^H + lambda I is not positive definite (lambda <= 0?)";
            return -1;
        }
        for (int64_t b = 0; b < n; ++b) {
            cd acc = 0.0;
            for (int i = 0; i < mm; ++i) acc += std::conj(gel(i, b)) * c[i];
            q0[b] = acc;
        }
    }
    std::vector<double> qh(static_cast<size_t>(2 * n));
    for (int64_t b = 0; b < n; ++b) {
        qh[2 * b] = q0[b].real();
        qh[2 * b + 1] = q0[b].imag();
    }
    if ((e = cudaMemcpyAsync(d + o_q, qh.data(), 16 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return fail("upload");
    const dim3 g2(blocks_for(n, 256), static_cast<unsigned>(n));
    apo_identity_kernel<<<g2, 256, 0, s>>>(D2(o_h), n);
    apo_grad_kernel<<<1, kApoThreads, 0, s>>>(F2(o_g), n, m, D(o_p2), D2(o_q), lambda, D2(o_r),
                                              D2(o_gr));
    count_launch(2);

    std::vector<double> r(static_cast<size_t>(2 * m)), gd(static_cast<size_t>(2 * m)), sums(12);
    const unsigned rows_blocks = blocks_for(n * 32, 256);
    for (int it = 0; it < kApoIterations; ++it) {
        // d = -H grad; along d: G q (from the gradient), G d, bilinear sums
        apo_hmv_kernel<<<rows_blocks, 256, 0, s>>>(D2(o_h), n, D2(o_gr), -1.0, D2(o_d));
        apo_line_kernel<<<1, kApoThreads, 0, s>>>(F2(o_g), n, m, D2(o_q), D2(o_d), D2(o_gd),
                                                  D2(o_sums));
        count_launch(2);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (m && (e = cudaMemcpyAsync(r.data(), d + o_r, 16 * m, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
            (m && (e = cudaMemcpyAsync(gd.data(), d + o_gd, 16 * m, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(sums.data(), d + o_sums, 48, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("APO line search");
        // line search (apo.rs:75-92): J(q + a d), a = i / 100, first minimum
        const cd sqq(sums[0], sums[1]), sqd(sums[2], sums[3]), sdd(sums[4], sums[5]);
        double alpha = 0.0, best = INFINITY;
        for (int li = 0; li < kApoLineSearch; ++li) {
            const double a = static_cast<double>(static_cast<float>(li) / static_cast<float>(kApoLineSearch));
            double v = 0.0;
            for (int64_t i = 0; i < m; ++i) {
                const cd ri = cd(r[2 * i], r[2 * i + 1]) + a * cd(gd[2 * i], gd[2 * i + 1]);
                const double t = std::norm(ri) - p2[i];
                v += t * t;
            }
            v += std::abs(sqq + 2.0 * a * sqd + a * a * sdd) * lambda;
            if (v < best) {
                best = v;
                alpha = a;
            }
        }
        apo_step_kernel<<<1, kApoThreads, 0, s>>>(n, alpha, D2(o_d), D2(o_q), D2(o_qn), D2(o_sums));
        count_launch();
        double dd[2];
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(dd, D2(o_sums) + 3, 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("APO step");
        if (std::sqrt(dd[0]) < kApoEps) break;  // apo.rs:127-129
        // quasi-Newton update (apo.rs:131-147): s = grad_new - grad, y = d, u = H s
        apo_grad_kernel<<<1, kApoThreads, 0, s>>>(F2(o_g), n, m, D(o_p2), D2(o_qn), lambda,
                                                  D2(o_r), D2(o_gn));
        apo_s_kernel<<<1, kApoThreads, 0, s>>>(n, D2(o_gn), D2(o_gr), D2(o_d), D2(o_sv), D2(o_sums));
        apo_hmv_kernel<<<rows_blocks, 256, 0, s>>>(D2(o_h), n, D2(o_sv), 1.0, D2(o_u));
        apo_su_kernel<<<1, kApoThreads, 0, s>>>(n, D2(o_sv), D2(o_u), D2(o_sums));
        count_launch(4);
        double ys_su[4];
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(ys_su, D2(o_sums) + 4, 32, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("APO update");
        const cd c1 = 1.0 / cd(ys_su[0], ys_su[1]), c2 = 1.0 / cd(ys_su[2], ys_su[3]);
        apo_update_kernel<<<g2, 256, 0, s>>>(D2(o_h), n, D2(o_d), D2(o_u),
                                             make_double2(c1.real(), c1.imag()),
                                             make_double2(c2.real(), c2.imag()));
        count_launch();
        // q = q_new, grad = grad_new
        if ((e = cudaMemcpyAsync(d + o_q, d + o_qn, 16 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d + o_gr, d + o_gn, 16 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return fail("APO update");
    }
    if ((e = cudaMemcpyAsync(qh.data(), d + o_q, 16 * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail("APO result");
    // apo.rs:150-157: amp *= |q_j| / camax(q), phase = arg q_j.  camax of a complex vector
    // (nalgebra 0.27.1) is the largest norm-1 value |re| + |im| of its entries.
    double max_coeff = 0.0;
    for (int64_t b = 0; b < n; ++b)
        max_coeff = std::max(max_coeff, std::fabs(qh[2 * b]) + std::fabs(qh[2 * b + 1]));
    for (int64_t b = 0; b < n; ++b) {
        const double mag = std::hypot(qh[2 * b], qh[2 * b + 1]);
        src[b * stride + iamp] = static_cast<float>(src[b * stride + iamp] * mag / max_coeff);
        src[b * stride + iphase] = static_cast<float>(std::atan2(qh[2 * b + 1], qh[2 * b]));
    }
    return 0;
}

}  // namespace afc
