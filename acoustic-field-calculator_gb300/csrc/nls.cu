// Nonlinear least-squares phase retrieval on the device: gradient descent, Gauss-Newton and
// Levenberg-Marquardt (acoustic-field-optimizer/src/multiple_foci/nls/{gradient_descent,
// gauss_newton,lm}.rs, with the shared helpers of nls/macros.rs:16-58).
//
// The reference builds B = [G | -diag(amps)] (m x N, N = n + m), the dense N x N matrix
// BhB = B^H B, and per iteration JtJ = Re(BhB o T T^H), Jtf = column sums of Im(BhB o T T^H)
// (T = exp(-i x)), F(x) = Re(t^H BhB t) (t = exp(i x)), solving N x N systems by QR (LM) or
// an SVD pseudo-inverse (Gauss-Newton).  B has only m rows, so every one of those is low rank
// and is evaluated here from B itself (the identities are exact, not approximations):
//     r = B t,  Jtf_b = Im(t_b conj((B^H r)_b)),  F = |r|^2,
//     JtJ = U^T U with U = [Re C; Im C], C = B diag(t)   (2m x N),
//     (JtJ + mu I)^-1 g = (g - U^T (mu I + U U^T)^-1 U g) / mu          (Woodbury, LM),
//     pinv(JtJ) g = U^T sum_{lambda_k > eps} w_k w_k^T U g / lambda_k^2  (U U^T = W Lambda W^T, GN),
//     U U^T from K = B B^H (fixed) and L = sum_b B_ib B_jb t_b^2.
// The device does the O(N m) and O(N m^2) work in f32 (one block per step; gradient descent's
// whole loop runs in one launch); the 2m x 2m solves and the control flow of the reference's
// loops run on the host in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "afc_internal.h"
#include "afc_solvers.h"

namespace afc {
namespace {

constexpr int kNlsThreads = 1024;

// Parameters of nls/{gradient_descent,gauss_newton,lm}.rs.
constexpr float kGdEps = 1e-6f;       // gradient_descent.rs:17
constexpr int kGdIterations = 10000;  // gradient_descent.rs:18
constexpr double kNlsEps1 = 1e-8;     // gauss_newton.rs:17, lm.rs:17
constexpr double kNlsEps2 = 1e-8;     // gauss_newton.rs:18, lm.rs:18
constexpr double kLmTau = 1e-3;       // lm.rs:19
constexpr int kNlsIterations = 200;   // gauss_newton.rs:19, lm.rs:20
constexpr double kPinvEps = 1e-3;     // gauss_newton.rs:64 (pseudo_inverse(1e-3))

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 warp_sum2(float2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum / max (kNlsThreads threads); `red` holds 32 floats.
__device__ float block_sum(float v, float* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    v = lane < (kNlsThreads >> 5) ? red[lane] : 0.f;
    return warp_sum(v);
}

__device__ float block_max(float v, float* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    v = lane < (kNlsThreads >> 5) ? red[lane] : -__int_as_float(0x7f800000);
    return warp_max(v);
}

// t_b = exp(i x_b) for the N parameters.
__device__ void phasors(const float* x, int64_t N, float2* t) {
    for (int64_t b = threadIdx.x; b < N; b += blockDim.x) {
        float s, c;
        sincosf(x[b], &s, &c);
        t[b] = make_float2(c, s);
    }
}

// r = B t: warp per row i (G row i, then -amps_i t_{n+i}).
__device__ void b_times(const float2* g, const float* amps, int64_t n, int64_t m, const float2* t,
                        float2* r) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t i = wid; i < m; i += nw) {
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t a = lane; a < n; a += 32) {
            const float2 v = cmul(g[i * n + a], t[a]);
            acc.x += v.x;
            acc.y += v.y;
        }
        acc = warp_sum2(acc);
        if (lane == 0) {
            const float2 p = t[n + i];
            r[i] = make_float2(acc.x - amps[i] * p.x, acc.y - amps[i] * p.y);
        }
    }
}

// Jtf_b = Im(t_b conj((B^H r)_b)); returns the thread's largest Jtf.
__device__ float gradient(const float2* g, const float* amps, int64_t n, int64_t m,
                          const float2* t, const float2* r, float* jtf) {
    float mx = -__int_as_float(0x7f800000);
    for (int64_t b = threadIdx.x; b < n + m; b += blockDim.x) {
        float2 w;
        if (b < n) {
            w = make_float2(0.f, 0.f);
            for (int64_t i = 0; i < m; ++i) {
                const float2 a = g[i * n + b], q = r[i];
                // conj(a) q
                w.x += a.x * q.x + a.y * q.y;
                w.y += a.x * q.y - a.y * q.x;
            }
        } else {
            const int64_t i = b - n;
            w = make_float2(-amps[i] * r[i].x, -amps[i] * r[i].y);
        }
        const float2 tb = t[b];
        const float v = tb.y * w.x - tb.x * w.y;
        jtf[b] = v;
        mx = fmaxf(mx, v);
    }
    return mx;
}

// Gradient descent (gradient_descent.rs:31-59) in one block: x <- x - 0.1 Jtf until
// max(Jtf) <= 1e-6 or 10000 steps.  t (N), r (m), jtf (N) are workspace; *iters receives the
// number of steps taken.
__global__ void __launch_bounds__(kNlsThreads)
    nls_gd_kernel(const float2* __restrict__ g, const float* __restrict__ amps, int64_t n,
                  int64_t m, float* x, float2* t, float2* r, float* jtf, int max_iter, float eps,
                  int* iters) {
    __shared__ float red[32];
    const int64_t N = n + m;
    int it = 0;
    for (; it < max_iter; ++it) {
        phasors(x, N, t);
        __syncthreads();
        b_times(g, amps, n, m, t, r);
        __syncthreads();
        const float mx = block_max(gradient(g, amps, n, m, t, r, jtf), red);
        if (mx <= eps) break;  // uniform: every thread holds the block maximum
        for (int64_t b = threadIdx.x; b < N; b += blockDim.x)
            x[b] = __fsub_rn(x[b], __fmul_rn(0.1f, jtf[b]));
        __syncthreads();
    }
    if (threadIdx.x == 0) *iters = it;
}

// Everything a Gauss-Newton / LM step needs at x: t, r, Jtf, and into `sc`: F = |r|^2,
// max(Jtf), |x|^2; U Jtf into ug (2m: Re rows then Im rows); with `with_l`, L_ij =
// sum_b B_ib B_jb t_b^2 (m x m, row-major) into l.
__global__ void __launch_bounds__(kNlsThreads)
    nls_eval_kernel(const float2* __restrict__ g, const float* __restrict__ amps, int64_t n,
                    int64_t m, const float* __restrict__ x, float2* t, float2* r, float* jtf,
                    float* sc, float* ug, float2* l, int with_l) {
    __shared__ float red[32];
    const int64_t N = n + m;
    phasors(x, N, t);
    __syncthreads();
    b_times(g, amps, n, m, t, r);
    __syncthreads();
    const float mx = block_max(gradient(g, amps, n, m, t, r, jtf), red);
    float f = 0.f;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) f += r[i].x * r[i].x + r[i].y * r[i].y;
    f = block_sum(f, red);
    float xx = 0.f;
    for (int64_t b = threadIdx.x; b < N; b += blockDim.x) xx += x[b] * x[b];
    xx = block_sum(xx, red);
    if (threadIdx.x == 0) {
        sc[0] = f;
        sc[1] = mx;
        sc[2] = xx;
    }
    __syncthreads();  // jtf complete
    // U Jtf: (Re C_i., Im C_i.) . Jtf, C_ib = B_ib t_b; warp per row
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t i = wid; i < m; i += nw) {
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t b = lane; b < n; b += 32) {
            const float2 c = cmul(g[i * n + b], t[b]);
            acc.x += c.x * jtf[b];
            acc.y += c.y * jtf[b];
        }
        acc = warp_sum2(acc);
        if (lane == 0) {
            const float2 p = t[n + i];
            const float gj = jtf[n + i];
            ug[i] = acc.x - amps[i] * p.x * gj;
            ug[m + i] = acc.y - amps[i] * p.y * gj;
        }
    }
    if (!with_l) return;
    // L_ij = sum_{b<n} G_ib G_jb t_b^2 + delta_ij amps_i^2 t_{n+i}^2; warp per (i, j)
    for (int64_t p = wid; p < m * m; p += nw) {
        const int64_t i = p / m, j = p % m;
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t b = lane; b < n; b += 32) {
            const float2 tb = t[b];
            const float2 t2 = make_float2(tb.x * tb.x - tb.y * tb.y, 2.f * tb.x * tb.y);
            const float2 v = cmul(cmul(g[i * n + b], g[j * n + b]), t2);
            acc.x += v.x;
            acc.y += v.y;
        }
        acc = warp_sum2(acc);
        if (lane == 0) {
            if (i == j) {
                const float2 tp = t[n + i];
                const float a2 = amps[i] * amps[i];
                acc.x += a2 * (tp.x * tp.x - tp.y * tp.y);
                acc.y += a2 * (2.f * tp.x * tp.y);
            }
            l[p] = acc;
        }
    }
}

// h = (coef_g Jtf - U^T y) * scale, x_new = x + h, and into sc: |h|^2, h.(mu h - Jtf).
// LM: coef_g = 1, scale = -1/mu (h = -(Jtf - U^T y)/mu); GN: coef_g = 0, scale = -1.
__global__ void __launch_bounds__(kNlsThreads)
    nls_step_kernel(const float2* __restrict__ g, const float* __restrict__ amps, int64_t n,
                    int64_t m, const float2* __restrict__ t, const float* __restrict__ jtf,
                    const float* __restrict__ y, float coef_g, float scale, float mu,
                    const float* __restrict__ x, float* h, float* x_new, float* sc) {
    __shared__ float red[32];
    float hh = 0.f, hd = 0.f;
    for (int64_t b = threadIdx.x; b < n + m; b += blockDim.x) {
        float u = 0.f;  // (U^T y)_b = sum_i Re(C_ib) y_i + Im(C_ib) y_{m+i}
        const float2 tb = t[b];
        if (b < n) {
            for (int64_t i = 0; i < m; ++i) {
                const float2 c = cmul(g[i * n + b], tb);
                u += c.x * y[i] + c.y * y[m + i];
            }
        } else {
            const int64_t i = b - n;
            u = -amps[i] * (tb.x * y[i] + tb.y * y[m + i]);
        }
        const float hb = (coef_g * jtf[b] - u) * scale;
        h[b] = hb;
        x_new[b] = x[b] + hb;
        hh += hb * hb;
        hd += hb * (mu * hb - jtf[b]);
    }
    hh = block_sum(hh, red);
    hd = block_sum(hd, red);
    if (threadIdx.x == 0) {
        sc[0] = hh;
        sc[1] = hd;
    }
}

// ------------------------------------------------------------------ host: small dense algebra

// Solve the SPD system a y = b (k x k, row-major, overwritten) by Cholesky; false if not SPD.
bool cholesky_solve(std::vector<double>& a, std::vector<double>& b, int k) {
    for (int j = 0; j < k; ++j) {
        double d = a[j * k + j];
        for (int p = 0; p < j; ++p) d -= a[j * k + p] * a[j * k + p];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        a[j * k + j] = d;
        for (int i = j + 1; i < k; ++i) {
            double s = a[i * k + j];
            for (int p = 0; p < j; ++p) s -= a[i * k + p] * a[j * k + p];
            a[i * k + j] = s / d;
        }
    }
    for (int i = 0; i < k; ++i) {  // L z = b
        double s = b[i];
        for (int p = 0; p < i; ++p) s -= a[i * k + p] * b[p];
        b[i] = s / a[i * k + i];
    }
    for (int i = k - 1; i >= 0; --i) {  // L^T y = z
        double s = b[i];
        for (int p = i + 1; p < k; ++p) s -= a[p * k + i] * b[p];
        b[i] = s / a[i * k + i];
    }
    return true;
}

// Cyclic Jacobi eigendecomposition of the symmetric k x k matrix a (row-major, destroyed):
// eigenvalues in lam, eigenvectors in the columns of v.
void jacobi_eigen(std::vector<double>& a, int k, std::vector<double>& lam, std::vector<double>& v) {
    v.assign(static_cast<size_t>(k) * k, 0.0);
    for (int i = 0; i < k; ++i) v[i * k + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                tot += a[i * k + j] * a[i * k + j];
                if (i != j) off += a[i * k + j] * a[i * k + j];
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = a[p * k + q];
                if (apq == 0.0) continue;
                const double theta = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
                const double tt = (theta >= 0 ? 1.0 : -1.0) /
                                  (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(tt * tt + 1.0), s = tt * c;
                for (int r = 0; r < k; ++r) {  // columns p, q
                    const double arp = a[r * k + p], arq = a[r * k + q];
                    a[r * k + p] = c * arp - s * arq;
                    a[r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {  // rows p, q
                    const double apr = a[p * k + r], aqr = a[q * k + r];
                    a[p * k + r] = c * apr - s * aqr;
                    a[q * k + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; ++r) {
                    const double vrp = v[r * k + p], vrq = v[r * k + q];
                    v[r * k + p] = c * vrp - s * vrq;
                    v[r * k + q] = s * vrp + c * vrq;
                }
            }
    }
    lam.resize(k);
    for (int i = 0; i < k; ++i) lam[i] = a[i * k + i];
}

struct NlsCtx {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    int device = -1;
};
NlsCtx g_nls;

}  // namespace

int solve_nls(int kind, int st, float* src, const float* k, const float* atten, int64_t n,
              const float* foci, const float* amps, int64_t m, std::string* err) {
    if (m > kNlsMaxFoci) {
        *err = "too many foci for the NLS solvers (" + std::to_string(m) + " > " +
               std::to_string(kNlsMaxFoci) + ")";
        return -1;
    }
    if (n == 0) return 0;
    const int stride = source_stride(st);
    const int iphase = st == SRC_T4010A1 ? 7 : 4;
    std::lock_guard<std::mutex> lock(g_nls.mu);
    cudaError_t e;
    auto fail = [&](const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return -1;
    };
    if (!g_nls.stream) {
        int count = 0;
        e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            *err = "no CUDA device available; this library has no CPU path";
            return -1;
        }
        if ((e = cudaGetDevice(&g_nls.device)) != cudaSuccess) return fail("cudaGetDevice");
        if ((e = cudaStreamCreateWithFlags(&g_nls.stream, cudaStreamNonBlocking)) != cudaSuccess) {
            g_nls.stream = nullptr;
            return fail("cudaStreamCreate");
        }
    }
    DeviceGuard dg;  // the solver's device while it runs; the caller's again on return
    if ((e = dg.set(g_nls.device)) != cudaSuccess) return fail("cudaSetDevice");
    cudaStream_t s = g_nls.stream;
    const int64_t N = n + m;
    // phases are zeroed first (nls/*.rs: set_phase(0.)); G is built from the zero-phase sources
    std::vector<float> raw(src, src + n * stride);
    for (int64_t j = 0; j < n; ++j) raw[j * stride + iphase] = 0.f;

    // device block: raw | k | atten | foci | amps | G | packed | x | x_new | h | t | r | jtf |
    //               ug | y | l | scalars | iters
    auto a256 = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += a256(bytes ? bytes : 1);
        return o;
    };
    const size_t o_raw = take(4 * n * stride), o_k = take(4 * n), o_at = take(4 * n),
                 o_foci = take(12 * m), o_amps = take(4 * m), o_g = take(8 * m * n),
                 o_pk = take(48 * n), o_x = take(4 * N), o_xn = take(4 * N), o_h = take(4 * N),
                 o_t = take(8 * N), o_r = take(8 * m), o_j = take(4 * N), o_ug = take(8 * m),
                 o_y = take(8 * m), o_l = take(8 * m * m), o_sc = take(64), o_it = take(4);
    char* d = nullptr;
    if ((e = cudaMalloc(&d, off)) != cudaSuccess) return fail("cudaMalloc");
    struct Free {
        char* p;
        ~Free() { cudaFree(p); }
    } free_d{d};
    auto F = [&](size_t o) { return reinterpret_cast<float*>(d + o); };
    auto F2 = [&](size_t o) { return reinterpret_cast<float2*>(d + o); };
    if ((e = cudaMemcpyAsync(d + o_raw, raw.data(), 4 * n * stride, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_k, k, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_at, atten, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (m && (e = cudaMemcpyAsync(d + o_foci, foci, 12 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (m && (e = cudaMemcpyAsync(d + o_amps, amps, 4 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (e = cudaMemsetAsync(d + o_x, 0, 4 * N, s)) != cudaSuccess)
        return fail("upload");
    if ((e = launch_build_g(st, F(o_raw), F(o_k), F(o_at), n, F(o_foci), m, F2(o_g), d + o_pk, s)) !=
        cudaSuccess)
        return fail("G");
    std::vector<float> x(static_cast<size_t>(N), 0.f);

    if (kind == NLS_GRADIENT_DESCENT) {
        nls_gd_kernel<<<1, kNlsThreads, 0, s>>>(F2(o_g), F(o_amps), n, m, F(o_x), F2(o_t), F2(o_r),
                                               F(o_j), kGdIterations, kGdEps,
                                               reinterpret_cast<int*>(d + o_it));
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return fail("gradient descent");
        if ((e = cudaMemcpyAsync(x.data(), d + o_x, 4 * N, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("gradient descent");
    } else {
        // K = B B^H = G G^H + diag(amps^2), fixed: from G on the host, in double
        std::vector<float> gh(static_cast<size_t>(2 * m * n));
        if ((e = cudaMemcpyAsync(gh.data(), d + o_g, 8 * m * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("G download");
        const int mm = static_cast<int>(m), k2 = 2 * mm;
        std::vector<double> kre(static_cast<size_t>(m * m)), kim(static_cast<size_t>(m * m));
        for (int i = 0; i < mm; ++i)
            for (int j = 0; j < mm; ++j) {
                double re = 0, im = 0;
                for (int64_t b = 0; b < n; ++b) {
                    const double ar = gh[2 * (i * n + b)], ai = gh[2 * (i * n + b) + 1];
                    const double br = gh[2 * (j * n + b)], bi = gh[2 * (j * n + b) + 1];
                    re += ar * br + ai * bi;  // a conj(b)
                    im += ai * br - ar * bi;
                }
                if (i == j) re += static_cast<double>(amps[i]) * amps[i];
                kre[i * mm + j] = re;
                kim[i * mm + j] = im;
            }
        // diag(JtJ)_b = sum_i |B_ib|^2 (independent of x), for LM's initial mu
        double a_max = 0;
        for (int64_t b = 0; b < n; ++b) {
            double s2 = 0;
            for (int i = 0; i < mm; ++i)
                s2 += static_cast<double>(gh[2 * (i * n + b)]) * gh[2 * (i * n + b)] +
                      static_cast<double>(gh[2 * (i * n + b) + 1]) * gh[2 * (i * n + b) + 1];
            a_max = std::max(a_max, s2);
        }
        for (int i = 0; i < mm; ++i) a_max = std::max(a_max, static_cast<double>(amps[i]) * amps[i]);

        std::vector<float> sc(16), ug(static_cast<size_t>(k2)), lh(static_cast<size_t>(2 * m * m)),
            y(static_cast<size_t>(k2));
        // evaluate at the device's x; with_l: also L (for a step from this x)
        auto eval = [&](size_t ox, bool with_l) -> bool {
            nls_eval_kernel<<<1, kNlsThreads, 0, s>>>(F2(o_g), F(o_amps), n, m, F(ox), F2(o_t),
                                                     F2(o_r), F(o_j), F(o_sc), F(o_ug), F2(o_l),
                                                     with_l ? 1 : 0);
            count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return false;
            if ((e = cudaMemcpyAsync(sc.data(), d + o_sc, 12, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(ug.data(), d + o_ug, 4 * k2, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                (with_l && (e = cudaMemcpyAsync(lh.data(), d + o_l, 8 * m * m, cudaMemcpyDeviceToHost, s)) != cudaSuccess))
                return false;
            return (e = cudaStreamSynchronize(s)) == cudaSuccess;
        };
        // M = U U^T from K and L (2m x 2m)
        std::vector<double> mat(static_cast<size_t>(k2 * k2));
        auto build_m = [&]() {
            for (int i = 0; i < mm; ++i)
                for (int j = 0; j < mm; ++j) {
                    const double lr = lh[2 * (i * mm + j)], li = lh[2 * (i * mm + j) + 1];
                    const double kr = kre[i * mm + j], ki = kim[i * mm + j];
                    mat[i * k2 + j] = 0.5 * (kr + lr);
                    mat[i * k2 + mm + j] = 0.5 * (li - ki);
                    mat[(mm + i) * k2 + j] = 0.5 * (li + ki);
                    mat[(mm + i) * k2 + mm + j] = 0.5 * (kr - lr);
                }
        };
        // one step from the x at o_x: y on the host, then h, x_new, |h|^2, h.(mu h - g) on the
        // device; false with *bad set when the small system cannot be solved
        auto step = [&](double mu, bool lm, bool* bad, float* hh, float* hd) -> bool {
            build_m();
            std::vector<double> rhs(ug.begin(), ug.end());
            if (lm) {
                for (int i = 0; i < k2; ++i) mat[i * k2 + i] += mu;
                if (!cholesky_solve(mat, rhs, k2)) {
                    *bad = true;
                    return true;
                }
                for (int i = 0; i < k2; ++i) y[i] = static_cast<float>(rhs[i]);
            } else {
                std::vector<double> lam, v;
                jacobi_eigen(mat, k2, lam, v);
                std::vector<double> yy(static_cast<size_t>(k2), 0.0);
                for (int q = 0; q < k2; ++q) {
                    if (!(lam[q] > kPinvEps)) continue;
                    double proj = 0;
                    for (int i = 0; i < k2; ++i) proj += v[i * k2 + q] * rhs[i];
                    for (int i = 0; i < k2; ++i) yy[i] += v[i * k2 + q] * proj / (lam[q] * lam[q]);
                }
                for (int i = 0; i < k2; ++i) y[i] = static_cast<float>(yy[i]);
            }
            if ((e = cudaMemcpyAsync(d + o_y, y.data(), 4 * k2, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return false;
            nls_step_kernel<<<1, kNlsThreads, 0, s>>>(
                F2(o_g), F(o_amps), n, m, F2(o_t), F(o_j), F(o_y), lm ? 1.f : 0.f,
                lm ? static_cast<float>(-1.0 / mu) : -1.f, static_cast<float>(mu), F(o_x), F(o_h),
                F(o_xn), F(o_sc) + 4);
            count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return false;
            float two[2];
            if ((e = cudaMemcpyAsync(two, F(o_sc) + 4, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                (e = cudaStreamSynchronize(s)) != cudaSuccess)
                return false;
            *hh = two[0];
            *hd = two[1];
            return true;
        };

        const bool lm = kind == NLS_LM;
        if (!eval(o_x, true)) return fail("NLS evaluation");
        double fx = sc[0];
        bool found = sc[1] <= kNlsEps1;
        double mu = kLmTau * a_max, nu = 2.0;
        for (int it = 0; it < kNlsIterations && !found; ++it) {
            bool bad = false;
            float hh = 0, hd = 0;
            const float xx = sc[2];  // |x|^2 at the current x (eval keeps sc[2] for it)
            if (!step(mu, lm, &bad, &hh, &hd)) return fail("NLS step");
            if (bad) break;
            if (std::sqrt(static_cast<double>(hh)) <=
                kNlsEps2 * (std::sqrt(static_cast<double>(xx)) + kNlsEps2)) {
                found = true;
                break;
            }
            if (!lm) {  // Gauss-Newton: accept x + h (gauss_newton.rs:72-79)
                if ((e = cudaMemcpyAsync(d + o_x, d + o_xn, 4 * N, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                    return fail("NLS update");
                if (!eval(o_x, true)) return fail("NLS evaluation");
                found = sc[1] <= kNlsEps1;
                continue;
            }
            // LM (lm.rs:75-96): gain ratio from F at x_new
            if (!eval(o_xn, false)) return fail("NLS evaluation");
            const double fx_new = sc[0];
            const double l0 = 0.5 * hd;
            const double rho = (fx - fx_new) / l0;
            fx = fx_new;
            if (rho > 0.0) {
                if ((e = cudaMemcpyAsync(d + o_x, d + o_xn, 4 * N, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                    return fail("NLS update");
                if (!eval(o_x, true)) return fail("NLS evaluation");
                found = sc[1] <= kNlsEps1;
                const double c = 2.0 * rho - 1.0;
                mu *= std::max(1.0 / 3.0, 1.0 - c * c * c);
                nu = 2.0;
            } else {
                // x, A and g stay (F takes F(x_new), as in the reference): re-evaluate at x to
                // restore the buffers the evaluation at x_new overwrote
                if (!eval(o_x, true)) return fail("NLS evaluation");
                mu *= nu;
                nu *= 2.0;
            }
        }
        if ((e = cudaMemcpyAsync(x.data(), d + o_x, 4 * N, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("NLS result");
    }
    for (int64_t j = 0; j < n; ++j) src[j * stride + iphase] = x[j];
    return 0;
}

}  // namespace afc
