// Matrix optimizers on the device: Horn (Inoue et al. 2015) and Long (Long et al. 2014),
// acoustic-field-optimizer/src/multiple_foci/matrix/{horn,long}.rs.
//
// Both start from the transfer matrix G (m foci x n sources, built as for GS-PAT from the
// zero-phase sources, multiple_foci/macros.rs:32-53) and reduce to m x m algebra through exact
// identities, so that the device does the O(n m^2) work and the host solves m x m systems in
// double:
//
//   Horn (horn.rs:71-129).  The regularised pseudo-inverse V diag(s / (s^2 + a^2)) U^H of G
//   (horn.rs:60-69, a = 1e-5) equals G^H (K + a^2 I)^-1 with K = G G^H.  Hence
//   I - G G_pinv = a^2 (K + a^2 I)^-1 and MM = a^2 P (K + a^2 I)^-1 P (P = diag(amps)).  In f32
//   the reference forms I - G G_pinv by subtraction; its entries (about a^2 / |K|, 1e-9) lie
//   far below f32 resolution, so its MM is rounding noise.  The form here keeps MM to double
//   accuracy.  The SDP's coordinate updates (horn.rs:87-117) are invariant to the scale of MM;
//   they run as one device block in f32 like the reference's (MM normalised to a largest entry
//   of 1), m * 100 steps.  Then u = the principal eigenvector of X and
//   q = G_pinv P u = G^H (K + a^2 I)^-1 P u.
//
//   Long (long.rs:48-105).  X = (amps_i conj(G_ij) / d_i)^T with d = G's row sums, so
//   R = G X = K diag(amps / d).  The phases e_k = arg V[imax, k] of the eigenvector matrix's
//   row imax (the reference indexes a row, long.rs:67-70) become the focus targets
//   f = amps e^{i e}.  The least-squares system (g^H g) q = g^H [f; 0], g = [G; diag(sigma)],
//   sigma_j^2 = sum_i |G_ij| amps_i / m, is solved by Woodbury:
//   q = S^-1 G^H (I + G S^-1 G^H)^-1 f with S = diag(sigma^2).
//
// Reference behaviour that no port can reproduce, and what runs here instead:
//   - Horn draws its coordinate order from an unseeded thread_rng (horn.rs:84-86), so two
//     reference runs differ.  Here index t is floor(m v_t), v_t = (x_t >> 9) 2^-23 (rand 0.8's
//     f32 draw in [0, 1)), x_t the high 32 bits of the t-th SplitMix64 output from seed
//     kHornSeed.  Every call uses the same order.
//   - Eigenvectors are defined up to a unit factor, and nalgebra's symmetric_eigen returns the
//     eigenpairs in an order of its own; both follow its internal conventions.  Here the
//     eigenvalues ascend and each eigenvector's first nonzero entry is real and positive
//     (dense::hermitian_eigen).  Both choices reach the result: Long reads row imax of the
//     eigenvector matrix, imax being the largest eigenvalue's position in that order, and takes
//     every eigenvector's phase there; Horn's drive turns by one global phase with its
//     eigenvector, which changes camax (a sum of |re| and |im|) and so the amplitude scale.
//   - symmetric_eigen reads only the lower triangle and the real diagonal of Long's R, which is
//     not Hermitian; hermitian_eigen reads the same part.
// Amplitude and phase are written as the reference does: amp *= |q_j| / camax(q), phase =
// arg q_j, camax being the largest |re| + |im| (nalgebra 0.27.1).
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

constexpr int kMatThreads = 256;
constexpr int kHornThreads = 1024;
constexpr int kHornRepeat = 100;      // horn.rs:18 (REPEAT_SDP)
constexpr double kHornLambda = 0.8;   // horn.rs:19 (LAMBDA_SDP)
constexpr double kHornAlpha = 1e-5;   // horn.rs:20 (TIKHONOV_DEFAULT)
constexpr uint64_t kHornSeed = 0x243F6A8885A308D3ull;

using cd = std::complex<double>;

__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Sum over the block (blockDim.x a multiple of 32, at most 1024), valid in thread 0.
__device__ double2 block_sum2(double2 v, double2* red) {
    v = warp_sum2(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? red[lane] : make_double2(0.0, 0.0);
        v = warp_sum2(v);
    }
    return v;
}

// out[i m + k] = sum_j G_ij w_j conj(G_kj) (w = 1 if null) for k <= i, the upper triangle its
// conjugate: K = G G^H, or G S^-1 G^H with w = 1 / sigma^2.  Block (k, i).
__global__ void __launch_bounds__(kMatThreads)
gram_kernel(const float2* __restrict__ g, int64_t n, int m, const double* __restrict__ w,
            double2* __restrict__ out) {
    __shared__ double2 red[32];
    const int k = blockIdx.x, i = blockIdx.y;
    if (k > i) return;
    const float2* gi = g + static_cast<int64_t>(i) * n;
    const float2* gk = g + static_cast<int64_t>(k) * n;
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const double2 a = make_double2(gi[j].x, gi[j].y), b = make_double2(gk[j].x, gk[j].y);
        const double s = w ? w[j] : 1.0;
        // a conj(b) s
        acc.x += s * (a.x * b.x + a.y * b.y);
        acc.y += s * (a.y * b.x - a.x * b.y);
    }
    acc = block_sum2(acc, red);
    if (threadIdx.x == 0) {
        out[static_cast<int64_t>(i) * m + k] = acc;
        out[static_cast<int64_t>(k) * m + i] = make_double2(acc.x, -acc.y);
    }
}

// Row sums d_i = sum_j G_ij (long.rs:61, nalgebra's column_sum).  Block i.
__global__ void __launch_bounds__(kMatThreads)
row_sum_kernel(const float2* __restrict__ g, int64_t n, double2* __restrict__ out) {
    __shared__ double2 red[32];
    const float2* gi = g + static_cast<int64_t>(blockIdx.x) * n;
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        acc.x += gi[j].x;
        acc.y += gi[j].y;
    }
    acc = block_sum2(acc, red);
    if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// inv_sig2_j = 1 / sigma_j^2, sigma_j^2 = sum_i |G_ij| amps_i / m (long.rs:72-83); 0 where
// sigma_j is 0, which the host rejects.  One thread per source.
__global__ void long_sigma_kernel(const float2* __restrict__ g, int64_t n, int m,
                                  const float* __restrict__ amps, double* __restrict__ inv_sig2) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int i = 0; i < m; ++i) {
        const float2 v = g[static_cast<int64_t>(i) * n + j];
        s += hypot(static_cast<double>(v.x), static_cast<double>(v.y)) * amps[i];
    }
    s /= m;
    inv_sig2[j] = s > 0.0 ? 1.0 / s : 0.0;
}

// q_j = w_j sum_i conj(G_ij) y_i (w = 1 if null).  One thread per source.
__global__ void backproject_kernel(const float2* __restrict__ g, int64_t n, int m,
                                   const double2* __restrict__ y, const double* __restrict__ w,
                                   double2* __restrict__ q) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double2 acc = make_double2(0.0, 0.0);
    for (int i = 0; i < m; ++i) {
        const float2 v = g[static_cast<int64_t>(i) * n + j];
        const double2 b = y[i];
        acc.x += v.x * b.x + v.y * b.y;
        acc.y += v.x * b.y - v.y * b.x;
    }
    const double s = w ? w[j] : 1.0;
    q[j] = make_double2(acc.x * s, acc.y * s);
}

// Horn's SDP by block-coordinate descent (horn.rs:84-117) in one block, in f32 like the
// reference: x (m x m, row-major, identity on entry) is updated in place, one coordinate idx[t]
// per step.  Step t with ii = idx[t]: c = column ii of mm without row ii; xb = x' c over the
// rows and columns other than ii; gamma = Re(xb^H c); row and column ii of x (but not x_ii)
// become -sqrt(lambda / gamma) xb (its conjugate in the row) if gamma > 0, else zero.  The
// steps are invariant to the scale of mm, which the host normalises to a largest entry of 1.
__global__ void __launch_bounds__(kHornThreads)
horn_sdp_kernel(int m, const float2* __restrict__ mm, const int* __restrict__ idx,
                int64_t steps, float lambda, float2* __restrict__ x) {
    extern __shared__ float2 shf[];
    float2* col = shf;     // m: column ii of mm, 0 at ii
    float2* xb = shf + m;  // m: x' c, 0 at ii
    __shared__ float s_scale;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t t = 0; t < steps; ++t) {
        const int ii = idx[t];
        for (int r = threadIdx.x; r < m; r += blockDim.x)
            col[r] = r == ii ? make_float2(0.f, 0.f) : mm[static_cast<int64_t>(r) * m + ii];
        __syncthreads();
        for (int r = warp; r < m; r += nw) {
            float2 acc = make_float2(0.f, 0.f);
            if (r != ii) {
                const float2* xr = x + static_cast<int64_t>(r) * m;
                for (int c = lane; c < m; c += 32) {
                    const float2 a = xr[c], b = col[c];
                    acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
                    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
                    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
                }
            }
            if (lane == 0) xb[r] = acc;
        }
        __syncthreads();
        if (warp == 0) {  // gamma = Re(sum_r conj(xb_r) c_r)
            float gp = 0.f;
            for (int r = lane; r < m; r += 32) gp = fmaf(xb[r].x, col[r].x, fmaf(xb[r].y, col[r].y, gp));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) gp += __shfl_xor_sync(0xffffffffu, gp, o);
            if (lane == 0) s_scale = gp > 0.f ? -sqrtf(lambda / gp) : 0.f;
        }
        __syncthreads();
        const float sc = s_scale;
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
            if (r == ii) continue;
            const float2 v = make_float2(xb[r].x * sc, xb[r].y * sc);
            x[static_cast<int64_t>(r) * m + ii] = v;
            x[static_cast<int64_t>(ii) * m + r] = make_float2(v.x, -v.y);
        }
        __syncthreads();
    }
}

unsigned blocks_for(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// The coordinate order of the Horn SDP (see the file comment).
std::vector<int> horn_indices(int m, int64_t steps) {
    std::vector<int> idx(static_cast<size_t>(steps));
    uint64_t state = kHornSeed;
    for (int64_t t = 0; t < steps; ++t) {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const uint32_t x = static_cast<uint32_t>(z >> 32);
        const float v = static_cast<float>(x >> 9) * (1.0f / 8388608.0f);
        idx[t] = std::min(static_cast<int>(static_cast<float>(m) * v), m - 1);
    }
    return idx;
}

std::mutex g_mat_mu;
cudaStream_t g_mat_stream = nullptr;
int g_mat_device = -1;

}  // namespace


int solve_matrix(int kind, int st, float* src, const float* k, const float* atten, int64_t n,
                 const float* foci, const float* amps, int64_t m, std::string* err) {
    const char* name = kind == MATRIX_HORN ? "Horn" : "Long";
    if (kind != MATRIX_HORN && kind != MATRIX_LONG) {
        *err = "unknown matrix optimizer";
        return -1;
    }
    if (m > kMatrixMaxFoci) {
        *err = std::string(name) + ": too many foci (" + std::to_string(m) + " > " +
               std::to_string(kMatrixMaxFoci) + ")";
        return -1;
    }
    if (n == 0) return 0;
    if (m == 0) {  // the reference takes imax() of an empty eigenvalue vector and panics
        *err = std::string(name) + ": no foci";
        return -1;
    }
    const int stride = source_stride(st);
    const int iamp = st == SRC_T4010A1 ? 6 : 3;
    const int iphase = st == SRC_T4010A1 ? 7 : 4;
    const int mi = static_cast<int>(m);
    std::lock_guard<std::mutex> lock(g_mat_mu);
    cudaError_t e;
    auto fail = [&](const char* what) {
        *err = std::string(name) + ": " + what + ": " + cudaGetErrorString(e);
        return -1;
    };
    if (!g_mat_stream) {
        int count = 0;
        e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            *err = "no CUDA device available; this library has no CPU path";
            return -1;
        }
        if ((e = cudaGetDevice(&g_mat_device)) != cudaSuccess) return fail("cudaGetDevice");
        if ((e = cudaStreamCreateWithFlags(&g_mat_stream, cudaStreamNonBlocking)) != cudaSuccess) {
            g_mat_stream = nullptr;
            return fail("cudaStreamCreate");
        }
    }
    DeviceGuard dg;  // the solver's device while it runs; the caller's again on return
    if ((e = dg.set(g_mat_device)) != cudaSuccess) return fail("cudaSetDevice");
    cudaStream_t s = g_mat_stream;
    // horn.rs:74-76, long.rs:51-53: phases zeroed, G from the zero-phase sources
    std::vector<float> raw(src, src + n * stride);
    for (int64_t j = 0; j < n; ++j) raw[j * stride + iphase] = 0.f;
    const int64_t steps = kind == MATRIX_HORN ? m * kHornRepeat : 0;

    // device block: raw | k | atten | foci | amps | G | packed | K (m x m) | X (m x m) | y (m) |
    //               rowsum (m) | inv_sig2 (n) | q (n) | idx (steps)
    auto a256 = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += a256(bytes ? bytes : 1);
        return o;
    };
    const size_t o_raw = take(4 * n * stride), o_k = take(4 * n), o_at = take(4 * n),
                 o_foci = take(12 * m), o_amps = take(4 * m), o_g = take(8 * m * n),
                 o_pk = take(48 * n), o_kk = take(16 * m * m), o_x = take(16 * m * m),
                 o_y = take(16 * m), o_rs = take(16 * m), o_is = take(8 * n), o_q = take(16 * n),
                 o_idx = take(4 * steps);
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
    if ((e = cudaMemcpyAsync(d + o_raw, raw.data(), 4 * n * stride, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_k, k, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_at, atten, 4 * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_foci, foci, 12 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d + o_amps, amps, 4 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return fail("upload");
    if ((e = launch_build_g(st, F(o_raw), F(o_k), F(o_at), n, F(o_foci), m, F2(o_g), d + o_pk, s)) !=
        cudaSuccess)
        return fail("G");
    const dim3 gram_grid(static_cast<unsigned>(m), static_cast<unsigned>(m));
    const size_t mm = static_cast<size_t>(m) * m;
    auto to_cd = [](const std::vector<double>& v) {
        std::vector<cd> c(v.size() / 2);
        for (size_t i = 0; i < c.size(); ++i) c[i] = cd(v[2 * i], v[2 * i + 1]);
        return c;
    };
    auto from_cd = [](const std::vector<cd>& c) {
        std::vector<double> v(2 * c.size());
        for (size_t i = 0; i < c.size(); ++i) {
            v[2 * i] = c[i].real();
            v[2 * i + 1] = c[i].imag();
        }
        return v;
    };
    std::vector<double> h(2 * mm);
    double* d_w = nullptr;  // back-projection weights (Long: 1 / sigma^2)

    if (kind == MATRIX_HORN) {
        // K = G G^H; MM = a^2 P (K + a^2 I)^-1 P
        gram_kernel<<<gram_grid, kMatThreads, 0, s>>>(F2(o_g), n, mi, nullptr, D2(o_kk));
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(h.data(), d + o_kk, 16 * mm, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("K");
        std::vector<cd> a = to_cd(h), ainv;
        const double a2 = kHornAlpha * kHornAlpha;
        for (int i = 0; i < mi; ++i) a[i * mi + i] += a2;
        if (!dense::hpd_inverse(a, ainv, mi)) {
            *err = std::string(name) + ": G G^H + a^2 I is not positive definite";
            return -1;
        }
        // MM in f32, scaled to a largest |re| or |im| of 1 (the SDP steps do not see the scale)
        std::vector<cd> mmat(mm);
        double mmax = 0.0;
        for (int i = 0; i < mi; ++i)
            for (int c = 0; c < mi; ++c) {
                mmat[i * mi + c] = a2 * static_cast<double>(amps[i]) * ainv[i * mi + c] *
                                   static_cast<double>(amps[c]);
                mmax = std::max(mmax, std::max(std::fabs(mmat[i * mi + c].real()),
                                               std::fabs(mmat[i * mi + c].imag())));
            }
        if (!(mmax > 0.0) || !std::isfinite(mmax)) {
            *err = std::string(name) + ": the SDP matrix is zero or not finite";
            return -1;
        }
        std::vector<float> mmf(2 * mm), xf(2 * mm, 0.f);
        for (size_t i = 0; i < mm; ++i) {
            mmf[2 * i] = static_cast<float>(mmat[i].real() / mmax);
            mmf[2 * i + 1] = static_cast<float>(mmat[i].imag() / mmax);
        }
        for (int i = 0; i < mi; ++i) xf[2 * (static_cast<size_t>(i) * mi + i)] = 1.f;
        const std::vector<int> idx = horn_indices(mi, steps);
        if ((e = cudaMemcpyAsync(d + o_kk, mmf.data(), 8 * mm, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d + o_x, xf.data(), 8 * mm, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d + o_idx, idx.data(), 4 * steps, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return fail("upload MM");
        const size_t shm = 2 * static_cast<size_t>(m) * sizeof(float2);
        horn_sdp_kernel<<<1, kHornThreads, shm, s>>>(mi, F2(o_kk), reinterpret_cast<int*>(d + o_idx),
                                                     steps, static_cast<float>(kHornLambda), F2(o_x));
        count_launch();
        std::vector<float> xo(2 * mm);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(xo.data(), d + o_x, 8 * mm, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("SDP");
        for (size_t i = 0; i < 2 * mm; ++i) h[i] = xo[i];
        // horn.rs:119-121: u = principal eigenvector of X; q = G_pinv P u = G^H (K + a^2 I)^-1 P u
        std::vector<cd> xm = to_cd(h), v;
        std::vector<double> lam;
        dense::hermitian_eigen(xm, mi, lam, v);
        const int imax = static_cast<int>(std::max_element(lam.begin(), lam.end()) - lam.begin());
        std::vector<cd> y(m, cd(0.0, 0.0));
        for (int i = 0; i < mi; ++i)
            for (int c = 0; c < mi; ++c)
                y[i] += ainv[i * mi + c] * (static_cast<double>(amps[c]) * v[c * mi + imax]);
        const std::vector<double> yh = from_cd(y);
        if ((e = cudaMemcpyAsync(d + o_y, yh.data(), 16 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return fail("upload y");
    } else {
        // long.rs:59-64: d = row sums, R = K diag(amps / d)
        gram_kernel<<<gram_grid, kMatThreads, 0, s>>>(F2(o_g), n, mi, nullptr, D2(o_kk));
        row_sum_kernel<<<static_cast<unsigned>(m), kMatThreads, 0, s>>>(F2(o_g), n, D2(o_rs));
        long_sigma_kernel<<<blocks_for(n, 256), 256, 0, s>>>(F2(o_g), n, mi, F(o_amps), D(o_is));
        count_launch(3);
        std::vector<double> rs(2 * m), is(n);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(h.data(), d + o_kk, 16 * mm, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(rs.data(), d + o_rs, 16 * m, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(is.data(), d + o_is, 8 * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("K");
        for (int64_t j = 0; j < n; ++j)
            if (!(is[j] > 0.0) || !std::isfinite(is[j])) {
                // the reference's QR solve of a singular g^H g fails and unwraps
                *err = std::string(name) + ": source " + std::to_string(j) +
                       " has sigma = 0 (no field at any focus)";
                return -1;
            }
        const std::vector<cd> kk = to_cd(h), dsum = to_cd(rs);
        std::vector<cd> r(mm);
        for (int i = 0; i < mi; ++i)
            for (int c = 0; c < mi; ++c)
                r[i * mi + c] = kk[i * mi + c] * (static_cast<double>(amps[c]) / dsum[c]);
        // long.rs:66-70: eigenvector matrix row imax -> focus phases
        std::vector<cd> v;
        std::vector<double> lam;
        dense::hermitian_eigen(r, mi, lam, v);
        const int imax = static_cast<int>(std::max_element(lam.begin(), lam.end()) - lam.begin());
        std::vector<cd> f(m);
        for (int c = 0; c < mi; ++c)
            f[c] = static_cast<double>(amps[c]) * std::exp(cd(0.0, std::arg(v[imax * mi + c])));
        // long.rs:85-97 by Woodbury: y = (I + G S^-1 G^H)^-1 f, q = S^-1 G^H y
        gram_kernel<<<gram_grid, kMatThreads, 0, s>>>(F2(o_g), n, mi, D(o_is), D2(o_kk));
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(h.data(), d + o_kk, 16 * mm, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("W");
        std::vector<cd> wm = to_cd(h);
        for (int i = 0; i < mi; ++i) wm[i * mi + i] += 1.0;
        if (!dense::hpd_solve(wm, f, mi)) {
            *err = std::string(name) + ": I + G S^-1 G^H is not positive definite";
            return -1;
        }
        const std::vector<double> yh = from_cd(f);
        if ((e = cudaMemcpyAsync(d + o_y, yh.data(), 16 * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return fail("upload y");
        d_w = D(o_is);
    }
    backproject_kernel<<<blocks_for(n, 256), 256, 0, s>>>(F2(o_g), n, mi, D2(o_y), d_w, D2(o_q));
    count_launch();
    std::vector<double> qh(2 * n);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(qh.data(), d + o_q, 16 * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail("q");
    // horn.rs:122-128, long.rs:99-104
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
