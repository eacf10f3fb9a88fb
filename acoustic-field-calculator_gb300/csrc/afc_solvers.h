// Multi-focus phase solvers on the GPU: transfer matrix G, GS-PAT, GS and naive linear
// synthesis (acoustic-field-optimizer/src/multiple_foci/).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

namespace afc {

enum SolverKind : int { SOLVER_GSPAT = 0, SOLVER_GS = 1, SOLVER_NAIVE = 2, SOLVER_GREEDY = 3 };

// Largest candidate-phase count of the greedy solver (one thread per candidate).
constexpr int kGreedyMaxDiv = 1024;

// Nonlinear least-squares solvers (nls.cu) and their focus limit (their small dense systems
// are 2m x 2m).
enum NlsKind : int { NLS_GRADIENT_DESCENT = 0, NLS_GAUSS_NEWTON = 1, NLS_LM = 2 };
constexpr int64_t kNlsMaxFoci = 256;

// REPEAT of gs_pat.rs:17 and gs.rs:17.
constexpr int kSolverRepeat = 100;
// Largest focus count the single-block iteration kernels accept.
constexpr int64_t kSolverMaxFoci = 4096;

// Device workspace (bytes, 256-aligned pieces) for n sources and m foci.
size_t solver_workspace_bytes(int64_t n, int64_t m);

// Everything on the device: sources in the ABI layout (d_raw, stride 9 or 6 floats), d_k,
// d_atten, foci (3 floats each), target amplitudes.  Writes (amp, phase) per source to d_out
// (2n floats).  `ws` must hold solver_workspace_bytes(n, m) bytes, 256-byte aligned.
cudaError_t launch_solver(int kind, int st, const float* d_raw, const float* d_k,
                          const float* d_atten, int64_t n, const float* d_foci,
                          const float* d_amps, int64_t m, int repeat, float* d_out, void* ws,
                          cudaStream_t s);

// Build the transfer matrix G (row-major m x n, float2) for the sources' current amplitudes
// and zero phase into d_g; `ws_packed` holds 48 n bytes.
cudaError_t launch_build_g(int st, const float* d_raw, const float* d_k, const float* d_atten,
                           int64_t n, const float* d_foci, int64_t m, float2* d_g,
                           void* ws_packed, cudaStream_t s);

// Greedy phase choice (combination/greedy.rs:39-83) on the device: G is built as for the other
// solvers, then one block takes the sources in order.  cand / cand_arg: the div candidate
// phasors and their arguments (computed on the host).  Writes (amp, phase) per source to d_out.
cudaError_t launch_greedy(int st, const float* d_raw, const float* d_k, const float* d_atten,
                          int64_t n, const float* d_foci, const float* d_amps, int64_t m,
                          const float2* d_cand, const float* d_cand_arg, int div, float* d_out,
                          void* ws, cudaStream_t s);

// Host-level: uploads, solves, and writes amp / phase into the host source array `src`
// (ABI layout) in place.  phase_div: candidate phases of SOLVER_GREEDY (1..kGreedyMaxDiv).
// Returns 0 on success, else fills *err.
int solve_multi_focus(int kind, int st, float* src, const float* k, const float* atten,
                      int64_t n, const float* foci, const float* amps, int64_t m,
                      std::string* err, int phase_div = 0);

// Gradient descent, Gauss-Newton or Levenberg-Marquardt phase retrieval
// (multiple_foci/nls/*.rs) on the device; writes the phases into the host source array `src`
// (ABI layout) in place, amplitudes unchanged.  Returns 0 on success, else fills *err.
int solve_nls(int kind, int st, float* src, const float* k, const float* atten, int64_t n,
              const float* foci, const float* amps, int64_t m, std::string* err);

// Acoustic power optimization (multiple_foci/nls/apo.rs) on the device, regularisation lambda;
// writes amplitudes and phases into `src` in place.  n <= 65535 (its n x n matrix).
int solve_apo(int st, float* src, const float* k, const float* atten, int64_t n,
              const float* foci, const float* amps, int64_t m, float lambda, std::string* err);

// Matrix optimizers (multiple_foci/matrix/{horn,long}.rs) on the device, m <= kMatrixMaxFoci
// (their m x m systems and Horn's m x 100 sequential SDP steps); write amplitudes and phases
// into `src` in place.  Returns 0 on success, else fills *err.
enum MatrixKind : int { MATRIX_HORN = 0, MATRIX_LONG = 1 };
constexpr int64_t kMatrixMaxFoci = 256;
int solve_matrix(int kind, int st, float* src, const float* k, const float* atten, int64_t n,
                 const float* foci, const float* amps, int64_t m, std::string* err);

}  // namespace afc
