"""ctypes bindings of the oracle (oracle/afc_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs import this module,
always as the checker or the timed CPU baseline, never as part of the product path.

Parity unpinned: the reference (Rust) cannot be built on these machines and ships no golden
vectors for this path; see the header of afc_oracle.c for what the oracle restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_float, c_double, c_int, c_int64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_afc.so")

SRC_SPHERE, SRC_T4010A1 = 0, 1
FIELD_PRESSURE, FIELD_POWER, FIELD_COMPLEX = 0, 1, 2

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (a second or two)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "afc_oracle.c")
        ):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = POINTER(c_float)
        dp = POINTER(c_double)
        L.oracle_sound_speed.argtypes = [c_float]
        L.oracle_sound_speed.restype = c_float
        L.oracle_attenuation_coef.argtypes = [c_float] * 5
        L.oracle_attenuation_coef.restype = c_float
        L.oracle_wavenum_atten.argtypes = [c_float, c_float, fp, fp]
        L.oracle_directivity_t4010a1.argtypes = [c_float]
        L.oracle_directivity_t4010a1.restype = c_float
        L.oracle_directivity_t4010a1_f64.argtypes = [c_double]
        L.oracle_directivity_t4010a1_f64.restype = c_double
        L.oracle_directivity_bin.argtypes = [c_float]
        L.oracle_directivity_bin.restype = c_int
        L.oracle_theta_of_cos.argtypes = [c_float]
        L.oracle_theta_of_cos.restype = c_float
        L.oracle_bins_of_cos.argtypes = [fp, c_int64, POINTER(c_int)]
        L.oracle_propagate.argtypes = [c_int, fp, c_float, c_float, c_float, c_float, c_float, fp]
        L.oracle_field_f32.argtypes = [c_int, fp, fp, fp, c_int64, fp, c_int64, c_int, fp, c_int]
        L.oracle_field_accurate_f32.argtypes = L.oracle_field_f32.argtypes
        L.oracle_field_f64.argtypes = [c_int, fp, fp, fp, c_int64, fp, c_int64, dp, c_int]
        L.oracle_axis_count.argtypes = [c_float, c_float, c_float]
        L.oracle_axis_count.restype = c_int64
        L.oracle_grid_points.argtypes = [c_int, fp, fp, c_float, POINTER(c_int), fp]
        L.oracle_grid_points.restype = c_int64
        L.oracle_focal_point.argtypes = [c_int, fp, c_int64, c_float, c_float, c_float, c_float]
        L.oracle_bessel_beam.argtypes = [c_int, fp, c_int64, c_float] + [c_float] * 7
        L.oracle_greedy_f32.argtypes = [c_int, fp, fp, fp, c_int64, fp, fp, c_int64, c_int]
        L.oracle_nls_f64.argtypes = [c_int, c_int, fp, fp, fp, c_int64, fp, fp, c_int64]
        L.oracle_apo_f64.argtypes = [c_int, fp, fp, fp, c_int64, fp, fp, c_int64, c_float]
        L.oracle_build_g_f32.argtypes = [c_int, fp, fp, fp, c_int64, fp, c_int64, fp]
        L.oracle_build_g_f64.argtypes = [c_int, fp, fp, fp, c_int64, fp, c_int64, dp, c_int]
        L.oracle_gspat_f64.argtypes = [c_int, fp, fp, fp, c_int64, fp, fp, c_int64, c_int, dp]
        L.oracle_gspat_f32.argtypes = L.oracle_gspat_f64.argtypes
        L.oracle_gs_f64.argtypes = L.oracle_gspat_f64.argtypes
        L.oracle_naive_f64.argtypes = [c_int, fp, fp, fp, c_int64, fp, fp, c_int64, dp]
        L.oracle_max_threads.restype = c_int
        L.oracle_set_acos_mode.argtypes = [c_int]
        _lib = L
    return _lib


ACOS_LIBM, ACOS_CORRECTLY_ROUNDED = 0, 1


def set_acos_mode(mode: int) -> None:
    """0: the platform libm's acosf (what the reference calls); 1: acos correctly rounded to
    f32 (what the GPU's near-bin-edge path computes).  They differ only where theta lies
    within one ulp of a directivity bin edge."""
    lib().oracle_set_acos_mode(mode)


class acos_mode:
    """Context manager that switches the oracle's acos rounding."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        set_acos_mode(self.mode)

    def __exit__(self, *exc):
        set_acos_mode(ACOS_LIBM)


def _f(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(POINTER(c_float))


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(POINTER(c_double))


def sound_speed(t: float) -> float:
    return float(lib().oracle_sound_speed(t))


def attenuation_coef(freq, hr, ps, ps0, t) -> float:
    return float(lib().oracle_attenuation_coef(freq, hr, ps, ps0, t))


def wavenum_atten(temperature: float, freq: float):
    k = c_float()
    a = c_float()
    lib().oracle_wavenum_atten(temperature, freq, ctypes.byref(k), ctypes.byref(a))
    return k.value, a.value


def directivity(theta: float) -> float:
    return float(lib().oracle_directivity_t4010a1(theta))


def directivity_f64(theta: float) -> float:
    return float(lib().oracle_directivity_t4010a1_f64(theta))


def directivity_bin(theta: float) -> int:
    """The reference's bin index for theta (NaN -> 0, clipped to 10)."""
    return int(lib().oracle_directivity_bin(theta))


def theta_of_cos(c: float) -> float:
    """acos(c) in f32 as the reference computes it (per the acos mode)."""
    return float(lib().oracle_theta_of_cos(c))


def bins_of_cos(c) -> np.ndarray:
    """The reference's directivity bin of acos(c) for each float32 c (per the acos mode)."""
    c = np.ascontiguousarray(c, dtype=np.float32)
    out = np.empty(len(c), dtype=np.int32)
    lib().oracle_bins_of_cos(_f(c), len(c), out.ctypes.data_as(POINTER(c_int)))
    return out


def _src_args(st, sources, k, atten):
    sources = np.ascontiguousarray(sources, dtype=np.float32)
    k = np.ascontiguousarray(k, dtype=np.float32)
    atten = np.ascontiguousarray(atten, dtype=np.float32)
    n = len(k)
    assert sources.size == n * (9 if st == SRC_T4010A1 else 6)
    return sources, k, atten, n


def field_f32(st, sources, k, atten, points, field=FIELD_COMPLEX, nthreads=0, accurate=False):
    """The reference CPU calculator on explicit points (float32 m x 3)."""
    sources, k, atten, n = _src_args(st, sources, k, atten)
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    m = pts.shape[0]
    out = np.empty(m * (2 if field == FIELD_COMPLEX else 1), dtype=np.float32)
    fn = lib().oracle_field_accurate_f32 if accurate else lib().oracle_field_f32
    fn(st, _f(sources), _f(k), _f(atten), n, _f(pts), m, field, _f(out), nthreads)
    if field == FIELD_COMPLEX:
        return out.view(np.complex64)
    return out


def field_f64(st, sources, k, atten, points, nthreads=0):
    """Complex field in float64 (error reference)."""
    sources, k, atten, n = _src_args(st, sources, k, atten)
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    m = pts.shape[0]
    out = np.empty(2 * m, dtype=np.float64)
    lib().oracle_field_f64(st, _f(sources), _f(k), _f(atten), n, _f(pts), m, _d(out), nthreads)
    return out.view(np.complex128)


def axis_count(lo, hi, res) -> int:
    return int(lib().oracle_axis_count(lo, hi, res))


def grid_points(dim, lo, hi, res, axes) -> np.ndarray:
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    ax = (c_int * 3)(*axes)
    m = lib().oracle_grid_points(dim, _f(lo), _f(hi), res, ax, None)
    out = np.empty((m, 3), dtype=np.float32)
    lib().oracle_grid_points(dim, _f(lo), _f(hi), res, ax, _f(out))
    return out


def focal_point(st, sources, sound_speed_, focus) -> np.ndarray:
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    n = s.size // (9 if st == SRC_T4010A1 else 6)
    lib().oracle_focal_point(st, _f(s), n, sound_speed_, *map(float, focus))
    return s


def bessel_beam(st, sources, sound_speed_, point, direction, theta) -> np.ndarray:
    """Sources with the Bessel-beam phases of bessel.rs:30-51 (f32)."""
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    n = s.size // (9 if st == SRC_T4010A1 else 6)
    lib().oracle_bessel_beam(st, _f(s), n, sound_speed_, *map(float, point),
                             *map(float, direction), float(theta))
    return s


def greedy_f32(st, sources, k, atten, foci, amps, phase_div=16) -> np.ndarray:
    """Sources with the greedy solver's phases (greedy.rs:39-83, f32)."""
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    k = np.ascontiguousarray(k, dtype=np.float32)
    atten = np.ascontiguousarray(atten, dtype=np.float32)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    amps = np.ascontiguousarray(amps, dtype=np.float32)
    lib().oracle_greedy_f32(st, _f(s), _f(k), _f(atten), len(k), _f(foci), _f(amps), len(amps),
                            int(phase_div))
    return s


NLS_GRADIENT_DESCENT, NLS_GAUSS_NEWTON, NLS_LM = 0, 1, 2


def nls_f64(kind, st, sources, k, atten, foci, amps) -> np.ndarray:
    """Sources with the phases of gradient descent / Gauss-Newton / LM (nls/*.rs, float64,
    dense formulas)."""
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    k = np.ascontiguousarray(k, dtype=np.float32)
    atten = np.ascontiguousarray(atten, dtype=np.float32)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    amps = np.ascontiguousarray(amps, dtype=np.float32)
    lib().oracle_nls_f64(kind, st, _f(s), _f(k), _f(atten), len(k), _f(foci), _f(amps),
                         len(amps))
    return s


def apo_f64(st, sources, k, atten, foci, amps, lambda_reg) -> np.ndarray:
    """Sources with APO's amplitudes and phases (nls/apo.rs, float64, dense R_i)."""
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    k = np.ascontiguousarray(k, dtype=np.float32)
    atten = np.ascontiguousarray(atten, dtype=np.float32)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    amps = np.ascontiguousarray(amps, dtype=np.float32)
    lib().oracle_apo_f64(st, _f(s), _f(k), _f(atten), len(k), _f(foci), _f(amps), len(amps),
                         float(lambda_reg))
    return s


def build_g_f32(st, sources, k, atten, foci) -> np.ndarray:
    sources, k, atten, n = _src_args(st, sources, k, atten)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    m = foci.shape[0]
    g = np.empty(2 * m * n, dtype=np.float32)
    lib().oracle_build_g_f32(st, _f(sources), _f(k), _f(atten), n, _f(foci), m, _f(g))
    return g.view(np.complex64).reshape(m, n)


def build_g_f64(st, sources, k, atten, foci, nthreads=0) -> np.ndarray:
    sources, k, atten, n = _src_args(st, sources, k, atten)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    m = foci.shape[0]
    g = np.empty(2 * m * n, dtype=np.float64)
    lib().oracle_build_g_f64(st, _f(sources), _f(k), _f(atten), n, _f(foci), m, _d(g), nthreads)
    return g.view(np.complex128).reshape(m, n)


def _solver(fn_name, st, sources, k, atten, foci, amps, repeat=None):
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1)
    k = np.ascontiguousarray(k, dtype=np.float32)
    atten = np.ascontiguousarray(atten, dtype=np.float32)
    n = len(k)
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    amps = np.ascontiguousarray(amps, dtype=np.float32)
    m = foci.shape[0]
    q = np.empty(2 * n, dtype=np.float64)
    fn = getattr(lib(), fn_name)
    args = [st, _f(s), _f(k), _f(atten), n, _f(foci), _f(amps), m]
    if repeat is not None:
        args.append(repeat)
    args.append(_d(q))
    fn(*args)
    return s, q.view(np.complex128)


def gspat_f64(st, sources, k, atten, foci, amps, repeat=100):
    """GS-PAT in float64; returns (updated sources, complex q)."""
    return _solver("oracle_gspat_f64", st, sources, k, atten, foci, amps, repeat)


def gspat_f32(st, sources, k, atten, foci, amps, repeat=100):
    """GS-PAT in f32 with the reference's operation order; returns (updated sources, q)."""
    return _solver("oracle_gspat_f32", st, sources, k, atten, foci, amps, repeat)


def gs_f64(st, sources, k, atten, foci, amps, repeat=100):
    return _solver("oracle_gs_f64", st, sources, k, atten, foci, amps, repeat)


def naive_f64(st, sources, k, atten, foci, amps):
    return _solver("oracle_naive_f64", st, sources, k, atten, foci, amps)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


# ------------------------------------------------------------------ matrix optimizers (float64)
#
# numpy restatements of acoustic-field-optimizer/src/multiple_foci/matrix/{horn,long}.rs in
# float64, following the reference's steps literally (SVD pseudo-inverse, I - G G_pinv by
# subtraction, QR solve of the normal equations).  Two things the reference leaves to chance or
# to nalgebra's internals are fixed here as the GPU library fixes them:
#   - Horn's coordinate order (an unseeded thread_rng in the reference): horn_indices;
#   - the eigenpairs' order (ascending eigenvalue, as eigh returns them) and each eigenvector's
#     unit factor: its first nonzero entry is real and positive (_phase_fixed).

HORN_SEED = 0x243F6A8885A308D3
_M64 = (1 << 64) - 1


def horn_indices(m: int, steps: int, seed: int = HORN_SEED) -> np.ndarray:
    """Coordinate t = floor(m v_t) in float32, v_t = (x_t >> 9) 2^-23 (rand 0.8's f32 draw in
    [0, 1)), x_t the high 32 bits of the t-th SplitMix64 output from `seed`."""
    out = np.empty(steps, dtype=np.int64)
    state = seed
    for t in range(steps):
        state = (state + 0x9E3779B97F4A7C15) & _M64
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        z ^= z >> 31
        v = np.float32((z >> 32) >> 9) * np.float32(1.0 / 8388608.0)
        out[t] = min(int(np.float32(m) * v), m - 1)
    return out


def _phase_fixed(v: np.ndarray) -> np.ndarray:
    """Columns scaled so that each one's first nonzero entry is real and positive (eigh's
    ascending eigenvalue order is the other half of the convention)."""
    v = v.copy()
    for j in range(v.shape[1]):
        nz = np.flatnonzero(v[:, j])
        if len(nz) == 0:
            continue
        a = v[nz[0], j]
        v[:, j] *= np.conj(a) / abs(a)
        v[nz[0], j] = abs(a)
    return v


def _matrix_setup(st, sources, k, atten, foci, amps):
    stride = 9 if st == SRC_T4010A1 else 6
    s = np.array(sources, dtype=np.float32, copy=True).reshape(-1, stride)
    s[:, 7 if st == SRC_T4010A1 else 4] = 0.0  # horn.rs:74-76, long.rs:51-53
    foci = np.ascontiguousarray(foci, dtype=np.float32).reshape(-1, 3)
    amps = np.ascontiguousarray(amps, dtype=np.float32).astype(np.float64)
    g = build_g_f64(st, s, k, atten, foci)
    return s, g, amps, stride


def _write_drive(st, s, q):
    """horn.rs:122-128, long.rs:99-104: amp *= |q_j| / camax(q) (largest |re| + |im|),
    phase = arg q_j."""
    iamp, iphase = (6, 7) if st == SRC_T4010A1 else (3, 4)
    max_coeff = np.max(np.abs(q.real) + np.abs(q.imag))
    s[:, iamp] = (s[:, iamp].astype(np.float64) * np.abs(q) / max_coeff).astype(np.float32)
    s[:, iphase] = np.angle(q).astype(np.float32)
    return s


def horn_mm_f64(g, amps, alpha=1e-5):
    """MM = P (I - G G_pinv) P with G_pinv = V diag(s / (s^2 + alpha^2)) U^H (horn.rs:60-69,
    83-84), and G_pinv itself."""
    u, sv, vh = np.linalg.svd(g, full_matrices=False)
    g_pinv = vh.conj().T @ np.diag(sv / (sv * sv + alpha * alpha)) @ u.conj().T
    p = np.diag(amps).astype(np.complex128)
    mm = p @ (np.eye(len(amps)) - g @ g_pinv) @ p
    return mm, g_pinv


def horn_sdp_f64(mm, idx, lam=0.8):
    """horn.rs:84-117: X = I, then one coordinate ii per step."""
    m = mm.shape[0]
    x = np.eye(m, dtype=np.complex128)
    for ii in idx:
        rest = np.r_[0:ii, ii + 1:m]
        xb = x[np.ix_(rest, rest)] @ mm[rest, ii]
        gamma = np.vdot(xb, mm[rest, ii])
        if gamma.real > 0:
            xb = xb * -np.sqrt(lam / gamma.real)
            x[ii, rest] = xb.conj()
            x[rest, ii] = xb
        else:
            x[ii, rest] = 0.0
            x[rest, ii] = 0.0
    return x


def horn_f64(st, sources, k, atten, foci, amps, repeat=100):
    """Horn (matrix/horn.rs:71-129) in float64; returns (updated sources, complex q)."""
    s, g, amps, stride = _matrix_setup(st, sources, k, atten, foci, amps)
    m = len(amps)
    mm, g_pinv = horn_mm_f64(g, amps)
    x = horn_sdp_f64(mm, horn_indices(m, m * repeat))
    w, v = np.linalg.eigh(x)
    u = _phase_fixed(v)[:, int(np.argmax(w))]
    q = g_pinv @ (amps * u)
    return _write_drive(st, s, q).reshape(-1), q


def long_f64(st, sources, k, atten, foci, amps):
    """Long (matrix/long.rs:48-105) in float64; returns (updated sources, complex q).
    symmetric_eigen reads R's lower triangle and real diagonal, as eigh (UPLO='L') does."""
    s, g, amps, stride = _matrix_setup(st, sources, k, atten, foci, amps)
    m, n = g.shape
    denomi = g.sum(axis=1)
    x = (amps[:, None] * g.conj() / denomi[:, None]).T
    r = g @ x
    w, v = np.linalg.eigh(r, UPLO="L")
    e_arg = np.angle(_phase_fixed(v)[int(np.argmax(w)), :])
    sigma = np.sqrt((np.abs(g) * amps[:, None]).sum(axis=0) / m)
    gg = np.vstack([g, np.diag(sigma).astype(np.complex128)])
    f = np.concatenate([amps * np.exp(1j * e_arg), np.zeros(n)])
    gtg = gg.conj().T @ gg
    gtf = gg.conj().T @ f
    qq, rr = np.linalg.qr(gtg)
    q = np.linalg.solve(rr, qq.conj().T @ gtf)
    return _write_drive(st, s, q).reshape(-1), q
