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


def gs_f64(st, sources, k, atten, foci, amps, repeat=100):
    return _solver("oracle_gs_f64", st, sources, k, atten, foci, amps, repeat)


def naive_f64(st, sources, k, atten, foci, amps):
    return _solver("oracle_naive_f64", st, sources, k, atten, foci, amps)


def max_threads() -> int:
    return int(lib().oracle_max_threads())
