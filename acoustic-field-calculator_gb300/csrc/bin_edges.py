"""Derivation of the exact directivity-bin thresholds on cos(theta) used by the field kernels
(kBinCos in propagate.cuh).

The T4010A1 directivity (acoustic-field-calculator/src/core/wave_sources/t4010a1.rs:107-120)
takes its bin from the f32 theta as i = ceil(theta / ANGLE_DIV) (0 -> 1.0, > 9 -> 0.0), with
theta = f32::acos(c) and ANGLE_DIV = f32(pi) / 18 in f32.  Rust's f32::acos is the platform
libm's acosf (glibc on Linux), which is not correctly rounded: near a bin edge its last-ulp
rounding decides the bin, and a pair there contributes a whole directivity jump (up to 17 % of
its term).  The thresholds therefore follow glibc's acosf itself, called here through ctypes.
theta is monotone non-increasing in c, and f32 division and ceil are monotone, so the bin is a
step function of the float c: for b = 1..10 there is a largest float L_b with bin(L_b) >= b,
and for every float c

    bin(c) (clipped to 0..10) = #{b : c <= L_b}        (a NaN c compares false: bin 0)

This script finds L_b by bisection over the ordered float32 values of [-1, 1], then checks the
identity exhaustively on 2^17 floats around every threshold (which also checks that acosf is
monotone there).  Run: python bin_edges.py
"""
import ctypes
import ctypes.util
import numpy as np

ANGLE_DIV = np.float32(np.float32(np.pi) / np.float32(18.0))

_LIBM = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_LIBM.acosf.argtypes = [ctypes.c_float]
_LIBM.acosf.restype = ctypes.c_float


def acosf_libm(c):
    """The platform libm's acosf, elementwise (float32 in, float32 out)."""
    c = np.asarray(c, dtype=np.float32)
    f = _LIBM.acosf
    return np.fromiter((f(v) for v in c.ravel().tolist()), dtype=np.float32,
                       count=c.size).reshape(c.shape)


def _key_to_f32(key):
    """Ordered integer key -> float32 (key 0 is +0.0; negative keys are negative floats)."""
    key = np.asarray(key, dtype=np.int64)
    bits = np.where(key >= 0, key, (-key) | 0x80000000).astype(np.uint32)
    return bits.view(np.float32)


def _f32_to_key(x):
    bits = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.int64)
    return np.where(bits & 0x80000000, -(bits & 0x7FFFFFFF), bits)


def ref_bin(c):
    """The reference's bin for float32 cos(theta) values, clipped to 0..10 (NaN -> 0)."""
    c = np.asarray(c, dtype=np.float32)
    with np.errstate(invalid="ignore"):
        theta = acosf_libm(c)
        q = np.ceil(theta / ANGLE_DIV)  # float32 division, round to nearest
    q = np.where(np.isnan(q), 0.0, q)
    return np.clip(q, 0, 10).astype(np.int64)


def thresholds():
    lo_key, hi_key = int(_f32_to_key(np.float32(-1.0))), int(_f32_to_key(np.float32(1.0)))
    out = []
    for b in range(1, 11):
        lo, hi = lo_key, hi_key  # invariant: bin(lo) >= b, bin(hi) < b
        assert ref_bin(_key_to_f32(lo)) >= b and ref_bin(_key_to_f32(hi)) < b
        while hi - lo > 1:
            mid = (lo + hi) // 2
            if ref_bin(_key_to_f32(mid)) >= b:
                lo = mid
            else:
                hi = mid
        out.append(np.float32(_key_to_f32(lo)))
    return out


def bin_from_thresholds(c, ths):
    c = np.asarray(c, dtype=np.float32)
    return sum((c <= t).astype(np.int64) for t in ths)


def check(ths, window=1 << 16):
    for t in ths:
        k = int(_f32_to_key(t))
        keys = np.arange(max(k - window, int(_f32_to_key(np.float32(-1.0)))),
                         min(k + window, int(_f32_to_key(np.float32(1.0)))) + 1)
        c = _key_to_f32(keys)
        assert np.array_equal(ref_bin(c), bin_from_thresholds(c, ths)), t
    rng = np.random.default_rng(0)
    c = rng.uniform(-1.0, 1.0, 1 << 20).astype(np.float32)
    assert np.array_equal(ref_bin(c), bin_from_thresholds(c, ths))
    return True


if __name__ == "__main__":
    ths = thresholds()
    check(ths)
    for b, t in enumerate(ths, 1):
        print(f"    {t.view(np.uint32):#010x}u,  // L_{b} = {float(t):.9g}")
