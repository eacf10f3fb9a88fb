"""Derivation of the cos(theta)-indexed directivity table of the field kernels
(dir_ctable.inc, used by directivity2_ctab in propagate.cuh).

The T4010A1 directivity (acoustic-field-calculator/src/core/wave_sources/t4010a1.rs:18-71,
107-120) is a cubic in theta inside each 10-degree bin.  The kernels avoid theta = acos(c),
whose square-root singularity at c = 1 costs a MUFU square root per pair: D is taken directly
as a function of c = cos(theta).  The c axis is cut into intervals of width 1/K (K = 128):
interval i covers c in [(i - BIAS)/K, (i - BIAS + 1)/K) (BIAS = 129, so that every c >= -1 has
an index of at least 1 and the kernels need no clamp), and within it the kernels evaluate a
cubic in x = c K - floor(c K) in [0, 1).  Each bin's function D_b(acos(c)) is analytic inside an
interval (bins 1..2, theta < 20 degrees, where c approaches the singularity, are the constant
1), so a cubic interpolating it at four Chebyshev nodes is within 1e-9 of it in float64.

A bin edge (the float thresholds L_b of bin_edges.py, b = 3..10: 20..90 degrees) splits the
interval that holds it.  Every interval therefore has two entries: 2 i for c > L (the upper
side, the smaller bin) and 2 i + 1 for c <= L, and the kernels take the side from the sign of
c - L (negedge[i] = -L; intervals without an edge store L = -1e30, so only entry 2 i is used).
Pairs whose fast c lies within kCTabMargin of L are recomputed exactly by the kernels' edge
path.  Intervals below -1/K give 0 (bin 10); entries from c = 1 on (a unit cosine rounded up,
or a non-unit direction, where the reference's acos is NaN and its bin 0) give 1.  The two
intervals around c = -1 carry the edge L = -1 (both sides 0): a point on a tilted source's back
axis can have the reference's f32 c rounded below -1, where its acos is NaN and D is 1, so such
pairs take the exact path too.

Writes dir_ctable.inc beside this script and checks, over every interval and side, the float32
Horner evaluation of the rounded coefficients against D_b(acos(c)) in float64.
Run: python dir_ctable.py
"""
import os

import numpy as np

from bin_edges import thresholds
from dir_table import ANGLE_DIV, reference_coefficients

K = 128
BIAS = 129           # index of the interval that starts at c = 0
SIZE = 512           # entries per side table (the kernels mask the index with SIZE - 1)
NO_EDGE = -1.0e30


def d_bin(b, c):
    """D_b(acos(c)) in float64 with the reference's float32 coefficients (bin b = 0..10+)."""
    c = np.asarray(c, dtype=np.float64)
    if b <= 2:
        return np.ones_like(c)
    if b >= 10:
        return np.zeros_like(c)
    a, bb, cc, dd = (np.float64(v) for v in reference_coefficients()[b])
    x = np.arccos(np.clip(c, -1.0, 1.0)) - (b - 1) * np.float64(ANGLE_DIV)
    return a + (bb + (cc + dd * x) * x) * x


def ref_bin_f64(c, ths):
    """Bin of c from the thresholds (bin = #{b : c <= L_b})."""
    return int(sum(1 for t in ths if c <= float(t)))


def fit(b, i):
    """Cubic coefficients (A, B, C, D) in x in [0, 1) of D_b on interval i, float64."""
    if b <= 2:
        return np.array([1.0, 0.0, 0.0, 0.0])
    if b >= 10:
        return np.zeros(4)
    nodes = 0.5 + 0.5 * np.cos((2 * np.arange(4) + 1) * np.pi / 8)  # Chebyshev nodes in [0, 1]
    c = ((i - BIAS) + nodes) / K
    y = d_bin(b, c)
    v = np.vander(nodes, 4, increasing=True)
    return np.linalg.solve(v, y)


def table():
    ths = thresholds()
    edges = [float(t) for t in ths[2:]]  # L_3 .. L_10: 20 .. 90 degrees
    negedge = np.full(SIZE, -NO_EDGE, dtype=np.float32)
    coef = np.zeros((2 * SIZE, 4), dtype=np.float64)
    bins = np.zeros((2 * SIZE,), dtype=np.int64)
    for i in range(SIZE):
        lo, hi = (i - BIAS) / K, (i - BIAS + 1) / K
        if hi <= 0 and lo < -1.0 / K:  # c < -1/K: theta beyond 90 degrees, bin 10
            bins[2 * i] = bins[2 * i + 1] = 10
            if lo <= -1.0 < hi or hi == -1.0:  # the back axis: edge at c = -1
                negedge[i] = np.float32(1.0)
            continue
        if lo >= 1.0:  # c >= 1: theta = 0 or the reference's acos is NaN, bin 0
            coef[2 * i] = coef[2 * i + 1] = (1.0, 0.0, 0.0, 0.0)
            continue
        inside = [e for e in edges if lo <= e < hi]
        assert len(inside) <= 1
        if inside:
            e = inside[0]
            negedge[i] = np.float32(-e)
            b_up = ref_bin_f64(np.nextafter(np.float32(e), np.float32(2)), ths)
            b_lo = ref_bin_f64(e, ths)
        else:
            b_up = b_lo = ref_bin_f64(np.float32(0.5 * (lo + hi)), ths)
        coef[2 * i], coef[2 * i + 1] = fit(b_up, i), fit(b_lo, i)
        bins[2 * i], bins[2 * i + 1] = b_up, b_lo
    return negedge, coef.astype(np.float32), bins


def horner_f32(cf, x):
    a, b, c, d = (np.float32(v) for v in cf)
    x = np.asarray(x, dtype=np.float32)
    return (a + (b + (c + d * x) * x) * x).astype(np.float32)


def check(negedge, coef, bins):
    """Largest |float32 cubic - D_b(acos(c))| over every interval side (float64 reference)."""
    worst = 0.0
    x = np.linspace(0.0, 1.0, 513, dtype=np.float64)[:-1].astype(np.float32)
    for i in range(BIAS - 1, BIAS + K):
        c = ((i - BIAS) + x.astype(np.float64)) / K
        for side in (0, 1):
            b = bins[2 * i + side]
            if b == 0:
                continue
            if -negedge[i] == NO_EDGE and side == 1:
                continue
            got = horner_f32(coef[2 * i + side], x).astype(np.float64)
            worst = max(worst, float(np.max(np.abs(got - d_bin(b, c)))))
    return worst


def write_inc(negedge, coef, path):
    def f(v):
        return float(v).hex() + "f" if np.isfinite(v) else "0.0f"

    lines = ["// Generated by dir_ctable.py: the cos(theta)-indexed T4010A1 directivity table.",
             "// Do not edit; regenerate with `python dir_ctable.py`.",
             f"#define AFC_CTAB_K {K}",
             f"#define AFC_CTAB_BIAS {BIAS}",
             f"#define AFC_CTAB_SIZE {SIZE}",
             "#define AFC_CTAB_NEGEDGE_INIT { \\"]
    for i in range(0, SIZE, 4):
        lines.append("    " + ", ".join(f(v) for v in negedge[i:i + 4]) + ", \\")
    lines.append("}")
    lines.append("#define AFC_CTAB_COEF_INIT { \\")
    for row in coef:
        lines.append("    {" + ", ".join(f(v) for v in row) + "}, \\")
    lines.append("}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    ne, cf, bn = table()
    print(f"max |float32 cubic - D(acos c)| over all intervals: {check(ne, cf, bn):.3e}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dir_ctable.inc")
    write_inc(ne, cf, out)
    print("wrote", out)
