"""Derivation of the directivity table the kernels use (AFC_DIR_TABLE_INIT in propagate.cuh).

The reference's T4010A1 directivity (acoustic-field-calculator/src/core/wave_sources/
t4010a1.rs:18-71,107-120) evaluates, in bin i = ceil(theta / ANGLE_DIV), the cubic
a + (b + (c + d x) x) x at x = theta - (i - 1) ANGLE_DIV in (0, ANGLE_DIV].  The kernels evaluate
the same cubic in xc = x - ANGLE_DIV / 2, the offset from the bin centre (which they get with
two fewer instructions), so each bin's coefficients are re-expanded about the centre in float64
and rounded to float32:
    A = a + b h + c h^2 + d h^3,  B = b + 2 c h + 3 d h^2,  C = c + 3 d h,  D = d,   h = ANGLE_DIV / 2.
Table layout (32 float4 entries (A, B, C, D)): entry 0 and the constant bins 1 and 2 give 1;
bins 3..9 the re-expanded cubics; entries 10..30 give 0 (theta beyond 90 degrees); entry 31
gives 1: the kernels' rounded bin index wraps to 31 when theta is within rounding of 0.
This script checks the float32 evaluation against the reference's own float32 evaluation over
every bin and prints the table.  Run: python dir_table.py
"""
import numpy as np

ANGLE_DIV = np.float32(np.float32(np.pi) / np.float32(18.0))


def reference_coefficients():
    """Per-bin (a, b, c, d) of t4010a1.rs:18-69 as f32 (x in radians): entries 0..2 give 1
    (the `0 => 1.0` arm and the two constant bins)."""
    return np.array([
        [1.0, 0.0, 0.0, 0.0],
        [1.0, 0.0, 0.0, 0.0],
        [1.0, 0.0, 0.0, 0.0],
        [1.0, -0.2633589359691162, -2.586746661956269, 0.0009174516976956062],
        [0.891250938, -0.8910683499820542, -1.0097633564074366, 0.0001704413361662757],
        [0.707945784, -1.1924098538381465, -0.7167962799004945, 4.362034715924911],
        [0.501187234, -1.0439934287916925, 0.027352097655185065, -2.238476800444034],
        [0.354813389, -0.7015151838490918, 0.39509604454751995, 1.274774620435337],
        [0.251188643, -0.4471050803642494, 1.0625664749725618, -1.1276955684895724],
        [0.199526231, -0.179254124486545, 0.008242027161100222, -0.9016569137759131],
    ], dtype=np.float32)


def centred(coef):
    h = np.float64(ANGLE_DIV) / 2
    a, b, c, d = (np.float64(v) for v in coef)
    return np.array([a + b * h + c * h * h + d * h ** 3, b + 2 * c * h + 3 * d * h * h,
                     c + 3 * d * h, d], dtype=np.float32)


def table():
    t = np.zeros((32, 4), dtype=np.float32)
    ref = reference_coefficients()
    for i in range(10):
        t[i] = centred(ref[i]) if i >= 3 else ref[i]
    t[31] = (1.0, 0.0, 0.0, 0.0)
    return t


def check(t):
    ref = reference_coefficients()
    worst = 0.0
    x = np.linspace(0, float(ANGLE_DIV), 100001).astype(np.float32)
    for i in range(3, 10):
        a, b, c, d = ref[i]
        d_ref = (a + (b + (c + d * x) * x) * x).astype(np.float32)
        xc = (x - ANGLE_DIV / np.float32(2)).astype(np.float32)
        A, B, C, D = t[i]
        d_new = (A + (B + (C + D * xc) * xc) * xc).astype(np.float32)
        worst = max(worst, float(np.max(np.abs(d_new.astype(np.float64) - d_ref))))
    return worst


if __name__ == "__main__":
    t = table()
    print(f"max |centred - reference| over bins 3..9: {check(t):.3e}")
    for i, row in enumerate(t):
        if i < 10 or i == 31:
            print(f"  {i:2d}: {{{', '.join(f'{float(v).hex()}f' for v in row)}}},")
