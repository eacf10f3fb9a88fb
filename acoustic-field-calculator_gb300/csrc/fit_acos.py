"""Derivation of the acos polynomial used by the field kernels (propagate.cuh).

acos(c) = sqrt(1 - c) * Q(c) with Q smooth on [-1, 1]; Q is fitted here by iteratively
re-weighted least squares on Chebyshev nodes of [-0.03, 1] (the kernels only need theta for
cos(theta) >= -0.03: beyond 90 degrees the T4010A1 directivity is 0).  The coefficients are
rounded to float32 and the float32 evaluation (Horner, then the product with sqrt(1 - c)) is
checked against numpy's float64 arccos.  Run: python fit_acos.py
"""
import numpy as np

LO, HI, DEG = -0.03, 1.0, 5


def fit(deg=DEG, lo=LO, hi=HI):
    x = np.cos(np.linspace(0, np.pi, 4000)) * (hi - lo) / 2 + (hi + lo) / 2
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.where(x < 1, np.arccos(x) / np.sqrt(1 - x), np.sqrt(2.0))
    w = np.ones_like(x)
    for _ in range(30):
        V = np.vander(x, deg + 1, increasing=True)
        coef, *_ = np.linalg.lstsq(V * w[:, None], f * w, rcond=None)
        err = V @ coef - f
        w = w * (1 + 0.5 * np.abs(err) / np.abs(err).max())
    return coef.astype(np.float32)


def max_error(c32, lo=LO):
    xt = np.linspace(lo, 1.0, 400001).astype(np.float32)
    q = np.full_like(xt, c32[-1])
    for k in range(len(c32) - 2, -1, -1):
        q = (q.astype(np.float64) * xt + c32[k]).astype(np.float32)
    s = np.sqrt(1.0 - xt.astype(np.float64)).astype(np.float32)
    th = (s.astype(np.float64) * q).astype(np.float32)
    return float(np.abs(th - np.arccos(xt.astype(np.float64))).max())


if __name__ == "__main__":
    c = fit()
    print("coefficients c0..c6:", [float(v) for v in c])
    print("max |theta - acos| in float32:", max_error(c))
