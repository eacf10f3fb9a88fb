"""Generate the golden fixtures of this directory from the oracle (oracle/afc_oracle.c, the C
restatement of the reference's CPU calculator and optimizers, in its default libm mode: acosf,
expf, sinf and cosf from the platform's glibc, as the reference's Rust calls them).  The
reference itself is Rust and cannot be built or imported here, and its repository ships no
golden vectors, so these fixtures pin the oracle (tests/test_golden.py re-runs it on the stored
inputs) and give the GPU tests stored expected outputs (tests/test_golden_gpu.py).

    python tests/golden/make_golden.py

Fixtures (numpy .npz, float32 unless noted):
  single_focus_249src_101x101.npz  the single-focus case: 249 T4010A1 transducers, amplitude 1,
                                    focal-law phases towards (centre, 150 mm); pressure on the
                                    101 x 101 XY grid at 1 mm, z = 150 (the f32 oracle, and
                                    the f64 oracle rounded to f32); the grid by lo, hi, res, axes
  scatter_37src_1000pts.npz         37 random sources of each type (sphere, T4010A1 with tilted
                                    directions), attenuation 5e-3 /mm, complex pressure at 1,000
                                    random points
  gspat_996src_8foci.npz            GS-PAT (100 iterations) on the 2 x 2 tiling with 8 foci:
                                    the solved records and the complex drive q (float64 oracle,
                                    q complex128)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "oracle"), os.path.join(REPO, "acoustic-field-calculator_gb300")]
import oracle as O  # noqa: E402
import workloads as W  # noqa: E402


def single_focus():
    w = W.single_focus()
    lo, hi = w.grid.lo_hi()
    pts = O.grid_points(2, lo, hi, w.grid.res, w.grid.axes)
    return dict(sources=w.sources, k=w.k, atten=w.atten, lo=np.float32(lo), hi=np.float32(hi),
                res=np.float32(w.grid.res), axes=np.int32(w.grid.axes),
                pressure_f32=O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_PRESSURE),
                pressure_f64=np.abs(O.field_f64(1, w.sources, w.k, w.atten, pts)).astype(
                    np.float32))


def scatter():
    rng = np.random.default_rng(20261203)
    out = {}
    pts = rng.uniform(-80, 80, (1000, 3)).astype(np.float32)
    pts[:, 2] = rng.uniform(30, 200, 1000)
    out["points"] = pts
    for st, name in ((0, "sphere"), (1, "t4010a1")):
        n = 37
        pos = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
        pos[:, 2] = rng.uniform(-5, 5, n)
        amp = rng.uniform(0.2, 1.0, n).astype(np.float32)
        ph = rng.uniform(-np.pi, np.pi, n).astype(np.float32)
        if st == 1:
            rec = W.t4010a1_records(pos, amp, ph)
            d = rng.normal(size=(n, 3)) * np.array([0.3, 0.3, 0.0]) + np.array([0, 0, 1.0])
            rec[:, 3:6] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        else:
            rec = W.sphere_records(pos, amp, ph)
        k = rng.uniform(0.70, 0.75, n).astype(np.float32)
        a = np.full(n, 5e-3, np.float32)
        out[f"{name}_sources"], out[f"{name}_k"], out[f"{name}_atten"] = rec, k, a
        out[f"{name}_complex_f32"] = O.field_f32(st, rec, k, a, pts, O.FIELD_COMPLEX)
    return out


def gspat():
    rng = np.random.default_rng(7)
    w, foci, amps = W.gspat_request(rng, 8)
    solved, q = O.gspat_f64(1, w.sources, w.k, w.atten, foci, amps)
    return dict(sources=w.sources, k=w.k, atten=w.atten, foci=foci, amps=amps,
                solved=solved.reshape(-1, 9), q=q)


def main():
    for name, fn in (("single_focus_249src_101x101", single_focus),
                     ("scatter_37src_1000pts", scatter), ("gspat_996src_8foci", gspat)):
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fn())
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
