"""The oracle reproduces the stored golden fixtures (tests/golden/, generated by
tests/golden/make_golden.py): a change to the oracle's arithmetic, or a platform whose libm
rounds differently, shows here first.  The f32 fields are deterministic per point (each
point's sum runs serially in source order), so the bar is a few float32 ulps of the peak; the
float64 GS-PAT drive agrees to 1e-12."""
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_single_focus_fixture():
    g = _load("single_focus_249src_101x101")
    pts = O.grid_points(2, g["lo"], g["hi"], float(g["res"]), tuple(int(a) for a in g["axes"]))
    assert len(pts) == 101 * 101
    p = O.field_f32(1, g["sources"], g["k"], g["atten"], pts, O.FIELD_PRESSURE)
    assert _rel(p, g["pressure_f32"]) <= 1e-6
    p64 = np.abs(O.field_f64(1, g["sources"], g["k"], g["atten"], pts))
    assert _rel(p64, g["pressure_f64"]) <= 1e-7
    # the focus is the peak, at the grid centre
    assert int(np.argmax(g["pressure_f32"])) == 50 * 101 + 50


def test_scatter_fixture():
    g = _load("scatter_37src_1000pts")
    for st, name in ((0, "sphere"), (1, "t4010a1")):
        p = O.field_f32(st, g[f"{name}_sources"], g[f"{name}_k"], g[f"{name}_atten"],
                        g["points"], O.FIELD_COMPLEX)
        assert _rel(p, g[f"{name}_complex_f32"]) <= 1e-6


def test_gspat_fixture():
    g = _load("gspat_996src_8foci")
    solved, q = O.gspat_f64(1, g["sources"], g["k"], g["atten"], g["foci"], g["amps"])
    assert _rel(q, g["q"]) <= 1e-12
    np.testing.assert_allclose(solved.reshape(-1, 9), g["solved"], rtol=0, atol=1e-6)
