"""The GPU path against the stored golden fixtures (tests/golden/), through the reference-facing
API: the expected outputs come from the fixture files, not from running the oracle.  Bars as
in the parity tests: max |p - p_ref| <= 1e-4 of the peak |p_ref| for fields, 1e-3 of the
largest |q| for the GS-PAT drive (the GPU iterates in float32)."""
import os

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-4


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_single_focus_against_fixture(gpu):
    afc = gpu
    g = _load("single_focus_249src_101x101")
    s = afc.UniformSystem(300.0)
    s.add_records(1, g["sources"], g["k"], g["atten"])
    lo, hi = g["lo"], g["hi"]
    spec = W.GridSpec(2, [(float(lo[0]), float(hi[0])), (float(lo[1]), float(hi[1])),
                          (float(lo[2]), float(hi[2]))], float(g["res"]),
                      tuple(int(a) for a in g["axes"]))
    area = afc.grid_from_spec(spec)
    for calc in ("CpuCalculator", "AccurateCalculator", "GpuCalculator"):
        out = getattr(afc, calc)().calculate(s, area, afc.PressureFieldBuffer())
        e32, e64 = _rel(out, g["pressure_f32"]), _rel(out, g["pressure_f64"])
        print(f"{calc}: vs stored f32 {e32:.2e}, vs stored f64 {e64:.2e}")
        assert e32 <= TOL and e64 <= TOL


@pytest.mark.parametrize("st,name", [(0, "sphere"), (1, "t4010a1")])
def test_scatter_against_fixture(gpu, st, name):
    afc = gpu
    g = _load("scatter_37src_1000pts")
    s = afc.UniformSystem(300.0)
    s.add_records(st, g[f"{name}_sources"], g[f"{name}_k"], g[f"{name}_atten"])
    area = afc.ScatterArea()
    area.add_observe_points(g["points"])
    out = afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer())
    e = _rel(out, g[f"{name}_complex_f32"])
    print(f"{name}: {e:.2e}")
    assert e <= TOL


def test_gspat_against_fixture(gpu):
    afc = gpu
    g = _load("gspat_996src_8foci")
    s = afc.UniformSystem(300.0)
    s.add_records(1, g["sources"], g["k"], g["atten"])
    afc.Optimizer.gs_pat(s, g["foci"], g["amps"])
    got = s.records()
    q = got[:, 6].astype(np.float64) * np.exp(1j * got[:, 7].astype(np.float64))
    e = _rel(q, g["q"])
    print(f"GS-PAT: max |dq| / max |q| = {e:.2e}")
    assert e <= 1e-3
