"""Observation points exactly at a source position, against the oracle.

The reference's pair term there is from_polar(amp * D * exp(-0 alpha) / 0, phase) with D = 1
(acos of 0/0 is NaN: bin 0), so a coincident point's complex field has components of +-inf, or
NaN (a zero amplitude, a phase of exactly 0, or infinities of both signs); its pressure is
sqrt(re^2 + im^2) of those (inf or NaN) and its power re^2 + im^2.  Every other point is finite
and held to the field bar (1e-4 of the peak finite |p|).  Cases cover scatter sets and grids
through the flat, rows and source-split kernels, both source types, and the Accurate tag."""
import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = {0: "PressureFieldBuffer", 1: "PowerFieldBuffer", 2: "ComplexPressureFieldBuffer"}


def _ref_field(ref_c, field):
    re = ref_c.real.astype(np.float32)
    im = ref_c.imag.astype(np.float32)
    with np.errstate(all="ignore"):
        ns = re * re + im * im  # norm_sqr in f32, no hypot: inf with NaN gives NaN
        return {0: np.sqrt(ns), 1: ns, 2: ref_c.astype(np.complex64)}[field]


def _check(out, ref):
    parts = (np.real, np.imag) if np.iscomplexobj(ref) else (lambda x: x,)
    finite = np.ones(len(ref), bool)
    for part in parts:
        o, r = part(out), part(ref)
        np.testing.assert_array_equal(np.isnan(o), np.isnan(r))
        inf = np.isinf(r)
        np.testing.assert_array_equal(np.isinf(o), inf)
        np.testing.assert_array_equal(o[inf], r[inf])  # the same signed infinities
        finite &= np.isfinite(r)
    assert (~finite).sum() > 0
    peak = float(np.max(np.abs(ref[finite])))
    err = float(np.max(np.abs(out[finite] - ref[finite]))) / peak
    return int((~finite).sum()), err


def _sources(rng, st, pos):
    n = len(pos)
    amp = rng.uniform(0.2, 1.0, n).astype(np.float32)
    ph = rng.uniform(-np.pi, np.pi, n).astype(np.float32)
    amp[1] = 0.0     # 0 / 0: NaN in both components
    amp[2] = -0.7    # negative amplitude: infinities of the other sign
    ph[3] = 0.0      # sin(0) = 0: inf * 0 = NaN in the imaginary part
    rec = W.sphere_records(pos, amp, ph) if st == 0 else W.t4010a1_records(pos, amp, ph)
    k = np.full(n, 0.7296, np.float32)
    return rec, k, np.full(n, 0.0115, np.float32)


def _run(afc, st, rec, k, a, handle, pts, field, calc):
    s = afc.UniformSystem(300.0)
    s.add_records(st, rec, k, a)
    calc_cls = afc.AccurateCalculator if calc == 1 else afc.GpuCalculator
    out = np.asarray(calc_cls().calculate(s, handle, getattr(afc, FIELDS[field])()))
    with np.errstate(all="ignore"):
        ref_c = O.field_f32(st, rec, k, a, pts, accurate=(calc == 1))
    return _check(out, _ref_field(ref_c, field))


@pytest.mark.parametrize("st", [0, 1])
@pytest.mark.parametrize("size", ["small", "split"])
@pytest.mark.parametrize("field,calc", [(2, 2), (0, 2), (1, 2), (2, 1)])
def test_scatter_points_on_sources(gpu, st, size, field, calc):
    afc = gpu
    rng = np.random.default_rng(1100 + st)
    m, n = (3000, 300) if size == "small" else (65536, 2000)
    pts = rng.uniform(-80, 80, (m, 3)).astype(np.float32)
    pts[:, 2] = rng.uniform(-20, 120, m)
    pos = rng.uniform(-80, 80, (n, 3)).astype(np.float32)
    pos[:, 2] = 0.0
    on = rng.choice(m, 40, replace=False)
    pos[:40] = pts[on]  # sources 0..39 sit on observation points (1, 2, 3: the special ones)
    pos[40] = pos[4]    # a duplicate source: two infinite terms at one point
    rec, k, a = _sources(rng, st, pos)
    sc = afc.ScatterArea()
    sc.add_observe_points(pts)
    bad, err = _run(afc, st, rec, k, a, sc, pts, field, calc)
    print(f"scatter st={st} m={m} n={n} field={field} calc={calc}: {bad} non-finite, {err:.2e}")
    assert err <= (2e-4 if field == 1 else 1e-4)


@pytest.mark.parametrize("st", [0, 1])
@pytest.mark.parametrize("shape", ["line", "plane", "plane_split"])
@pytest.mark.parametrize("field,calc", [(2, 2), (0, 2), (2, 1)])
def test_grid_points_on_sources(gpu, st, shape, field, calc):
    """Grids in the sources' plane: the line takes the flat kernel, the planes the rows
    tiling (the larger one with its sources split over a cluster)."""
    afc = gpu
    rng = np.random.default_rng(1200 + st)
    res = 1.27
    if shape == "line":
        spec, n = W.GridSpec(1, [(-40.0, 60.0), (3.0, 3.0), (0.0, 0.0)], res, (1, 2, 3)), 200
    elif shape == "plane":
        spec, n = W.GridSpec(2, [(-40.0, 40.0), (-30.0, 30.0), (0.0, 0.0)], res, (1, 2, 3)), 300
    else:
        spec, n = W.GridSpec(2, [(-160.0, 160.0), (-80.0, 80.0), (0.0, 0.0)], res, (1, 2, 3)), 2000
    lo, hi = spec.lo_hi()
    pts = O.grid_points(spec.dim, lo, hi, spec.res, spec.axes)
    pos = rng.uniform(-40, 40, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-5.0, -1.0, n).astype(np.float32)
    on = rng.choice(len(pts), 40, replace=False)
    pos[:40] = pts[on]
    pos[40] = pos[4]
    rec, k, a = _sources(rng, st, pos)
    bad, err = _run(afc, st, rec, k, a, afc.grid_from_spec(spec), pts, field, calc)
    print(f"grid {shape} st={st} m={len(pts)} n={n} field={field} calc={calc}: "
          f"{bad} non-finite, {err:.2e}")
    assert err <= 1e-4
