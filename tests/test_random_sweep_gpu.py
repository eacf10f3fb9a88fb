"""A seeded sweep over the combinations of the calculator ABI against the oracle: source type
and count (including tile edges), shared or tilted directions, attenuation, observation area
(grids of one to three dimensions in every axis order and with partial tiles, scatter sets of
awkward sizes), field type and calculator tag, with points in front of the sources, around
them and behind them.

Each case goes through AFC_Calculate as the reference's python/afc/afc.py drives it and is
compared with the oracle's float32 restatement of the reference CPU calculator (the Accurate
tag with the oracle's accurate mode).  Bar: max |p_gpu - p_ref| <= 1e-4 max |p_ref| (2e-4 for
the power field, a square)."""
import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = {0: "PressureFieldBuffer", 1: "PowerFieldBuffer", 2: "ComplexPressureFieldBuffer"}
CALCS = {0: "CpuCalculator", 1: "AccurateCalculator", 2: "GpuCalculator"}
N_CASES = 200


def _sources(rng, st, n, tilted, atten):
    pos = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-5, 5, n)
    amp = rng.uniform(0.2, 1.0, n).astype(np.float32)
    ph = rng.uniform(-np.pi, np.pi, n).astype(np.float32)
    if st == 1:
        rec = W.t4010a1_records(pos, amp, ph)
        if tilted:
            d = rng.normal(size=(n, 3)) * np.array([0.4, 0.4, 0.2]) + np.array([0, 0, 1.0])
            rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    else:
        rec = W.sphere_records(pos, amp, ph)
    k = rng.uniform(0.70, 0.75, n).astype(np.float32)
    return rec, k, np.full(n, atten, np.float32)


def _case(seed):
    rng = np.random.default_rng(9000 + seed)
    st = int(rng.integers(0, 2))
    n = int(rng.choice([1, 2, 31, 255, 256, 257, 700, 1500]))
    tilted = bool(rng.integers(0, 2))
    atten = float(rng.choice([0.0, 0.0115]))
    # where the points lie: in front (z 30-200), around the sources (z -40-40), behind (z < 0)
    zone = int(rng.choice([0, 0, 1, 2]))
    zlo = {0: 30.0, 1: -40.0, 2: -160.0}[zone]
    field = int(rng.integers(0, 3))
    calc = int(rng.integers(0, 3))
    if rng.random() < 0.6:
        dim = int(rng.integers(1, 4))
        axes = tuple(int(a) for a in rng.permutation([1, 2, 3]))
        res = float(rng.choice([0.5, 0.7, 1.0, 1.5]))
        cap = {1: 4000, 2: 160, 3: 28}[dim]  # per-axis counts keep the grid small
        counts = [int(rng.integers(1, cap + 1)) for _ in range(dim)]
        starts = {1: rng.uniform(-60, 0), 2: rng.uniform(-60, 0), 3: zlo + rng.uniform(0, 20)}
        ranges = []
        for j, ax in enumerate(axes):
            lo = float(np.float32(starts[ax]))
            if j < dim:
                # a quarter step of slack keeps the f32 count at counts[j]
                ranges.append((lo, float(np.float32(lo + (counts[j] - 0.75) * res))))
            else:
                ranges.append((lo, lo))
        area = ("grid", W.GridSpec(dim, ranges, res, axes))
    else:
        m = int(rng.choice([1, 100, 511, 2047, 2048, 2049, 5000]))
        pts = rng.uniform(-80, 80, (m, 3)).astype(np.float32)
        pts[:, 2] = rng.uniform(zlo, zlo + 170, m)
        area = ("scatter", pts)
    return rng, st, n, tilted, atten, field, calc, area


@pytest.mark.parametrize("seed", range(N_CASES))
def test_random_case(gpu, seed):
    afc = gpu
    rng, st, n, tilted, atten, field, calc, area = _case(seed)
    rec, k, a = _sources(rng, st, n, tilted, atten)
    s = afc.UniformSystem(300.0)
    s.add_records(st, rec, k, a)
    if area[0] == "grid":
        g = area[1]
        handle = afc.grid_from_spec(g)
        lo, hi = g.lo_hi()
        pts = O.grid_points(g.dim, lo, hi, g.res, g.axes)
        desc = f"grid{g.dim}D axes={g.axes} res={g.res}"
    else:
        pts = area[1]
        handle = afc.ScatterArea()
        handle.add_observe_points(pts)
        desc = "scatter"
    out = getattr(afc, CALCS[calc])().calculate(s, handle, getattr(afc, FIELDS[field])())
    ref_c = O.field_f32(st, rec, k, a, pts, accurate=(calc == 1))
    ref = {0: np.abs(ref_c), 1: np.abs(ref_c) ** 2, 2: ref_c}[field]
    out = np.asarray(out)
    assert out.shape[0] == len(pts)
    peak = float(np.max(np.abs(ref)))
    if peak == 0.0:  # every point behind every source: D = 0 for each pair
        assert np.all(out == 0)
        return
    err = float(np.max(np.abs(out - ref)) / peak)
    print(f"case {seed}: st={st} n={n} tilted={tilted} atten={atten} {desc} m={len(pts)} "
          f"field={field} calc={calc}: {err:.2e}")
    assert err <= (2e-4 if field == 1 else 1e-4)
