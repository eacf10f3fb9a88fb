"""Pairs next to a directivity bin edge (10-degree multiples from 20 to 90 degrees), where the
fast directivity switches bins and the exact edge path takes over, in both field bodies: the
general one (scatter points, theta-binned directivity; one source per point, so each pair's
value is checked on its own) and the rows tiling (cos(theta)-indexed table; a large grid with
sources placed on rays through one grid node at the edge angles).  Offsets from the edge run
from 0 to 1e-4 rad on both sides, through the edge paths' margins (1e-5 rad in theta, 4e-6 in
cos(theta))."""
import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

EDGES_DEG = np.arange(20, 91, 10)
OFFSETS = np.array([-1e-4, -1e-5, -3e-6, -1e-6, -2e-7, 0.0, 2e-7, 1e-6, 3e-6, 1e-5, 1e-4])


def _directions(rng, tilted, n):
    if not tilted:
        return np.tile(np.array([0.0, 0.0, 1.0]), (n, 1))
    d = rng.normal(size=(n, 3)) * np.array([0.4, 0.4, 0.0]) + np.array([0, 0, 1.0])
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _basis(n):
    """Two unit vectors orthogonal to n."""
    a = np.array([1.0, 0.0, 0.0]) if abs(n[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    e1 = np.cross(n, a)
    e1 /= np.linalg.norm(e1)
    return e1, np.cross(n, e1)


@pytest.mark.parametrize("tilted", [False, True])
def test_single_pairs_at_bin_edges(gpu, tilted):
    afc = gpu
    rng = np.random.default_rng(3 + tilted)
    n_dir = _directions(rng, tilted, 1)[0]
    e1, e2 = _basis(n_dir)
    pts = []
    for deg in EDGES_DEG:
        for off in OFFSETS:
            th = np.deg2rad(deg) + off
            for az in (0.3, 1.9, 4.4):
                u = np.cos(th) * n_dir + np.sin(th) * (np.cos(az) * e1 + np.sin(az) * e2)
                pts.append(rng.uniform(15, 40) * u)
    pts = np.asarray(pts, dtype=np.float32)
    rec = W.t4010a1_records(np.zeros((1, 3), np.float32), 1.0, 0.4)
    rec[0, 3:6] = n_dir
    k = np.full(1, W.wavenumber(), np.float32)
    a = np.zeros(1, np.float32)
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    area = afc.ScatterArea()
    area.add_observe_points(pts)
    got = np.asarray(afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer()))
    ref = O.field_f32(1, rec, k, a, pts)
    scale = 1.0 / np.linalg.norm(pts, axis=1)  # |term| without directivity
    err = np.abs(got - ref) / scale
    worst = int(np.argmax(err))
    print(f"{len(pts)} pairs, worst |p - ref| / (1/r) = {err[worst]:.2e} at {pts[worst]}")
    # A pair in the wrong bin is off by the directivity's jump at that edge: 5e-5 at 60 degrees,
    # 3e-3 to 1.7e-1 at the others.  sin/cos of the unreduced phase (k r <= 30 rad here) costs
    # up to ~4e-6.
    assert err.max() <= 2e-5


@pytest.mark.parametrize("tilted", [False, True])
def test_rows_tiling_at_bin_edges(gpu, tilted):
    """96 x 96 x 72 grid (the rows tiling) with 88 sources on rays through one grid node at
    the edge angles, at 15-40 mm; the node's value is checked against the sum of |terms|, the
    whole grid against the usual bar."""
    afc = gpu
    rng = np.random.default_rng(11 + tilted)
    counts, res = (96, 96, 72), 0.5
    lo = np.array([-24.0, -24.0, 120.0], np.float32)
    node = (lo + res * np.array([40, 51, 23])).astype(np.float32)
    dirs, pos = [], []
    for deg in EDGES_DEG:
        for off in OFFSETS:
            nd = _directions(rng, tilted, 1)[0]
            e1, e2 = _basis(nd)
            th = np.deg2rad(deg) + off
            az = rng.uniform(0, 2 * np.pi)
            u = np.cos(th) * nd + np.sin(th) * (np.cos(az) * e1 + np.sin(az) * e2)
            pos.append(node - rng.uniform(15, 40) * u)
            dirs.append(nd)
    pos = np.asarray(pos, dtype=np.float32)
    n = len(pos)
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, n).astype(np.float32),
                            rng.uniform(-np.pi, np.pi, n).astype(np.float32))
    rec[:, 3:6] = np.asarray(dirs, dtype=np.float32)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.full(n, 1e-3, np.float32)
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    g = W.GridSpec(3, [(float(lo[j]), float(lo[j] + (counts[j] - 0.5) * res)) for j in range(3)],
                   res, (1, 2, 3))
    area = afc.grid_from_spec(g)
    assert tuple(int(c) for c in area.grid_desc().count) == counts
    got = np.asarray(afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer()))
    # the node alone, against the sum of its terms' moduli
    ref_node = O.field_f32(1, rec, k, a, node[None, :])[0]
    g_node = got[40 + counts[0] * (51 + counts[1] * 23)]
    bound = np.sum(rec[:, 6] / np.linalg.norm(pos - node, axis=1))
    print(f"node: |p - ref| / sum|terms| = {abs(g_node - ref_node) / bound:.2e}")
    # one of the 88 terms in the wrong bin: >= 3e-3 / 88 of the bound (but for 60 degrees)
    assert abs(g_node - ref_node) <= 1e-5 * bound
    # every grid point
    glo, ghi = g.lo_hi()
    pts = O.grid_points(3, glo, ghi, res, (1, 2, 3))
    assert np.array_equal(pts[40 + counts[0] * (51 + counts[1] * 23)], node)
    ref = O.field_f32(1, rec, k, a, pts)
    err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print(f"grid: rel {err:.2e}")
    assert err <= 1e-4


def _ref_cos(d, n):
    """The reference's f32 cos(theta): ((nx dx + ny dy) + nz dz) / sqrt((dx dx + dy dy) + dz dz)."""
    f = np.float32
    d = d.astype(f)
    n = n.astype(f)
    dist = np.sqrt(((d[:, 0] * d[:, 0]) + (d[:, 1] * d[:, 1])) + (d[:, 2] * d[:, 2]))
    dot = ((n[:, 0] * d[:, 0]) + (n[:, 1] * d[:, 1])) + (n[:, 2] * d[:, 2])
    return (dot / dist).astype(f)


def _back_axis_sources(rng, nodes):
    """One tilted source per node, 20-120 mm in front of it, so that the node sits exactly on
    the source's back axis; returns records and the reference's f32 cos(theta) of each pair."""
    m = len(nodes)
    n = rng.normal(size=(m, 3)) * np.array([0.5, 0.5, 0.2]) + np.array([0, 0, 1.0])
    n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
    r = rng.uniform(20, 120, m).astype(np.float32)
    pos = (nodes + r[:, None] * n.astype(np.float64)).astype(np.float32)
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, m).astype(np.float32),
                            rng.uniform(-np.pi, np.pi, m).astype(np.float32))
    rec[:, 3:6] = n
    return rec, _ref_cos(nodes - pos, n)


@pytest.mark.parametrize("body", ["general", "rows"])
def test_back_axis_pairs(gpu, body):
    """A point exactly on a tilted source's back axis: the reference's f32 cos(theta) rounds to
    -1 or just below, and below -1 its acos is NaN, so the directivity is 1 (bin 0) instead of
    0.  Both bodies route such pairs through the exact path."""
    afc = gpu
    rng = np.random.default_rng(31 if body == "general" else 32)
    if body == "general":
        nodes = np.stack([rng.uniform(-20, 20, 300), rng.uniform(-20, 20, 300),
                          rng.uniform(100, 140, 300)], 1).astype(np.float32)
        rec, c = _back_axis_sources(rng, nodes)
        area = afc.ScatterArea()
        area.add_observe_points(nodes)
        pts = nodes
    else:
        counts, res = (96, 96, 72), 0.5
        lo = np.array([-24.0, -24.0, 120.0], np.float32)
        idx = np.stack([rng.integers(0, c_, 300) for c_ in counts], 1)
        nodes = (lo + res * idx).astype(np.float32)
        rec, c = _back_axis_sources(rng, nodes)
        g = W.GridSpec(3, [(float(lo[j]), float(lo[j] + (counts[j] - 0.5) * res))
                           for j in range(3)], res, (1, 2, 3))
        area = afc.grid_from_spec(g)
        glo, ghi = g.lo_hi()
        pts = O.grid_points(3, glo, ghi, res, (1, 2, 3))
    assert np.count_nonzero(c < -1) >= 20  # pairs whose reference directivity is 1
    k = np.full(len(rec), W.wavenumber(), np.float32)
    a = np.zeros(len(rec), np.float32)
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    got = np.asarray(afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer()))
    ref = O.field_f32(1, rec, k, a, pts)
    err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print(f"{body}: {np.count_nonzero(c < -1)} pairs with c < -1, rel {err:.2e}")
    assert err <= 1e-4
