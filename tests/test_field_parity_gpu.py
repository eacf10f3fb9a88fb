"""Parity of the GPU field kernels with the oracle, through the reference-facing C ABI
(AFC_Calculate, driven like the reference's python/afc/afc.py) and the device-level ABI.

Tolerance (the stated bar): max |p_gpu - p_ref| over points <= 1e-4 * max |p_ref|, with
p_ref the oracle's restatement of the reference CPU calculator (float32) and, where stated,
its float64 twin.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_err(p, ref):
    p = np.asarray(p)
    ref = np.asarray(ref)
    return float(np.max(np.abs(p - ref)) / np.max(np.abs(ref)))


def make_system(afc, st, records, k, atten):
    s = afc.UniformSystem(300.0)
    s.add_records(st, records, k, atten)
    return s


def random_sources(rng, st, n, spread=60.0, atten=0.005):
    pos = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-5, 5, n)
    amp = rng.uniform(0.2, 1.0, n).astype(np.float32)
    ph = rng.uniform(-np.pi, np.pi, n).astype(np.float32)
    if st == 1:
        rec = W.t4010a1_records(pos, amp, ph)
        d = rng.normal(size=(n, 3)) * np.array([0.3, 0.3, 0.0]) + np.array([0, 0, 1.0])
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rec[:, 3:6] = d
    else:
        rec = W.sphere_records(pos, amp, ph)
    k = rng.uniform(0.70, 0.75, n).astype(np.float32)
    a = np.full(n, atten, np.float32)
    return rec, k, a


def random_points(rng, m):
    pts = rng.uniform(-80, 80, (m, 3)).astype(np.float32)
    pts[:, 2] = rng.uniform(30, 200, m)
    return pts


def scatter(afc, pts):
    area = afc.ScatterArea()
    area.add_observe_points(pts)
    return area


FIELDS = {0: "PressureFieldBuffer", 1: "PowerFieldBuffer", 2: "ComplexPressureFieldBuffer"}
CALCS = ["CpuCalculator", "AccurateCalculator", "GpuCalculator"]


def check_field(out, ref_c, field):
    """Compare a field buffer with the oracle's complex field."""
    if field == 2:
        assert rel_err(out, ref_c) <= TOL
    elif field == 0:
        assert rel_err(out, np.abs(ref_c)) <= TOL
    else:
        assert rel_err(out, np.abs(ref_c) ** 2) <= 2 * TOL


def test_single_focus_all_calculators(gpu):
    afc = gpu
    w = W.single_focus()
    s = make_system(afc, 1, w.sources, w.k, w.atten)
    area = afc.grid_from_spec(w.grid)
    assert area.get_size() == (101, 101, 1)
    lo, hi = w.grid.lo_hi()
    pts = O.grid_points(2, lo, hi, w.grid.res, w.grid.axes)
    ref = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_PRESSURE)
    ref64 = np.abs(O.field_f64(1, w.sources, w.k, w.atten, pts))
    for calc in CALCS:
        out = getattr(afc, calc)().calculate(s, area, afc.PressureFieldBuffer())
        assert out.shape == (101 * 101,)
        e = rel_err(out, ref)
        print(f"single focus {calc}: max err / peak vs f32 oracle {e:.2e}, "
              f"vs f64 {rel_err(out, ref64):.2e}")
        assert e <= TOL
        assert rel_err(out, ref64) <= TOL
    # the focus is the peak and sits at the grid centre (reference example)
    assert np.argmax(ref) == 50 * 101 + 50


@pytest.mark.parametrize("st", [0, 1])
@pytest.mark.parametrize("field", [0, 1, 2])
@pytest.mark.parametrize("calc", CALCS)
def test_scatter_random(gpu, st, field, calc):
    afc = gpu
    rng = np.random.default_rng(100 + 10 * st + field)
    rec, k, a = random_sources(rng, st, 37)
    pts = random_points(rng, 1000)
    s = make_system(afc, st, rec, k, a)
    out = getattr(afc, calc)().calculate(s, scatter(afc, pts), getattr(afc, FIELDS[field])())
    ref = O.field_f32(st, rec, k, a, pts, O.FIELD_COMPLEX)
    check_field(out, ref, field)


@pytest.mark.parametrize("dim,axes", [(1, (1, 2, 3)), (1, (3, 2, 1)), (2, (1, 2, 3)),
                                      (2, (2, 1, 3)), (2, (3, 1, 2)), (3, (1, 2, 3)),
                                      (3, (3, 1, 2)), (3, (2, 3, 1))])
def test_grid_orders(gpu, dim, axes):
    afc = gpu
    rng = np.random.default_rng(7 + dim)
    rec, k, a = random_sources(rng, 1, 50)
    ranges = [(-20.0, 25.0), (-10.0, 30.0), (60.0, 95.0)]
    res = 1.5 if dim == 3 else 0.7
    spec_ranges = []
    for j, ax in enumerate(axes):
        lo_, hi_ = ranges[ax - 1]
        spec_ranges.append((lo_, hi_) if j < dim else (lo_, lo_))
    g = W.GridSpec(dim, spec_ranges, res, axes)
    s = make_system(afc, 1, rec, k, a)
    area = afc.grid_from_spec(g)
    lo, hi = g.lo_hi()
    pts = O.grid_points(dim, lo, hi, res, axes)
    out = afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer())
    assert out.shape[0] == len(pts)
    ref = O.field_f32(1, rec, k, a, pts)
    assert rel_err(out, ref) <= TOL


@pytest.mark.parametrize("n,m", [(1, 1), (1, 1025), (257, 1), (513, 1023), (256, 1024),
                                 (1000, 3)])
def test_tails(gpu, n, m):
    afc = gpu
    rng = np.random.default_rng(n * 7 + m)
    rec, k, a = random_sources(rng, 1, n)
    pts = random_points(rng, m)
    s = make_system(afc, 1, rec, k, a)
    out = afc.GpuCalculator().calculate(s, scatter(afc, pts), afc.ComplexPressureFieldBuffer())
    ref = O.field_f32(1, rec, k, a, pts)
    assert rel_err(out, ref) <= TOL


def test_no_sources_gives_zero_field(gpu):
    afc = gpu
    # a native system with no sources (the Python wrapper creates it on the first add)
    s2 = afc.UniformSystem(300.0)
    s2.set_source_type(0)
    afc.DLL.AFC_CreateUniformSystem(ctypes.byref(s2.handle), 300.0, 0)
    area = afc.GridAreaBuilder().x_range((0, 10)).y_at(0).z_at(10).resolution(1).generate()
    out = afc.GpuCalculator().calculate(s2, area, afc.PressureFieldBuffer())
    assert out.shape == (11,) and np.all(out == 0)


def test_empty_scatter_area(gpu):
    afc = gpu
    s = afc.UniformSystem(300.0)
    s.add_wave_source(afc.SphereWaveSource((0, 0, 0), 1.0, 0.0, 40e3))
    n, ptr = afc.GpuCalculator().calculate_raw(s, afc.ScatterArea(), afc.PressureFieldBuffer())
    assert n == 0 and ptr


def test_point_on_a_source_is_not_finite_like_the_reference(gpu):
    afc = gpu
    rec = W.sphere_records(np.array([[0, 0, 0], [5, 0, 0]], np.float32), 1.0, 0.0)
    k = np.full(2, 0.7, np.float32)
    a = np.zeros(2, np.float32)
    pts = np.array([[0, 0, 0], [0, 0, 50]], np.float32)
    s = make_system(afc, 0, rec, k, a)
    out = afc.GpuCalculator().calculate(s, scatter(afc, pts), afc.ComplexPressureFieldBuffer())
    ref = O.field_f32(0, rec, k, a, pts)
    assert not np.isfinite(out[0]) and not np.isfinite(ref[0])
    assert abs(out[1] - ref[1]) <= TOL * abs(ref[1])


def test_in_place_source_mutation_is_seen(gpu):
    """python/main.py:57-63 rewrites phases through AFC_GetWaveSources between calculations."""
    afc = gpu
    rng = np.random.default_rng(11)
    rec, k, a = random_sources(rng, 1, 64)
    pts = random_points(rng, 500)
    s = make_system(afc, 1, rec, k, a)
    area = scatter(afc, pts)
    calc = afc.GpuCalculator()
    f = afc.ComplexPressureFieldBuffer()
    calc.calculate(s, area, f)
    arr = s.get_wave_sources()
    for i in range(len(arr)):
        arr[i].phase = float(rng.uniform(-3, 3))
        arr[i].amp = float(rng.uniform(0.1, 1))
    out = calc.calculate(s, area, f)
    ref = O.field_f32(1, s.records().copy(), k, a, pts)
    assert rel_err(out, ref) <= TOL


def test_scatter_points_added_between_calls(gpu):
    afc = gpu
    rng = np.random.default_rng(12)
    rec, k, a = random_sources(rng, 0, 20)
    pts = random_points(rng, 300)
    s = make_system(afc, 0, rec, k, a)
    area = scatter(afc, pts[:100])
    calc = afc.CpuCalculator()
    f = afc.PressureFieldBuffer()
    first = calc.calculate(s, area, f).copy()
    area.add_observe_points(pts[100:])
    second = calc.calculate(s, area, f)
    ref = np.abs(O.field_f32(0, rec, k, a, pts))
    assert len(second) == 300
    assert rel_err(second, ref) <= TOL
    assert rel_err(first, ref[:100]) <= TOL


def test_new_scatter_area_after_free_is_not_the_cached_one(gpu):
    """An area freed and a new one created (often at the same address) with as many points: the
    calculator must upload the new points, not reuse its device copy of the old ones."""
    import gc

    afc = gpu
    rng = np.random.default_rng(13)
    rec, k, a = random_sources(rng, 0, 20)
    s = make_system(afc, 0, rec, k, a)
    calc = afc.CpuCalculator()
    f = afc.PressureFieldBuffer()
    for _ in range(4):
        pts = random_points(rng, 100)
        area = scatter(afc, pts)
        out = calc.calculate(s, area, f).copy()
        assert rel_err(out, np.abs(O.field_f32(0, rec, k, a, pts))) <= TOL
        del area
        gc.collect()


def test_focal_point_then_field(gpu):
    """Reference example flow: AFO_FocalPoint, then the pressure on an XY slice."""
    afc = gpu
    s = afc.UniformSystem(300.0)
    pos = W.unit_array(10.18)
    for p in pos:
        s.add_wave_source(afc.T4010A1(tuple(p), (0, 0, 1), 1.0, 0.0, 40e3))
    cen = W.array_center(pos)
    afc.Optimizer.focus(s, (float(cen[0]), float(cen[1]), 150.0))
    area = (afc.GridAreaBuilder().x_range((cen[0] - 50, cen[0] + 50))
            .y_range((cen[1] - 50, cen[1] + 50)).z_at(150.0).resolution(1.0).generate())
    out = afc.GpuCalculator().calculate(s, area, afc.PressureFieldBuffer())
    k, a = O.wavenum_atten(300.0, 40e3)
    n = len(pos)
    lo = np.array([cen[0] - 50, cen[1] - 50, 150], np.float32)
    hi = np.array([cen[0] + 50, cen[1] + 50, 150], np.float32)
    pts = O.grid_points(2, lo, hi, 1.0, (1, 2, 3))
    ref = O.field_f32(1, s.records().copy(), np.full(n, k, np.float32),
                      np.full(n, a, np.float32), pts, O.FIELD_PRESSURE)
    assert rel_err(out, ref) <= TOL


def test_device_api_matches_c_abi(gpu):
    torch = pytest.importorskip("torch")
    afc = gpu
    rng = np.random.default_rng(13)
    rec, k, a = random_sources(rng, 1, 300)
    g = W.GridSpec(3, [(-20.0, 20.0), (-15.0, 15.0), (80.0, 100.0)], 1.0, (1, 2, 3))
    s = make_system(afc, 1, rec, k, a)
    area = afc.grid_from_spec(g)
    host = afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer())
    desc = area.grid_desc()
    m = int(desc.count[0] * desc.count[1] * desc.count[2])
    d_src = torch.from_numpy(rec.reshape(-1)).cuda()
    d_k = torch.from_numpy(k).cuda()
    d_a = torch.from_numpy(a).cuda()
    ws_bytes = afc.DLL.AFC_FieldWorkspaceBytes(len(k))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    out = torch.empty(2 * m, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = afc.DLL.AFC_FieldGridDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                     len(k), ctypes.byref(desc), out.data_ptr(), ws.data_ptr(),
                                     ws_bytes, stream)
    assert rc == 0, afc.last_error()
    torch.cuda.synchronize()
    dev = out.cpu().numpy().view(np.complex64)
    np.testing.assert_array_equal(dev, host.astype(np.complex64))
    # the scatter entry point on the materialised grid gives the same numbers
    lo, hi = g.lo_hi()
    pts = torch.from_numpy(O.grid_points(3, lo, hi, 1.0, (1, 2, 3)).reshape(-1)).cuda()
    out2 = torch.empty(2 * m, dtype=torch.float32, device="cuda")
    rc = afc.DLL.AFC_FieldScatterDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(),
                                        d_a.data_ptr(), len(k), pts.data_ptr(), m,
                                        out2.data_ptr(), ws.data_ptr(), ws_bytes, stream)
    assert rc == 0, afc.last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out2.cpu().numpy().view(np.complex64), dev)


def test_large_grid_subsample_vs_f64(gpu):
    """The 3984-source, 256^3-point complex field, checked on a seeded 0.1 % subsample against
    the float64 oracle (and the float32 oracle)."""
    torch = pytest.importorskip("torch")
    afc = gpu
    w = W.large_grid()
    s = make_system(afc, 1, w.sources, w.k, w.atten)
    area = afc.grid_from_spec(w.grid)
    desc = area.grid_desc()
    m = int(desc.count[0] * desc.count[1] * desc.count[2])
    assert m == 256 ** 3
    d_src = torch.from_numpy(w.sources.reshape(-1)).cuda()
    d_k = torch.from_numpy(w.k).cuda()
    d_a = torch.from_numpy(w.atten).cuda()
    ws_bytes = afc.DLL.AFC_FieldWorkspaceBytes(w.n)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    out = torch.empty(2 * m, dtype=torch.float32, device="cuda")
    rc = afc.DLL.AFC_FieldGridDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                     w.n, ctypes.byref(desc), out.data_ptr(), ws.data_ptr(),
                                     ws_bytes, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, afc.last_error()
    torch.cuda.synchronize()
    field = out.cpu().numpy().view(np.complex64)
    rng = np.random.default_rng(2024)
    idx = np.sort(rng.choice(m, m // 1000, replace=False))
    lo, hi = w.grid.lo_hi()
    i0 = idx % 256
    i1 = (idx // 256) % 256
    i2 = idx // 65536
    pts = np.stack([lo[0] + i0.astype(np.float32) * np.float32(0.5),
                    lo[1] + i1.astype(np.float32) * np.float32(0.5),
                    lo[2] + i2.astype(np.float32) * np.float32(0.5)], axis=1).astype(np.float32)
    ref64 = O.field_f64(1, w.sources, w.k, w.atten, pts)
    ref32 = O.field_f32(1, w.sources, w.k, w.atten, pts)
    e64 = rel_err(field[idx], ref64)
    e32 = rel_err(field[idx], ref32)
    rl2 = float(np.linalg.norm(field[idx] - ref64) / np.linalg.norm(ref64))
    print(f"large grid subsample ({len(idx)} pts): max err/peak vs f64 {e64:.2e}, vs f32 oracle "
          f"{e32:.2e}, oracle f32 vs f64 {rel_err(ref32, ref64):.2e}, rel-L2 vs f64 {rl2:.2e}")
    assert e64 <= TOL and e32 <= TOL


@pytest.mark.parametrize("layout", ["all_far", "mixed_tiles"])
def test_far_phases_take_the_reduced_path(gpu, layout):
    """Phases above the kernels' unreduced bound (640 rad) are reduced to [-pi, pi] first, tile
    by tile: every source tile 1 m from the points ("all_far", phases ~ 740-790 rad), or the
    first tile of 256 near and the following tiles far ("mixed_tiles").  The drive focuses on
    the observed region (the reference focal law), so the sum is coherent and both float32
    paths are well within the bar of the float64 field; checked against the f32 and the f64
    oracle, on a grid and on scatter points."""
    afc = gpu
    rng = np.random.default_rng(31)
    n = 700
    pos = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-5, 5, n)
    if layout == "all_far":
        pos[:, 2] -= 1000.0
    else:
        pos[256:, 2] -= 1000.0
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, n).astype(np.float32),
                            W.focal_phases(pos, (0.0, 0.0, 120.0)))
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.zeros(n, np.float32)
    s = make_system(afc, 1, rec, k, a)
    pts = rng.uniform(-40, 40, (3000, 3)).astype(np.float32)
    pts[:, 2] = rng.uniform(100, 140, 3000)
    g = W.GridSpec(2, [(-40.0, 40.25), (-40.0, 40.25), (120.0, 120.0)], 0.5, (1, 2, 3))
    lo, hi = g.lo_hi()
    gp = O.grid_points(2, lo, hi, 0.5, (1, 2, 3))
    calc = afc.GpuCalculator()
    for area, p in ((scatter(afc, pts), pts), (afc.grid_from_spec(g), gp)):
        out = calc.calculate(s, area, afc.ComplexPressureFieldBuffer())
        assert out.shape[0] == len(p)
        assert rel_err(out, O.field_f32(1, rec, k, a, p, O.FIELD_COMPLEX)) <= TOL
        assert rel_err(out, O.field_f64(1, rec, k, a, p)) <= TOL


def test_grid_beyond_2_31_points(gpu):
    """A 2048 x 2048 x 513 grid (2,151,677,952 points, past 2^31) through the device entry
    point, pressure kept on the device (8.6 GB): every point index is 64-bit.  4,096 sampled
    points, among them the last one and the ones past 2^31, match the oracle."""
    torch = pytest.importorskip("torch")
    afc = gpu
    rng = np.random.default_rng(2 ** 31 % 1000)
    rec, k, a = random_sources(rng, 1, 3)
    counts, res = (2048, 2048, 513), 0.5
    lo0 = (-512.0, -512.0, 40.0)
    g = W.GridSpec(3, [(lo0[j], lo0[j] + (counts[j] - 0.75) * res) for j in range(3)], res,
                   (1, 2, 3))
    area = afc.grid_from_spec(g)
    desc = area.grid_desc()
    assert tuple(int(c) for c in desc.count) == counts
    m = counts[0] * counts[1] * counts[2]
    assert m > 2 ** 31
    d_src = torch.from_numpy(rec.reshape(-1)).cuda()
    d_k = torch.from_numpy(k).cuda()
    d_a = torch.from_numpy(a).cuda()
    ws_bytes = afc.DLL.AFC_FieldWorkspaceBytes(len(k))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    out = torch.empty(m, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = afc.DLL.AFC_FieldGridDevice(1, 0, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                     len(k), ctypes.byref(desc), out.data_ptr(), ws.data_ptr(),
                                     ws_bytes, stream)
    assert rc == 0, afc.last_error()
    torch.cuda.synchronize()
    idx = np.concatenate([rng.integers(0, m, 4000), np.arange(2 ** 31 - 40, 2 ** 31 + 40),
                          np.arange(m - 16, m)]).astype(np.int64)
    got = out[torch.from_numpy(idx).cuda()].cpu().numpy()
    del out
    torch.cuda.empty_cache()
    i0 = idx % counts[0]
    i1 = (idx // counts[0]) % counts[1]
    i2 = idx // (counts[0] * counts[1])
    lo, _ = g.lo_hi()
    # o + (i as f32 * res), as the reference generates grid points
    pts = np.stack([lo[0] + (i0.astype(np.float32) * np.float32(res)),
                    lo[1] + (i1.astype(np.float32) * np.float32(res)),
                    lo[2] + (i2.astype(np.float32) * np.float32(res))], 1).astype(np.float32)
    ref = np.abs(O.field_f32(1, rec, k, a, pts))
    err = rel_err(got, ref)
    print(f"2^31+ grid: {m} points, sampled rel err {err:.2e}")
    assert err <= TOL


@pytest.mark.parametrize("calc", ["GpuCalculator", "AccurateCalculator"])
@pytest.mark.parametrize("tilted", [False, True])
def test_rows_split_mid_size(gpu, calc, tilted):
    """A 128 x 128 x 40 grid (655,360 points) has 320 rows tiles, half a wave short of filling
    its second wave, so the launch splits every tile's 996 sources over a cluster of blocks and
    combines the partial sums in rank order (plain and compensated).  Checked in full against
    the oracle."""
    afc = gpu
    rng = np.random.default_rng(17 + tilted)
    pos = W.tiled_array(2, 2)
    n = len(pos)
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, n).astype(np.float32),
                            rng.uniform(0, 2 * np.pi, n).astype(np.float32))
    if tilted:
        d = rng.normal(size=(n, 3)) * np.array([0.3, 0.3, 0.0]) + np.array([0, 0, 1.0])
        rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.full(n, 0.0115, np.float32)
    cen = W.array_center(pos)
    x0, y0 = float(cen[0]) - 32.0, float(cen[1]) - 32.0
    g = W.GridSpec(3, [(x0, x0 + 127.25 * 0.5), (y0, y0 + 127.25 * 0.5), (80.0, 80.0 + 39.25 * 0.5)],
                   0.5, (1, 2, 3))
    s = make_system(afc, 1, rec, k, a)
    lo, hi = g.lo_hi()
    pts = O.grid_points(3, lo, hi, 0.5, (1, 2, 3))
    assert len(pts) == 128 * 128 * 40
    out = getattr(afc, calc)().calculate(s, afc.grid_from_spec(g), afc.ComplexPressureFieldBuffer())
    ref = O.field_f32(1, rec, k, a, pts, accurate=(calc == "AccurateCalculator"))
    err = rel_err(out, ref)
    print(f"rows split {calc} tilted={tilted}: {err:.2e}")
    assert err <= TOL


@pytest.mark.parametrize("dist", [1000.0, 1500.0, 3000.0])
def test_far_field_with_random_phases(gpu, dist):
    """Every point 1, 1.5 or 3 m from a 4 x 4 tiling (3,984 sources) driven with random phases,
    no attenuation: the sum is incoherent, so the field's relative error is about the per-pair
    phase error, which grows with k r.  The far tiles take r through a Newton step, the phase
    rounded as the reference rounds it and a two-constant 2 pi reduction (the single-job
    kernels' careful tier; the mid tier of the batch and serving kernels, below 1,024 rad, is
    checked in test_batch_gpu.py).  Checked against the f32 oracle on a grid and scatter
    points."""
    afc = gpu
    rng = np.random.default_rng(int(dist))
    pos = W.tiled_array(4, 4)
    n = len(pos)
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, n).astype(np.float32),
                            rng.uniform(0, 2 * np.pi, n).astype(np.float32))
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.zeros(n, np.float32)
    s = make_system(afc, 1, rec, k, a)
    cen = W.array_center(pos)
    x0, y0 = float(cen[0]) - 40.0, float(cen[1]) - 40.0
    g = W.GridSpec(2, [(x0, x0 + 80.25), (y0, y0 + 80.25), (dist, dist)], 1.0, (1, 2, 3))
    lo, hi = g.lo_hi()
    gp = O.grid_points(2, lo, hi, 1.0, (1, 2, 3))
    pts = np.stack([rng.uniform(x0, x0 + 80, 2000), rng.uniform(y0, y0 + 80, 2000),
                    rng.uniform(dist, dist + 100, 2000)], 1).astype(np.float32)
    calc = afc.GpuCalculator()
    for area, p in ((afc.grid_from_spec(g), gp), (scatter(afc, pts), pts)):
        out = calc.calculate(s, area, afc.ComplexPressureFieldBuffer())
        err = rel_err(out, O.field_f32(1, rec, k, a, p, O.FIELD_COMPLEX))
        print(f"far field at {dist:.0f} mm, {len(p)} points: {err:.2e}")
        assert err <= TOL


@pytest.mark.parametrize("dim,axes,counts", [
    (3, (1, 2, 3), (64, 40, 3)), (3, (1, 3, 2), (64, 40, 3)), (3, (2, 1, 3), (64, 40, 3)),
    (3, (2, 3, 1), (64, 40, 3)), (3, (3, 1, 2), (64, 40, 3)), (3, (3, 2, 1), (64, 40, 3)),
    (2, (1, 2, 3), (128, 50, 1)), (2, (3, 1, 2), (250, 17, 1)), (3, (1, 2, 3), (256, 256, 10)),
])
@pytest.mark.parametrize("tilted", [False, True])
def test_rows_tiling(gpu, dim, axes, counts, tilted):
    """Grids evaluated by the rows kernel (a thread's points consecutive along the second axis,
    offsets along the other two shared): every axis order, counts that leave partial tiles, and
    (256 x 256 x 10) enough points for four point pairs per thread; sources facing one way or
    tilted (per-source directions)."""
    afc = gpu
    rng = np.random.default_rng(sum(counts) + dim + 3 * tilted)
    n = 300
    rec, k, a = random_sources(rng, 1, n)
    if not tilted:
        rec[:, 3:6] = (0.0, 0.0, 1.0)
    res = 0.75
    origin = {1: -30.0, 2: -20.0, 3: 70.0}
    spec = []
    for j, ax in enumerate(axes):
        lo_ = origin[ax]
        spec.append((lo_, lo_ + (counts[j] - 1) * res + 0.5 * res) if j < dim else (lo_, lo_))
    g = W.GridSpec(dim, spec, res, axes)
    s = make_system(afc, 1, rec, k, a)
    area = afc.grid_from_spec(g)
    assert tuple(int(c) for c in area.grid_desc().count) == tuple(counts[:dim]) + (1,) * (3 - dim)
    lo, hi = g.lo_hi()
    pts = O.grid_points(dim, lo, hi, res, axes)
    out = afc.GpuCalculator().calculate(s, area, afc.ComplexPressureFieldBuffer())
    assert out.shape[0] == len(pts)
    sel = np.arange(len(pts)) if len(pts) <= 40000 else np.random.default_rng(1).choice(
        len(pts), 40000, replace=False)
    ref = O.field_f32(1, rec, k, a, pts[sel], O.FIELD_COMPLEX)
    assert rel_err(out[sel], ref) <= TOL


def test_concurrent_calculators_match_serial(gpu):
    """Four Python threads, each with its own calculator and field buffer, calculate at the same
    time (ctypes releases the GIL around AFC_Calculate), five times each, on scatter and grid
    areas of one system: every result equals the serial one bit for bit (each calculator has
    its own stream and buffers; the kernels are deterministic)."""
    import threading

    afc = gpu
    rng = np.random.default_rng(21)
    rec, k, a = random_sources(rng, 1, 300)
    s = make_system(afc, 1, rec, k, a)
    pts = random_points(rng, 5000)
    areas = [scatter(afc, pts),
             afc.grid_from_spec(W.GridSpec(2, [(-30.0, 30.0), (-30.0, 30.0), (120.0, 120.0)], 0.5,
                                           (1, 2, 3)))]
    serial = [np.array(afc.GpuCalculator().calculate(s, ar, afc.ComplexPressureFieldBuffer()))
              for ar in areas]
    results, errors = [], []

    def work(t):
        try:
            calc = afc.GpuCalculator()
            f = afc.ComplexPressureFieldBuffer()
            for it in range(5):
                i = (t + it) % 2
                results.append((i, np.array(calc.calculate(s, areas[i], f))))
        except Exception as e:  # reported after the join
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    assert len(results) == 20
    for i, r in results:
        np.testing.assert_array_equal(r, serial[i])
