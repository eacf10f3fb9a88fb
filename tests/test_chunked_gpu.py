"""The chunked launches (field_chunk_kernel or field_rows_chunk_kernel, then
field_chunk_combine_kernel).

Scatter sets whose 2,048-point tiles cannot fill the GPU's resident blocks (tens of tiles against
3,984 sources) are cut into contiguous ranges of (tile, source) work over persistent blocks:
each block sums one or two source ranges of one or two tiles, writes their partial sums, and a
second launch adds each point's partial sums in source order.  The reference sums every point
serially over its sources (uniform_medium.rs:122-128); the partial sums only regroup that sum,
so the bar is the same 1e-4 of the peak against the f32 oracle.  Checked here:
  * the launch takes the chunked path (pack + chunk + combine: three launches);
  * the field against the oracle at sizes with a ragged last tile, in full and (262,144 points)
    on a seeded subsample;
  * the same inputs give the same bits on every call (the split depends on the device only);
  * a point on a source comes out non-finite like the reference's (the combine's fix-up);
  * grids the rows tiling takes (a 64^3 grid; a 600 x 400 slice, ragged along both axes of its
    32 x 64 tiles) run the same launch over the rows tiles, and a 450 x 300 slice, which the
    rows tiles would leave 12 % idle, over the flat numbering's tiles; checked against the
    oracle.
"""
import numpy as np
import pytest

import oracle as O
import workloads as W

from test_field_parity_gpu import TOL, make_system, rel_err, scatter

pytestmark = pytest.mark.gpu


def _array_system(afc, seed):
    rng = np.random.default_rng(seed)
    pos = W.tiled_array(4, 4)
    n = len(pos)
    rec = W.t4010a1_records(pos, rng.uniform(0.5, 1.0, n).astype(np.float32),
                            rng.uniform(0, 2 * np.pi, n).astype(np.float32))
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.full(n, 0.0115, np.float32)
    return rng, pos, rec, k, a, make_system(afc, 1, rec, k, a)


def _calc(afc, calc, s, area):
    n0 = afc.DLL.AFC_KernelLaunchCount()
    out = calc.calculate(s, area, afc.ComplexPressureFieldBuffer())
    return out, afc.DLL.AFC_KernelLaunchCount() - n0


@pytest.mark.parametrize("m", [40_000, 65_536 + 77])
def test_chunked_scatter_in_full(gpu, m):
    afc = gpu
    rng, pos, rec, k, a, s = _array_system(afc, m)
    pts = W.scatter_box(m, m, W.array_center(pos)[:2])
    area = scatter(afc, pts)
    calc = afc.GpuCalculator()
    out, launched = _calc(afc, calc, s, area)
    assert launched == 3, "expected pack + chunked field + combine"
    err = rel_err(out, O.field_f32(1, rec, k, a, pts, O.FIELD_COMPLEX))
    print(f"chunked scatter, {m} points: {err:.2e}")
    assert err <= TOL
    again, _ = _calc(afc, calc, s, area)
    np.testing.assert_array_equal(again.view(np.uint32), out.view(np.uint32))


def test_chunked_scatter_262144_sampled(gpu):
    afc = gpu
    m = 262_144
    rng, pos, rec, k, a, s = _array_system(afc, 7)
    pts = W.scatter_box(7, m, W.array_center(pos)[:2])
    out, launched = _calc(afc, afc.GpuCalculator(), s, scatter(afc, pts))
    assert launched == 3
    idx = np.sort(rng.choice(m, 4000, replace=False))
    idx[-1] = m - 1
    err = rel_err(out[idx], O.field_f32(1, rec, k, a, pts[idx], O.FIELD_COMPLEX))
    print(f"chunked scatter, {m} points, 4,000 sampled: {err:.2e}")
    assert err <= TOL


def test_chunked_point_on_a_source(gpu):
    afc = gpu
    rng, pos, rec, k, a, s = _array_system(afc, 11)
    m = 40_000
    pts = W.scatter_box(11, m, W.array_center(pos)[:2])
    hit = 12_345
    pts[hit] = rec[1000, :3]
    out, launched = _calc(afc, afc.GpuCalculator(), s, scatter(afc, pts))
    assert launched == 3
    ref = O.field_f32(1, rec, k, a, pts, O.FIELD_COMPLEX)
    assert not np.isfinite(out[hit]) and not np.isfinite(ref[hit])
    keep = np.ones(m, bool)
    keep[hit] = False
    assert np.all(np.isfinite(out[keep]))
    assert rel_err(out[keep], ref[keep]) <= TOL


@pytest.mark.parametrize("shape", ["cube64", "slice600x400", "slice450x300"])
def test_chunked_grid(gpu, shape):
    afc = gpu
    rng, pos, rec, k, a, s = _array_system(afc, {"cube64": 64, "slice600x400": 600}.get(shape, 450))
    cen = W.array_center(pos)
    res = 0.5
    if shape == "cube64":
        counts = (64, 64, 64)
        lo = (float(cen[0]) - 16.0, float(cen[1]) - 16.0, 60.0)
        g = W.GridSpec(3, [(lo[j], lo[j] + (counts[j] - 0.75) * res) for j in range(3)], res,
                       (1, 2, 3))
    else:
        c0, c1 = (600, 400) if shape == "slice600x400" else (450, 300)
        counts = (c0, c1, 1)
        lo = (float(cen[0]) - 150.0, float(cen[1]) - 100.0, 150.0)
        g = W.GridSpec(2, [(lo[0], lo[0] + (c0 - 0.75) * res), (lo[1], lo[1] + (c1 - 0.75) * res),
                           (lo[2], lo[2])], res, (1, 2, 3))
    area = afc.grid_from_spec(g)
    out, launched = _calc(afc, afc.GpuCalculator(), s, area)
    assert launched == 3, "expected pack + chunked field + combine"
    glo, ghi = g.lo_hi()
    pts = O.grid_points(g.dim, glo, ghi, res, (1, 2, 3))
    assert len(pts) == counts[0] * counts[1] * counts[2] == len(out)
    idx = np.sort(rng.choice(len(pts), 6000, replace=False))
    idx[0], idx[-1] = 0, len(pts) - 1
    err = rel_err(out[idx], O.field_f32(1, rec, k, a, pts[idx], O.FIELD_COMPLEX))
    print(f"chunked grid {shape}: {err:.2e}")
    assert err <= TOL


def test_stream_capture_falls_back_to_the_cluster_split(gpu):
    """Under stream capture the chunked launch cannot take its partial sums from the stream, so a
    launch it would take runs as the cluster split inside the graph: the replayed graph's field
    matches the oracle and the eager (chunked) launch's to the parity bar."""
    torch = pytest.importorskip("torch")
    afc = gpu
    rng, pos, rec, k, a, s = _array_system(afc, 77)
    m = 65_536
    pts = W.scatter_box(77, m, W.array_center(pos)[:2])
    d_src, d_k, d_a, d_pts = (torch.from_numpy(x.reshape(-1)).cuda() for x in (rec, k, a, pts))
    n = len(k)
    wsb = afc.DLL.AFC_FieldWorkspaceBytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    eager = torch.empty(2 * m, dtype=torch.float32, device="cuda")
    captured = torch.full((2 * m,), float("nan"), dtype=torch.float32, device="cuda")

    def field(out, stream):
        return afc.DLL.AFC_FieldScatterDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(),
                                              d_a.data_ptr(), n, d_pts.data_ptr(), m,
                                              out.data_ptr(), ws.data_ptr(), wsb, stream)

    n0 = afc.DLL.AFC_KernelLaunchCount()
    assert field(eager, torch.cuda.current_stream().cuda_stream) == 0, afc.last_error()
    assert afc.DLL.AFC_KernelLaunchCount() - n0 == 3  # pack + chunked field + combine
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        n0 = afc.DLL.AFC_KernelLaunchCount()
        assert field(captured, torch.cuda.current_stream().cuda_stream) == 0, afc.last_error()
        assert afc.DLL.AFC_KernelLaunchCount() - n0 == 2  # pack + cluster split
    graph.replay()
    torch.cuda.synchronize()
    got_c = captured.cpu().numpy().view(np.complex64)
    got_e = eager.cpu().numpy().view(np.complex64)
    idx = np.sort(rng.choice(m, 4000, replace=False))
    ref = O.field_f32(1, rec, k, a, pts[idx], O.FIELD_COMPLEX)
    assert rel_err(got_c[idx], ref) <= TOL
    assert rel_err(got_c, got_e) <= TOL
