"""Serving engine: requests admitted under an HBM budget run overlapped on the GPU, and each
result is the same alone as in the mix (same kernels, deterministic: compared exactly, and
against the oracle within 1e-4 of the peak)."""
import numpy as np
import pytest

import oracle as O
import serving_client as SC
import workloads as W

pytestmark = pytest.mark.gpu


def _geometries():
    g1 = W.tiled_array(1, 1)
    g4 = W.tiled_array(2, 2)
    out = []
    for pos in (g1, g4):
        src = W.t4010a1_records(pos, 1.0, 0.0)
        k = np.full(len(pos), W.wavenumber(), np.float32)
        a = np.full(len(pos), 1.15e-2, np.float32)
        out.append((src, k, a))
    return out


def _requests(afc, seed, geoms, n_field=12, n_gspat=6, slice_half=30.0):
    """GS-PAT requests (the slow ones: 100 solver iterations) first, then field requests that
    arrive while they run."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_gspat):
        M = int(rng.integers(2, 17))
        pos = geoms[1][0][:, :3]
        cen = W.array_center(pos)
        foci = np.empty((M, 3), np.float32)
        foci[:, 0] = rng.uniform(cen[0] - 50, cen[0] + 50, M)
        foci[:, 1] = rng.uniform(cen[1] - 50, cen[1] + 50, M)
        foci[:, 2] = rng.uniform(100, 200, M)
        tamps = rng.uniform(0.5, 1.0, M).astype(np.float32)
        desc, spec = SC.slice_desc(afc, cen, float(foci[:, 2].mean()), half=slice_half)
        reqs.append(("gspat", 1, foci, tamps, None, desc, spec, None))
    for i in range(n_field):
        g = int(rng.integers(0, 2))
        n = len(geoms[g][1])
        amps, phases = W.random_pattern(rng, n)
        ft = int(rng.integers(0, 3))
        cen = W.array_center(geoms[g][0][:, :3])
        if i % 2 == 0:
            desc, spec = SC.slice_desc(afc, cen, float(rng.uniform(60, 180)), half=20.0,
                                       res=float(rng.uniform(0.5, 2.0)))
            reqs.append(("field", g, amps, phases, ft, desc, spec, None))
        else:
            m = int(rng.integers(1, 3000))
            pts = W.scatter_box(int(rng.integers(1 << 30)), m, cen[:2], box=(80, 80), z=(60, 180))
            reqs.append(("field", g, amps, phases, ft, None, None, pts))
    return reqs


def _submit(eng, gids, geoms, r):
    kind, g, a, b, ft, desc, spec, pts = r
    if kind == "field":
        rid, out = eng.submit_field(gids[g], a, b, ft, grid=desc, points=pts)
        return rid, (out,)
    rid, out, ap = eng.submit_gspat(gids[g], len(geoms[g][1]), a, b, desc)
    return rid, (out, ap)


def test_results_same_alone_and_in_the_mix(gpu):
    afc = gpu
    geoms = _geometries()
    eng = SC.Engine(afc, 1 << 30, 1 << 28, 8)
    try:
        gids = [eng.add_geometry(1, *g) for g in geoms]
        reqs = _requests(afc, 7, geoms)
        # all at once: they overlap on the device
        pending = [_submit(eng, gids, geoms, r) for r in reqs]
        mixed = []
        for rid, outs in pending:
            eng.wait(rid)
            mixed.append([o.copy() for o in outs])
        st = eng.stats()
        assert st["peak_inflight"] > 1 and st["failed"] == 0
        # one at a time
        for r, mix in zip(reqs, mixed):
            rid, outs = _submit(eng, gids, geoms, r)
            eng.wait(rid)
            for o, m in zip(outs, mix):
                np.testing.assert_array_equal(o, m)
        # the field requests against the oracle (1e-4 of the peak)
        for r, mix in zip(reqs, mixed):
            kind, g, amps, phases, ft, desc, spec, pts = r
            if kind != "field":
                continue
            src, k, a = geoms[g]
            s = src.copy()
            s[:, 6], s[:, 7] = amps, phases
            if spec is not None:
                lo, hi = spec.lo_hi()
                pts = O.grid_points(2, lo, hi, spec.res, spec.axes)
            ref = O.field_f32(1, s, k, a, pts, field=ft)
            got = mix[0].view(np.complex64) if ft == 2 else mix[0]
            assert got.shape == ref.shape
            assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref))
    finally:
        eng.close()


def test_gspat_request_matches_the_optimizer_call(gpu):
    """A served GS-PAT request gives the drive of AFO_GSPAT and the slice of AFC_Calculate."""
    afc = gpu
    geoms = _geometries()
    eng = SC.Engine(afc, 1 << 30, 1 << 28, 4)
    try:
        gids = [eng.add_geometry(1, *g) for g in geoms]
        r = _requests(afc, 11, geoms, n_field=0, n_gspat=1)[0]
        rid, outs = _submit(eng, gids, geoms, r)
        eng.wait(rid)
        slice_out, ap = outs
        src, k, a = geoms[1]
        s = afc.UniformSystem(300.0)
        s.add_records(1, src, k, a)
        afc.Optimizer.gs_pat(s, r[2], r[3])
        rec = s.records()
        np.testing.assert_allclose(ap[0::2], rec[:, 6], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(ap[1::2], rec[:, 7], atol=1e-6)
        area = afc.grid_from_spec(r[6])
        ref = afc.GpuCalculator().calculate(s, area, afc.PressureFieldBuffer())
        assert np.max(np.abs(slice_out - ref)) <= 1e-5 * np.max(ref)
    finally:
        eng.close()


def test_hbm_budget_limits_admission(gpu):
    afc = gpu
    geoms = _geometries()
    # room for one 41x41-point complex field request of the 996-source geometry at a time: its
    # drive, packed sources and result, and the partial sums of its 7 source chunks (a request
    # that small is cut into chunks of at least 128 sources to spread over the GPU)
    one = 256 * 4 + 8 * 996 + 48 * 996 + 8 * 1681 + 8 * 7 * 1681 + 4096
    eng = SC.Engine(afc, one, 1 << 26, 8)
    try:
        gid = eng.add_geometry(1, *geoms[1])
        cen = W.array_center(geoms[1][0][:, :3])
        desc, _ = SC.slice_desc(afc, cen, 120.0, half=20.0, res=1.0)  # 41 x 41
        rng = np.random.default_rng(3)
        subs = []
        for _ in range(6):
            amps, phases = W.random_pattern(rng, 996)
            subs.append(eng.submit_field(gid, amps, phases, 2, grid=desc)[0])
        for rid in subs:
            eng.wait(rid)
        st = eng.stats()
        assert st["completed"] >= 6 and st["peak_inflight"] == 1
        assert st["peak_hbm_bytes"] <= st["hbm_budget_bytes"]
        big, _ = SC.slice_desc(afc, cen, 120.0, half=60.0, res=0.5)
        with pytest.raises(RuntimeError, match="budget"):
            eng.submit_field(gid, amps, phases, 2, grid=big)
    finally:
        eng.close()
