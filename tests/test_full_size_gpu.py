"""Parity of the two largest configured workloads at their real size.

Batch: the 2,048-job uneven mix (249 / 498 / 996 / 2,490 transducers, 1e3-1e6 points, grid
slices and scatter sets, three field types), planned with the autotuner and replayed from the
CUDA graph, as the benchmark runs it.  A seeded sample of jobs covering every source count,
both point kinds, every field type and the largest point counts is compared on a seeded point
subsample with the oracle (the reference's CPU calculator restated), for the graph replay and
for the one-by-one launches.

Serving: a seeded Poisson stream at 3,000 req/s of the configured mix (70 % field jobs from
the batched-job pool, 30 % GS-PAT requests with 2-64 foci on the 2 x 2 tiling, each followed by
a 201 x 201 pressure slice) through an engine with 32 slots.  Every result must equal its alone
run bit for bit (the reference's contract is one blocking AFC_Calculate per job,
capi/src/calculator.rs:53-117, whose field cannot depend on other work); a sample of field
results is compared with the oracle and a sample of GS-PAT drives with the float64 restatement
of gs_pat.rs.

Bars: max |p - p_ref| <= 1e-4 * max |p_ref| on the sampled points (2e-4 for the power field,
whose relative error doubles), for field results and for the GS-PAT slices (the field of the
served drive); GS-PAT drive max |q - q64| <= max(1e-4, 3 e32) * max |q64|, e32 the distance
from float64 of the reference's own f32 arithmetic on the same request (see GSPAT_SPREAD).
"""
import numpy as np
import pytest

import batch_device as BD
import oracle as O
import serving_client as SC
import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-4
SAMPLE_POINTS = 400
# GS-PAT's 100 normalised iterations converge to a fixed point that rounding moves on
# ill-conditioned foci sets: the reference's own f32 arithmetic (the oracle's gspat_f32) lands
# up to 1.6e-3 of the peak drive from float64 on requests of this stream, against a median of
# 1.1e-5.  A served drive must lie within max(1e-4, GSPAT_SPREAD x that f32 distance) of float64.
GSPAT_SPREAD = 3.0


def _transform(ref_c, ft):
    return ref_c if ft == 2 else (np.abs(ref_c) if ft == 0 else np.abs(ref_c) ** 2)


def _check(got, ref_c, ft, what):
    ref = _transform(ref_c, ft)
    peak = float(np.max(np.abs(ref)))
    err = float(np.max(np.abs(got - ref))) / peak
    assert err <= (2 if ft == 1 else 1) * TOL, f"{what}: {err:.3e}"
    return err


def _as_field(arr, ft):
    return arr.view(np.complex64) if ft == 2 else arr


def _sample_jobs(jobs, rng):
    """Indices of a job sample: for every (source count, grid or scatter, field type) the
    largest job and two others at random, and the 8 largest jobs overall."""
    pick = set()
    groups = {}
    for i, jb in enumerate(jobs):
        groups.setdefault((jb.n, jb.grid is not None, jb.field_type), []).append(i)
    for key, idx in groups.items():
        idx = sorted(idx, key=lambda i: -jobs[i].n_points)
        pick.add(idx[0])
        rest = idx[1:]
        pick.update(int(i) for i in rng.choice(rest, min(2, len(rest)), replace=False))
    pick.update(sorted(range(len(jobs)), key=lambda i: -jobs[i].n_points)[:8])
    return sorted(pick)


def test_batch_2048_jobs_autotuned_vs_oracle(gpu):
    torch = pytest.importorskip("torch")
    afc = gpu
    jobs = W.batch_jobs(n_jobs=2048)
    assert {jb.n for jb in jobs} == {249, 498, 996, 2490}
    arr, outs, pts, keep = BD.materialize(afc, torch, jobs)
    st = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2048)
    sample = _sample_jobs(jobs, rng)
    assert len(sample) >= 64
    # points and oracle fields of the sample (seeded point subsample per job)
    refs = {}
    for i in sample:
        jb = jobs[i]
        rows = np.sort(rng.choice(jb.n_points, min(SAMPLE_POINTS, jb.n_points), replace=False))
        if jb.grid is not None:
            lo, hi = jb.grid.lo_hi()
            p = O.grid_points(2, lo, hi, jb.grid.res, jb.grid.axes)
            assert len(p) == jb.n_points
            p = p[rows]
        else:
            p = pts[i].cpu().numpy()[rows]
        refs[i] = (rows, O.field_f32(1, jb.sources, jb.k, jb.atten, p))
    plan = BD.create_plan(afc, arr, True, st)
    try:
        info = BD.describe(afc, plan)
        worst = {}
        for mode in ("graph", "one_by_one"):
            for o in outs:
                o.fill_(float("nan"))
            fn = afc.DLL.AFC_BatchRun if mode == "graph" else afc.DLL.AFC_BatchRunOneByOne
            assert fn(plan, st) == 0, afc.last_error()
            torch.cuda.synchronize()
            worst[mode] = 0.0
            for i in sample:
                jb = jobs[i]
                rows, ref_c = refs[i]
                got = _as_field(outs[i].cpu().numpy(), jb.field_type)
                assert np.all(np.isfinite(got)), f"job {i}: unwritten or non-finite points"
                e = _check(got[rows], ref_c, jb.field_type, f"{mode} job {i} (n={jb.n}, "
                           f"m={jb.n_points}, grid={jb.grid is not None}, ft={jb.field_type})")
                worst[mode] = max(worst[mode], e)
        print(f"batch 2048 jobs, {len(sample)} sampled, plan {info}: worst {worst}")
    finally:
        afc.DLL.AFC_BatchFree(plan)


def _serving_setup(afc, eng):
    pool = W.batch_jobs(n_jobs=256)
    gid_of_n = {}
    for jb in pool:
        if jb.n not in gid_of_n:
            gid_of_n[jb.n] = eng.add_geometry(1, jb.sources, jb.k, jb.atten)
    gpos = W.tiled_array(2, 2)
    gsrc = W.t4010a1_records(gpos, 1.0, 0.0)
    gk = np.full(len(gpos), W.wavenumber(), np.float32)
    ga = np.zeros(len(gpos), np.float32)
    gid_gspat = eng.add_geometry(1, gsrc, gk, ga)
    return pool, gid_of_n, (gid_gspat, gsrc, gk, ga, W.array_center(gpos))


def _submit(afc, eng, pool, gid_of_n, gs, r, pts_cache):
    if r.kind == "field":
        jb = pool[r.job]
        amps = np.ascontiguousarray(jb.sources[:, 6])
        phases = np.ascontiguousarray(jb.sources[:, 7])
        if jb.grid is not None:
            desc = afc.grid_from_spec(jb.grid).grid_desc()
            rid, out = eng.submit_field(gid_of_n[jb.n], amps, phases, jb.field_type, grid=desc)
        else:
            if r.job not in pts_cache:
                pts_cache[r.job] = W.batch_job_points(jb)
            rid, out = eng.submit_field(gid_of_n[jb.n], amps, phases, jb.field_type,
                                        points=pts_cache[r.job])
        return rid, (out,)
    gid, gsrc, gk, ga, cen = gs
    desc, _ = SC.slice_desc(afc, cen, float(r.foci[:, 2].mean()), half=100.0, res=1.0)
    rid, out, ap = eng.submit_gspat(gid, len(gk), r.foci, r.amps, desc)
    return rid, (out, ap)


def test_serving_stream_at_load_same_alone_and_vs_oracle(gpu):
    afc = gpu
    import time

    eng = SC.Engine(afc, hbm_budget_bytes=2 << 30, pinned_bytes=2 << 30, max_inflight=32)
    try:
        pool, gid_of_n, gs = _serving_setup(afc, eng)
        stream = W.serving_stream(3000.0, 480, len(pool), seed=17)
        assert max(len(r.foci) for r in stream if r.kind == "gspat") >= 48
        pts_cache = {}
        # the stream on its arrival schedule: requests overlap on the device
        pending = []
        t0 = time.perf_counter()
        for r in stream:
            while time.perf_counter() - t0 < r.arrival:
                pass
            pending.append(_submit(afc, eng, pool, gid_of_n, gs, r, pts_cache))
        mixed = []
        for rid, outs in pending:
            eng.wait(rid)
            mixed.append([o.copy() for o in outs])
        st = eng.stats()
        assert st["failed"] == 0
        assert st["peak_inflight"] > 1, "the stream never overlapped on the device"
        # every request alone gives the same bits
        for r, mix in zip(stream, mixed):
            rid, outs = _submit(afc, eng, pool, gid_of_n, gs, r, pts_cache)
            eng.wait(rid)
            for o, m in zip(outs, mix):
                np.testing.assert_array_equal(o, m)
    finally:
        eng.close()
    # a sample against the oracle
    rng = np.random.default_rng(3000)
    gid, gsrc, gk, ga, cen = gs
    fields = [i for i, r in enumerate(stream) if r.kind == "field"]
    gspats = [i for i, r in enumerate(stream) if r.kind == "gspat"]
    worst_field, worst_slice, gspat_ratio = 0.0, 0.0, []
    for i in rng.choice(fields, 40, replace=False):
        jb = pool[stream[i].job]
        got = _as_field(mixed[i][0], jb.field_type)
        rows = np.sort(rng.choice(len(got), min(SAMPLE_POINTS, len(got)), replace=False))
        if jb.grid is not None:
            lo, hi = jb.grid.lo_hi()
            p = O.grid_points(2, lo, hi, jb.grid.res, jb.grid.axes)[rows]
        else:
            p = pts_cache[stream[i].job][rows]
        worst_field = max(worst_field, _check(got[rows],
                                              O.field_f32(1, jb.sources, jb.k, jb.atten, p),
                                              jb.field_type, f"served field request {i}"))
    big_first = sorted(gspats, key=lambda i: -len(stream[i].foci))
    for i in big_first[:4] + list(rng.choice(big_first[4:], 12, replace=False)):
        r = stream[i]
        slice_out, ap = mixed[i]
        q = ap[0::2].astype(np.float64) * np.exp(1j * ap[1::2].astype(np.float64))
        _, q64 = O.gspat_f64(1, gsrc, gk, ga, r.foci, r.amps)
        _, q32 = O.gspat_f32(1, gsrc, gk, ga, r.foci, r.amps)
        e = float(np.max(np.abs(q - q64)) / np.max(np.abs(q64)))
        e32 = float(np.max(np.abs(q32 - q64)) / np.max(np.abs(q64)))
        assert e <= max(TOL, GSPAT_SPREAD * e32), (
            f"GS-PAT request {i} (M={len(r.foci)}): drive {e:.3e}, reference f32 {e32:.3e}")
        gspat_ratio.append((e, e32, len(r.foci)))
        # the slice is the pressure field of the solved drive
        drive = gsrc.copy()
        drive[:, 6], drive[:, 7] = ap[0::2], ap[1::2]
        _, spec = SC.slice_desc(afc, cen, float(r.foci[:, 2].mean()), half=100.0, res=1.0)
        lo, hi = spec.lo_hi()
        rows = np.sort(rng.choice(201 * 201, SAMPLE_POINTS, replace=False))
        p = O.grid_points(2, lo, hi, spec.res, spec.axes)[rows]
        worst_slice = max(worst_slice, _check(slice_out[rows], O.field_f32(1, drive, gk, ga, p),
                                              0, f"GS-PAT slice {i}"))
    print(f"serving stream: worst field {worst_field:.2e}, worst slice {worst_slice:.2e}, "
          f"GS-PAT drive (gpu vs f64, reference f32 vs f64, M): "
          f"{[(f'{a:.1e}', f'{b:.1e}', m) for a, b, m in sorted(gspat_ratio)[-5:]]}")
