"""Opt-in source tracking (AFC_UniformSystemTrackSources / AFC_UniformSystemSourcesChanged).

The reference reads the host source array on every calculation (capi/src/calculator.rs:52-117)
and its consumers rewrite phases in place through AFC_GetWaveSources between calculations
(python/main.py:57-63).  By default every AFC_Calculate therefore uploads and packs the sources
again.  A caller that opts in and announces its in-place writes lets the calculator reuse its
packed device copy.  These tests check that:
  * without the opt-in an in-place write is always seen, also after tracking was on and off;
  * with it, unchanged sources are not uploaded or packed again (one kernel launch per call
    instead of two), an announced write is seen, and library-side changes (added sources,
    the optimizers) are seen without an announcement;
  * two systems alternating on one calculator, or a system created after another was freed,
    never get each other's packed copy.
"""
import numpy as np
import pytest

import oracle as O

from test_field_parity_gpu import TOL, make_system, random_points, random_sources, rel_err, scatter

pytestmark = pytest.mark.gpu


def _launches(afc):
    return afc.DLL.AFC_KernelLaunchCount()


def _calc(afc, calc, s, area, f):
    n0 = _launches(afc)
    out = calc.calculate(s, area, f)
    return out, _launches(afc) - n0


def _rewrite(rng, s):
    """Write new phases and amplitudes through the source array, as python/main.py does."""
    arr = s.records()
    arr[:, 7] = rng.uniform(-3, 3, len(arr)).astype(np.float32)
    arr[:, 6] = rng.uniform(0.1, 1.0, len(arr)).astype(np.float32)
    return arr


def _setup(afc, seed, n=64, m=400):
    rng = np.random.default_rng(seed)
    rec, k, a = random_sources(rng, 1, n)
    pts = random_points(rng, m)
    s = make_system(afc, 1, rec, k, a)
    return rng, s, k, a, pts, scatter(afc, pts), afc.GpuCalculator(), afc.ComplexPressureFieldBuffer()


def test_default_always_sees_in_place_writes(gpu):
    afc = gpu
    rng, s, k, a, pts, area, calc, f = _setup(afc, 41)
    arr = _rewrite(rng, s)  # the view is kept and written again below, without any call
    calc.calculate(s, area, f)
    for _ in range(3):
        arr[:, 7] = rng.uniform(-3, 3, len(arr)).astype(np.float32)
        out, launched = _calc(afc, calc, s, area, f)
        assert launched == 2  # pack + field: the sources were uploaded again
        assert rel_err(out, O.field_f32(1, arr.copy(), k, a, pts)) <= TOL


def test_tracked_sources_are_reused_until_announced(gpu):
    afc = gpu
    rng, s, k, a, pts, area, calc, f = _setup(afc, 42)
    arr = s.records()
    s.track_sources(True)
    first, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    again, launched = _calc(afc, calc, s, area, f)
    assert launched == 1  # field kernel only: the packed copy was reused
    np.testing.assert_array_equal(again, first)
    # a write through a view taken earlier is not seen until it is announced (the contract)
    arr[:, 7] = rng.uniform(-3, 3, len(arr)).astype(np.float32)
    stale, launched = _calc(afc, calc, s, area, f)
    assert launched == 1
    np.testing.assert_array_equal(stale, first)
    s.sources_changed()
    fresh, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    assert rel_err(fresh, O.field_f32(1, arr.copy(), k, a, pts)) <= TOL


def test_tracking_off_again_sees_unannounced_writes(gpu):
    afc = gpu
    rng, s, k, a, pts, area, calc, f = _setup(afc, 43)
    arr = s.records()
    s.track_sources(True)
    calc.calculate(s, area, f)
    calc.calculate(s, area, f)
    s.track_sources(False)
    arr[:, 7] = rng.uniform(-3, 3, len(arr)).astype(np.float32)
    out, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    assert rel_err(out, O.field_f32(1, arr.copy(), k, a, pts)) <= TOL


def test_library_changes_are_seen_while_tracking(gpu):
    afc = gpu
    rng, s, k, a, pts, area, calc, f = _setup(afc, 44)
    s.track_sources(True)
    calc.calculate(s, area, f)
    # the focal law rewrites every phase in the library
    afc.Optimizer.focus(s, (5.0, -3.0, 120.0))
    out, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    assert rel_err(out, O.field_f32(1, s.records().copy(), k, a, pts)) <= TOL
    # an added source changes the count
    rec2, k2, a2 = random_sources(rng, 1, 3)
    s.add_records(1, rec2, k2, a2)
    out, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    kk, aa = np.concatenate([k, k2]), np.concatenate([a, a2])
    assert rel_err(out, O.field_f32(1, s.records().copy(), kk, aa, pts)) <= TOL
    # GS-PAT writes amplitudes and phases in the library
    foci = np.array([[0.0, 0.0, 150.0], [20.0, 10.0, 140.0]], np.float32)
    afc.Optimizer.gs_pat(s, foci, np.array([1.0, 0.8], np.float32))
    out, launched = _calc(afc, calc, s, area, f)
    assert launched == 2
    assert rel_err(out, O.field_f32(1, s.records().copy(), kk, aa, pts)) <= TOL


def test_systems_alternating_on_one_calculator(gpu):
    afc = gpu
    rng = np.random.default_rng(45)
    pts = random_points(rng, 300)
    area = scatter(afc, pts)
    calc = afc.GpuCalculator()
    f = afc.ComplexPressureFieldBuffer()
    systems = []
    for _ in range(2):
        rec, k, a = random_sources(rng, 1, 48)
        s = make_system(afc, 1, rec, k, a)
        s.track_sources(True)
        systems.append((s, rec, k, a))
    for _ in range(2):
        for s, rec, k, a in systems:
            out = calc.calculate(s, area, f)
            assert rel_err(out, O.field_f32(1, rec, k, a, pts)) <= TOL
    # a system freed and another created (possibly at the same address) with other sources
    s0 = systems[0][0]
    calc.calculate(s0, area, f)
    del systems[0], s0
    rec, k, a = random_sources(rng, 1, 48)
    s_new = make_system(afc, 1, rec, k, a)
    s_new.track_sources(True)
    out = calc.calculate(s_new, area, f)
    assert rel_err(out, O.field_f32(1, rec, k, a, pts)) <= TOL
