"""CPU tests of libafccapi.so: it loads, exports every symbol declared in include/*.h, and its
host-side logic (handles, set-up arithmetic, grid sizes, info strings, focal law, errors)
matches the oracle.  No compute is launched here."""
import ctypes
import math
import os
import re
from ctypes import byref, c_float, c_uint, c_void_p

import numpy as np
import pytest

import oracle as O
import workloads as W

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for fn in ("afccapi.h", "afc_gpu.h"):
        text = open(os.path.join(REPO, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(AF[CO]_[A-Za-z0-9]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(afc_mod):
    names = _declared_functions()
    assert len(names) >= 48  # 38 reference exports + the additions
    lib = ctypes.CDLL(afc_mod.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_binding_list_is_declared(afc_mod):
    from afc import nativemethods as nm

    names = _declared_functions()
    for n in nm.REFERENCE_EXPORTS + nm.NEW_EXPORTS:
        assert n in names, n


def _system(afc_mod, temperature=300.0):
    sys_ = afc_mod.UniformSystem(temperature)
    return sys_


def test_add_sources_derives_k_and_alpha_like_the_reference(afc_mod):
    s = _system(afc_mod, 300.0)
    for x in range(3):
        s.add_wave_source(afc_mod.T4010A1((10.0 * x, 0, 0), (0, 0, 1), 1.0, 0.0, 40e3))
    k, a = O.wavenum_atten(300.0, 40e3)
    info = s.source_info_string(1)
    assert s.sound_speed() == O.sound_speed(300.0)
    assert f"Wavenumber: " in info and "Np/mm" in info
    # the ABI does not expose k directly; the info string carries it in Rust's formatting
    kv = float(re.search(r"Wavenumber: ([0-9.e-]+)", info).group(1))
    av = float(re.search(r"Attenuation: ([0-9.e-]+)", info).group(1))
    assert np.float32(kv) == np.float32(k)
    assert np.float32(av) == np.float32(a)


def test_info_strings_use_rust_float_formatting(afc_mod):
    s = _system(afc_mod, 300.0)
    s.add_wave_source(afc_mod.SphereWaveSource((0, 0, 0), 1.0, 0.0, 40e3))
    info = s.info_string()
    # f32 300 - 273.15 = 26.850006 and Rust prints the shortest round-trip form
    t = np.float32(300.0) - np.float32(273.15)
    c = O.sound_speed(300.0)
    assert info == ("Uniform Medium:\n Temperature: 300 K = " + repr(float(t)).rstrip("0")
                    .rstrip(".") + " ℃\n Sound Speed: " + f"{np.float32(c)}" + " mm/s") or \
        info.startswith("Uniform Medium:\n Temperature: 300 K = 26.850006")
    assert "Sound Speed: 347201.38 mm/s" in info


def test_get_wave_sources_is_a_mutable_view(afc_mod):
    s = _system(afc_mod)
    for i in range(4):
        s.add_wave_source(afc_mod.T4010A1((i, 0, 0), (0, 0, 1), 1.0, 0.0, 40e3))
    arr = s.get_wave_sources()
    arr[2].phase = 1.25
    arr[3].amp = 0.5
    rec = s.records()
    assert rec[2, 7] == np.float32(1.25)
    assert rec[3, 6] == np.float32(0.5)
    assert len(arr) == 4


def test_focal_point_matches_oracle(afc_mod):
    pos = W.unit_array()
    s = _system(afc_mod, 300.0)
    s.add_records(1, W.t4010a1_records(pos, 1.0, 0.0))
    focus = (86.36, 66.04, 150.0)
    afc_mod.Optimizer.focus(s, focus)
    expect = O.focal_point(1, W.t4010a1_records(pos, 1.0, 0.0), O.sound_speed(300.0), focus)
    np.testing.assert_array_equal(s.records().reshape(-1), expect)


@pytest.mark.parametrize("st", [0, 1])
@pytest.mark.parametrize("direction,theta", [((0.0, 0.0, 1.0), 0.3), ((0.3, -0.2, 0.93), 0.15),
                                             ((-0.5, 0.1, 0.86), 0.05)])
def test_bessel_beam_matches_oracle(afc_mod, st, direction, theta):
    """AFO_BesselBeam (host set-up, bessel.rs:30-51) equals the oracle bit for bit, for axial
    and tilted beams, on both source types; other record fields are untouched."""
    pos = W.tiled_array(2, 1)
    rng = np.random.default_rng(5)
    rec = (W.t4010a1_records if st == 1 else W.sphere_records)(
        pos, rng.uniform(0.5, 1.0, len(pos)).astype(np.float32), 0.0)
    s = _system(afc_mod, 293.0)
    s.add_records(st, rec)
    point = (90.0, 70.0, 0.0)
    afc_mod.Optimizer.bessel(s, point, direction, theta)
    expect = O.bessel_beam(st, rec, O.sound_speed(293.0), point, direction, theta)
    np.testing.assert_array_equal(s.records().reshape(-1), expect)
    iph = 7 if st == 1 else 4
    assert np.all(np.abs(s.records()[:, iph]) <= 2 * np.pi)
    assert np.ptp(s.records()[:, iph]) > 1.0  # the phases vary across the array


@pytest.mark.parametrize("spec", [
    (1, [(0.0, 10.0), (3.0, 3.0), (4.0, 4.0)], 0.7, (2, 1, 3)),
    (2, [(36.36, 136.36), (16.04, 116.04), (150.0, 150.0)], 1.0, (1, 2, 3)),
    (2, [(-5.0, 5.0), (0.0, 3.3), (7.0, 7.0)], 0.1, (3, 1, 2)),
    (3, [(0.0, 1.0), (0.0, 2.0), (0.0, 3.0)], 0.25, (2, 3, 1)),
])
def test_grid_size_matches_oracle(afc_mod, spec):
    dim, ranges, res, axes = spec
    g = W.GridSpec(dim, ranges, res, axes)
    area = afc_mod.grid_from_spec(g)
    lo, hi = g.lo_hi()
    expect = tuple(O.axis_count(lo[i], hi[i], res) for i in range(3))
    assert area.get_size() == expect
    d = area.grid_desc()
    assert list(d.axis) == list(axes)
    cnt = [expect[a - 1] for a in axes]
    assert list(d.count) == [cnt[k] if k < dim else 1 for k in range(3)]


def test_bad_axes_are_rejected_not_aborted(afc_mod):
    h = c_void_p()
    afc_mod.DLL.AFC_CreateGridArea2D(byref(h), 0, 1, 0, 1, 0, 0.1, 1, 1, 3)
    assert not h
    assert "axis" in afc_mod.last_error()


def test_unknown_tags_are_rejected(afc_mod):
    h = c_void_p()
    afc_mod.DLL.AFC_CreateCalculator(byref(h), 7)
    assert not h
    assert "calculator" in afc_mod.last_error()
    afc_mod.DLL.AFC_CreateUniformSystem(byref(h), 300.0, 5)
    assert not h


def test_calculate_without_gpu_fails_loudly(afc_mod, has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    s = _system(afc_mod)
    s.add_wave_source(afc_mod.SphereWaveSource((0, 0, 0), 1.0, 0.0, 40e3))
    area = afc_mod.GridAreaBuilder().x_range((0, 1)).y_at(0).z_at(10).resolution(1).generate()
    with pytest.raises(RuntimeError, match="no CUDA device"):
        afc_mod.GpuCalculator().calculate(s, area, afc_mod.PressureFieldBuffer())


def test_mismatched_tags_are_rejected(afc_mod):
    s = _system(afc_mod)
    s.add_wave_source(afc_mod.SphereWaveSource((0, 0, 0), 1.0, 0.0, 40e3))
    area = afc_mod.GridAreaBuilder().x_range((0, 1)).y_at(0).z_at(10).resolution(1).generate()
    calc = afc_mod.CpuCalculator()
    f = afc_mod.PressureFieldBuffer()
    out = c_void_p()
    # field type 1 (power) against a pressure buffer
    n = afc_mod.DLL.AFC_Calculate(calc.handle, s.handle, area.handle, f.handle, byref(out), 0,
                                  0, 0, 1)
    assert n == 0 and not out
    assert "field type" in afc_mod.last_error()


def test_unsupported_optimizers_leave_system_unchanged(afc_mod):
    s = _system(afc_mod)
    s.add_records(1, W.t4010a1_records(W.unit_array()[:5], 1.0, 0.25))
    before = s.records().copy()
    with pytest.raises(RuntimeError, match="not provided"):
        v = afc_mod.Vector3
        afc_mod.Optimizer.ifft(s, "pattern.bmp", v((0, 0, 0)), v((0, 10, 0)), v((10, 0, 0)), 1.0,
                               100.0)
    np.testing.assert_array_equal(s.records(), before)


def test_workspace_bytes(afc_mod):
    assert afc_mod.DLL.AFC_FieldWorkspaceBytes(0) == 0
    assert afc_mod.DLL.AFC_FieldWorkspaceBytes(1) == 256
    assert afc_mod.DLL.AFC_FieldWorkspaceBytes(3984) >= 3984 * 48


def test_grid_whose_point_count_would_wrap_is_rejected(afc_mod):
    """Counts whose product does not fit in 62 bits (here 4,194,305 per axis) make AFC_Calculate
    fail with an error before any device work, instead of computing a wrapped size.  (A zero
    resolution keeps the reference's release-build behaviour: the count, inf as usize plus 1,
    wraps to 0 and the field is empty.)"""
    s = _system(afc_mod)
    s.add_records(1, W.t4010a1_records(W.unit_array()[:5], 1.0, 0.0))
    big = (afc_mod.GridAreaBuilder().x_range((0.0, 4194304.0)).y_range((0.0, 4194304.0))
           .z_range((0.0, 4194304.0)).resolution(1.0).generate())
    assert big.get_size() == (4194305, 4194305, 4194305)
    with pytest.raises(RuntimeError, match="too many points"):
        afc_mod.GpuCalculator().calculate(s, big, afc_mod.PressureFieldBuffer())


def test_workspace_sizes_beyond_the_limits_are_zero(afc_mod):
    """Sizes whose byte counts could wrap report a zero workspace (and the calls taking them
    reject the problem) instead of a wrapped, too small size."""
    dll = afc_mod.DLL
    assert dll.AFC_FieldWorkspaceBytes(1 << 40) == 0
    assert dll.AFC_MultiPatternWorkspaceBytes(1 << 31, 1000, 8, 1) == 0
    assert dll.AFC_MultiPatternWorkspaceBytes(3984, 1 << 31, 8, 1) == 0
    assert dll.AFC_MultiPatternWorkspaceBytes(1 << 30, 1 << 30, 8, 1) == 0
    assert dll.AFC_MultiPatternWorkspaceBytes(3984, 262144, 1024, 1) > 8_000_000_000


def test_source_tracking_flags_check_their_handle(afc_mod):
    """The opt-in source-tracking calls accept a system of the matching tag and reject anything
    else with AFC_ERR_INVALID (-1), without touching the sources."""
    s = _system(afc_mod)
    s.add_records(1, W.t4010a1_records(W.unit_array()[:4], 1.0, 0.5))
    before = s.records().copy()
    dll = afc_mod.DLL
    assert dll.AFC_UniformSystemTrackSources(s.handle, 1, 1) == 0
    assert dll.AFC_UniformSystemSourcesChanged(s.handle, 1) == 0
    assert dll.AFC_UniformSystemTrackSources(s.handle, 1, 0) == 0
    assert dll.AFC_UniformSystemTrackSources(s.handle, 0, 1) == -1  # wrong source tag
    assert "source type" in afc_mod.last_error()
    assert dll.AFC_UniformSystemSourcesChanged(None, 1) == -1
    area = afc_mod.GridAreaBuilder().x_range((0, 1)).y_at(0).z_at(10).resolution(1).generate()
    assert dll.AFC_UniformSystemSourcesChanged(area.handle, 1) == -1  # not a system
    np.testing.assert_array_equal(s.records(), before)
    s.track_sources(True)
    s.sources_changed()
