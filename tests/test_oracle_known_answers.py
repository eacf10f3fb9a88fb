"""Known-answer tests that pin the oracle (oracle/afc_oracle.c) to the reference's formulas.

The reference ships no golden vectors for this path and cannot be built here (Rust), so each
test recomputes a formula independently in numpy (float64 unless stated) from the cited
reference lines and compares it with the oracle.  CPU only.
"""
import math

import numpy as np
import pytest

import oracle as O
import workloads as W

# t4010a1.rs:18-69, re-typed here independently of the C oracle.
DIR = np.array([
    [0., 0., 0., 0.],
    [1.0, 0., 0., 0.],
    [1.0, 0., 0., 0.],
    [1.0, -0.2633589359691162, -2.586746661956269, 0.0009174516976956062],
    [0.891250938, -0.8910683499820542, -1.0097633564074366, 0.0001704413361662757],
    [0.707945784, -1.1924098538381465, -0.7167962799004945, 4.362034715924911],
    [0.501187234, -1.0439934287916925, 0.027352097655185065, -2.238476800444034],
    [0.354813389, -0.7015151838490918, 0.39509604454751995, 1.274774620435337],
    [0.251188643, -0.4471050803642494, 1.0625664749725618, -1.1276955684895724],
    [0.199526231, -0.179254124486545, 0.008242027161100222, -0.9016569137759131],
], dtype=np.float64)


def directivity_np(theta: float) -> float:
    """t4010a1.rs:107-120 in float64."""
    div = math.pi / 18
    i = math.ceil(theta / div)
    if i == 0:
        return 1.0
    if i > 9:
        return 0.0
    a, b, c, d = DIR[i]
    x = theta - (i - 1) * div
    return a + (b + (c + d * x) * x) * x


def attenuation_np(freq, hr, ps, ps0, t):
    """attenuation.rs:31-48 (Bass et al. 1995) in float64."""
    T0, T01 = 293.15, 273.16
    psat = ps0 * 10 ** (-6.8346 * (T01 / t) ** 1.261 + 4.6151)
    h = ps0 * (hr / ps) * (psat / ps0)
    f_ro = (24 + 4.04e4 * h * (0.02 + h) / (0.391 + h)) / ps0
    f_rn = (1 / ps0) * (9 + 280 * h * math.exp(-4.17 * ((T0 / t) ** (1 / 3) - 1))) * (T0 / t) ** 0.5
    f = freq / ps
    alpha = (f * f) / ps0 * ps * (1.84 * (t / T0) ** 0.5 * 1e-11 + (t / T0) ** -2.5 * (
        0.01278 * math.exp(-2239.1 / t) / (f_ro + f * f / f_ro)
        + 0.1068 * math.exp(-3352 / t) / (f_rn + f * f / f_rn)))
    return alpha * 1e-3


@pytest.mark.parametrize("t", [273.15, 287.684, 293.15, 300.0, 310.5])
def test_sound_speed(t):
    # sound_speed.rs:22-24, float32 arithmetic in the same order
    f = np.float32
    expect = f(f(331.3) * np.sqrt(f(t) / f(273.15))) * f(1000.0)
    assert O.sound_speed(t) == expect
    assert O.sound_speed(t) == pytest.approx(331.3 * math.sqrt(t / 273.15) * 1000, rel=1e-6)


@pytest.mark.parametrize("t", [280.0, 300.0])
@pytest.mark.parametrize("freq", [20e3, 40e3, 70e3])
def test_attenuation(t, freq):
    assert O.attenuation_coef(freq, 30, 1, 1, t) == pytest.approx(
        attenuation_np(freq, 30, 1, 1, t), rel=2e-5)


def test_attenuation_value_at_300k():
    # 40 kHz, 30 % RH, 1 atm, 300 K: 1.646e-4 Np/mm
    assert O.attenuation_coef(40e3, 30, 1, 1, 300.0) == pytest.approx(1.646e-4, rel=1e-3)


def test_wavenumber_from_temperature():
    k, a = O.wavenum_atten(300.0, 40e3)
    c = O.sound_speed(300.0)
    assert k == pytest.approx(2 * math.pi * 40e3 / c, rel=1e-6)
    assert a == O.attenuation_coef(40e3, 30, 1, 1, 300.0)


@pytest.mark.parametrize("deg", [0.0, 5.0, 10.0, 19.9, 20.0, 20.1, 25.0, 29.99, 30.01, 45.0,
                                 59.5, 60.5, 75.0, 85.0, 89.9, 90.5, 120.0, 180.0])
def test_directivity_values(deg):
    th = math.radians(deg)
    # the oracle keeps the reference's f32 coefficients, so float64 agrees to their rounding
    assert O.directivity_f64(th) == pytest.approx(directivity_np(th), abs=1e-7)
    assert O.directivity(th) == pytest.approx(directivity_np(th), abs=2e-6)


def test_directivity_regions():
    assert O.directivity(0.0) == 1.0
    for deg in np.linspace(0.01, 19.99, 50):
        assert O.directivity(math.radians(deg)) == 1.0
    for deg in np.linspace(90.01, 180, 50):
        assert O.directivity(math.radians(deg)) == 0.0
    assert O.directivity(float("nan")) == 1.0  # Rust `NaN as usize` == 0


def test_directivity_bin_edges_follow_the_table():
    # just above each 10-degree edge the cubic restarts at the next bin's `a`
    for i in range(3, 10):
        edge = (i - 1) * math.pi / 18
        assert O.directivity_f64(edge + 1e-9) == pytest.approx(DIR[i][0], abs=1e-7)


def _single_sphere(amp=0.8, phase=0.3, alpha=0.01, k=0.7):
    src = W.sphere_records(np.array([[1.0, -2.0, 0.5]], np.float32), amp, phase)
    return src, np.array([k], np.float32), np.array([alpha], np.float32)


def test_single_sphere_source_is_analytic():
    src, k, a = _single_sphere()
    rng = np.random.default_rng(0)
    pts = rng.uniform(-50, 50, (200, 3)).astype(np.float32)
    pts[:, 2] = np.abs(pts[:, 2]) + 10
    p = O.field_f32(O.SRC_SPHERE, src, k, a, pts, O.FIELD_COMPLEX)
    d = pts.astype(np.float64) - src[0, :3].astype(np.float64)
    r = np.linalg.norm(d, axis=1)
    expect = 0.8 * np.exp(-0.01 * r) / r * np.exp(1j * (0.3 + 0.7 * r))
    assert np.max(np.abs(p - expect)) <= 2e-6 * np.max(np.abs(expect))
    pr = O.field_f32(O.SRC_SPHERE, src, k, a, pts, O.FIELD_PRESSURE)
    pw = O.field_f32(O.SRC_SPHERE, src, k, a, pts, O.FIELD_POWER)
    np.testing.assert_allclose(pr, np.abs(expect), rtol=2e-6)
    np.testing.assert_allclose(pw, np.abs(expect) ** 2, rtol=4e-6)


def test_single_t4010a1_matches_numpy_restatement():
    rng = np.random.default_rng(1)
    pos = np.array([[3.0, 4.0, 0.0]], np.float32)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    src = W.t4010a1_records(pos, 0.9, 1.1)
    src[0, 3:6] = d
    k = np.array([0.73], np.float32)
    a = np.array([0.002], np.float32)
    pts = rng.uniform(-80, 80, (300, 3)).astype(np.float32)
    p = O.field_f32(O.SRC_T4010A1, src, k, a, pts)
    p64 = O.field_f64(O.SRC_T4010A1, src, k, a, pts)
    for i in range(0, 300, 7):
        dv = pts[i].astype(np.float64) - pos[0]
        r = np.linalg.norm(dv)
        th = math.acos(np.dot(src[0, 3:6].astype(np.float64), dv) / r)
        amp, ph, kk, al = (float(np.float32(v)) for v in (0.9, 1.1, 0.73, 0.002))
        e = amp * directivity_np(th) * math.exp(-al * r) / r * np.exp(1j * (ph + kk * r))
        # float64 oracle vs float64 numpy: equal up to the f32 directivity coefficients
        assert abs(p64[i] - e) <= 1e-6 * max(abs(e), 1e-30) + 1e-15
        if abs(math.degrees(th) % 10) > 1e-3:  # away from a bin edge
            # f32: the phase k r (~60 rad) carries ~4e-6 rad of rounding
            assert abs(p[i] - e) <= 2e-5 * (0.9 / r)


def test_coherent_focus_sums_magnitudes():
    """With the reference focal law every source arrives at the focus in phase (up to the f32
    rounding of k and lambda), so |p(focus)| equals the sum of the term magnitudes."""
    w = W.single_focus()
    cen = W.array_center(W.unit_array())
    focus = np.array([[cen[0], cen[1], 150.0]], np.float32)
    p = O.field_f32(1, w.sources, w.k, w.atten, focus)
    pos = w.sources[:, :3].astype(np.float64)
    d = focus[0].astype(np.float64) - pos
    r = np.linalg.norm(d, axis=1)
    th = np.arccos(d[:, 2] / r)
    mags = np.array([directivity_np(t) for t in th]) / r
    assert abs(p[0]) == pytest.approx(mags.sum(), rel=1e-4)


def test_focal_law_matches_numpy():
    pos = W.unit_array()
    src = W.t4010a1_records(pos, 1.0, 0.0)
    c = O.sound_speed(300.0)
    focus = (80.0, 60.0, 150.0)
    out = O.focal_point(1, src, c, focus).reshape(-1, 9)
    wl = c / 40e3
    d = np.linalg.norm(pos.astype(np.float64) - np.array(focus), axis=1)
    expect = -2 * math.pi * (np.fmod(d, wl) / wl)
    # away from the wrap point the f32 law agrees with float64 to rounding
    ok = np.abs(np.fmod(d, wl) / wl - 0.5) < 0.49
    np.testing.assert_allclose(out[ok, 7], expect[ok], atol=2e-5)


def test_grid_counts_truncate_in_f32():
    # builder.rs:150-152: ((max - min) / res) as usize + 1 in f32
    for lo, hi, res in [(0.0, 0.3, 0.1), (0.0, 1.0, 0.1), (-5.0, 5.0, 0.5), (10.0, 10.0, 1.0),
                        (36.36, 136.36, 1.0), (0.0, 127.75, 0.5)]:
        f = np.float32
        expect = int(np.trunc(f(f(hi) - f(lo)) / f(res))) + 1
        assert O.axis_count(lo, hi, res) == expect


def test_single_focus_grid_is_101_by_101():
    w = W.single_focus()
    lo, hi = w.grid.lo_hi()
    assert [O.axis_count(lo[i], hi[i], 1.0) for i in range(3)] == [101, 101, 1]


def test_large_grid_is_256_cubed():
    w = W.large_grid()
    lo, hi = w.grid.lo_hi()
    assert [O.axis_count(lo[i], hi[i], 0.5) for i in range(3)] == [256, 256, 256]
    assert w.n == 3984


@pytest.mark.parametrize("axes", [(1, 2, 3), (2, 1, 3), (3, 1, 2), (1, 3, 2), (2, 3, 1),
                                  (3, 2, 1)])
def test_grid_ordering_first_axis_fastest(axes):
    lo = np.array([1.0, 2.0, 3.0], np.float32)
    hi = np.array([3.0, 5.0, 7.0], np.float32)
    pts = O.grid_points(3, lo, hi, 1.0, axes)
    n = [3, 4, 5]
    order = [a - 1 for a in axes]
    assert len(pts) == 60
    idx = 0
    for i2 in range(n[order[2]]):
        for i1 in range(n[order[1]]):
            for i0 in range(n[order[0]]):
                e = lo.copy()
                e[order[0]] = lo[order[0]] + np.float32(i0) * np.float32(1.0)
                e[order[1]] = lo[order[1]] + np.float32(i1)
                e[order[2]] = lo[order[2]] + np.float32(i2)
                np.testing.assert_array_equal(pts[idx], e)
                idx += 1


def test_grid_2d_and_1d_fixed_axes():
    lo = np.array([1.0, 2.0, 9.0], np.float32)
    hi = np.array([3.0, 5.0, 9.0], np.float32)
    p2 = O.grid_points(2, lo, hi, 0.5, (2, 1, 3))  # y fastest, then x, z fixed
    assert len(p2) == 7 * 5
    assert np.all(p2[:, 2] == 9.0)
    np.testing.assert_array_equal(p2[:7, 1], np.float32(2.0) + np.arange(7, dtype=np.float32)
                                  * np.float32(0.5))
    assert np.all(p2[:7, 0] == 1.0) and p2[7, 0] == 1.5
    lo1 = np.array([1.0, 2.0, 9.0], np.float32)
    hi1 = np.array([1.0, 2.0, 12.0], np.float32)
    p1 = O.grid_points(1, lo1, hi1, 1.0, (3, 1, 2))
    np.testing.assert_array_equal(p1[:, 2], [9, 10, 11, 12])


def test_f32_oracle_within_tolerance_of_f64_on_single_focus():
    w = W.single_focus()
    lo, hi = w.grid.lo_hi()
    pts = O.grid_points(2, lo, hi, w.grid.res, w.grid.axes)
    p32 = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_COMPLEX)
    p64 = O.field_f64(1, w.sources, w.k, w.atten, pts)
    err = np.max(np.abs(p32 - p64)) / np.max(np.abs(p64))
    assert err < 1e-5


def test_libm_and_correctly_rounded_acos_differ_only_at_bin_edges():
    """glibc's acosf is not correctly rounded.  The two oracle modes may differ only where a
    pair's theta lies within an ulp of a directivity bin edge; everywhere else they agree
    exactly."""
    rng = np.random.default_rng(10)
    n = 50
    pos = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
    pos[:, 2] = rng.uniform(-5, 5, n)
    rec = W.t4010a1_records(pos, rng.uniform(0.2, 1, n), rng.uniform(-3, 3, n))
    d = rng.normal(size=(n, 3)) * np.array([0.3, 0.3, 0.0]) + np.array([0, 0, 1.0])
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    k = np.full(n, 0.72, np.float32)
    a = np.full(n, 0.005, np.float32)
    lo = np.array([-20, -10, 60], np.float32)
    hi = np.array([25, 30, 95], np.float32)
    pts = O.grid_points(3, lo, hi, 1.5, (1, 2, 3))
    p_libm = O.field_f32(1, rec, k, a, pts)
    with O.acos_mode(O.ACOS_CORRECTLY_ROUNDED):
        p_cr = O.field_f32(1, rec, k, a, pts)
    # a one-ulp theta changes D by ~1e-7 (invisible at this scale); a bin flip by up to 0.164
    diff = np.nonzero(np.abs(p_libm - p_cr) > 1e-5 * np.max(np.abs(p_cr)))[0]
    # the points that differ visibly: some pair's theta within 2 ulp of a 10-degree edge
    div = np.float32(np.float32(math.pi) / np.float32(18))
    for i in diff:
        dv = (pts[i] - rec[:, :3]).astype(np.float64)
        th = np.arccos(np.sum(dv * rec[:, 3:6], axis=1) / np.linalg.norm(dv, axis=1))
        q = th / float(div)
        assert np.min(np.abs(q - np.round(q))) < 4e-6
    assert len(diff) < 0.01 * len(pts)


def test_accurate_oracle_close_to_plain():
    w = W.single_focus()
    rng = np.random.default_rng(3)
    pts = rng.uniform([36, 16, 100], [136, 116, 200], (500, 3)).astype(np.float32)
    p = O.field_f32(1, w.sources, w.k, w.atten, pts)
    pa = O.field_f32(1, w.sources, w.k, w.atten, pts, accurate=True)
    p64 = O.field_f64(1, w.sources, w.k, w.atten, pts)
    peak = np.max(np.abs(p64))
    assert np.max(np.abs(pa - p64)) / peak < 1e-5
    assert np.max(np.abs(p - p64)) / peak < 1e-5


def test_gspat_oracle_reaches_targets():
    rng = np.random.default_rng(5)
    w, foci, amps = W.gspat_request(rng, 8, tiles=(1, 1))
    src, q = O.gspat_f64(1, w.sources, w.k, w.atten, foci, amps)
    src = src.reshape(-1, 9)
    assert np.all(np.isfinite(src[:, 6:8]))
    np.testing.assert_allclose(src[:, 6], np.abs(q), rtol=1e-6)
    p = O.field_f64(1, src, w.k, w.atten, foci)
    ratio = np.abs(p) / amps
    assert ratio.std() / ratio.mean() < 0.05


def test_gs_and_naive_oracles_run():
    rng = np.random.default_rng(6)
    w, foci, amps = W.gspat_request(rng, 4, tiles=(1, 1))
    for fn in (O.gs_f64, O.naive_f64):
        src, q = fn(1, w.sources, w.k, w.atten, foci, amps) if fn is O.naive_f64 else fn(
            1, w.sources, w.k, w.atten, foci, amps)
        assert np.all(np.isfinite(q))


def test_gspat_f32_restatement_tracks_f64():
    """The f32 GS-PAT restatement (the reference's own arithmetic) stays within 1e-4 of the
    float64 one on well-separated foci, reaches the same focal amplitudes, and leaves
    positions, directions and frequencies untouched."""
    rng = np.random.default_rng(5)
    w, foci, amps = W.gspat_request(rng, 6)
    s32, q32 = O.gspat_f32(1, w.sources, w.k, w.atten, foci, amps)
    s64, q64 = O.gspat_f64(1, w.sources, w.k, w.atten, foci, amps)
    s32, s64 = s32.reshape(-1, 9), s64.reshape(-1, 9)
    assert np.max(np.abs(q32 - q64)) <= 1e-4 * np.max(np.abs(q64))
    np.testing.assert_allclose(s32[:, 6], np.abs(q32), rtol=1e-6)
    p32 = np.abs(O.field_f64(1, s32, w.k, w.atten, foci))
    p64 = np.abs(O.field_f64(1, s64, w.k, w.atten, foci))
    assert np.max(np.abs(p32 - p64)) <= 1e-4 * np.max(p64)
    np.testing.assert_array_equal(s32[:, [0, 1, 2, 3, 4, 5, 8]], w.sources[:, [0, 1, 2, 3, 4, 5, 8]])


def _focus_points(seed, m=400):
    rng = np.random.default_rng(seed)
    cen = W.array_center(W.unit_array())
    pts = np.empty((m, 3), np.float32)
    pts[:, 0] = rng.uniform(cen[0] - 60, cen[0] + 60, m)
    pts[:, 1] = rng.uniform(cen[1] - 60, cen[1] + 60, m)
    pts[:, 2] = rng.uniform(60, 220, m)
    return pts


def test_doubling_every_amplitude_doubles_the_field_exactly():
    """uniform_medium.rs:111-128 weights each term by its source's amplitude and sums the terms:
    scaling every amplitude by two scales every f32 product and partial sum by two exactly (no
    overflow or subnormal here), so the field doubles bit for bit."""
    w = W.single_focus()
    pts = _focus_points(3)
    p1 = O.field_f32(1, w.sources, w.k, w.atten, pts)
    s2 = w.sources.copy()
    s2[:, 6] *= 2.0
    p2 = O.field_f32(1, s2, w.k, w.atten, pts)
    np.testing.assert_array_equal(p2.view(np.float32), (2 * p1).view(np.float32))


def test_field_types_are_the_complex_sum_transformed():
    """field_buffer/{power,pressure}_field.rs:35-37: the power field is re*re + im*im of the
    complex sum (f32, each operation rounded), the pressure field its square root, so both follow
    bit for bit from the complex field."""
    w = W.single_focus()
    pts = _focus_points(4)
    pc = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_COMPLEX)
    pw = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_POWER)
    pr = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_PRESSURE)
    re = np.ascontiguousarray(pc.real, dtype=np.float32)
    im = np.ascontiguousarray(pc.imag, dtype=np.float32)
    ns = (re * re) + (im * im)  # float32 products and sum, each rounded
    assert ns.dtype == np.float32
    np.testing.assert_array_equal(pw, ns)
    np.testing.assert_array_equal(pr, np.sqrt(ns))


def test_superposition_of_two_source_sets():
    """The field is a sum over sources (uniform_medium.rs:122-128): the field of two source sets
    together equals the sum of their fields, up to the float association of the sum."""
    w = W.single_focus()
    pts = _focus_points(5)
    half = w.n // 2
    a = O.field_f32(1, w.sources[:half], w.k[:half], w.atten[:half], pts)
    b = O.field_f32(1, w.sources[half:], w.k[half:], w.atten[half:], pts)
    ab = O.field_f32(1, w.sources, w.k, w.atten, pts)
    peak = float(np.max(np.abs(ab)))
    assert float(np.max(np.abs(ab - (a + b)))) <= 2e-6 * peak
