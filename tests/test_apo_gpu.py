"""Acoustic power optimization on the device (AFO_APO; multiple_foci/nls/apo.rs) against the
oracle's float64 restatement with the reference's explicit n x n matrices R_i, dense q0 solve
and dense quasi-Newton matrix.  The device uses R_i's rank-one structure (q^H R_i q = |(G q)_i|^2,
R_i q = G^H e_i (G q)_i), solves q0 through the m x m system (G G^H + lambda I) and keeps H dense.
The line search picks the first minimum of J over a = 0, 0.01, .., 0.99, so once a
step is taken a float32 run can pick a different a than a float64 one; the device carries the
iteration in float64 (G in float32), and the compared quantity is the achieved focal amplitude
|p(f_j)| (float64 field of the resulting drive) relative to its peak."""
import time

import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu


def _grid_array(nx, ny, pitch=10.16):
    """nx x ny transducers on a plain grid (the reference's examples use 18 x 14)."""
    y, x = np.mgrid[0:ny, 0:nx]
    return np.stack([x.ravel() * pitch, y.ravel() * pitch, np.zeros(nx * ny)], 1).astype(np.float32)


def _run(afc, rec, k, a, foci, amps, lam):
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    t0 = time.perf_counter()
    afc.Optimizer.apo(s, foci, amps, lam)
    dt = time.perf_counter() - t0
    return s.records().copy(), dt


def _compare(afc, rec, k, a, foci, amps, lam, label):
    got, t_gpu = _run(afc, rec, k, a, foci, amps, lam)
    t0 = time.perf_counter()
    ref = O.apo_f64(1, rec, k, a, foci, amps, lam).reshape(-1, 9)
    t_ref = time.perf_counter() - t0
    assert np.all(np.isfinite(got[:, 6])) and np.all(np.isfinite(got[:, 7]))
    # amp |q| / camax(q) with camax the largest |re| + |im|: every amplitude lies in (0, amp]
    assert np.all(got[:, 6] <= rec[:, 6] * (1 + 1e-6)) and np.all(got[:, 6] >= 0)
    p_gpu = np.abs(O.field_f64(1, got, k, a, foci))
    p_ref = np.abs(O.field_f64(1, ref, k, a, foci))
    err = float(np.max(np.abs(p_gpu - p_ref)) / np.max(p_ref))
    print(f"APO {label}: |p| gpu {np.round(p_gpu, 5)} oracle {np.round(p_ref, 5)} rel {err:.2e}; "
          f"{t_gpu * 1e3:.1f} ms vs dense f64 {t_ref * 1e3:.1f} ms")
    return err


def test_apo_reference_example(gpu):
    """The reference's foci example: 18 x 14 transducers, two foci 50 mm either side of the
    array's axis at 150 mm, amplitudes 1 and lambda 2."""
    afc = gpu
    pos = _grid_array(18, 14)
    n = len(pos)
    rec = W.t4010a1_records(pos, 1.0, 0.0)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.zeros(n, np.float32)
    c = W.array_center(pos)
    foci = np.array([[c[0] + 50, c[1], 150], [c[0] - 50, c[1], 150]], np.float32)
    amps = np.ones(2, np.float32)
    # the float32 transfer matrix alone moves the float64 iteration's result by 1.5e-4
    assert _compare(afc, rec, k, a, foci, amps, 2.0, "18x14, 2 foci, lambda 2") <= 1e-3


@pytest.mark.parametrize("n,m,scale,lam,seed", [
    (64, 3, 1.0, 1e-2, 1), (64, 3, 0.05, 1e-4, 2), (96, 4, 0.02, 1e-6, 3), (128, 6, 0.5, 1e-3, 4)])
def test_apo_matches_dense_f64(gpu, n, m, scale, lam, seed):
    afc = gpu
    rng = np.random.default_rng(seed)
    pos = W.tiled_array(1, 1)[:n]
    rec = W.t4010a1_records(pos, rng.uniform(0.6, 1.0, n).astype(np.float32), 0.0)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.full(n, 1.15e-2, np.float32)
    c = W.array_center(pos)
    foci = np.empty((m, 3), np.float32)
    foci[:, 0] = rng.uniform(c[0] - 25, c[0] + 25, m)
    foci[:, 1] = rng.uniform(c[1] - 25, c[1] + 25, m)
    foci[:, 2] = rng.uniform(100, 160, m)
    amps = (scale * rng.uniform(0.5, 1.0, m)).astype(np.float32)
    assert _compare(afc, rec, k, a, foci, amps, lam, f"n={n} m={m} lambda={lam}") <= 1e-4


@pytest.mark.parametrize("seed", [0, 9])
def test_apo_long_trajectory(gpu, seed):
    """12 transducers, two near foci: seed 9 takes 63 quasi-Newton steps, seed 0 four; the
    device's float64 state follows the oracle's iteration all the way."""
    afc = gpu
    rng = np.random.default_rng(seed)
    n, m = 12, 2
    pos = W.tiled_array(1, 1)[:n]
    rec = W.t4010a1_records(pos, 1.0, 0.0)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.zeros(n, np.float32)
    foci = np.array([[pos[:, 0].mean() + rng.uniform(-10, 10), pos[:, 1].mean(),
                      rng.uniform(30, 80)] for _ in range(m)], np.float32)
    amps = rng.uniform(0.01, 0.2, m).astype(np.float32)
    lam = float(10 ** rng.uniform(-6, -1))
    assert _compare(afc, rec, k, a, foci, amps, lam, f"n=12 seed {seed}") <= 1e-4


def test_apo_large_array_runs(gpu):
    """996 transducers and 16 foci: the dense reference would hold 16 matrices of 996 x 996 and
    solve a 996 x 996 system; the device run finishes and reports its time."""
    afc = gpu
    rng = np.random.default_rng(5)
    w, foci, amps = W.gspat_request(rng, 16)
    s = afc.UniformSystem(300.0)
    s.add_records(1, w.sources, w.k, w.atten)
    t0 = time.perf_counter()
    afc.Optimizer.apo(s, foci, amps * np.float32(0.05), 1e-3)
    dt = time.perf_counter() - t0
    got = s.records()
    p = np.abs(O.field_f64(1, got, w.k, w.atten, foci))
    print(f"APO n=996 m=16: {dt * 1e3:.1f} ms, |p|/max {np.round(p / p.max(), 3)}")
    assert np.all(np.isfinite(got[:, 6:8]))
    assert np.max(got[:, 6]) <= 1.0 + 1e-6


def test_apo_edge_cases(gpu):
    afc = gpu
    pos = W.tiled_array(1, 1)[:40]
    rec = W.t4010a1_records(pos, 1.0, 0.3)
    k = np.full(40, W.wavenumber(), np.float32)
    a = np.zeros(40, np.float32)
    # no foci: q = 0, so amp |q| / camax(q) is 0 / 0 as in the reference, and every phase 0
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    afc.Optimizer.apo(s, np.zeros((0, 3), np.float32), np.zeros(0, np.float32), 1.0)
    assert np.all(np.isnan(s.records()[:, 6])) and np.all(s.records()[:, 7] == 0.0)
    ref = O.apo_f64(1, rec, k, a, np.zeros((0, 3), np.float32), np.zeros(0, np.float32), 1.0)
    assert np.all(np.isnan(ref.reshape(-1, 9)[:, 6]))
    # too many foci: an error, the records untouched
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    before = s.records().copy()
    big = np.zeros((300, 3), np.float32)
    big[:, 2] = 100.0
    with pytest.raises(RuntimeError, match="too many foci"):
        afc.Optimizer.apo(s, big, np.ones(300, np.float32), 1.0)
    np.testing.assert_array_equal(s.records(), before)


def test_apo_sphere_sources(gpu):
    """APO on sphere sources (source type 0, D = 1): 64 sources, 3 foci, lambda 1e-2.  This
    problem takes 81 quasi-Newton steps, and over them the float32 transfer matrix alone moves
    the float64 iteration's focal amplitudes by 1.6e-4 (the oracle's own iteration run from its
    f32 and its f64 G), so the bar is the reference example's 1e-3."""
    afc = gpu
    rng = np.random.default_rng(31)
    n, m, lam = 64, 3, 1e-2
    pos = W.tiled_array(1, 1)[:n]
    rec = W.sphere_records(pos, rng.uniform(0.6, 1.0, n).astype(np.float32), 0.0)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.full(n, 1.15e-2, np.float32)
    c = W.array_center(pos)
    foci = np.stack([rng.uniform(c[0] - 25, c[0] + 25, m), rng.uniform(c[1] - 25, c[1] + 25, m),
                     rng.uniform(100, 160, m)], 1).astype(np.float32)
    amps = rng.uniform(0.5, 1.0, m).astype(np.float32)
    s = afc.UniformSystem(300.0)
    s.add_records(0, rec, k, a)
    afc.Optimizer.apo(s, foci, amps, lam)
    got = s.records().copy()
    ref = O.apo_f64(0, rec, k, a, foci, amps, lam).reshape(-1, 6)
    assert np.all(np.isfinite(got[:, 3])) and np.all(np.isfinite(got[:, 4]))
    p_gpu = np.abs(O.field_f64(0, got, k, a, foci))
    p_ref = np.abs(O.field_f64(0, ref, k, a, foci))
    err = float(np.max(np.abs(p_gpu - p_ref)) / np.max(p_ref))
    print(f"APO sphere: rel {err:.2e}")
    assert err <= 1e-3
