"""Gradient descent, Gauss-Newton and Levenberg-Marquardt phase retrieval on the device
(AFO_GradientDescent, AFO_GaussNewton, AFO_LM; multiple_foci/nls/*.rs) against the oracle's
float64 restatement with the reference's dense N x N formulas.  The device evaluates the same
quantities through the low-rank structure of B = [G | -diag(amps)] in float32, so the two runs
follow the same iteration up to rounding; the NLS objective does not change under a common
phase shift of all parameters, so the compared quantity is the achieved focal amplitude |p(f_j)|
(float64 field of the resulting drive)."""
import time

import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

KINDS = {O.NLS_GRADIENT_DESCENT: "gradient_descent", O.NLS_GAUSS_NEWTON: "gauss_newton",
         O.NLS_LM: "lm"}


def _problem(seed, n, m):
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
    amps = rng.uniform(0.5, 1.0, m).astype(np.float32)
    return rec, k, a, foci, amps


@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("n,m", [(48, 3), (96, 6)])
def test_nls_matches_dense_f64(gpu, kind, n, m):
    afc = gpu
    rec, k, a, foci, amps = _problem(10 * n + m + kind, n, m)
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    t0 = time.perf_counter()
    getattr(afc.Optimizer, KINDS[kind])(s, foci, amps)
    t_gpu = time.perf_counter() - t0
    got = s.records().copy()
    t0 = time.perf_counter()
    ref = O.nls_f64(kind, 1, rec, k, a, foci, amps).reshape(-1, 9)
    t_ref = time.perf_counter() - t0
    np.testing.assert_array_equal(got[:, 6], rec[:, 6])
    p_gpu = np.abs(O.field_f64(1, got, k, a, foci))
    p_ref = np.abs(O.field_f64(1, ref, k, a, foci))
    err = float(np.max(np.abs(p_gpu - p_ref)) / np.max(p_ref))
    print(f"{KINDS[kind]} n={n} m={m}: |p| gpu {np.round(p_gpu, 4)} oracle {np.round(p_ref, 4)} "
          f"rel {err:.2e}; {t_gpu * 1e3:.1f} ms vs dense f64 {t_ref * 1e3:.1f} ms")
    assert np.all(np.isfinite(got[:, 7]))
    # gradient descent and LM follow the dense iteration to float32 rounding; Gauss-Newton's
    # pseudo-inverse drops eigenvalues below 1e-3, a cut that float32 and float64 place a little
    # differently
    assert err <= {O.NLS_GRADIENT_DESCENT: 1e-4, O.NLS_LM: 1e-2, O.NLS_GAUSS_NEWTON: 5e-2}[kind]


def test_nls_large_array_runs(gpu):
    """996 transducers and 16 foci (N = 1,012 parameters): every solver finishes, improves the
    objective over the zero drive and reports its time (the dense formulation would solve
    1,012 x 1,012 systems every step)."""
    afc = gpu
    rng = np.random.default_rng(17)
    w, foci, amps = W.gspat_request(rng, 16)
    for kind, name in KINDS.items():
        s = afc.UniformSystem(300.0)
        s.add_records(1, w.sources, w.k, w.atten)
        t0 = time.perf_counter()
        getattr(afc.Optimizer, name)(s, foci, amps)
        dt = time.perf_counter() - t0
        p = np.abs(O.field_f64(1, s.records(), w.k, w.atten, foci))
        p0 = np.abs(O.field_f64(1, w.sources, w.k, w.atten, foci))
        print(f"{name} n=996 m=16: {dt * 1e3:.1f} ms, |p|/amp {np.round(p / amps, 3)}")
        assert np.all(np.isfinite(p))
        assert np.sum((p / np.max(p) - amps / np.max(amps)) ** 2) < np.sum(
            (p0 / np.max(p0) - amps / np.max(amps)) ** 2)


def test_nls_edge_cases(gpu):
    afc = gpu
    rec, k, a, foci, amps = _problem(3, 40, 2)
    for name in KINDS.values():
        s = afc.UniformSystem(300.0)
        s.add_records(1, rec, k, a)
        getattr(afc.Optimizer, name)(s, np.zeros((0, 3), np.float32), np.zeros(0, np.float32))
        assert np.all(s.records()[:, 7] == 0.0)  # no foci: the gradient is 0 at x = 0
    s = afc.UniformSystem(300.0)
    s.add_records(1, rec, k, a)
    before = s.records().copy()
    big = np.zeros((300, 3), np.float32)
    big[:, 2] = 100.0
    with pytest.raises(RuntimeError, match="too many foci"):
        afc.Optimizer.lm(s, big, np.ones(300, np.float32))
    np.testing.assert_array_equal(s.records(), before)


@pytest.mark.parametrize("kind", sorted(KINDS))
def test_nls_sphere_sources(gpu, kind):
    """The three NLS solvers on sphere sources (source type 0, D = 1), 48 sources, 3 foci, with
    the same comparison and bars as the T4010A1 cases."""
    afc = gpu
    rec9, k, a, foci, amps = _problem(700 + kind, 48, 3)
    rec = W.sphere_records(rec9[:, :3], rec9[:, 6], rec9[:, 7])
    s = afc.UniformSystem(300.0)
    s.add_records(0, rec, k, a)
    getattr(afc.Optimizer, KINDS[kind])(s, foci, amps)
    got = s.records().copy()
    ref = O.nls_f64(kind, 0, rec, k, a, foci, amps).reshape(-1, 6)
    np.testing.assert_array_equal(got[:, 3], rec[:, 3])
    p_gpu = np.abs(O.field_f64(0, got, k, a, foci))
    p_ref = np.abs(O.field_f64(0, ref, k, a, foci))
    err = float(np.max(np.abs(p_gpu - p_ref)) / np.max(p_ref))
    print(f"{KINDS[kind]} sphere: rel {err:.2e}")
    assert np.all(np.isfinite(got[:, 4]))
    assert err <= {O.NLS_GRADIENT_DESCENT: 1e-4, O.NLS_LM: 1e-2, O.NLS_GAUSS_NEWTON: 5e-2}[kind]
