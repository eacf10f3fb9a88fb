"""Host side of the serving workload: the seeded Poisson stream and the GS-PAT slice."""
import numpy as np

import serving_client as SC
import workloads as W


def test_stream_is_seeded_poisson_with_the_stated_mix():
    s = W.serving_stream(1000.0, 4000, 256, seed=5)
    t = np.array([r.arrival for r in s])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1e-3) < 0.1e-3  # rate 1000/s
    assert abs(np.std(gaps) / gaps.mean() - 1.0) < 0.1  # exponential: cv = 1
    field = [r for r in s if r.kind == "field"]
    gspat = [r for r in s if r.kind == "gspat"]
    assert abs(len(field) / len(s) - 0.7) < 0.03
    assert all(0 <= r.job < 256 for r in field)
    ms = np.array([len(r.amps) for r in gspat])
    assert ms.min() == 2 and ms.max() == 64
    cen = W.array_center(W.tiled_array(2, 2))
    f = np.concatenate([r.foci for r in gspat])
    assert np.all(np.abs(f[:, :2] - cen[:2]) <= 50.0)
    assert f[:, 2].min() >= 100.0 and f[:, 2].max() <= 200.0
    a = np.concatenate([r.amps for r in gspat])
    assert a.min() >= 0.5 and a.max() <= 1.0
    s2 = W.serving_stream(1000.0, 4000, 256, seed=5)
    assert [r.arrival for r in s2] == [r.arrival for r in s]


def test_scatter_points_of_a_job_are_seeded_and_in_its_box():
    jobs = W.batch_jobs(n_jobs=8)
    jb = next(j for j in jobs if j.grid is None)
    p = W.batch_job_points(jb)
    assert p.shape == (jb.n_points, 3) and p.dtype == np.float32
    assert np.all(p >= np.asarray(jb.box_lo, np.float32))
    assert np.all(p <= np.asarray(jb.box_hi, np.float32))
    np.testing.assert_array_equal(p, W.batch_job_points(jb))


def test_gspat_slice_is_201_by_201(afc_mod):
    cen = W.array_center(W.tiled_array(2, 2))
    desc, spec = SC.slice_desc(afc_mod, cen, 150.0, half=100.0, res=1.0)
    counts = sorted(int(c) for c in desc.count)
    assert counts == [1, 201, 201]
    assert desc.res == 1.0
