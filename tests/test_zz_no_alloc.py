"""AFC_FieldGridDeviceNoAlloc: the field entry point for callers that cannot allocate GPU
memory while they run (a real-time array-control loop, a host that owns all device memory,
a plugin barred from allocating in callbacks).  It must give the same field as
AFC_FieldGridDevice -- which takes a caller-allocated workspace -- on consecutive calls, since
its fixed scratch array is reused and keeps the previous call's contents.

This file is named to be collected last, so a run that stops at its first failure has run
every other test before it.  It also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-4  # max |difference| <= TOL * max |reference field|, the bar of the other GPU tests


def _setup(afc, torch, n_tiles, seed, count):
    w = W.large_grid(seed=seed, count=count, tiles=n_tiles)
    area = afc.grid_from_spec(w.grid)
    desc = area.grid_desc()
    m = int(desc.count[0] * desc.count[1] * desc.count[2])
    d_src = torch.from_numpy(w.sources.reshape(-1)).cuda()
    d_k = torch.from_numpy(w.k).cuda()
    d_a = torch.from_numpy(w.atten).cuda()
    return w, area, desc, m, d_src, d_k, d_a


def _with_workspace(afc, torch, w, desc, m, d_src, d_k, d_a, stream):
    ws_bytes = afc.DLL.AFC_FieldWorkspaceBytes(w.n)
    ws = torch.empty(max(ws_bytes, 256), dtype=torch.uint8, device="cuda")
    out = torch.empty(2 * m, dtype=torch.float32, device="cuda")
    rc = afc.DLL.AFC_FieldGridDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                     w.n, ctypes.byref(desc), out.data_ptr(), ws.data_ptr(),
                                     ws_bytes, stream)
    assert rc == 0, afc.last_error()
    return out


def _no_alloc(afc, w, desc, out, d_src, d_k, d_a, stream):
    return afc.DLL.AFC_FieldGridDeviceNoAlloc(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(),
                                              d_a.data_ptr(), w.n, ctypes.byref(desc),
                                              out.data_ptr(), stream)


def _oracle_sample(w, rows):
    """The oracle's field (the reference CPU calculator restated) at grid points `rows`."""
    lo, hi = w.grid.lo_hi()
    pts = O.grid_points(3, lo, hi, w.grid.res, w.grid.axes)[rows]
    return O.field_f32(1, w.sources, w.k, w.atten, pts)


def test_no_alloc_matches_workspace_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    afc = gpu
    stream = torch.cuda.current_stream().cuda_stream
    # two different systems in a row: the second call must not see the first one's scratch
    for tiles, seed in (((4, 4), 11), ((2, 2), 12)):
        w, area, desc, m, d_src, d_k, d_a = _setup(afc, torch, tiles, seed, 48)
        ref = _with_workspace(afc, torch, w, desc, m, d_src, d_k, d_a, stream)
        rows = np.sort(np.random.default_rng(seed).choice(m, 2000, replace=False))
        want = _oracle_sample(w, rows)
        for _ in range(2):
            out = torch.full((2 * m,), float("nan"), dtype=torch.float32, device="cuda")
            rc = _no_alloc(afc, w, desc, out, d_src, d_k, d_a, stream)
            assert rc == 0, afc.last_error()
            torch.cuda.synchronize()
            a = out.cpu().numpy().view(np.complex64)
            b = ref.cpu().numpy().view(np.complex64)
            assert np.all(np.isfinite(a))
            assert np.max(np.abs(a - b)) <= TOL * np.max(np.abs(b))
            # and against the oracle itself, so that a fault shared by both entry points shows
            assert np.max(np.abs(a[rows] - want)) <= TOL * np.max(np.abs(want))


def test_no_alloc_rejects_more_sources_than_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    afc = gpu
    w, area, desc, m, d_src, d_k, d_a = _setup(afc, torch, (1, 1), 13, 8)
    out = torch.zeros(2 * m, dtype=torch.float32, device="cuda")
    too_many = 16384 + 1
    rc = afc.DLL.AFC_FieldGridDeviceNoAlloc(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(),
                                            d_a.data_ptr(), too_many, ctypes.byref(desc),
                                            out.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)
    assert rc == -4  # AFC_ERR_TOO_LARGE
    assert "16384" in afc.last_error()
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0  # nothing was launched
