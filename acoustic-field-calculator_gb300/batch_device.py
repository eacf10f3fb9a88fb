"""Device buffers for a list of workloads.BatchJob and the AfcFieldJob array that
AFC_BatchCreate takes.  PyTorch only provides the device memory here."""
from __future__ import annotations

import ctypes


def materialize(afc, torch, jobs, device="cuda"):
    """Returns (AfcFieldJob array, [output tensor per job], [points tensor or None per job],
    keep-alive list).  Scatter points are drawn on the device from each job's seed."""
    from afc import nativemethods as nm

    arr = (nm.FieldJob * len(jobs))()
    outs, pts_list, keep = [], [], []
    for i, jb in enumerate(jobs):
        src = torch.from_numpy(jb.sources.reshape(-1)).to(device)
        k = torch.from_numpy(jb.k).to(device)
        a = torch.from_numpy(jb.atten).to(device)
        keep += [src, k, a]
        f = arr[i]
        f.n_sources = jb.n
        f.d_sources, f.d_wavenums, f.d_attens = src.data_ptr(), k.data_ptr(), a.data_ptr()
        f.field_type = jb.field_type
        if jb.grid is not None:
            area = afc.grid_from_spec(jb.grid)
            f.is_grid = 1
            f.grid = area.grid_desc()
            m = int(f.grid.count[0] * f.grid.count[1] * f.grid.count[2])
            pts_list.append(None)
        else:
            gen = torch.Generator(device=device)
            gen.manual_seed(jb.points_seed)
            lo = torch.tensor(jb.box_lo, dtype=torch.float32, device=device)
            hi = torch.tensor(jb.box_hi, dtype=torch.float32, device=device)
            pts = lo + (hi - lo) * torch.rand((jb.n_points, 3), generator=gen, device=device)
            pts = pts.contiguous()
            keep.append(pts)
            pts_list.append(pts)
            f.is_grid = 0
            f.d_points = pts.data_ptr()
            f.n_points = jb.n_points
            m = jb.n_points
        out = torch.empty(m * (2 if jb.field_type == 2 else 1), dtype=torch.float32,
                          device=device)
        f.d_out = out.data_ptr()
        outs.append(out)
    return arr, outs, pts_list, keep


def create_plan(afc, arr, tune: bool, stream):
    plan = ctypes.c_void_p()
    rc = afc.DLL.AFC_BatchCreate(1, arr, len(arr), 1 if tune else 0, ctypes.byref(plan), stream)
    if rc != 0:
        raise RuntimeError(afc.last_error())
    return plan


def describe(afc, plan):
    pairs = ctypes.c_int32()
    bps = ctypes.c_int32()
    items = ctypes.c_uint64()
    evals = ctypes.c_double()
    afc.DLL.AFC_BatchDescribe(plan, ctypes.byref(pairs), ctypes.byref(bps), ctypes.byref(items),
                              ctypes.byref(evals))
    rp, rb, ri = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
    fp, fb, fi = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
    afc.DLL.AFC_BatchDescribeKernels(plan, ctypes.byref(rp), ctypes.byref(rb), ctypes.byref(ri),
                                     ctypes.byref(fp), ctypes.byref(fb), ctypes.byref(fi))
    return {"pairs_per_thread": pairs.value, "blocks_per_sm": bps.value, "items": items.value,
            "evals": evals.value,
            "rows_kernel": {"pairs_per_thread": rp.value, "blocks_per_sm": rb.value,
                            "items": ri.value},
            "flat_kernel": {"pairs_per_thread": fp.value, "blocks_per_sm": fb.value,
                            "items": fi.value}}
