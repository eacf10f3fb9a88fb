"""Python side of the serving engine (AFC_Serve* of include/afc_gpu.h): keeps each request's
host buffers alive from submission until its result has been waited for."""
from __future__ import annotations

import ctypes

import numpy as np

import workloads as W


class Engine:
    def __init__(self, afc, hbm_budget_bytes: int, pinned_bytes: int, max_inflight: int):
        from afc import nativemethods as nm

        self.afc = afc
        self.lib = afc.DLL
        self.nm = nm
        cfg = nm.ServeConfig(hbm_budget_bytes, pinned_bytes, max_inflight)
        self.h = ctypes.c_void_p()
        if self.lib.AFC_ServeCreate(ctypes.byref(cfg), ctypes.byref(self.h)) != 0:
            raise RuntimeError(afc.last_error())
        self.live = {}

    def add_geometry(self, st, sources, k, atten) -> int:
        gid = ctypes.c_int32()
        src = np.ascontiguousarray(sources, np.float32)
        k = np.ascontiguousarray(k, np.float32)
        atten = np.ascontiguousarray(atten, np.float32)
        rc = self.lib.AFC_ServeAddGeometry(self.h, st, src.ctypes.data, k.ctypes.data,
                                           atten.ctypes.data, len(k), ctypes.byref(gid))
        if rc != 0:
            raise RuntimeError(self.afc.last_error())
        return gid.value

    def submit_field(self, gid, amps, phases, field_type, grid=None, points=None):
        """grid: an AfcGridDesc; points: (m, 3) float32.  Returns (request id, output array)."""
        amps = np.ascontiguousarray(amps, np.float32)
        phases = np.ascontiguousarray(phases, np.float32)
        if grid is not None:
            m = int(grid.count[0] * grid.count[1] * grid.count[2])
            pts_ptr, n_pts = None, 0
        else:
            points = np.ascontiguousarray(points, np.float32)
            m = len(points)
            pts_ptr, n_pts = points.ctypes.data, m
        out = np.empty(m * (2 if field_type == 2 else 1), np.float32)
        rid = self.lib.AFC_ServeSubmitField(self.h, gid, amps.ctypes.data, phases.ctypes.data,
                                            field_type, 1 if grid is not None else 0,
                                            ctypes.byref(grid) if grid is not None else None,
                                            pts_ptr, n_pts, out.ctypes.data)
        if rid < 0:
            raise RuntimeError(self.afc.last_error())
        self.live[rid] = out
        return rid, out

    def submit_gspat(self, gid, n_sources, foci, amps, slice_desc):
        foci = np.ascontiguousarray(foci, np.float32)
        amps = np.ascontiguousarray(amps, np.float32)
        m = int(slice_desc.count[0] * slice_desc.count[1] * slice_desc.count[2])
        out = np.empty(m, np.float32)
        ap = np.empty(2 * n_sources, np.float32)
        rid = self.lib.AFC_ServeSubmitGspat(self.h, gid, foci.ctypes.data, amps.ctypes.data,
                                            len(amps), ctypes.byref(slice_desc), out.ctypes.data,
                                            ap.ctypes.data)
        if rid < 0:
            raise RuntimeError(self.afc.last_error())
        self.live[rid] = (out, ap)
        return rid, out, ap

    def wait(self, rid):
        lat = ctypes.c_double()
        q = ctypes.c_double()
        rc = self.lib.AFC_ServeWait(self.h, rid, ctypes.byref(lat), ctypes.byref(q))
        self.live.pop(rid, None)
        if rc != 0:
            raise RuntimeError(self.afc.last_error())
        return lat.value, q.value

    def stats(self):
        s = self.nm.ServeStats()
        self.lib.AFC_ServeStats(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if self.h:
            self.lib.AFC_ServeDestroy(self.h)
            self.h = ctypes.c_void_p()


def slice_desc(afc, center_xy, z, half=100.0, res=1.0):
    """A (2 half / res + 1)^2 XY grid slice at depth z centred on center_xy (a half step of
    padding makes the f32 point count exact)."""
    cx, cy = float(center_xy[0]), float(center_xy[1])
    spec = W.GridSpec(2, [(cx - half, cx + half + 0.5 * res), (cy - half, cy + half + 0.5 * res),
                          (z, z)], res, (W.AXIS_X, W.AXIS_Y, W.AXIS_Z))
    area = afc.grid_from_spec(spec)
    return area.grid_desc(), spec
