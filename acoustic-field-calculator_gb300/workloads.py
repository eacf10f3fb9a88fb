"""Seeded synthetic workloads of the acoustic-field path.

All inputs are generated here from a seed: there is no dataset.  Geometry follows the
reference examples (acoustic-field-calculator/examples/main.rs:17-21, 59-131): an 18 x 14
array of T4010A1 transducers in the z = 0 plane facing +z, here at a 10.16 mm pitch with
three holes, 40 kHz, c = 340 m/s.  Units are millimetres, as in the reference.

Source records use the reference's C-ABI layout (capi/src/system.rs:123-129):
T4010A1 = 9 float32 {x, y, z, nx, ny, nz, amp, phase, freq} (t4010a1.rs:76-82) and
SphereWaveSource = 6 float32 {x, y, z, amp, phase, freq} (sphere_sources.rs:22-27).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

PITCH = 10.16
NUM_X, NUM_Y = 18, 14
HOLES = ((1, 1), (2, 1), (16, 1))  # (x, y) indices left empty in the unit array
FREQ = 40e3
SOUND_SPEED = 340e3  # mm/s
AXIS_X, AXIS_Y, AXIS_Z = 1, 2, 3  # observe_area/grid/dimension.rs:23-39


def unit_array(pitch: float = PITCH) -> np.ndarray:
    """Positions (249 x 3, float32) of one 18 x 14 unit with its three holes."""
    pos = [
        (pitch * x, pitch * y, 0.0)
        for y in range(NUM_Y)
        for x in range(NUM_X)
        if (x, y) not in HOLES
    ]
    return np.asarray(pos, dtype=np.float32)


def tiled_array(tx: int, ty: int, pitch: float = PITCH) -> np.ndarray:
    """tx x ty tiling of the unit array, unit offsets (18 pitch, 14 pitch)."""
    unit = unit_array(pitch).astype(np.float64)
    out = []
    for j in range(ty):
        for i in range(tx):
            out.append(unit + np.array([NUM_X * pitch * i, NUM_Y * pitch * j, 0.0]))
    return np.concatenate(out).astype(np.float32)


def array_center(positions: np.ndarray) -> np.ndarray:
    """Centre of the full rectangular lattice that the positions belong to."""
    lo = positions.min(axis=0).astype(np.float64)
    hi = positions.max(axis=0).astype(np.float64)
    return ((lo + hi) / 2.0).astype(np.float32)


def wavenumber(freq: float = FREQ, c: float = SOUND_SPEED) -> np.float32:
    """k = 2 * PI * f / c in float32, the reference's expression (uniform_medium.rs:104)."""
    two_pi = np.float32(2.0) * np.float32(math.pi)
    return np.float32(np.float32(two_pi * np.float32(freq)) / np.float32(c))


def focal_phases(positions: np.ndarray, focus, c: float = SOUND_SPEED, freq: float = FREQ):
    """The reference focal law (focal_point.rs:28-39) in float32:
    phase = -2 * PI * ((|pos - f| mod lambda) / lambda), lambda = c / f."""
    f = np.asarray(focus, dtype=np.float32)
    d = positions.astype(np.float32) - f
    dist = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    wl = np.float32(np.float32(c) / np.float32(freq))
    ph = np.fmod(dist, wl) / wl
    return (np.float32(-2.0) * np.float32(math.pi)) * ph


def t4010a1_records(positions, amp, phase, freq: float = FREQ) -> np.ndarray:
    n = len(positions)
    rec = np.zeros((n, 9), dtype=np.float32)
    rec[:, 0:3] = positions
    rec[:, 5] = 1.0  # facing +z
    rec[:, 6] = amp
    rec[:, 7] = phase
    rec[:, 8] = freq
    return rec


def sphere_records(positions, amp, phase, freq: float = FREQ) -> np.ndarray:
    n = len(positions)
    rec = np.zeros((n, 6), dtype=np.float32)
    rec[:, 0:3] = positions
    rec[:, 3] = amp
    rec[:, 4] = phase
    rec[:, 5] = freq
    return rec


@dataclasses.dataclass
class GridSpec:
    """Arguments of AFC_CreateGridArea{1,2,3}D (capi/src/observe_area.rs:42-228): ranges in
    specification order (a fixed axis has start == end), resolution and axis codes."""

    dim: int
    ranges: list  # [(start, end)] * 3, in specification order
    res: float
    axes: tuple  # axis codes in specification order

    def lo_hi(self):
        lo = [0.0, 0.0, 0.0]
        hi = [0.0, 0.0, 0.0]
        for (a, b), ax in zip(self.ranges, self.axes):
            lo[ax - 1] = a
            hi[ax - 1] = b
        return np.asarray(lo, np.float32), np.asarray(hi, np.float32)


@dataclasses.dataclass
class Workload:
    name: str
    source_type: int  # 0 sphere, 1 T4010A1
    sources: np.ndarray  # (n, 9) or (n, 6) float32
    k: np.ndarray  # (n,) float32
    atten: np.ndarray  # (n,) float32
    grid: GridSpec | None = None
    points: np.ndarray | None = None  # (m, 3) float32 scatter points
    field_type: int = 0  # 0 pressure, 1 power, 2 complex

    @property
    def n(self) -> int:
        return len(self.k)


def _uniform_k_atten(n, alpha, freq=FREQ, c=SOUND_SPEED):
    return (np.full(n, wavenumber(freq, c), dtype=np.float32),
            np.full(n, alpha, dtype=np.float32))


def single_focus(z: float = 150.0, half: float = 50.0, res: float = 1.0) -> Workload:
    """One unit (249 transducers), amplitude 1, reference focal law towards
    (centre x, centre y, 150); pressure amplitude on a 101 x 101 XY grid at 1 mm, z = 150,
    no attenuation."""
    pos = unit_array()
    cen = array_center(pos)
    focus = (float(cen[0]), float(cen[1]), z)
    ph = focal_phases(pos, focus)
    src = t4010a1_records(pos, 1.0, ph)
    k, a = _uniform_k_atten(len(pos), 0.0)
    cx, cy = float(cen[0]), float(cen[1])
    grid = GridSpec(2, [(cx - half, cx + half), (cy - half, cy + half), (z, z)], res,
                    (AXIS_X, AXIS_Y, AXIS_Z))
    return Workload("single_focus_249src_101x101_pressure", 1, src, k, a, grid=grid,
                    field_type=0)


def random_pattern(rng: np.random.Generator, n: int):
    phase = rng.uniform(0.0, 2.0 * math.pi, n).astype(np.float32)
    amp = rng.uniform(0.5, 1.0, n).astype(np.float32)
    return amp, phase


def large_grid(seed: int = 1, count: int = 256, res: float = 0.5, z0: float = 50.0,
               tiles=(4, 4), alpha: float = 1.15e-2, field_type: int = 2) -> Workload:
    """4 x 4 tiling (3984 transducers), random phases/amplitudes, attenuation 1.15e-2 /mm,
    complex pressure on a 256^3 grid at 0.5 mm centred over the array, z from 50 mm.
    Each range is padded by half a step so that the f32 count ((end - start) / res) as usize + 1
    is exactly `count`."""
    rng = np.random.default_rng(seed)
    pos = tiled_array(*tiles)
    cen = array_center(pos)
    amp, phase = random_pattern(rng, len(pos))
    src = t4010a1_records(pos, amp, phase)
    k, a = _uniform_k_atten(len(pos), alpha)
    span = (count - 1) * res
    pad = 0.5 * res
    cx, cy = float(cen[0]), float(cen[1])
    ranges = [(cx - span / 2, cx + span / 2 + pad), (cy - span / 2, cy + span / 2 + pad),
              (z0, z0 + span + pad)]
    grid = GridSpec(3, ranges, res, (AXIS_X, AXIS_Y, AXIS_Z))
    return Workload(f"tiled{tiles[0]}x{tiles[1]}_{len(pos)}src_{count}^3_grid_complex", 1, src,
                    k, a, grid=grid, field_type=field_type)


def scatter_box(seed: int, m: int, center_xy, box=(200.0, 200.0), z=(50.0, 200.0)):
    rng = np.random.default_rng(seed)
    pts = np.empty((m, 3), dtype=np.float32)
    pts[:, 0] = rng.uniform(center_xy[0] - box[0] / 2, center_xy[0] + box[0] / 2, m)
    pts[:, 1] = rng.uniform(center_xy[1] - box[1] / 2, center_xy[1] + box[1] / 2, m)
    pts[:, 2] = rng.uniform(z[0], z[1], m)
    return pts


def multi_pattern(seed: int = 2, m: int = 262144, patterns: int = 1024, tiles=(4, 4),
                  alpha: float = 1.15e-2):
    """Fixed geometry of the large grid workload, m scatter points in a 200 x 200 x 150 mm box
    (z 50-200) and `patterns` random (amp, phase) patterns: returns (workload with the first
    pattern, amps (patterns x n), phases (patterns x n))."""
    rng = np.random.default_rng(seed)
    pos = tiled_array(*tiles)
    cen = array_center(pos)
    pts = scatter_box(seed + 1000, m, cen[:2])
    amps = rng.uniform(0.5, 1.0, (patterns, len(pos))).astype(np.float32)
    phases = rng.uniform(0.0, 2.0 * math.pi, (patterns, len(pos))).astype(np.float32)
    src = t4010a1_records(pos, amps[0], phases[0])
    k, a = _uniform_k_atten(len(pos), alpha)
    wl = Workload(f"multi_pattern_{len(pos)}src_{m}pts_{patterns}pat", 1, src, k, a,
                  points=pts, field_type=2)
    return wl, amps, phases


def gspat_request(rng: np.random.Generator, n_foci: int, tiles=(2, 2), z=(100.0, 200.0)):
    """A GS-PAT request on a tiling (996 transducers for 2 x 2): foci uniform in a
    100 x 100 mm box over the array centre at z 100-200, amplitudes U[0.5, 1]."""
    pos = tiled_array(*tiles)
    cen = array_center(pos)
    foci = np.empty((n_foci, 3), dtype=np.float32)
    foci[:, 0] = rng.uniform(cen[0] - 50, cen[0] + 50, n_foci)
    foci[:, 1] = rng.uniform(cen[1] - 50, cen[1] + 50, n_foci)
    foci[:, 2] = rng.uniform(z[0], z[1], n_foci)
    amps = rng.uniform(0.5, 1.0, n_foci).astype(np.float32)
    src = t4010a1_records(pos, 1.0, 0.0)
    k, a = _uniform_k_atten(len(pos), 0.0)
    return Workload(f"gspat_{len(pos)}src_{n_foci}foci", 1, src, k, a, points=foci,
                    field_type=0), foci, amps


# transducer counts of the batched-job mix and the tilings that give them
JOB_TILINGS = {249: (1, 1), 498: (2, 1), 996: (2, 2), 2490: (5, 2)}


@dataclasses.dataclass
class BatchJob:
    """One job of a batch: its sources (ABI records), and either a 2-D XY grid slice or a count
    of scatter points drawn uniformly over the array from `points_seed`."""

    sources: np.ndarray
    k: np.ndarray
    atten: np.ndarray
    field_type: int
    grid: GridSpec | None
    n_points: int
    points_seed: int
    box_lo: tuple
    box_hi: tuple

    @property
    def n(self):
        return len(self.k)


def batch_jobs(seed: int = 3, n_jobs: int = 2048, m_range=(1e3, 1e6),
               counts=(249, 498, 996, 2490), alpha: float = 1.15e-2):
    """The uneven-job mix: transducer count uniform over `counts` (array tilings), point count
    log-uniform in `m_range`, half the jobs 2-D XY grid slices at 0.5-2 mm spacing (z 50-200 mm
    over the array centre), half scatter sets in a box over the array; random phases and
    amplitudes; field type uniform over pressure / power / complex."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n_jobs):
        n = int(rng.choice(counts))
        pos = tiled_array(*JOB_TILINGS[n])
        cen = array_center(pos)
        amp, phase = random_pattern(rng, n)
        src = t4010a1_records(pos, amp, phase)
        k, a = _uniform_k_atten(n, alpha)
        m = int(round(math.exp(rng.uniform(math.log(m_range[0]), math.log(m_range[1])))))
        field_type = int(rng.integers(0, 3))
        z = float(rng.uniform(50.0, 200.0))
        if i % 2 == 0:
            res = float(rng.uniform(0.5, 2.0))
            side = max(1, int(round(math.sqrt(m))))
            span = (side - 1) * res
            cx, cy = float(cen[0]), float(cen[1])
            pad = 0.5 * res
            grid = GridSpec(2, [(cx - span / 2, cx + span / 2 + pad),
                                (cy - span / 2, cy + span / 2 + pad), (z, z)], res,
                            (AXIS_X, AXIS_Y, AXIS_Z))
            jobs.append(BatchJob(src, k, a, field_type, grid, side * side, 0, (), ()))
        else:
            half = float(rng.uniform(30.0, 120.0))
            lo = (float(cen[0]) - half, float(cen[1]) - half, 50.0)
            hi = (float(cen[0]) + half, float(cen[1]) + half, 200.0)
            jobs.append(BatchJob(src, k, a, field_type, None, m, int(rng.integers(1 << 30)), lo,
                                 hi))
    return jobs


def batch_job_points(job: BatchJob) -> np.ndarray:
    """The scatter points of a scatter-set BatchJob drawn on the host from its seed
    (float32 m x 3, uniform in the job's box)."""
    rng = np.random.default_rng(job.points_seed)
    lo = np.asarray(job.box_lo, np.float32)
    hi = np.asarray(job.box_hi, np.float32)
    return (lo + (hi - lo) * rng.random((job.n_points, 3), dtype=np.float32)).astype(np.float32)


@dataclasses.dataclass
class ServingRequest:
    """One request of the serving stream: `arrival` seconds after the stream starts; a field
    job (`job` indexes the payload pool of batch_jobs) or a GS-PAT hologram request on the
    2 x 2 tiling (`foci`, `amps`; the slice is 201 x 201 at 1 mm over the array centre at the
    foci's mean depth)."""

    arrival: float
    kind: str  # "field" | "gspat"
    job: int = -1
    foci: np.ndarray | None = None
    amps: np.ndarray | None = None


def serving_stream(lam: float, n_requests: int, pool_size: int, seed: int = 4,
                   field_share: float = 0.7, foci_range=(2, 64)):
    """A seeded Poisson stream at rate `lam` req/s: exponential inter-arrival gaps; each request
    a field job (probability `field_share`, payload uniform over the pool) or a GS-PAT request
    with M uniform in foci_range (inclusive), foci uniform in a 100 x 100 mm box over the 2 x 2
    tiling's centre at z 100-200 mm, target amplitudes U[0.5, 1]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / lam, n_requests))
    cen = array_center(tiled_array(2, 2))
    out = []
    for i in range(n_requests):
        if rng.random() < field_share:
            out.append(ServingRequest(float(t[i]), "field", job=int(rng.integers(pool_size))))
        else:
            m = int(rng.integers(foci_range[0], foci_range[1] + 1))
            foci = np.empty((m, 3), np.float32)
            foci[:, 0] = rng.uniform(cen[0] - 50, cen[0] + 50, m)
            foci[:, 1] = rng.uniform(cen[1] - 50, cen[1] + 50, m)
            foci[:, 2] = rng.uniform(100.0, 200.0, m)
            amps = rng.uniform(0.5, 1.0, m).astype(np.float32)
            out.append(ServingRequest(float(t[i]), "gspat", foci=foci, amps=amps))
    return out
