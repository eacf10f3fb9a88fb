"""Benchmark of the direct source->point summation on the large-grid workload:
3984 T4010A1 transducers (4 x 4 tiling of the 249-element array, random phases and amplitudes,
attenuation 1.15e-2 /mm), complex pressure on a 256^3 grid at 0.5 mm (16,777,216 points),
i.e. 6.68e10 source-point evaluations per step.  Metric: evaluations per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Arms
  ours       `value`: the device-level C-ABI call (AFC_FieldGridDevice) with sources already
             in HBM, timed with CUDA events on the launching stream; the L2 is flushed (a
             256 MiB write) between timed steps, outside the events.
             `e2e`: the reference-facing C-ABI call AFC_Calculate with host buffers: each step
             uploads the sources and downloads the 134 MB complex field into the field
             buffer (pinned host memory) -- wall-clock per call, the call synchronises.
             `cpu_baseline`: the oracle (C restatement of the reference CPU calculator,
             OpenMP over points) on a bounded z-slab of the same grid, on this host's cores;
             its `parity` checks the timed launches' field on that slab against the oracle's
             (max |p - p_ref| over the slab's peak |p_ref|, bar 1e-4).
             After the headline and outside its timed region, the same line carries the other
             configured workloads (skip them with --no-extras; single GPU only):
               `single_focus_e2e`  the 249-source single focus through AFC_Calculate, us per
                                   call by default and with opt-in source tracking, next to
                                   the oracle's CPU time for the same call;
               `multipattern`      1,024 patterns on 262,144 points x 3,984 sources: split-BF16
                                   and FP16 tensor-core contractions and FP32 direct summation,
                                   each with its error against float64 on 128 seeded rows;
               `batch`             2,048 uneven jobs, graph replay vs one by one;
               `serving`           Poisson streams at 1,000, 3,000 and 10,000 req/s: p50/p99,
                                   achieved req/s and evals/s.
  reference  the reference's CPU calculator restated in C (the oracle: the Rust reference
             cannot be built here), all host threads, each step one bounded z-slab sample.

Multi-GPU (torchrun): replicas only -- every rank evaluates its own copy of the workload with
no collective on the data path (weak scaling); `value` = evals of all ranks / max time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "acoustic-field-calculator_gb300"))

import workloads as W  # noqa: E402

METRIC = "source-point evaluations/s (FP32 direct summation, complex field)"
UNIT = "evals/s"
# canonical per-evaluation cost of the summation (rsqrt, sqrt in acos, ex2, sin, cos on the
# MUFU pipe; 32 FP32-pipe operations)
MUFU_PER_EVAL = 5
FP32_PER_EVAL = 32
# DRAM bytes (read + write) of one 256^3 launch of the field kernel, from an ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum (3.55 MB + 75.95 MB; part of the 134 MB output
# is still in L2 when the launch ends)
FIELD_TRAFFIC_256 = 79.50e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="grid: skip the other workloads that the default run measures after "
                         "the headline (single focus end to end, multi-pattern, batch, "
                         "serving)")
    ap.add_argument("--workload", default="grid",
                    choices=["grid", "multipattern", "batch", "serving", "scatter"],
                    help="grid: the headline 256^3 field; multipattern: 1,024 patterns on "
                         "262,144 points through the tensor-core contraction; batch: 2,048 "
                         "uneven jobs in one persistent launch from a CUDA graph; serving: a "
                         "Poisson request stream swept over arrival rates; scatter: the "
                         "3,984-source field at --scatter-points scattered points (the "
                         "general body)")
    ap.add_argument("--lams", default="100,300,1000,3000,10000",
                    help="serving: arrival rates (req/s) of the sweep")
    # smaller cases of the same kernels (profiling); the defaults are the workloads above
    ap.add_argument("--grid-count", type=int, default=256, help="grid: points per axis")
    ap.add_argument("--mp-points", type=int, default=262144, help="multipattern: points")
    ap.add_argument("--mp-patterns", type=int, default=1024, help="multipattern: patterns")
    ap.add_argument("--batch-jobs", type=int, default=2048, help="batch: job count")
    ap.add_argument("--batch-fixed-plan", action="store_true",
                    help="batch: the fixed plan (4 point pairs, occupancy blocks per SM) instead of "
                         "the autotuned one, so that a profiler sees no tuning launches")
    ap.add_argument("--scatter-points", type=int, default=262144,
                    help="scatter: points, drawn uniformly in the multi-pattern box")
    ap.add_argument("--serve-slots", type=int, default=32,
                    help="serving: requests in flight on the GPU at most")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def config_dict(w, count, extra=None):
    d = {"workload": w.name, "sources": w.n, "grid": [count] * 3, "resolution_mm": 0.5,
         "points": count ** 3, "evals_per_step": w.n * count ** 3, "field": "complex pressure",
         "attenuation_per_mm": 1.15e-2, "seed": 1, "parallelism": "replicas (no collective)"}
    if extra:
        d.update(extra)
    return d


# ------------------------------------------------------------------ CPU (oracle) legs

def cpu_slab(w, n_planes: int):
    """The first n_planes z-planes of the grid as explicit points (the slab the CPU times)."""
    lo, _ = w.grid.lo_hi()
    i = np.arange(256, dtype=np.float32)
    xs = lo[0] + i * np.float32(0.5)
    ys = lo[1] + i * np.float32(0.5)
    zs = lo[2] + np.arange(n_planes, dtype=np.float32) * np.float32(0.5)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float32)


def cpu_rate(w, pts, repeats=1):
    """Time the oracle's f32 field on pts; returns (times, threads, the last field)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O  # the CPU baseline only

    O.field_f32(1, w.sources, w.k, w.atten, pts[:256], O.FIELD_COMPLEX)  # warm
    times = []
    field = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        field = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_COMPLEX)
        times.append(time.perf_counter() - t0)
    return times, O.max_threads(), field


def cpu_baseline(w, gpu_field=None, target_s=12.0):
    """The oracle timed on a z-slab of the grid.  gpu_field (the timed launches' output, host
    complex64, grid order) is checked against the oracle's slab as it goes: the bar is 1e-4 of
    the slab's peak |p|."""
    # calibrate on a quarter plane, then size the slab to ~target_s of CPU work
    probe = cpu_slab(w, 1)[:16384]
    t, threads, _ = cpu_rate(w, probe)
    per_pt = t[0] / len(probe)
    planes = int(max(1, min(64, target_s / (per_pt * 65536))))
    pts = cpu_slab(w, planes)
    t, threads, ref = cpu_rate(w, pts)
    evals = len(pts) * w.n
    out = {"value": evals / t[0], "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{planes} z-plane(s) of the 256^3 grid = {len(pts)} points x {w.n} "
                     f"sources ({evals:.3e} evals) in {t[0]:.2f} s, oracle f32, "
                     f"{threads} OpenMP threads"}
    if gpu_field is not None and len(gpu_field) >= len(ref):
        err = float(np.max(np.abs(gpu_field[:len(ref)] - ref)) / np.max(np.abs(ref)))
        out["parity"] = {"max_abs_err_over_peak": err, "bar": 1e-4, "pass": err <= 1e-4,
                         "points": len(ref), "against": "oracle f32 (the reference CPU "
                                                       "calculator's restatement)"}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = W.large_grid()
    planes = 1
    pts = cpu_slab(w, planes)
    evals = len(pts) * w.n
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    for _ in range(max(0, args.warmup)):
        O.field_f32(1, w.sources, w.k, w.atten, pts[:4096], O.FIELD_COMPLEX)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_COMPLEX)
    dt = time.perf_counter() - t0
    value = evals * args.steps / dt
    threads = O.max_threads()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": config_dict(w, 256, {"sample_points_per_step": len(pts)}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: 1 z-plane of the grid ({len(pts)} points x "
                                       f"{w.n} sources = {evals:.3e} evals); the reference is "
                                       "Rust and cannot be built here, so its CPU calculator "
                                       "runs as the C restatement in oracle/"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ ranks

def max_over_ranks(seconds: float, dist, device) -> float:
    """The slowest rank's time (every rank gets it); `dist` None means one process."""
    if dist is None:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units processed by all ranks (replicas: each rank does the same work) per second."""
    return units_per_rank * world / seconds


# ------------------------------------------------------------------ GPU arm

def run_ours(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl")
    import afc

    lib = afc.DLL
    if lib.AFC_SetDevice(local) != 0:
        raise RuntimeError(afc.last_error())
    count = args.grid_count
    w = W.large_grid(count=count)
    evals = w.n * count ** 3

    # ---- device-resident arm (value)
    system = afc.UniformSystem(300.0)
    system.add_records(1, w.sources, w.k, w.atten)
    area = afc.grid_from_spec(w.grid)
    desc = area.grid_desc()
    m = int(desc.count[0] * desc.count[1] * desc.count[2])
    assert m == count ** 3
    dev = torch.device("cuda", local)
    d_src = torch.from_numpy(w.sources.reshape(-1)).to(dev)
    d_k = torch.from_numpy(w.k).to(dev)
    d_a = torch.from_numpy(w.atten).to(dev)
    ws_bytes = lib.AFC_FieldWorkspaceBytes(w.n)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    out = torch.empty(2 * m, dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step():
        rc = lib.AFC_FieldGridDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                     w.n, ctypes.byref(desc), out.data_ptr(), ws.data_ptr(),
                                     ws_bytes, sh)
        if rc != 0:
            raise RuntimeError(afc.last_error())

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()

    rates = (ctypes.c_double * 6)()
    clk = ctypes.c_double()
    nsm = ctypes.c_int32()
    if lib.AFC_MeasurePipeRates(rates, ctypes.byref(clk), ctypes.byref(nsm)) != 0:
        raise RuntimeError(afc.last_error())

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = lib.AFC_KernelLaunchCount()
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)  # L2 flush, outside the timed events
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        launches = lib.AFC_KernelLaunchCount() - launches0
        if dist:
            dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) * 1e-3
    total_s = max_over_ranks(total_s, dist, dev)
    value = whole_job_rate(evals * args.steps, world, total_s)
    per_gpu = evals * args.steps / total_s

    # ---- end-to-end arm through AFC_Calculate (host buffers)
    calc = afc.GpuCalculator()
    field = afc.ComplexPressureFieldBuffer()
    for _ in range(2):
        calc.calculate_raw(system, area, field)
    e2e_steps = max(1, min(args.steps, 5))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        calc.calculate_raw(system, area, field)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, dist, dev)
    h2d = w.n * (9 + 2) * 4
    d2h = m * 8

    # ---- roofline of the summation kernel (FP32 + MUFU issue)
    clock_summary = clocks.summary()
    sm_mhz = clock_summary.get("sm_mhz") or clk.value / 1e6
    mufu_names = ["ex2", "rsqrt", "sqrt", "sin", "cos"]
    mufu_rates = {nm: rates[i] for i, nm in enumerate(mufu_names)}
    # one of each MUFU op per evaluation: the MUFU pipe's time per eval is the sum of 1/rate
    mufu_bound = 1.0 / sum(1.0 / r for r in mufu_rates.values())
    fp32_bound = rates[5] / FP32_PER_EVAL
    peak_measured = min(mufu_bound, fp32_bound)
    peak_nominal = nsm.value * sm_mhz * 1e6 * min(16 / MUFU_PER_EVAL, 128 / FP32_PER_EVAL)
    roofline = {
        "bound": "fp32+sfu issue (compute)",
        "achieved": per_gpu, "unit": "evals/s",
        "peak": peak_measured, "frac": per_gpu / peak_measured if peak_measured else None,
        "peak_source": "measured here with pipe microbenchmarks (AFC_MeasurePipeRates): "
                       "peak = min(1/sum(1/rate) over ex2, rsqrt, sqrt, sin, cos; "
                       f"fp32/{FP32_PER_EVAL})",
        "mufu_ops_per_s": mufu_rates, "fp32_ops_per_s": rates[5],
        "mufu_bound_evals_per_s": mufu_bound, "fp32_bound_evals_per_s": fp32_bound,
        "calibration_sm_clock_mhz": clk.value / 1e6,
        "peak_nominal_at_sampled_clock": peak_nominal,
        "frac_of_nominal": per_gpu / peak_nominal if peak_nominal else None,
        "traffic": FIELD_TRAFFIC_256 if count == 256 else None,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one 256^3 launch",
        "algorithmic_bytes": d2h + 48 * w.n,
        "hbm_write_gbs": d2h / (total_s / args.steps) / 1e9,
    }

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": config_dict(w, count, {"l2": "flushed between timed steps (256 MiB write)"}),
            "e2e": {"value": evals * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                    "api": "AFC_Calculate (reference C ABI), host buffers"},
            "gpu_launches": int(launches), "roofline": roofline, "clocks": clock_summary,
            "wall_s_timed": wall}
    if rank == 0 and not args.no_cpu_baseline:
        # the timed launches' field on the first 64 planes (at most the slab the CPU runs)
        slab = min(m, 64 * count * count)
        gpu_field = out[:2 * slab].cpu().numpy().view(np.complex64)
        line["cpu_baseline"] = cpu_baseline(w, gpu_field if count == 256 else None)
    if world == 1 and count == 256 and not args.no_extras:
        del out, ws, flush
        torch.cuda.empty_cache()
        line.update(secondary_workloads(afc, torch, local, args))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


# ------------------------------------------------------------------ scatter points

def run_scatter(args):
    """The general (scatter-point) body alone: the 3,984-source large-grid geometry on
    --scatter-points points drawn uniformly in a 200 x 200 x 150 mm box over the array (seed 7),
    complex field, through the device-level AFC_FieldScatterDevice with everything resident;
    the L2 is flushed between timed steps.  Roofline: the FP32 + MUFU bound measured on this GPU,
    as for the headline."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    import afc

    lib = afc.DLL
    lib.AFC_SetDevice(local)
    w = W.large_grid()
    m = args.scatter_points
    pts = W.scatter_box(7, m, W.array_center(w.sources[:, :3])[:2])
    dev = torch.device("cuda", local)
    d_src = torch.from_numpy(w.sources.reshape(-1)).to(dev)
    d_k = torch.from_numpy(w.k).to(dev)
    d_a = torch.from_numpy(w.atten).to(dev)
    d_pts = torch.from_numpy(pts.reshape(-1)).to(dev)
    ws_bytes = lib.AFC_FieldWorkspaceBytes(w.n)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    out = torch.empty(2 * m, dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        rc = lib.AFC_FieldScatterDevice(1, 2, 0, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(),
                                        w.n, d_pts.data_ptr(), m, out.data_ptr(), ws.data_ptr(),
                                        ws_bytes, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(afc.last_error())

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    rates = (ctypes.c_double * 6)()
    clk = ctypes.c_double()
    nsm = ctypes.c_int32()
    if lib.AFC_MeasurePipeRates(rates, ctypes.byref(clk), ctypes.byref(nsm)) != 0:
        raise RuntimeError(afc.last_error())
    ts = []
    launches0 = lib.AFC_KernelLaunchCount()
    for _ in range(args.steps):
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    launches = lib.AFC_KernelLaunchCount() - launches0
    t = statistics.median(ts)
    evals = w.n * m
    mufu_bound = 1.0 / sum(1.0 / rates[i] for i in range(5))
    peak = min(mufu_bound, rates[5] / FP32_PER_EVAL)
    line = {"metric": "source-point evaluations/s (FP32 direct summation, scatter points)",
            "value": evals / t, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"scatter_{w.n}src_{m}pts_complex", "sources": w.n,
                       "points": m, "l2": "flushed between timed steps (256 MiB write)"},
            "roofline": {"bound": "fp32+sfu issue (compute)", "achieved": evals / t,
                         "peak": peak, "unit": "evals/s", "frac": evals / t / peak,
                         "peak_source": "measured here (AFC_MeasurePipeRates), as the headline"},
            "gpu_launches": int(launches)}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ shared timing helper

def event_times(torch, stream, fn, steps, warm):
    """CUDA-event durations [s] of `steps` calls of fn on `stream` after `warm` untimed ones."""
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    return ts


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


# ------------------------------------------------------------------ multi-pattern workload

BF16X3, FP16 = 1, 2


def multipattern_measure(afc, torch, local, m, K, steps, warmup, check_rows=128):
    """1,024 random patterns (K) on the 3,984-source geometry at m scatter points: P = G Q by
    the split-BF16 and row-scaled FP16 tensor-core contractions (G built once per geometry,
    timed apart) and by FP32 direct summation (one field launch per pattern).  Each form's P is
    compared on `check_rows` seeded rows (every pattern) with P computed in float64 from the
    oracle's float64 G."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    lib = afc.DLL
    w, amps, phases = W.multi_pattern(m=m, patterns=K)
    n = w.n
    dev = torch.device("cuda", local)
    d_src = torch.from_numpy(w.sources.reshape(-1)).to(dev)
    d_k = torch.from_numpy(w.k).to(dev)
    d_a = torch.from_numpy(w.atten).to(dev)
    d_pts = torch.from_numpy(w.points.reshape(-1)).to(dev)
    d_amps = torch.from_numpy(amps.reshape(-1)).to(dev)
    d_ph = torch.from_numpy(phases.reshape(-1)).to(dev)
    out = torch.empty(2 * m * K, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    rows = np.sort(np.random.default_rng(99).choice(m, min(check_rows, m), replace=False))
    idx = torch.from_numpy(rows).to(dev)
    # float64 reference on the sampled rows: G of unit amplitude and zero phase (the patterns
    # carry the drive) times Q
    unit = w.sources.copy()
    unit[:, 6], unit[:, 7] = 1.0, 0.0
    g64 = O.build_g_f64(1, unit, w.k, w.atten, w.points[rows])
    p64 = g64 @ (amps.astype(np.float64) * np.exp(1j * phases.astype(np.float64))).T

    def errs(pattern_major=False):
        # the contractions store P point-major (m x K), the direct path pattern by pattern
        if pattern_major:
            got = out.view(K, m, 2)[:, idx].permute(1, 0, 2).contiguous()
        else:
            got = out.view(m, K, 2)[idx]
        got = got.cpu().numpy().view(np.complex64)[..., 0]
        return {"max_abs_err_over_peak": float(np.max(np.abs(got - p64)) / np.max(np.abs(p64))),
                "rel_l2_err": float(np.linalg.norm(got - p64) / np.linalg.norm(p64)),
                "rows_checked": int(len(rows)), "against": "float64 (oracle G in float64)"}

    results = {}
    launches0 = lib.AFC_KernelLaunchCount()
    for prec, name in ((BF16X3, "split_bf16"), (FP16, "fp16_row_scaled")):
        wsb = lib.AFC_MultiPatternWorkspaceBytes(n, m, K, prec)
        ws = torch.empty(wsb + 256, dtype=torch.uint8, device=dev)
        base = (ws.data_ptr() + 255) // 256 * 256

        def build():
            rc = lib.AFC_MultiPatternBuildG(1, prec, d_src.data_ptr(), d_k.data_ptr(),
                                            d_a.data_ptr(), n, d_pts.data_ptr(), m, K, base, wsb,
                                            sh)
            assert rc == 0, afc.last_error()

        def apply():
            rc = lib.AFC_MultiPatternApply(prec, d_amps.data_ptr(), d_ph.data_ptr(), n, m, K,
                                           out.data_ptr(), base, wsb, sh)
            assert rc == 0, afc.last_error()

        tb = event_times(torch, stream, build, 1, 1)
        ta = event_times(torch, stream, apply, steps, max(warmup, 1))
        assert lib.AFC_MultiPatternStatus(prec, n, m, K, base, sh) == 0
        results[name] = {"apply_ms": statistics.median(ta) * 1e3, "build_g_ms": tb[0] * 1e3,
                         "workspace_gb": wsb / 1e9, **errs()}
        del ws
    # FP32 direct summation: one field evaluation per pattern
    wsd = 2 * lib.AFC_FieldWorkspaceBytes(n)
    ws = torch.empty(wsd, dtype=torch.uint8, device=dev)

    def direct():
        rc = lib.AFC_MultiPatternDirect(1, d_src.data_ptr(), d_k.data_ptr(), d_a.data_ptr(), n,
                                        d_pts.data_ptr(), m, d_amps.data_ptr(), d_ph.data_ptr(),
                                        K, out.data_ptr(), ws.data_ptr(), wsd, sh)
        assert rc == 0, afc.last_error()

    td = event_times(torch, stream, direct, 1, 1)
    results["fp32_direct"] = {"apply_ms": td[0] * 1e3, **errs(pattern_major=True)}
    launches = lib.AFC_KernelLaunchCount() - launches0
    del ws, out
    evals = n * m * K
    for v in results.values():
        v["evals_per_s"] = evals / (v["apply_ms"] * 1e-3)
    bf = results["split_bf16"]["apply_ms"] * 1e-3
    alg_flops = 8.0 * n * m * K  # 8 real flops per complex multiply-add
    kpad = (2 * n + 63) // 64 * 64
    hw_flops = 3 * 2.0 * m * (2 * K) * kpad  # hi.hi + hi.lo + lo.hi on the padded real GEMM
    peak = measured_peaks().get("bf16_tflops")
    peak_src = "MEASURED_PEAKS.json bf16_tflops (burst)"
    if not peak:
        peak, peak_src = 1900.0, "fallback 1.9 PFLOP/s (MEASURED_PEAKS.json absent)"
    return {
        "workload": w.name, "sources": n, "points": m, "patterns": K, "evals": evals,
        "results": results,
        "speedup_split_bf16_vs_fp32_direct": results["fp32_direct"]["apply_ms"] * 1e-3 / bf,
        "speedup_fp16_vs_fp32_direct": results["fp32_direct"]["apply_ms"] /
                                       results["fp16_row_scaled"]["apply_ms"],
        "roofline": {"bound": "tensor", "achieved": alg_flops / bf / 1e12,
                     "hardware_tflops": hw_flops / bf / 1e12, "peak": peak, "unit": "TFLOP/s",
                     "frac": alg_flops / bf / 1e12 / peak,
                     "frac_hardware": hw_flops / bf / 1e12 / peak, "peak_source": peak_src,
                     "note": "achieved = algorithmic flops (8 per complex MAC); hardware = "
                             "the three BF16 products the split form issues"},
        "gpu_launches": int(launches),
    }


def run_multipattern(args):
    """The multi-pattern workload alone: value = split-BF16 source-point-pattern evaluations
    per second of the contraction."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    import afc

    afc.DLL.AFC_SetDevice(local)
    r = multipattern_measure(afc, torch, local, args.mp_points, args.mp_patterns, args.steps,
                             args.warmup)
    bf = r["results"]["split_bf16"]
    line = {"metric": "source-point-pattern evaluations/s (split-BF16 tensor-core contraction)",
            "value": bf["evals_per_s"], "unit": "evals/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": bf["apply_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 (fp32 accumulate)",
            "data": "synthetic (seeded)",
            "config": {"workload": r["workload"], "sources": r["sources"],
                       "points": r["points"], "patterns": r["patterns"],
                       "l2": "inputs (8.4 GB of G planes) larger than L2"},
            "speedup_vs_fp32_direct": r["speedup_split_bf16_vs_fp32_direct"],
            "results": r["results"], "roofline": r["roofline"],
            "gpu_launches": r["gpu_launches"]}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ batched uneven jobs

def batch_measure(afc, torch, n_jobs, steps, warmup, one_by_one_steps=3, tune=True):
    """n_jobs independent field jobs (249/498/996/2,490 transducers, 1e3-1e6 points, half grid
    slices, half scatter sets) as one persistent launch replayed from a CUDA graph (autotuned
    plan), against the same jobs launched one by one."""
    import batch_device as BD

    lib = afc.DLL
    jobs = W.batch_jobs(n_jobs=n_jobs)
    arr, outs, pts, keep = BD.materialize(afc, torch, jobs)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    t0 = time.perf_counter()
    plan = BD.create_plan(afc, arr, tune, sh)
    create_s = time.perf_counter() - t0
    info = BD.describe(afc, plan)

    def run_graph():
        assert lib.AFC_BatchRun(plan, sh) == 0, afc.last_error()

    def run_each():
        assert lib.AFC_BatchRunOneByOne(plan, sh) == 0, afc.last_error()

    try:
        launches0 = lib.AFC_KernelLaunchCount()
        tb = event_times(torch, stream, run_graph, steps, max(warmup, 1))
        launches = (lib.AFC_KernelLaunchCount() - launches0) // (steps + max(warmup, 1))
        te = event_times(torch, stream, run_each, max(1, one_by_one_steps), 1)
    finally:
        lib.AFC_BatchFree(plan)
    evals = info["evals"]
    tbm, tem = statistics.median(tb), statistics.median(te)
    return {"workload": f"batch_{len(jobs)}_uneven_jobs", "jobs": len(jobs),
            "evals_per_step": evals, "points_per_step": int(sum(j.n_points for j in jobs)),
            "autotuned": info, "tuned": tune, "plan_create_s": create_s,
            "replay_ms": tbm * 1e3, "evals_per_s": evals / tbm,
            "one_by_one_ms": tem * 1e3, "one_by_one_evals_per_s": evals / tem,
            "one_by_one_launches_per_step": 2 * len(jobs),
            "speedup_vs_one_by_one": tem / tbm, "gpu_launches_per_replay": int(launches)}


def run_batch(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    import afc

    afc.DLL.AFC_SetDevice(local)
    r = batch_measure(afc, torch, args.batch_jobs, args.steps, args.warmup,
                      tune=not args.batch_fixed_plan)
    line = {"metric": "source-point evaluations/s (2,048 uneven jobs, one persistent launch)",
            "value": r["evals_per_s"], "unit": "evals/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["replay_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": r["workload"], "jobs": r["jobs"],
                       "evals_per_step": r["evals_per_step"],
                       "points_per_step": r["points_per_step"], "autotuned": r["autotuned"],
                       "plan_create_s": r["plan_create_s"]},
            "one_by_one": {"value": r["one_by_one_evals_per_s"], "ms_per_step": r["one_by_one_ms"],
                           "launches_per_step": r["one_by_one_launches_per_step"]},
            "speedup_vs_one_by_one": r["speedup_vs_one_by_one"],
            "gpu_launches": r["gpu_launches_per_replay"]}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ serving

def serving_measure(afc, lams, slots, warmup, max_requests=5000):
    """A seeded Poisson request stream through the serving engine (AFC_Serve*), swept over
    arrival rates: 70% field jobs drawn from a pool of the batched-job mix (the first 256
    jobs: 249-2,490 transducers, 1e3-1e6 points, grid slices and scatter sets), 30% GS-PAT
    requests on the 2 x 2 tiling (M uniform in 2..64, 100 iterations, then a 201 x 201
    pressure slice at the foci's mean depth).  Geometries are registered once and stay
    resident; each request uploads only its drive (or foci) and points, from host memory, and
    its result comes back to host memory.  Latency = submission to completion of the result's
    device-to-host copy, measured by the engine."""
    import serving_client as SC

    lib = afc.DLL
    pool = W.batch_jobs(n_jobs=256)
    eng = SC.Engine(afc, hbm_budget_bytes=2 << 30, pinned_bytes=2 << 30, max_inflight=slots)
    try:
        gid_of_n = {}
        for jb in pool:
            if jb.n not in gid_of_n:
                gid_of_n[jb.n] = eng.add_geometry(1, jb.sources, jb.k, jb.atten)
        gpos = W.tiled_array(2, 2)
        gcen = W.array_center(gpos)
        gsrc = W.t4010a1_records(gpos, 1.0, 0.0)
        n_g = len(gpos)
        gid_gspat = eng.add_geometry(1, gsrc, np.full(n_g, W.wavenumber(), np.float32),
                                     np.zeros(n_g, np.float32))
        # per pool job: (geometry, amps, phases, field type, grid desc or None, points, m, n)
        payload = []
        for jb in pool:
            amps = np.ascontiguousarray(jb.sources[:, 6])
            phases = np.ascontiguousarray(jb.sources[:, 7])
            if jb.grid is not None:
                desc = afc.grid_from_spec(jb.grid).grid_desc()
                m = int(desc.count[0] * desc.count[1] * desc.count[2])
                payload.append((gid_of_n[jb.n], amps, phases, jb.field_type, desc, None, m, jb.n))
            else:
                pts = W.batch_job_points(jb)
                payload.append((gid_of_n[jb.n], amps, phases, jb.field_type, None, pts,
                                jb.n_points, jb.n))
        slice_evals = n_g * 201 * 201

        def prepare(stream):
            out = []
            for r in stream:
                if r.kind == "field":
                    out.append(("field", r.arrival, payload[r.job]))
                else:
                    desc, _ = SC.slice_desc(afc, gcen, float(r.foci[:, 2].mean()), half=100.0,
                                            res=1.0)
                    out.append(("gspat", r.arrival, (r.foci, r.amps, desc)))
            return out

        def submit(item):
            kind, _, p = item
            if kind == "field":
                gid, amps, phases, ft, desc, pts, m, n = p
                rid, _ = eng.submit_field(gid, amps, phases, ft, grid=desc, points=pts)
                return rid, n * m
            foci, tamps, desc = p
            rid, _, _ = eng.submit_gspat(gid_gspat, n_g, foci, tamps, desc)
            return rid, slice_evals

        def run_stream(items):
            """Submit on the arrival schedule from this thread; a second thread waits."""
            import queue as Q

            q = Q.Queue()
            lat, qwait = [], []
            t_end = [0.0]

            def waiter():
                while True:
                    got = q.get()
                    if got is None:
                        return
                    rid, t_sub = got
                    la, qw = eng.wait(rid)
                    lat.append(la)
                    qwait.append(qw)
                    t_end[0] = max(t_end[0], t_sub + la)

            th = threading.Thread(target=waiter)
            th.start()
            evals = 0
            t0 = time.perf_counter()
            for it in items:
                while time.perf_counter() - t0 < it[1]:
                    pass
                t_sub = time.perf_counter()
                rid, ev = submit(it)
                evals += ev
                q.put((rid, t_sub))
            q.put(None)
            th.join()
            return np.asarray(lat), np.asarray(qwait), t_end[0] - t0, evals

        warm = prepare(W.serving_stream(1000.0, max(warmup, 1) * 20, len(pool), seed=99))
        run_stream(warm)
        launches0 = lib.AFC_KernelLaunchCount()
        st0 = eng.stats()
        sweep = []
        for i, lam in enumerate(lams):
            n_req = int(min(max(lam * 2.0, 200), max_requests))
            items = prepare(W.serving_stream(lam, n_req, len(pool), seed=4 + i))
            lat, qw, span, evals = run_stream(items)
            sweep.append({"offered_req_s": lam, "requests": n_req,
                          "gspat_requests": sum(1 for it in items if it[0] == "gspat"),
                          "achieved_req_s": n_req / span, "span_s": span,
                          "p50_ms": float(np.percentile(lat, 50) * 1e3),
                          "p99_ms": float(np.percentile(lat, 99) * 1e3),
                          "queue_p50_ms": float(np.percentile(qw, 50) * 1e3),
                          "queue_p99_ms": float(np.percentile(qw, 99) * 1e3),
                          "evals_per_s": evals / span})
        launches = lib.AFC_KernelLaunchCount() - launches0
        st = eng.stats()
    finally:
        eng.close()
    return {"workload": "serving_poisson_field70_gspat30", "pool_jobs": len(pool),
            "gspat_sources": n_g, "gspat_foci": [2, 64], "gspat_iterations": 100,
            "slice": [201, 201], "hbm_budget_bytes": st["hbm_budget_bytes"],
            "max_inflight": slots, "sweep": sweep,
            "engine": {"completed": st["completed"] - st0["completed"], "failed": st["failed"],
                       "peak_inflight": st["peak_inflight"],
                       "peak_hbm_bytes": st["peak_hbm_bytes"]},
            "gpu_launches": int(launches)}


def run_serving(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    import afc

    afc.DLL.AFC_SetDevice(local)
    lams = [float(x) for x in args.lams.split(",")]
    r = serving_measure(afc, lams, args.serve_slots, args.warmup)
    best = max(r["sweep"], key=lambda x: x["achieved_req_s"])
    line = {"metric": "requests/s (serving: Poisson stream, 70% field jobs / 30% GS-PAT)",
            "value": best["achieved_req_s"], "unit": "req/s", "n_gpus": 1,
            "steps": len(lams), "warmup": max(args.warmup, 1),
            "ms_per_step": best["span_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {k: r[k] for k in ("workload", "pool_jobs", "gspat_sources", "gspat_foci",
                                         "gspat_iterations", "slice", "hbm_budget_bytes",
                                         "max_inflight")},
            "sweep": r["sweep"], "engine": r["engine"],
            "e2e": {"value": best["achieved_req_s"], "unit": "req/s",
                    "note": "host buffers in and out; every request's copies are inside its "
                            "latency"},
            "gpu_launches": r["gpu_launches"]}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ single focus, end to end

def single_focus_e2e(afc, calls=200):
    """The 249-transducer single focus (101 x 101 pressure slice at z = 150 mm) through the
    reference-facing AFC_Calculate with host buffers, as the reference's example calls it:
    wall-clock per call, by default (sources uploaded and packed on every call) and with the
    opt-in source tracking (unchanged sources reused), next to the oracle's CPU time for the
    same call on this host's cores.  The result is checked against the oracle."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    w = W.single_focus()
    s = afc.UniformSystem(300.0)
    s.add_records(1, w.sources, w.k, w.atten)
    area = afc.grid_from_spec(w.grid)
    calc = afc.GpuCalculator()
    field = afc.PressureFieldBuffer()
    out = {}
    for mode, track in (("default", False), ("sources_tracked", True)):
        s.track_sources(track)
        for _ in range(20):
            calc.calculate_raw(s, area, field)
        t = []
        for _ in range(calls):
            t0 = time.perf_counter()
            calc.calculate_raw(s, area, field)
            t.append(time.perf_counter() - t0)
        out[mode] = {"median_us": statistics.median(t) * 1e6,
                     "p99_us": float(np.percentile(t, 99) * 1e6), "calls": calls}
    s.track_sources(False)
    got = calc.calculate(s, area, field)
    lo, hi = w.grid.lo_hi()
    pts = O.grid_points(2, lo, hi, w.grid.res, w.grid.axes)
    O.field_f32(1, w.sources, w.k, w.atten, pts[:256], O.FIELD_PRESSURE)  # warm
    tc = []
    for _ in range(5):
        t0 = time.perf_counter()
        ref = O.field_f32(1, w.sources, w.k, w.atten, pts, O.FIELD_PRESSURE)
        tc.append(time.perf_counter() - t0)
    evals = w.n * len(pts)
    cpu_us = statistics.median(tc) * 1e6
    return {"workload": w.name, "sources": w.n, "points": len(pts), "evals": evals,
            "api": "AFC_Calculate (reference C ABI), host buffers, one call per field",
            **{f"{k}_us_per_call": v["median_us"] for k, v in out.items()},
            "calls": out,
            "evals_per_s": evals / (out["default"]["median_us"] * 1e-6),
            "cpu_oracle_us_per_call": cpu_us, "cpu_oracle_threads": O.max_threads(),
            "speedup_vs_cpu_oracle": cpu_us / out["default"]["median_us"],
            "max_abs_err_over_peak": float(np.max(np.abs(got - ref)) / np.max(ref))}


def secondary_workloads(afc, torch, local, args):
    """The other configured workloads, measured after the headline and outside its timed
    region, for the same JSON line."""
    extras = {}
    t0 = time.perf_counter()
    extras["single_focus_e2e"] = single_focus_e2e(afc)
    extras["multipattern"] = multipattern_measure(afc, torch, local, 262144, 1024,
                                                  min(args.steps, 5), 2)
    torch.cuda.empty_cache()
    extras["batch"] = batch_measure(afc, torch, 2048, min(args.steps, 5), 1)
    torch.cuda.empty_cache()
    # the same warm-up stream as --workload serving (60 requests): with fewer, kernels first used
    # inside the measured 1,000 req/s stream put their loading into its p99
    extras["serving"] = serving_measure(afc, [1000.0, 3000.0, 10000.0], args.serve_slots, 3)
    extras["extras_wall_s"] = time.perf_counter() - t0
    return extras


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "multipattern":
        run_multipattern(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "scatter":
        run_scatter(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
