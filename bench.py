#!/usr/bin/env python
"""Tb.Th + Tb.Sp throughput of the GB300 library (one JSON line on stdout).

A step is one full pass of the hot path over one specimen: the exact squared
EDT and the local thickness of ROI-clipped bone (Tb.Th) and of in-ROI marrow
(Tb.Sp), reduced to mean / SD / max (metrics.rs:97-121).  The metric is input
voxels (counted once per specimen) per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gpu|reference]
  python bench.py --profile-case N [--plates]

--impl gpu (default): device-resident timing (``value``) with CUDA events on the
launching stream, per-kernel event timing (roofline of the dominant kernel),
an end-to-end leg through the host-pointer C ABI entry point with H2D/D2H in
the timed region (``e2e``), the CPU oracle timed on a bounded sample
(``cpu_baseline``), and nvidia-smi clock samples taken during the timed region.
At N = 1 the extras add the 1024^3 plate specimen (the same legs), the
64-specimen batch and the Poisson serving runs.
--impl reference: the reference algorithm's CPU implementation (the C++
oracle, OpenMP over all host cores; the Rust reference cannot be built here)
on the whole specimen of the workload, every step.
--profile-case N: a small case for profilers with a kernel filter (no timing):
Tb.Th and Tb.Sp of a seeded N^3 specimen twice, phases one after the other --
the first call is the warm-up (tables built), the second holds the launches
worth capturing.  The specimen is the 512^3 workload's generator at edge N
(sigma 5, BV/TV 0.15, cylinder ROI of radius 0.47 N); with --plates the 1024^3
workload's (sigma (4, 4, 8), BV/TV 0.30, sphere ROI of radius 500 N / 1024).

Multi-process (torchrun): every rank processes its own specimen (different
seed, same shape) with no data exchange -- replicas, weak scaling; rank 0
prints the line with the max time over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Gvoxel/s Tb.Th+Tb.Sp (EDT+local thickness), batched vs per-volume; p99 ms"
UNIT = "Gvoxel/s"

# Algorithmic bytes per voxel of each kernel family for one phase (reads +
# writes a perfect kernel must make; bitmask words count 1/8 byte per voxel).
ALGO_BYTES_PER_VOXEL = {
    "edt_x": 2.0 + 4.0 + 0.125,        # bone + roi in, u32 out, selection bits out
    "edt_y": 8.0,                      # u32 in, u32 out
    "edt_z": 8.0,
    "ridge": 4.0,                      # u32 distance map in (ridge records counted separately)
    "fill": 4.0,                       # u32 squared-thickness map out
    "fill_rank": 0.0,                  # per-r^2 tables only
    "fill_bin": 0.0,                   # per-ridge work (ridge records in, bin entries out)
    "templates": 0.0,
    "fill_sites": 0.0,                 # per-ridge work (sphere points of each ridge)
    "cleanup_final": 4.0 + 0.25 + 4.0,  # r^2 map in, two bitmasks in, f32 map out (the statistics read it)
    "stats_order": 8.0,                # f32 map read twice (chunk sums, chunk functions)
    "count_roi": 2.0,
}
EDT_FAMILIES = ("edt_x", "edt_y", "edt_z")

WORKLOADS = {
    "single512": dict(desc="512^3, sigma 5, BV/TV 0.15, cylinder ROI r240, 19.5 um", maker="config_single_512"),
    "plain128": dict(desc="128^3, sigma 3, BV/TV 0.25, cylinder ROI r56, 10 um", maker="config_plain_128"),
    "single1024": dict(desc="1024^3, sigma (4,4,8), BV/TV 0.30, sphere ROI r500, 8 um",
                       maker="config_single_1024"),
}


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gpu", "reference"), default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="single512")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 64-specimen batch and the Poisson serving measurements")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-rate-light", type=float, default=80.0,
                    help="second Poisson rate, below the GPU's capacity for the mix (0: skip)")
    ap.add_argument("--cpu-sample-slices", type=int, default=0,
                    help="z-slab depth of the GPU arm's CPU-baseline sample (default: sized to ~10 s)")
    ap.add_argument("--extra-steps", type=int, default=5, help="timed steps of the 1024^3 extra leg")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N",
                    help="run the profiling case at edge N instead of the benchmark")
    ap.add_argument("--plates", action="store_true", help="profiling case with the 1024^3 plate generator")
    ap.add_argument("--fill-rows", type=int, default=0, choices=(0, 32, 64),
                    help="profiling case: the fill's tile rows (0: 64, as on the 512^3 and 1024^3 workloads)")
    return ap.parse_args(argv)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_specimen(workload: str, rank: int):
    from bone_morphometry_gb300 import synthetic as S

    maker = getattr(S, WORKLOADS[workload]["maker"])
    base = maker.__defaults__[0]
    if workload == "single1024":
        # scipy on the host would take minutes for 1 G voxels: same recipe on the GPU
        return S.make_specimen_torch((1024, 1024, 1024), (4.0, 4.0, 8.0), 0.30, "sphere", 500.0, 8.0,
                                     base + 7919 * rank)
    return maker(seed=base + 7919 * rank)


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_run(sp, z0: int, slices: int, threads: int):
    """Both phases of the oracle (the reference algorithm) on z-slices
    [z0, z0 + slices) of the specimen -- the whole specimen when they cover it;
    returns (voxels, seconds)."""
    import numpy as np

    import oracle as O

    if threads:
        O.set_threads(threads)
    d = sp.bone.shape[0]
    whole = z0 == 0 and slices >= d
    bone = sp.bone if whole else np.ascontiguousarray(sp.bone[z0:z0 + slices])
    roi = sp.roi if whole else np.ascontiguousarray(sp.roi[z0:z0 + slices])
    t0 = time.perf_counter()
    for sel in (True, False):
        m = O.phase_inside(bone, roi, sel)
        lt = O.local_thickness(m, O.FOREGROUND)
        O.nonzero_stats(lt.thickness, sp.spacing_um)
    return bone.size, time.perf_counter() - t0


def default_slices(sp):
    d, h, w = sp.bone.shape
    # aim at ~10 s on a 16-core Grace host (~8 Mvoxel/s for both phases of the 512^3 data)
    target_vox = 80e6
    return max(4, min(d, int(target_vox / (h * w))))


def workload_config(workload: str, shape, world: int) -> dict:
    """The ``config`` object of the JSON line (the same for both arms)."""
    d, h, w = shape
    n_vox = d * h * w
    return {"workload": "%s: %s" % (workload, WORKLOADS[workload]["desc"]),
            "shape_whd": [w, h, d], "voxels_per_specimen": n_vox, "phases": ["Tb.Th", "Tb.Sp"],
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "inputs (%d MiB) and u32 maps (%d MiB each) larger than the 129 MB L2"
                  % (2 * n_vox >> 20, 4 * n_vox >> 20)}


def run_reference(args, rank, world):
    """CPU implementation of the reference algorithm (oracle port), all host
    threads, on the whole specimen of the workload every step (metrics.rs:97-121:
    both phases' local thickness and statistics)."""
    import oracle as O

    if rank != 0:
        return 0
    sp = make_specimen(args.workload, 0)
    d, h, w = sp.bone.shape
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    for _ in range(max(0, args.warmup)):
        cpu_run(sp, 0, d, threads)
    times = []
    vox = 0
    for _ in range(args.steps):
        vox, dt = cpu_run(sp, 0, d, threads)
        times.append(dt)
    total = sum(times)
    value = vox * len(times) / total / 1e9
    sample = "the whole %dx%dx%d %s specimen every step, both phases" % (w, h, d, args.workload)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u32/f32",
        "data": "synthetic (seeded Gaussian-smoothed noise, thresholded; no public dataset)",
        "config": workload_config(args.workload, sp.bone.shape, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the Rust reference cannot be built here (no cargo/rustc); the timed CPU path is the C++ "
                "restatement of edt.rs / local_thickness.rs / metrics.rs with OpenMP in place of rayon "
                "(serial where the reference is serial)",
    }
    print(json.dumps(line), flush=True)
    return 0


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    pos = q * (len(xs) - 1)
    lo, hi = int(pos), min(int(pos) + 1, len(xs) - 1)
    return xs[lo] + (pos - lo) * (xs[hi] - xs[lo])


def bench_batch(ctx, n_items=64):
    """64 specimens of uneven sizes: plain per-specimen calls vs the batched
    form, its settings (workers, site method, phase scheduling) picked by the
    library's tuner and kept in its cache file."""
    import torch

    from bone_morphometry_gb300 import analyze_thickness
    from bone_morphometry_gb300 import synthetic as S
    from bone_morphometry_gb300.serving import TUNE_CANDIDATES, SpecimenInput, tuned_batch_tbth_tbsp

    specs = S.batch_specs(n_items)
    items = []
    for sp in specs:
        d, h, w = sp.shape
        t = S.make_specimen_torch(sp.shape, sp.sigma, sp.bvtv, "cylinder", 0.45 * min(w, h), sp.spacing_um, sp.seed,
                                  to_host=False)
        items.append(t)
    torch.cuda.synchronize()
    vox = sum(int(t.bone.numel()) for t in items)
    dev = [SpecimenInput(t.bone, t.roi, t.spacing_um) for t in items]

    def plain():
        out = []
        for t in items:
            out.append(analyze_thickness(t.bone, t.roi, t.spacing_um, ctx=ctx))
        torch.cuda.synchronize()
        return out

    plain()  # warm buffers
    plain_times = []
    for _ in range(3):
        t0 = time.perf_counter()
        ref = plain()
        plain_times.append(time.perf_counter() - t0)
    t_plain = min(plain_times)
    # device time of the plain loop's kernels, each with the GPU to itself (phases one
    # after the other, so that no two timed kernels overlap)
    ctx.set_concurrent_phases(False)
    ctx.profile(True)
    plain()
    busy_ms = sum(v[1] for v in ctx.kernel_times().values())
    ctx.profile(False)
    ctx.set_concurrent_phases(True)
    t0 = time.perf_counter()
    _, tuning = tuned_batch_tbth_tbsp(dev, ctx=ctx)  # on a cache miss: every candidate, warm-up + 2 runs
    tune_s = time.perf_counter() - t0
    for _ in range(3):  # the stored choice: every worker's buffers grown to the mix's largest specimens
        tuned_batch_tbth_tbsp(dev, ctx=ctx)
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        res, _ = tuned_batch_tbth_tbsp(dev, ctx=ctx)
        times.append(time.perf_counter() - t0)
    t_batch = min(times)
    ctx.set_site_method(0)
    ctx.set_fill_tile_rows(0)
    ctx.set_concurrent_phases(True)
    same = all(r[2] == 0 and r[0].mean == a.thickness.mean and r[1].mean == a.spacing.mean
               and r[0].standard_deviation == a.thickness.standard_deviation for r, a in zip(res, ref))
    return {"specimens": n_items, "voxels": vox, "plain_gvoxel_s": vox / t_plain / 1e9,
            "batched_gvoxel_s": vox / t_batch / 1e9, "speedup": t_plain / t_batch, "plain_ms": 1e3 * t_plain,
            "batched_ms": 1e3 * t_batch, "workers": tuning.workers, "timing": "best of 3 runs of each form",
            "plain_ms_runs": [round(1e3 * t, 2) for t in plain_times],
            "batched_ms_runs": [round(1e3 * t, 2) for t in times],
            "kernels_one_at_a_time_ms": round(busy_ms, 2),
            "kernels_one_at_a_time_gvoxel_s": vox / (busy_ms * 1e-3) / 1e9,
            "tuning": {"workers": tuning.workers, "site_method": ["auto", "spheres", "chains"][tuning.site_method],
                       "fill_tile_rows": tuning.fill_tile_rows,
                       "concurrent_phases": tuning.concurrent_phases, "candidates": len(TUNE_CANDIDATES),
                       "from_cache": tuning.from_cache, "tuned_batch_ms": round(tuning.batch_ms, 2),
                       "tuning_s": round(tune_s, 2)},
            "results_identical_to_plain": bool(same),
            "data": "torch GPU generator, sizes log-uniform [96,384] per axis"}


_SERVING_POOL: list = []  # the 24 generated serving specimens, shared by the serving measurements


def bench_serving(n_requests=64, rate=200.0, budget=120e9, workers=(2, 4)):
    """Poisson arrivals (rate req/s) of specimens with edges log-uniform in
    [64, 768]; 24 distinct generated specimens are cycled.  Served form
    (continuous admission, HBM budget, several workers) vs serial plain
    processing of the same arrival sequence (one request at a time, measured),
    plus the p99 of an ideal serial queue built from each specimen's service
    time measured alone."""
    import numpy as np
    import torch

    from bone_morphometry_gb300 import Context, analyze_thickness
    from bone_morphometry_gb300 import synthetic as S
    from bone_morphometry_gb300.serving import Server

    pool = _SERVING_POOL
    if not pool:
        for sp in S.serving_specs(24):
            d, h, w = sp.shape
            pool.append(S.make_specimen_torch(sp.shape, sp.sigma, sp.bvtv, "cylinder", 0.45 * min(w, h),
                                              sp.spacing_um, sp.seed, to_host=True))
        torch.cuda.empty_cache()
    rng = np.random.default_rng(1234)
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    order = [i % len(pool) for i in range(n_requests)]
    # serial plain service time of each distinct specimen (host pointers, same path as a request)
    ctx = Context(0)
    service = []
    alone = []
    for sp in pool:
        analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx)
        t0 = time.perf_counter()
        alone.append(analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx))
        service.append(time.perf_counter() - t0)
    ctx.close()
    # ideal serial queue (each request's service time measured alone, no
    # overheads between requests), for reference
    t_arr = np.cumsum(gaps)
    end = 0.0
    lat_serial = []
    for i, k in enumerate(order):
        start = max(t_arr[i], end)
        end = start + service[k]
        lat_serial.append(end - t_arr[i])
    span_serial = end - t_arr[0]
    # served
    by_size = sorted(range(len(pool)), key=lambda k: -pool[k].bone.size)

    def serve(nworkers):
        with Server(workers=nworkers, hbm_budget_bytes=budget) as srv:
            # warm the workers (device buffers grown to the largest specimen,
            # tables built): every specimen once, the largest once per worker
            warm = [srv.submit(pool[k].bone, pool[k].roi, pool[k].spacing_um)
                    for k in [by_size[0]] * nworkers + by_size]
            for t in warm:
                srv.result(t)
            tickets = []
            t_start = time.perf_counter()
            for i, k in enumerate(order):
                target = t_start + t_arr[i] - t_arr[0]
                delay = target - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets.append((k, srv.submit(pool[k].bone, pool[k].roi, pool[k].spacing_um)))
            return [(k, srv.result(t)) for k, t in tickets]

    # serial plain, measured: one request at a time in arrival order (a single
    # worker).  Served: the same arrival sequence with several workers; the
    # worker count with the lowest p99 is reported (all are listed)
    runs = {}
    for nworkers in (1,) + tuple(w for w in workers if w != 1):
        res_w = serve(nworkers)
        lat_w = [r.latency_s for _, r in res_w]
        runs[nworkers] = (percentile(lat_w, 0.99), res_w)
    best = min((k for k in runs if k != 1), key=lambda k: runs[k][0])
    results = runs[best][1]
    vox = sum(int(pool[k].bone.size) for k in order)

    def summary(res):
        first = min(r.submit_s for _, r in res)
        last = max(r.end_s for _, r in res)
        lat = [r.latency_s for _, r in res]
        return vox / (last - first) / 1e9, 1e3 * percentile(lat, 0.5), 1e3 * percentile(lat, 0.99)

    served = summary(results)
    serial = summary(runs[1][1])
    same = all(r.status == 0 and r.thickness.mean == alone[k].thickness.mean
               and r.spacing.standard_deviation == alone[k].spacing.standard_deviation
               for res_w in (v[1] for v in runs.values()) for k, r in res_w)
    return {"requests": n_requests, "offered_req_s": rate, "distinct_specimens": len(pool),
            "mean_voxels_per_request": vox / n_requests, "hbm_budget_gb": budget / 1e9, "workers": best,
            "p99_ms_by_workers": {str(k): round(1e3 * v[0], 2) for k, v in runs.items()},
            "served_gvoxel_s": served[0], "served_p50_ms": served[1], "served_p99_ms": served[2],
            "serial_plain_gvoxel_s": serial[0], "serial_plain_p50_ms": serial[1], "serial_plain_p99_ms": serial[2],
            "serial_ideal_p99_ms": 1e3 * percentile(lat_serial, 0.99),
            "results_identical_to_alone": bool(same),
            "data": "torch GPU generator, edges log-uniform [64,768]; host-pointer requests (H2D inside)"}


def measure_specimen(ctx, sp, steps: int, warmup: int, local: int, barrier, reduce_max):
    """Device-resident timing, per-kernel event timing and the end-to-end leg
    of one specimen (both phases, metrics.rs:97-121) on one context."""
    import torch

    from bone_morphometry_gb300 import analyze_thickness

    n_vox = sp.bone.size
    stream = torch.cuda.current_stream()
    bone = torch.from_numpy(sp.bone).cuda()
    roi = torch.from_numpy(sp.roi).cuda()
    for _ in range(max(3, warmup)):
        ref_res = analyze_thickness(bone, roi, sp.spacing_um, ctx=ctx)
    torch.cuda.synchronize()

    # -- device-resident leg (Tb.Th and Tb.Sp side by side, the library default) ---------------
    launches0 = ctx.launches
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(steps):
            res = analyze_thickness(bone, roi, sp.spacing_um, ctx=ctx)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = ctx.launches - launches0
    ms = reduce_max(ev0.elapsed_time(ev1) / steps)
    assert res.thickness.mean == ref_res.thickness.mean and res.spacing.mean == ref_res.spacing.mean
    # -- per-kernel times for the roofline: the phases one after the other, so that
    # every kernel has the GPU to itself; CUDA events on each launch's stream ----------------
    ctx.set_concurrent_phases(False)
    ctx.profile(True)
    for _ in range(steps):
        analyze_thickness(bone, roi, sp.spacing_um, ctx=ctx)
    torch.cuda.synchronize()
    ktimes = ctx.kernel_times()
    ctx.profile(False)
    ctx.set_concurrent_phases(True)
    del bone, roi

    # -- end-to-end leg through the host-pointer entry point (pinned host inputs) --------------
    hb = torch.empty(sp.bone.shape, dtype=torch.uint8, pin_memory=True)
    hr = torch.empty(sp.roi.shape, dtype=torch.uint8, pin_memory=True)
    hb.numpy()[:] = sp.bone
    hr.numpy()[:] = sp.roi
    hbn, hrn = hb.numpy(), hr.numpy()
    analyze_thickness(hbn, hrn, sp.spacing_um, ctx=ctx)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        res_e = analyze_thickness(hbn, hrn, sp.spacing_um, ctx=ctx)
    e2e_s = (time.perf_counter() - t0) / steps
    assert res_e.thickness.mean == ref_res.thickness.mean
    e2e_s = reduce_max(e2e_s)
    del hb, hr, hbn, hrn
    return {"ms": ms, "e2e_s": e2e_s, "ktimes": ktimes, "clocks": clk.summary(), "launches": launches,
            "result": res}


def kernel_report(ktimes, n_vox: int, traffic: dict):
    """(kernels, roofline of the dominant kernel, EDT roofline) from the profiler's families."""
    total_kernel_ms = sum(v[1] for v in ktimes.values()) or 1.0
    kernels = {}
    for name, (nl, tms) in ktimes.items():
        if nl == 0:
            continue
        kernels[name] = {"launches": nl, "ms_per_launch": tms / nl, "share": tms / total_kernel_ms}
    peak, peak_src = measured_peak_gbs()

    def roof(name):
        nl, tms = ktimes[name]
        bpl = ALGO_BYTES_PER_VOXEL[name] * n_vox
        achieved = bpl / (tms / nl * 1e-3) / 1e9
        return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic.get(name), "algorithmic_bytes": bpl,
                "peak_source": peak_src}

    dominant = max((k for k in ktimes if ktimes[k][0] and ALGO_BYTES_PER_VOXEL.get(k, 0) > 0),
                   key=lambda k: ktimes[k][1])
    edt_ms = sum(ktimes[k][1] for k in EDT_FAMILIES) / max(1, ktimes["edt_x"][0])
    edt_bytes = sum(ALGO_BYTES_PER_VOXEL[k] for k in EDT_FAMILIES) * n_vox
    edt_achieved = edt_bytes / (edt_ms * 1e-3) / 1e9
    edt_roof = {"bound": "hbm", "achieved": edt_achieved, "peak": peak, "unit": "GB/s", "frac": edt_achieved / peak,
                "algorithmic_bytes_per_phase": edt_bytes, "ms_per_phase": edt_ms, "peak_source": peak_src}
    return kernels, roof(dominant), edt_roof


def bench_single1024(args, local):
    """The 1024^3 plate specimen (the largest single-GPU configuration): the
    same legs as the headline, on a context of its own."""
    import torch

    from bone_morphometry_gb300 import Context

    sp = make_specimen("single1024", 0)
    n_vox = sp.bone.size
    ctx = Context(local)
    try:
        m = measure_specimen(ctx, sp, args.extra_steps, 3, local, lambda: None, lambda v: v)
    finally:
        ctx.close()
        torch.cuda.empty_cache()
    kernels, roofline, edt_roof = kernel_report(m["ktimes"], n_vox, committed_traffic().get("single1024", {}))
    res = m["result"]
    return {"workload": "single1024: " + WORKLOADS["single1024"]["desc"], "shape_whd": [1024, 1024, 1024],
            "steps": args.extra_steps, "warmup": 3, "value": n_vox / (m["ms"] * 1e-3) / 1e9, "unit": UNIT,
            "ms_per_step": m["ms"],
            "e2e": {"value": n_vox / m["e2e_s"] / 1e9, "unit": UNIT, "h2d_bytes_per_step": 2 * n_vox,
                    "d2h_bytes_per_step": 2 * 104, "ms_per_step": m["e2e_s"] * 1e3},
            "gpu_launches": m["launches"], "roofline": roofline, "edt_roofline": edt_roof, "kernels": kernels,
            "clocks": m["clocks"],
            "result": {"TbTh_mean_um": res.thickness.mean, "TbTh_sd_um": res.thickness.standard_deviation,
                       "TbSp_mean_um": res.spacing.mean, "TbSp_sd_um": res.spacing.standard_deviation},
            "data": "torch GPU generator (seeded), inputs 2 GiB and maps 4 GiB each: larger than L2"}


def run_gpu(args, rank, world, local):
    import torch

    from bone_morphometry_gb300 import Context
    from bone_morphometry_gb300.replicas import max_over_ranks

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    sp = make_specimen(args.workload, rank)
    n_vox = sp.bone.size
    ctx = Context(local)
    m = measure_specimen(ctx, sp, args.steps, args.warmup, local, barrier, max_over_ranks)
    ms, res = m["ms"], m["result"]
    value = world * n_vox / (ms * 1e-3) / 1e9
    e2e_value = world * n_vox / m["e2e_s"] / 1e9

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    kernels, roofline, edt_roof = kernel_report(m["ktimes"], n_vox, committed_traffic().get(args.workload, {}))

    extras = {}
    if world == 1 and not args.no_extras:
        if args.workload != "single1024":
            extras["single1024"] = bench_single1024(args, local)
        extras["batch64"] = bench_batch(ctx)
        extras["serving"] = bench_serving(args.serve_requests, args.serve_rate)
        if args.serve_rate_light > 0:
            # the same mix at a rate the GPU keeps up with: latency without a growing queue
            extras["serving_light"] = bench_serving(args.serve_requests, args.serve_rate_light)

    # -- CPU baseline (rank 0, N = 1 only): the oracle on a bounded sample, after every GPU leg
    # (its host threads then cannot slow the GPU legs' host side) --------------------------------
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        d, h, w = sp.bone.shape
        slices = args.cpu_sample_slices or default_slices(sp)
        z0 = max(0, d // 2 - slices // 2)
        vox, dt = cpu_run(sp, z0, slices, threads)
        # one thread too, on a slab 1/8 as thick (the same algorithm, no parallelism)
        slices1 = max(4, slices // 8)
        vox1, dt1 = cpu_run(sp, max(0, d // 2 - slices1 // 2), slices1, 1)
        cpu = {"value": vox / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "z-slab %dx%dx%d of the same specimen, both phases, %.1f s" % (w, h, slices, dt),
               "value_1_thread": vox1 / dt1 / 1e9,
               "sample_1_thread": "z-slab %dx%dx%d, both phases, %.1f s" % (w, h, slices1, dt1)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u32/f32 (integer EDT and r^2, f32 map, f64 stats in the reference's order)",
        "data": "synthetic (seeded Gaussian-smoothed noise, thresholded; no public dataset)",
        "config": workload_config(args.workload, sp.bone.shape, world),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * n_vox,
                "d2h_bytes_per_step": 2 * 104, "ms_per_step": m["e2e_s"] * 1e3},
        "gpu_launches": m["launches"],
        "roofline": roofline,
        "edt_roofline": edt_roof,
        "kernels": kernels,
        "clocks": m["clocks"],
        "cpu_baseline": cpu,
        "result": {"TbTh_mean_um": res.thickness.mean, "TbTh_sd_um": res.thickness.standard_deviation,
                   "TbSp_mean_um": res.spacing.mean, "TbSp_sd_um": res.spacing.standard_deviation},
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_profile_case(args) -> int:
    """A small case for profilers with a kernel filter (no timing, no JSON line):
    Tb.Th and Tb.Sp of one specimen twice (the first call builds the tables and
    grows the buffers; the second holds the launches worth capturing), the
    phases one after the other so that each kernel runs alone."""
    import torch

    from bone_morphometry_gb300 import Context, analyze_thickness
    from bone_morphometry_gb300 import synthetic as S

    n = args.profile_case
    if args.plates:
        sp = S.make_specimen_torch((n, n, n), (4.0, 4.0, 8.0), 0.30, "sphere", 500.0 * n / 1024, 8.0, 1003,
                                   to_host=True)
    else:
        sp = S.make_specimen((n, n, n), 5.0, 0.15, "cylinder", 0.47 * n, 19.5, 1002)
    ctx = Context(0)
    ctx.set_concurrent_phases(False)
    # the fill tile shape of the 512^3 and 1024^3 workloads (a 384^3 case alone would get 32-row tiles)
    ctx.set_fill_tile_rows(64 if args.fill_rows == 0 else args.fill_rows)
    bone = torch.from_numpy(sp.bone).cuda()
    roi = torch.from_numpy(sp.roi).cuda()
    for _ in range(2):
        analyze_thickness(bone, roi, sp.spacing_um, ctx=ctx)
    torch.cuda.synchronize()
    ctx.close()
    print("profile case done: %d^3%s" % (n, " plates" if args.plates else ""))
    return 0


def main(argv=None):
    args = parse_args(argv)
    if args.profile_case:
        return run_profile_case(args)
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
