"""Batched and served forms of the Tb.Th / Tb.Sp path (bm_batch_tbth_tbsp and
bm_server_* in include/bm.h).

``batch_tbth_tbsp`` runs many specimens of uneven sizes through the context's
native worker pool: each worker owns a CUDA stream and buffers, so several
specimens are in flight on the GPU at once.  ``Server`` is the request loop:
submissions are admitted in arrival order while the estimated device footprint
of the running requests stays within an HBM budget, and each result carries
submit / start / end timestamps for latency percentiles.  Both use the
per-specimen arithmetic, so every result equals the specimen's result alone.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import tempfile
import time
from dataclasses import dataclass

import numpy as np

from ._lib import (BM_ERR_BUSY, BM_OK, BM_SITES_AUTO, BM_SITES_CHAINS, BM_SITES_SPHERES, BmResult, BmSpecimen,
                   BmStats, BoneMorphometryError, Context, default_context, last_error, load, raise_for)
from .api import DistributionStats, FeatureMode, _flags, _is_cuda_tensor


@dataclass
class SpecimenInput:
    bone: object          # (d, h, w) uint8 numpy array or CUDA tensor
    roi: object
    spacing_um: float


def _specimen_struct(sp: SpecimenInput) -> BmSpecimen:
    if _is_cuda_tensor(sp.bone):
        d, h, w = sp.bone.shape
        return BmSpecimen(sp.bone.data_ptr(), sp.roi.data_ptr(), w, h, d, float(sp.spacing_um))
    b = np.ascontiguousarray(sp.bone, np.uint8)
    r = np.ascontiguousarray(sp.roi, np.uint8)
    if b.shape != r.shape:
        raise ValueError("bone and roi shapes differ")
    d, h, w = b.shape
    return BmSpecimen(b.ctypes.data, r.ctypes.data, w, h, d, float(sp.spacing_um))


def batch_tbth_tbsp(specimens, feature_mode=FeatureMode.CLASSIC, ctx: Context | None = None, workers: int | None = None):
    """Tb.Th / Tb.Sp of every specimen; returns [(thickness, spacing, status)]."""
    ctx = ctx or default_context()
    lib = load()
    if workers is not None:
        raise_for(lib.bm_ctx_set_workers(ctx.handle, int(workers)), ctx.handle)
    items = list(specimens)
    if not items:
        return []
    device = _is_cuda_tensor(items[0].bone)
    keep = []
    arr = (BmSpecimen * len(items))()
    for i, sp in enumerate(items):
        if not device:
            sp = SpecimenInput(np.ascontiguousarray(sp.bone, np.uint8), np.ascontiguousarray(sp.roi, np.uint8),
                               sp.spacing_um)
            keep.append(sp)
        arr[i] = _specimen_struct(sp)
    th = (BmStats * len(items))()
    spc = (BmStats * len(items))()
    st = (ctypes.c_int * len(items))()
    lib.bm_batch_tbth_tbsp(ctx.handle, arr, len(items), 1 if device else 0, _flags(feature_mode), th, spc, st)
    return [(DistributionStats.from_c(th[i]), DistributionStats.from_c(spc[i]), int(st[i])) for i in range(len(items))]


# ---- settings of the batched form, picked by measurement ----------------------------------
#
# Four settings change how fast a batch runs and never what it returns: the
# number of workers, how the fill finds the non-selected voxels that ridge
# spheres reach (the sphere lattice points, a scatter per ridge, or the chain
# passes, a gather along the distance transform's argmins; local_thickness.rs:169-202
# paints them too), the fill's tile shape (by each specimen's size, or 32 x 32 x 16
# or 32 x 64 x 16 voxels for all),
# and whether each specimen's two phases run side by side.  The tuner runs the
# whole batch for every candidate and keeps the fastest, per GPU and per mix of
# specimen sizes, in a JSON file, so a later batch of the same kind starts from
# the stored choice.

TUNE_CANDIDATES = tuple((w, m, r, c) for w in (6, 8) for m in (BM_SITES_AUTO, BM_SITES_SPHERES, BM_SITES_CHAINS)
                        for r in (0, 32, 64) for c in (True, False))
_TUNE_FIELDS = ("workers", "site_method", "fill_tile_rows", "concurrent_phases")


@dataclass
class Tuning:
    workers: int
    site_method: int
    fill_tile_rows: int
    concurrent_phases: bool
    batch_ms: float          # the chosen candidate's time when it was measured
    from_cache: bool = False

    def setting(self):
        return (self.workers, self.site_method, self.fill_tile_rows, self.concurrent_phases)


def tuning_cache_path() -> str:
    """BM_TUNE_CACHE, else ~/.cache/bone_morphometry_gb300/batch_tuning.json."""
    return os.environ.get("BM_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                           "bone_morphometry_gb300", "batch_tuning.json")


def mix_signature(shapes) -> str:
    """Buckets of a mix: specimen count (octaves), total and largest voxel
    counts (half octaves)."""
    vox = [int(np.prod(s)) for s in shapes]
    if not vox:
        return "empty"
    half_octave = lambda v: int(round(2.0 * math.log2(max(v, 1))))
    return "n%d-t%d-m%d" % (len(vox).bit_length(), half_octave(sum(vox)), half_octave(max(vox)))


def device_key(device: int = 0) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda:%d" % device


def _load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _save_cache(path: str, data: dict) -> None:
    d = os.path.dirname(path) or "."
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, prefix=".tuning-", suffix=".json")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)  # readers see the old file or the new one, never a partial one


def autotune(run, key: str, path: str, candidates=TUNE_CANDIDATES, retune: bool = False,
             clock=time.perf_counter, repeats: int = 3):
    """run(workers, site_method, fill_tile_rows, concurrent_phases) -> results.  On a cache
    miss (or retune) every candidate runs once untimed (a new setting gives
    the pool new worker contexts, whose buffers grow on their first batch),
    then `repeats` times timed; the candidate with the lowest median time is
    stored under key (single batch times vary by ~15% from run to run).  On a
    hit only the stored candidate runs.  Returns (results, Tuning)."""
    candidates = tuple(candidates)
    if not candidates:
        raise ValueError("autotune needs at least one candidate setting")
    cache = _load_cache(path)
    hit = cache.get(key)
    if hit is not None and all(f in hit for f in _TUNE_FIELDS) and not retune:
        t = Tuning(int(hit["workers"]), int(hit["site_method"]), int(hit["fill_tile_rows"]),
                   bool(hit["concurrent_phases"]), float(hit["batch_ms"]), True)
        return run(*t.setting()), t
    best = None
    for cand in candidates:
        run(*cand)  # warm-up of this setting
        times = []
        for _ in range(max(1, repeats)):
            t0 = clock()
            res = run(*cand)
            times.append(clock() - t0)
        dt = sorted(times)[len(times) // 2]
        if best is None or dt < best[0]:
            best = (dt, cand, res)
    dt, (w, m, r, c), res = best
    t = Tuning(int(w), int(m), int(r), bool(c), 1e3 * dt)
    cache[key] = dict(zip(_TUNE_FIELDS, t.setting()), batch_ms=round(t.batch_ms, 3))
    _save_cache(path, cache)
    return res, t


def tuned_batch_tbth_tbsp(specimens, feature_mode=FeatureMode.CLASSIC, ctx: Context | None = None,
                          cache_path: str | None = None, retune: bool = False, candidates=TUNE_CANDIDATES):
    """batch_tbth_tbsp with the settings the tuner picks for this GPU and mix
    (they stay set on the context).  Returns ([(thickness, spacing, status)], Tuning)."""
    ctx = ctx or default_context()
    items = list(specimens)
    key = device_key(ctx.device) + "|" + mix_signature([tuple(sp.bone.shape) for sp in items])

    def run(workers, site_method, fill_rows, concurrent):
        ctx.call("bm_ctx_set_workers", int(workers))
        ctx.set_site_method(site_method)
        ctx.set_fill_tile_rows(fill_rows)
        ctx.set_concurrent_phases(concurrent)
        return batch_tbth_tbsp(items, feature_mode, ctx)

    return autotune(run, key, cache_path or tuning_cache_path(), candidates, retune)


def footprint_bytes(shape) -> int:
    d, h, w = shape
    return int(load().bm_footprint_bytes(w, h, d))


@dataclass
class Result:
    ticket: int
    status: int
    thickness: DistributionStats
    spacing: DistributionStats
    submit_s: float
    start_s: float
    end_s: float
    footprint_bytes: int
    message: str = ""  # error text when status != 0

    @property
    def latency_s(self) -> float:
        return self.end_s - self.submit_s


class Server:
    """Request loop over the native worker pool with HBM-budget admission."""

    def __init__(self, device: int = 0, workers: int = 4, hbm_budget_bytes: float = 120e9):
        self._lib = load()
        h = ctypes.c_void_p()
        st = self._lib.bm_server_create(int(device), int(workers), float(hbm_budget_bytes), ctypes.byref(h))
        if st != BM_OK:
            raise BoneMorphometryError(st, last_error(None) or "server creation failed")
        self.handle = h
        self._inputs = {}

    def submit(self, bone, roi, spacing_um: float, feature_mode=FeatureMode.CLASSIC) -> int:
        sp = SpecimenInput(np.ascontiguousarray(bone, np.uint8), np.ascontiguousarray(roi, np.uint8), spacing_um)
        s = _specimen_struct(sp)
        t = ctypes.c_uint64()
        st = self._lib.bm_server_submit(self.handle, ctypes.byref(s), _flags(feature_mode), ctypes.byref(t))
        if st != BM_OK:
            raise BoneMorphometryError(st, "request exceeds the HBM budget" if st == BM_ERR_BUSY else "submit failed")
        self._inputs[t.value] = sp  # keep the host buffers alive until the result is taken
        return t.value

    def submit_tiff(self, bone_path, roi_path=None, spacing_um: float = 1.0, threshold: int = 0,
                    strict_binary: bool = False, feature_mode=FeatureMode.CLASSIC) -> int:
        """A request read from TIFF stacks on the worker (tiff_io.rs:19-31): decoded
        into the worker's page-locked buffers, no host copy in between."""
        t = ctypes.c_uint64()
        st = self._lib.bm_server_submit_tiff(self.handle, os.fsencode(os.fspath(bone_path)),
                                             None if roi_path is None else os.fsencode(os.fspath(roi_path)),
                                             int(threshold), 1 if strict_binary else 0, float(spacing_um),
                                             _flags(feature_mode), ctypes.byref(t))
        if st != BM_OK:
            raise BoneMorphometryError(st, "request exceeds the HBM budget" if st == BM_ERR_BUSY else last_error(None))
        return t.value

    def result(self, ticket: int, wait: bool = True):
        r = BmResult()
        st = self._lib.bm_server_poll(self.handle, ctypes.c_uint64(ticket), 1 if wait else 0, ctypes.byref(r))
        if st == BM_ERR_BUSY:
            return None
        if st != BM_OK:
            raise BoneMorphometryError(st, "unknown ticket %d" % ticket)
        self._inputs.pop(ticket, None)
        return Result(ticket, r.status, DistributionStats.from_c(r.thickness), DistributionStats.from_c(r.spacing),
                      r.submit_s, r.start_s, r.end_s, int(r.footprint_bytes), r.message.decode("utf-8", "replace"))

    def stats(self):
        q, run, b = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        self._lib.bm_server_stats(self.handle, ctypes.byref(q), ctypes.byref(run), ctypes.byref(b))
        return int(q.value), int(run.value), float(b.value)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.bm_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
