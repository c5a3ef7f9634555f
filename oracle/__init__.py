"""CPU oracle for the Tb.Th / Tb.Sp hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package, and only as the reference results to compare
against or the timed CPU baseline.  The product library (``bone_morphometry_gb300``) never imports it
and has no CPU fallback.

The C++ restatement in ``bm_oracle.cpp`` follows the reference line by line
(citations there).  This module adds numpy conveniences and two checks that
do not exist in the reference:

* ``exact_moment_sums`` -- the exact sum and sum of squares of the
  f32-scaled map values, correctly rounded to f64 (the reference sums
  sequentially in f64, metrics.rs:215-226; the exact sums are what the GPU
  reproduces bit for bit).
* ``stats_from_sums`` -- the reference's mean / SD formulas
  (metrics.rs:232-241) applied to given sums.

Parity pins: the reference's known-answer tests (edt.rs:240-274,
local_thickness.rs:364-401, metrics.rs:304-326, volume.rs:123-136) and
scipy's exact EDT, checked in tests/test_oracle.py.  Beyond those tiny
cases the local-thickness stages (ridge, fill, cleanup) are pinned only by
this restatement of the source: the reference ships no Tb.Th / Tb.Sp
fixtures and cannot be built here (no Rust toolchain).
"""

from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

FOREGROUND = 0
BACKGROUND = 1

_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        f32p = ctypes.POINTER(ctypes.c_float)
        f64p = ctypes.POINTER(ctypes.c_double)
        sz = ctypes.c_size_t
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_num_threads.argtypes = [ctypes.c_int]
        L.orc_phase_inside.argtypes = [u8p, u8p, sz, ctypes.c_int, u8p]
        L.orc_edt_sq.argtypes = [u8p, sz, sz, sz, ctypes.c_int, u32p]
        L.orc_edt_sq.restype = ctypes.c_int
        L.orc_create_templates.argtypes = [u32p, sz, u32p, u32p, u32p]
        L.orc_integer_sqrt.argtypes = [ctypes.c_uint32]
        L.orc_integer_sqrt.restype = ctypes.c_uint32
        L.orc_ceiling_sqrt.argtypes = [ctypes.c_uint32]
        L.orc_ceiling_sqrt.restype = ctypes.c_uint32
        L.orc_distance_ridges.argtypes = [u8p, sz, sz, sz, ctypes.c_int, u32p, u64p, u32p, sz]
        L.orc_distance_ridges.restype = sz
        L.orc_propagate.argtypes = [sz, sz, sz, u64p, u32p, sz, u32p]
        L.orc_r2_to_diameter.argtypes = [u32p, sz, f32p]
        L.orc_cleanup.argtypes = [f32p, sz, sz, sz, f32p]
        L.orc_local_thickness.argtypes = [u8p, sz, sz, sz, ctypes.c_int, f32p, u32p, u32p,
                                          ctypes.POINTER(sz)]
        L.orc_local_thickness.restype = ctypes.c_int
        L.orc_nonzero_stats.argtypes = [f32p, sz, ctypes.c_double, f64p]
        L.orc_nonzero_stats.restype = ctypes.c_int
        L.orc_quantiles.argtypes = [f32p, sz, ctypes.c_double, f64p, sz, f64p]
        L.orc_quantiles.restype = ctypes.c_int
        L.orc_exact_moment_sums.argtypes = [f32p, sz, ctypes.c_double, u64p, u64p, f64p]
        L.orc_exact_moment_sums.restype = ctypes.c_uint64
        _LIB = L
    return _LIB


def _p(a: np.ndarray, ct):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ct))


class OracleError(RuntimeError):
    pass


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def _dims(vol: np.ndarray):
    d, h, w = vol.shape  # index = (z*h + y)*w + x, x fastest
    return w, h, d


def phase_inside(bone: np.ndarray, roi: np.ndarray, select_bone: bool) -> np.ndarray:
    bone = np.ascontiguousarray(bone, np.uint8)
    roi = np.ascontiguousarray(roi, np.uint8)
    out = np.empty_like(bone)
    lib().orc_phase_inside(_p(bone, ctypes.c_uint8), _p(roi, ctypes.c_uint8), bone.size,
                           1 if select_bone else 0, _p(out, ctypes.c_uint8))
    return out


def edt_sq(vol: np.ndarray, phase: int = FOREGROUND) -> np.ndarray:
    vol = np.ascontiguousarray(vol, np.uint8)
    w, h, d = _dims(vol)
    out = np.empty(vol.shape, np.uint32)
    rc = lib().orc_edt_sq(_p(vol, ctypes.c_uint8), w, h, d, phase, _p(out, ctypes.c_uint32))
    if rc:
        raise OracleError("distance transform is undefined for an all-%s volume unless an exterior "
                          "convention is specified" % ("foreground" if phase == 0 else "background"))
    return out


def create_templates(values) -> np.ndarray:
    v = np.ascontiguousarray(np.asarray(values, np.uint32))
    t = np.empty((3, v.size), np.uint32)
    lib().orc_create_templates(_p(v, ctypes.c_uint32), v.size, _p(t[0], ctypes.c_uint32),
                               _p(t[1], ctypes.c_uint32), _p(t[2], ctypes.c_uint32))
    return t


def distance_ridges(vol: np.ndarray, phase: int, sq: np.ndarray):
    """Ridge records (linear index, r^2) in ascending index order."""
    vol = np.ascontiguousarray(vol, np.uint8)
    sq = np.ascontiguousarray(sq, np.uint32)
    w, h, d = _dims(vol)
    L = lib()
    n = L.orc_distance_ridges(_p(vol, ctypes.c_uint8), w, h, d, phase, _p(sq, ctypes.c_uint32),
                              None, None, 0)
    idx = np.empty(n, np.uint64)
    r2 = np.empty(n, np.uint32)
    L.orc_distance_ridges(_p(vol, ctypes.c_uint8), w, h, d, phase, _p(sq, ctypes.c_uint32),
                          _p(idx, ctypes.c_uint64), _p(r2, ctypes.c_uint32), n)
    return idx, r2


def propagate(shape, idx: np.ndarray, r2: np.ndarray) -> np.ndarray:
    d, h, w = shape
    idx = np.ascontiguousarray(idx, np.uint64)
    r2 = np.ascontiguousarray(r2, np.uint32)
    out = np.empty(shape, np.uint32)
    lib().orc_propagate(w, h, d, _p(idx, ctypes.c_uint64), _p(r2, ctypes.c_uint32), idx.size,
                        _p(out, ctypes.c_uint32))
    return out


def r2_to_diameter(r2: np.ndarray) -> np.ndarray:
    r2 = np.ascontiguousarray(r2, np.uint32)
    out = np.empty(r2.shape, np.float32)
    lib().orc_r2_to_diameter(_p(r2, ctypes.c_uint32), r2.size, _p(out, ctypes.c_float))
    return out


def cleanup(dia: np.ndarray) -> np.ndarray:
    dia = np.ascontiguousarray(dia, np.float32)
    d, h, w = dia.shape
    out = np.empty_like(dia)
    lib().orc_cleanup(_p(dia, ctypes.c_float), w, h, d, _p(out, ctypes.c_float))
    return out


@dataclass
class LocalThickness:
    thickness: np.ndarray      # f32 diameters in voxels, masked by phase
    edt: np.ndarray            # u32 squared EDT
    propagated: np.ndarray     # u32 squared-thickness map (unmasked, before sqrt)
    n_ridges: int


def local_thickness(vol: np.ndarray, phase: int = FOREGROUND) -> LocalThickness:
    vol = np.ascontiguousarray(vol, np.uint8)
    w, h, d = _dims(vol)
    out = np.empty(vol.shape, np.float32)
    edt = np.empty(vol.shape, np.uint32)
    prop = np.empty(vol.shape, np.uint32)
    nr = ctypes.c_size_t(0)
    rc = lib().orc_local_thickness(_p(vol, ctypes.c_uint8), w, h, d, phase, _p(out, ctypes.c_float),
                                   _p(edt, ctypes.c_uint32), _p(prop, ctypes.c_uint32),
                                   ctypes.byref(nr))
    if rc:
        raise OracleError("distance transform is undefined for an all-%s volume unless an exterior "
                          "convention is specified" % ("foreground" if phase == 0 else "background"))
    return LocalThickness(out, edt, prop, int(nr.value))


@dataclass
class Stats:
    count: int
    mean: float
    sd: float
    max: float
    sum: float
    sum_sq: float


def nonzero_stats(values: np.ndarray, scale: float) -> Stats:
    """Reference statistics with its sequential f64 accumulation (metrics.rs:204-241)."""
    v = np.ascontiguousarray(values, np.float32).ravel()
    out = np.zeros(6, np.float64)
    rc = lib().orc_nonzero_stats(_p(v, ctypes.c_float), v.size, float(scale), _p(out, ctypes.c_double))
    if rc:
        raise OracleError("cannot compute statistics because the selected phase is empty")
    return Stats(int(out[0]), float(out[1]), float(out[2]), float(out[3]), float(out[4]), float(out[5]))


def quantiles(values: np.ndarray, scale: float, qs=(0.5, 0.1, 0.25, 0.75, 0.9)):
    v = np.ascontiguousarray(values, np.float32).ravel()
    q = np.ascontiguousarray(np.asarray(qs, np.float64))
    out = np.zeros(q.size, np.float64)
    rc = lib().orc_quantiles(_p(v, ctypes.c_float), v.size, float(scale), _p(q, ctypes.c_double), q.size,
                             _p(out, ctypes.c_double))
    if rc:
        raise OracleError("cannot compute statistics because the selected phase is empty")
    return out


def exact_moment_sums(values: np.ndarray, scale: float):
    """Exact sum and sum of squares of v = f32(raw * f32(scale)) over finite raw > 0,
    each correctly rounded to f64, plus count and max.

    The per-exponent integer sums come from the C++ oracle (OpenMP, no
    temporaries, so it serves 1024^3 maps); they are combined here in Python
    ints.  ``exact_moment_sums_numpy`` computes the same with numpy alone.
    """
    raw = np.ascontiguousarray(values, np.float32).ravel()
    s1 = np.zeros(256, np.uint64)
    s2 = np.zeros(512, np.uint64)
    mx = ctypes.c_double(0.0)
    n = int(lib().orc_exact_moment_sums(_p(raw, ctypes.c_float), raw.size, float(scale), _p(s1, ctypes.c_uint64),
                                        _p(s2, ctypes.c_uint64), ctypes.byref(mx)))
    if n == 0:
        raise OracleError("cannot compute statistics because the selected phase is empty")
    total = 0
    total_sq = 0
    for e in range(256):
        if s1[e]:
            total += int(s1[e]) << e                                     # sum * 2**150
            total_sq += ((int(s2[2 * e + 1]) << 64) | int(s2[2 * e])) << (2 * e)  # sum_sq * 2**300
    return n, _int_ratio_to_f64(total, 150), _int_ratio_to_f64(total_sq, 300), float(mx.value)


def exact_moment_sums_numpy(values: np.ndarray, scale: float):
    """``exact_moment_sums`` in numpy and Python ints alone (an independent
    check of the C++ bins; memory grows with the map, so for small maps).

    Every v is an f32, so v = m * 2**e with an integer 24-bit m; v*v = m*m * 2**(2e)
    is exact.  Integer sums per exponent are exact in Python ints.
    """
    raw = np.ascontiguousarray(values, np.float32).ravel()
    keep = np.isfinite(raw) & (raw > 0)
    v = raw[keep] * np.float32(scale)
    n = int(v.size)
    if n == 0:
        raise OracleError("cannot compute statistics because the selected phase is empty")
    bits = v.view(np.uint32).astype(np.int64)
    e = (bits >> 23) & 0xFF
    frac = bits & 0x7FFFFF
    m = np.where(e > 0, frac | (1 << 23), frac)
    e = np.where(e > 0, e, 1)  # value = m * 2**(e - 150)
    total = 0
    total_sq = 0
    for ee in np.unique(e):
        sel = e == ee
        ms = m[sel]
        s1 = int(ms.sum())  # < 2**24 * 2**39, fits int64
        hi = ms >> 12
        lo = ms & 0xFFF
        # m*m = hi*hi*2**24 + 2*hi*lo*2**12 + lo*lo, each partial sum fits int64 for < 2**27 terms
        s2 = 0
        for chunk in range(0, ms.size, 1 << 26):
            h = hi[chunk:chunk + (1 << 26)]
            l = lo[chunk:chunk + (1 << 26)]
            s2 += (int((h * h).sum()) << 24) + (int((2 * h * l).sum()) << 12) + int((l * l).sum())
        total += s1 << int(ee)          # sum * 2**150
        total_sq += s2 << (2 * int(ee))  # sum_sq * 2**300
    s = _int_ratio_to_f64(total, 150)
    ss = _int_ratio_to_f64(total_sq, 300)
    return n, s, ss, float(v.max())


def _int_ratio_to_f64(num: int, shift: int) -> float:
    """Correctly rounded num / 2**shift (Python's int/int true division is correctly rounded)."""
    return num / (1 << shift)


def stats_from_sums(count: int, s: float, ss: float, mx: float):
    """The reference's mean / SD formulas (metrics.rs:232-241) on given f64 sums."""
    c = float(count)
    mean = s / c
    centered = (c * ss - s * s) / c
    sd = math.sqrt(centered / (c - 1.0)) if (count > 1 and centered > 0.0) else 0.0
    return mean, sd, mx
