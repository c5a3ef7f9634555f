"""ctypes binding of libbm_gb300.so (the C ABI declared in include/bm.h).

The library is loaded from this package's in-tree ``_build/`` directory.  If it
is missing it is built with nvcc; if that is impossible, or no CUDA device is
present, calls raise ``BoneMorphometryError`` -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

BM_OK = 0
BM_SITES_AUTO, BM_SITES_SPHERES, BM_SITES_CHAINS = 0, 1, 2
BM_ERR_ALL_SELECTED = 1
BM_ERR_DIMS = 2
BM_ERR_OOM = 3
BM_ERR_CUDA = 4
BM_ERR_TIMEOUT = 5
BM_ERR_INVALID = 6
BM_ERR_EMPTY = 7
BM_ERR_ROI_EMPTY = 8
BM_ERR_NO_BONE = 9
BM_ERR_NO_MARROW = 10
BM_ERR_NO_DEVICE = 11
BM_ERR_SPACING = 12
BM_ERR_ROI_FULL = 13
BM_ERR_BUSY = 14

BM_FLAG_QUANTILES = 1
BM_FLAG_BONEJ_ROI = 2


class BoneMorphometryError(RuntimeError):
    """A non-zero bm_status from the library, with the reference's message text."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class BmKernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double)]


class BmStats(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_uint64),
        ("mean", ctypes.c_double),
        ("standard_deviation", ctypes.c_double),
        ("maximum", ctypes.c_double),
        ("median", ctypes.c_double),
        ("percentile_10", ctypes.c_double),
        ("percentile_25", ctypes.c_double),
        ("percentile_75", ctypes.c_double),
        ("percentile_90", ctypes.c_double),
        ("interquartile_range", ctypes.c_double),
        ("coefficient_of_variation", ctypes.c_double),
        ("sum", ctypes.c_double),
        ("sum_of_squares", ctypes.c_double),
        ("exact_sum", ctypes.c_double),
        ("exact_sum_of_squares", ctypes.c_double),
    ]


class BmVolumeMetrics(ctypes.Structure):
    _fields_ = [
        ("bone_voxels", ctypes.c_uint64),
        ("roi_voxels", ctypes.c_uint64),
        ("boundary_bone_voxels", ctypes.c_uint64),
        ("bone_volume", ctypes.c_double),
        ("total_volume", ctypes.c_double),
        ("bone_volume_fraction", ctypes.c_double),
        ("roi_boundary_bone_fraction", ctypes.c_double),
    ]


class BmSpecimen(ctypes.Structure):
    _fields_ = [("bone", ctypes.c_void_p), ("roi", ctypes.c_void_p), ("width", ctypes.c_size_t),
                ("height", ctypes.c_size_t), ("depth", ctypes.c_size_t), ("spacing_um", ctypes.c_double)]


class BmResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("thickness", BmStats), ("spacing", BmStats), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("end_s", ctypes.c_double), ("footprint_bytes", ctypes.c_uint64),
                ("message", ctypes.c_char * 256)]


# name -> (restype, argtypes); every symbol declared in include/bm.h
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_i = ctypes.c_int
_u = ctypes.c_uint
_d = ctypes.c_double
_pctx = ctypes.c_void_p
_u8p = ctypes.c_void_p
SIGNATURES = {
    "bm_ctx_create": (_i, [_i, ctypes.POINTER(ctypes.c_void_p)]),
    "bm_ctx_destroy": (None, [_pctx]),
    "bm_status_string": (ctypes.c_char_p, [_i]),
    "bm_last_error": (_sz, [_pctx, ctypes.c_char_p, _sz]),
    "bm_ctx_trim": (_i, [_pctx]),
    "bm_edt_sq": (_i, [_pctx, _u8p, _sz, _sz, _sz, _i, _vp]),
    "bm_local_thickness": (_i, [_pctx, _u8p, _sz, _sz, _sz, _i, _vp, _vp]),
    "bm_tbth_tbsp": (_i, [_pctx, _u8p, _u8p, _sz, _sz, _sz, _d, _u, ctypes.POINTER(BmStats),
                          ctypes.POINTER(BmStats), _vp, _vp]),
    "bm_edt_sq_device": (_i, [_pctx, _u8p, _sz, _sz, _sz, _i, _vp, _vp]),
    "bm_local_thickness_device": (_i, [_pctx, _u8p, _sz, _sz, _sz, _i, _vp, _vp, _vp]),
    "bm_tbth_tbsp_device": (_i, [_pctx, _u8p, _u8p, _sz, _sz, _sz, _d, _u, ctypes.POINTER(BmStats),
                                 ctypes.POINTER(BmStats), _vp, _vp, _vp]),
    "bm_ctx_launch_count": (ctypes.c_uint64, [_pctx]),
    "bm_profile_enable": (_i, [_pctx, _i]),
    "bm_profile_read": (_i, [_pctx, _vp, _sz, ctypes.POINTER(_sz)]),
    "bm_edt_sq_device_noalloc": (_i, [_u8p, _sz, _sz, _sz, _i, _vp, _vp]),
    "bm_nonzero_stats": (_i, [_pctx, _vp, _sz, _d, _u, ctypes.POINTER(BmStats)]),
    "bm_nonzero_stats_device": (_i, [_pctx, _vp, _sz, _d, _u, ctypes.POINTER(BmStats), _vp]),
    "bm_volume_metrics_compute": (_i, [_pctx, _u8p, _u8p, _sz, _sz, _sz, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(BmVolumeMetrics)]),
    "bm_volume_metrics_device": (_i, [_pctx, _u8p, _u8p, _sz, _sz, _sz, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(BmVolumeMetrics), _vp]),
    "bm_batch_tbth_tbsp": (_i, [_pctx, ctypes.POINTER(BmSpecimen), _sz, _i, _u, ctypes.POINTER(BmStats),
                                ctypes.POINTER(BmStats), ctypes.POINTER(ctypes.c_int)]),
    "bm_ctx_set_workers": (_i, [_pctx, _i]),
    "bm_server_create": (_i, [_i, _i, _d, ctypes.POINTER(ctypes.c_void_p)]),
    "bm_server_submit": (_i, [_vp, ctypes.POINTER(BmSpecimen), _u, ctypes.POINTER(ctypes.c_uint64)]),
    "bm_server_submit_tiff": (_i, [_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint, _i, _d, _u,
                                   ctypes.POINTER(ctypes.c_uint64)]),
    "bm_server_poll": (_i, [_vp, ctypes.c_uint64, _i, ctypes.POINTER(BmResult)]),
    "bm_server_stats": (_i, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.c_double)]),
    "bm_server_destroy": (None, [_vp]),
    "bm_footprint_bytes": (ctypes.c_uint64, [_sz, _sz, _sz]),
    "bm_ctx_set_concurrent_phases": (_i, [_vp, _i]),
    "bm_ctx_set_site_method": (_i, [_vp, _i]),
    "bm_ctx_set_fill_tile_rows": (_i, [_vp, _i]),
    "bm_ctx_set_wait_cycles": (_i, [_vp, ctypes.c_longlong]),
    "bm_tiff_read": (_i, [ctypes.c_char_p, ctypes.c_uint, _i, _vp, _sz, ctypes.POINTER(_sz), ctypes.POINTER(_sz),
                          ctypes.POINTER(_sz)]),
}

_LIB = None
_LOCK = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load() -> ctypes.CDLL:
    """Load (building in-tree if absent) libbm_gb300.so and declare its signatures."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if not os.path.exists(path):
            try:
                path = _build.build()
            except Exception as exc:  # no nvcc / compile error: fail loudly
                raise BoneMorphometryError(BM_ERR_NO_DEVICE,
                                           "libbm_gb300.so is missing and could not be built: %s" % exc)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def last_error(ctx) -> str:
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.bm_last_error(ctx, buf, len(buf))
    return buf.value.decode("utf-8", "replace")


def raise_for(status: int, ctx) -> None:
    if status != BM_OK:
        msg = last_error(ctx) or load().bm_status_string(status).decode()
        raise BoneMorphometryError(status, msg)


class Context:
    """Owns one bm_ctx (device, stream, cached buffers and template table)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = ctypes.c_void_p()
        st = lib.bm_ctx_create(int(device), ctypes.byref(h))
        if st != BM_OK:
            raise BoneMorphometryError(st, last_error(None) or lib.bm_status_string(st).decode())
        self.handle = h
        self.device = device
        self._lib = lib

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.bm_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self._lib.bm_ctx_launch_count(self.handle))

    def profile(self, on: bool = True) -> None:
        """Start (clearing totals) or stop CUDA-event timing of library kernels."""
        self.call("bm_profile_enable", 1 if on else 0)

    def set_concurrent_phases(self, on: bool = True) -> None:
        """Tb.Th and Tb.Sp side by side on two streams (default) or one after the other."""
        self.call("bm_ctx_set_concurrent_phases", 1 if on else 0)

    def set_site_method(self, method: int = 0) -> None:
        """How the fill finds the non-selected voxels ridge spheres reach:
        BM_SITES_AUTO (0), BM_SITES_SPHERES (1) or BM_SITES_CHAINS (2)."""
        self.call("bm_ctx_set_site_method", int(method))

    def set_fill_tile_rows(self, rows: int = 0) -> None:
        """Rows of y in the sphere fill's tiles: 0 (by volume size), 16, 32 or 64."""
        self.call("bm_ctx_set_fill_tile_rows", int(rows))

    def set_wait_cycles(self, cycles: int = -1) -> None:
        """Cycle limit of the device-side bounded waits (-1: the default, ~2 s;
        0: give up at once, to exercise the timeout path)."""
        self.call("bm_ctx_set_wait_cycles", int(cycles))

    def kernel_times(self) -> dict:
        """{family: (launches, total_ms)} of the kernels timed since profile(True)."""
        arr = (BmKernelTime * 32)()
        n = ctypes.c_size_t(0)
        self.call("bm_profile_read", ctypes.cast(arr, ctypes.c_void_p), 32, ctypes.byref(n))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(min(n.value, 32))}

    def call(self, name: str, *args) -> None:
        st = getattr(self._lib, name)(self.handle, *args)
        raise_for(st, self.handle)


_DEFAULT = {}


def default_context(device: int = 0) -> Context:
    ctx = _DEFAULT.get(device)
    if ctx is None or ctx.handle is None:
        ctx = Context(device)
        _DEFAULT[device] = ctx
    return ctx
