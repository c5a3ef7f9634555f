"""Python mirror of the reference's interface for the Tb.Th / Tb.Sp path.

Names, argument meaning and errors follow the Rust modules they replace:

* ``BinaryVolume`` / ``phase_inside``          -- volume.rs:4-105
* ``Phase``                                     -- edt.rs:8-32
* ``euclidean_distance_transform_squared``      -- edt.rs:57-156
* ``local_thickness``                           -- local_thickness.rs:16-44
* ``analyze_thickness`` (the Tb.Th / Tb.Sp part of ``analyze``) -- metrics.rs:64-121
* ``DistributionStats``                         -- metrics.rs:27-38

Every computation runs in libbm_gb300.so on the GPU through the C ABI of
include/bm.h; numpy arrays are host buffers (the host-pointer entry points
copy them in and out), torch CUDA tensors are passed as device pointers.
Errors are raised as ``BoneMorphometryError`` carrying the reference's
message text.
"""

from __future__ import annotations

import ctypes
import enum
import math
from dataclasses import dataclass

import numpy as np

from ._lib import (BM_ERR_DIMS, BM_ERR_INVALID, BM_FLAG_BONEJ_ROI, BM_FLAG_QUANTILES, BmStats, BmVolumeMetrics,
                   BoneMorphometryError, Context, default_context)


class Phase(enum.IntEnum):
    """edt.rs:8-24: Foreground selects value != 0, Background selects value == 0."""

    FOREGROUND = 0
    BACKGROUND = 1

    def is_selected(self, value: int) -> bool:
        return value != 0 if self is Phase.FOREGROUND else value == 0


class FeatureMode(enum.Enum):
    """metrics.rs:12-24.  Only the effect on Tb.Th / Tb.Sp is modelled: quantiles
    are computed in Standard and Experimental, Bonej rejects an ROI without
    outside voxels (metrics.rs:93-95, 106-109)."""

    BONEJ = "bonej"
    STANDARD = "standard"
    CLASSIC = "classic"
    REFINED = "refined"
    EXPERIMENTAL = "experimental"


class BinaryVolume:
    """Dense u8 volume, x fastest: index = (z*height + y)*width + x (volume.rs:4-46)."""

    def __init__(self, data, width: int, height: int, depth: int):
        arr = np.ascontiguousarray(np.asarray(data, dtype=np.uint8)).reshape(-1)
        expected = int(width) * int(height) * int(depth)
        if arr.size != expected:
            raise BoneMorphometryError(
                BM_ERR_DIMS, "volume has %d voxels, but dimensions %dx%dx%d require %d"
                % (arr.size, width, height, depth, expected))
        if width < 2 or height < 2 or depth < 2:
            raise BoneMorphometryError(
                BM_ERR_DIMS, "all dimensions must be at least 2 for 3-D morphometry; got %dx%dx%d"
                % (width, height, depth))
        self.data = arr
        self.width, self.height, self.depth = int(width), int(height), int(depth)

    @classmethod
    def from_array(cls, arr: np.ndarray) -> "BinaryVolume":
        d, h, w = arr.shape
        return cls(arr, w, h, d)

    @property
    def shape(self):
        return (self.depth, self.height, self.width)

    def array(self) -> np.ndarray:
        return self.data.reshape(self.shape)

    def index(self, x: int, y: int, z: int) -> int:
        return (z * self.height + y) * self.width + x

    def __len__(self) -> int:
        return self.data.size

    def slice_len(self) -> int:
        return self.width * self.height

    def same_shape(self, other: "BinaryVolume") -> bool:
        return (self.width, self.height, self.depth) == (other.width, other.height, other.depth)

    def phase_inside(self, roi: "BinaryVolume", select_bone: bool) -> "BinaryVolume":
        """volume.rs:84-105.  A host-side convenience; the GPU path fuses this
        selection into its first EDT pass instead of materialising it."""
        if not self.same_shape(roi):
            raise BoneMorphometryError(
                BM_ERR_INVALID, "binary image dimensions %dx%dx%d do not match ROI dimensions %dx%dx%d"
                % (self.width, self.height, self.depth, roi.width, roi.height, roi.depth))
        data = ((roi.data != 0) & ((self.data != 0) == bool(select_bone))).astype(np.uint8)
        return BinaryVolume(data, self.width, self.height, self.depth)


def _as_volume(volume) -> BinaryVolume:
    if isinstance(volume, BinaryVolume):
        return volume
    arr = np.asarray(volume)
    if arr.ndim != 3:
        raise BoneMorphometryError(BM_ERR_INVALID, "expected a BinaryVolume or a (depth, height, width) array")
    return BinaryVolume.from_array(arr)


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and bool(getattr(x, "is_cuda"))


def _tensor_dims(t):
    if t.dim() != 3:
        raise BoneMorphometryError(BM_ERR_INVALID, "expected a (depth, height, width) tensor")
    if not t.is_contiguous():
        raise BoneMorphometryError(BM_ERR_INVALID, "tensor must be contiguous")
    d, h, w = t.shape
    return int(w), int(h), int(d)


def _stream_ptr(t):
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def euclidean_distance_transform_squared(volume, phase: Phase = Phase.FOREGROUND, ctx: Context | None = None):
    """edt.rs:57-156: exact squared EDT of the selected phase (u32), 0 on non-selected voxels.

    ``volume`` is a BinaryVolume / numpy array (result: numpy u32, same shape) or a
    CUDA uint8 tensor (result: CUDA int32 tensor holding the u32 bit patterns)."""
    ctx = ctx or default_context()
    if _is_cuda_tensor(volume):
        import torch

        w, h, d = _tensor_dims(volume)
        out = torch.empty_like(volume, dtype=torch.int32)
        ctx.call("bm_edt_sq_device", ctypes.c_void_p(volume.data_ptr()), w, h, d, int(phase),
                 ctypes.c_void_p(out.data_ptr()), _stream_ptr(volume))
        return out
    vol = _as_volume(volume)
    out = np.empty(vol.shape, np.uint32)
    ctx.call("bm_edt_sq", _ptr(vol.data), vol.width, vol.height, vol.depth, int(phase), _ptr(out))
    return out


def local_thickness(volume, phase: Phase = Phase.FOREGROUND, ctx: Context | None = None,
                    return_squared: bool = False):
    """local_thickness.rs:16-44: local thickness (diameter, voxel units, f32), 0 off-phase.

    With ``return_squared`` also returns the propagated u32 squared-thickness map."""
    ctx = ctx or default_context()
    if _is_cuda_tensor(volume):
        import torch

        w, h, d = _tensor_dims(volume)
        out = torch.empty(volume.shape, dtype=torch.float32, device=volume.device)
        sq = torch.empty(volume.shape, dtype=torch.int32, device=volume.device) if return_squared else None
        ctx.call("bm_local_thickness_device", ctypes.c_void_p(volume.data_ptr()), w, h, d, int(phase),
                 ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(sq.data_ptr() if sq is not None else 0),
                 _stream_ptr(volume))
        return (out, sq) if return_squared else out
    vol = _as_volume(volume)
    out = np.empty(vol.shape, np.float32)
    sq = np.empty(vol.shape, np.uint32) if return_squared else None
    ctx.call("bm_local_thickness", _ptr(vol.data), vol.width, vol.height, vol.depth, int(phase), _ptr(out),
             _ptr(sq) if sq is not None else ctypes.c_void_p(0))
    return (out, sq) if return_squared else out


@dataclass
class DistributionStats:
    """metrics.rs:27-38, micrometres.  Quantile fields are NaN unless requested.
    mean and standard_deviation come from the reference's own sequential sums
    (metrics.rs:215-241), reproduced bit for bit."""

    mean: float
    standard_deviation: float
    maximum: float
    median: float
    percentile_10: float
    percentile_25: float
    percentile_75: float
    percentile_90: float
    interquartile_range: float
    coefficient_of_variation: float
    count: int = 0
    sum: float = math.nan              # the reference's sequential f64 accumulators
    sum_of_squares: float = math.nan
    exact_sum: float = math.nan        # the same sums, exact, rounded once
    exact_sum_of_squares: float = math.nan

    @classmethod
    def from_c(cls, s: BmStats) -> "DistributionStats":
        return cls(s.mean, s.standard_deviation, s.maximum, s.median, s.percentile_10, s.percentile_25,
                   s.percentile_75, s.percentile_90, s.interquartile_range, s.coefficient_of_variation,
                   int(s.count), s.sum, s.sum_of_squares, s.exact_sum, s.exact_sum_of_squares)


@dataclass
class ThicknessMetrics:
    thickness: DistributionStats   # Tb.Th
    spacing: DistributionStats     # Tb.Sp
    thickness_map: object = None   # optional f32 diameter maps (voxel units)
    spacing_map: object = None


def nonzero_stats(values, scale: float, include_quantiles: bool = False, ctx: Context | None = None
                  ) -> DistributionStats:
    """metrics.rs:204-269 on an f32 map (numpy array or CUDA float32 tensor)."""
    ctx = ctx or default_context()
    out = BmStats()
    flags = BM_FLAG_QUANTILES if include_quantiles else 0
    if _is_cuda_tensor(values):
        import torch

        if values.dtype != torch.float32 or not values.is_contiguous():
            raise BoneMorphometryError(BM_ERR_INVALID, "expected a contiguous float32 tensor")
        ctx.call("bm_nonzero_stats_device", ctypes.c_void_p(values.data_ptr()), values.numel(), float(scale), flags,
                 ctypes.byref(out), _stream_ptr(values))
    else:
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float32)).reshape(-1)
        ctx.call("bm_nonzero_stats", _ptr(v), v.size, float(scale), flags, ctypes.byref(out))
    return DistributionStats.from_c(out)


@dataclass
class VolumeMetrics:
    """metrics.rs:123-132 and 166-202."""

    bone_voxels: int
    roi_voxels: int
    boundary_bone_voxels: int
    bone_volume: float
    total_volume: float
    bone_volume_fraction: float
    roi_boundary_bone_fraction: float


def volume_metrics(bone, roi, voxel_spacing, ctx: Context | None = None) -> VolumeMetrics:
    """BV, TV, BV/TV and the ROI-boundary bone fraction of one specimen."""
    ctx = ctx or default_context()
    if isinstance(voxel_spacing, (int, float)):
        voxel_spacing = (float(voxel_spacing),) * 3
    sp = (ctypes.c_double * 3)(*[float(v) for v in voxel_spacing])
    out = BmVolumeMetrics()
    if _is_cuda_tensor(bone):
        w, h, d = _tensor_dims(bone)
        ctx.call("bm_volume_metrics_device", ctypes.c_void_p(bone.data_ptr()), ctypes.c_void_p(roi.data_ptr()),
                 w, h, d, sp, ctypes.byref(out), _stream_ptr(bone))
    else:
        b, r = _as_volume(bone), _as_volume(roi)
        if not b.same_shape(r):
            raise BoneMorphometryError(BM_ERR_INVALID, "binary image dimensions do not match ROI dimensions")
        ctx.call("bm_volume_metrics_compute", _ptr(b.data), _ptr(r.data), b.width, b.height, b.depth, sp,
                 ctypes.byref(out))
    return VolumeMetrics(int(out.bone_voxels), int(out.roi_voxels), int(out.boundary_bone_voxels), out.bone_volume,
                         out.total_volume, out.bone_volume_fraction, out.roi_boundary_bone_fraction)


def _flags(feature_mode) -> int:
    fm = FeatureMode(feature_mode) if not isinstance(feature_mode, FeatureMode) else feature_mode
    flags = 0
    if fm in (FeatureMode.STANDARD, FeatureMode.EXPERIMENTAL):
        flags |= BM_FLAG_QUANTILES
    if fm is FeatureMode.BONEJ:
        flags |= BM_FLAG_BONEJ_ROI
    return flags


def analyze_thickness(bone, roi, voxel_spacing, feature_mode=FeatureMode.CLASSIC, ctx: Context | None = None,
                      return_maps: bool = False) -> ThicknessMetrics:
    """Tb.Th and Tb.Sp of one specimen: metrics.rs:64-121 (bails, phase build, two
    local-thickness maps, nonzero_stats scaled by voxel_spacing[0])."""
    ctx = ctx or default_context()
    if isinstance(voxel_spacing, (int, float)):
        voxel_spacing = (float(voxel_spacing),) * 3
    sp = [float(v) for v in voxel_spacing]
    if any((not math.isfinite(v)) or v <= 0.0 for v in sp):
        from ._lib import BM_ERR_SPACING

        raise BoneMorphometryError(BM_ERR_SPACING, "voxel spacings must be finite and positive; got %r" % (sp,))
    flags = _flags(feature_mode)
    th, spc = BmStats(), BmStats()
    if _is_cuda_tensor(bone):
        import torch

        w, h, d = _tensor_dims(bone)
        if tuple(roi.shape) != tuple(bone.shape):
            raise BoneMorphometryError(BM_ERR_INVALID, "binary image dimensions do not match ROI dimensions")
        tm = torch.empty(bone.shape, dtype=torch.float32, device=bone.device) if return_maps else None
        sm = torch.empty(bone.shape, dtype=torch.float32, device=bone.device) if return_maps else None
        ctx.call("bm_tbth_tbsp_device", ctypes.c_void_p(bone.data_ptr()), ctypes.c_void_p(roi.data_ptr()), w, h, d,
                 sp[0], flags, ctypes.byref(th), ctypes.byref(spc),
                 ctypes.c_void_p(tm.data_ptr() if tm is not None else 0),
                 ctypes.c_void_p(sm.data_ptr() if sm is not None else 0), _stream_ptr(bone))
        return ThicknessMetrics(DistributionStats.from_c(th), DistributionStats.from_c(spc), tm, sm)
    b = _as_volume(bone)
    r = _as_volume(roi)
    if not b.same_shape(r):
        raise BoneMorphometryError(
            BM_ERR_INVALID, "binary image dimensions %dx%dx%d do not match ROI dimensions %dx%dx%d"
            % (b.width, b.height, b.depth, r.width, r.height, r.depth))
    tm = np.empty(b.shape, np.float32) if return_maps else None
    sm = np.empty(b.shape, np.float32) if return_maps else None
    ctx.call("bm_tbth_tbsp", _ptr(b.data), _ptr(r.data), b.width, b.height, b.depth, sp[0], flags,
             ctypes.byref(th), ctypes.byref(spc), _ptr(tm) if tm is not None else ctypes.c_void_p(0),
             _ptr(sm) if sm is not None else ctypes.c_void_p(0))
    return ThicknessMetrics(DistributionStats.from_c(th), DistributionStats.from_c(spc), tm, sm)
