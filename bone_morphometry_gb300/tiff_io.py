"""TIFF stacks into host buffers (tiff_io.rs:19-149) through the library's
native decoder (`bm_tiff_read`).

`read_binary_tiff(path, threshold, strict_binary)` and `read_roi_tiff(path)`
mirror the reference's functions: every page must be 8-bit grayscale with the
first page's dimensions, samples are validated (strict binary: 0 or 255; ROI
masks: 0, 1 or 255) and the volume holds (sample > threshold) as 0/1.  With
`pinned=True` the voxels are decoded straight into page-locked host memory
(a torch tensor) so that they can be copied to the GPU without staging.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from ._lib import BoneMorphometryError, last_error, load
from .api import BinaryVolume

TIFF_ANY, TIFF_ZERO_OR_255, TIFF_ROI_MASK = 0, 1, 2


def _read(path, threshold: int, accepted: int, pinned: bool) -> BinaryVolume:
    lib = load()
    p = os.fsencode(os.fspath(path))
    w, h, d = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    st = lib.bm_tiff_read(p, int(threshold), accepted, None, 0, ctypes.byref(w), ctypes.byref(h), ctypes.byref(d))
    if st != 0:
        raise BoneMorphometryError(st, last_error(None))
    n = w.value * h.value * d.value
    if pinned:
        import torch

        holder = torch.empty(n, dtype=torch.uint8, pin_memory=True)
        arr = holder.numpy()
    else:
        holder = None
        arr = np.empty(n, np.uint8)
    st = lib.bm_tiff_read(p, int(threshold), accepted, arr.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(w),
                          ctypes.byref(h), ctypes.byref(d))
    if st != 0:
        raise BoneMorphometryError(st, last_error(None))
    vol = BinaryVolume(arr, w.value, h.value, d.value)
    vol.pinned_storage = holder  # keeps the page-locked allocation alive with the volume
    return vol


def read_binary_tiff(path, threshold: int = 0, strict_binary: bool = False, pinned: bool = False) -> BinaryVolume:
    """tiff_io.rs:19-26: u8(sample > threshold); strict_binary requires samples 0 or 255."""
    return _read(path, threshold, TIFF_ZERO_OR_255 if strict_binary else TIFF_ANY, pinned)


def read_roi_tiff(path, pinned: bool = False) -> BinaryVolume:
    """tiff_io.rs:28-31: ROI encodings 0/1 or 0/255, stored as u8(sample > 0)."""
    return _read(path, 0, TIFF_ROI_MASK, pinned)
