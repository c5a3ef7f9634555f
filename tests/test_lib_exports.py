"""The C-ABI library builds, loads and exports every symbol include/bm.h declares
(no compute call: this runs on machines without a GPU)."""

import ctypes
import os
import re

from bone_morphometry_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "bm.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("bm_edt_sq", "bm_local_thickness", "bm_tbth_tbsp", "bm_ctx_create", "bm_last_error"):
        assert name in syms


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_status_strings_without_device():
    lib = _lib.load()
    assert lib.bm_status_string(0) == b"ok"
    assert lib.bm_status_string(1) == b"all voxels selected"


def test_create_without_gpu_fails_loudly():
    import torch

    if torch.cuda.is_available():
        return
    lib = _lib.load()
    h = ctypes.c_void_p()
    st = lib.bm_ctx_create(0, ctypes.byref(h))
    assert st == _lib.BM_ERR_NO_DEVICE
    assert "no CUDA device" in _lib.last_error(None)
