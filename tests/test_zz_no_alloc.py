"""The no-allocation EDT entry point (bm_edt_sq_device_noalloc).

Callers that cannot call cudaMalloc -- a fixed device-memory budget owned by
their own pool allocator, a footprint that must not grow after start-up, an
embedding whose allocator they do not control -- use this variant: its scratch
is a static 32 MiB device array instead of context buffers.  These tests call
it through the C ABI and check it against the existing entry point
(bm_edt_sq_device) on two calls in a row, bit for bit (integer output, so the
tolerance is zero), and the second call's map against the CPU oracle.  The file name makes pytest collect it last.
"""

import ctypes

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc_edt(vol_t, phase, out_t):
    import torch

    lib = _lib.load()
    d, h, w = vol_t.shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.bm_edt_sq_device_noalloc(ctypes.c_void_p(vol_t.data_ptr()), w, h, d, int(phase),
                                        ctypes.c_void_p(out_t.data_ptr()), stream)


def _existing_edt(ctx, vol_t, phase):
    import torch

    d, h, w = vol_t.shape
    out = torch.empty(vol_t.shape, dtype=torch.int32, device=vol_t.device)
    ctx.call("bm_edt_sq_device", ctypes.c_void_p(vol_t.data_ptr()), w, h, d, int(phase),
             ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return out


def test_noalloc_matches_existing_entry_point_two_calls(gpu_ctx):
    import torch

    rng = np.random.default_rng(2024)
    # first call on a larger volume, second on a smaller one: the second must not
    # see anything the first left behind in the shared array
    cases = [((128, 128, 128), 0.6, 0), ((37, 53, 61), 0.9, 1)]
    for shape, p, phase in cases:
        vol = torch.from_numpy(((rng.random(shape) < p) * 255).astype(np.uint8)).cuda()
        out = torch.full(shape, -1, dtype=torch.int32, device="cuda")
        st = _noalloc_edt(vol, phase, out)
        assert st == _lib.BM_OK, _lib.last_error(None)
        ref = _existing_edt(gpu_ctx, vol, phase)
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    # the second call's map also against the oracle directly
    assert np.array_equal(out.cpu().numpy().view(np.uint32), O.edt_sq(vol.cpu().numpy(), phase))


def test_noalloc_rejects_oversized_volume():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vol = torch.zeros((2, 2, 2), dtype=torch.uint8, device="cuda")  # pointer only; sizes are checked first
    out = torch.zeros((2, 2, 2), dtype=torch.int32, device="cuda")
    lib = _lib.load()
    st = lib.bm_edt_sq_device_noalloc(ctypes.c_void_p(vol.data_ptr()), 256, 256, 256, 0,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert st == _lib.BM_ERR_DIMS
    assert "no-allocation EDT holds" in _lib.last_error(None)


def test_noalloc_all_selected_error():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vol = torch.full((5, 6, 7), 255, dtype=torch.uint8, device="cuda")
    out = torch.empty((5, 6, 7), dtype=torch.int32, device="cuda")
    st = _noalloc_edt(vol, 0, out)
    assert st == _lib.BM_ERR_ALL_SELECTED
    assert "all-foreground" in _lib.last_error(None)
