"""GPU paths that the benchmark specimens do not reach, against the oracle.
Marked gpu.

* The per-ball atomic-max sphere fill (lt.cu fill_kernel), which replaces the
  tile fill when a squared distance exceeds 65536 (a ball of radius above 256
  voxels), when there are 65535 or more distinct r^2 values, or when the
  (ball, tile) work list would exceed 2^32 entries: local_thickness.rs:169-202.
* The bounded mbarrier wait of the TMA-staged y pass: with the context's wait
  limit at 0 cycles every block gives up at once, records the timeout, drains
  its copy and returns; the call reports BM_ERR_TIMEOUT and the next call on
  the same context is exact (edt.rs:61-66 for the status-code style).
"""

import numpy as np
import pytest

import oracle as O
from refstats import assert_reference_stats
from bone_morphometry_gb300 import (BoneMorphometryError, Phase, _lib, analyze_thickness,
                                    euclidean_distance_transform_squared, local_thickness)

pytestmark = pytest.mark.gpu

# (shape (d, h, w), non-selected voxels (z, y, x)): far sites, r^2 above 65536
FAR_CASES = [
    ((2, 3, 600), [(0, 0, 0)]),
    ((3, 4, 530), [(0, 0, 0), (2, 3, 529)]),
    ((4, 5, 1100), [(1, 2, 0), (3, 4, 700), (0, 0, 1099)]),
    ((3, 300, 300), [(1, 0, 0)]),
]


@pytest.mark.parametrize("shape,sites", FAR_CASES)
@pytest.mark.parametrize("phase", [Phase.FOREGROUND, Phase.BACKGROUND])
def test_scatter_fill_fallback_bitwise(gpu_ctx, shape, sites, phase):
    vol = np.full(shape, 1 if phase == Phase.FOREGROUND else 0, np.uint8)
    for z, y, x in sites:
        vol[z, y, x] = 0 if phase == Phase.FOREGROUND else 255
    ref = O.local_thickness(vol, int(phase))
    assert int(ref.edt.max()) > 65536  # the tile fill's limit: this case takes the fallback
    gpu_ctx.profile(True)
    got, sq = local_thickness(vol, phase, ctx=gpu_ctx, return_squared=True)
    times = gpu_ctx.kernel_times()
    gpu_ctx.profile(False)
    # the fallback paints every voxel itself: no site kernel or chain pass ran
    assert times["fill"][0] == 1 and times["fill_sites"][0] == 0
    assert np.array_equal(sq, ref.propagated)
    assert np.array_equal(got.view(np.uint32), ref.thickness.view(np.uint32))


def test_scatter_fill_fallback_tbth_tbsp(gpu_ctx):
    """Tb.Sp of a specimen with a marrow cavity wider than 512 voxels."""
    d, h, w = 3, 40, 700
    bone = np.zeros((d, h, w), np.uint8)
    bone[:, :, :4] = 255
    bone[1, 20, 350] = 255
    roi = np.ones((d, h, w), np.uint8)
    res = analyze_thickness(bone, roi, 12.5, ctx=gpu_ctx, return_maps=True)
    for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
        ref = O.local_thickness(O.phase_inside(bone, roi, sel), O.FOREGROUND)
        assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
        assert_reference_stats(got, ref.thickness, 12.5)


def test_tma_wait_timeout_reports_and_recovers(gpu_ctx):
    rng = np.random.default_rng(77)
    vol = ((rng.random((40, 64, 64)) < 0.7) * 255).astype(np.uint8)  # width 64: the TMA-staged y pass
    gpu_ctx.set_wait_cycles(0)
    try:
        with pytest.raises(BoneMorphometryError) as ei:
            euclidean_distance_transform_squared(vol, ctx=gpu_ctx)
        assert ei.value.status == _lib.BM_ERR_TIMEOUT
        assert "bounded device-side wait" in str(ei.value)
        with pytest.raises(BoneMorphometryError) as ei:
            local_thickness(vol, ctx=gpu_ctx)
        assert ei.value.status == _lib.BM_ERR_TIMEOUT
    finally:
        gpu_ctx.set_wait_cycles(-1)
    # the same context, the default limit: exact again
    assert np.array_equal(euclidean_distance_transform_squared(vol, ctx=gpu_ctx), O.edt_sq(vol))
    got, sq = local_thickness(vol, ctx=gpu_ctx, return_squared=True)
    ref = O.local_thickness(vol, O.FOREGROUND)
    assert np.array_equal(sq, ref.propagated)
    assert np.array_equal(got.view(np.uint32), ref.thickness.view(np.uint32))
