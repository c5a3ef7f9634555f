"""Tb.Th / Tb.Sp from host inputs of at least 2^22 voxels: bone and ROI are
uploaded in slabs of planes on a copy stream, and each slab's ROI counts and x
and y passes start as soon as it has landed (metrics.rs:90-121 for the bails
and the two phases).  The results must equal those of the device-pointer path,
bit for bit, maps included, whether the phases run side by side or one after
the other; the bails must still be reported; and the context must stay usable
after one.  Marked gpu."""

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import BoneMorphometryError, Context, analyze_thickness
from bone_morphometry_gb300 import synthetic as S
from refstats import assert_reference_stats

pytestmark = pytest.mark.gpu

# (d, h, w): a width that takes the 16-voxel x pass and the TMA y pass (640), and
# one that takes neither (173); depths that do not split evenly into 8 slabs
SHAPES = [(37, 181, 640), (151, 167, 173)]


def specimen(shape, seed):
    return S.make_specimen(shape, 3.0, 0.25, "cylinder", 0.45 * min(shape[1], shape[2]), 14.5, seed)


def same(a, b):
    assert a.count == b.count
    assert a.mean == b.mean and a.standard_deviation == b.standard_deviation and a.maximum == b.maximum
    assert a.exact_sum == b.exact_sum and a.exact_sum_of_squares == b.exact_sum_of_squares


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("side_by_side", [True, False])
def test_host_upload_pipeline_equals_device_path(shape, side_by_side):
    import torch

    assert int(np.prod(shape)) >= 1 << 22
    sp = specimen(shape, 17 + shape[2])
    ctx = Context()
    try:
        ctx.set_concurrent_phases(side_by_side)
        dev = analyze_thickness(torch.from_numpy(sp.bone).cuda(), torch.from_numpy(sp.roi).cuda(), sp.spacing_um,
                                ctx=ctx, return_maps=True)
        torch.cuda.synchronize()
        for _ in range(2):  # the second call reuses the copy stream, events and buffers
            host = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx, return_maps=True)
            same(host.thickness, dev.thickness)
            same(host.spacing, dev.spacing)
            assert np.array_equal(host.thickness_map.view(np.uint32),
                                  dev.thickness_map.cpu().numpy().view(np.uint32))
            assert np.array_equal(host.spacing_map.view(np.uint32), dev.spacing_map.cpu().numpy().view(np.uint32))
    finally:
        ctx.close()


def test_host_upload_pipeline_against_oracle():
    sp = specimen(SHAPES[0], 5)
    ctx = Context()
    try:
        res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx, return_maps=True)
    finally:
        ctx.close()
    for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
        ref = O.local_thickness(O.phase_inside(sp.bone, sp.roi, sel), O.FOREGROUND)
        assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
        assert_reference_stats(got, ref.thickness, sp.spacing_um)


def test_host_upload_pipeline_bails_and_recovers():
    """The bails of metrics.rs:90-104 come after every slab is counted; the
    passes that already ran leave the context usable."""
    shape = SHAPES[1]
    sp = specimen(shape, 9)
    ctx = Context()
    try:
        ref = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx)
        empty = np.zeros(shape, np.uint8)
        with pytest.raises(BoneMorphometryError, match="ROI mask contains no included voxels"):
            analyze_thickness(sp.bone, empty, sp.spacing_um, ctx=ctx)
        with pytest.raises(BoneMorphometryError, match="ROI contains no bone voxels"):
            analyze_thickness(empty, sp.roi, sp.spacing_um, ctx=ctx)
        solid = np.full(shape, 255, np.uint8)
        with pytest.raises(BoneMorphometryError, match="ROI contains no marrow voxels"):
            analyze_thickness(solid, sp.roi, sp.spacing_um, ctx=ctx)
        got = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=ctx)
        same(got.thickness, ref.thickness)
        same(got.spacing, ref.spacing)
    finally:
        ctx.close()
