"""GPU parity through the C ABI against the CPU oracle: bit-exact maps and
statistics identical to the reference's (its own sequential f64 sums).  Marked gpu."""

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import (BinaryVolume, BoneMorphometryError, Phase, analyze_thickness,
                                    euclidean_distance_transform_squared, local_thickness)
from bone_morphometry_gb300 import _lib
from bone_morphometry_gb300 import synthetic as S

from refstats import assert_reference_stats

pytestmark = pytest.mark.gpu


def rand_volume(shape, p, seed):
    rng = np.random.default_rng(seed)
    return (rng.random(shape) < p).astype(np.uint8) * np.uint8(255)


def blob_volume(shape, sigma, frac, seed):
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    f = gaussian_filter(rng.standard_normal(shape).astype(np.float32), sigma)
    thr = np.quantile(f, 1 - frac)
    return (f > thr).astype(np.uint8)


EDT_CASES = [
    ((3, 3, 3), 0.5, 1), ((2, 2, 2), 0.5, 2), ((5, 7, 11), 0.3, 3), ((33, 31, 65), 0.9, 4),
    ((17, 129, 40), 0.97, 5), ((64, 64, 64), 0.5, 6), ((2, 300, 3), 0.99, 7), ((41, 2, 257), 0.8, 8),
    ((16, 16, 1100), 0.995, 9), ((300, 200, 64), 0.999, 10), ((130, 140, 70), 0.98, 11),
    ((257, 129, 33), 0.7, 12),
    # widths that are multiples of 16 take the 16-voxels-per-lane x pass: an odd
    # number of 16-voxel groups (48), a single group (16), more than 32 groups (528)
    ((5, 9, 48), 0.6, 13), ((3, 4, 16), 0.5, 14), ((6, 10, 528), 0.9, 15),
]


@pytest.mark.parametrize("shape,p,seed", EDT_CASES)
@pytest.mark.parametrize("phase", [Phase.FOREGROUND, Phase.BACKGROUND])
def test_edt_bitwise(gpu_ctx, shape, p, seed, phase):
    vol = rand_volume(shape, p, seed)
    sel = vol != 0 if phase == Phase.FOREGROUND else vol == 0
    if sel.all():
        vol.flat[0] = 0 if phase == Phase.FOREGROUND else 255
    got = euclidean_distance_transform_squared(vol, phase, ctx=gpu_ctx)
    ref = O.edt_sq(vol, int(phase))
    assert np.array_equal(got, ref)


def test_edt_kat_center(gpu_ctx):
    # edt.rs:240-274
    data = np.ones((3, 3, 3), np.uint8)
    data[1, 1, 1] = 0
    e = euclidean_distance_transform_squared(data, Phase.FOREGROUND, ctx=gpu_ctx).ravel()
    assert e[13] == 0 and e[12] == 1 and e[0] == 3
    e = euclidean_distance_transform_squared(1 - data, Phase.BACKGROUND, ctx=gpu_ctx).ravel()
    assert e[13] == 0 and e[12] == 1 and e[0] == 3


def test_edt_single_site_far(gpu_ctx):
    vol = np.ones((40, 70, 90), np.uint8)
    vol[0, 0, 0] = 0
    assert np.array_equal(euclidean_distance_transform_squared(vol, ctx=gpu_ctx), O.edt_sq(vol))


def test_errors(gpu_ctx):
    with pytest.raises(BoneMorphometryError, match="all-foreground volume") as ei:
        euclidean_distance_transform_squared(np.ones((4, 4, 4), np.uint8), ctx=gpu_ctx)
    assert ei.value.status == _lib.BM_ERR_ALL_SELECTED
    with pytest.raises(BoneMorphometryError, match="all-background volume"):
        local_thickness(np.zeros((4, 4, 4), np.uint8), Phase.BACKGROUND, ctx=gpu_ctx)
    with pytest.raises(BoneMorphometryError, match="at least 2"):
        euclidean_distance_transform_squared(np.ones((1, 4, 4), np.uint8), ctx=gpu_ctx)
    bone = np.zeros((6, 6, 6), np.uint8)
    roi = np.zeros((6, 6, 6), np.uint8)
    with pytest.raises(BoneMorphometryError, match="ROI mask contains no included voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    roi[1:5, 1:5, 1:5] = 1
    with pytest.raises(BoneMorphometryError, match="ROI contains no bone voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    bone[:] = 255
    with pytest.raises(BoneMorphometryError, match="ROI contains no marrow voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    with pytest.raises(BoneMorphometryError, match="finite and positive"):
        analyze_thickness(bone, roi, float("nan"), ctx=gpu_ctx)
    with pytest.raises(BoneMorphometryError, match="site method must be"):
        gpu_ctx.set_site_method(3)
    # the context stays usable after errors
    vol = rand_volume((9, 9, 9), 0.5, 0)
    assert np.array_equal(euclidean_distance_transform_squared(vol, ctx=gpu_ctx), O.edt_sq(vol))


LT_CASES = [
    ("kat", None), ("rand", ((20, 21, 22), 0.6, 11)), ("rand", ((7, 40, 33), 0.3, 12)),
    ("blob", ((48, 40, 56), 2.0, 0.3, 13)), ("blob", ((64, 64, 64), 3.0, 0.7, 14)),
    ("blob", ((30, 90, 17), 1.5, 0.5, 15)),
]


@pytest.fixture(params=[_lib.BM_SITES_SPHERES, _lib.BM_SITES_CHAINS], ids=["spheres", "chains"])
def site_method(request, gpu_ctx):
    """Both ways of finding the non-selected voxels a ridge sphere reaches."""
    gpu_ctx.set_site_method(request.param)
    yield request.param
    gpu_ctx.set_site_method(_lib.BM_SITES_AUTO)


@pytest.mark.parametrize("kind,args", LT_CASES)
@pytest.mark.parametrize("phase", [Phase.FOREGROUND, Phase.BACKGROUND])
def test_local_thickness_bitwise(gpu_ctx, site_method, kind, args, phase):
    if kind == "kat":
        vol = np.zeros((3, 3, 3), np.uint8)
        vol[1, 1, 1] = 1
        if phase == Phase.BACKGROUND:
            vol = 1 - vol
    elif kind == "rand":
        vol = rand_volume(*args)
    else:
        vol = blob_volume(*args)
    ref = O.local_thickness(vol, int(phase))
    got, sq = local_thickness(vol, phase, ctx=gpu_ctx, return_squared=True)
    assert np.array_equal(sq, ref.propagated)
    assert np.array_equal(got.view(np.uint32), ref.thickness.view(np.uint32))


def test_local_thickness_huge_balls(gpu_ctx, site_method):
    # one site in a corner: r^2 up to ~3000, balls spanning many fill tiles
    vol = np.ones((24, 30, 36), np.uint8)
    vol[0, 0, 0] = 0
    vol[23, 5, 30] = 0
    ref = O.local_thickness(vol, O.FOREGROUND)
    got, sq = local_thickness(vol, Phase.FOREGROUND, ctx=gpu_ctx, return_squared=True)
    assert np.array_equal(sq, ref.propagated)
    assert np.array_equal(got.view(np.uint32), ref.thickness.view(np.uint32))


def test_isolated_voxel_has_diameter_two(gpu_ctx):
    # local_thickness.rs:364-374
    vol = np.zeros((3, 3, 3), np.uint8)
    vol[1, 1, 1] = 1
    t = local_thickness(vol, ctx=gpu_ctx).ravel()
    assert t[13] == 2.0 and (t > 0).sum() == 1


def test_background_matches_complement(gpu_ctx):
    # local_thickness.rs:376-393
    data = np.zeros((5, 5, 5), np.uint8)
    data[1:4, 1:4, 1:4] = 1
    a = local_thickness(data, Phase.BACKGROUND, ctx=gpu_ctx)
    b = local_thickness(1 - data, Phase.FOREGROUND, ctx=gpu_ctx)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def check_stats(got, ref_map, scale):
    assert_reference_stats(got, ref_map, scale)


def test_tbth_tbsp_plain_128(gpu_ctx, site_method):
    sp = S.config_plain_128()
    res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True)
    for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
        m = O.phase_inside(sp.bone, sp.roi, sel)
        ref = O.local_thickness(m, O.FOREGROUND)
        assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
        check_stats(got, ref.thickness, sp.spacing_um)


@pytest.mark.parametrize("seed", [21, 22])
def test_tbth_tbsp_small_random_specimens(gpu_ctx, site_method, seed):
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(20, 70, size=3))
    sp = S.make_specimen(shape, float(rng.uniform(1.5, 3)), float(rng.uniform(0.1, 0.4)), "cylinder",
                         0.45 * min(shape[1], shape[2]), float(rng.uniform(5, 25)), seed)
    res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True)
    for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
        m = O.phase_inside(sp.bone, sp.roi, sel)
        ref = O.local_thickness(m, O.FOREGROUND)
        assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
        check_stats(got, ref.thickness, sp.spacing_um)


@pytest.mark.parametrize("shape", [(20, 24, 48), (9, 12, 528), (11, 13, 47)])
def test_tbth_tbsp_row_widths(gpu_ctx, shape):
    """Tb.Th / Tb.Sp maps bit-exact for widths on and off the 16-voxel x-pass path."""
    sp = S.make_specimen(shape, 2.0, 0.3, "cylinder", 0.45 * min(shape[1], shape[2]), 12.0, 31)
    res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True)
    for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
        m = O.phase_inside(sp.bone, sp.roi, sel)
        ref = O.local_thickness(m, O.FOREGROUND)
        assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
        check_stats(got, ref.thickness, sp.spacing_um)


@pytest.mark.parametrize("rows", [16, 32, 64])
def test_fill_tile_rows(gpu_ctx, rows):
    """Every fill tile shape (32 x 16, 32 or 64 x 16 voxels) gives the
    reference's maps, on heights that are and are not multiples of 64."""
    for shape, seed in (((40, 100, 72), 61), ((33, 128, 64), 62)):
        sp = S.make_specimen(shape, 3.0, 0.2, "cylinder", 0.45 * min(shape[1], shape[2]), 11.0, seed)
        gpu_ctx.set_fill_tile_rows(rows)
        try:
            res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True)
        finally:
            gpu_ctx.set_fill_tile_rows(0)
        for sel, got, gmap in ((True, res.thickness, res.thickness_map), (False, res.spacing, res.spacing_map)):
            m = O.phase_inside(sp.bone, sp.roi, sel)
            ref = O.local_thickness(m, O.FOREGROUND)
            assert np.array_equal(gmap.view(np.uint32), ref.thickness.view(np.uint32))
            check_stats(got, ref.thickness, sp.spacing_um)
    with pytest.raises(BoneMorphometryError, match="fill tile rows must be"):
        gpu_ctx.set_fill_tile_rows(48)


def test_device_tensor_path(gpu_ctx):
    import torch

    sp = S.config_plain_128()
    bone = torch.from_numpy(sp.bone).cuda()
    roi = torch.from_numpy(sp.roi).cuda()
    res_d = analyze_thickness(bone, roi, sp.spacing_um, ctx=gpu_ctx)
    res_h = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx)
    assert res_d.thickness.mean == res_h.thickness.mean
    assert res_d.spacing.standard_deviation == res_h.spacing.standard_deviation
    vol = torch.from_numpy(O.phase_inside(sp.bone, sp.roi, True)).cuda()
    e = euclidean_distance_transform_squared(vol, ctx=gpu_ctx).cpu().numpy().view(np.uint32)
    assert np.array_equal(e, O.edt_sq(vol.cpu().numpy()))


def test_device_inputs_at_odd_offsets(gpu_ctx):
    """Bone and ROI tensors that start off a 16-byte boundary (byte-loop count
    and scalar x pass) give the same results as aligned ones."""
    import torch

    sp = S.make_specimen((18, 26, 64), 2.0, 0.3, "cylinder", 11.0, 9.0, 81)
    n = sp.bone.size
    ref = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx)
    for ob, orr in ((1, 3), (0, 5), (7, 0)):
        bb = torch.zeros(n + 16, dtype=torch.uint8, device="cuda")
        rb = torch.zeros(n + 16, dtype=torch.uint8, device="cuda")
        bb[ob:ob + n] = torch.from_numpy(sp.bone.ravel()).cuda()
        rb[orr:orr + n] = torch.from_numpy(sp.roi.ravel()).cuda()
        got = analyze_thickness(bb[ob:ob + n].view(sp.bone.shape), rb[orr:orr + n].view(sp.roi.shape),
                                sp.spacing_um, ctx=gpu_ctx)
        assert got.thickness.mean == ref.thickness.mean and got.spacing.mean == ref.spacing.mean
        assert got.spacing.maximum == ref.spacing.maximum


@pytest.mark.parametrize("shape", [(4, 4, 4), (3, 5, 7), (6, 9, 37)])
def test_roi_counts_in_the_tail(gpu_ctx, shape):
    """The bails see ROI and bone voxels that sit only in the last n % 32 bytes."""
    n = int(np.prod(shape))
    bone = np.zeros(shape, np.uint8)
    roi = np.zeros(shape, np.uint8)
    with pytest.raises(BoneMorphometryError, match="ROI mask contains no included voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    flat_r = roi.reshape(-1)
    flat_r[n - 2:] = 1
    with pytest.raises(BoneMorphometryError, match="ROI contains no bone voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    bone.reshape(-1)[n - 2:] = 255
    with pytest.raises(BoneMorphometryError, match="ROI contains no marrow voxels"):
        analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    bone.reshape(-1)[n - 1] = 0
    res = analyze_thickness(bone, roi, 1.0, ctx=gpu_ctx)
    assert res.thickness.mean > 0 and res.spacing.mean > 0


def test_phases_side_by_side_or_sequential_agree(gpu_ctx):
    """Tb.Th / Tb.Sp with the two phases on two streams (default) and one after
    the other: identical maps and statistics, quantiles included."""
    sp = S.make_specimen((30, 44, 52), 2.5, 0.3, "cylinder", 19.0, 13.0, 71)
    from bone_morphometry_gb300 import FeatureMode
    a = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True,
                          feature_mode=FeatureMode.STANDARD)
    gpu_ctx.set_concurrent_phases(False)
    try:
        b = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, ctx=gpu_ctx, return_maps=True,
                              feature_mode=FeatureMode.STANDARD)
    finally:
        gpu_ctx.set_concurrent_phases(True)
    assert np.array_equal(a.thickness_map.view(np.uint32), b.thickness_map.view(np.uint32))
    assert np.array_equal(a.spacing_map.view(np.uint32), b.spacing_map.view(np.uint32))
    for x, y in ((a.thickness, b.thickness), (a.spacing, b.spacing)):
        assert x.mean == y.mean and x.standard_deviation == y.standard_deviation and x.median == y.median
        assert x.percentile_90 == y.percentile_90
