"""GPU statistics and quantiles (metrics.rs:204-298) against the oracle.  Marked gpu."""

import math

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import BoneMorphometryError, FeatureMode, analyze_thickness, nonzero_stats
from bone_morphometry_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

QS = (0.5, 0.1, 0.25, 0.75, 0.9)


def check_quantiles(got, values, scale):
    med, p10, p25, p75, p90 = O.quantiles(values, scale, QS)
    # exact order statistics and the reference's own interpolation: bit-equal
    assert got.median == med and got.percentile_10 == p10 and got.percentile_25 == p25
    assert got.percentile_75 == p75 and got.percentile_90 == p90
    assert got.interquartile_range == p75 - p25
    assert got.coefficient_of_variation == got.standard_deviation / got.mean


def test_quantiles_use_numpy_linear_interpolation(gpu_ctx):
    # metrics.rs:304-313 (there with scale 1 and no zero entries)
    st = nonzero_stats(np.array([1, 2, 3, 4], np.float32), 1.0, True, ctx=gpu_ctx)
    assert abs(st.percentile_10 - 1.3) < 1e-6 and abs(st.median - 2.5) < 1e-6 and abs(st.percentile_90 - 3.7) < 1e-6


def test_distribution_statistics_include_cv(gpu_ctx):
    # metrics.rs:315-326
    st = nonzero_stats(np.array([0, 1, 2, 3, 4], np.float32), 2.0, True, ctx=gpu_ctx)
    assert abs(st.mean - 5.0) < 1e-12
    assert abs(st.median - 5.0) < 1e-12
    assert abs(st.percentile_10 - 2.6) < 1e-6
    assert abs(st.percentile_90 - 7.4) < 1e-6
    assert abs(st.maximum - 8.0) < 1e-12
    assert abs(st.standard_deviation - 2.581988897471611) < 1e-12
    assert abs(st.coefficient_of_variation - st.standard_deviation / 5.0) < 1e-12


def test_stats_without_quantiles_are_nan(gpu_ctx):
    st = nonzero_stats(np.array([0, 1, 2], np.float32), 1.0, False, ctx=gpu_ctx)
    assert math.isnan(st.median) and math.isnan(st.interquartile_range)


def test_empty_phase_bails(gpu_ctx):
    with pytest.raises(BoneMorphometryError, match="selected phase is empty"):
        nonzero_stats(np.array([0, -1, np.nan, np.inf], np.float32), 1.0, True, ctx=gpu_ctx)


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (7, 2), (1000, 3), (123457, 4)])
def test_random_values_exact(gpu_ctx, n, seed):
    rng = np.random.default_rng(seed)
    v = (rng.random(n) * 300).astype(np.float32)
    v[rng.random(n) < 0.2] = 0
    v[rng.random(n) < 0.05] = -3.0
    if not (v > 0).any():
        v[0] = 1.5
    st = nonzero_stats(v, 19.5, True, ctx=gpu_ctx)
    cnt, s, ss, mx = O.exact_moment_sums(v, 19.5)
    mean, sd, mxr = O.stats_from_sums(cnt, s, ss, mx)
    assert (st.count, st.mean, st.standard_deviation, st.maximum) == (cnt, mean, sd, mxr)
    check_quantiles(st, v, 19.5)


def test_tbth_tbsp_standard_mode_quantiles(gpu_ctx):
    sp = S.config_plain_128()
    res = analyze_thickness(sp.bone, sp.roi, sp.spacing_um, FeatureMode.STANDARD, ctx=gpu_ctx)
    for sel, got in ((True, res.thickness), (False, res.spacing)):
        ref = O.local_thickness(O.phase_inside(sp.bone, sp.roi, sel), O.FOREGROUND).thickness
        check_quantiles(got, ref, sp.spacing_um)


def test_bonej_mode_rejects_full_roi(gpu_ctx):
    sp = S.config_plain_128()
    with pytest.raises(BoneMorphometryError, match="both inside and outside"):
        analyze_thickness(sp.bone, np.ones_like(sp.roi), sp.spacing_um, FeatureMode.BONEJ, ctx=gpu_ctx)


def test_roi_controls_volume_and_boundary_fraction(gpu_ctx):
    # metrics.rs:328-354 (BV, TV, BV/TV and the ROI boundary bone fraction parts)
    from bone_morphometry_gb300 import volume_metrics

    bone = np.zeros((5, 5, 5), np.uint8)
    bone[2, 2, 1] = 1
    roi = np.zeros((5, 5, 5), np.uint8)
    roi[1:4, 1:4, 1:4] = 1
    vm = volume_metrics(bone, roi, 1.0, ctx=gpu_ctx)
    assert vm.bone_volume == 1.0 and vm.total_volume == 27.0
    assert abs(vm.bone_volume_fraction - 1.0 / 27.0) < 1e-12
    assert vm.roi_boundary_bone_fraction == 1.0


def test_volume_metrics_random(gpu_ctx):
    from bone_morphometry_gb300 import volume_metrics

    sp = S.config_plain_128()
    spacing = (10.0, 11.0, 12.5)
    vm = volume_metrics(sp.bone, sp.roi, spacing, ctx=gpu_ctx)
    b = (sp.bone != 0) & (sp.roi != 0)
    r = sp.roi != 0
    vv = (1.0 * spacing[0]) * spacing[1] * spacing[2]
    assert vm.bone_volume == b.sum() * vv and vm.total_volume == r.sum() * vv
    rp = np.pad(r, 1, constant_values=False)
    nb = np.zeros_like(b)
    for ax in range(3):
        for sh in (-1, 1):
            nb |= ~np.roll(rp, sh, axis=ax)[1:-1, 1:-1, 1:-1]
    assert vm.boundary_bone_voxels == int((b & nb).sum())


@pytest.mark.parametrize("spacing", [1e-39, 3e-38, 0.37, 7.5e33])
def test_tbth_tbsp_exact_sums_at_extreme_spacings(gpu_ctx, spacing):
    """Fixed-point and per-exponent statistic paths (subnormal, tiny, ordinary
    and huge calibrations) against an exact summation of the oracle's maps."""
    sp = S.make_specimen((24, 26, 28), 2.0, 0.3, "cylinder", 11.0, spacing, 41)
    res = analyze_thickness(sp.bone, sp.roi, spacing, ctx=gpu_ctx)
    for sel, got in ((True, res.thickness), (False, res.spacing)):
        ref = O.local_thickness(O.phase_inside(sp.bone, sp.roi, sel), O.FOREGROUND).thickness
        n, s, ss, mx = O.exact_moment_sums(ref, spacing)
        mean, sd, mxr = O.stats_from_sums(n, s, ss, mx)
        assert got.count == n
        assert got.sum == s and got.sum_of_squares == ss
        assert got.mean == mean and got.standard_deviation == sd and got.maximum == mxr
