"""GPU statistics and quantiles (metrics.rs:204-298) against the oracle.  Marked gpu."""

import math

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import BoneMorphometryError, FeatureMode, analyze_thickness, nonzero_stats
from bone_morphometry_gb300 import synthetic as S
from refstats import assert_reference_stats

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
    assert_reference_stats(st, v, 19.5)
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
    """Fixed-point and per-exponent exact-sum paths and the reference-order sums
    (subnormal, tiny, ordinary and huge calibrations) against the oracle."""
    sp = S.make_specimen((24, 26, 28), 2.0, 0.3, "cylinder", 11.0, spacing, 41)
    res = analyze_thickness(sp.bone, sp.roi, spacing, ctx=gpu_ctx)
    for sel, got in ((True, res.thickness), (False, res.spacing)):
        ref = O.local_thickness(O.phase_inside(sp.bone, sp.roi, sel), O.FOREGROUND).thickness
        assert_reference_stats(got, ref, spacing)


# -- the reference-order sums on maps made to stress them --------------------------------------

def _ties_map(n, seed):
    """A huge first value, then odd multiples of half the running sum's ulp
    (round-half-even decided by the sum's parity), values below half an ulp
    (lost), skipped entries and ordinary values."""
    rng = np.random.default_rng(seed)
    v = np.zeros(n, np.float32)
    kind = rng.random(n)
    odd = (2 * rng.integers(1, 1 << 15, size=n) + 1).astype(np.float64) * 128.0
    v[kind < 0.5] = odd[kind < 0.5].astype(np.float32)
    small = (kind >= 0.5) & (kind < 0.7)
    v[small] = rng.integers(1, 128, size=int(small.sum())).astype(np.float32)
    other = kind >= 0.8
    v[other] = (rng.random(int(other.sum())) * 1e6).astype(np.float32)
    v[0] = 2.0 ** 60
    return v


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (255, 2), (256, 3), (257, 4), (8191, 5), (8193, 6),
                                    (300_001, 7), (2_100_000, 8)])
def test_reference_order_sums_on_ties(gpu_ctx, n, seed):
    v = _ties_map(n, seed)
    for scale in (1.0, 0.75):
        assert_reference_stats(nonzero_stats(v, scale, ctx=gpu_ctx), v, scale)


@pytest.mark.parametrize("n,seed", [(5_000_000, 11), (33_554_433, 12)])
def test_reference_order_sums_many_crossings(gpu_ctx, n, seed):
    """Values over eight decades after tiny ones: the running sums cross more
    than a hundred binades, some within one chunk of 256 entries."""
    rng = np.random.default_rng(seed)
    v = (10.0 ** rng.uniform(-3, 5, size=n)).astype(np.float32)
    v[rng.random(n) < 0.4] = 0.0
    v[: 1000] = (10.0 ** rng.uniform(-30, -20, size=1000)).astype(np.float32)
    assert_reference_stats(nonzero_stats(v, 19.5, ctx=gpu_ctx), v, 19.5)


def test_reference_order_sums_leading_zeros(gpu_ctx):
    """Millions of empty entries before the first value (outside the ROI)."""
    v = np.zeros(12_000_000, np.float32)
    rng = np.random.default_rng(13)
    v[9_000_000:] = (rng.random(3_000_000) * 300).astype(np.float32)
    assert_reference_stats(nonzero_stats(v, 8.0, ctx=gpu_ctx), v, 8.0)


def test_reference_order_sums_overflow_to_inf(gpu_ctx):
    """raw * scale overflowing f32 gives +inf values: sums +inf as in the reference."""
    v = np.array([0, 3.0, 2.0e30, 5.0, 0, 1e-3] * 1000, np.float32)
    st = nonzero_stats(v, 1e10, ctx=gpu_ctx)
    seq = O.nonzero_stats(v, 1e10)
    assert st.sum == seq.sum == float("inf") and st.count == seq.count
    assert st.sum_of_squares == seq.sum_sq and st.mean == seq.mean and st.maximum == seq.max
