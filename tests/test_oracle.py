"""Pins of the CPU oracle: the reference's own known-answer tests and an
independent exact EDT (scipy).  CPU only."""

import numpy as np
import pytest

import oracle as O


# -- edt.rs:229-274 ------------------------------------------------------------------------------

def test_phase_selection_direction_is_correct():
    # edt.rs:229-238: Foreground selects value != 0, Background selects value == 0.
    for value in (0, 1, 255):
        fg = np.zeros((2, 2, 2), np.uint8)
        fg[0, 0, 0] = value  # every other voxel is a foreground site
        assert (O.edt_sq(fg, O.FOREGROUND)[0, 0, 0] > 0) == (value != 0)
        bg = np.ones((2, 2, 2), np.uint8)
        bg[0, 0, 0] = value  # every other voxel is a background site
        assert (O.edt_sq(bg, O.BACKGROUND)[0, 0, 0] > 0) == (value == 0)


def test_edt_center_background():
    # edt.rs:240-261: 3^3 of ones with the centre 0
    data = np.ones(27, np.uint8)
    data[13] = 0
    e = np.sqrt(O.edt_sq(data.reshape(3, 3, 3), O.FOREGROUND).ravel().astype(np.float32))
    assert e[13] == 0.0
    assert abs(e[12] - 1.0) < 1e-6
    assert abs(e[0] - np.float32(3.0) ** 0.5) < 1e-6


def test_background_phase_uses_foreground_as_sites():
    # edt.rs:263-274
    data = np.zeros(27, np.uint8)
    data[13] = 1
    e = np.sqrt(O.edt_sq(data.reshape(3, 3, 3), O.BACKGROUND).ravel().astype(np.float32))
    assert e[13] == 0.0
    assert abs(e[12] - 1.0) < 1e-6
    assert abs(e[0] - np.float32(3.0) ** 0.5) < 1e-6


def test_all_selected_bails():
    # edt.rs:61-66
    with pytest.raises(O.OracleError, match="all-foreground"):
        O.edt_sq(np.ones((3, 3, 3), np.uint8), O.FOREGROUND)
    with pytest.raises(O.OracleError, match="all-background"):
        O.edt_sq(np.zeros((3, 3, 3), np.uint8), O.BACKGROUND)


# -- local_thickness.rs:364-401 ------------------------------------------------------------------

def test_isolated_voxel_has_diameter_two():
    data = np.zeros(27, np.uint8)
    data[13] = 1
    t = O.local_thickness(data.reshape(3, 3, 3), O.FOREGROUND).thickness.ravel()
    assert abs(t[13] - 2.0) < 1e-6
    assert (t > 0).sum() == 1


def test_background_phase_matches_complemented_foreground_phase():
    data = np.zeros((5, 5, 5), np.uint8)
    data[1:4, 1:4, 1:4] = 1
    direct = O.local_thickness(data, O.BACKGROUND).thickness
    comp = O.local_thickness((data == 0).astype(np.uint8), O.FOREGROUND).thickness
    assert np.array_equal(direct.view(np.uint32), comp.view(np.uint32))


def test_search_template_matches_known_single_voxel_radius():
    t = O.create_templates([1])
    assert list(t[:, 0]) == [4, 5, 6]


# -- metrics.rs:304-326, volume.rs:123-136 -------------------------------------------------------

def test_quantiles_use_numpy_linear_interpolation():
    q = O.quantiles(np.array([1, 2, 3, 4], np.float32), 1.0, (0.1, 0.5, 0.9))
    assert abs(q[0] - 1.3) < 1e-6 and abs(q[1] - 2.5) < 1e-6 and abs(q[2] - 3.7) < 1e-6


def test_distribution_statistics_include_cv():
    vals = np.array([0, 1, 2, 3, 4], np.float32)
    s = O.nonzero_stats(vals, 2.0)
    med, p10, p25, p75, p90 = O.quantiles(vals, 2.0)
    assert abs(s.mean - 5.0) < 1e-12
    assert abs(med - 5.0) < 1e-12
    assert abs(p10 - 2.6) < 1e-6
    assert abs(p90 - 7.4) < 1e-6
    assert abs(s.max - 8.0) < 1e-12
    assert abs(s.sd - 2.581988897471611) < 1e-12
    assert abs(s.sd / s.mean - s.sd / 5.0) < 1e-12


def test_phase_inside_distinguishes_marrow_from_outside_roi():
    bone = np.array([0, 1, 0, 1, 0, 1, 0, 1], np.uint8).reshape(2, 2, 2)
    roi = np.array([0, 0, 1, 1, 1, 1, 0, 0], np.uint8).reshape(2, 2, 2)
    assert list(O.phase_inside(bone, roi, True).ravel()) == [0, 0, 0, 1, 0, 1, 0, 0]
    assert list(O.phase_inside(bone, roi, False).ravel()) == [0, 0, 1, 0, 1, 0, 0, 0]


def test_empty_stats_bail():
    with pytest.raises(O.OracleError, match="selected phase is empty"):
        O.nonzero_stats(np.zeros(5, np.float32), 1.0)


# -- independent pins ------------------------------------------------------------------------------

@pytest.mark.parametrize("shape", [(17, 23, 31), (40, 33, 29), (2, 2, 2), (3, 64, 5)])
@pytest.mark.parametrize("p", [0.05, 0.5, 0.95])
def test_edt_matches_scipy(shape, p):
    from scipy.ndimage import distance_transform_edt

    rng = np.random.default_rng(hash((shape, p)) & 0xFFFF)
    vol = (rng.random(shape) < p).astype(np.uint8)
    if vol.all():
        vol.flat[0] = 0
    for phase, sel in ((O.FOREGROUND, vol != 0), (O.BACKGROUND, vol == 0)):
        if sel.all():
            continue
        ref = distance_transform_edt(sel)
        ref2 = np.rint(ref.astype(np.float64) ** 2).astype(np.uint32)
        assert np.array_equal(O.edt_sq(vol, phase), ref2)


def test_exact_sums_match_fsum():
    import math

    rng = np.random.default_rng(7)
    vals = (rng.random(5000).astype(np.float32) * 50).astype(np.float32)
    vals[::7] = 0
    n, s, ss, mx = O.exact_moment_sums(vals, 19.5)
    v = vals[vals > 0] * np.float32(19.5)
    assert n == v.size
    assert s == math.fsum(v.astype(np.float64))
    assert ss == math.fsum((v.astype(np.float64)) ** 2)
    assert mx == float(v.max())


@pytest.mark.parametrize("scale", [19.5, 1e-39, 3e-38, 7.5e33, 0.37])
def test_exact_sums_c_bins_match_numpy(scale):
    """The C++ per-exponent bins (used on 1024^3 maps) against the numpy sums,
    at spacings that make values subnormal, tiny or huge."""
    rng = np.random.default_rng(11)
    vals = (rng.random(200_000) * 300).astype(np.float32)
    vals[::5] = 0
    vals[3] = np.inf
    vals[4] = -2.0
    vals[5] = np.nan
    assert O.exact_moment_sums(vals, scale) == O.exact_moment_sums_numpy(vals, scale)
