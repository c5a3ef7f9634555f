"""Native TIFF stack decoder (tiff_io.rs:19-149) on files written by
tests/tiffgen.py: every supported layout and encoding decodes to the source
voxels, the validation modes and the reference's error texts.  Host code only:
runs without a GPU (pinned-memory and GPU round trips are marked gpu)."""

import itertools

import numpy as np
import pytest

from bone_morphometry_gb300 import BoneMorphometryError
from bone_morphometry_gb300.tiff_io import read_binary_tiff, read_roi_tiff

import tiffgen as T


def stack(seed, d=5, h=23, w=37, binary=True):
    rng = np.random.default_rng(seed)
    if binary:
        return (rng.random((d, h, w)) < 0.4).astype(np.uint8) * np.uint8(255)
    # smooth-ish gray values with runs, so that PackBits/LZW see repeats
    base = rng.integers(0, 256, size=(d, h, w // 4 + 1)).astype(np.uint8)
    return np.repeat(base, 4, axis=2)[:, :, :w].copy()


LAYOUTS = [dict(rows_per_strip=None), dict(rows_per_strip=1), dict(rows_per_strip=7), dict(tile=(16, 16))]
CODINGS = [(T.NONE, 1), (T.PACKBITS, 1), (T.LZW, 1), (T.LZW, 2), (T.DEFLATE, 1), (T.DEFLATE, 2)]


@pytest.mark.parametrize("layout,coding,big,order",
                         list(itertools.product(range(len(LAYOUTS)), range(len(CODINGS)), [False, True], ["<", ">"])))
def test_round_trip(tmp_path, layout, coding, big, order):
    vol = stack(100 + layout * 10 + coding, binary=False)
    comp, pred = CODINGS[coding]
    p = tmp_path / "s.tif"
    T.write_tiff(p, list(vol), compression=comp, predictor=pred, big=big, byteorder=order, **LAYOUTS[layout])
    got = read_binary_tiff(p, threshold=100)
    assert (got.width, got.height, got.depth) == (vol.shape[2], vol.shape[1], vol.shape[0])
    assert np.array_equal(got.array(), (vol > 100).astype(np.uint8))


def test_lzw_table_resets_on_long_pages(tmp_path):
    rng = np.random.default_rng(7)
    vol = rng.integers(0, 256, size=(3, 200, 300)).astype(np.uint8)  # incompressible: many Clear codes
    p = tmp_path / "l.tif"
    T.write_tiff(p, list(vol), compression=T.LZW)
    assert np.array_equal(read_binary_tiff(p, threshold=0).array(), (vol > 0).astype(np.uint8))


def test_strict_binary_and_roi_values(tmp_path):
    vol = stack(3)
    p = tmp_path / "b.tif"
    T.write_tiff(p, list(vol), compression=T.DEFLATE)
    assert np.array_equal(read_binary_tiff(p, 0, strict_binary=True).array(), (vol > 0).astype(np.uint8))
    roi = (vol // 255).astype(np.uint8)  # 0/1 encoding
    q = tmp_path / "r.tif"
    T.write_tiff(q, list(roi), compression=T.PACKBITS)
    assert np.array_equal(read_roi_tiff(q).array(), roi)


def test_invalid_sample_messages(tmp_path):
    vol = stack(4)
    vol[1, 2, 3] = 7
    p = tmp_path / "bad.tif"
    T.write_tiff(p, list(vol))
    with pytest.raises(BoneMorphometryError) as ei:
        read_binary_tiff(p, 0, strict_binary=True)
    assert str(ei.value).endswith("%s is not a valid binary image: page 2, sample %d has value 7 (expected 0 or 255)"
                                  % (p, 2 * vol.shape[2] + 3))
    roi = (vol > 0).astype(np.uint8)
    roi[4, 0, 1] = 2
    q = tmp_path / "badroi.tif"
    T.write_tiff(q, list(roi), compression=T.LZW)
    with pytest.raises(BoneMorphometryError) as ei:
        read_roi_tiff(q)
    assert str(ei.value).endswith("%s is not a valid binary image: page 5, sample 1 has value 2 (expected 0/1 or 0/255)"
                                  % q)
    # without the strict check any value is accepted and thresholded
    assert read_binary_tiff(p, 6).array()[1, 2, 3] == 1


def test_page_type_and_dimension_errors(tmp_path):
    vol = stack(5)
    p16 = tmp_path / "g16.tif"
    T.write_tiff(p16, [v.astype(np.uint16) for v in vol], bits=16)
    with pytest.raises(BoneMorphometryError, match="must contain 8-bit grayscale pages; found Gray\\(16\\)"):
        read_binary_tiff(p16)
    prgb = tmp_path / "rgb.tif"
    T.write_tiff(prgb, [np.stack([v, v, v], axis=-1) for v in vol], photometric=2, samples=3)
    with pytest.raises(BoneMorphometryError, match="found RGB\\(8\\)"):
        read_binary_tiff(prgb)
    pdim = tmp_path / "dims.tif"
    T.write_tiff(pdim, [vol[0], vol[1], vol[2][:, :-1]])
    with pytest.raises(BoneMorphometryError) as ei:
        read_binary_tiff(pdim)
    assert str(ei.value) == ("TIFF pages in %s do not have consistent dimensions: expected %dx%d, got %dx%d"
                             % (pdim, vol.shape[2], vol.shape[1], vol.shape[2] - 1, vol.shape[1]))
    psigned = tmp_path / "i8.tif"
    T.write_tiff(psigned, list(vol), sample_format=2)
    with pytest.raises(BoneMorphometryError, match="decoded to an unsupported pixel type"):
        read_binary_tiff(psigned)


def test_first_failing_page_is_reported(tmp_path):
    # the reference checks page by page: an invalid sample on page 1 wins over a
    # dimension mismatch on page 3
    vol = stack(6)
    vol[0, 0, 0] = 9
    p = tmp_path / "order.tif"
    T.write_tiff(p, [vol[0], vol[1], vol[2][:-1]])
    with pytest.raises(BoneMorphometryError, match="page 1, sample 0 has value 9"):
        read_binary_tiff(p, 0, strict_binary=True)


def test_thin_stacks_rejected(tmp_path):
    p = tmp_path / "one.tif"
    T.write_tiff(p, [stack(8)[0]])
    with pytest.raises(BoneMorphometryError, match="all dimensions must be at least 2 for 3-D morphometry; got 37x23x1"):
        read_binary_tiff(p)


def test_missing_file(tmp_path):
    with pytest.raises(BoneMorphometryError, match="opening"):
        read_binary_tiff(tmp_path / "nope.tif")


@pytest.mark.gpu
def test_tiff_stack_to_thickness_on_gpu(tmp_path, gpu_ctx):
    """A bone stack and an ROI stack decoded into pinned memory give the same
    Tb.Th / Tb.Sp as the arrays they were written from."""
    from bone_morphometry_gb300 import analyze_thickness
    from bone_morphometry_gb300 import synthetic as S

    sp = S.make_specimen((24, 40, 48), 2.5, 0.3, "cylinder", 18.0, 11.0, 51)
    pb, pr = tmp_path / "bone.tif", tmp_path / "roi.tif"
    T.write_tiff(pb, list(sp.bone), compression=T.LZW, predictor=2, rows_per_strip=8)
    T.write_tiff(pr, list(sp.roi), compression=T.DEFLATE, tile=(16, 16))
    bone = read_binary_tiff(pb, 0, strict_binary=True, pinned=True)
    roi = read_roi_tiff(pr, pinned=True)
    got = analyze_thickness(bone.array(), roi.array(), sp.spacing_um, ctx=gpu_ctx)
    ref = analyze_thickness((sp.bone > 0).astype(np.uint8), sp.roi, sp.spacing_um, ctx=gpu_ctx)
    assert got.thickness.mean == ref.thickness.mean and got.spacing.mean == ref.spacing.mean
    assert got.thickness.standard_deviation == ref.thickness.standard_deviation
    assert got.spacing.maximum == ref.spacing.maximum


@pytest.mark.parametrize("mode", sorted(T.DEFLATE_MODES))
@pytest.mark.parametrize("kind", ["binary", "gray", "noise"])
def test_deflate_every_block_type(tmp_path, mode, kind):
    """Stored, fixed-code and dynamic-code Deflate blocks (zlib's strategies),
    strips of a whole 200x300 page (several blocks each) and of 3 rows."""
    rng = np.random.default_rng(hash((mode, kind)) & 0xFFFF)
    if kind == "binary":
        vol = stack(5, d=3, h=200, w=300)
    elif kind == "gray":
        vol = stack(6, d=3, h=200, w=300, binary=False)
    else:
        vol = rng.integers(0, 256, size=(3, 200, 300)).astype(np.uint8)
    for rps in (None, 3):
        p = tmp_path / ("d%s.tif" % rps)
        T.write_tiff(p, list(vol), compression=T.DEFLATE, rows_per_strip=rps, deflate_mode=mode)
        for thr in (0, 100, 200):
            assert np.array_equal(read_binary_tiff(p, threshold=thr).array(), (vol > thr).astype(np.uint8))


def test_corrupt_deflate_data_is_an_error(tmp_path):
    vol = stack(8, d=2, h=64, w=64, binary=False)
    p = tmp_path / "c.tif"
    T.write_tiff(p, list(vol), compression=T.DEFLATE)
    raw = bytearray(p.read_bytes())
    rng = np.random.default_rng(3)
    failures = 0
    for trial in range(40):
        bad = bytearray(raw)
        # flip bytes inside the first strip's data (after the 8-byte header)
        for k in rng.integers(10, 200, size=4):
            bad[int(k)] ^= 0xA5
        q = tmp_path / ("c%d.tif" % trial)
        q.write_bytes(bytes(bad))
        try:
            read_binary_tiff(q, threshold=100)
        except BoneMorphometryError:
            failures += 1  # a clean error, never a crash
    assert failures > 0
