"""Batched and served forms: every result equals the specimen's result alone
(bit for bit), admission respects the HBM budget.  Marked gpu."""

import time

import numpy as np
import pytest

from bone_morphometry_gb300 import FeatureMode, analyze_thickness
from bone_morphometry_gb300 import synthetic as S
from bone_morphometry_gb300.serving import Server, SpecimenInput, batch_tbth_tbsp, footprint_bytes

pytestmark = pytest.mark.gpu


def small_specimens(n=8, seed=7):
    specs = S.batch_specs(n, 24, 72, seed=seed)
    return [S.make_batch_item(s) for s in specs]


def same(a, b):
    return (a.count, a.mean, a.standard_deviation, a.maximum) == (b.count, b.mean, b.standard_deviation, b.maximum)


def test_batch_equals_alone(gpu_ctx):
    items = small_specimens()
    alone = [analyze_thickness(s.bone, s.roi, s.spacing_um, ctx=gpu_ctx) for s in items]
    res = batch_tbth_tbsp([SpecimenInput(s.bone, s.roi, s.spacing_um) for s in items], ctx=gpu_ctx, workers=3)
    for a, (th, sp, st) in zip(alone, res):
        assert st == 0
        assert same(a.thickness, th) and same(a.spacing, sp)


def test_batch_device_pointers_and_quantiles(gpu_ctx):
    import torch

    items = small_specimens(5, seed=11)
    alone = [analyze_thickness(s.bone, s.roi, s.spacing_um, FeatureMode.STANDARD, ctx=gpu_ctx) for s in items]
    dev = [SpecimenInput(torch.from_numpy(s.bone).cuda(), torch.from_numpy(s.roi).cuda(), s.spacing_um) for s in items]
    torch.cuda.synchronize()
    res = batch_tbth_tbsp(dev, FeatureMode.STANDARD, ctx=gpu_ctx)
    for a, (th, sp, st) in zip(alone, res):
        assert st == 0 and same(a.thickness, th) and same(a.spacing, sp)
        assert a.thickness.median == th.median and a.spacing.percentile_90 == sp.percentile_90


def test_tuned_batch_equals_alone(gpu_ctx, tmp_path):
    """The tuner runs the batch under each candidate (worker count, site
    method, fill tile rows, phase scheduling): the results equal the
    specimens' results alone, and the second call reads its settings from the
    cache."""
    from bone_morphometry_gb300 import Context
    from bone_morphometry_gb300._lib import BM_SITES_AUTO, BM_SITES_CHAINS, BM_SITES_SPHERES
    from bone_morphometry_gb300.serving import tuned_batch_tbth_tbsp

    items = small_specimens(6, seed=5)
    alone = [analyze_thickness(s.bone, s.roi, s.spacing_um, ctx=gpu_ctx) for s in items]
    inputs = [SpecimenInput(s.bone, s.roi, s.spacing_um) for s in items]
    cands = ((2, BM_SITES_AUTO, 32, True), (3, BM_SITES_SPHERES, 64, False), (2, BM_SITES_CHAINS, 64, True))
    path = str(tmp_path / "tuning.json")
    ctx = Context()
    try:
        res, t = tuned_batch_tbth_tbsp(inputs, ctx=ctx, cache_path=path, candidates=cands)
        assert not t.from_cache and t.setting() in cands
        for a, (th, sp, st) in zip(alone, res):
            assert st == 0 and same(a.thickness, th) and same(a.spacing, sp)
        res2, t2 = tuned_batch_tbth_tbsp(inputs, ctx=ctx, cache_path=path, candidates=cands)
        assert t2.from_cache and (t2.workers, t2.site_method) == (t.workers, t.site_method)
        for a, (th, sp, st) in zip(alone, res2):
            assert st == 0 and same(a.thickness, th) and same(a.spacing, sp)
    finally:
        ctx.close()


def test_batch_reports_per_specimen_errors(gpu_ctx):
    items = small_specimens(3, seed=3)
    bad = SpecimenInput(np.zeros((8, 8, 8), np.uint8), np.zeros((8, 8, 8), np.uint8), 10.0)
    res = batch_tbth_tbsp([SpecimenInput(s.bone, s.roi, s.spacing_um) for s in items] + [bad], ctx=gpu_ctx)
    assert [r[2] for r in res[:3]] == [0, 0, 0]
    assert res[3][2] == 8  # BM_ERR_ROI_EMPTY


def test_server_results_alone_and_in_mix(gpu_ctx):
    items = small_specimens(10, seed=5)
    alone = [analyze_thickness(s.bone, s.roi, s.spacing_um, ctx=gpu_ctx) for s in items]
    with Server(workers=4, hbm_budget_bytes=4e9) as srv:
        tickets = []
        for s in items:  # staggered arrivals: later requests join while earlier ones run
            tickets.append(srv.submit(s.bone, s.roi, s.spacing_um))
            time.sleep(0.002)
        results = [srv.result(t) for t in tickets]
    for a, r in zip(alone, results):
        assert r.status == 0
        assert same(a.thickness, r.thickness) and same(a.spacing, r.spacing)
        assert r.submit_s <= r.start_s <= r.end_s


def test_server_budget_admission():
    items = small_specimens(6, seed=9)
    fp = max(footprint_bytes(s.bone.shape) for s in items)
    # room for one request at a time: no two may overlap
    with Server(workers=4, hbm_budget_bytes=fp * 1.5) as srv:
        tickets = [srv.submit(s.bone, s.roi, s.spacing_um) for s in items]
        results = sorted((srv.result(t) for t in tickets), key=lambda r: r.start_s)
    for a, b in zip(results, results[1:]):
        if a.footprint_bytes + b.footprint_bytes > fp * 1.5:
            assert b.start_s >= a.end_s
    with Server(workers=1, hbm_budget_bytes=1e6) as srv:
        with pytest.raises(Exception, match="budget"):
            srv.submit(items[0].bone, items[0].roi, items[0].spacing_um)


def test_server_tiff_requests(tmp_path, gpu_ctx):
    """Requests read from TIFF stacks on the workers give the results of the
    arrays they were written from; a missing ROI means every voxel, and a
    decoding or shape error comes back in the result with its message."""
    import tiffgen as T

    sp = S.make_specimen((20, 36, 44), 2.5, 0.25, "cylinder", 16.0, 9.5, 61)
    pb, pr = tmp_path / "b.tif", tmp_path / "r.tif"
    T.write_tiff(pb, list(sp.bone), compression=T.DEFLATE, predictor=2)
    T.write_tiff(pr, list(sp.roi), compression=T.PACKBITS, rows_per_strip=5)
    bad_roi = tmp_path / "r2.tif"
    T.write_tiff(bad_roi, list(sp.roi[:, :-1, :]))
    ref = analyze_thickness((sp.bone > 0).astype(np.uint8), sp.roi, sp.spacing_um, ctx=gpu_ctx)
    ref_all = analyze_thickness((sp.bone > 0).astype(np.uint8), np.ones_like(sp.roi), sp.spacing_um, ctx=gpu_ctx)
    with Server(workers=2, hbm_budget_bytes=8e9) as srv:
        t1 = srv.submit_tiff(pb, pr, sp.spacing_um, strict_binary=True)
        t2 = srv.submit_tiff(pb, None, sp.spacing_um)
        t3 = srv.submit_tiff(pb, bad_roi, sp.spacing_um)
        r1, r2, r3 = srv.result(t1), srv.result(t2), srv.result(t3)
    assert r1.status == 0 and r1.thickness.mean == ref.thickness.mean and r1.spacing.mean == ref.spacing.mean
    assert r2.status == 0 and r2.spacing.standard_deviation == ref_all.spacing.standard_deviation
    assert r3.status != 0
    assert r3.message == "binary image dimensions 44x36x20 do not match ROI dimensions 44x35x20"
