"""Bit-exact parity at the full benchmark sizes: the 512^3 specimen (sigma 5,
BV/TV 0.15, cylinder ROI r240, 19.5 um) and the 1024^3 plate specimen (sigma
(4, 4, 8), BV/TV 0.30, sphere ROI r500, 8 um), the same data the benchmark
times.  Marked gpu (and slow: the oracle needs about 20 s per 512^3 phase and
about a minute and 20 GiB of host memory per 1024^3 phase).

For each phase (ROI-clipped bone = Tb.Th, in-ROI marrow = Tb.Sp) the GPU's
u32 squared EDT (edt.rs:57-156), u32 propagated squared-thickness map
(local_thickness.rs:169-202) and f32 thickness map (local_thickness.rs:204-281)
must equal the oracle's voxel for voxel, with both site methods; the
statistics must equal the reference's bit for bit: its sequential f64 sums,
mean, SD and max (metrics.rs:215-241).  At these sizes the windowed EDT passes run
with their exact-envelope redo, the chain passes with wide halos, and the
tile fill with hundreds of r^2 bins per tile.

For the record, the deviation of the reference's sequential mean and SD from
those of the exactly rounded sums (the reference's own rounding error, which
the GPU reproduces) is written to the JSON-lines file named by
BM_PARITY_REPORT when set.
"""

import json
import os

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import Phase, _lib, analyze_thickness, euclidean_distance_transform_squared
from bone_morphometry_gb300 import local_thickness
from bone_morphometry_gb300 import synthetic as S
from refstats import assert_reference_stats

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

METHODS = [(_lib.BM_SITES_SPHERES, "spheres"), (_lib.BM_SITES_CHAINS, "chains")]


def report(record):
    path = os.environ.get("BM_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(record) + "\n")


def exact_deviation(config, phase_name, got):
    """The reference's rounding error: its sequential mean / SD (which the GPU
    returns) against the mean / SD of the exactly rounded sums."""
    emean = got.exact_sum / got.count
    c = float(got.count)
    centered = (c * got.exact_sum_of_squares - got.exact_sum * got.exact_sum) / c
    esd = (centered / (c - 1.0)) ** 0.5 if got.count > 1 and centered > 0 else 0.0
    rec = {"config": config, "phase": phase_name, "count": got.count, "mean": got.mean, "mean_exact_sums": emean,
           "sd": got.standard_deviation, "sd_exact_sums": esd,
           "rel_mean": abs(got.mean - emean) / abs(emean), "rel_sd": abs(got.standard_deviation - esd) / esd}
    report(rec)
    return rec


def to_u32(t):
    return t.cpu().numpy().view(np.uint32)


def to_f32bits(t):
    return t.cpu().numpy().view(np.uint32)


def run_config(gpu_ctx, config, sp):
    """Both phases of one specimen: EDT, r^2 and f32 maps with both site
    methods, then analyze_thickness (the fused Tb.Th / Tb.Sp entry point)
    against the same oracle maps and the reference's statistics."""
    import torch

    bone_d = torch.from_numpy(sp.bone).cuda()
    roi_d = torch.from_numpy(sp.roi).cuda()
    res = analyze_thickness(bone_d, roi_d, sp.spacing_um, ctx=gpu_ctx, return_maps=True)
    torch.cuda.synchronize()
    for sel, name, got, gmap in ((True, "TbTh", res.thickness, res.thickness_map),
                                 (False, "TbSp", res.spacing, res.spacing_map)):
        m = O.phase_inside(sp.bone, sp.roi, sel)
        ref = O.local_thickness(m, O.FOREGROUND)
        m_d = torch.from_numpy(m).cuda()
        e = euclidean_distance_transform_squared(m_d, Phase.FOREGROUND, ctx=gpu_ctx)
        assert np.array_equal(to_u32(e), ref.edt), "%s %s: EDT map differs" % (config, name)
        del e
        for method, mname in METHODS:
            gpu_ctx.set_site_method(method)
            try:
                t, sq = local_thickness(m_d, Phase.FOREGROUND, ctx=gpu_ctx, return_squared=True)
            finally:
                gpu_ctx.set_site_method(_lib.BM_SITES_AUTO)
            assert np.array_equal(to_u32(sq), ref.propagated), "%s %s %s: r^2 map differs" % (config, name, mname)
            del sq
            assert np.array_equal(to_f32bits(t), ref.thickness.view(np.uint32)), \
                "%s %s %s: thickness map differs" % (config, name, mname)
            del t
        del m_d
        assert np.array_equal(to_f32bits(gmap), ref.thickness.view(np.uint32)), \
            "%s %s: analyze map differs" % (config, name)
        assert_reference_stats(got, ref.thickness, sp.spacing_um)
        exact_deviation(config, name, got)
        del ref, m
    del res


def test_config_single_512_bitexact(gpu_ctx):
    """512^3, the default benchmark specimen (numpy / scipy generator)."""
    sp = S.config_single_512()
    run_config(gpu_ctx, "single512", sp)


def test_config_single_1024_bitexact(gpu_ctx):
    """1024^3 plate specimen as the benchmark makes it (torch generator on the GPU)."""
    sp = S.make_specimen_torch((1024, 1024, 1024), (4.0, 4.0, 8.0), 0.30, "sphere", 500.0, 8.0,
                               S.config_single_1024.__defaults__[0])
    run_config(gpu_ctx, "single1024", sp)
