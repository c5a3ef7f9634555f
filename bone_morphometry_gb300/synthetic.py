"""Seeded synthetic trabecular volumes (bone u8 0/255 + ROI u8 0/1).

There is no public dataset for this path: the reference's 24 validation
specimens are not distributed.  Volumes are made the way the benchmark
configurations describe them: i.i.d. N(0, 1) noise, a Gaussian filter with
the given per-axis sigma (truncate 4 sigma, float32), and a threshold at the
(1 - BV/TV) quantile so that the requested fraction of the box is bone.  The
ROI is a centred cylinder along z (radius in voxels, centre (dim-1)/2) or a
centred sphere.

Layout matches the reference (volume.rs:44-46): arrays are shaped
(depth, height, width) and x is the fastest axis.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Specimen:
    bone: np.ndarray   # u8, 0/255, shape (d, h, w)
    roi: np.ndarray    # u8, 0/1, shape (d, h, w)
    spacing_um: float
    meta: dict = field(default_factory=dict)

    @property
    def shape(self):
        return self.bone.shape


def smoothed_noise(shape, sigma, seed: int) -> np.ndarray:
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape, dtype=np.float32)
    sig = sigma if isinstance(sigma, (tuple, list)) else (sigma, sigma, sigma)
    # sigma is given per (x, y, z); numpy axes are (z, y, x)
    return gaussian_filter(noise, sigma=(sig[2], sig[1], sig[0]), truncate=4.0, output=np.float32)


def threshold_bone(field_: np.ndarray, bvtv: float) -> np.ndarray:
    flat = field_.ravel()
    k = int(round((1.0 - bvtv) * (flat.size - 1)))
    thr = np.partition(flat, k)[k]
    return np.where(field_ > thr, np.uint8(255), np.uint8(0))


def cylinder_roi(shape, radius: float) -> np.ndarray:
    d, h, w = shape
    cy, cx = (h - 1) / 2.0, (w - 1) / 2.0
    y = np.arange(h, dtype=np.float64)[:, None]
    x = np.arange(w, dtype=np.float64)[None, :]
    disk = ((x - cx) ** 2 + (y - cy) ** 2) <= radius * radius
    return np.broadcast_to(disk[None, :, :], shape).astype(np.uint8)


def sphere_roi(shape, radius: float) -> np.ndarray:
    d, h, w = shape
    cz, cy, cx = (d - 1) / 2.0, (h - 1) / 2.0, (w - 1) / 2.0
    z = np.arange(d, dtype=np.float64)[:, None, None]
    y = np.arange(h, dtype=np.float64)[None, :, None]
    x = np.arange(w, dtype=np.float64)[None, None, :]
    return (((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) <= radius * radius).astype(np.uint8)


def make_specimen(shape, sigma, bvtv: float, roi_kind: str, roi_radius: float, spacing_um: float,
                  seed: int) -> Specimen:
    """shape = (d, h, w); sigma scalar or (sx, sy, sz)."""
    f = smoothed_noise(shape, sigma, seed)
    bone = threshold_bone(f, bvtv)
    del f
    if roi_kind == "cylinder":
        roi = cylinder_roi(shape, roi_radius)
    elif roi_kind == "sphere":
        roi = sphere_roi(shape, roi_radius)
    elif roi_kind == "all":
        roi = np.ones(shape, np.uint8)
    else:
        raise ValueError(roi_kind)
    return Specimen(bone, np.ascontiguousarray(roi), spacing_um,
                    dict(shape=tuple(shape), sigma=sigma, bvtv=bvtv, roi=roi_kind, roi_radius=roi_radius,
                         spacing_um=spacing_um, seed=seed))


# The five workloads.  Seeds are fixed per configuration.
def config_plain_128(seed: int = 1001) -> Specimen:
    """128^3, sigma 3, BV/TV 0.25, cylinder ROI radius 56, 10 um."""
    return make_specimen((128, 128, 128), 3.0, 0.25, "cylinder", 56.0, 10.0, seed)


def config_single_512(seed: int = 1002) -> Specimen:
    """512^3, sigma 5, BV/TV 0.15, cylinder ROI radius 240, 19.5 um."""
    return make_specimen((512, 512, 512), 5.0, 0.15, "cylinder", 240.0, 19.5, seed)


def config_single_1024(seed: int = 1003) -> Specimen:
    """1024^3, sigma (4, 4, 8), BV/TV 0.30, sphere ROI radius 500, 8 um."""
    return make_specimen((1024, 1024, 1024), (4.0, 4.0, 8.0), 0.30, "sphere", 500.0, 8.0, seed)


@dataclass
class BatchItemSpec:
    shape: tuple
    sigma: float
    bvtv: float
    spacing_um: float
    seed: int


def batch_specs(n: int = 64, edge_lo: int = 96, edge_hi: int = 384, seed: int = 1004):
    """Per-axis edges log-uniform in [edge_lo, edge_hi], sigma U[2,6], BV/TV U[0.08,0.40],
    spacing U[5,25] um; cylinder ROI of radius 0.45 * min(x, y)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        edges = np.exp(rng.uniform(math.log(edge_lo), math.log(edge_hi), size=3))
        w, h, d = (int(round(e)) for e in edges)
        out.append(BatchItemSpec((d, h, w), float(rng.uniform(2, 6)), float(rng.uniform(0.08, 0.40)),
                                 float(rng.uniform(5, 25)), int(rng.integers(0, 2**31 - 1))))
    return out


def make_batch_item(spec: BatchItemSpec) -> Specimen:
    d, h, w = spec.shape
    return make_specimen(spec.shape, spec.sigma, spec.bvtv, "cylinder", 0.45 * min(w, h), spec.spacing_um,
                         spec.seed)


def make_specimen_torch(shape, sigma, bvtv: float, roi_kind: str, roi_radius: float, spacing_um: float,
                        seed: int, device: str = "cuda", to_host: bool = True) -> Specimen:
    """The same generator on the GPU (torch): N(0,1) noise, separable Gaussian
    filter truncated at 4 sigma with reflected borders, threshold at the
    (1 - BV/TV) quantile (estimated from a 1/8 subsample above 64 M voxels).
    Used for the large benchmark workloads, where scipy on the host would take
    minutes; the voxel pattern differs from make_specimen's for the same seed."""
    import torch
    import torch.nn.functional as F

    d, h, w = shape
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    f = torch.randn((1, 1, d, h, w), generator=g, device=device, dtype=torch.float32)
    sig = sigma if isinstance(sigma, (tuple, list)) else (sigma, sigma, sigma)
    for axis, s in ((4, sig[0]), (3, sig[1]), (2, sig[2])):  # x, y, z
        r = int(4.0 * s + 0.5)
        t = torch.arange(-r, r + 1, device=device, dtype=torch.float32)
        k = torch.exp(-0.5 * (t / s) ** 2)
        k = k / k.sum()
        shape_k = [1, 1, 1, 1, 1]
        shape_k[axis] = 2 * r + 1
        pad = [0, 0, 0, 0, 0, 0]
        pad[2 * (4 - axis)] = r
        pad[2 * (4 - axis) + 1] = r
        f = F.conv3d(F.pad(f, pad, mode="reflect"), k.view(shape_k))
    f = f.view(d, h, w)
    flat = f.reshape(-1)
    sample = flat if flat.numel() <= (1 << 26) else flat[:: 8]
    k = max(1, int(round((1.0 - bvtv) * (sample.numel() - 1))) + 1)
    thr = torch.kthvalue(sample, k).values
    bone = torch.where(f > thr, 255, 0).to(torch.uint8)
    del f, flat, sample
    if roi_kind == "cylinder":
        yy = torch.arange(h, device=device, dtype=torch.float64).view(h, 1)
        xx = torch.arange(w, device=device, dtype=torch.float64).view(1, w)
        disk = ((xx - (w - 1) / 2.0) ** 2 + (yy - (h - 1) / 2.0) ** 2) <= roi_radius * roi_radius
        roi = disk.view(1, h, w).expand(d, h, w).to(torch.uint8).contiguous()
    elif roi_kind == "sphere":
        zz = torch.arange(d, device=device, dtype=torch.float64).view(d, 1, 1)
        yy = torch.arange(h, device=device, dtype=torch.float64).view(1, h, 1)
        xx = torch.arange(w, device=device, dtype=torch.float64).view(1, 1, w)
        roi = (((xx - (w - 1) / 2.0) ** 2 + (yy - (h - 1) / 2.0) ** 2 + (zz - (d - 1) / 2.0) ** 2)
               <= roi_radius * roi_radius).to(torch.uint8)
    else:
        roi = torch.ones((d, h, w), device=device, dtype=torch.uint8)
    meta = dict(shape=tuple(shape), sigma=sigma, bvtv=bvtv, roi=roi_kind, roi_radius=roi_radius,
                spacing_um=spacing_um, seed=seed, generator="torch")
    if to_host:
        return Specimen(bone.cpu().numpy(), roi.cpu().numpy(), spacing_um, meta)
    return Specimen(bone, roi, spacing_um, meta)


def serving_specs(n: int = 24, edge_lo: int = 64, edge_hi: int = 768, seed: int = 1005):
    """Request sizes for the serving workload: per-axis edges log-uniform in
    [edge_lo, edge_hi], the batch distributions for sigma / BV/TV / spacing."""
    return batch_specs(n, edge_lo, edge_hi, seed)
