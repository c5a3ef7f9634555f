"""The chain passes' method, checked on the CPU against the oracle: the
non-selected voxels a ridge sphere reaches, and their max r^2, follow from
pushing each ridge's r^2 backwards through the tied argmins of the separable
EDT's z, y and x passes (the library's chain_z / chain_y kernels).  numpy on
small specimens; the GPU parity tests check the kernels themselves."""

import numpy as np
import pytest

import oracle as O
from bone_morphometry_gb300 import synthetic as S

BIG = 1 << 40  # "no site"


def passes(sel):
    """f, g, m: the x, y and z pass outputs of the separable squared EDT."""
    d, h, w = sel.shape
    f = np.full(sel.shape, BIG, np.int64)
    xs = np.arange(w)
    for z in range(d):
        for y in range(h):
            s = np.nonzero(~sel[z, y])[0]
            if s.size:
                f[z, y] = ((xs[:, None] - s[None, :]) ** 2).min(1)

    def line_pass(inp, axis):
        a = np.moveaxis(inp, axis, -1)
        q = np.arange(a.shape[-1])
        out = (a[..., None, :] + (q[:, None] - q[None, :]) ** 2).min(-1)
        return np.moveaxis(np.minimum(out, BIG), -1, axis)

    g = line_pass(f, 1)
    return f, g, line_pass(g, 0)


def push_back(v, inp, out, axis):
    """max of v(q) over the outputs q whose minimum inp(p) + (q - p)^2 = out(q)
    is attained at p, for every p of every line along axis."""
    a_in, a_out, a_v = (np.moveaxis(t, axis, -1) for t in (inp, out, v))
    q = np.arange(a_in.shape[-1])
    hit = (a_in[..., None, :] + (q[:, None] - q[None, :]) ** 2) == a_out[..., :, None]  # [..., q, p]
    return np.moveaxis(np.where(hit & (a_v[..., :, None] > 0), a_v[..., :, None], 0).max(-2), -1, axis)


@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("select_bone", [True, False])
def test_sites_by_chains_match_ball_fill(seed, select_bone):
    sp = S.make_specimen((18, 22, 26), 2.0, 0.3, "cylinder", 9.0, 12.0, seed)
    m8 = O.phase_inside(sp.bone, sp.roi, select_bone)
    sel = m8 != 0
    f, g, m = passes(sel)
    sq = O.edt_sq(m8, O.FOREGROUND).astype(np.int64)
    assert np.array_equal(np.where(sel, m, 0), sq)
    idx, r2 = O.distance_ridges(m8, O.FOREGROUND, sq.astype(np.uint32))
    v = np.zeros(sel.size, np.int64)
    v[idx] = r2
    chain = push_back(v.reshape(sel.shape), g, m, 0)          # chain_z
    u = push_back(chain, f, g, 1)                              # chain_y ...
    sites = push_back(u, np.where(sel, BIG, 0), f, 2)          # ... and its x step
    ref = O.propagate(sel.shape, idx, r2).astype(np.int64)     # the reference's max over balls
    assert (sites[sel] == 0).all()                             # chains end on non-selected voxels only
    assert np.array_equal(sites[~sel], ref[~sel])
    assert (ref[~sel] > 0).sum() > 0
