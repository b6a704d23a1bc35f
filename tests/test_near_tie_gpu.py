"""FP64 re-test of near ties (ae_rt_retest_near_ties) against the oracle's
double-precision brute force over every triangle.

Rays aimed at shared edges and vertices of the terrain grid (and straight
down a shared triangle edge) have two or more equal nearest hits; the FP32
traversal flags them, and the re-test must name the same triangle (the
lowest BVH-order index among the equal double distances), the same distance
and the same second distance as the brute force -- bit for bit, both sides
rounding every double operation separately in the formula's order.
"""
import numpy as np
import pytest

import atlas_rt
import pyoracle
import near_tie_util as U
from atlas_rt import BVH, HIT64_DTYPE, HIT_FLAG_HIT, HIT_FLAG_NEAR_TIE, HIT_FLAG_RETESTED, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = atlas_rt.Context(device=0)
    yield c
    c.close()


def retest(ctx, tris, rays8):
    import torch
    b = BVH(tris)
    gt = b.pack_triangles()
    retest.order = b.order
    mid = ctx.upload_mesh(b.nodes, gt)
    tmin, tmax = float(rays8[0, 6]), float(rays8[0, 7])
    rays = torch.from_numpy(scenes.pack_rays(rays8[:, 0:3], rays8[:, 3:6])).cuda()
    n = len(rays8)
    hits = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
    ctx.trace_closest(mid, rays, tmin, tmax, out=hits, n_rays=n)
    out = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
    cnt = ctx.retest_near_ties(mid, rays, hits, tmin, tmax, out, n_rays=n)
    h32 = hits.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
    h64 = out.cpu().numpy().view(HIT64_DTYPE).reshape(-1)
    return gt, h32, h64, cnt


def check_against_brute(gt, rays8, h32, h64, cnt, limit=600, order=None):
    if order is None:
        order = retest.order
    flagged = np.nonzero(h32["flags"] & HIT_FLAG_NEAR_TIE)[0]
    assert cnt == len(flagged)
    # pass-through of the others
    rest = np.setdiff1d(np.arange(len(h32)), flagged)
    assert np.all(h64["triPtr"][rest] == h32["triPtr"][rest])
    assert np.all((h64["flags"][rest] & HIT_FLAG_RETESTED) == 0)
    np.testing.assert_array_equal(h64["t"][rest][h32["triPtr"][rest] >= 0],
                                  h32["t"][rest][h32["triPtr"][rest] >= 0].astype(np.float64))
    sel = flagged[:limit]
    ptr, t, t2 = pyoracle.closest_f64_brute(gt, rays8[sel])
    assert np.all(h64["flags"][sel] & HIT_FLAG_RETESTED)
    # a flagged ray may have no double-precision hit (a triangle rejected
    # within its rounding error flags the ray too)
    np.testing.assert_array_equal((h64["flags"][sel] & HIT_FLAG_HIT) != 0, ptr >= 0)
    hit = ptr >= 0
    # the same triangle (a spatial split may store it twice: compare original indices)
    np.testing.assert_array_equal(order[h64["triPtr"][sel][hit]], order[ptr[hit]])
    np.testing.assert_array_equal(h64["t"][sel][hit], t[hit])
    np.testing.assert_array_equal(h64["t_second"][sel][hit], U.windowed_second(t, t2)[hit])
    return len(flagged)


def test_retest_shared_edge(ctx):
    tris = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]],
                     [[1, 0, 0], [1, 1, 0], [0, 1, 0]]], np.float32)
    o = np.array([[0.5, 0.5, -1], [0.25, 0.25, -1], [0.75, 0.75, -1]], np.float32)
    d = np.array([[0, 0, 1]] * 3, np.float32)
    rays8 = scenes.rays8(o, d, 0.0, 10.0)
    gt, h32, h64, cnt = retest(ctx, tris, rays8)
    assert cnt == 1 and h32["flags"][0] & HIT_FLAG_NEAR_TIE
    check_against_brute(gt, rays8, h32, h64, cnt)
    # both triangles at exactly t = 1: the lower BVH index, second distance equal
    assert h64["t"][0] == 1.0 and h64["t_second"][0] == 1.0


def test_retest_terrain_grid_edges_and_vertices(ctx):
    """Tilted rays aimed at points of shared terrain edges and at shared
    vertices: their nearest hits are within float rounding of each other."""
    tris, obj = scenes.terrain_boxes()
    rng = np.random.default_rng(5)
    n = 2048
    terrain = np.nonzero(obj == 0)[0]
    pick = terrain[rng.integers(0, len(terrain), n)]
    va = tris[pick, 0].astype(np.float64)
    vb = tris[pick, 1].astype(np.float64)
    f = rng.uniform(0.2, 0.8, n)[:, None]
    target = np.where(np.arange(n)[:, None] < n // 2, va + f * (vb - va), va)
    d = np.stack([rng.uniform(-0.3, 0.3, n), -np.ones(n), rng.uniform(-0.3, 0.3, n)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = (target - 30.0 * d).astype(np.float32)
    rays8 = scenes.rays8(o, d.astype(np.float32), 1e-4, 1e4)
    gt, h32, h64, cnt = retest(ctx, tris, rays8)
    assert (h32["triPtr"] >= 0).mean() > 0.9
    flagged = check_against_brute(gt, rays8, h32, h64, cnt)
    assert flagged > 100, flagged


def test_flag_complete_and_equal_to_oracle(ctx):
    """100,000 rays aimed at terrain grid edges and vertices, box edges and
    the lines where box walls meet the terrain: the GPU's near-tie flags are
    the oracle's bit for bit, every ray whose FP64 brute-force gap is
    <= 1e-6 is flagged, and the re-test gives the brute force's answer on
    every flagged ray."""
    import near_tie_util as U
    import torch
    tris, obj = U.near_tie_scene()
    r8, lab = U.near_tie_rays(tris, obj)
    nodes, order, eon = pyoracle.build_bvh(tris)
    b = BVH(tris)
    gt = b.pack_triangles()
    assert np.array_equal(b.nodes_f32.view(np.uint32), nodes.view(np.uint32))
    mid = ctx.upload_mesh(b.nodes, gt)
    rays = torch.from_numpy(scenes.pack_rays(r8[:, 0:3], r8[:, 3:6])).cuda()
    n = len(r8)
    hits = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
    ctx.trace_closest(mid, rays, 1e-4, 1e4, out=hits, n_rays=n)
    out = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
    cnt = ctx.retest_near_ties(mid, rays, hits, 1e-4, 1e4, out, n_rays=n)
    h32 = hits.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
    h64 = out.cpu().numpy().view(HIT64_DTYPE).reshape(-1)
    p, tuv, flags, second = pyoracle.closest_glsl_ties(nodes, gt, r8)
    assert np.array_equal(h32["triPtr"], p)
    assert np.array_equal(h32["flags"] & (HIT_FLAG_HIT | HIT_FLAG_NEAR_TIE), flags)
    assert np.array_equal(h32["tSecond"].view(np.uint32), second.view(np.uint32))
    ptr, t1, t2, gap = U.brute_gaps(gt, r8)
    flagged = (h32["flags"] & HIT_FLAG_NEAR_TIE) != 0
    assert (gap <= 1e-6).sum() > 20000
    assert not np.any((gap <= 1e-6) & ~flagged)
    assert cnt == flagged.sum()
    f = np.nonzero(flagged)[0]
    hit = ptr[f] >= 0
    np.testing.assert_array_equal(h64["triPtr"][f] >= 0, hit)
    np.testing.assert_array_equal(order[h64["triPtr"][f][hit]], order[ptr[f][hit]])
    np.testing.assert_array_equal(h64["t"][f][hit], t1[f][hit])
    np.testing.assert_array_equal(h64["t_second"][f][hit], U.windowed_second(t1[f], t2[f])[hit])
    assert (np.isfinite(h64["t_second"][f][hit]) == (gap[f][hit] <= 1e-5)).mean() > 0.99


def test_no_near_ties_switch_keeps_hits():
    """A context created with AE_RT_CFG_NO_NEAR_TIES returns the same hits
    (triangle, t, u, v, second distance) as the default one; its near-tie
    flags are the ones the second accepted distance alone shows, a subset of
    the complete flags."""
    import near_tie_util as U
    import torch
    tris, obj = U.near_tie_scene()
    r8, lab = U.near_tie_rays(tris, obj)
    b = BVH(tris)
    gt = b.pack_triangles()
    rays = torch.from_numpy(scenes.pack_rays(r8[:, 0:3], r8[:, 3:6])).cuda()
    n = len(r8)
    res = []
    for near in (True, False):
        c = atlas_rt.Context(device=0, near_ties=near)
        try:
            mid = c.upload_mesh(b.nodes, gt)
            hits = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
            c.trace_closest(mid, rays, 1e-4, 1e4, out=hits, n_rays=n)
            c.synchronize()
            res.append(hits.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1))
        finally:
            c.close()
    full, off = res
    for k in ("triPtr", "t", "u", "v", "tSecond"):
        assert np.array_equal(full[k].view(np.uint32), off[k].view(np.uint32)), k
    hit = full["triPtr"] >= 0
    legacy = hit & (off["tSecond"] - off["t"] <= np.float32(1e-6) * off["t"])
    np.testing.assert_array_equal((off["flags"] & HIT_FLAG_NEAR_TIE) != 0, legacy)
    assert not np.any(((off["flags"] & HIT_FLAG_NEAR_TIE) != 0) & ((full["flags"] & HIT_FLAG_NEAR_TIE) == 0))
    assert ((full["flags"] & HIT_FLAG_NEAR_TIE) != 0).sum() > ((off["flags"] & HIT_FLAG_NEAR_TIE) != 0).sum()
