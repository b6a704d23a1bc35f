"""GPU BVH build (ae_rt_mesh_build): a linear BVH made on the device in the
engine's node and triangle layouts.

* structure: a permutation of the input triangles, one per leaf, n - 1
  nodes, every node box containing its children;
* traversal on it is bit-identical to the oracle's shader restatement run
  on the same (downloaded) tree;
* against the engine's own builder's tree: every ray gets the same hit or
  miss; the nearest distance and triangle agree except for near ties.  The
  shader's closest-hit result is itself order-dependent at the ulp level: a
  triangle lying in its box's face is hit at a distance rounded differently
  from the box's entry distance, and when another hit has already brought the
  search bound between the two, the box is culled -- so which of two hits
  within an ulp or two is kept depends on the visiting order, i.e. on the
  tree.  Such rays must be near ties (relative difference <= 1e-6) and rare.
"""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, HIT_FLAG_HIT, HIT_FLAG_NEAR_TIE, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = atlas_rt.Context(device=0)
    yield c
    c.close()


def check_structure(nodes, tris_gpu, order, verts):
    n = len(verts)
    assert len(nodes) == n - 1 and len(tris_gpu) == n
    assert sorted(order.tolist()) == list(range(n))
    # triangle records: vertices of the input triangle, one per leaf
    np.testing.assert_array_equal(tris_gpu[:, 0:3], verts[order, 0])
    np.testing.assert_array_equal(tris_gpu[:, 4:7], verts[order, 1])
    np.testing.assert_array_equal(tris_gpu[:, 8:11], verts[order, 2])
    assert (tris_gpu[:, 3] > 0).all()
    # every leaf referenced once, every inner node below the root once
    seen_leaf = np.zeros(n, int)
    seen_node = np.zeros(n - 1, int)
    for side in ("leftPtr", "rightPtr"):
        p = nodes[side].astype(np.int64)
        np.add.at(seen_leaf, ~p[p < 0], 1)
        np.add.at(seen_node, p[p >= 0], 1)
    assert (seen_leaf == 1).all()
    assert seen_node[0] == 0 and (seen_node[1:] == 1).all()
    # boxes: a leaf box is its triangle's bound; inner boxes contain their children's
    lo_t = verts[order].min(axis=1)
    hi_t = verts[order].max(axis=1)
    for side, mn, mx in (("leftPtr", "leftMin", "leftMax"), ("rightPtr", "rightMin", "rightMax")):
        p = nodes[side].astype(np.int64)
        leaf = p < 0
        np.testing.assert_array_equal(nodes[mn][leaf], lo_t[~p[leaf]])
        np.testing.assert_array_equal(nodes[mx][leaf], hi_t[~p[leaf]])
        inner = ~leaf
        c = p[inner]
        cl = np.minimum(nodes["leftMin"][c], nodes["rightMin"][c])
        ch = np.maximum(nodes["leftMax"][c], nodes["rightMax"][c])
        np.testing.assert_array_equal(nodes[mn][inner], cl)
        np.testing.assert_array_equal(nodes[mx][inner], ch)


def compare_with_reference_tree(ctx, verts, rays8, mid_gpu, order_gpu):
    tmin, tmax = float(rays8[0, 6]), float(rays8[0, 7])
    pr = scenes.pack_rays(rays8[:, 0:3], rays8[:, 3:6])
    hg = ctx.trace_closest(mid_gpu, pr, tmin, tmax)
    og = ctx.trace_any(mid_gpu, pr, tmin, tmax)
    b = BVH(verts)
    gt = b.pack_triangles()
    mid_ref = ctx.upload_mesh(b.nodes, gt)
    hr = ctx.trace_closest(mid_ref, pr, tmin, tmax)
    orf = ctx.trace_any(mid_ref, pr, tmin, tmax)
    hit_g = hg["triPtr"] >= 0
    hit_r = hr["triPtr"] >= 0
    assert np.array_equal(hit_g, hit_r)
    assert np.array_equal(og, orf)
    tg = hg["t"][hit_g].astype(np.float64)
    tr = hr["t"][hit_r].astype(np.float64)
    idx_g = order_gpu[hg["triPtr"][hit_g]]
    idx_r = b.order[hr["triPtr"][hit_r]]
    differ = (idx_g != idx_r) | (tg != tr)
    assert differ.mean() < 1e-3, differ.mean()
    if differ.any():
        assert np.all(np.abs(tg - tr)[differ] <= 1e-6 * tr[differ]), "a differing hit that is not a near tie"
        # the tree that visited both hits flags the ray as a near tie
        flagged = ((hg["flags"][hit_g] | hr["flags"][hit_r]) & HIT_FLAG_NEAR_TIE) != 0
        assert flagged[differ].all(), "a differing hit on a ray neither tree flags as a near tie"
    return hit_g.mean(), int(differ.sum())


def test_random65536(ctx):
    verts = scenes.random_triangles()
    mid, order = ctx.build_mesh(verts)
    nodes, tris = ctx.mesh_bvh(mid)
    check_structure(nodes, tris, order, verts)
    o, d = scenes.sphere_rays()
    rays8 = scenes.rays8(o[:200000], d[:200000], 1e-4, 10.0)
    # traversal on the GPU tree == the oracle's shader restatement on it
    pr = scenes.pack_rays(rays8[:, 0:3], rays8[:, 3:6])
    hits = ctx.trace_closest(mid, pr, 1e-4, 10.0)
    occ = ctx.trace_any(mid, pr, 1e-4, 10.0)
    ptr, tuv = pyoracle.closest_glsl(nodes.view(np.float32).reshape(-1, 16), tris, rays8)
    assert np.array_equal(hits["triPtr"], ptr)
    assert np.array_equal(hits["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    assert np.array_equal(occ, pyoracle.any_glsl(nodes.view(np.float32).reshape(-1, 16), tris, rays8))
    rate, _ = compare_with_reference_tree(ctx, verts, rays8, mid, order)
    assert rate > 0.5


def test_terrain_boxes_and_device_input(ctx):
    import torch
    verts, _ = scenes.terrain_boxes()
    mid, order = ctx.build_mesh(torch.from_numpy(verts).cuda())
    nodes, tris = ctx.mesh_bvh(mid)
    check_structure(nodes, tris, order, verts)
    cam = scenes.pinhole_camera(480, 270)
    o, d = scenes.pinhole_rays(cam)
    rays8 = scenes.rays8(o, d, 1e-4, 1e4)
    rate, differ = compare_with_reference_tree(ctx, verts, rays8, mid, order)
    assert rate > 0.5


def test_material_opacity_and_small_meshes(ctx):
    verts = scenes.random_triangles(1000, seed=9)
    mat = np.arange(1000, dtype=np.int32) * 3
    op = np.linspace(0, 1, 1000).astype(np.float32)
    mid, order = ctx.build_mesh(verts, mat, op)
    _, tris = ctx.mesh_bvh(mid)
    np.testing.assert_array_equal(tris[:, 7].view(np.int32), mat[order])
    np.testing.assert_array_equal(tris[:, 11], op[order])
    for n in (0, 1, 2, 3):
        v = scenes.random_triangles(max(n, 1), seed=40 + n)[:n]
        m, order = ctx.build_mesh(v)
        nodes, tris = ctx.mesh_bvh(m)
        o = np.tile(np.array([[0.5, 0.5, -2.0]], np.float32), (64, 1))
        tgt = np.random.default_rng(n).uniform(0, 1, (64, 3)).astype(np.float32)
        dd = tgt - o
        dd /= np.linalg.norm(dd, axis=1, keepdims=True)
        rays8 = scenes.rays8(o, dd.astype(np.float32), 1e-4, 10.0)
        hits = ctx.trace_closest(m, scenes.pack_rays(o, dd.astype(np.float32)), 1e-4, 10.0)
        if n == 0:
            assert len(nodes) == 0 and (hits["triPtr"] < 0).all()
            continue
        ref_ptr, _, _ = pyoracle.closest_f64_brute(BVH(v).pack_triangles(), rays8)
        assert np.array_equal(hits["triPtr"] >= 0, ref_ptr >= 0)


def test_degenerate_centroids(ctx):
    """All triangles share one centroid (equal Morton codes): the index part
    of the keys still gives a valid, balanced tree."""
    base = scenes.random_triangles(1, seed=5)[0]
    rng = np.random.default_rng(6)
    verts = np.repeat(base[None], 4096, axis=0).astype(np.float32)
    jitter = rng.uniform(-1e-3, 1e-3, (4096, 3, 3)).astype(np.float32)
    verts = (verts + jitter - jitter.mean(axis=1, keepdims=True)).astype(np.float32)
    mid, order = ctx.build_mesh(verts)
    nodes, tris = ctx.mesh_bvh(mid)
    check_structure(nodes, tris, order, verts)
