"""AE_RT_CFG_APPROXIMATE: the approximate traversal (conservative approximate
box tests, one-reciprocal triangle tests) against the exact one -- the
shader's traversal bit for bit -- on the same rays: the same hit or miss and
the same triangle for all but grazing rays and exact ties, distances and
barycentrics of the same triangle within 1.5 units of 2^-24 (one rounding of
the reciprocal; the tests allow 2.4e-7 relative), occlusion the same, and the
near-tie flag only where a second hit lies within 1e-6 relative t."""
import numpy as np
import pytest

import atlas_rt
from atlas_rt import BVH, HIT_FLAG_NEAR_TIE, scenes

pytestmark = pytest.mark.gpu


def compare(he, ha, oe, oa):
    hit_e, hit_a = he["triPtr"] >= 0, ha["triPtr"] >= 0
    assert (hit_e == hit_a).mean() > 0.9995
    both = hit_e & hit_a
    same = he["triPtr"][both] == ha["triPtr"][both]
    assert same.mean() > 0.999
    # a different triangle only where the distances (nearly) tie
    np.testing.assert_allclose(ha["t"][both], he["t"][both], rtol=2e-5)
    # t, u, v of the same triangle: one rounding of the reciprocal apart
    np.testing.assert_allclose(ha["t"][both][same], he["t"][both][same], rtol=2.4e-7)
    np.testing.assert_allclose(ha["u"][both][same], he["u"][both][same], rtol=2.4e-7, atol=1e-30)
    np.testing.assert_allclose(ha["v"][both][same], he["v"][both][same], rtol=2.4e-7, atol=1e-30)
    # the near-tie flag as with AE_RT_CFG_NO_NEAR_TIES: a second accepted
    # triangle within 1e-6 relative t
    flagged = (ha["flags"] & HIT_FLAG_NEAR_TIE) != 0
    assert np.all(ha["tSecond"][flagged] - ha["t"][flagged] <= np.float32(1e-6) * ha["t"][flagged])
    assert (oe == oa).mean() > 0.9995
    assert hit_e.mean() > 0.3 and oe.mean() > 0.1


@pytest.mark.parametrize("rays", ["camera", "sphere"])
def test_approximate_mesh_traces_match_exact(rays):
    tris, _ = scenes.terrain_boxes(grid=128, extent=100.0, n_boxes=60)
    b = BVH(tris)
    gt = b.pack_triangles()
    if rays == "camera":
        o, d = scenes.pinhole_rays(scenes.pinhole_camera(640, 360))
    else:
        # from a sphere around the terrain to random points above it: grazing
        # and steep rays of every direction
        rng = np.random.default_rng(5)
        u = rng.normal(size=(200_000, 3))
        o = np.array([50.0, 5.0, 50.0]) + 90.0 * u / np.linalg.norm(u, axis=1, keepdims=True)
        tgt = np.stack([rng.uniform(0, 100, 200_000), rng.uniform(0, 15, 200_000), rng.uniform(0, 100, 200_000)], 1)
        d = (tgt - o) / np.linalg.norm(tgt - o, axis=1, keepdims=True)
    packed = scenes.pack_rays(o.astype(np.float32), d.astype(np.float32))
    res = []
    for approx in (False, True):
        ctx = atlas_rt.Context(device=0, approximate=approx)
        try:
            m = ctx.upload_mesh(b.nodes, gt)
            res.append((ctx.trace_closest(m, packed, 1e-4, 1e4), ctx.trace_any(m, packed, 1e-4, 1e4)))
        finally:
            ctx.close()
    compare(res[0][0], res[1][0], res[0][1], res[1][1])


def test_approximate_scene_traces_match_exact():
    """A two-level scene of instanced meshes under rotations and scales."""
    meshes, boxes, insts = [], [], []
    rng = np.random.default_rng(3)
    srcs = [scenes.terrain_boxes(seed=11, grid=32, extent=20.0, n_boxes=8)[0], scenes.random_triangles(3000, seed=4)]
    bvhs = [BVH(t) for t in srcs]
    for k in range(6):
        mi = k % 2
        M = np.eye(4)
        a = rng.uniform(0, 2 * np.pi)
        M[:3, :3] = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]) * rng.uniform(0.5, 3)
        M[:3, 3] = rng.uniform(-30, 30, 3)
        insts.append(atlas_rt.make_instance(M, mi, atlas_rt.MASK_ALL))
        lo, hi = atlas_rt.mesh_bounds(bvhs[mi])
        boxes.append(atlas_rt.transform_aabb(lo, hi, M))
    insts = np.array(insts, atlas_rt.INSTANCE_DTYPE)
    u = rng.normal(size=(100_000, 3))
    o = 80.0 * u / np.linalg.norm(u, axis=1, keepdims=True)
    tgt = np.array(boxes, np.float64).reshape(-1, 2, 3).mean(axis=1)[rng.integers(0, 6, 100_000)]
    tgt += rng.normal(0.0, 3.0, tgt.shape)
    d = (tgt - o) / np.linalg.norm(tgt - o, axis=1, keepdims=True)
    packed = scenes.pack_rays(o.astype(np.float32), d.astype(np.float32))
    res = []
    for approx in (False, True):
        ctx = atlas_rt.Context(device=0, approximate=approx)
        try:
            for bv in bvhs:
                ctx.upload_mesh(bv.nodes, bv.pack_triangles())
            ctx.scene_build(insts, np.array(boxes, np.float32))
            h = ctx.trace_scene_closest(packed, 1e-4, 1e4)
            oc = ctx.trace_scene_any(packed, 1e-4, 1e4)
            ctx.synchronize()
            res.append((h, oc))
        finally:
            ctx.close()
    compare(res[0][0], res[1][0], res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][0]["instance"][res[0][0]["triPtr"] >= 0][:10],
                                  res[1][0]["instance"][res[0][0]["triPtr"] >= 0][:10])
