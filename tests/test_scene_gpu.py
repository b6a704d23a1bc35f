"""Two-level traversal (TLAS over instances, HitClosest / HitAny with
CheckInstance) on the GPU against the oracle's restatement, bit for bit:
triangle index, instance index, t, u, v and occlusion, under instance
transforms (rotation, non-uniform scale, translation) and cull masks."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, MASK_ALL, MASK_SHADOW, scenes

pytestmark = pytest.mark.gpu


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def make_meshes():
    tris_a = scenes.random_triangles(4000, seed=301)
    grid, _ = scenes.terrain_boxes(seed=302, grid=32, extent=4.0, n_boxes=3)
    tris_c = scenes._box_triangles(np.array([-0.5, -0.5, -0.5], np.float32), np.array([0.5, 0.5, 0.5], np.float32))
    out = []
    for t in (tris_a, grid, tris_c):
        b = BVH(t)
        out.append((b, b.pack_triangles()))
    return out


def build_scene(ctx, meshes, n_inst, seed):
    rng = np.random.default_rng(seed)
    mids = [ctx.upload_mesh(b.nodes, gt) for b, gt in meshes]
    insts, boxes = [], []
    masks = [MASK_ALL, MASK_ALL | MASK_SHADOW, MASK_SHADOW, MASK_ALL | MASK_SHADOW]
    for i in range(n_inst):
        k = int(rng.integers(len(meshes)))
        R = random_rotation(rng)
        S = np.diag(rng.uniform(0.5, 2.0, 3)) if i % 3 else np.eye(3) * rng.uniform(0.5, 2.0)
        M = np.eye(4)
        M[:3, :3] = R @ S
        M[:3, 3] = rng.uniform(-10, 10, 3)
        insts.append(atlas_rt.make_instance(M, mids[k], masks[i % len(masks)], material_offset=k))
        lo, hi = atlas_rt.mesh_bounds(meshes[k][0])
        boxes.append(atlas_rt.transform_aabb(lo, hi, M))
    insts = np.array(insts, atlas_rt.INSTANCE_DTYPE)
    boxes = np.array(boxes, np.float32)
    order = ctx.scene_build(insts, boxes)
    # the same top level on the host, for the oracle
    top = BVH(boxes_only=boxes)
    assert np.array_equal(order, top.order)
    ordered = insts[top.order].copy()
    ordered["nextInstance"] = np.where(top.end_of_node > 0, -1, np.arange(len(ordered)) + 1)
    oracle_meshes = [(b.nodes_f32, gt) for b, gt in meshes]
    return top, ordered, oracle_meshes


def scene_rays(n, seed, radius=25.0):
    o, d = scenes.sphere_rays(n, seed=seed, radius=radius, center=(0.0, 0.0, 0.0))
    tgt = np.random.default_rng(seed).uniform(-10, 10, (n, 3)).astype(np.float32)
    d = scenes._normalize(tgt - o)
    return o, d


@pytest.mark.parametrize("n_inst,seed", [(1, 11), (2, 12), (37, 13), (200, 14)])
@pytest.mark.parametrize("cull", [0xFFFFFFFF, MASK_ALL, MASK_SHADOW])
def test_scene_bitwise_vs_oracle(n_inst, seed, cull):
    ctx = atlas_rt.Context(device=0)
    try:
        meshes = make_meshes()
        top, ordered, om = build_scene(ctx, meshes, n_inst, seed)
        o, d = scene_rays(30000, seed + 100)
        tmin, tmax = 1e-4, 1e3
        rays8 = scenes.rays8(o, d, tmin, tmax)
        packed = scenes.pack_rays(o, d)
        hits = ctx.trace_scene_closest(packed, tmin, tmax, cull)
        occ = ctx.trace_scene_any(packed, tmin, tmax, cull)
        ptr, ino, tuv = pyoracle.scene_closest_glsl(top.nodes_f32, ordered, om, rays8, cull)
        assert np.array_equal(hits["triPtr"], ptr), f"{np.sum(hits['triPtr'] != ptr)} triangle mismatches"
        assert np.array_equal(hits["instance"], ino)
        assert np.array_equal(hits["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
        hit = ptr >= 0
        assert np.array_equal(hits["u"][hit].view(np.uint32), tuv[hit, 1].view(np.uint32))
        assert np.array_equal(hits["v"][hit].view(np.uint32), tuv[hit, 2].view(np.uint32))
        occ_ref = pyoracle.scene_any_glsl(top.nodes_f32, ordered, om, rays8, cull)
        assert np.array_equal(occ, occ_ref)
        if cull != MASK_SHADOW and n_inst >= 37:
            assert hit.mean() > 0.05
        # masked-out instances are never reported
        if hit.any():
            m = ordered["mask"][hits["instance"][hit]]
            assert np.all((m & cull) != 0)
    finally:
        ctx.close()


def test_single_identity_instance_matches_blas_trace():
    """With one identity instance the scene query returns the mesh query's
    hits (the engine's traversal always runs through the top level)."""
    ctx = atlas_rt.Context(device=0)
    try:
        tris = scenes.random_triangles(20000, seed=401)
        b = BVH(tris)
        gt = b.pack_triangles()
        mid = ctx.upload_mesh(b.nodes, gt)
        lo, hi = atlas_rt.mesh_bounds(b)
        inst = np.array([atlas_rt.make_instance(np.eye(4), mid)], atlas_rt.INSTANCE_DTYPE)
        order = ctx.scene_build(inst, np.concatenate([lo, hi])[None, :])
        assert list(order) == [0, 0]   # the reference lists a single instance twice
        o, d = scenes.sphere_rays(100000, seed=402)
        packed = scenes.pack_rays(o, d)
        a = ctx.trace_closest(mid, packed, 1e-4, 10.0)
        s = ctx.trace_scene_closest(packed, 1e-4, 10.0)
        assert np.array_equal(a["triPtr"], s["triPtr"])
        assert np.array_equal(a["t"].view(np.uint32), s["t"].view(np.uint32))
        assert np.all(s["instance"][s["triPtr"] >= 0] == 0)
        assert np.array_equal(ctx.trace_any(mid, packed, 1e-4, 10.0), ctx.trace_scene_any(packed, 1e-4, 10.0))
    finally:
        ctx.close()


def test_scene_validation():
    ctx = atlas_rt.Context(device=0)
    try:
        b = BVH(scenes.random_triangles(50, seed=501))
        mid = ctx.upload_mesh(b.nodes, b.pack_triangles())
        inst = np.array([atlas_rt.make_instance(np.eye(4), mid)] * 3, atlas_rt.INSTANCE_DTYPE)
        top = BVH(boxes_only=np.array([[0, 0, 0, 1, 1, 1], [2, 0, 0, 3, 1, 1], [4, 0, 0, 5, 1, 1]], np.float32))
        bad = top.nodes.copy()
        bad[0]["leftPtr"] = ~7                      # instance index out of range
        with pytest.raises(atlas_rt.AeRtError) as e:
            ctx.scene_set(bad, inst)
        assert e.value.status == 2
        inst2 = inst.copy()
        inst2["meshOffset"][1] = 99                 # unknown mesh
        with pytest.raises(atlas_rt.AeRtError) as e:
            ctx.scene_set(top.nodes, inst2)
        assert e.value.status == 1
        with pytest.raises(atlas_rt.AeRtError):
            atlas_rt.Context(device=0).trace_scene_closest(np.zeros((4, 12), np.float32), 0.0, 1.0)
    finally:
        ctx.close()
