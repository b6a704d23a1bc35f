"""The transparency traversal variants on the GPU against the oracle, bit for
bit: HitClosestTransparency (triangle, instance, t, u, v) and
HitAnyTransparency (the returned transparency) over multi-instance scenes
with transforms, cull masks, per-triangle opacities and material opacities
(negative stored opacity), with and without opacity textures (random UVs
in and beyond [0, 1], R8 / RGBA8 / R32F texels, invertUVs, out-of-range
texture indices)."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, MASK_ALL, MASK_SHADOW, MATERIAL_DTYPE, scenes

from test_scene_gpu import random_rotation, scene_rays

pytestmark = pytest.mark.gpu


def materials(n, rng):
    m = np.zeros(n, MATERIAL_DTYPE)
    m["opacity"] = rng.uniform(0.0, 1.0, n)
    for t in ("baseColorTexture", "opacityTexture", "normalTexture", "roughnessTexture", "metalnessTexture",
              "aoTexture"):
        m[t] = -1
    return m


def textures(rng):
    return [rng.integers(0, 256, (16, 32), dtype=np.uint8),
            rng.integers(0, 256, (8, 5, 4), dtype=np.uint8),
            rng.uniform(-0.2, 1.2, (33, 7)).astype(np.float32)]


def build(ctx, n_inst, seed, textured=False):
    rng = np.random.default_rng(seed)
    srcs = [scenes.random_triangles(3000, seed=seed + 1),
            scenes.terrain_boxes(seed=seed + 2, grid=24, extent=4.0, n_boxes=3)[0],
            scenes._box_triangles(np.array([-0.5, -0.5, -0.5], np.float32), np.array([0.5, 0.5, 0.5], np.float32))]
    meshes, mids = [], []
    for k, t in enumerate(srcs):
        b = BVH(t)
        n = len(t)
        op = rng.uniform(0.0, 1.0, n).astype(np.float32)
        kind = rng.integers(0, 3, n)
        op[kind == 0] = -1.0                     # material opacity
        op[kind == 1] = 0.0                      # clear
        mat = rng.integers(0, 4, n).astype(np.int32)
        gt = b.pack_triangles(mat, op)
        sh = b.pack_shading(None, mat, op)
        if textured:
            b.pack_uvs(sh, rng.uniform(-1.5, 2.5, (n, 6)).astype(np.float32))
        mids.append(ctx.upload_mesh(b.nodes, gt, sh))
        meshes.append((b, gt, sh))
    insts, boxes = [], []
    masks = [MASK_ALL, MASK_ALL | MASK_SHADOW, MASK_SHADOW]
    for i in range(n_inst):
        k = int(rng.integers(len(meshes)))
        M = np.eye(4)
        M[:3, :3] = random_rotation(rng) @ np.diag(rng.uniform(0.5, 2.0, 3))
        M[:3, 3] = rng.uniform(-10, 10, 3)
        insts.append(atlas_rt.make_instance(M, mids[k], masks[i % 3], material_offset=4 * k))
        lo, hi = atlas_rt.mesh_bounds(meshes[k][0])
        boxes.append(atlas_rt.transform_aabb(lo, hi, M))
    insts = np.array(insts, atlas_rt.INSTANCE_DTYPE)
    boxes = np.array(boxes, np.float32)
    ctx.scene_build(insts, boxes)
    mats = materials(12, rng)
    tex = None
    if textured:
        tex = textures(rng)
        mats["opacityTexture"] = rng.integers(-1, 4, len(mats))     # 3: out of range, samples 1.0
        mats["invertUVs"] = rng.integers(0, 2, len(mats))
        ctx.set_textures(tex)
    ctx.set_materials(mats)
    top = BVH(boxes_only=boxes)
    ordered = insts[top.order].copy()
    ordered["nextInstance"] = np.where(top.end_of_node > 0, -1, np.arange(len(ordered)) + 1)
    om = [(b.nodes_f32, gt, sh) for b, gt, sh in meshes]
    return top, ordered, om, mats, tex


@pytest.mark.parametrize("n_inst,seed", [(1, 21), (9, 22), (60, 23)])
@pytest.mark.parametrize("cull", [0xFFFFFFFF, MASK_SHADOW])
@pytest.mark.parametrize("textured", [False, True])
def test_transparency_bitwise_vs_oracle(n_inst, seed, cull, textured):
    ctx = atlas_rt.Context(device=0)
    try:
        top, ordered, om, mats, tex = build(ctx, n_inst, seed, textured)
        o, d = scene_rays(20000, seed + 100)
        tmin, tmax = 1e-4, 1e3
        rays8 = scenes.rays8(o, d, tmin, tmax)
        packed = scenes.pack_rays(o, d)
        hits = ctx.trace_scene_closest_transparency(packed, tmin, tmax, cull)
        tr = ctx.trace_scene_any_transparency(packed, tmin, tmax, cull)
        ctx.synchronize()
        ptr, ino, tuv = pyoracle.scene_closest_transparency_glsl(top.nodes_f32, ordered, om, mats, rays8, cull,
                                                                 textures=tex)
        ref_t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, ordered, om, mats, rays8, cull, textures=tex)
        np.testing.assert_array_equal(hits["triPtr"], ptr)
        np.testing.assert_array_equal(hits["instance"], np.where(ptr >= 0, ino, -1))
        hit = ptr >= 0
        np.testing.assert_array_equal(hits["t"][hit], tuv[hit, 0])
        np.testing.assert_array_equal(hits["u"][hit], tuv[hit, 1])
        np.testing.assert_array_equal(hits["v"][hit], tuv[hit, 2])
        np.testing.assert_array_equal(tr, ref_t)
        if n_inst > 1:
            assert hit.mean() > 0.01
            assert 0.02 < (tr < 1.0).mean() and (tr > 0.0).any()
    finally:
        ctx.close()
