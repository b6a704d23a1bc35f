"""A textured variant of the path tracer's terrain-and-boxes scene for the
material-model tests: planar UVs, vertex colours, and per-material base
colour (RGBA8), roughness / metalness / ao (R8 and R32F) and normal-map
(RGBA8) textures, as GetSurfaceParameters reads them (surface.hsh:83-124)."""
import numpy as np

import atlas_rt
from atlas_rt import BVH, ptscene


def textures(seed=5):
    rng = np.random.default_rng(seed)
    base = rng.integers(40, 256, (32, 32, 4), dtype=np.uint8)
    rough = rng.integers(20, 256, (16, 16), dtype=np.uint8)
    metal = (np.indices((8, 8)).sum(0) % 2 * 255).astype(np.uint8)
    ao = rng.uniform(0.3, 1.0, (16, 16)).astype(np.float32)
    # normal map: tilted unit normals in [0, 1] encoding, z up
    n = np.concatenate([rng.uniform(-0.6, 0.6, (32, 32, 2)), np.ones((32, 32, 1))], axis=2)
    n /= np.linalg.norm(n, axis=2, keepdims=True)
    nm = np.concatenate([np.round((n * 0.5 + 0.5) * 255), np.full((32, 32, 1), 255)], axis=2).astype(np.uint8)
    return [base, rough, metal, ao, nm]


def build(seed=7, grid=48, n_boxes=12):
    """The scene dict of ptscene.build with its shading triangles textured,
    and the materials pointing at textures()."""
    sc = ptscene.build(seed=seed, grid=grid, n_boxes=n_boxes)
    tris = sc["tris"]
    rng = np.random.default_rng(seed + 1)
    uvs = tris[:, :, [0, 2]].reshape(-1, 6) / np.float32(7.0)      # planar x-z mapping, tiling
    colors = rng.uniform(0.4, 1.0, (len(tris), 3, 4)).astype(np.float32)
    bvh = sc["bvh"]
    gt = bvh.pack_triangles(sc["obj"])
    shading = bvh.pack_shading(sc["normals"], sc["obj"])
    bvh.pack_attributes(shading, uvs, sc["normals"], colors)
    mats = sc["materials"].copy()
    k = np.arange(len(mats))
    light = sc["light_obj"]
    mats["baseColorTexture"] = np.where(k % 3 != 2, 0, -1)
    mats["roughnessTexture"] = np.where(k % 2 == 0, 1, 4)           # 4: out of range, samples 1.0
    mats["metalnessTexture"] = np.where(k % 4 == 1, 2, -1)
    mats["aoTexture"] = np.where(k % 3 == 0, 3, -1)
    mats["normalTexture"] = np.where(k % 2 == 1, 4, -1)
    mats["normalScale"] = np.where(k % 4 == 3, 0.5, 1.0)
    mats["useVertexColors"] = k % 2
    mats["invertUVs"] = (k // 2) % 2
    for t in ("baseColorTexture", "roughnessTexture", "metalnessTexture", "aoTexture", "normalTexture"):
        mats[light][t] = -1
    mats[light]["useVertexColors"] = 0
    sc["materials"] = mats
    return sc, gt, shading, textures()


def oracle_scene(sc, gt, shading):
    bvh = sc["bvh"]
    lights = ptscene.lights_for(sc, shading)
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(bvh)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    ordered = inst[top.order].copy()
    model = np.eye(3, 4, dtype=np.float32).reshape(1, -1)
    return (top.nodes_f32, ordered, model, [(bvh.nodes_f32, gt, shading)], sc["materials"], lights), lights


def upload(ctx, sc, gt, shading, tex):
    bvh = sc["bvh"]
    mid = ctx.upload_mesh(bvh.nodes, gt, shading)
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(bvh)
    ctx.scene_build(inst, np.concatenate([lo, hi])[None, :])
    ctx.set_materials(sc["materials"])
    ctx.set_textures(tex)
    ctx.set_lights(ptscene.lights_for(sc, shading))
