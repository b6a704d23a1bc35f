"""The path-traced terrain + boxes scene: geometry, materials, the area light
and the engine-side records the path tracer reads.

* Geometry: the terrain + boxes scene of scenes.terrain_boxes plus one 4 x 4
  rectangular area light (two triangles) at height 60 facing down.
* Materials (GPUMaterial), one per object, seeded: the terrain and about half
  of the boxes are diffuse ("Lambertian": metalness 0, no specular
  reflectance), the other boxes GGX metals (metalness 1, roughness uniform in
  [0.05, 1]); albedo uniform in [0.1, 0.9] per channel; the light has
  emissive radiance 20 and no reflectance.  All two-sided.
* Lights: one GPULight per emissive triangle, as
  RayTracingWorld::BuildTriangleLightsForMesh (RayTracingWorld.cpp:322-376)
  and RayTracingHelper::UpdateLights (selection pdf 1 when all lights fit)
  build them.
"""
from __future__ import annotations

import numpy as np

from . import BVH, MASK_ALL, MASK_SHADOW, MATERIAL_DTYPE, make_instance, mesh_bounds, scenes

F32 = np.float32


def _bits(x, dtype=np.int32):
    return np.asarray(x, dtype).view(F32)


def _unpack10(bits):
    c = np.asarray(bits, F32).view(np.int32)
    return np.stack([((c >> s) & 1023).astype(F32) / F32(1023.0) * F32(2.0) - F32(1.0) for s in (0, 10, 20)], -1)


def build(seed: int = scenes.DEFAULT_SEED, light_center=(50.0, 60.0, 50.0), light_size: float = 4.0,
          radiance: float = 20.0, grid: int = 512, n_boxes: int = 200):
    """Returns a dict with the triangles, per-triangle object ids, normals,
    materials and the BVH, ready for upload()."""
    tris, obj = scenes.terrain_boxes(seed=seed, grid=grid, n_boxes=n_boxes)
    cx, cy, cz = light_center
    h = light_size / 2
    q = np.array([[cx - h, cy, cz - h], [cx + h, cy, cz - h], [cx + h, cy, cz + h], [cx - h, cy, cz + h]], F32)
    light = np.stack([q[[0, 1, 2]], q[[0, 2, 3]]]).astype(F32)
    light_obj = n_boxes + 1
    tris = np.concatenate([tris, light]).astype(F32)
    obj = np.concatenate([obj, np.full(2, light_obj, np.int32)])
    # face normals (terrain up, boxes outward), the light facing down
    e0 = tris[:, 1] - tris[:, 0]
    e1 = tris[:, 2] - tris[:, 0]
    n = np.cross(e0, e1)
    n /= np.linalg.norm(n, axis=1, keepdims=True) + 1e-30
    n[-2:] = [0.0, -1.0, 0.0]
    normals = np.repeat(n[:, None, :], 3, axis=1).astype(F32)

    rng = np.random.Generator(np.random.PCG64(seed + 31))
    mats = np.zeros(light_obj + 1, MATERIAL_DTYPE)
    mats["ID"] = np.arange(len(mats))
    mats["opacity"] = 1.0
    mats["ao"] = 1.0
    mats["normalScale"] = 1.0
    mats["twoSided"] = 1
    for t in ("baseColorTexture", "opacityTexture", "normalTexture", "roughnessTexture", "metalnessTexture",
              "aoTexture"):
        mats[t] = -1
    albedo = rng.uniform(0.1, 0.9, (len(mats), 3)).astype(F32)
    is_ggx = rng.random(len(mats)) < 0.5
    is_ggx[0] = False                       # the terrain is diffuse
    rough = rng.uniform(0.05, 1.0, len(mats)).astype(F32)
    mats["baseColor"] = albedo
    mats["metalness"] = np.where(is_ggx, 1.0, 0.0)
    mats["roughness"] = np.where(is_ggx, rough, 1.0)
    mats["reflectance"] = 0.0
    mats[light_obj]["baseColor"] = 0.0
    mats[light_obj]["emissiveColor"] = radiance
    mats[light_obj]["metalness"] = 0.0
    mats[light_obj]["roughness"] = 1.0
    bvh = BVH(tris)
    return {"tris": tris, "obj": obj, "normals": normals, "materials": mats, "bvh": bvh, "light_obj": light_obj,
            "is_ggx": is_ggx}


def lights_for(scene: dict, shading: np.ndarray, instance: int = 0) -> np.ndarray:
    """GPULight records (n, 16) float32 for the emissive triangles, in the
    BVH order of the shading triangles."""
    bvh = scene["bvh"]
    mats = scene["materials"]
    mat_of = shading[:, 15].view(np.int32)
    out = []
    for i in np.nonzero(np.any(mats["emissiveColor"][mat_of] > 0, axis=1))[0]:
        t = shading[i]
        v0, v1, v2 = t[0:3], t[4:7], t[8:11]
        nn = _unpack10(np.array([t[3], t[7], t[11]], F32))
        P = (v0 + v1 + v2) / F32(3.0)
        N = nn.mean(axis=0)
        a = np.linalg.norm(v1 - v0)
        b = np.linalg.norm(v2 - v0)
        c = np.linalg.norm(v1 - v2)
        s = 0.5 * (a + b + c)
        area = np.sqrt(max(s * (s - a) * (s - b) * (s - c), 0.0))
        rad = mats["emissiveColor"][mat_of[i]]
        rec = np.zeros(16, F32)
        rec[0:3], rec[3] = P, 1.0
        rec[4:7] = N
        rec[8:11] = rad
        rec[12] = _bits((1 << 28) | int(i), np.uint32)
        rec[13] = 1.0                       # selection pdf: every light fits the light buffer
        rec[14] = area
        rec[15] = _bits(instance, np.int32)
        out.append(rec)
    del bvh
    return np.array(out, F32).reshape(-1, 16)


def upload(ctx, scene: dict):
    """Uploads mesh, shading triangles, the one-instance scene, materials and
    lights to an atlas_rt.Context.  Returns (mesh_id, shading, lights)."""
    bvh = scene["bvh"]
    opacity = scene.get("opacity")          # per input triangle, optional (1)
    gt = bvh.pack_triangles(scene["obj"], opacity)
    shading = bvh.pack_shading(scene["normals"], scene["obj"], opacity)
    mid = ctx.upload_mesh(bvh.nodes, gt, shading)
    inst = np.array([make_instance(np.eye(4), mid, MASK_ALL | MASK_SHADOW)])
    lo, hi = mesh_bounds(bvh)
    ctx.scene_build(inst, np.concatenate([lo, hi])[None, :])
    ctx.set_materials(scene["materials"])
    lights = lights_for(scene, shading)
    ctx.set_lights(lights)
    return mid, shading, lights, gt


def rel_mse(img, ref, eps: float = 1e-2) -> float:
    """mean((x - ref)^2 / (ref^2 + eps)) over pixels and channels (eps = 1e-2)."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))
