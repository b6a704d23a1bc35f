"""Inputs of the pass tests (RTAO, reflections, RTGI, DDGI probe rays): the
path tracer's terrain-and-boxes scene at a small size, and G-buffers in the
engine's form -- NDC depth, octahedral view-space normals
(EncodeNormal, common/normalencode.hsh:3-16), inverse projection and view --
rendered with the oracle's closest-hit traversal."""
import numpy as np

import atlas_rt
import pyoracle
from atlas_rt import BVH, ptscene, scenes
from atlas_rt.gbuffer import encode_normal, look_at, perspective, view_rays


def small_scene(seed=7, cull_terrain_backfaces=False):
    sc = ptscene.build(seed=seed, grid=48, n_boxes=12)
    if cull_terrain_backfaces:
        sc["materials"][0]["twoSided"] = 0
        sc["materials"][0]["cullBackFaces"] = 1
    bvh = sc["bvh"]
    gt = bvh.pack_triangles(sc["obj"])
    shading = bvh.pack_shading(sc["normals"], sc["obj"])
    lights = ptscene.lights_for(sc, shading)
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(bvh)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    ordered = inst[top.order].copy()
    model = np.tile(np.eye(3, 4, dtype=np.float32).reshape(-1), (len(ordered), 1))
    oracle_scene = (top.nodes_f32, ordered, model, [(bvh.nodes_f32, gt, shading)], sc["materials"], lights)
    return {"sc": sc, "gt": gt, "shading": shading, "lights": lights, "boxes": np.concatenate([lo, hi])[None, :],
            "oracle": oracle_scene}


def upload(ctx, s):
    bvh = s["sc"]["bvh"]
    mid = ctx.upload_mesh(bvh.nodes, s["gt"], s["shading"])
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    ctx.scene_build(inst, s["boxes"])
    ctx.set_materials(s["sc"]["materials"])
    ctx.set_lights(s["lights"])


def gbuffer(s, w, h, eye=(50.0, 40.0, -15.0), target=(50.0, 0.0, 50.0), up=(0.0, 1.0, 0.0), half_res=False,
            seed=3, roughness=None, samples=False):
    """A G-buffer of the scene seen from `eye`.  With half_res, the depth
    comes from the pixel of each 2x2 block that `offset` names."""
    rng = np.random.default_rng(seed)
    V = look_at(eye, target, up)
    P = perspective(60.0, w / h, 0.5, 400.0)
    offset = rng.integers(0, 4, w * h).astype(np.uint8) if half_res else None
    o, d = view_rays(V, P, w, h, offset)
    rays8 = scenes.rays8(o.astype(np.float32), d.astype(np.float32), 0.0, 1e12)
    tl, inst, model, meshes, mats, lights = s["oracle"]
    ptr, ino, tuv = pyoracle.scene_closest_glsl(tl, inst, meshes, rays8)
    hit = ptr >= 0
    pos = o + d * tuv[:, :1].astype(np.float64)
    clip = np.concatenate([pos, np.ones((len(pos), 1))], axis=1) @ (P @ V).T
    depth = np.where(hit, clip[:, 2] / clip[:, 3], 1.0)
    sh = s["shading"]
    tri = sh[np.maximum(ptr, 0)]
    n = np.cross(tri[:, 4:7] - tri[:, 0:3], tri[:, 8:11] - tri[:, 0:3]).astype(np.float64)
    n /= np.linalg.norm(n, axis=1, keepdims=True) + 1e-30
    n *= np.where((n * d).sum(axis=1, keepdims=True) > 0, -1.0, 1.0)
    nv = n @ V[:3, :3].T
    nv /= np.linalg.norm(nv, axis=1, keepdims=True) + 1e-30
    enc = np.where(hit[:, None], encode_normal(nv), 0.0)
    gb = {"depth": depth.astype(np.float32).reshape(h, w), "normal": enc.astype(np.float32).reshape(h, w, 2),
          "half_res": int(half_res), "ip_matrix": np.linalg.inv(P), "iv_matrix": np.linalg.inv(V)}
    if half_res:
        gb["offset"] = offset.reshape(h, w)
    if roughness is not None:
        gb["roughness"] = roughness.astype(np.float32).reshape(h, w)
    if samples:
        gb["samples"] = rng.random((h, w, 2), dtype=np.float32) * np.float32(0.999)
    return gb


def to_device(gb):
    import torch
    out = {}
    for k, v in gb.items():
        out[k] = torch.from_numpy(np.ascontiguousarray(v)).cuda() if k in (
            "depth", "normal", "offset", "roughness", "samples") else v
    return out


def fibonacci_dirs(n):
    """Spherical Fibonacci directions (n, 4), w = 0."""
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    theta = np.pi * (1 + 5 ** 0.5) * i
    d = np.stack([np.cos(theta) * np.sin(phi), np.cos(phi), np.sin(theta) * np.sin(phi), np.zeros(n)], axis=1)
    return d.astype(np.float32)


def unpack_ray_hits(h):
    """UnpackRayHit (ddgi.hsh:70-83): direction (n, 3), radiance (n, 3), distance (n,)."""
    bits = h.view(np.uint32)
    lo = (bits[:, :3] & 0xFFFF).astype(np.uint16).view(np.float16).astype(np.float32)
    hi = (bits[:, :3] >> 16).astype(np.uint16).view(np.float16).astype(np.float32)
    direction = np.stack([lo[:, 0], hi[:, 0], lo[:, 2]], axis=1)
    radiance = np.stack([lo[:, 1], hi[:, 1], hi[:, 2]], axis=1)
    return direction, radiance, h[:, 3]
