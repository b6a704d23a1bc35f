"""Writes tests/golden/glsl_shading.npz: golden vectors of the engine's shading
math and scene traversal, produced by the reference's own GLSL
(data/shader/brdf/*.hsh, raytracer/lights.hsh, raytracer/intersections.hsh,
raytracer/bvh.hsh, common/random.hsh, pathtracer/rayGen.csh) compiled on the
host by the recipe oracle/glsl/make_ref.py.  The ray-generation goldens
(raygen_*) are whole dispatches of rayGen.csh.  The traversal goldens
(trav_*) are traced over
traversal_scene(), a seeded scene in the engine's buffer layouts, whose
digest the fixture keeps so that the tests can rebuild the same scene.

Needs the reference tree (this container); the fixture it writes is what the
tests compare the oracle's restatement and the GPU's device functions with.

    python tests/golden/gen_glsl_goldens.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
OUT = REPO / "tests" / "golden" / "glsl_shading.npz"
F32 = np.float32


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _hemi(rng, N, lo=0.02):
    """Unit vectors in the hemisphere around N with cos >= lo."""
    out = np.empty_like(N)
    for i in range(len(N)):
        while True:
            v = rng.normal(size=3)
            v /= np.linalg.norm(v)
            c = v @ N[i]
            if c < 0:
                v, c = -v, -c
            if c >= lo:
                out[i] = v
                break
    return out


def inputs(seed=20261204, n=512):
    """Seeded input rows of every golden set (float32)."""
    rng = np.random.default_rng(seed)
    N = _unit(rng, n)
    V = _hemi(rng, N)
    L = _hemi(rng, N, lo=-0.3)              # a few below the surface: NdotL saturates at 0
    base = rng.uniform(0.0, 1.0, (n, 3))
    rough = np.concatenate([rng.uniform(0.02, 1.0, n - 8), [0.0, 0.001, 0.05, 0.1, 0.3, 0.5, 0.9, 1.0]])
    metal = np.where(rng.random(n) < 0.4, 0.0, np.where(rng.random(n) < 0.5, 1.0, rng.random(n)))
    refl = rng.uniform(0.0, 1.0, n)
    surf = np.concatenate([V, N, L, base, rough[:, None], metal[:, None], refl[:, None]], 1).astype(F32)
    u = rng.uniform(0.0, 1.0, (n, 2)).astype(F32)
    u[:4] = [[0.0, 0.0], [0.999999, 0.5], [0.5, 0.999999], [0.25, 0.0]]
    sample = np.concatenate([surf, u], 1).astype(F32)
    # triangle lights: vertices, normals, area, r0, r1, shaded point
    v = rng.uniform(-5, 5, (n, 9))
    nn = np.concatenate([_unit(rng, n), _unit(rng, n), _unit(rng, n)], 1)
    e0, e1 = v[:, 3:6] - v[:, 0:3], v[:, 6:9] - v[:, 0:3]
    area = 0.5 * np.linalg.norm(np.cross(e0, e1), axis=1)
    light = np.concatenate([v, nn, area[:, None], rng.uniform(0, 1, (n, 2)), rng.uniform(-5, 5, (n, 3))],
                           1).astype(F32)
    # rays against triangles (half aimed inside, some at edges) and boxes
    tri = rng.uniform(-1, 1, (n, 9))
    w = rng.dirichlet([1, 1, 1], n)
    w[: n // 8] = np.stack([rng.uniform(0, 1, n // 8), np.zeros(n // 8), np.zeros(n // 8)], 1)
    w[: n // 8, 1] = 1 - w[: n // 8, 0]
    target = w[:, 0:1] * tri[:, 0:3] + w[:, 1:2] * tri[:, 3:6] + w[:, 2:3] * tri[:, 6:9]
    target[n // 2:] += rng.normal(0, 0.3, (n - n // 2, 3))
    o = rng.uniform(-4, 4, (n, 3))
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    itri = np.concatenate([o, d, tri], 1).astype(F32)
    lo = rng.uniform(-1, 0, (n, 3))
    hi = lo + rng.uniform(0, 1.5, (n, 3))
    hi[: n // 16, 1] = lo[: n // 16, 1]          # flat boxes
    bt = lo + rng.uniform(0, 1, (n, 3)) * (hi - lo)
    bt[n // 2:] += rng.normal(0, 0.5, (n - n // 2, 3))
    ob = rng.uniform(-4, 4, (n, 3))
    db = bt - ob
    db /= np.linalg.norm(db, axis=1, keepdims=True)
    tm = np.stack([np.zeros(n), np.where(rng.random(n) < 0.3, rng.uniform(1, 6, n), 1e4)], 1)
    ibox = np.concatenate([ob, db, lo, hi, tm], 1).astype(F32)
    xs = np.concatenate([np.arange(32, dtype=F32), rng.uniform(0, 4096, 32).astype(F32)])
    return {"eval_in": surf, "sample_in": sample, "light_in": light, "tri_in": itri, "box_in": ibox,
            "random_x": xs}


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def traversal_scene(seed=20261205, n_inst=12, n_rays=4096):
    """A seeded two-level scene in the engine's layouts: three meshes (random
    triangles, a terrain patch with boxes, a box) with per-triangle opacities
    (opaque, clear, partial, or the material's through a negative value),
    twelve instances with rotations, scales, translations, the three cull
    masks and material offsets, twelve materials of random opacity (some
    with an opacity texture, some with inverted UVs), three opacity textures
    (R8, RGBA8, R32F), and rays aimed into it.
    Built with the library's BVH builder (byte-identical to the reference's)
    and packers; deterministic, so the tests rebuild it."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    import atlas_rt
    from atlas_rt import BVH, MATERIAL_DTYPE, scenes
    rng = np.random.default_rng(seed)
    srcs = [scenes.random_triangles(600, seed=seed + 1),
            scenes.terrain_boxes(seed=seed + 2, grid=10, extent=4.0, n_boxes=2)[0],
            scenes._box_triangles(np.array([-0.5, -0.5, -0.5], F32), np.array([0.5, 0.5, 0.5], F32))]
    meshes, bvhs = [], []
    for t in srcs:
        b = BVH(t)
        n = len(t)
        op = rng.uniform(0.0, 1.0, n).astype(F32)
        kind = rng.integers(0, 4, n)
        op[kind == 0] = -1.0                  # the material's opacity (and texture)
        op[kind == 1] = 0.0                   # clear
        op[kind == 2] = 1.0                   # opaque
        mat = rng.integers(0, 4, n).astype(np.int32)
        gt = b.pack_triangles(mat, op)
        sh = b.pack_shading(None, mat, op)
        b.pack_uvs(sh, rng.uniform(-1.5, 2.5, (n, 6)).astype(F32))
        meshes.append((b.nodes_f32.copy(), gt, sh))
        bvhs.append(b)
    insts, boxes, centres = [], [], []
    masks = [atlas_rt.MASK_ALL, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW, atlas_rt.MASK_SHADOW]
    for i in range(n_inst):
        k = int(rng.integers(len(meshes)))
        M = np.eye(4)
        M[:3, :3] = _rotation(rng) @ np.diag(rng.uniform(0.5, 2.0, 3))
        M[:3, 3] = rng.uniform(-6, 6, 3)
        centres.append(M[:3, 3].copy())
        insts.append(atlas_rt.make_instance(M, k, masks[i % 3], material_offset=4 * k))
        lo, hi = atlas_rt.mesh_bounds(bvhs[k])
        boxes.append(atlas_rt.transform_aabb(lo, hi, M))
    insts = np.array(insts, atlas_rt.INSTANCE_DTYPE)
    boxes = np.array(boxes, F32)
    top = BVH(boxes_only=boxes)
    ordered = insts[top.order].copy()
    ordered["nextInstance"] = np.where(top.end_of_node > 0, -1, np.arange(len(ordered)) + 1)
    mats = np.zeros(12, MATERIAL_DTYPE)
    mats["opacity"] = rng.uniform(0.0, 1.0, 12)
    for t in ("baseColorTexture", "normalTexture", "roughnessTexture", "metalnessTexture", "aoTexture"):
        mats[t] = -1
    # -1: none; an index past the table is undefined in the engine (a
    # bindless read out of bounds), so the goldens stay within it
    mats["opacityTexture"] = rng.integers(-1, 3, 12)
    mats["invertUVs"] = rng.integers(0, 2, 12)
    tex = [rng.integers(0, 256, (16, 32), dtype=np.uint8),
           rng.integers(0, 256, (8, 5, 4), dtype=np.uint8),
           rng.uniform(-0.2, 1.2, (33, 7)).astype(F32)]
    o, d = scenes.sphere_rays(n_rays, seed=seed + 3, radius=20.0, center=(0.0, 0.0, 0.0))
    # three in four rays aimed at an instance, the rest anywhere in the scene
    tgt = rng.uniform(-6, 6, (n_rays, 3))
    aim = rng.random(n_rays) < 0.75
    tgt[aim] = np.array(centres)[rng.integers(0, n_inst, aim.sum())] + rng.normal(0, 0.8, (aim.sum(), 3))
    d = scenes._normalize((tgt - o).astype(F32))
    rays8 = scenes.rays8(o, d, 1e-4, 1e3)
    return {"top": top.nodes_f32.copy(), "instances": ordered, "meshes": meshes, "materials": mats,
            "textures": tex, "rays8": rays8}


def texture_rgba(t):
    """A texel array of the library's formats as RGBA float texels, as a
    sampler returns them: R8 / RGBA8 unorm c / 255, R32F as stored, absent
    channels (0, 0, 1)."""
    h, w = t.shape[:2]
    out = np.zeros((h, w, 4), F32)
    out[..., 3] = 1.0
    if t.dtype == np.uint8 and t.ndim == 2:
        out[..., 0] = t.astype(F32) / F32(255.0)
    elif t.dtype == np.uint8:
        out[...] = t.astype(F32) / F32(255.0)
    else:
        out[..., 0] = t
    return np.ascontiguousarray(out)


def scene_digest(sc):
    import hashlib
    h = hashlib.sha256()
    for a in [sc["top"], sc["instances"], sc["materials"], sc["rays8"], *sc["textures"],
              *[x for m in sc["meshes"] for x in m]]:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def trace_scene(lib: C.CDLL, sc: dict) -> dict:
    """The reference's HitClosest / HitAny (cull mask: all) and
    HitClosestTransparency / HitAnyTransparency (all and shadow) over sc."""
    P = C.c_void_p
    keep = [sc["top"], sc["instances"], sc["materials"]]
    nodes = (P * 3)(*[m[0].ctypes.data for m in sc["meshes"]])
    bt = (P * 3)(*[m[1].ctypes.data for m in sc["meshes"]])
    tr = (P * 3)(*[m[2].ctypes.data for m in sc["meshes"]])
    rgba = [texture_rgba(t) for t in sc["textures"]]
    tp = (P * len(rgba))(*[t.ctypes.data for t in rgba])
    wh = np.array([[t.shape[1], t.shape[0]] for t in rgba], np.int32).reshape(-1)
    lib.aeglsl_scene(P(keep[0].ctypes.data), P(keep[1].ctypes.data), C.c_int(3), nodes, bt, tr,
                     P(keep[2].ctypes.data), C.c_int(len(rgba)), tp, P(wh.ctypes.data))
    rays = np.ascontiguousarray(sc["rays8"], F32)
    out = {}
    for name, kind, cull in (("closest", 0, 0xFFFFFFFF), ("any", 1, 0xFFFFFFFF),
                             ("closest_transparency", 2, 0xFFFFFFFF), ("any_transparency", 3, 0xFFFFFFFF),
                             ("closest_shadow", 0, 1 << 6), ("closest_transparency_shadow", 2, 1 << 6),
                             ("any_transparency_shadow", 3, 1 << 6)):
        o = np.zeros((len(rays), 4), F32)
        lib.aeglsl_scene_trace(C.c_int(kind), P(rays.ctypes.data), C.c_int(len(rays)), C.c_uint(cull),
                               P(o.ctypes.data))
        out["trav_" + name] = o
    return out


# (width, height, sampleCount): one dispatch of rayGen.csh over the whole
# image each; 30 x 17 has partial work groups on the right and at the bottom
RAYGEN_CASES = ((64, 40, 3), (30, 17, 7), (101, 67, 12))


def raygen_camera(w, h):
    """The camera the raygen goldens use (scenes.pinhole_camera): origin,
    right, bottom, location as 4 floats each."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    from atlas_rt import scenes
    c = scenes.pinhole_camera(w, h)
    return np.concatenate([np.append(c[k], 0.0) for k in ("origin", "right", "bottom", "location")]).astype(F32)


def trace_raygen(lib: C.CDLL) -> dict:
    """rayGen.csh (not REALTIME) dispatched over whole images: the packed rays
    in the order the shader writes them, and the frame's jitter."""
    P = C.c_void_p
    lib.aeglsl_random2.restype = C.c_float
    lib.aeglsl_random2.argtypes = [C.c_float, C.c_float]
    out = {}
    for w, h, s in RAYGEN_CASES:
        cam = raygen_camera(w, h)
        ints = np.array([w, h, 0, 0, w, h, s], np.int32)
        rays = np.zeros((w * h, 12), F32)
        n = lib.aeglsl_raygen(P(cam.ctypes.data), P(ints.ctypes.data), P(rays.ctypes.data), C.c_int(w * h))
        assert n == w * h
        # the shader leaves the ray's hit distance and hit instance unset
        # (rayGen.csh:46-55), so PackRay copies whatever they held: not kept
        rays[:, 8] = 0.0
        rays[:, 10] = 0.0
        out[f"raygen_{w}x{h}"] = rays
        out[f"raygen_{w}x{h}_jitter"] = np.array([lib.aeglsl_random2(float(s), 0.0), lib.aeglsl_random2(float(s), 1.0)],
                                                 F32)
    return out


# ---- the engine's own path tracer: rayGen.csh, the trace dispatch and
# rayHit.csh run invocation by invocation (glsl_capi.cpp: aeglsl_pt_render) ----

def single_light(sc):
    """The scene with one emissive triangle: the others of the emitter are
    dropped.  The engine's light selection and light sampling draw the same
    random numbers (direct.hsh: GetLight and SampleLight take the seed by
    value), which biases its estimator once a scene has two lights; with one
    light the choice is certain and the estimator is unbiased."""
    from atlas_rt import BVH
    emissive = np.any(sc["materials"]["emissiveColor"][sc["obj"]] > 0, axis=1)
    keep = ~emissive
    keep[np.nonzero(emissive)[0][0]] = True
    out = dict(sc, tris=sc["tris"][keep], obj=sc["obj"][keep], normals=sc["normals"][keep])
    if sc.get("opacity") is not None:
        out["opacity"] = sc["opacity"][keep]
    out["bvh"] = BVH(out["tris"])
    return out


def pt_cases():
    """name -> (scene in ptscene.build's layout, camera dict, width, height,
    samples, bounces, block): a small terrain + boxes scene under one
    triangle of the area light (3 bounces), a half-opaque sheet over a floor
    under one emitter triangle (1 bounce: the transmission branch), and the
    diffuse floor under its two-triangle emitter (1 bounce), where the
    engine's correlated light sampling shows."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    sys.path.insert(0, str(REPO / "tests"))
    from atlas_rt import ptscene, scenes
    import test_pt_quadrature as Q
    return {"terrain": (single_light(ptscene.build(grid=48, n_boxes=12)), scenes.pinhole_camera(80, 45), 80, 45,
                        2048, 3, 5),
            "sheet": (single_light(Q.pass_through_scene()), Q.camera(), Q.W, Q.H, 8192, 1, 4),
            "two_lights": (Q.furnace_scene("diffuse"), Q.camera(), Q.W, Q.H, 8192, 1, 4)}


def pt_arrays(sc):
    """The one-instance scene of a ptscene-layout dict in the engine's buffers:
    (TLAS nodes, instances, model matrices, meshes [(nodes, BVH triangles,
    shading triangles)], materials, lights) -- what the oracle's path tracer
    takes too."""
    import atlas_rt
    from atlas_rt import BVH, ptscene
    b = sc["bvh"]
    gt = b.pack_triangles(sc["obj"], sc.get("opacity"))
    sh = b.pack_shading(sc["normals"], sc["obj"], sc.get("opacity"))
    lights = ptscene.lights_for(sc, sh)
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)],
                    atlas_rt.INSTANCE_DTYPE)
    ordered = inst[top.order].copy()
    ordered["nextInstance"] = np.where(top.end_of_node > 0, -1, np.arange(len(ordered)) + 1)
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (len(ordered), 1))
    return (top.nodes_f32.copy(), ordered, model, [(b.nodes_f32.copy(), gt, sh)],
            np.ascontiguousarray(sc["materials"]), np.ascontiguousarray(lights, F32))


def trace_pt(lib: C.CDLL, name: str) -> dict:
    """The engine's path tracer over one case, one sample per call (the
    hit shader's seeds drawn uniformly per sample and bounce, as the engine
    does): the mean image, and per block of pixels the mean and the
    per-sample variance of the block mean (what a statistical comparison
    needs)."""
    sc, camd, w, h, spp, mb, blk = pt_cases()[name]
    tl, inst, model, meshes, mats, lights = pt_arrays(sc)
    P = C.c_void_p
    (nodes, gt, sh), = meshes
    lib.aeglsl_pt_scene(P(tl.ctypes.data), P(inst.ctypes.data), C.c_int(1), (P * 1)(nodes.ctypes.data),
                        (P * 1)(gt.ctypes.data), (P * 1)(sh.ctypes.data), P(mats.ctypes.data),
                        P(lights.ctypes.data), C.c_int(len(lights)))
    cam = np.concatenate([np.append(camd[k], 0.0) for k in ("origin", "right", "bottom", "location")]).astype(F32)
    seeds = np.random.default_rng(sum(map(ord, name)) + 20261206).random((spp, mb + 1)).astype(F32)
    total = np.zeros((h, w, 3))
    bsum = np.zeros((h // blk, w // blk, 3))
    bsq = np.zeros_like(bsum)
    acc = np.zeros((h, w, 4), F32)
    for s in range(spp):
        acc[...] = 0.0
        sd = np.ascontiguousarray(seeds[s])
        lib.aeglsl_pt_render(P(cam.ctypes.data), C.c_int(w), C.c_int(h), C.c_int(1), C.c_int(s), C.c_int(mb),
                             C.c_int(1), P(sd.ctypes.data), P(acc.ctypes.data))
        img = acc[..., :3].astype(np.float64)
        total += img
        bm = img[:h // blk * blk, :w // blk * blk].reshape(h // blk, blk, w // blk, blk, 3).mean(axis=(1, 3))
        bsum += bm
        bsq += bm * bm
    bmean = bsum / spp
    return {f"pt_{name}_mean": (total / spp).astype(F32), f"pt_{name}_block_mean": bmean,
            f"pt_{name}_block_var": np.maximum(bsq / spp - bmean * bmean, 0.0),
            f"pt_{name}_spp": np.array([spp, mb, blk], np.int32)}


def evaluate(lib: C.CDLL, ins: dict) -> dict:
    P = C.c_void_p

    def run(fn, x, width, *extra):
        x = np.ascontiguousarray(x, F32)
        out = np.zeros((len(x), width), F32)
        fn(x.ctypes.data_as(P), C.c_int(len(x)), *extra, out.ctypes.data_as(P))
        return out
    out = {"eval_out": run(lib.aeglsl_eval, ins["eval_in"], 16),
           "sample_diffuse_out": run(lib.aeglsl_sample, ins["sample_in"], 8, C.c_int(0)),
           "sample_specular_out": run(lib.aeglsl_sample, ins["sample_in"], 8, C.c_int(1)),
           "light_out": run(lib.aeglsl_triangle_light, ins["light_in"], 7),
           "tri_out": run(lib.aeglsl_intersect_triangle, ins["tri_in"], 4),
           "box_out": run(lib.aeglsl_intersect_aabb, ins["box_in"], 2)}
    xs = np.ascontiguousarray(ins["random_x"], F32)
    r = np.zeros((len(xs), 8), F32)
    lib.aeglsl_random(xs.ctypes.data_as(P), C.c_int(len(xs)), C.c_float(1.0), C.c_int(8), r.ctypes.data_as(P))
    out["random_out"] = r
    return out


# rtao.csh over half-resolution G-buffers of the traversal scene: (width,
# height).  96 x 64 is a whole number of the shader's tiles (four work groups
# of 8 pixels across); 44 x 20 is not, and the engine's dispatch of
# ceil(w / 8) * ceil(h / 4) groups (AORenderer.cpp:85-88) then reaches only
# part of the last tile column.
RTAO_CASES = ((96, 64), (44, 20))
RTAO_RADIUS = 8.0
RTAO_FRAMES = (5, 300)          # uniforms.frameSeed; 300 wraps the sample index


def pass_scene(seed=20261207):
    """A seeded two-level scene for the screen-space pass goldens: a terrain
    patch with boxes (mesh 0, one identity instance), a box with
    per-triangle opacities (mesh 1) standing on it four times, and a sheet
    of sixteen quads with per-triangle opacities (mesh 2) hovering over it
    three times (tilted; one visible to the shadow mask only); twelve
    materials of random opacity, some with an opacity texture.  Laid out
    like traversal_scene (the library's builder and packers; deterministic,
    so the tests rebuild it)."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    import atlas_rt
    from atlas_rt import BVH, MATERIAL_DTYPE, scenes
    rng = np.random.default_rng(seed)
    extent = 16.0
    terrain = scenes.terrain_boxes(seed=seed + 1, grid=32, extent=extent, n_boxes=16)[0]
    box = scenes._box_triangles(np.array([-0.5, 0.0, -0.5], F32), np.array([0.5, 1.0, 0.5], F32))
    q = np.linspace(-1.0, 1.0, 5, dtype=F32)
    sheet = []
    for i in range(4):
        for j in range(4):
            a, b = [q[i], 0.0, q[j]], [q[i + 1], 0.0, q[j]]
            c, d = [q[i + 1], 0.0, q[j + 1]], [q[i], 0.0, q[j + 1]]
            sheet += [[a, c, b], [a, d, c]]
    sheet = np.array(sheet, F32)
    meshes, bvhs = [], []
    for k, t in enumerate((terrain, box, sheet)):
        b = BVH(t)
        n = len(t)
        op = rng.uniform(0.0, 1.0, n).astype(F32)
        kind = rng.integers(0, 4, n)
        if k == 0:
            kind = np.where(rng.random(n) < 0.9, 2, 0)   # the ground: mostly opaque
        op[kind == 0] = -1.0
        op[kind == 1] = 0.0
        op[kind == 2] = 1.0
        mat = rng.integers(0, 4, n).astype(np.int32)
        gt = b.pack_triangles(mat, op)
        sh = b.pack_shading(None, mat, op)
        b.pack_uvs(sh, rng.uniform(-1.5, 2.5, (n, 6)).astype(F32))
        meshes.append((b.nodes_f32.copy(), gt, sh))
        bvhs.append(b)
    insts, boxes = [], []
    MA, MS = atlas_rt.MASK_ALL, atlas_rt.MASK_SHADOW

    def add(M, k, mask):
        insts.append(atlas_rt.make_instance(M, k, mask, material_offset=4 * k))
        lo, hi = atlas_rt.mesh_bounds(bvhs[k])
        boxes.append(atlas_rt.transform_aabb(lo, hi, M))

    add(np.eye(4), 0, MA)
    for i in range(7):
        x, z = rng.uniform(2.0, extent - 2.0, 2)
        ground = float(scenes.terrain_height(seed + 1, np.array([x], F32), np.array([z], F32))[0])
        a = rng.uniform(0.0, 2.0 * np.pi)
        R = np.array([[np.cos(a), 0.0, np.sin(a)], [0.0, 1.0, 0.0], [-np.sin(a), 0.0, np.cos(a)]])
        M = np.eye(4)
        if i < 4:
            M[:3, :3] = R @ np.diag(rng.uniform(0.8, 2.5, 3))
            M[:3, 3] = (x, ground - 0.3, z)
            add(M, 1, (MA, MA | MS)[i % 2])
        else:
            M[:3, :3] = _rotation(rng) @ np.diag([rng.uniform(2.0, 3.5), 1.0, rng.uniform(2.0, 3.5)])
            M[:3, :3] = 0.35 * M[:3, :3] + 0.65 * R @ np.diag([2.5, 1.0, 2.5])
            M[:3, 3] = (x, ground + rng.uniform(0.6, 1.5), z)
            add(M, 2, (MA | MS, MA, MS)[i - 4])
    insts = np.array(insts, atlas_rt.INSTANCE_DTYPE)
    top = BVH(boxes_only=np.array(boxes, F32))
    ordered = insts[top.order].copy()
    ordered["nextInstance"] = np.where(top.end_of_node > 0, -1, np.arange(len(ordered)) + 1)
    mats = np.zeros(12, MATERIAL_DTYPE)
    mats["opacity"] = rng.uniform(0.0, 1.0, 12)
    mats["opacity"][0] = 1.0
    for t in ("baseColorTexture", "normalTexture", "roughnessTexture", "metalnessTexture", "aoTexture"):
        mats[t] = -1
    mats["opacityTexture"] = rng.integers(-1, 3, 12)
    mats["invertUVs"] = rng.integers(0, 2, 12)
    mats["baseColor"] = rng.uniform(0.2, 0.9, (12, 3))
    mats["roughness"] = rng.uniform(0.05, 1.0, 12)
    mats["metalness"] = np.where(rng.random(12) < 0.3, 1.0, 0.0)
    mats["reflectance"] = rng.uniform(0.2, 0.8, 12)
    mats["ao"] = 1.0
    mats["emissiveColor"][[5, 9]] = [[2.0, 1.5, 1.0], [0.5, 1.0, 2.0]]
    tex = [rng.integers(0, 256, (16, 32), dtype=np.uint8),
           rng.integers(0, 256, (8, 5, 4), dtype=np.uint8),
           rng.uniform(-0.2, 1.2, (33, 7)).astype(F32)]
    # one directional light (GPULight: N is the light's direction; type 0 in
    # the top bits of data.x; selection pdf 1)
    light = np.zeros((1, 16), F32)
    light[0, 4:7] = np.array([-0.35, -1.0, 0.45]) / np.linalg.norm([-0.35, -1.0, 0.45])
    light[0, 8:11] = (2.5, 2.3, 2.0)
    light[0, 13] = 1.0
    return {"top": top.nodes_f32.copy(), "instances": ordered, "meshes": meshes, "materials": mats,
            "textures": tex, "lights": light, "rays8": np.zeros((0, 8), F32)}


def set_scene(lib: C.CDLL, sc: dict, keep: list):
    """Points the reference programs' scene buffers at sc (kept alive in keep)."""
    P = C.c_void_p
    nodes = (P * 3)(*[m[0].ctypes.data for m in sc["meshes"]])
    bt = (P * 3)(*[m[1].ctypes.data for m in sc["meshes"]])
    tr = (P * 3)(*[m[2].ctypes.data for m in sc["meshes"]])
    rgba = [texture_rgba(t) for t in sc["textures"]]
    tp = (P * len(rgba))(*[t.ctypes.data for t in rgba])
    wh = np.array([[t.shape[1], t.shape[0]] for t in rgba], np.int32).reshape(-1)
    keep += [rgba, tp, wh, nodes, bt, tr]
    lib.aeglsl_scene(P(sc["top"].ctypes.data), P(sc["instances"].ctypes.data), C.c_int(3), nodes, bt, tr,
                     P(sc["materials"].ctypes.data), C.c_int(len(rgba)), tp, P(wh.ctypes.data))


def blue_noise_textures(seed=20261206):
    """Stand-ins for the engine's blue-noise textures (RGBA8, 128 x 128
    scrambling / ranking and 256 x 1 Sobol sequence): seeded bytes, since
    what is pinned is the sampler's arithmetic over whatever they hold."""
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 256, (128, 128, 4), dtype=np.uint8), rng.integers(0, 256, (256, 4), dtype=np.uint8))


def pass_camera(w: int, h: int):
    """View and projection matrices of the screen-space pass goldens."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    from atlas_rt import gbuffer as G
    return G.look_at((8.0, 16.0, -5.0), (8.0, 4.0, 9.0)), G.perspective(60.0, w / h, 0.5, 400.0)


def pass_gbuffer(lib: C.CDLL, sc: dict, w: int, h: int, half_res: bool = True, seed: int = 7):
    """A G-buffer of pass_scene (the lib's scene must be sc): the eye ray of
    each pixel (at half resolution through 2 * pixel + offset + 0.5 of the
    full one) traced by the reference's HitClosest; depth = the hit's NDC
    depth (1 where nothing is hit), normal = the encoded view-space face
    normal of the hit triangle, turned towards the eye; a roughness plane
    with mirror (0, <= 0.01), glossy, rough and untraced (> 1) pixels."""
    sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
    from atlas_rt import gbuffer as G
    from atlas_rt import scenes
    rng = np.random.default_rng(seed)
    V, P = pass_camera(w, h)
    offset = rng.integers(0, 4, w * h).astype(np.uint8) if half_res else np.zeros(w * h, np.uint8)
    o, d = G.view_rays(V, P, w, h, offset if half_res else None)
    rays8 = np.ascontiguousarray(scenes.rays8(o.astype(F32), d.astype(F32), 0.0, 1e12), F32)
    hits = np.zeros((w * h, 4), F32)
    lib.aeglsl_scene_trace(C.c_int(0), C.c_void_p(rays8.ctypes.data), C.c_int(w * h), C.c_uint(0xFFFFFFFF),
                           C.c_void_p(hits.ctypes.data))
    tri, inst = hits[:, 0].view(np.int32), hits[:, 1].view(np.int32)
    hit = tri >= 0
    od, dd = rays8[:, 0:3].astype(np.float64), rays8[:, 3:6].astype(np.float64)
    pos = od + dd * hits[:, 2:3].astype(np.float64)
    clip = np.concatenate([pos, np.ones((len(pos), 1))], axis=1) @ (P @ V).T
    depth = np.where(hit, clip[:, 2] / clip[:, 3], 1.0)
    n = np.zeros((w * h, 3))
    for i in np.flatnonzero(hit):
        ins = sc["instances"][inst[i]]
        t = sc["meshes"][ins["meshOffset"]][2][tri[i], :12].astype(np.float64)
        no = np.cross(t[4:7] - t[0:3], t[8:11] - t[0:3])
        n[i] = np.asarray(ins["inverseMatrix"], np.float64).reshape(3, 4)[:, :3].T @ no
    n /= np.linalg.norm(n, axis=1, keepdims=True) + 1e-30
    n *= np.where((n * dd).sum(axis=1, keepdims=True) > 0, -1.0, 1.0)
    nv = n @ V[:3, :3].T
    nv /= np.linalg.norm(nv, axis=1, keepdims=True) + 1e-30
    enc = np.zeros((w * h, 2))
    enc[hit] = G.encode_normal(nv[hit])
    rough = rng.uniform(0.0, 1.1, w * h)
    rough[rng.random(w * h) < 0.15] = 0.0
    rough[rng.random(w * h) < 0.05] = 0.008
    return {"depth": depth.astype(F32).reshape(h, w), "normal": enc.astype(F32).reshape(h, w, 2),
            "offset": offset.reshape(h, w), "roughness": rough.astype(F32).reshape(h, w), "half_res": int(half_res),
            "ip_matrix": np.linalg.inv(P), "iv_matrix": np.linalg.inv(V)}


def column_major(m):
    return np.ascontiguousarray(np.asarray(m, np.float64).astype(F32).T.reshape(-1))


# rtreflection.csh / rtgi.csh: (width, height, half resolution), their
# uniforms (radianceLimit, bias, roughnessCutoff, the environment's colour)
# and frame seed
SHADE_CASES = ((64, 40, False), (48, 30, True))
SHADE_PARAMS = (4.0, 0.1, 0.8, 0.05, 0.1, 0.2)
SHADE_FRAME = 7


# DDGI probe rays: a 4 x 3 x 4 grid over pass_scene (some probes under the
# ground or inside boxes, so back faces are met), 32 rays per probe and 8 for
# inactive ones, the environment's colour and the hit shader's seed
DDGI_GRID = (4, 3, 4)
DDGI_VOLUME = ((1.0, 8.5, 1.0), (4.5, 1.6, 4.5))
DDGI_RAYS = (32, 8)
DDGI_ENV = (0.25, 0.5, 0.75)
DDGI_SEED = 0.37


def fibonacci_dirs(n):
    """n unit directions on a Fibonacci sphere as vec4 (w = 0)."""
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    r = np.sqrt(1.0 - z * z)
    phi = np.pi * (3.0 - np.sqrt(5.0)) * i
    return np.stack([r * np.cos(phi), z, r * np.sin(phi), np.zeros(n)], axis=1).astype(F32)


def ddgi_inputs(seed=20261209):
    """Probe states (new, active, inactive), history offsets, the two
    direction sets and the frame's rotation (4 x 4, row-major) of the DDGI
    goldens; and pass_scene's materials without opacity textures (the hit
    shader reads textures at mip level 4, and the harness's textures have
    level 0 only)."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(DDGI_GRID))
    states = rng.integers(0, 3, n).astype(np.uint32)
    offsets = np.zeros((n, 4), F32)
    offsets[:, :3] = rng.uniform(-0.3, 0.3, (n, 3))
    rot = np.eye(4)
    rot[:3, :3] = _rotation(rng)
    return states, offsets, fibonacci_dirs(DDGI_RAYS[0]), fibonacci_dirs(DDGI_RAYS[1]), rot


def ddgi_materials(sc):
    m = sc["materials"].copy()
    m["opacityTexture"] = -1
    m["cullBackFaces"][::2] = 1        # back faces of these are reported (negative distance)
    return m


def trace_passes(lib: C.CDLL) -> dict:
    """Over pass_scene: one dispatch of the reference's rtao.csh (HitAny and,
    with OPACITY_CHECK, HitAnyTransparency) per case, frame seed and variant,
    unwritten pixels staying -1, and the blue-noise vectors of one 128 x 128
    period per frame seed, stored as the integers v * 256 - 0.5; one
    dispatch of rtreflection.csh and of rtgi.csh per case and variant."""
    P = C.c_void_p
    sc, keep = pass_scene(), []
    set_scene(lib, sc, keep)
    lib.aeglsl_scene_lights(P(sc["lights"].ctypes.data), C.c_int(len(sc["lights"])))
    out = {"pass_scene_digest": np.frombuffer(scene_digest(sc).encode(), np.uint8)}
    rank, sobol = blue_noise_textures()
    rank_f, sobol_f = texture_rgba(rank), texture_rgba(sobol[None])
    for f in RTAO_FRAMES:
        bn = np.zeros((128, 128, 2), F32)
        lib.aeglsl_blue_noise(C.c_int(128), C.c_int(128), P(rank_f.ctypes.data), P(sobol_f.ctypes.data), C.c_int(f),
                              P(bn.ctypes.data))
        q = bn * F32(256.0) - F32(0.5)
        assert np.array_equal(q, np.round(q)) and q.min() >= 0 and q.max() <= 255
        out[f"rtao_blue_noise_{f}"] = q.astype(np.uint8)
    for w, h in RTAO_CASES:
        gb = pass_gbuffer(lib, sc, w, h)
        key = f"rtao_{w}x{h}"
        for k in ("depth", "normal", "offset"):
            out[f"{key}_{k}"] = gb[k]
        off = np.ascontiguousarray(gb["offset"], np.int32)
        ip, iv = column_major(gb["ip_matrix"]), column_major(gb["iv_matrix"])
        for f in RTAO_FRAMES:
            for opacity in (0, 1):
                ao = np.full((h, w), -1.0, F32)
                lib.aeglsl_rtao(C.c_int(opacity), C.c_int(w), C.c_int(h), P(gb["depth"].ctypes.data),
                                P(gb["normal"].ctypes.data), P(off.ctypes.data), P(rank_f.ctypes.data),
                                P(sobol_f.ctypes.data), P(ip.ctypes.data), P(iv.ctypes.data), C.c_float(RTAO_RADIUS),
                                C.c_int(f), P(ao.ctypes.data))
                out[f"{key}_ao_{f}_{opacity}"] = ao
    params = np.array(SHADE_PARAMS, F32)
    for w, h, half in SHADE_CASES:
        gb = pass_gbuffer(lib, sc, w, h, half_res=half, seed=11)
        key = f"shade_{w}x{h}"
        for k in ("depth", "normal", "offset", "roughness"):
            out[f"{key}_{k}"] = gb[k]
        off = np.ascontiguousarray(gb["offset"], np.int32)
        ip, iv = column_major(gb["ip_matrix"]), column_major(gb["iv_matrix"])
        for kind, name in ((0, "reflections"), (1, "rtgi")):
            for opacity in (0, 1):
                img = np.full((h, w, 4), -1.0, F32)
                lib.aeglsl_screen_pass(C.c_int(kind), C.c_int(opacity), C.c_int(w), C.c_int(h), C.c_int(int(half)),
                                       P(gb["depth"].ctypes.data), P(gb["normal"].ctypes.data), P(off.ctypes.data),
                                       P(gb["roughness"].ctypes.data), P(rank_f.ctypes.data), P(sobol_f.ctypes.data),
                                       P(ip.ctypes.data), P(iv.ctypes.data), P(params.ctypes.data),
                                       C.c_uint(SHADE_FRAME), P(img.ctypes.data))
                out[f"{key}_{name}_{opacity}"] = img
    # DDGI: the scene again with the materials of ddgi_materials
    dsc = dict(sc, materials=ddgi_materials(sc))
    set_scene(lib, dsc, keep)
    states, offsets, dirs, dirs_in, rot = ddgi_inputs()
    n = len(states)
    grid = np.array(DDGI_GRID, np.int32)
    vmin, cell = (np.array(v, F32) for v in DDGI_VOLUME)
    env = np.array(DDGI_ENV, F32)
    rotc = column_major(rot)
    for opacity in (0, 1):
        origins = np.zeros((n, 4), F32)
        hits = np.full((n * DDGI_RAYS[0], 4), -7.0, F32)
        lib.aeglsl_ddgi(P(grid.ctypes.data), P(vmin.ctypes.data), P(cell.ctypes.data), C.c_uint(DDGI_RAYS[0]),
                        C.c_uint(DDGI_RAYS[1]), P(states.ctypes.data), P(offsets.ctypes.data), P(dirs.ctypes.data),
                        P(dirs_in.ctypes.data), P(rotc.ctypes.data), C.c_int(opacity), P(env.ctypes.data),
                        C.c_float(DDGI_SEED), P(origins.ctypes.data), P(hits.ctypes.data))
        out[f"ddgi_origins_{opacity}"] = origins
        out[f"ddgi_hits_{opacity}"] = hits
    return out


def reference_lib():
    """Builds (if needed) and loads the reference's GLSL compiled on the host;
    None where the reference tree is absent."""
    sys.path.insert(0, str(REPO / "oracle"))
    sys.path.insert(0, str(REPO / "oracle" / "glsl"))
    import pyoracle
    import make_ref
    if not (pyoracle.REFERENCE_ROOT / "data" / "shader" / "brdf" / "brdf.hsh").exists():
        return None
    return C.CDLL(str(make_ref.build(pyoracle.REFERENCE_ROOT)))


def main():
    lib = reference_lib()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate the GLSL goldens")
    ins = inputs()
    sc = traversal_scene()
    trav = trace_scene(lib, sc)
    pt = {}
    for name in pt_cases():
        pt.update(trace_pt(lib, name))
    np.savez_compressed(OUT, **ins, **evaluate(lib, ins), **trav, **trace_raygen(lib), **pt, **trace_passes(lib),
                        trav_scene_digest=np.frombuffer(scene_digest(sc).encode(), np.uint8))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
