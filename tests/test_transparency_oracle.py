"""Known answers of the oracle's transparency traversal variants
(HitClosestTransparency / HitAnyTransparency, bvh.hsh:275-357, :443-524) on
stacks of parallel quads, including the reference's re-multiplication of the
running transparency at every leaf (bvh.hsh:500: `transparency *=
CheckLeafTransparency(..., transparency)`)."""
import numpy as np

import atlas_rt
import pyoracle
from atlas_rt import BVH, MATERIAL_DTYPE, scenes


def quads(zs):
    out = []
    for z in zs:
        a, b, c, d = [0, 0, z], [1, 0, z], [1, 1, z], [0, 1, z]
        out += [[a, b, d], [b, c, d]]
    return np.array(out, np.float32)


def one_instance_scene(tris, opacity, material=None):
    b = BVH(tris)
    gt = b.pack_triangles()
    sh = b.pack_shading(None, material, opacity)
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL)], atlas_rt.INSTANCE_DTYPE)
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    ordered = inst[top.order].copy()
    return b, top, ordered, [(b.nodes_f32, gt, sh)]


def materials(opacities):
    m = np.zeros(len(opacities), MATERIAL_DTYPE)
    m["opacity"] = opacities
    for t in ("baseColorTexture", "opacityTexture", "normalTexture", "roughnessTexture", "metalnessTexture",
              "aoTexture"):
        m[t] = -1
    return m


def rays_through(pt, n=1):
    o = np.tile(np.array([[pt[0], pt[1], 0.0]], np.float32), (n, 1))
    d = np.tile(np.array([[0, 0, 1]], np.float32), (n, 1))
    return scenes.rays8(o, d, 1e-4, 100.0)


def test_any_transparency_squares_per_leaf():
    """One quad of two triangles (two one-triangle leaves whose boxes both
    contain the ray).  The leaf with the accepted hit gives T = 1 * (1 * 0.5);
    the other leaf accepts nothing but still returns its starting value, so
    T = 0.5 * 0.5: the reference squares the running transparency at every
    visited leaf."""
    tris = quads([1.0])
    b, top, inst, meshes = one_instance_scene(tris, np.full(len(tris), 0.5, np.float32))
    assert list(b.nodes["leftPtr"]) == [-1] and list(b.nodes["rightPtr"]) == [-2]
    t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, materials([1.0]), rays_through((0.25, 0.5)))
    assert t[0] == np.float32(0.25)
    # missing the quad's boxes: nothing visited, fully clear
    t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, materials([1.0]), rays_through((2.0, 2.0)))
    assert t[0] == 1.0
    # a clear quad (opacity 0) leaves it at 1
    b, top, inst, meshes = one_instance_scene(tris, np.zeros(len(tris), np.float32))
    t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, materials([1.0]), rays_through((0.25, 0.5)))
    assert t[0] == 1.0


def test_any_transparency_opaque_ends_at_zero():
    tris = quads([1.0, 2.0])
    op = np.array([0.5, 0.5, 1.0, 1.0], np.float32)
    b, top, inst, meshes = one_instance_scene(tris, op)
    t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, materials([1.0]), rays_through((0.25, 0.5)))
    assert t[0] == 0.0


def test_closest_transparency_skips_clear_triangles():
    tris = quads([1.0, 2.0, 3.0])
    op = np.array([0.0, 0.0, 0.3, 0.3, 1.0, 1.0], np.float32)
    b, top, inst, meshes = one_instance_scene(tris, op)
    ptr, ino, tuv = pyoracle.scene_closest_transparency_glsl(top.nodes_f32, inst, meshes, materials([1.0]),
                                                             rays_through((0.25, 0.5)))
    assert tuv[0, 0] == 2.0 and b.order[ptr[0]] == 2 and ino[0] == 0
    # the opaque query takes the clear quad at t = 1
    p2, _, tuv2 = pyoracle.scene_closest_glsl(top.nodes_f32, inst, [m[:2] for m in meshes], rays_through((0.25, 0.5)))
    assert tuv2[0, 0] == 1.0


def test_negative_opacity_reads_the_material():
    tris = quads([1.0, 2.0])
    op = np.full(len(tris), -1.0, np.float32)
    mat = np.array([0, 0, 1, 1], np.int32)           # first quad material 0, second material 1
    b, top, inst, meshes = one_instance_scene(tris, op, mat)
    mats = materials([0.0, 0.75])
    ptr, _, tuv = pyoracle.scene_closest_transparency_glsl(top.nodes_f32, inst, meshes, mats,
                                                           rays_through((0.25, 0.5)))
    assert tuv[0, 0] == 2.0
    # one quad with material opacity 0.75: the hit leaf gives 0.25, the other
    # visited leaf squares it
    b, top, inst, meshes = one_instance_scene(quads([1.0]), np.full(2, -1.0, np.float32), np.array([1, 1], np.int32))
    t = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, mats, rays_through((0.25, 0.5)))
    assert t[0] == np.float32(0.0625)
