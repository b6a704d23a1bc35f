"""Texture-sampled opacity of the transparency variants, on the CPU: the
UV packing of the host library (packHalf2x16, MeshData.cpp:172-239) against
numpy's binary16 rounding, the oracle's bilinear lookup (the engine's bindless
sampler: linear filter, repeat addressing, level 0; MainRenderer.cpp:922-929,
texture.hsh:18-25) against known answers and against a float32 numpy
restatement, and GetOpacity (surface.hsh:147-159) through the traversal on a
textured quad."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, MATERIAL_DTYPE, scenes


def np_sample(tex, u, v):
    """float32 numpy restatement of the lookup (one rounding per operation)."""
    f32 = np.float32
    h, w = tex.shape[:2]
    if tex.dtype == np.uint8:
        ch = tex if tex.ndim == 2 else tex[..., 0]
        tv = ch.astype(f32) / f32(255.0)
    else:
        tv = tex

    def axis(s, n):
        x = f32(f32(s) * f32(n)) - f32(0.5)
        if not np.isfinite(x) or abs(x) >= 9.0e18:
            x = f32(0.0)
        fx = np.floor(x)
        a = f32(x - fx)
        i0 = int(fx) % n
        return i0, (i0 + 1) % n, a

    x0, x1, a = axis(u, w)
    y0, y1, b = axis(v, h)
    ia, ib = f32(1) - a, f32(1) - b
    r = f32(ia * ib) * tv[y0, x0]
    r = f32(r + f32(a * ib) * tv[y0, x1])
    r = f32(r + f32(ia * b) * tv[y1, x0])
    return f32(r + f32(a * b) * tv[y1, x1])


def test_half_decode_known_answers():
    assert pyoracle.half_to_float(0x3C00) == 1.0
    assert pyoracle.half_to_float(0xC000) == -2.0
    assert pyoracle.half_to_float(0x0001) == 2.0 ** -24
    assert pyoracle.half_to_float(0x03FF) == 1023 * 2.0 ** -24
    assert pyoracle.half_to_float(0x7BFF) == 65504.0
    assert pyoracle.half_to_float(0x7C00) == np.inf
    assert np.isnan(pyoracle.half_to_float(0x7E00))
    bits = np.arange(0, 1 << 16, 7, dtype=np.uint16)
    ref = bits.view(np.float16).astype(np.float32)
    got = np.array([pyoracle.half_to_float(int(b)) for b in bits], np.float32)
    fin = np.isfinite(ref)
    np.testing.assert_array_equal(got[fin], ref[fin])


@pytest.mark.parametrize("mesh", ["random", "terrain"])
def test_uv_packing_rounds_like_binary16(mesh):
    """UVs are per input triangle; the terrain's root spatial split repeats
    some triangles in BVH order, and each copy carries its source's UVs."""
    rng = np.random.default_rng(5)
    if mesh == "random":
        tris = scenes.random_triangles(4000, seed=3)
    else:
        tris = scenes.terrain_boxes(seed=23, grid=24, extent=4.0, n_boxes=3)[0]
    n = len(tris)
    b = BVH(tris)
    assert mesh == "random" or len(b.order) > n
    sh = b.pack_shading()
    uv = rng.uniform(-3, 3, (n, 6)).astype(np.float32)
    # ties between halves, subnormals, overflow, signed zero
    special = np.array([1 + 2 ** -11, 1 + 3 * 2 ** -11, 2 ** -25, 3 * 2 ** -26, 2 ** -14 - 2 ** -25, 65519.0,
                        65520.0, -0.0, 1e-30, 70000.0, 2048 + 1, 2048 + 3], np.float32)
    uv.reshape(-1)[:len(special)] = special
    uv[10:20] *= np.float32(1e-5)
    b.pack_uvs(sh, uv)
    packed = sh[:, 12:15].copy().view(np.uint32)                   # BVH order
    src = uv[b.order].reshape(-1, 3, 2)
    with np.errstate(over="ignore"):
        want = src.astype(np.float16).view(np.uint16).astype(np.uint32)
    want = want[..., 0] | (want[..., 1] << 16)
    np.testing.assert_array_equal(packed, want)


def test_bilinear_known_answers():
    t = np.array([[0, 255], [255, 0]], np.uint8)
    s = lambda u, v, tid=0: pyoracle.sample_r_bilinear([t], tid, u, v)
    assert s(0.25, 0.25) == 0.0 and s(0.75, 0.25) == 1.0 and s(0.25, 0.75) == 1.0
    assert s(0.5, 0.25) == 0.5                      # halfway between two texel centres
    assert s(0.5, 0.5) == 0.5
    assert s(1.25, 0.25) == 0.0 and s(-0.75, 0.25) == 0.0 and s(0.25, 7.25) == 0.0   # repeat
    assert s(0.0, 0.25) == 0.5                      # the edge blends with the wrapped texel
    assert s(np.nan, 0.25) == 0.0 and s(np.inf, 0.75) == 1.0   # non-finite: texel column 0
    assert s(0.25, 0.25, tid=-1) == 1.0 and s(0.25, 0.25, tid=1) == 1.0   # absent / out of range
    rgba = np.zeros((1, 2, 4), np.uint8)
    rgba[0, 1, 0] = 51
    rgba[0, 0, 1:] = 255                           # only the first channel is read
    assert pyoracle.sample_r_bilinear([rgba], 0, 0.25, 0.5) == 0.0
    assert pyoracle.sample_r_bilinear([rgba], 0, 0.75, 0.5) == np.float32(51) / np.float32(255)
    f = np.array([[0.25, -2.0]], np.float32)
    assert pyoracle.sample_r_bilinear([f], 0, 0.5, 0.0) == np.float32(-0.875)


@pytest.mark.parametrize("kind", ["r8", "rgba8", "r32f"])
def test_bilinear_matches_float32_restatement(kind):
    rng = np.random.default_rng({"r8": 1, "rgba8": 2, "r32f": 3}[kind])
    h, w = 37, 53
    if kind == "r8":
        tex = rng.integers(0, 256, (h, w), dtype=np.uint8)
    elif kind == "rgba8":
        tex = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    else:
        tex = rng.uniform(-1, 2, (h, w)).astype(np.float32)
    uv = np.concatenate([rng.uniform(-2, 3, (3000, 2)), rng.uniform(-1e6, 1e6, (200, 2)),
                         (rng.integers(-3 * w, 3 * w, (200, 2)) + 0.5) / np.array([w, h])]).astype(np.float32)
    for u, v in uv:
        assert pyoracle.sample_r_bilinear([tex], 0, u, v) == np_sample(tex, u, v), (u, v)


def textured_quad(invert):
    """A unit quad at z = 1 whose UVs equal its (x, y), one material with a
    2x2 checkerboard opacity texture."""
    q = np.array([[[0, 0, 1], [1, 0, 1], [0, 1, 1]], [[1, 0, 1], [1, 1, 1], [0, 1, 1]]], np.float32)
    b = BVH(q)
    sh = b.pack_shading(None, np.zeros(2, np.int32), np.full(2, -1.0, np.float32))
    b.pack_uvs(sh, q[:, :, :2].reshape(2, 6))
    gt = b.pack_triangles()
    m = np.zeros(1, MATERIAL_DTYPE)
    m["opacity"] = 1.0
    for t in ("baseColorTexture", "normalTexture", "roughnessTexture", "metalnessTexture", "aoTexture"):
        m[t] = -1
    m["opacityTexture"] = 0
    m["invertUVs"] = 1 if invert else 0
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL)], atlas_rt.INSTANCE_DTYPE)
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    return top, inst[top.order].copy(), [(b.nodes_f32, gt, sh)], m


@pytest.mark.parametrize("invert", [False, True])
def test_textured_quad_opacity(invert):
    top, inst, meshes, mats = textured_quad(invert)
    tex = [np.array([[0, 255], [255, 0]], np.uint8)]
    pts = np.array([[0.25, 0.25], [0.75, 0.25], [0.25, 0.75], [0.75, 0.75]], np.float32)
    o = np.concatenate([pts, np.zeros((4, 1), np.float32)], 1)
    d = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))
    rays8 = scenes.rays8(o, d, 1e-4, 100.0)
    ptr, _, tuv = pyoracle.scene_closest_transparency_glsl(top.nodes_f32, inst, meshes, mats, rays8, textures=tex)
    tr = pyoracle.scene_any_transparency_glsl(top.nodes_f32, inst, meshes, mats, rays8, textures=tex)
    # texel (0, 0) and (1, 1) are clear, (1, 0) and (0, 1) opaque; invertUVs
    # swaps the rows, which on this checkerboard swaps clear and opaque
    opaque = np.array([False, True, True, False]) ^ invert
    np.testing.assert_array_equal(ptr >= 0, opaque)
    assert np.all(tuv[opaque, 0] == 1.0)
    np.testing.assert_array_equal(tr[opaque], 0.0)
    assert np.all(tr[~opaque] == 1.0)
    # without the texture the material's opacity alone counts: every ray hits
    ptr, _, _ = pyoracle.scene_closest_transparency_glsl(top.nodes_f32, inst, meshes, mats, rays8)
    assert np.all(ptr >= 0)


def test_attribute_packing_tangent_frame_and_colours():
    """ae_bvh_pack_attributes: the UV-derived tangent frame (MeshData.cpp:
    176-197) against a float64 restatement, vertex colours as packUnorm4x8."""
    rng = np.random.default_rng(9)
    tris = scenes.terrain_boxes(seed=4, grid=16, extent=4.0, n_boxes=2)[0]
    n = len(tris)
    b = BVH(tris)
    sh = b.pack_shading()
    uv = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    col = rng.uniform(-0.2, 1.2, (n, 12)).astype(np.float32)
    b.pack_attributes(sh, uv, None, col)
    src = b.order
    t = tris[src].astype(np.float64)
    u = uv[src].astype(np.float64)
    e1, e2 = t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]
    du1, dv1, du2, dv2 = u[:, 2] - u[:, 0], u[:, 3] - u[:, 1], u[:, 4] - u[:, 0], u[:, 5] - u[:, 1]
    r = 1.0 / (du1 * dv2 - du2 * dv1)
    sdir = (dv2[:, None] * e1 - dv1[:, None] * e2) * r[:, None]
    tdir = (du1[:, None] * e2 - du2[:, None] * e1) * r[:, None]
    nrm = np.cross(e1, e2)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    tg = sdir - nrm * (nrm * sdir).sum(1, keepdims=True)
    tg /= np.linalg.norm(tg, axis=1, keepdims=True)
    cr = np.cross(tg, nrm)
    hand = np.where((cr * tdir).sum(1) < 0, 1.0, -1.0)
    bt = hand[:, None] * cr / np.linalg.norm(cr, axis=1, keepdims=True)

    def unpack10(bits):
        c = bits.view(np.int32)
        return np.stack([((c >> s) & 1023) / 1023.0 * 2.0 - 1.0 for s in (0, 10, 20)], axis=1)

    ok = np.abs(r) < 1e4          # well-conditioned UV triangles
    np.testing.assert_allclose(unpack10(sh[:, 16].copy())[ok], tg[ok], atol=4e-3)
    np.testing.assert_allclose(unpack10(sh[:, 17].copy())[ok], bt[ok], atol=4e-3)
    packed = sh[:, 20:23].copy().view(np.uint32)
    want = np.round(np.clip(col[src].reshape(-1, 3, 4), 0, 1) * 255).astype(np.uint32)
    want = want[..., 0] | (want[..., 1] << 8) | (want[..., 2] << 16) | (want[..., 3] << 24)
    np.testing.assert_array_equal(packed, want)


def test_textured_oracle_image_differs_from_plain():
    """The material textures reach the oracle's shading: a textured render
    differs from the same scene with the texture indices cleared."""
    from textured_util import build, oracle_scene
    sc, gt, sh, tex = build(grid=24, n_boxes=4)
    osc, _ = oracle_scene(sc, gt, sh)
    cam = scenes.pinhole_camera(32, 18)
    camv = np.concatenate([cam["location"], cam["origin"], cam["right"], cam["bottom"]]).astype(np.float32)
    a = pyoracle.pathtrace(*osc, camv, 32, 18, 16, textures=tex)
    plain = osc[4].copy()
    for t in ("baseColorTexture", "roughnessTexture", "metalnessTexture", "aoTexture", "normalTexture"):
        plain[t] = -1
    plain["useVertexColors"] = 0
    b = pyoracle.pathtrace(*osc[:4], plain, osc[5], camv, 32, 18, 16, textures=tex)
    assert np.isfinite(a).all() and a.mean() > 0
    assert abs(a.mean() - b.mean()) / b.mean() > 0.05


def test_mip_chain_known_answers():
    """Level k + 1 = 2 x 2 box of level k (UNORM rounding (a+b+c+d+2)//4),
    indices clamped at odd edges, down to 1 x 1."""
    t = np.array([[0, 4, 8, 12], [2, 6, 10, 255]], np.uint8)
    levels = pyoracle.mip_chain(t)
    assert [lv.shape for lv in levels] == [(1, 2), (1, 1)]
    np.testing.assert_array_equal(levels[0], [[(0 + 4 + 2 + 6 + 2) // 4, (8 + 12 + 10 + 255 + 2) // 4]])
    np.testing.assert_array_equal(levels[1], [[(3 + 3 + 71 + 71 + 2) // 4]])
    odd = np.arange(9, dtype=np.float32).reshape(3, 3)
    lv = pyoracle.mip_chain(odd)
    assert [x.shape for x in lv] == [(1, 1)]
    assert lv[0][0, 0] == np.float32(((0 + 1) + (3 + 4)) * 0.25)
    rgba = np.zeros((2, 2, 4), np.uint8)
    rgba[..., 2] = [[10, 20], [30, 41]]
    assert pyoracle.mip_chain(rgba)[0][0, 0, 2] == (10 + 20 + 30 + 41 + 2) // 4


def test_surface_lookups_read_the_requested_level():
    """The passes' surface lookups read uniforms.textureLevel: on the textured
    scene, RTGI at level 3 (box-filtered textures) differs from level 0,
    while levels past the chain's end clamp to its last level."""
    from passes_util import gbuffer
    from textured_util import build, oracle_scene
    sc, gt, sh, tex = build(grid=24, n_boxes=4)
    osc, _ = oracle_scene(sc, gt, sh)
    gb = gbuffer({"oracle": osc, "shading": sh}, 48, 27, samples=True)
    run = lambda lv: pyoracle.pass_screen("rtgi", osc + (tex,), gb, radiance_limit=4.0, texture_level=lv)
    a, b = run(0), run(3)
    assert np.abs(a - b).max() > 1e-3
    np.testing.assert_array_equal(run(20), run(5))     # the largest texture has 6 levels
