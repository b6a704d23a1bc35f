"""Known answers of the oracle's passes (RTAO, reflections, RTGI, DDGI probe
rays; ao/rtao.csh, reflection/rtreflection.csh, rtgi/rtgi.csh,
ddgi/rayGen.csh + rayHit.csh) on a sandwich scene: a huge floor at y = 0
and a huge emissive ceiling at y = 1, no lights.  Every reflection, GI ray
and upward probe ray ends on the ceiling, so their radiance is the
ceiling's emission exactly; AO is 0 or 1 by the ray length alone."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, MATERIAL_DTYPE

from passes_util import fibonacci_dirs, gbuffer, unpack_ray_hits

EMIT = np.array([2.0, 3.0, 4.0], np.float32)
BIG = 1.0e4


def sandwich(ceiling_two_sided=True):
    """Floor (material 0, diffuse, facing up) and ceiling (material 1,
    emissive, facing down; one-sided and culling back faces on request)."""
    def quad(y, down):
        a, b, c, d = [-BIG, y, -BIG], [BIG, y, -BIG], [BIG, y, BIG], [-BIG, y, BIG]
        # cross(v0 - v1, v0 - v2), the normal of the backface test: -y for (a, b, c)
        return [[a, b, c], [a, c, d]] if down else [[a, c, b], [a, d, c]]
    tris = np.array(quad(0.0, False) + quad(1.0, True), np.float32)
    obj = np.array([0, 0, 1, 1], np.int32)
    m = np.zeros(2, MATERIAL_DTYPE)
    m["opacity"], m["ao"], m["roughness"], m["baseColor"] = 1.0, 1.0, 1.0, 0.5
    for t in ("baseColorTexture", "opacityTexture", "normalTexture", "roughnessTexture", "metalnessTexture",
              "aoTexture"):
        m[t] = -1
    m["twoSided"] = 1
    m[1]["emissiveColor"] = EMIT
    m[1]["baseColor"] = 0.0
    if not ceiling_two_sided:
        m[1]["twoSided"], m[1]["cullBackFaces"] = 0, 1
    b = BVH(tris)
    gt = b.pack_triangles(obj)
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    sh = b.pack_shading(np.repeat(n[:, None, :], 3, axis=1), obj)
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    model = np.tile(np.eye(3, 4, dtype=np.float32).reshape(-1), (1, 1))
    oracle = (top.nodes_f32, inst[top.order].copy(), model, [(b.nodes_f32, gt, sh)], m, np.zeros((0, 16), np.float32))
    return {"oracle": oracle, "shading": sh, "gt": gt, "bvh": b, "materials": m,
            "boxes": np.concatenate([lo, hi])[None, :]}


def floor_gbuffer(s, w=24, h=16, **kw):
    """The floor seen from straight above, from between the two planes."""
    return gbuffer(s, w, h, eye=(0.0, 0.5, 0.0), target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0), **kw)


@pytest.fixture(scope="module")
def sand():
    return sandwich()


def test_gbuffer_sees_the_floor(sand):
    gb = floor_gbuffer(sand)
    assert np.all(gb["depth"] < 1.0)


@pytest.mark.parametrize("half_res", [False, True])
def test_rtao_known_answers(sand, half_res):
    gb = floor_gbuffer(sand, half_res=half_res)
    # origins sit 0.1 + 0.1 * L.y above the floor: the ceiling is >= 0.8 away
    assert np.all(pyoracle.pass_screen("rtao", sand["oracle"], gb, radius=0.5) == 1.0)
    assert np.all(pyoracle.pass_screen("rtao", sand["oracle"], gb, radius=1e5) == 0.0)
    far = dict(gb, depth=np.ones_like(gb["depth"]))         # nothing drawn
    assert np.all(pyoracle.pass_screen("rtao", sand["oracle"], far, radius=1e5) == 1.0)


@pytest.mark.parametrize("kind", ["reflections", "rtgi"])
def test_reflection_and_gi_see_the_ceiling(sand, kind):
    """Mirror reflections (roughness <= 0.01) and cosine-weighted GI rays all
    leave the floor upwards."""
    h, w = 16, 24
    rough = np.where(np.arange(h * w) % 3 == 0, 0.0, 0.008).reshape(h, w)
    gb = floor_gbuffer(sand, roughness=rough, samples=True)
    out = pyoracle.pass_screen(kind, sand["oracle"], gb, radiance_limit=10.0, roughness_cutoff=0.9)
    np.testing.assert_array_equal(out[..., :3], np.broadcast_to(EMIT, (h, w, 3)))
    assert np.all(out[..., 3] == 1.0)
    # the radiance limit scales the colour so no channel exceeds it
    out = pyoracle.pass_screen(kind, sand["oracle"], gb, radiance_limit=2.5, roughness_cutoff=0.9)
    np.testing.assert_allclose(out[..., :3], np.broadcast_to(EMIT * np.float32(2.5 / 4.0), (h, w, 3)), rtol=1e-6)


def test_reflection_roughness_gates(sand):
    """Mirror pixels see the ceiling; glossy GGX samples see the ceiling or,
    below the surface, the unlit floor; pixels above the cutoff, or rougher
    than 1, trace nothing."""
    h, w = 16, 24
    rough = np.tile(np.array([0.0, 0.5, 0.95, 1.2], np.float32), h * w // 4).reshape(h, w)
    gb = floor_gbuffer(sand, roughness=rough)
    out = pyoracle.pass_screen("reflections", sand["oracle"], gb, roughness_cutoff=0.9)
    mirror, glossy = rough == 0.0, rough == 0.5
    np.testing.assert_array_equal(out[mirror, :3], np.broadcast_to(EMIT, (mirror.sum(), 3)))
    g = out[glossy, :3]
    ceiling = np.all(g == EMIT, axis=1)
    assert np.all(ceiling | np.all(g == 0.0, axis=1)) and ceiling.mean() > 0.6
    np.testing.assert_array_equal(out[~(mirror | glossy), :3], 0.0)


def test_ddgi_known_answers():
    s = sandwich(ceiling_two_sided=False)
    dirs = fibonacci_dirs(32)
    dirs_in = fibonacci_dirs(8)
    probes = np.array([[0.0, 0.4, 0.0, 0.0], [3.0, 0.7, 1.0, 0.0], [0.0, 0.5, 0.0, 0.0], [0.0, 5.0, 0.0, 0.0]],
                      np.float32)
    probes[1, 3] = np.uint32(1).view(np.float32)          # active
    probes[2, 3] = np.uint32(2).view(np.float32)          # inactive: 8 rays along dirs_in
    rot = np.eye(4)
    c, si = np.cos(0.3), np.sin(0.3)
    rot[:3, :3] = [[c, 0, si], [0, 1, 0], [-si, 0, c]]
    out = np.full((len(probes) * len(dirs), 4), -7.0, np.float32)
    pyoracle.pass_ddgi(s["oracle"], probes, dirs, rot, out, ray_dirs_inactive=dirs_in, inactive_ray_count=8,
                       environment=(0.25, 0.5, 0.75))
    d, rad, dist = unpack_ray_hits(out)
    for p, pr in enumerate(probes):
        inactive = p == 2
        src = dirs_in if inactive else dirs
        k = len(src)
        sl = slice(p * len(dirs), p * len(dirs) + k)
        want = src[:, :3] @ rot[:3, :3].T
        want /= np.linalg.norm(want, axis=1, keepdims=True)
        np.testing.assert_allclose(d[sl], want, atol=2e-3)            # half precision
        up = want[:, 1] > 0
        y = pr[1]
        if y < 1.0:
            # up: the ceiling's emission at (1 - y) / dir.y; down: the floor, no light
            np.testing.assert_allclose(dist[sl][up], (1.0 - y) / want[up, 1], rtol=1e-4)
            np.testing.assert_allclose(dist[sl][~up], -y / want[~up, 1], rtol=1e-4)
            np.testing.assert_array_equal(rad[sl][up], np.broadcast_to(EMIT, (up.sum(), 3)))
            np.testing.assert_array_equal(rad[sl][~up], 0.0)
        else:
            # above the ceiling: upward rays miss (environment, INF); downward
            # rays meet the ceiling's culled back face (radiance 0, -distance)
            np.testing.assert_array_equal(rad[sl][up], np.broadcast_to(np.float16([0.25, 0.5, 0.75]), (up.sum(), 3)))
            assert np.all(dist[sl][up] == np.float32(1e12))
            np.testing.assert_allclose(dist[sl][~up], -(y - 1.0) / -want[~up, 1], rtol=1e-4)
            np.testing.assert_array_equal(rad[sl][~up], 0.0)
        # entries beyond the probe's ray count stay as they were
        assert np.all(out[p * len(dirs) + k:(p + 1) * len(dirs)] == -7.0)
