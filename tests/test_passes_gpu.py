"""The library's RTAO, reflection, GI and DDGI passes on the GPU: the
oracle's known answers on the sandwich scene (exact), and agreement with the
oracle on the terrain-and-boxes scene with lights.  Both sides draw the same
random numbers; their sin/cos/sqrt and the device's fused multiply-adds
differ in the last bits, so a ray that grazes an edge can land differently
and the comparison allows a small fraction of differing pixels."""
import numpy as np
import pytest

import atlas_rt
import pyoracle

from passes_util import fibonacci_dirs, gbuffer, small_scene, to_device, unpack_ray_hits, upload
from test_passes_oracle import EMIT, floor_gbuffer, sandwich

pytestmark = pytest.mark.gpu


def upload_sandwich(ctx, s):
    mid = ctx.upload_mesh(s["bvh"].nodes, s["gt"], s["shading"])
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    ctx.scene_build(inst, s["boxes"])
    ctx.set_materials(s["materials"])
    ctx.set_lights(np.zeros((0, 16), np.float32))


def run(ctx, kind, gb, **params):
    import torch
    h, w = gb["depth"].shape
    out = torch.full((h, w) if kind == "rtao" else (h, w, 4), -5.0, dtype=torch.float32, device="cuda")
    getattr(ctx, kind)(to_device(gb), out, **params)
    ctx.synchronize()
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def sand_ctx():
    ctx = atlas_rt.Context(device=0)
    s = sandwich()
    upload_sandwich(ctx, s)
    yield ctx, s
    ctx.close()


@pytest.mark.parametrize("half_res", [False, True])
@pytest.mark.parametrize("opacity", [False, True])
def test_rtao_known_answers(sand_ctx, half_res, opacity):
    ctx, s = sand_ctx
    gb = floor_gbuffer(s, half_res=half_res)
    assert np.all(run(ctx, "rtao", gb, radius=0.5, opacity_check=opacity) == 1.0)
    assert np.all(run(ctx, "rtao", gb, radius=1e5, opacity_check=opacity) == 0.0)
    far = dict(gb, depth=np.ones_like(gb["depth"]))
    assert np.all(run(ctx, "rtao", far, radius=1e5, opacity_check=opacity) == 1.0)


@pytest.mark.parametrize("kind", ["reflections", "rtgi"])
def test_reflection_and_gi_known_answers(sand_ctx, kind):
    ctx, s = sand_ctx
    h, w = 16, 24
    rough = np.where(np.arange(h * w) % 3 == 0, 0.0, 0.008).reshape(h, w)
    gb = floor_gbuffer(s, roughness=rough, samples=True)
    out = run(ctx, kind, gb, radiance_limit=10.0, roughness_cutoff=0.9)
    np.testing.assert_array_equal(out[..., :3], np.broadcast_to(EMIT, (h, w, 3)))
    assert np.all(out[..., 3] == 1.0)
    out = run(ctx, kind, gb, radiance_limit=2.5, roughness_cutoff=0.9)
    np.testing.assert_allclose(out[..., :3], np.broadcast_to(EMIT * np.float32(2.5 / 4.0), (h, w, 3)), rtol=1e-6)


def test_ddgi_known_answers():
    import torch
    ctx = atlas_rt.Context(device=0)
    try:
        s = sandwich(ceiling_two_sided=False)
        upload_sandwich(ctx, s)
        dirs, dirs_in = fibonacci_dirs(32), fibonacci_dirs(8)
        probes = np.array([[0.0, 0.4, 0.0, 0.0], [3.0, 0.7, 1.0, 0.0], [0.0, 0.5, 0.0, 0.0], [0.0, 5.0, 0.0, 0.0]],
                          np.float32)
        probes[1, 3] = np.uint32(1).view(np.float32)
        probes[2, 3] = np.uint32(2).view(np.float32)
        rot = np.eye(4)
        c, si = np.cos(0.3), np.sin(0.3)
        rot[:3, :3] = [[c, 0, si], [0, 1, 0], [-si, 0, c]]
        ref = np.full((len(probes) * len(dirs), 4), -7.0, np.float32)
        pyoracle.pass_ddgi(s["oracle"], probes, dirs, rot, ref, ray_dirs_inactive=dirs_in, inactive_ray_count=8,
                           environment=(0.25, 0.5, 0.75))
        out = torch.full(ref.shape, -7.0, dtype=torch.float32, device="cuda")
        dev = lambda a: torch.from_numpy(a).cuda()
        ctx.ddgi_trace(dev(probes), dev(dirs), rot, out, ray_dirs_inactive=dev(dirs_in), inactive_ray_count=8,
                       environment=(0.25, 0.5, 0.75))
        ctx.synchronize()
        got = out.cpu().numpy()
        gd, gr, gdist = unpack_ray_hits(got)
        rd, rr, rdist = unpack_ray_hits(ref)
        untouched = np.all(ref == -7.0, axis=1)
        assert np.array_equal(untouched, np.all(got == -7.0, axis=1))
        np.testing.assert_array_equal(gr[~untouched], rr[~untouched])       # radiance: EMIT, 0 or environment
        np.testing.assert_allclose(gd[~untouched], rd[~untouched], atol=1e-3)
        np.testing.assert_allclose(gdist[~untouched], rdist[~untouched], rtol=1e-5)
        assert (gdist[~untouched] < 0).sum() > 0                            # back faces were met
    finally:
        ctx.close()


@pytest.fixture(scope="module")
def terrain_ctx():
    ctx = atlas_rt.Context(device=0)
    s = small_scene(cull_terrain_backfaces=False)
    upload(ctx, s)
    yield ctx, s
    ctx.close()


@pytest.mark.parametrize("half_res,samples", [(False, False), (True, True)])
@pytest.mark.parametrize("opacity", [False, True])
def test_rtao_matches_oracle(terrain_ctx, half_res, samples, opacity):
    ctx, s = terrain_ctx
    gb = gbuffer(s, 160, 90, half_res=half_res, samples=samples)
    params = dict(radius=25.0, opacity_check=opacity, frame_seed=5, seed=3)
    got = run(ctx, "rtao", gb, **params)
    ref = pyoracle.pass_screen("rtao", s["oracle"], gb, **params)
    drawn = gb["depth"] < 1.0
    assert drawn.mean() > 0.5 and 0.03 < (ref[drawn] < 1.0).mean() < 0.97
    assert np.all(got[~drawn] == 1.0)
    assert (got == ref).mean() > 0.99


@pytest.mark.parametrize("kind", ["reflections", "rtgi"])
@pytest.mark.parametrize("opacity", [False, True])
def test_shading_passes_match_oracle(terrain_ctx, kind, opacity):
    ctx, s = terrain_ctx
    rng = np.random.default_rng(11)
    rough = rng.uniform(0.0, 1.1, (90, 160)).astype(np.float32)
    rough[rng.random((90, 160)) < 0.2] = 0.0
    gb = gbuffer(s, 160, 90, roughness=rough, samples=kind == "rtgi")
    params = dict(radiance_limit=4.0, roughness_cutoff=0.8, bias=0.1, environment=(0.05, 0.1, 0.2),
                  opacity_check=opacity, frame_seed=2, seed=9)
    got = run(ctx, kind, gb, **params)
    ref = pyoracle.pass_screen(kind, s["oracle"], gb, **params)
    assert np.all(got[..., 3] == 1.0)
    close = np.all(np.abs(got[..., :3] - ref[..., :3]) <= 1e-3 * np.abs(ref[..., :3]) + 1e-5, axis=2)
    assert close.mean() > 0.97
    lit = ref[..., :3].sum(axis=2) > 0.0
    assert lit.mean() > 0.3
    # the image means agree to within the few differing pixels
    np.testing.assert_allclose(got[..., :3].mean(), ref[..., :3].mean(), rtol=0.02)


def test_ddgi_matches_oracle():
    import torch
    ctx = atlas_rt.Context(device=0)
    try:
        s = small_scene(cull_terrain_backfaces=True)
        upload(ctx, s)
        g = np.stack(np.meshgrid(np.linspace(5, 95, 8), [-3.0, 6.0, 15.0], np.linspace(5, 95, 8), indexing="ij"),
                     -1).reshape(-1, 3)
        probes = np.concatenate([g, np.zeros((len(g), 1))], 1).astype(np.float32)
        states = np.arange(len(g)) % 3
        probes[:, 3] = states.astype(np.uint32).view(np.float32)
        dirs, dirs_in = fibonacci_dirs(96), fibonacci_dirs(24)
        rot = np.eye(4)
        rot[:3, :3] = np.linalg.qr(np.random.default_rng(4).normal(size=(3, 3)))[0]
        params = dict(environment=(0.3, 0.4, 0.5), frame_seed=7, seed=2)
        ref = np.full((len(probes) * len(dirs), 4), -7.0, np.float32)
        pyoracle.pass_ddgi(s["oracle"], probes, dirs, rot, ref, ray_dirs_inactive=dirs_in, inactive_ray_count=24,
                           **params)
        out = torch.full(ref.shape, -7.0, dtype=torch.float32, device="cuda")
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        ctx.ddgi_trace(dev(probes), dev(dirs), rot, out, ray_dirs_inactive=dev(dirs_in), inactive_ray_count=24,
                       **params)
        ctx.synchronize()
        got = out.cpu().numpy()
        untouched = np.all(ref == -7.0, axis=1)
        assert untouched.sum() == (states == 2).sum() * (96 - 24)
        assert np.array_equal(untouched, np.all(got == -7.0, axis=1))
        gd, gr, gdist = unpack_ray_hits(got[~untouched])
        rd, rr, rdist = unpack_ray_hits(ref[~untouched])
        np.testing.assert_allclose(gd, rd, atol=1e-3)
        same_t = np.abs(gdist - rdist) <= 1e-4 * np.abs(rdist)
        assert same_t.mean() > 0.99
        assert (rdist < 0).mean() > 0.05                     # probes under the one-sided terrain
        close = np.all(np.abs(gr - rr) <= 4e-3 * np.abs(rr) + 1e-4, axis=1)
        assert close.mean() > 0.97
    finally:
        ctx.close()


def test_device_gbuffer_matches_oracle_gbuffer(terrain_ctx):
    """atlas_rt.gbuffer.device_gbuffer (the library's closest hits) against
    the G-buffer made with the oracle's traversal."""
    from atlas_rt.gbuffer import device_gbuffer, look_at, perspective
    ctx, s = terrain_ctx
    w, h = 160, 90
    for half_res in (False, True):
        ref = gbuffer(s, w, h, half_res=half_res)
        V = look_at((50.0, 40.0, -15.0), (50.0, 0.0, 50.0))
        P = perspective(60.0, w / h, 0.5, 400.0)
        got = device_gbuffer(ctx, s["shading"], V, P, w, h, half_res=half_res)
        if half_res:
            np.testing.assert_array_equal(got["offset"].cpu().numpy(), ref["offset"])
        gd, rd = got["depth"].cpu().numpy(), ref["depth"]
        np.testing.assert_array_equal(gd >= 1.0, rd >= 1.0)
        assert (np.abs(gd - rd) <= 1e-6).mean() > 0.99
        same_n = np.all(np.abs(got["normal"].cpu().numpy() - ref["normal"]) <= 1e-5, axis=2)
        assert same_n.mean() > 0.99


def test_pass_argument_errors(sand_ctx):
    """Invalid calls return a status (no launch): host G-buffer planes, a
    missing roughness plane for reflections, host outputs, no scene."""
    import torch
    ctx, s = sand_ctx
    gb = floor_gbuffer(s)
    dev = to_device(gb)
    out = torch.empty((16, 24, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.rtao(gb, out[..., 0].contiguous())                 # host planes
    assert "device memory" in str(e.value)
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.reflections(dev, out)                              # no roughness plane
    assert "roughness" in str(e.value)
    with pytest.raises(atlas_rt.AeRtError):
        ctx.rtgi(dev, np.zeros((16, 24, 4), np.float32))       # host output
    empty = atlas_rt.Context(device=0)
    try:
        with pytest.raises(atlas_rt.AeRtError) as e:
            empty.rtao(dev, out[..., 0].contiguous())
        assert "scene" in str(e.value)
    finally:
        empty.close()
    # an empty G-buffer is a no-op
    z = dict(dev, depth=dev["depth"][:0], normal=dev["normal"][:0])
    ctx.rtao(z, out[..., 0].contiguous())
    ctx.synchronize()


def test_texture_argument_errors(sand_ctx):
    ctx, _ = sand_ctx
    with pytest.raises(ValueError):
        ctx.set_textures([np.zeros((4, 4, 3), np.uint8)])     # RGB8 is not a format
    with pytest.raises(atlas_rt.AeRtError):
        ctx.set_textures([np.zeros((0, 4), np.uint8)])        # empty texture
    ctx.set_textures([])                                       # clears the table


@pytest.mark.parametrize("kind,level", [("reflections", 0), ("rtgi", 0), ("rtgi", 2)])
def test_shading_passes_textured_match_oracle(kind, level):
    """The passes shade hits with the full material model too, at the
    texture level they are given (the device's mip chain against the
    oracle's)."""
    import textured_util
    ctx = atlas_rt.Context(device=0)
    try:
        sc, gt, sh, tex = textured_util.build()
        textured_util.upload(ctx, sc, gt, sh, tex)
        osc, _ = textured_util.oracle_scene(sc, gt, sh)
        s = {"oracle": osc, "shading": sh}
        rng = np.random.default_rng(12)
        rough = rng.uniform(0.0, 0.9, (90, 160)).astype(np.float32)
        gb = gbuffer(s, 160, 90, roughness=rough, samples=True)
        params = dict(radiance_limit=4.0, roughness_cutoff=0.8, environment=(0.05, 0.1, 0.2), frame_seed=4, seed=5,
                      texture_level=level)
        got = run(ctx, kind, gb, **params)
        ref = pyoracle.pass_screen(kind, osc + (tex,), gb, **params)
        close = np.all(np.abs(got[..., :3] - ref[..., :3]) <= 1e-3 * np.abs(ref[..., :3]) + 1e-5, axis=2)
        assert close.mean() > 0.97, close.mean()
        np.testing.assert_allclose(got[..., :3].mean(), ref[..., :3].mean(), rtol=0.02)
    finally:
        ctx.close()


def test_ddgi_textured_matches_oracle():
    """DDGI probe rays shade their hits with the surface textures at level 4
    (ddgi/rayHit.csh:79), on the GPU as in the oracle."""
    import torch
    import textured_util
    ctx = atlas_rt.Context(device=0)
    try:
        sc, gt, sh, tex = textured_util.build()
        textured_util.upload(ctx, sc, gt, sh, tex)
        osc, _ = textured_util.oracle_scene(sc, gt, sh)
        g = np.stack(np.meshgrid(np.linspace(5, 95, 6), [4.0, 12.0], np.linspace(5, 95, 6), indexing="ij"),
                     -1).reshape(-1, 3)
        probes = np.concatenate([g, np.zeros((len(g), 1))], 1).astype(np.float32)
        dirs = fibonacci_dirs(64)
        rot = np.eye(4)
        params = dict(environment=(0.3, 0.4, 0.5), frame_seed=3, seed=6)
        ref = np.zeros((len(probes) * len(dirs), 4), np.float32)
        pyoracle.pass_ddgi(osc + (tex,), probes, dirs, rot, ref, **params)
        out = torch.zeros(ref.shape, dtype=torch.float32, device="cuda")
        ctx.ddgi_trace(torch.from_numpy(probes).cuda(), torch.from_numpy(dirs).cuda(), rot, out, **params)
        ctx.synchronize()
        _, gr, gd = unpack_ray_hits(out.cpu().numpy())
        _, rr, rd = unpack_ray_hits(ref)
        assert (np.abs(gd - rd) <= 1e-4 * np.abs(rd)).mean() > 0.99
        close = np.all(np.abs(gr - rr) <= 4e-3 * np.abs(rr) + 1e-4, axis=1)
        assert close.mean() > 0.97, close.mean()
    finally:
        ctx.close()
