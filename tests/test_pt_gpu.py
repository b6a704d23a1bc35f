"""GPU path tracer against the CPU restatement of the same estimator.

Both sides draw the same random numbers (PCG hash keyed by pixel, sample,
bounce, dimension); their transcendental functions and summation orders
differ, so a path can diverge where rounding sends it down another branch.
Two comparisons follow: path for path (at low sample counts nearly every
pixel equals the oracle's to 1e-4) and statistical (at high sample counts
the two images agree to within their noise).
"""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, ptscene, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pt_setup():
    ctx = atlas_rt.Context(device=0)
    sc = ptscene.build()
    mid, shading, lights, gt = ptscene.upload(ctx, sc)
    bvh = sc["bvh"]
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(bvh)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    ordered = inst[top.order].copy()
    model = np.tile(np.eye(3, 4, dtype=np.float32).reshape(-1), (len(ordered), 1))
    oracle_scene = (top.nodes_f32, ordered, model, [(bvh.nodes_f32, gt, shading)], sc["materials"], lights)
    yield ctx, sc, oracle_scene
    ctx.close()


def gpu_render(ctx, w, h, spp, offset=0, accum64=False, seed=1, mis=False):
    import torch
    cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h))
    acc = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
    acc64 = torch.zeros((h * w, 3), dtype=torch.float64, device="cuda") if accum64 else None
    ctx.pathtrace(cam, acc, acc64, spp=spp, sample_offset=offset, seed=seed, mis=mis)
    ctx.synchronize()
    img = acc.cpu().numpy()[:, :3].reshape(h, w, 3)
    img64 = acc64.cpu().numpy().reshape(h, w, 3) if accum64 else None
    return img, img64


def cpu_render(oracle_scene, w, h, spp, offset=0, seed=1):
    camd = scenes.pinhole_camera(w, h)
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(np.float32)
    tl, inst, model, meshes, mats, lights = oracle_scene
    return pyoracle.pathtrace(tl, inst, model, meshes, mats, lights, camv, w, h, spp, sample_offset=offset, seed=seed)


def test_pt_matches_cpu_restatement(pt_setup):
    ctx, sc, osc = pt_setup
    w, h, spp = 64, 36, 2048
    g, g64 = gpu_render(ctx, w, h, spp, accum64=True)
    c = cpu_render(osc, w, h, spp)
    g, g64, c = g / spp, g64 / spp, c / spp
    # FP32 and FP64 accumulation of the same samples agree
    np.testing.assert_allclose(g, g64, rtol=1e-3, atol=1e-6)
    # whole-image energy within 1 %
    assert abs(g64.mean() - c.mean()) / c.mean() < 0.01, (g64.mean(), c.mean())
    # 4x4-pixel blocks within 5 % or 3e-4 absolute
    gb = g64.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))
    cb = c.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))
    bad = np.abs(gb - cb) > np.maximum(0.05 * cb, 3e-4)
    assert bad.mean() < 0.01, f"{bad.sum()} of {bad.size} blocks differ"
    # the relative MSE between the two estimates is at the noise level
    assert ptscene.rel_mse(g64, c) < 1e-4


def test_pt_sample_streams_continue(pt_setup):
    """Two calls of 256 samples (offset 0 and 256) equal one call of 512."""
    ctx, sc, osc = pt_setup
    a, _ = gpu_render(ctx, 48, 32, 256, offset=0)
    b, _ = gpu_render(ctx, 48, 32, 256, offset=256)
    ab, _ = gpu_render(ctx, 48, 32, 512, offset=0)
    np.testing.assert_allclose(a + b, ab, rtol=1e-4, atol=1e-6)


def test_pt_converges_with_spp(pt_setup):
    """rel-MSE against a high-spp image falls roughly as 1/spp."""
    ctx, sc, osc = pt_setup
    w, h = 96, 54
    ref, ref64 = gpu_render(ctx, w, h, 4096, offset=100000, accum64=True, seed=7)
    ref64 /= 4096
    errs = []
    for spp in (16, 64, 256):
        img, _ = gpu_render(ctx, w, h, spp, seed=3)
        errs.append(ptscene.rel_mse(img / spp, ref64))
    assert errs[0] > errs[1] > errs[2]
    assert 2.0 < errs[0] / errs[1] < 8.0 and 2.0 < errs[1] / errs[2] < 8.0, errs


def test_pt_mis_same_image(pt_setup):
    """The MIS option (next-event estimation + BRDF-sampled light hits,
    power heuristic, with the engine's capped GGX term restored on the BRDF
    side) converges to the engine estimator's image, and its error at 64
    samples is no worse."""
    ctx, sc, osc = pt_setup
    w, h = 96, 54
    _, ref = gpu_render(ctx, w, h, 8192, offset=300000, accum64=True, seed=7)
    _, mis = gpu_render(ctx, w, h, 8192, offset=300000, accum64=True, seed=9, mis=True)
    ref /= 8192
    mis /= 8192
    assert abs(mis.mean() - ref.mean()) / ref.mean() < 0.01, (mis.mean(), ref.mean())
    rb = ref.reshape(h // 6, 6, w // 6, 6, 3).mean(axis=(1, 3))
    mb = mis.reshape(h // 6, 6, w // 6, 6, 3).mean(axis=(1, 3))
    bad = np.abs(rb - mb) > np.maximum(0.05 * rb, 3e-4)
    assert bad.mean() < 0.02, f"{bad.sum()} of {bad.size} blocks differ"
    plain64, _ = gpu_render(ctx, w, h, 64, seed=3)
    mis64, _ = gpu_render(ctx, w, h, 64, seed=3, mis=True)
    e_plain = ptscene.rel_mse(plain64 / 64, ref)
    e_mis = ptscene.rel_mse(mis64 / 64, ref)
    assert e_mis < 1.2 * e_plain, (e_mis, e_plain)


def test_pt_textured_matches_cpu_restatement():
    """The material model of GetSurfaceParameters (vertex colours, base
    colour / roughness / metalness / ao textures, normal maps) on the GPU
    against the oracle's restatement, statistically, as the untextured test."""
    import textured_util
    ctx = atlas_rt.Context(device=0)
    try:
        sc, gt, sh, tex = textured_util.build()
        textured_util.upload(ctx, sc, gt, sh, tex)
        osc, _ = textured_util.oracle_scene(sc, gt, sh)
        w, h, spp = 64, 36, 2048
        _, g64 = gpu_render(ctx, w, h, spp, accum64=True)
        camd = scenes.pinhole_camera(w, h)
        camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(np.float32)
        c = pyoracle.pathtrace(*osc, camv, w, h, spp, textures=tex)
        g64, c = g64 / spp, c / spp
        assert abs(g64.mean() - c.mean()) / c.mean() < 0.01, (g64.mean(), c.mean())
        gb = g64.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))
        cb = c.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))
        bad = np.abs(gb - cb) > np.maximum(0.05 * cb, 3e-4)
        assert bad.mean() < 0.01, f"{bad.sum()} of {bad.size} blocks differ"
        assert ptscene.rel_mse(g64, c) < 1e-4
    finally:
        ctx.close()


def test_realtime_accumulation(pt_setup):
    """The real-time mode (rayHit.csh:134-150): at one sample per frame the
    frame holds each pixel's radiance as float bits, the same sum the
    non-real-time accumulation gets; at 4 samples the quantised unsigned
    sums, scaled back, agree with the float sums to the quantisation step
    per contribution.  Both trace the real-time primary rays: pixel centres
    plus the camera jitter / 4 (rayGen.csh:37-38)."""
    import torch
    ctx, sc, osc = pt_setup
    w, h = 64, 36
    camd = scenes.pinhole_camera(w, h)
    camd["jitter"] = (0.3, -0.2)
    cam = atlas_rt.make_camera(camd)
    for spp, offset in ((1, 5), (4, 40)):
        acc = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
        ctx.pathtrace(cam, acc, spp=spp, sample_offset=offset, centered=True)
        fr = torch.full((3, h, w), 7, dtype=torch.int32, device="cuda")
        ctx.pathtrace_realtime(cam, fr, max_radiance=64.0, spp=spp, sample_offset=offset)
        ctx.synchronize()
        ref = acc.cpu().numpy()[:, :3].reshape(h, w, 3).transpose(2, 0, 1)
        got = fr.cpu().numpy()
        if spp == 1:
            np.testing.assert_allclose(got.view(np.float32), ref, rtol=1e-5, atol=1e-7)
        else:
            step = 64.0 / (0xFFFFFFFF // spp)
            scaled = got.view(np.uint32).astype(np.float64) * step
            np.testing.assert_allclose(scaled, ref, rtol=1e-5, atol=64 * step)
        assert (ref > 0).mean() > 0.3


def test_tonemap_output():
    """ae_rt_pt_tonemap against the formula of rayHit.csh:124-130."""
    import torch
    ctx = atlas_rt.Context(device=0)
    try:
        rng = np.random.default_rng(3)
        acc = rng.uniform(0, 50, (33 * 17, 4)).astype(np.float32)
        out = torch.zeros((33 * 17, 4), dtype=torch.float32, device="cuda")
        ctx.tonemap(torch.from_numpy(acc).cuda(), 33, 17, 16, 1.5, 1 / 2.2, out)
        ctx.synchronize()
        want = np.power(1 - np.exp(-acc[:, :3].astype(np.float64) * 1.5 / 16), 1 / 2.2)
        np.testing.assert_allclose(out.cpu().numpy()[:, :3], want, rtol=2e-6, atol=1e-6)
        assert np.all(out.cpu().numpy()[:, 3] == 1.0)
    finally:
        ctx.close()


def test_tiles_reproduce_the_whole_image(pt_setup):
    """PathTracingRenderer's image subdivisions (rayGen.csh:25-30): tracing
    the image as 3 x 2 tiles (edges not multiples of 8) gives every pixel the
    same samples as one whole-image call, and a tile leaves the other pixels
    alone."""
    import torch
    ctx, sc, osc = pt_setup
    w, h = 66, 38
    cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h))
    whole = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
    ctx.pathtrace(cam, whole, spp=8, sample_offset=3)
    tiled = torch.zeros_like(whole)
    xs, ys = [0, 22, 44, 66], [0, 19, 38]
    for j in range(2):
        for i in range(3):
            ctx.pathtrace(cam, tiled, spp=8, sample_offset=3, tile=(xs[i], ys[j], xs[i + 1] - xs[i], ys[j + 1] - ys[j]))
    one = torch.zeros_like(whole)
    ctx.pathtrace(cam, one, spp=8, sample_offset=3, tile=(22, 19, 22, 19))
    ctx.synchronize()
    a, b, c = (t.cpu().numpy()[:, :3].reshape(h, w, 3) for t in (whole, tiled, one))
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(c[19:38, 22:44], a[19:38, 22:44])
    mask = np.ones((h, w), bool)
    mask[19:38, 22:44] = False
    assert np.all(c[mask] == 0) and (a > 0).mean() > 0.3
    for bad in ((60, 0, 10, 4), (0, 0, 0, 4), (0, 30, 4, 9)):
        with pytest.raises(atlas_rt.AeRtError):
            ctx.pathtrace(cam, one, spp=1, tile=bad)


def test_realtime_gbuffer(pt_setup):
    """The G-buffer of the real-time mode's first sample (rayHit.csh:76-116)
    against the same quantities rebuilt on the host from the primary rays'
    closest hits: view-space depth, material id, encoded geometry normal and
    the velocity under a camera that moved and an object that moved."""
    import torch
    from atlas_rt import gbuffer as gbm
    ctx, sc, osc = pt_setup
    w, h = 80, 45
    camd = scenes.pinhole_camera(w, h)
    camd["jitter"] = (0.0, 0.0)
    cam = atlas_rt.make_camera(camd)
    eye, target = np.array([50.0, 45.0, -22.0]), np.array([50.0, 0.0, 48.0])
    V = gbm.look_at(eye, target)
    P = gbm.perspective(60.0, w / h, 0.5, 2000.0)
    PV_last = P @ gbm.look_at(eye + [0.7, 0.2, 0.0], target + [0.7, 0.0, 0.0])
    last = np.eye(4)[:3].copy()
    last[:, 3] = [0.5, 0.0, -0.25]                      # the terrain instance moved since the last frame
    planes = {"depth": torch.zeros(h * w, dtype=torch.float32, device="cuda"),
              "material_idx": torch.zeros(h * w, dtype=torch.int32, device="cuda"),
              "normal": torch.zeros((h * w, 2), dtype=torch.float32, device="cuda"),
              "velocity": torch.zeros((h * w, 2), dtype=torch.float32, device="cuda")}
    fr = torch.zeros((3, h, w), dtype=torch.int32, device="cuda")
    # one matrix per instance on the device: a one-instance scene holds its
    # instance twice (the reference's single-box build, BVH.cpp:58-100)
    n_dev = len(osc[1])
    ctx.pathtrace_realtime(cam, fr, spp=1, gbuffer=dict(planes, view=V, proj=P, pv_last=PV_last,
                                                          last_matrices=np.repeat(last[None], n_dev, axis=0)))
    ctx.synchronize()
    depth = planes["depth"].cpu().numpy()
    mat = planes["material_idx"].cpu().numpy().view(np.uint32)
    nrm = planes["normal"].cpu().numpy()
    vel = planes["velocity"].cpu().numpy()

    # the host side: centre rays, their closest hits, the same formulas in float64
    px, py = np.meshgrid(np.arange(w), np.arange(h))
    u = ((px.reshape(-1) + 0.5) / w).astype(np.float32)
    v = ((py.reshape(-1) + 0.5) / h).astype(np.float32)
    d = camd["origin"] + camd["right"] * u[:, None] + camd["bottom"] * v[:, None] - camd["location"]
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    o = np.tile(camd["location"], (w * h, 1)).astype(np.float32)
    hits = torch.zeros((w * h, 8), dtype=torch.float32, device="cuda")
    ctx.trace_scene_closest(torch.from_numpy(scenes.pack_rays(o, d)).cuda(), 0.0, 1e12, out=hits, n_rays=w * h)
    ctx.synchronize()
    hh = hits.cpu().numpy()
    t, tri = hh[:, 0].astype(np.float64), hh[:, 1].view(np.int32)
    hit = tri >= 0
    assert 0.5 < hit.mean() < 1.0
    shading = sc["bvh"].pack_shading(sc["normals"], sc["obj"])
    tv = shading[np.maximum(tri, 0)]
    want_mat = np.where(hit, tv[:, 15].view(np.int32), 65535).astype(np.uint32)
    agree = want_mat == mat
    assert agree.mean() > 0.98, agree.mean()           # silhouettes may pick the neighbour
    Pw = np.where(hit[:, None], o + d.astype(np.float64) * t[:, None], o + d.astype(np.float64) * 100.0)
    vs = np.c_[Pw, np.ones(len(Pw))] @ V.T
    want_depth = np.where(hit, vs[:, 2], 1e12)
    m = agree & hit
    np.testing.assert_allclose(depth[m], want_depth[m], rtol=2e-4)
    assert np.all(depth[~hit & agree] == np.float32(1e12))
    n = np.cross(tv[:, 0:3] - tv[:, 4:7], tv[:, 0:3] - tv[:, 8:11])
    n /= np.linalg.norm(n, axis=1, keepdims=True) + 1e-30
    n = np.where(((n * d).sum(1) > 0)[:, None], -n, n)          # two-sided: faces the ray
    n = np.where(hit[:, None], n, [1.0, 0.0, 0.0])
    np.testing.assert_allclose(nrm[agree], gbm.encode_normal(n)[agree], atol=2e-3)
    lastP = np.where(hit[:, None], Pw + last[:, 3], Pw)
    cur = np.c_[Pw, np.ones(len(Pw))] @ (P @ V).T
    prev = np.c_[lastP, np.ones(len(Pw))] @ PV_last.T
    want_vel = (prev[:, :2] / prev[:, 3:] - cur[:, :2] / cur[:, 3:]) * 0.5
    np.testing.assert_allclose(vel[agree], want_vel[agree], atol=2e-4 + 1e-3 * np.abs(want_vel[agree]).max())
    assert np.abs(vel[m]).max() > 1e-3                          # the motion is visible


def test_pt_equals_cpu_restatement_path_for_path(pt_setup):
    """Both sides draw the same random numbers, so a path differs only where
    float rounding (fast-math shading on the GPU, exact arithmetic in the
    oracle) sends it down another branch: at 1 and 8 samples with 3 bounces,
    at least 99.5 % of the pixels equal the oracle's to 1e-4 relative
    (measured: 99.9 %), and the image means agree to 2e-3."""
    import torch
    ctx, sc, osc = pt_setup
    w, h = 96, 54
    for spp in (1, 8):
        acc = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((h * w, 3), dtype=torch.float64, device="cuda")
        ctx.pathtrace(atlas_rt.make_camera(scenes.pinhole_camera(w, h)), acc, acc64, spp=spp, max_bounces=3)
        ctx.synchronize()
        g = acc64.cpu().numpy().reshape(h, w, 3)
        c = cpu_render(osc, w, h, spp)
        rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-6)
        equal = np.all(rel < 1e-4, axis=2)
        assert equal.mean() >= 0.995, equal.mean()
        # the few diverged paths move the image mean (measured 2e-4 at 1 sample)
        assert abs(g.mean() - c.mean()) / c.mean() < 2e-3, (g.mean(), c.mean())
