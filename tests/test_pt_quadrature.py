"""A known answer for the path tracer's estimator, independent of both
implementations: a floor under a 2 x 2 emitter, one bounce (max_bounces = 0:
the first hit's emission and next-event estimation).  Each pixel's expected
radiance is the integral over the light of f(V, L) E cos(theta_x)
cos(theta_l) / d^2, computed here by a 400 x 400 midpoint rule in float64,
with f transcribed from the reference's GLSL once more:

* a grey diffuse floor: EvaluateDiffuseBRDF with RenormalizedDisneyDiffuse
  (brdf/brdfEval.hsh:8-19, brdf/brdf.hsh:15-25); the specular term vanishes
  for reflectance 0 and metalness 0;
* a rough metal floor: EvaluateSpecularBRDF, FresnelSchlick x
  DistributionGGX x VisibilitySmithGGXCorrelated (brdfEval.hsh:21-32,
  brdf.hsh:9-13, :34-53) with F0 = the base colour.

The oracle's restatement (CPU) and the GPU path tracer must both converge to
it: this pins the light selection, the triangle sampling and its pdf, the
area-to-solid-angle conversion and the shadow-ray setup (direct.hsh:12-86,
lights.hsh:11-29, rayHit.csh:209-235, :327-338) against quadrature rather
than against each other.  A second set of scenes (the floor alone under a
constant environment) does the same for the BRDF-sampled continuation; and
on all of them the GPU equals the oracle pixel for pixel, sample for sample.
"""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, MATERIAL_DTYPE, ptscene, scenes

F32 = np.float32
ALBEDO, RADIANCE, LIGHT_Y, HALF = 0.5, 10.0, 2.0, 1.0
FLOORS = {"diffuse": dict(base=ALBEDO, metalness=0.0, roughness=1.0),
          "metal": dict(base=0.8, metalness=1.0, roughness=0.5)}
# (mean, per pixel) relative tolerances at the test's sample counts: area
# sampling of the peaked GGX lobe is noisier (measured spread at 16,384
# samples: 0.8 % per pixel diffuse, 3.3 % metal)
TOL_ORACLE = {"diffuse": (0.005, 0.03), "metal": (0.01, 0.10)}
TOL_GPU = {"diffuse": (0.002, 0.01), "metal": (0.005, 0.04)}
EYE, TARGET = (0.3, 1.5, 0.2), (0.3, 0.0, 0.2)
W = H = 16
FOV = 40.0


def furnace_scene(floor_kind="diffuse"):
    """Floor (object 0) at y = 0 facing up, emitter (object 1) at y = 2 facing down."""
    big = 10.0
    a, b, c, d = [-big, 0, -big], [big, 0, -big], [big, 0, big], [-big, 0, big]
    floor = [[a, c, b], [a, d, c]]
    la, lb = [-HALF, LIGHT_Y, -HALF], [HALF, LIGHT_Y, -HALF]
    lc, ld = [HALF, LIGHT_Y, HALF], [-HALF, LIGHT_Y, HALF]
    light = [[la, lb, lc], [la, lc, ld]]
    tris = np.array(floor + light, F32)
    obj = np.array([0, 0, 1, 1], np.int32)
    normals = np.zeros((4, 3, 3), F32)
    normals[:2] = [0, 1, 0]
    normals[2:] = [0, -1, 0]
    mats = np.zeros(2, MATERIAL_DTYPE)
    mats["ID"] = [0, 1]
    mats["opacity"], mats["ao"], mats["normalScale"], mats["twoSided"] = 1.0, 1.0, 1.0, 1
    mats["roughness"], mats["metalness"], mats["reflectance"] = 1.0, 0.0, 0.0
    for t in ("baseColorTexture", "opacityTexture", "normalTexture", "roughnessTexture", "metalnessTexture",
              "aoTexture"):
        mats[t] = -1
    fl = FLOORS[floor_kind]
    mats[0]["baseColor"] = fl["base"]
    mats[0]["metalness"] = fl["metalness"]
    mats[0]["roughness"] = fl["roughness"]
    mats[1]["baseColor"] = 0.0
    mats[1]["emissiveColor"] = RADIANCE
    return {"tris": tris, "obj": obj, "normals": normals, "materials": mats, "bvh": BVH(tris), "light_obj": 1}


def camera():
    return scenes.pinhole_camera(W, H, fov_deg=FOV, eye=EYE, target=TARGET, up=(0.0, 0.0, 1.0))


def disney(NdotV, NdotL, LdotH, lr):
    """RenormalizedDisneyDiffuse (brdf/brdf.hsh)."""
    bias, factor = 0.5 * lr, 1.0 + (1.0 / 1.51 - 1.0) * lr
    fd90 = bias + 2.0 * LdotH * LdotH * lr
    return (1.0 + (fd90 - 1.0) * (1.0 - NdotL) ** 5) * (1.0 + (fd90 - 1.0) * (1.0 - NdotV) ** 5) * factor


def brdf(kind, NdotV, NdotL, NdotH, LdotH):
    fl = FLOORS[kind]
    a = max(fl["roughness"] ** 2, 1e-5)
    if fl["metalness"] == 0.0:
        return fl["base"] / np.pi * disney(NdotV, NdotL, LdotH, a)
    F0 = fl["base"]                                           # mix(0.16 reflectance^2, base, metalness)
    F90 = min(max(50.0 * (F0 * 0.333 * 3), 0.0), 1.0)
    F = F0 + (F90 - F0) * (1.0 - LdotH) ** 5
    a2 = a * a
    f = (NdotH * a2 - NdotH) * NdotH + 1.0
    D = a2 / (f * f + 1e-7) / np.pi
    gl = NdotV * np.sqrt((-NdotL * a2 + NdotL) * NdotL + a2)
    gv = NdotL * np.sqrt((-NdotV * a2 + NdotV) * NdotV + a2)
    G = 0.5 / (gl + gv + 1e-7)
    return F * D * G


def expected_image(kind="diffuse", n=400):
    """Per pixel centre: the floor point it sees and the midpoint-rule integral of the direct light."""
    cam = camera()
    u = (np.arange(W) + 0.5) / W
    v = (np.arange(H) + 0.5) / H
    d = (cam["origin"][None, None, :].astype(np.float64) + cam["right"][None, None, :] * u[None, :, None]
         + cam["bottom"][None, None, :] * v[:, None, None] - cam["location"])
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    eye = np.asarray(EYE, np.float64)
    x = eye + d * (-eye[1] / d[..., 1:2])                     # on the floor, y = 0
    g = (np.arange(n) + 0.5) / n * 2 * HALF - HALF
    ly = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    lp = np.stack([ly[:, 0], np.full(len(ly), LIGHT_Y), ly[:, 1]], 1)
    dA = (2 * HALF / n) ** 2
    out = np.zeros((H, W))
    for i in range(H):
        for j in range(W):
            p = x[i, j]
            V = (eye - p) / np.linalg.norm(eye - p)
            toL = lp - p
            d2 = (toL ** 2).sum(1)
            L = toL / np.sqrt(d2)[:, None]
            Hh = L + V
            Hh /= np.linalg.norm(Hh, axis=1, keepdims=True)
            NdotL = np.clip(L[:, 1], 0, 1)
            NdotV = np.clip(V[1], 0, 1)
            LdotH = np.clip((L * Hh).sum(1), 0, 1)
            NdotH = np.clip(Hh[:, 1], 0, 1)
            cos_l = np.clip(L[:, 1], 0, 1)                    # the light faces down: dot((0,-1,0), -L)
            f = brdf(kind, NdotV, NdotL, NdotH, LdotH)
            out[i, j] = np.sum(f * RADIANCE * NdotL * cos_l / d2) * dA
    return out


_EXPECTED = {}


def expected_for(kind):
    if kind not in _EXPECTED:
        _EXPECTED[kind] = expected_image(kind)
    return _EXPECTED[kind]


@pytest.mark.parametrize("kind", sorted(FLOORS))
def test_oracle_direct_light_matches_quadrature(kind):
    expected = expected_for(kind)
    sc = furnace_scene(kind)
    b = sc["bvh"]
    gt = b.pack_triangles(sc["obj"])
    sh = b.pack_shading(sc["normals"], sc["obj"])
    lights = ptscene.lights_for(sc, sh)
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (len(top.order), 1))
    camd = camera()
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(F32)
    spp = 4096
    img = pyoracle.pathtrace(top.nodes_f32, inst[top.order].copy(), model, [(b.nodes_f32, gt, sh)], sc["materials"],
                             lights, camv, W, H, spp, max_bounces=0)[..., 0] / spp
    tm, tp = TOL_ORACLE[kind]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(FLOORS))
def test_gpu_direct_light_matches_quadrature(kind):
    import torch
    expected = expected_for(kind)
    ctx = atlas_rt.Context(device=0)
    try:
        ptscene.upload(ctx, furnace_scene(kind))
        cam = atlas_rt.make_camera(camera())
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
        spp = 32768
        ctx.pathtrace(cam, acc, acc64, spp=spp, max_bounces=0)
        ctx.synchronize()
        img = acc64.cpu().numpy()[:, 0].reshape(H, W) / spp
    finally:
        ctx.close()
    tm, tp = TOL_GPU[kind]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)


# ---------------------------------------------------------------------------
# BRDF-sampled continuations: the floor alone under a constant environment
# ---------------------------------------------------------------------------
#
# No lights, max_bounces = 1: the first hit contributes nothing itself; its
# continuation (lobe choice, cosine or GGX-VNDF sampling and their pdfs,
# Russian roulette; rayHit.csh:237-325, brdfSample.hsh:8-90) escapes and adds
# min(E * throughput, 10) (rayHit.csh:166-171).  The expectation is E times the
# BRDF's directional albedo at the pixel's view angle, a hemisphere
# quadrature here.

ENV = 1.0


def floor_only_scene(kind):
    sc = furnace_scene(kind)
    keep = sc["obj"] == 0
    tris = sc["tris"][keep]
    sc.update(tris=tris, obj=sc["obj"][keep], normals=sc["normals"][keep], bvh=BVH(tris))
    sc["materials"] = sc["materials"][:1].copy()
    return sc


def directional_albedo(kind, mu_v, n_mu=2000, n_phi=720):
    """Integral over the upper hemisphere of f(V, L) cos(theta_L) for
    V at cos(theta) = mu_v (midpoint rule in cos(theta_L) and phi)."""
    mu = (np.arange(n_mu) + 0.5) / n_mu
    phi = (np.arange(n_phi) + 0.5) / n_phi * 2 * np.pi
    M, P = np.meshgrid(mu, phi, indexing="ij")
    s = np.sqrt(1 - M * M)
    L = np.stack([s * np.cos(P), M, s * np.sin(P)], -1)
    V = np.array([np.sqrt(1 - mu_v * mu_v), mu_v, 0.0])
    Hh = L + V
    Hh /= np.linalg.norm(Hh, axis=-1, keepdims=True)
    f = brdf(kind, mu_v, M, np.clip(Hh[..., 1], 0, 1), np.clip((L * Hh).sum(-1), 0, 1))
    return float(np.sum(f * M) * (1.0 / n_mu) * (2 * np.pi / n_phi))


def expected_env_image(kind):
    cam = camera()
    u = (np.arange(W) + 0.5) / W
    v = (np.arange(H) + 0.5) / H
    d = (cam["origin"][None, None, :].astype(np.float64) + cam["right"][None, None, :] * u[None, :, None]
         + cam["bottom"][None, None, :] * v[:, None, None] - cam["location"])
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    mu_v = -d[..., 1]                                         # N = (0, 1, 0), V = -d
    grid = np.linspace(mu_v.min() - 1e-3, min(mu_v.max() + 1e-3, 1.0), 16)
    table = np.array([directional_albedo(kind, m) for m in grid])
    return ENV * np.interp(mu_v, grid, table)


_ENV_EXPECTED = {}
# measured spread at 16,384 samples: 1.0 % per pixel diffuse, 1.5 % metal
TOL_ENV_ORACLE = {"diffuse": (0.005, 0.05), "metal": (0.005, 0.05)}
TOL_ENV_GPU = {"diffuse": (0.002, 0.02), "metal": (0.002, 0.02)}


def env_expected_for(kind):
    if kind not in _ENV_EXPECTED:
        _ENV_EXPECTED[kind] = expected_env_image(kind)
    return _ENV_EXPECTED[kind]


@pytest.mark.parametrize("kind", sorted(FLOORS))
def test_oracle_continuation_matches_albedo_quadrature(kind):
    expected = env_expected_for(kind)
    sc = floor_only_scene(kind)
    b = sc["bvh"]
    gt = b.pack_triangles(sc["obj"])
    sh = b.pack_shading(sc["normals"], sc["obj"])
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (len(top.order), 1))
    camd = camera()
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(F32)
    spp = 4096
    img = pyoracle.pathtrace(top.nodes_f32, inst[top.order].copy(), model, [(b.nodes_f32, gt, sh)], sc["materials"],
                             np.zeros((0, 16), F32), camv, W, H, spp, max_bounces=1,
                             environment=(ENV, ENV, ENV))[..., 0] / spp
    tm, tp = TOL_ENV_ORACLE[kind]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(FLOORS))
def test_gpu_continuation_matches_albedo_quadrature(kind):
    import torch
    expected = env_expected_for(kind)
    ctx = atlas_rt.Context(device=0)
    try:
        ptscene.upload(ctx, floor_only_scene(kind))
        ctx.set_environment((ENV, ENV, ENV))
        cam = atlas_rt.make_camera(camera())
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
        spp = 32768
        ctx.pathtrace(cam, acc, acc64, spp=spp, max_bounces=1)
        ctx.synchronize()
        img = acc64.cpu().numpy()[:, 0].reshape(H, W) / spp
        # the radiance cache refuses a scene with an environment
        rc = atlas_rt.RadianceCache(ctx, (-10.0, -1.0, -10.0), (10.0, 3.0, 10.0), log2_table=12)
        with pytest.raises(atlas_rt.AeRtError):
            rc.render(cam, 0, acc)
        rc.close()
    finally:
        ctx.close()
    tm, tp = TOL_ENV_GPU[kind]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(FLOORS))
@pytest.mark.parametrize("mode", ["direct", "environment"])
def test_gpu_equals_oracle_sample_for_sample(kind, mode):
    """Both sides draw the same random numbers (keyed by pixel, sample,
    bounce and dimension), and on these one-bounce scenes no path can take a
    different branch: every pixel agrees to float rounding, not statistically."""
    import torch
    sc = floor_only_scene(kind) if mode == "environment" else furnace_scene(kind)
    mb = 1 if mode == "environment" else 0
    env = (ENV, ENV, ENV) if mode == "environment" else None
    spp = 64
    ctx = atlas_rt.Context(device=0)
    try:
        mid, sh, lights, gt = ptscene.upload(ctx, sc)
        if env:
            ctx.set_environment(env)
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
        ctx.pathtrace(atlas_rt.make_camera(camera()), acc, acc64, spp=spp, max_bounces=mb)
        ctx.synchronize()
        g = acc64.cpu().numpy().reshape(H, W, 3)
    finally:
        ctx.close()
    b = sc["bvh"]
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (len(top.order), 1))
    camd = camera()
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(F32)
    c = pyoracle.pathtrace(top.nodes_f32, inst[top.order].copy(), model, [(b.nodes_f32, gt, sh)], sc["materials"],
                           lights if mode == "direct" else np.zeros((0, 16), F32), camv, W, H, spp, max_bounces=mb,
                           environment=env)
    assert (c > 0).mean() > 0.5
    np.testing.assert_allclose(g, c, rtol=2e-5, atol=1e-6)


# ---------------------------------------------------------------------------
# The opacity check: transparent surfaces in the path tracer's traversals
# ---------------------------------------------------------------------------
#
# The engine traces the path tracer's rays with its opacity check
# (PathTracingRenderer.cpp:186; CheckLeafClosestTransparency, bvh.hsh:106-134:
# a hit counts where its opacity is > 0) and weights each light sample by
# HitAnyTransparency (rayHit.csh:327-338).  Each case adds one large triangle
# to the direct-light scene:
#   * "half": opacity 0.5 between the floor and the light.  The shadow rays
#     visit its leaf alone, so their visibility is 1 * (1 * 0.5): every light
#     sample loses half (HitAnyTransparency multiplies the running value into
#     each leaf's result again, bvh.hsh:495, so a ray through several partly
#     transparent leaves would lose more; that order-dependent case is pinned
#     against the oracle's restatement in tests/test_transparency_gpu.py).
#   * "clear": opacity 0 between the camera and the floor: the camera sees
#     through it and the shadow rays lose nothing.

SHEETS = {"half": (1.8, 0.5, 0.5), "clear": (1.0, 0.0, 1.0)}     # (height, opacity, expected factor)


def sheet_scene(case, kind="diffuse"):
    sc = furnace_scene(kind)
    y, opa, _ = SHEETS[case]
    tri = np.array([[[-10.0, y, -10.0], [-10.0, y, 30.0], [30.0, y, -10.0]]], F32)   # covers x, z in [-10, 10]
    tris = np.concatenate([sc["tris"], tri]).astype(F32)
    obj = np.concatenate([sc["obj"], np.array([2], np.int32)])
    normals = np.concatenate([sc["normals"], np.tile(np.array([0, 1, 0], F32), (1, 3, 1))]).astype(F32)
    mats = np.zeros(3, MATERIAL_DTYPE)
    mats[:2] = sc["materials"]
    mats[2] = sc["materials"][0]
    mats[2]["ID"] = 2
    opacity = np.array([1, 1, 1, 1, opa], F32)
    sc.update(tris=tris, obj=obj, normals=normals, materials=mats, bvh=BVH(tris), opacity=opacity)
    return sc


def _oracle_image(sc, spp, mb):
    b = sc["bvh"]
    gt = b.pack_triangles(sc["obj"], sc.get("opacity"))
    sh = b.pack_shading(sc["normals"], sc["obj"], sc.get("opacity"))
    lights = ptscene.lights_for(sc, sh)
    lo, hi = atlas_rt.mesh_bounds(b)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    inst = np.array([atlas_rt.make_instance(np.eye(4), 0, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (len(top.order), 1))
    camd = camera()
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(F32)
    return pyoracle.pathtrace(top.nodes_f32, inst[top.order].copy(), model, [(b.nodes_f32, gt, sh)],
                              sc["materials"], lights, camv, W, H, spp, max_bounces=mb)


@pytest.mark.parametrize("case", sorted(SHEETS))
def test_oracle_opacity_check_matches_quadrature(case):
    expected = SHEETS[case][2] * expected_for("diffuse")
    spp = 4096
    img = _oracle_image(sheet_scene(case), spp, 0)[..., 0] / spp
    tm, tp = TOL_ORACLE["diffuse"]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(SHEETS))
def test_gpu_opacity_check_matches_quadrature_and_oracle(case):
    import torch
    expected = SHEETS[case][2] * expected_for("diffuse")
    sc = sheet_scene(case)
    ctx = atlas_rt.Context(device=0)
    try:
        ptscene.upload(ctx, sc)
        cam = atlas_rt.make_camera(camera())
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
        ctx.pathtrace(cam, acc, acc64, spp=32768, max_bounces=0)
        ctx.synchronize()
        img = acc64.cpu().numpy()[:, 0].reshape(H, W) / 32768
        acc64.zero_()
        ctx.pathtrace(cam, acc, acc64, spp=64, max_bounces=0)
        ctx.synchronize()
        g64 = acc64.cpu().numpy().reshape(H, W, 3)
        # the radiance cache refuses a scene that is not opaque
        rc = atlas_rt.RadianceCache(ctx, (-10.0, -1.0, -10.0), (10.0, 3.0, 10.0), log2_table=12)
        with pytest.raises(atlas_rt.AeRtError):
            rc.render(cam, 0, acc)
        rc.close()
    finally:
        ctx.close()
    tm, tp = TOL_GPU["diffuse"]
    assert abs(img.mean() - expected.mean()) / expected.mean() < tm, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=tp)
    # the same random numbers as the oracle: equal sample for sample
    np.testing.assert_allclose(g64, _oracle_image(sc, 64, 0), rtol=2e-5, atol=1e-6)


# ---------------------------------------------------------------------------
# The pass-through of a partially opaque surface the camera sees
# ---------------------------------------------------------------------------
#
# A diffuse sheet of opacity ALPHA at y = 1, between the camera (y = 1.5) and
# the floor, under the light (y = 2); max_bounces = 1.  EvaluateIndirectLight
# (rayHit.csh:237-325) passes through the sheet with chance
# clamp(1 - opacity, 0.1, 0.9) and throughput (1 - opacity) / chance, keeping
# the direction (:282-291); the reflection lobes take the rest and meet only
# the light's back or nothing (emission counts at bounce 0 only).  So a
# pixel's expectation is
#     ALPHA^2 D_sheet + (1 - ALPHA)^2 D_floor
# with D the direct-light quadrature at the sheet's and the floor's point on
# the camera ray: the sheet's own light sample carries the engine's opacity^2
# factor, and the floor's is reached with expected throughput 1 - ALPHA and
# seen through the sheet with visibility 1 - ALPHA (HitAnyTransparency).

ALPHA, SHEET_Y = 0.5, 1.0


def expected_at_height(y0, n=400):
    """expected_image's direct-light quadrature for a grey diffuse plane at
    height y0 (its normal up), at the point each pixel centre's ray meets it."""
    cam = camera()
    u = (np.arange(W) + 0.5) / W
    v = (np.arange(H) + 0.5) / H
    d = (cam["origin"][None, None, :].astype(np.float64) + cam["right"][None, None, :] * u[None, :, None]
         + cam["bottom"][None, None, :] * v[:, None, None] - cam["location"])
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    eye = np.asarray(EYE, np.float64)
    x = eye + d * ((y0 - eye[1]) / d[..., 1:2])
    g = (np.arange(n) + 0.5) / n * 2 * HALF - HALF
    ly = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    lp = np.stack([ly[:, 0], np.full(len(ly), LIGHT_Y), ly[:, 1]], 1)
    dA = (2 * HALF / n) ** 2
    out = np.zeros((H, W))
    for i in range(H):
        for j in range(W):
            p = x[i, j]
            V = (eye - p) / np.linalg.norm(eye - p)
            toL = lp - p
            d2 = (toL ** 2).sum(1)
            L = toL / np.sqrt(d2)[:, None]
            Hh = L + V
            Hh /= np.linalg.norm(Hh, axis=1, keepdims=True)
            NdotL = np.clip(L[:, 1], 0, 1)
            f = brdf("diffuse", np.clip(V[1], 0, 1), NdotL, np.clip(Hh[:, 1], 0, 1),
                     np.clip((L * Hh).sum(1), 0, 1))
            out[i, j] = np.sum(f * RADIANCE * NdotL * NdotL / d2) * dA
    return out


def pass_through_scene():
    sc = furnace_scene("diffuse")
    tri = np.array([[[-10.0, SHEET_Y, -10.0], [-10.0, SHEET_Y, 30.0], [30.0, SHEET_Y, -10.0]]], F32)
    tris = np.concatenate([sc["tris"], tri]).astype(F32)
    obj = np.concatenate([sc["obj"], np.array([2], np.int32)])
    normals = np.concatenate([sc["normals"], np.tile(np.array([0, 1, 0], F32), (1, 3, 1))]).astype(F32)
    mats = np.zeros(3, MATERIAL_DTYPE)
    mats[:2] = sc["materials"]
    mats[2] = sc["materials"][0]
    mats[2]["ID"] = 2
    mats[2]["opacity"] = ALPHA          # the triangles' opacity is the material's (MeshData.cpp:141)
    opacity = np.array([1, 1, 1, 1, ALPHA], F32)
    sc.update(tris=tris, obj=obj, normals=normals, materials=mats, bvh=BVH(tris), opacity=opacity)
    return sc


_PASS_EXPECTED = []


def pass_expected():
    if not _PASS_EXPECTED:
        _PASS_EXPECTED.append(ALPHA ** 2 * expected_at_height(SHEET_Y) + (1 - ALPHA) ** 2 * expected_at_height(0.0))
    return _PASS_EXPECTED[0]


def test_quadrature_at_height_zero_is_the_floors():
    np.testing.assert_allclose(expected_at_height(0.0, n=100), expected_image("diffuse", n=100), rtol=1e-12)


def test_oracle_pass_through_matches_quadrature():
    expected = pass_expected()
    spp = 8192
    img = _oracle_image(pass_through_scene(), spp, 1)[..., 0] / spp
    # the branch choice doubles the per-pixel variance of the one-bounce case
    assert abs(img.mean() - expected.mean()) / expected.mean() < 0.005, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=0.04)


@pytest.mark.gpu
def test_gpu_pass_through_matches_quadrature_and_oracle():
    import torch
    expected = pass_expected()
    sc = pass_through_scene()
    ctx = atlas_rt.Context(device=0)
    try:
        ptscene.upload(ctx, sc)
        cam = atlas_rt.make_camera(camera())
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
        spp = 65536
        ctx.pathtrace(cam, acc, acc64, spp=spp, max_bounces=1)
        ctx.synchronize()
        img = acc64.cpu().numpy()[:, 0].reshape(H, W) / spp
        acc64.zero_()
        ctx.pathtrace(cam, acc, acc64, spp=64, max_bounces=1)
        ctx.synchronize()
        g64 = acc64.cpu().numpy().reshape(H, W, 3)
    finally:
        ctx.close()
    assert abs(img.mean() - expected.mean()) / expected.mean() < 0.002, (img.mean(), expected.mean())
    np.testing.assert_allclose(img, expected, rtol=0.015)
    # both sides draw the same random numbers, the pass-through choice included
    np.testing.assert_allclose(g64, _oracle_image(sc, 64, 1), rtol=2e-5, atol=1e-6)
