"""The engine's shading math pinned to the reference's own code.

tests/golden/glsl_shading.npz holds golden vectors written by the reference's
GLSL helpers -- UpdateSurface, EvaluateDiffuseBRDF / EvaluateSpecularBRDF,
SampleDiffuseBRDF / SampleSpecularBRDF (GGX VNDF), SampleTriangleLight,
IntersectTriangle / IntersectAABB, the engine's random(), the software
scene traversals HitClosest / HitAny / HitClosestTransparency /
HitAnyTransparency of raytracer/bvh.hsh over a seeded two-level scene, the
path tracer's ray generation (pathtracer/rayGen.csh, whole dispatches), and
the engine's whole path tracer (rayGen.csh, the trace dispatch and
pathtracer/rayHit.csh, bounce by bounce; block statistics of thousands of its
samples), and the ambient-occlusion pass (ao/rtao.csh with and without
OPACITY_CHECK, whole dispatches over G-buffers, with its blue-noise sampler) --
compiled unmodified on the host by oracle/glsl/make_ref.py.  Here the oracle's
restatement (CPU) and the path tracer's and traversal's own device functions
(GPU, through ae_rt_selftest_shading) are held to them: the intersections bit
for bit, the BRDF from the reference's own surface terms to a few ulps, and
everything from raw vectors within the rounding of normalize / sqrt / pow
(shading_util.check states the tolerance and why).
"""
import numpy as np
import pytest

import shading_util as S


def test_fixture_is_what_the_reference_writes():
    """Where the reference tree is present, rebuilding the goldens from its
    GLSL gives the committed fixture bit for bit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import gen_glsl_goldens as G
    lib = G.reference_lib()
    if lib is None:
        pytest.skip("reference tree not present")
    g = S.golden()
    ins = G.inputs()
    for k, v in ins.items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k
    for k, v in G.evaluate(lib, ins).items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k
    sc = G.traversal_scene()
    assert G.scene_digest(sc) == bytes(g["trav_scene_digest"]).decode()
    for k, v in G.trace_scene(lib, sc).items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k
    for k, v in G.trace_raygen(lib).items():
        assert np.array_equal(v.view(np.uint32), g[k].view(np.uint32)), k
    for name in G.pt_cases():
        for k, v in G.trace_pt(lib, name).items():
            assert np.array_equal(np.asarray(v, g[k].dtype), g[k]), k
    for k, v in G.trace_passes(lib).items():
        assert np.array_equal(np.asarray(v).view(np.uint8), np.asarray(g[k]).view(np.uint8)), k


def test_reference_random_is_the_documented_hash():
    """random(x, seed) of common/random.hsh: Jenkins' one-at-a-time hash of the
    bits of vec2(x, seed), its low 23 bits as a float in [0, 1); the engine's
    draws, restated in numpy, equal the compiled GLSL's (the library's own
    RNG is a PCG hash instead, a documented deviation)."""
    g = S.golden()

    def h(x):
        x = np.uint64(x)
        M = np.uint64(0xFFFFFFFF)
        x = (x + (x << np.uint64(10))) & M
        x ^= x >> np.uint64(6)
        x = (x + (x << np.uint64(3))) & M
        x ^= x >> np.uint64(11)
        x = (x + (x << np.uint64(15))) & M
        return x
    out = np.zeros_like(g["random_out"])
    for i, x in enumerate(g["random_x"]):
        seed = np.float32(1.0)
        for k in range(8):
            bx, bs = np.float32(x).view(np.uint32), np.float32(seed).view(np.uint32)
            m = (int(bx) ^ int(h(int(bs)))) & 0xFFFFFFFF
            m = int(h(m)) & 0x007FFFFF | 0x3F800000
            out[i, k] = np.uint32(m).view(np.float32) - np.float32(1.0)
            seed = np.float32(seed + np.float32(1.0))
    assert np.array_equal(out.view(np.uint32), g["random_out"].view(np.uint32))


@pytest.mark.parametrize("name", sorted(S.SETS))
def test_oracle_matches_reference_glsl(name):
    g = S.golden()
    ik, ok, w, fn, extra, _ = S.SETS[name]
    got = S.run_oracle(fn, g[ik], w, *extra)
    S.check(name, got, g[ok], exact=name in ("triangle", "aabb", "triangle_light"))


def test_oracle_brdf_from_reference_terms():
    """The restated BRDF formulas, fed the reference's own surface terms, give
    its values to a few ulps (x^5 as products where the GLSL calls pow)."""
    g = S.golden()
    rows, ref = S.terms_rows(g)
    got = S.run_oracle("aeo_shade_eval_terms", rows, 6)
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(S.SETS))
def test_gpu_device_functions_match_reference_glsl(name):
    import atlas_rt
    g = S.golden()
    ik, ok, w, _, _, kind = S.SETS[name]
    ctx = atlas_rt.Context(device=0)
    try:
        got = S.run_gpu(ctx, kind, g[ik], w)
    finally:
        ctx.close()
    S.check(name, got, g[ok], exact=name in ("triangle", "aabb"))


@pytest.mark.gpu
def test_gpu_brdf_from_reference_terms():
    """The path tracer's BRDF device functions, fed the reference's own surface
    terms, give its values to a few ulps."""
    import atlas_rt
    g = S.golden()
    rows, ref = S.terms_rows(g)
    ctx = atlas_rt.Context(device=0)
    try:
        got = S.run_gpu(ctx, 4, rows, 6)
    finally:
        ctx.close()
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-30)


# ---- scene traversal: HitClosest / HitAny / HitClosestTransparency /
# HitAnyTransparency (raytracer/bvh.hsh) compiled from the reference's GLSL ----

# golden name -> (traversal, cull mask)
TRAVERSALS = {"closest": ("closest", 0xFFFFFFFF), "any": ("any", 0xFFFFFFFF),
              "closest_transparency": ("closest_transparency", 0xFFFFFFFF),
              "any_transparency": ("any_transparency", 0xFFFFFFFF),
              "closest_shadow": ("closest", 1 << 6),
              "closest_transparency_shadow": ("closest_transparency", 1 << 6),
              "any_transparency_shadow": ("any_transparency", 1 << 6)}


def _generator():
    import sys
    from pathlib import Path
    p = str(Path(__file__).resolve().parent / "golden")
    if p not in sys.path:
        sys.path.insert(0, p)
    import gen_glsl_goldens as G
    return G


_SCENE = {}


def traversal_scene():
    """The seeded scene the trav_* goldens were traced over, rebuilt (the
    library's builder and packers are deterministic) and checked against the
    fixture's digest of every array."""
    if "sc" not in _SCENE:
        G = _generator()
        sc = G.traversal_scene()
        assert G.scene_digest(sc) == bytes(S.golden()["trav_scene_digest"]).decode()
        _SCENE["sc"] = sc
    return _SCENE["sc"]


def check_traversal(name, ptr, inst, t, value):
    """ptr / inst / t: triangle, instance and distance of a closest-hit
    traversal (None for the any-hit ones), value: occlusion or transparency;
    all held to the reference's bit for bit.  A miss leaves hitID and
    hitInstanceID at -1 and hitDistance at tmax."""
    g = S.golden()["trav_" + name]
    gid, ginst = g[:, 0].view(np.int32), g[:, 1].view(np.int32)
    if ptr is not None:
        np.testing.assert_array_equal(ptr, gid)
        hit = gid >= 0
        np.testing.assert_array_equal(inst[hit], ginst[hit])
        assert (ginst[~hit] == -1).all()
        np.testing.assert_array_equal(t[hit].view(np.uint32), g[hit, 2].view(np.uint32))
        assert 0.05 < hit.mean() < 0.95
    else:
        np.testing.assert_array_equal(np.asarray(value, np.float32).view(np.uint32), g[:, 3].view(np.uint32))
        if name.startswith("any_transparency"):
            assert ((value > 0) & (value < 1)).mean() > 0.02    # partial opacities were crossed


def test_traversal_scene_is_the_golden_scene():
    traversal_scene()


@pytest.mark.parametrize("name", sorted(TRAVERSALS))
def test_oracle_scene_traversal_matches_reference_glsl(name):
    """The oracle's restated traversals give the reference's own HitClosest /
    HitAny / HitClosestTransparency / HitAnyTransparency results bit for bit:
    triangle, instance and distance, occlusion, and the product of the
    opacities crossed (per-triangle, material and texture opacity)."""
    import pyoracle
    sc = traversal_scene()
    kind, cull = TRAVERSALS[name]
    args = (sc["top"], sc["instances"], sc["meshes"])
    if kind == "closest":
        ptr, ino, tuv = pyoracle.scene_closest_glsl(*args, sc["rays8"], cull)
        check_traversal(name, ptr, ino, tuv[:, 0], None)
    elif kind == "any":
        check_traversal(name, None, None, None, pyoracle.scene_any_glsl(*args, sc["rays8"], cull).astype(np.float32))
    elif kind == "closest_transparency":
        ptr, ino, tuv = pyoracle.scene_closest_transparency_glsl(*args, sc["materials"], sc["rays8"], cull,
                                                                 textures=sc["textures"])
        check_traversal(name, ptr, ino, tuv[:, 0], None)
    else:
        tr = pyoracle.scene_any_transparency_glsl(*args, sc["materials"], sc["rays8"], cull, textures=sc["textures"])
        check_traversal(name, None, None, None, tr)


@pytest.mark.gpu
def test_gpu_scene_traversal_matches_reference_glsl():
    """The GPU's scene traversals (ae_rt_trace_scene_closest / _any /
    _closest_transparency / _any_transparency) over the reference-layout
    scene the goldens were traced on give the reference's results bit for
    bit."""
    import atlas_rt
    from atlas_rt import scenes
    sc = traversal_scene()
    r8 = sc["rays8"]
    tmin, tmax = float(r8[0, 6]), float(r8[0, 7])
    assert (r8[:, 6] == r8[0, 6]).all() and (r8[:, 7] == r8[0, 7]).all()
    packed = scenes.pack_rays(r8[:, 0:3], r8[:, 3:6])
    ctx = atlas_rt.Context(device=0)
    try:
        for k, (nodes, gt, sh) in enumerate(sc["meshes"]):
            assert ctx.upload_mesh(nodes, gt, sh) == k       # instances name meshes 0, 1, 2
        ctx.scene_set(sc["top"], sc["instances"])
        ctx.set_materials(sc["materials"])
        ctx.set_textures(sc["textures"])
        for name, (kind, cull) in sorted(TRAVERSALS.items()):
            if kind == "closest":
                h = ctx.trace_scene_closest(packed, tmin, tmax, cull)
            elif kind == "closest_transparency":
                h = ctx.trace_scene_closest_transparency(packed, tmin, tmax, cull)
            elif kind == "any":
                v = ctx.trace_scene_any(packed, tmin, tmax, cull)
            else:
                v = ctx.trace_scene_any_transparency(packed, tmin, tmax, cull)
            ctx.synchronize()
            if kind.startswith("closest"):
                check_traversal(name, h["triPtr"], h["instance"], h["t"], None)
            else:
                check_traversal(name, None, None, None, v.astype(np.float32))
    finally:
        ctx.close()


# ---- ray generation: pathtracer/rayGen.csh dispatched over whole images ----

def _raygen_case(w, h):
    G = _generator()
    g = S.golden()
    rays = g[f"raygen_{w}x{h}"]
    jitter = g[f"raygen_{w}x{h}_jitter"]
    return G, rays, jitter


@pytest.mark.parametrize("w,h", [(64, 40), (30, 17), (101, 67)])
def test_host_camera_rays_match_reference_raygen(w, h):
    """The host formula the oracle and the bench use (scenes.pinhole_rays:
    normalize(origin + right u + bottom v - location), (u, v) = (pixel +
    jitter) / resolution) gives the reference shader's rays, pixel by pixel,
    with the shader's per-frame jitter: origins bit for bit, directions to
    one unit in the last place -- the shim's normalize is the specification's
    x / length(x), the library's x * (1 / length(x)); a GPU driver's is an
    approximate reciprocal square root, so the last bit is not the engine's
    to fix.  The shader writes every pixel once."""
    from atlas_rt import scenes
    G, rays, jitter = _raygen_case(w, h)
    ids = rays[:, 3].view(np.int32)
    assert np.array_equal(np.sort(ids), np.arange(w * h))
    cam = scenes.pinhole_camera(w, h)
    o, d = scenes.pinhole_rays(cam, jitter=(float(jitter[0]), float(jitter[1])))
    assert np.array_equal(rays[:, 0:3], o[ids])
    ulps = np.abs(rays[:, 4:7].view(np.int32).astype(np.int64) - d[ids].view(np.int32))
    assert ulps.max() <= 1, ulps.max()


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(64, 40), (30, 17), (101, 67)])
def test_gpu_raygen_matches_reference_raygen(w, h):
    """ae_rt_raygen with the frame's jitter writes the reference shader's rays
    slot for slot: the same pixel (ray ID) in every queue position -- the
    8 x 8 work-group order, then the partial groups on the right, then
    those at the bottom -- with the same origin bits and directions to one
    unit in the last place (normalize; see the host test)."""
    import atlas_rt
    import torch
    from atlas_rt import scenes
    G, rays, jitter = _raygen_case(w, h)
    camd = scenes.pinhole_camera(w, h)
    camd["jitter"] = (float(jitter[0]), float(jitter[1]))
    cam = atlas_rt.make_camera(camd)
    ctx = atlas_rt.Context(device=0)
    try:
        out = torch.zeros((w * h, 12), dtype=torch.float32, device="cuda")
        ctx.raygen(cam, out)
        ctx.synchronize()
        got = out.cpu().numpy()
    finally:
        ctx.close()
    np.testing.assert_array_equal(got[:, 3].view(np.int32), rays[:, 3].view(np.int32))
    np.testing.assert_array_equal(got[:, 0:3].view(np.uint32), rays[:, 0:3].view(np.uint32))
    ulps = np.abs(got[:, 4:7].view(np.int32).astype(np.int64) - rays[:, 4:7].view(np.int32))
    assert ulps.max() <= 1, ulps.max()


# ---- the engine's own path tracer: rayGen.csh, the trace dispatch and
# rayHit.csh compiled on the host, run invocation by invocation ----

def pt_case(name):
    G = _generator()
    g = S.golden()
    sc, camd, w, h, _, _, _ = G.pt_cases()[name]
    spp, mb, blk = (int(x) for x in g[f"pt_{name}_spp"])
    return G, sc, camd, w, h, spp, mb, blk, g[f"pt_{name}_block_mean"], g[f"pt_{name}_block_var"]


def check_against_engine(name, img, n):
    """img: an image averaged over n samples of another estimator of the same
    expectation.  Per block of pixels, its mean against the engine's (the
    golden), in units of the standard error of the difference (the engine's
    per-sample block variance over both sample counts): the z values of an
    unbiased match are standard normal."""
    G, sc, camd, w, h, spp, mb, blk, bm, bv = pt_case(name)
    ob = img[:h // blk * blk, :w // blk * blk].reshape(h // blk, blk, w // blk, blk, 3).mean(axis=(1, 3))
    sig = np.sqrt(bv / spp + bv / n)
    live = sig > 0
    assert np.allclose(ob[~live], bm[~live], atol=1e-9)       # blocks that only ever see the black sky
    z = (ob[live] - bm[live]) / sig[live]
    assert z.size > 40
    assert (z ** 2).mean() < 1.6 and np.abs(z).max() < 5.0, ((z ** 2).mean(), np.abs(z).max())


@pytest.mark.parametrize("name", ["terrain", "sheet"])
def test_oracle_path_tracer_matches_the_engines_estimator(name):
    """The oracle's path tracer against the engine's own (rayGen.csh + the
    trace dispatch + rayHit.csh, compiled unmodified on the host; the golden
    holds 2,048 / 8,192 of its samples): the same expectation per block of
    pixels, within the noise -- 3 bounces over terrain and boxes with glossy
    and diffuse materials, and the transmission branch through a half-opaque
    sheet.  The scenes have one light triangle (see the two-light test)."""
    import pyoracle
    G, sc, camd, w, h, spp, mb, blk, bm, bv = pt_case(name)
    tl, inst, model, meshes, mats, lights = G.pt_arrays(sc)
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(np.float32)
    n = 8192 if name == "terrain" else 65536
    img = pyoracle.pathtrace(tl, inst, model, meshes, mats, lights, camv, w, h, n, max_bounces=mb) / n
    check_against_engine(name, img, n)


def test_engine_estimator_is_biased_with_two_lights():
    """A documented deviation.  The engine's GetLight and SampleLight
    (direct.hsh:12-86) take the random seed by value, so the light choice
    and the point sampled on the chosen light draw the same numbers; with two
    lights each light triangle is sampled over part of itself only.  Over the
    diffuse floor under its two-triangle emitter the engine's own estimator
    (golden) sits 12 % below the quadrature of the direct light, while the
    library's estimator, whose draws are independent, meets it (the
    quadrature tests); with one light triangle the two agree (above)."""
    import test_pt_quadrature as Q
    g = S.golden()
    ref = g["pt_two_lights_block_mean"][..., 0].mean()
    expected = Q.expected_for("diffuse").mean()
    assert 0.86 < ref / expected < 0.90, ref / expected


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["terrain", "sheet"])
def test_gpu_path_tracer_matches_the_engines_estimator(name):
    """The GPU path tracer against the engine's own estimator, as the oracle
    above: same scenes, same block statistics."""
    import atlas_rt
    import torch
    from atlas_rt import ptscene
    G, sc, camd, w, h, spp, mb, blk, bm, bv = pt_case(name)
    n = 32768 if name == "terrain" else 65536
    ctx = atlas_rt.Context(device=0)
    try:
        ptscene.upload(ctx, sc)
        cam = atlas_rt.make_camera(camd)
        acc = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
        acc64 = torch.zeros((w * h, 3), dtype=torch.float64, device="cuda")
        ctx.pathtrace(cam, acc, acc64, spp=n, max_bounces=mb)
        ctx.synchronize()
        img = acc64.cpu().numpy().reshape(h, w, 3) / n
    finally:
        ctx.close()
    check_against_engine(name, img, n)


# ---- the ambient-occlusion pass: ao/rtao.csh dispatched over G-buffers ----

_RTAO = {}


def pass_scene():
    """The seeded scene of the rtao_* and shade_* goldens, rebuilt and
    checked against the fixture's digest, with the oracle's scene tuple
    (instance model matrices inverted from the instances' inverse ones)."""
    if "sc" not in _RTAO:
        G = _generator()
        sc = G.pass_scene()
        assert G.scene_digest(sc) == bytes(S.golden()["pass_scene_digest"]).decode()
        model = np.zeros((len(sc["instances"]), 12), np.float32)
        for i, ins in enumerate(sc["instances"]):
            a = np.eye(4)
            a[:3] = np.asarray(ins["inverseMatrix"], np.float64).reshape(3, 4)
            model[i] = np.linalg.inv(a)[:3].reshape(-1)
        oracle = (sc["top"], sc["instances"], model, sc["meshes"], sc["materials"], sc["lights"], sc["textures"])
        _RTAO["sc"] = (sc, oracle)
    return _RTAO["sc"]


def upload_pass_scene(sc):
    """A context holding pass_scene: its three meshes, instances, materials,
    opacity textures and light."""
    import atlas_rt
    ctx = atlas_rt.Context(device=0)
    for k, (nodes, gt, sh) in enumerate(sc["meshes"]):
        assert ctx.upload_mesh(nodes, gt, sh) == k
    ctx.scene_set(sc["top"], sc["instances"])
    ctx.set_materials(sc["materials"])
    ctx.set_textures(sc["textures"])
    ctx.set_lights(sc["lights"])
    return ctx


def to_device(gb):
    import torch
    return {k: (torch.from_numpy(np.ascontiguousarray(v)).cuda() if isinstance(v, np.ndarray) and k not in
                ("ip_matrix", "iv_matrix") else v) for k, v in gb.items()}


def rtao_gbuffer(w, h):
    """The golden G-buffer of one case as Context.rtao / pyoracle.pass_screen
    take it (numpy), with the blue-noise textures."""
    G = _generator()
    g = S.golden()
    key = f"rtao_{w}x{h}"
    V, P = G.pass_camera(w, h)
    rank, sobol = G.blue_noise_textures()
    return {"depth": g[key + "_depth"], "normal": g[key + "_normal"], "offset": g[key + "_offset"], "half_res": 1,
            "ip_matrix": np.linalg.inv(P), "iv_matrix": np.linalg.inv(V), "scrambling_ranking": rank,
            "sobol_sequence": sobol}


def assert_ao_equal(got, ref):
    """Occlusion by HitAny is 0 or 1 and must match exactly.  With the
    opacity check, a ray that crossed only partly transparent surfaces
    carries the product of their opacities, which varies continuously with
    where the ray meets them: the opacity textures of the scene change by
    up to ~256 per world unit (random texels, 8 UV units per world unit),
    and a direction that differs from the shader's in its last bits (sin,
    cos and normalize round differently on the host and on the device)
    moves a hit 8 units away by ~5e-7, so those values agree to rtol 1e-3."""
    binary = (ref == 0.0) | (ref == 1.0)
    np.testing.assert_array_equal(got[binary], ref[binary])
    np.testing.assert_allclose(got[~binary], ref[~binary], rtol=1e-3, atol=1e-6)
    return binary


def check_rtao(got, ref, opacity):
    """got against the reference's rtao.csh where its dispatch wrote (ref !=
    -1), as assert_ao_equal states.  Returns the number of pixels the
    dispatch left unwritten."""
    wr = ref != -1.0
    r = ref[wr]
    binary = assert_ao_equal(got[wr], r)
    if opacity:
        assert (~binary).sum() > 0                      # partial opacities were crossed
    else:
        assert binary.all()
    drawn = rtao_gbuffer(*ref.shape[::-1])["depth"][wr] < 1.0
    assert 0.1 < (r[drawn] == 0.0).mean() < 0.5         # occluded and open pixels both occur
    return int((~wr).sum())


def _rtao_cases():
    G = _generator()
    return [(w, h, f, op) for (w, h) in G.RTAO_CASES for f in G.RTAO_FRAMES for op in (0, 1)]


def test_oracle_blue_noise_matches_reference():
    """The oracle's SampleBlueNoise gives the reference's bluenoise.hsh
    values bit for bit over a whole 128 x 128 period, for a sample index
    below 256 and one that wraps."""
    import pyoracle
    G = _generator()
    rank, sobol = G.blue_noise_textures()
    g = S.golden()
    for f in G.RTAO_FRAMES:
        ref = (g[f"rtao_blue_noise_{f}"].astype(np.float32) + np.float32(0.5)) / np.float32(256.0)
        got = pyoracle.blue_noise(rank, sobol, 128, 128, f)
        np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
        # the pattern repeats every 128 pixels
        big = pyoracle.blue_noise(rank, sobol, 300, 260, f)
        np.testing.assert_array_equal(big[128:256, 256:300], ref[:, :44])


@pytest.mark.parametrize("w,h,frame,opacity", _rtao_cases())
def test_oracle_rtao_matches_reference_rtao(w, h, frame, opacity):
    """The oracle's RTAO pass (blue-noise samples from the G-buffer's
    textures) against the reference's rtao.csh compiled on the host: one
    whole dispatch each, with and without OPACITY_CHECK."""
    import pyoracle
    sc, oracle = pass_scene()
    G = _generator()
    ref = S.golden()[f"rtao_{w}x{h}_ao_{frame}_{opacity}"]
    got = pyoracle.pass_screen("rtao", oracle, rtao_gbuffer(w, h), radius=G.RTAO_RADIUS, opacity_check=bool(opacity),
                               frame_seed=frame)
    unwritten = check_rtao(got, ref, opacity)
    assert unwritten == (0 if w % 32 == 0 else unwritten) and (unwritten > 0) == (w % 32 != 0)


def test_engine_rtao_dispatch_leaves_part_of_the_last_tile_column():
    """rtao.csh lays its one-dimensional dispatch onto tiles four work groups
    (32 pixels) wide, but AORenderer.cpp:85-88 dispatches only
    ceil(w / 8) * ceil(h / 4) groups: when ceil(w / 8) is not a multiple of
    4, the last tile gets fewer groups than it spans and pixels of its
    columns are never written (the engine's image keeps older values
    there).  The library writes every pixel."""
    g = S.golden()
    ref = g["rtao_44x20_ao_5_0"]
    gx, gy = (44 + 7) // 8, (20 + 3) // 4
    covered = np.zeros((20, 44), bool)
    for grp in range(gx * gy):
        tile, idx = divmod(grp, 4 * gy)
        x0, y0 = (tile * 4 + idx % 4) * 8, (idx // 4) * 4
        covered[y0:y0 + 4, x0:x0 + 8] = True
    np.testing.assert_array_equal(ref != -1.0, covered)
    assert not covered[:, 32:].all() and covered[:, :32].all()


@pytest.mark.gpu
def test_gpu_rtao_matches_reference_rtao():
    """The GPU's RTAO (ae_rt_rtao, blue-noise vectors drawn on the device
    from the G-buffer's textures) against the reference's rtao.csh over the
    same scene and G-buffers: every case, frame seed and variant; pixels
    the engine's dispatch leaves unwritten are held to the oracle."""
    import torch
    import atlas_rt
    import pyoracle
    sc, oracle = pass_scene()
    G = _generator()
    ctx = upload_pass_scene(sc)
    try:
        for w, h, frame, opacity in _rtao_cases():
            gb = rtao_gbuffer(w, h)
            dev = to_device(gb)
            out = torch.full((h, w), -5.0, dtype=torch.float32, device="cuda")
            params = dict(radius=G.RTAO_RADIUS, opacity_check=bool(opacity), frame_seed=frame)
            ctx.rtao(dev, out, **params)
            ctx.synchronize()
            got = out.cpu().numpy()
            ref = S.golden()[f"rtao_{w}x{h}_ao_{frame}_{opacity}"]
            check_rtao(got, ref, opacity)
            gap = ref == -1.0
            if gap.any():
                orc = pyoracle.pass_screen("rtao", oracle, gb, **params)
                assert_ao_equal(got[gap], orc[gap])
            # the same vectors handed over as samples give the same image
            samples = pyoracle.blue_noise(gb["scrambling_ranking"], gb["sobol_sequence"], w, h, frame)
            dev2 = {k: v for k, v in dev.items() if k not in ("scrambling_ranking", "sobol_sequence")}
            dev2["samples"] = torch.from_numpy(samples).cuda()
            out2 = torch.full((h, w), -5.0, dtype=torch.float32, device="cuda")
            ctx.rtao(dev2, out2, **params)
            ctx.synchronize()
            np.testing.assert_array_equal(out2.cpu().numpy(), got)
    finally:
        ctx.close()


# ---- the reflection and GI passes: rtreflection.csh and rtgi.csh ----

SHADE_KINDS = ("reflections", "rtgi")


def shade_gbuffer(w, h, half):
    G = _generator()
    g = S.golden()
    key = f"shade_{w}x{h}"
    V, P = G.pass_camera(w, h)
    rank, sobol = G.blue_noise_textures()
    return {"depth": g[key + "_depth"], "normal": g[key + "_normal"], "offset": g[key + "_offset"],
            "roughness": g[key + "_roughness"], "half_res": int(half), "ip_matrix": np.linalg.inv(P),
            "iv_matrix": np.linalg.inv(V), "scrambling_ranking": rank, "sobol_sequence": sobol}


def shade_params(opacity):
    G = _generator()
    lim, bias, cut, r, g, b = G.SHADE_PARAMS
    return dict(radiance_limit=lim, bias=bias, roughness_cutoff=cut, environment=(r, g, b),
                opacity_check=bool(opacity), frame_seed=G.SHADE_FRAME)


def shade_error(got, ref, atol):
    """Per pixel: the largest channel difference over atol + the pixel's
    largest channel (a radiance bound of atol absolute plus 1 relative)."""
    d = np.abs(got[..., :3] - ref[..., :3]).max(-1)
    return d / (atol + np.abs(ref[..., :3]).max(-1))


def _shade_cases():
    G = _generator()
    return [(w, h, half, kind, op) for (w, h, half) in G.SHADE_CASES for kind in SHADE_KINDS for op in (0, 1)]


@pytest.mark.parametrize("w,h,half,kind,opacity", _shade_cases())
def test_oracle_shading_passes_match_reference(w, h, half, kind, opacity):
    """The oracle's reflection and GI passes against the reference's
    rtreflection.csh / rtgi.csh compiled on the host: one whole dispatch each
    over a full- and a half-resolution G-buffer (mirror, glossy, rough,
    cut-off and untraced pixels), with and without OPACITY_CHECK, one
    directional light (shadows by HitAnyTransparency), emissive and
    partly transparent surfaces, the radiance limit and a constant
    environment.  Most pixels agree bit for bit; every pixel to 1e-5 + 1e-3
    of its largest channel (the rest differ by the rounding of the ray
    setup and the BRDF, which a dim pixel's cancellations magnify), alpha is
    1 everywhere, and pixels whose light term is negative (a one-sided back
    face lit from its front side) keep it as the shaders do."""
    import pyoracle
    sc, oracle = pass_scene()
    ref = S.golden()[f"shade_{w}x{h}_{kind}_{opacity}"]
    got = pyoracle.pass_screen(kind, oracle, shade_gbuffer(w, h, half), **shade_params(opacity))
    assert (got[..., 3] == 1.0).all() and (ref[..., 3] == 1.0).all()
    err = shade_error(got, ref, 1e-2)
    assert err.max() < 1e-3, err.max()
    assert (err == 0).mean() > 0.8
    assert (ref[..., :3] < 0).any(axis=-1).sum() > 0 and (ref[..., :3] > 0.5).any(axis=-1).sum() > 0


@pytest.mark.gpu
def test_gpu_shading_passes_match_reference():
    """The GPU's reflection and GI passes (ae_rt_reflections / ae_rt_rtgi,
    blue-noise vectors drawn on the device) against the reference's
    rtreflection.csh / rtgi.csh over the same scene and G-buffers.  Most
    pixels agree bit for bit and 99 % to 1e-4 of (1e-2 + the pixel's largest
    channel); the device's ray setup and BRDF use fast single-precision sin /
    cos / pow / rsqrt, which a dim pixel's cancellations magnify, so every
    pixel is held to 5e-3 of that bound."""
    import torch
    sc, oracle = pass_scene()
    ctx = upload_pass_scene(sc)
    try:
        for w, h, half, kind, opacity in _shade_cases():
            gb = shade_gbuffer(w, h, half)
            out = torch.full((h, w, 4), -5.0, dtype=torch.float32, device="cuda")
            getattr(ctx, kind)(to_device(gb), out, **shade_params(opacity))
            ctx.synchronize()
            got = out.cpu().numpy()
            ref = S.golden()[f"shade_{w}x{h}_{kind}_{opacity}"]
            assert (got[..., 3] == 1.0).all()
            err = shade_error(got, ref, 1e-2)
            assert err.max() < 5e-3 and (err < 1e-4).mean() > 0.99, (kind, opacity, w, err.max())
            assert (err == 0).mean() > 0.8
    finally:
        ctx.close()


# ---- DDGI probe rays: ddgi/rayGen.csh, the trace dispatch, ddgi/rayHit.csh ----

def ddgi_case(opacity):
    """The golden DDGI pass: the probes as the library takes them (the
    engine's ray origins, probe state bits in w), the direction sets, the
    rotation and the reference's PackedRayHit buffer (-7 where untouched)."""
    G = _generator()
    g = S.golden()
    states, offsets, dirs, dirs_in, rot = G.ddgi_inputs()
    probes = g[f"ddgi_origins_{opacity}"].copy()
    probes[:, 3] = states.view(np.float32)
    return probes, dirs, dirs_in, rot, g[f"ddgi_hits_{opacity}"]


def unpack_ray_hits(h):
    """PackedRayHit (ddgi/ddgi.hsh:70-98) -> direction, radiance, distance."""
    u = np.ascontiguousarray(h[:, :3]).view(np.uint32)
    lo = (u & 0xFFFF).astype(np.uint16).view(np.float16).astype(np.float32)
    hi = (u >> 16).astype(np.uint16).view(np.float16).astype(np.float32)
    d = np.stack([lo[:, 0], hi[:, 0], lo[:, 2]], 1)
    r = np.stack([lo[:, 1], hi[:, 1], hi[:, 2]], 1)
    return d, r, h[:, 3]


def check_ddgi(got, ref, dir_tol, rad_tol, dist_tol):
    untouched = np.all(ref == -7.0, axis=1)
    np.testing.assert_array_equal(untouched, np.all(got == -7.0, axis=1))
    gd, gr, gt = unpack_ray_hits(got[~untouched])
    rd, rr, rt = unpack_ray_hits(ref[~untouched])
    np.testing.assert_array_equal(np.signbit(gt), np.signbit(rt))       # back faces: negative distance
    assert (rt < 0).mean() > 0.05 and 0.2 < untouched.mean() < 0.5
    np.testing.assert_allclose(gd, rd, rtol=0, atol=dir_tol)
    np.testing.assert_allclose(gr, rr, rtol=rad_tol, atol=rad_tol * 0.1)
    np.testing.assert_allclose(gt, rt, rtol=dist_tol)


@pytest.mark.parametrize("opacity", [0, 1])
def test_oracle_ddgi_matches_reference(opacity):
    """The oracle's DDGI probe rays against the reference's ddgi/rayGen.csh,
    trace dispatch and ddgi/rayHit.csh compiled on the host over a 4 x 3 x 4
    probe grid (new, active and inactive probes; 32 and 8 rays; some probes
    under the ground or inside boxes, so one-sided back faces report a
    negative distance), one directional light and emitters: the packed
    directions and radiance bit for bit, distances to 1e-5."""
    import pyoracle
    sc, oracle = pass_scene()
    G = _generator()
    probes, dirs, dirs_in, rot, ref = ddgi_case(opacity)
    oracle = oracle[:4] + (G.ddgi_materials(sc),) + oracle[5:]
    got = np.full(ref.shape, -7.0, np.float32)
    pyoracle.pass_ddgi(oracle, probes, dirs, rot, got, ray_dirs_inactive=dirs_in, inactive_ray_count=len(dirs_in),
                       environment=G.DDGI_ENV, opacity_check=bool(opacity))
    np.testing.assert_array_equal(got[:, :3].view(np.uint32), ref[:, :3].view(np.uint32))
    check_ddgi(got, ref, 0.0, 0.0, 1e-5)


@pytest.mark.gpu
def test_gpu_ddgi_matches_reference():
    """The GPU's DDGI probe rays (ae_rt_ddgi_trace) against the reference's
    rayGen.csh, trace dispatch and rayHit.csh: the same slots written, the
    back faces the same, directions to one half-precision step, radiance to
    2e-3 (fast sin / cos / pow in the BRDF, then half precision) and
    distances to 1e-4."""
    import torch
    sc, oracle = pass_scene()
    G = _generator()
    ctx = upload_pass_scene(sc)
    try:
        ctx.set_materials(G.ddgi_materials(sc))
        for opacity in (0, 1):
            probes, dirs, dirs_in, rot, ref = ddgi_case(opacity)
            out = torch.full(ref.shape, -7.0, dtype=torch.float32, device="cuda")
            dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
            ctx.ddgi_trace(dev(probes), dev(dirs), rot, out, ray_dirs_inactive=dev(dirs_in),
                           inactive_ray_count=len(dirs_in), environment=G.DDGI_ENV, opacity_check=bool(opacity))
            ctx.synchronize()
            check_ddgi(out.cpu().numpy(), ref, 2.0 ** -10, 2e-3, 1e-4)
    finally:
        ctx.close()
