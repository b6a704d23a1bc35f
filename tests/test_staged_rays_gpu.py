"""Staged ray queue (AE_RT_CFG_STAGED_RAYS): warps take their rays in tiles
of 16 that one bulk copy (TMA) brings into shared memory.  Only where the
rays come from changes, so every result equals the plain loads' bit for bit:
single-mesh and scene traces, closest and any hit, ray counts around the
tile size, queue launches whose count is read on the device, and the path
tracer's per-ray shadow distances."""
import numpy as np
import pytest

import atlas_rt
from atlas_rt import BVH, scenes

from test_scene_gpu import build_scene, make_meshes, scene_rays

pytestmark = pytest.mark.gpu


def both(fn):
    out = []
    for staged in (False, True):
        ctx = atlas_rt.Context(device=0, staged_rays=staged)
        try:
            out.append(fn(ctx))
        finally:
            ctx.close()
    return out


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 33, 100_003])
def test_mesh_traces_equal_plain_loads(n):
    tris = scenes.random_triangles(30000, seed=41)
    o, d = scenes.sphere_rays(max(n, 1), seed=42)
    b = BVH(tris)
    gt = b.pack_triangles()
    rays = scenes.pack_rays(o[:n], d[:n])

    def run(ctx):
        m = ctx.upload_mesh(b.nodes, gt)
        h = ctx.trace_closest(m, rays, 1e-4, 10.0, n_rays=n)
        a = ctx.trace_any(m, rays, 1e-4, 10.0, n_rays=n)
        return h, a
    (h0, a0), (h1, a1) = both(run)
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
    assert np.array_equal(a0, a1)
    if n > 1000:
        assert 0.1 < (h0["triPtr"] >= 0).mean() < 0.95


@pytest.mark.parametrize("k", [0, 5, 65_541])
def test_queue_traces_equal_plain_loads(k):
    """Device-side counts (the wavefront queues): only the first `count` of
    the buffer's rays are traced (none for a zero count)."""
    import torch
    tris = scenes.random_triangles(30000, seed=43)
    o, d = scenes.sphere_rays(70_000, seed=44)
    b = BVH(tris)
    gt = b.pack_triangles()
    rays = torch.from_numpy(scenes.pack_rays(o, d)).cuda()
    count = torch.tensor([k], dtype=torch.int32, device="cuda")

    def run(ctx):
        m = ctx.upload_mesh(b.nodes, gt)
        hits = torch.full((len(o), 8), -7.0, device="cuda")
        occ = torch.full((len(o),), 3, dtype=torch.uint8, device="cuda")
        ctx.trace_closest_queue(m, rays, count, len(o), 1e-4, 10.0, hits)
        ctx.trace_any_queue(m, rays, count, len(o), 1e-4, 10.0, occ)
        ctx.synchronize()
        return hits.cpu().numpy(), occ.cpu().numpy()
    (h0, a0), (h1, a1) = both(run)
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
    assert np.array_equal(a0, a1)
    assert (h1[k:] == -7.0).all() and (a1[k:] == 3).all()


@pytest.mark.parametrize("cull", [0xFFFFFFFF, atlas_rt.MASK_SHADOW])
def test_scene_traces_equal_plain_loads(cull):
    meshes = make_meshes()
    o, d = scene_rays(50_000, 45)
    rays = scenes.pack_rays(o, d)

    def run(ctx):
        build_scene(ctx, meshes, 37, 46)
        h = ctx.trace_scene_closest(rays, 1e-4, 1e3, cull)
        a = ctx.trace_scene_any(rays, 1e-4, 1e3, cull)
        return h, a
    (h0, a0), (h1, a1) = both(run)
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
    assert np.array_equal(a0, a1)
    assert (h0["triPtr"] >= 0).mean() > 0.05


def test_cast_pass_and_path_tracer_equal_plain_loads():
    """The camera pass (primary, bounce and shadow queues) and the path
    tracer (shadow rays with per-ray distances) through the staged kernels."""
    import torch
    from atlas_rt import ptscene
    W, H = 320, 180
    sc = ptscene.build(grid=128, n_boxes=20)
    cam = atlas_rt.make_camera(scenes.pinhole_camera(W, H))
    bp = atlas_rt.make_bounce_params((0.4, 1.0, 0.3), 0.1, seed=1)

    def run(ctx):
        mid = ptscene.upload(ctx, sc)[0]
        ph = np.zeros((W * H, 8), np.float32)
        sh = np.zeros((W * H, 8), np.float32)
        occ = np.zeros(W * H, np.uint8)
        sr = np.zeros((W * H, 12), np.float32)
        dr = np.zeros((W * H, 12), np.float32)
        counts = ctx.cast_pass(mid, cam, bp, primary_hits=ph, secondary_rays=sr, secondary_hits=sh,
                               shadow_rays=dr, shadow_occluded=occ)
        acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
        ctx.pathtrace(cam, acc, spp=4, seed=9)
        ctx.synchronize()
        # the spawn's appends order the queues differently from run to run:
        # compare each queue's results by ray (pixel) ID
        o_sec = np.argsort(sr[:counts[1], 3].view(np.int32), kind="stable")
        o_shd = np.argsort(dr[:counts[2], 3].view(np.int32), kind="stable")
        return counts, ph, sh[:counts[1]][o_sec], occ[:counts[2]][o_shd], acc.cpu().numpy()
    r0, r1 = both(run)
    assert r0[0] == r1[0]
    for a, b in zip(r0[1:4], r1[1:4]):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    np.testing.assert_allclose(r1[4], r0[4], rtol=1e-5, atol=1e-6)
    assert r0[4][:, :3].mean() > 0
