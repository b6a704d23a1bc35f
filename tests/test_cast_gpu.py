"""The camera ray-cast pass (ray generation, bounce/shadow spawn, queue-driven
traces) on the GPU, checked against host arithmetic and the oracle."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def terrain(ctx):
    tris, _ = scenes.terrain_boxes()
    b = BVH(tris)
    gt = b.pack_triangles()
    return b, gt, ctx.upload_mesh(b.nodes, gt)


def rays8(packed, tmin, tmax):
    r = np.empty((len(packed), 8), np.float32)
    r[:, 0:3] = packed[:, 0:3]
    r[:, 3:6] = packed[:, 4:7]
    r[:, 6], r[:, 7] = tmin, tmax
    return r


@pytest.mark.parametrize("w,h", [(64, 40), (30, 17), (1920, 1080)])
def test_raygen_matches_host_formula(ctx, w, h):
    import torch
    camd = scenes.pinhole_camera(w, h)
    cam = atlas_rt.make_camera(camd)
    rays = torch.zeros((w * h, 12), dtype=torch.float32, device="cuda")
    ctx.raygen(cam, rays)
    ctx.synchronize()
    got = rays.cpu().numpy()
    ids = got[:, 3].view(np.int32)
    assert np.array_equal(np.sort(ids), np.arange(w * h))
    o, d = scenes.pinhole_rays(camd)
    assert np.array_equal(got[:, 0:3], o[ids])
    assert np.array_equal(got[:, 4:7].view(np.uint32), d[ids].view(np.uint32))
    if w % 8 == 0 and h % 8 == 0:
        # 8x8 tile order: the first 64 slots are the top-left tile
        first = ids[:64]
        assert set((first % w).tolist()) == set(range(8)) and set((first // w).tolist()) == set(range(8))


@pytest.mark.parametrize("host", ["pageable", "pinned"])
def test_cast_pass_parity(ctx, terrain, host):
    """Pageable host outputs go through device scratch and copies; pinned
    ones are written by the trace kernels directly where nothing on the
    device reads them again (bounce hits, shadow occlusion)."""
    b, gt, mid = terrain
    import torch
    w, h = 640, 360
    camd = scenes.pinhole_camera(w, h)
    cam = atlas_rt.make_camera(camd)
    bp = atlas_rt.make_bounce_params((0.4, 1.0, 0.3), 0.1, seed=3)
    n = w * h
    if host == "pinned":
        bufs = [torch.full(shape, -3, dtype=dt, pin_memory=True)
                for shape, dt in (((n, 8), torch.float32), ((n, 12), torch.float32), ((n, 8), torch.float32),
                                  ((n, 12), torch.float32), ((n,), torch.uint8))]
        args = bufs
        ph, sr, sh, dr, oc = (t.numpy() for t in bufs)
        ph, sh = ph.view(atlas_rt.HIT_DTYPE).reshape(n), sh.view(atlas_rt.HIT_DTYPE).reshape(n)
    else:
        ph = np.zeros(n, atlas_rt.HIT_DTYPE)
        sr = np.zeros((n, 12), np.float32)
        sh = np.zeros(n, atlas_rt.HIT_DTYPE)
        dr = np.zeros((n, 12), np.float32)
        oc = np.zeros(n, np.uint8)
        args = [ph, sr, sh, dr, oc]
    n0, n1, n2 = ctx.cast_pass(mid, cam, bp, primary_hits=args[0], secondary_rays=args[1], secondary_hits=args[2],
                               shadow_rays=args[3], shadow_occluded=args[4])
    assert n0 == n and 0 < n1 <= n and 0 < n2 <= n1
    # primary rays regenerated on the host in the same tile order
    prim = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
    ctx.raygen(cam, prim)
    ctx.synchronize()
    prim = prim.cpu().numpy()
    ptr, tuv = pyoracle.closest_glsl(b.nodes_f32, gt, rays8(prim, 0.0, 1e12))
    assert np.array_equal(ph["triPtr"], ptr)
    assert np.array_equal(ph["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    assert n1 == int((ptr >= 0).sum())
    # bounce rays: traced bit-identically; unit directions in the upper hemisphere
    sec = sr[:n1]
    p2, t2 = pyoracle.closest_glsl(b.nodes_f32, gt, rays8(sec, 0.0, 1e12))
    assert np.array_equal(sh["triPtr"][:n1], p2)
    assert np.array_equal(sh["t"][:n1].view(np.uint32), t2[:, 0].view(np.uint32))
    np.testing.assert_allclose(np.linalg.norm(sec[:, 4:7], axis=1), 1.0, atol=1e-5)
    # shadow rays: occlusion bit-identical to the oracle
    shd = dr[:n2]
    o2 = pyoracle.any_glsl(b.nodes_f32, gt, rays8(shd, 0.0, 1e12 - 0.2))
    assert np.array_equal(oc[:n2], o2)
    L = np.array([0.4, 1.0, 0.3]) / np.linalg.norm([0.4, 1.0, 0.3])
    np.testing.assert_allclose(shd[:, 4:7], np.broadcast_to(L.astype(np.float32), (n2, 3)), atol=1e-7)
    # every ray keeps the pixel ID of its primary ray
    prim_ids = set(prim[ph["triPtr"] >= 0, 3].view(np.int32).tolist())
    assert set(sec[:, 3].view(np.int32).tolist()) == prim_ids
    assert set(shd[:, 3].view(np.int32).tolist()) <= prim_ids


def test_cast_pass_cosine_distribution(ctx):
    """Bounce directions off a flat floor follow cos(theta)/pi: E[cos] = 2/3."""
    tris = np.array([[[-100, 0, -100], [100, 0, 100], [100, 0, -100]],
                     [[-100, 0, -100], [-100, 0, 100], [100, 0, 100]]], np.float32)
    b = BVH(tris)
    mid = ctx.upload_mesh(b.nodes, b.pack_triangles())
    camd = scenes.pinhole_camera(256, 256, eye=(0, 10, 0), target=(0, 0, 0.001), up=(0, 0, 1))
    cam = atlas_rt.make_camera(camd)
    sr = np.zeros((256 * 256, 12), np.float32)
    n0, n1, _ = ctx.cast_pass(mid, cam, atlas_rt.make_bounce_params(seed=11), secondary_rays=sr)
    assert n1 == n0
    cy = sr[:n1, 5]
    assert np.all(cy > 0)
    assert abs(cy.mean() - 2.0 / 3.0) < 0.01


def _by_id(rows):
    rows = rows.view(np.uint32)
    return rows[np.argsort(rows[:, 3].view(np.int32), kind="stable")]


@pytest.mark.parametrize("w,h", [(64, 40), (30, 17), (1920, 1080)])
def test_camera_trace_equals_raygen_then_trace(ctx, terrain, w, h):
    """trace_camera_closest makes each lane's ray in the traversal kernel:
    its hits equal raygen + trace_closest word for word (partial 8x8 tiles
    included), and spawn_bounce_camera appends the same bounce and shadow
    rays as spawn_bounce over the stored rays (queue order differs: the
    appends are atomics)."""
    import torch
    b, gt, mid = terrain
    n = w * h
    cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h))
    cam.jitter[0], cam.jitter[1] = 0.3, -0.7
    bp = atlas_rt.make_bounce_params((0.4, 1.0, 0.3), 0.1, seed=5)
    dev = "cuda"
    prim = torch.zeros((n, 12), dtype=torch.float32, device=dev)
    ref = torch.zeros((n, 8), dtype=torch.float32, device=dev)
    got = torch.full((n, 8), -7.0, dtype=torch.float32, device=dev)
    ctx.raygen(cam, prim)
    ctx.trace_closest(mid, prim, 0.0, float("inf"), out=ref, n_rays=n)
    ctx.trace_camera_closest(mid, cam, got)
    host = np.zeros((n, 8), np.float32)
    ctx.trace_camera_closest(mid, cam, host)   # pageable host hits: through scratch and a copy
    ctx.synchronize()
    assert np.array_equal(got.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32))
    assert np.array_equal(host.view(np.uint32), ref.cpu().numpy().view(np.uint32))
    qs = []
    for camera in (False, True):
        sec = torch.zeros((n, 12), dtype=torch.float32, device=dev)
        shd = torch.zeros((n, 12), dtype=torch.float32, device=dev)
        counts = torch.zeros(4, dtype=torch.int32, device=dev)
        if camera:
            ctx.spawn_bounce_camera(mid, cam, got, bp, sec, shd, counts)
        else:
            ctx.spawn_bounce(mid, prim, ref, n, bp, sec, shd, counts)
        ctx.synchronize()
        c = counts.cpu().numpy()
        qs.append((c[:2].tolist(), _by_id(sec[:c[0]].cpu().numpy()), _by_id(shd[:c[1]].cpu().numpy())))
    assert qs[0][0] == qs[1][0] and qs[0][0][0] > 0
    assert np.array_equal(qs[0][1], qs[1][1]) and np.array_equal(qs[0][2], qs[1][2])


def test_camera_trace_general_paths(terrain):
    """Where the traversal kernel cannot make the rays (a tree deeper than
    128 levels, or the approximate traversal) the camera trace writes them to
    scratch first; the hits still equal raygen + trace_closest."""
    import torch
    from test_trace_gpu import chain_bvh
    w, h = 48, 24
    n = w * h
    cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h, eye=(0.5, 0.5, -2.0), target=(0.5, 0.5, 1.0)))
    b, gt, _ = terrain
    for kwargs, mesh in (({}, chain_bvh(300)), ({"approximate": True}, (b.nodes, gt))):
        c = atlas_rt.Context(device=0, **kwargs)
        try:
            mid = c.upload_mesh(*mesh)
            prim = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
            ref = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
            got = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
            c.raygen(cam, prim)
            c.trace_closest(mid, prim, 0.0, float("inf"), out=ref, n_rays=n)
            c.trace_camera_closest(mid, cam, got)
            c.synchronize()
            r = ref.cpu().numpy()
            assert np.array_equal(got.cpu().numpy().view(np.uint32), r.view(np.uint32))
            assert (r[:, 0].view(np.int32) >= 0).any()
        finally:
            c.close()
