"""GPU traversal parity through the C ABI.

* Against the oracle's restatement of the shader traversal (HitClosest /
  HitAny on one BLAS): bit-identical triangle index, t, u and v for every ray.
* Against the reference's own host query (golden fixtures and full-size
  digests made by the compiled reference): identical original triangle index
  for every ray except near ties (checked in FP64), t/u/v within 1e-5
  relative.
* Edge cases: empty mesh, NaN and axis-aligned directions, tmin/tmax
  windows, host vs device buffers, and the bounded failure modes (BVH
  validator, stack overflow, step cap) which return status codes.
"""
import hashlib

import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, HIT_FLAG_HIT, HIT_FLAG_NEAR_TIE, scenes

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5   # t, u, v against the reference host query


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def upload(ctx, tris):
    b = BVH(tris)
    gt = b.pack_triangles()
    mid = ctx.upload_mesh(b.nodes, gt)
    return b, gt, mid


def packed(rays8):
    return scenes.pack_rays(rays8[:, 0:3], rays8[:, 3:6])


def assert_bitwise_glsl(b, gt, rays8, hits, occ=None):
    ptr, tuv = pyoracle.closest_glsl(b.nodes_f32, gt, rays8)
    assert np.array_equal(hits["triPtr"], ptr), f"{np.sum(hits['triPtr'] != ptr)} triangle mismatches"
    assert np.array_equal(hits["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    hit = ptr >= 0
    assert np.array_equal(hits["u"][hit].view(np.uint32), tuv[hit, 1].view(np.uint32))
    assert np.array_equal(hits["v"][hit].view(np.uint32), tuv[hit, 2].view(np.uint32))
    assert np.array_equal((hits["flags"] & HIT_FLAG_HIT) != 0, hit)
    if occ is not None:
        o = pyoracle.any_glsl(b.nodes_f32, gt, rays8)
        assert np.array_equal(occ, o)


def test_random65536_bitwise_vs_shader_oracle_and_reference_digest(ctx, golden):
    _, dg = golden
    d = dg["random65536"]
    tris = scenes.random_triangles()
    o, dirs = scenes.sphere_rays()
    rays8 = scenes.rays8(o, dirs, dg["tmin"], dg["tmax"])
    b, gt, mid = upload(ctx, tris)
    pr = packed(rays8)
    hits = ctx.trace_closest(mid, pr, dg["tmin"], dg["tmax"])
    occ = ctx.trace_any(mid, pr, dg["tmin"], dg["tmax"])
    assert_bitwise_glsl(b, gt, rays8, hits, occ)
    # against the reference host query (digests made by the compiled reference)
    idx = np.where(hits["triPtr"] >= 0, b.order[np.maximum(hits["triPtr"], 0)].astype(np.int64), -1)
    idx = idx.astype(np.int32)
    tuv = np.stack([hits["t"], np.where(idx >= 0, hits["u"], 0), np.where(idx >= 0, hits["v"], 0)], 1)
    tuv = tuv.astype(np.float32)
    assert int((idx >= 0).sum()) == d["hits"]
    assert sha(idx) == d["closest_idx_sha"], "nearest-triangle index differs from the reference"
    assert sha(tuv) == d["closest_tuv_sha"]
    assert sha(occ) == d["any_sha"]
    assert int(occ.sum()) == d["occluded"]


CASES = ["rand1", "rand2", "rand3", "rand64", "rand2000", "identical9", "flat500", "big300"]


@pytest.mark.parametrize("name", CASES)
def test_golden_small_cases_vs_reference(ctx, golden, name):
    g, _ = golden
    tris = g[f"{name}/tris"]
    rays8 = g[f"{name}/rays"]
    tmin, tmax = float(rays8[0, 6]), float(rays8[0, 7])
    b, gt, mid = upload(ctx, tris)
    assert np.array_equal(b.nodes_f32.view(np.uint32), g[f"{name}/nodes"].view(np.uint32))
    hits = ctx.trace_closest(mid, packed(rays8), tmin, tmax)
    occ = ctx.trace_any(mid, packed(rays8), tmin, tmax)
    assert_bitwise_glsl(b, gt, rays8, hits, occ)
    ref_idx = g[f"{name}/closest_idx"].astype(np.int64)
    idx = np.where(hits["triPtr"] >= 0, b.order[np.maximum(hits["triPtr"], 0)].astype(np.int64), -1)
    bad = np.nonzero(idx != ref_idx)[0]
    if len(bad):
        _, t64, t64b = pyoracle.closest_f64_brute(gt, rays8[bad])
        assert np.all((t64b - t64) / np.maximum(t64, 1e-30) <= 1e-6), "mismatch that is not a near tie"
    same = (ref_idx >= 0) & (idx == ref_idx)
    ref_tuv = g[f"{name}/closest_tuv"]
    np.testing.assert_allclose(hits["t"][same], ref_tuv[same, 0], rtol=REL_TOL)
    np.testing.assert_allclose(hits["u"][same], ref_tuv[same, 1], rtol=REL_TOL, atol=1e-6)
    np.testing.assert_allclose(hits["v"][same], ref_tuv[same, 2], rtol=REL_TOL, atol=1e-6)


def test_terrain_boxes_primary_rays_bitwise(ctx):
    tris, _ = scenes.terrain_boxes()
    b, gt, mid = upload(ctx, tris)
    cam = scenes.pinhole_camera(480, 270)
    o, d = scenes.pinhole_rays(cam)
    rays8 = scenes.rays8(o, d, 1e-4, 1e4)
    hits = ctx.trace_closest(mid, packed(rays8), 1e-4, 1e4)
    occ = ctx.trace_any(mid, packed(rays8), 1e-4, 1e4)
    assert_bitwise_glsl(b, gt, rays8, hits, occ)
    assert (hits["triPtr"] >= 0).mean() > 0.5


def test_near_tie_flag_on_shared_edge(ctx):
    """Two triangles sharing an edge: rays through the edge have two equal
    nearest hits and are flagged as near ties."""
    tris = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]],
                     [[1, 0, 0], [1, 1, 0], [0, 1, 0]]], np.float32)
    b, gt, mid = upload(ctx, tris)
    # straight down the z axis through the shared edge (x + y = 1) and
    # through the two interiors; both triangles are hit at t = 1 on the edge
    o = np.array([[0.5, 0.5, -1], [0.25, 0.25, -1], [0.75, 0.75, -1]], np.float32)
    d = np.array([[0, 0, 1]] * 3, np.float32)
    rays8 = scenes.rays8(o, d, 0.0, 10.0)
    hits = ctx.trace_closest(mid, packed(rays8), 0.0, 10.0)
    assert np.all(hits["flags"] & HIT_FLAG_HIT)
    assert hits["flags"][0] & HIT_FLAG_NEAR_TIE
    assert not hits["flags"][1] & HIT_FLAG_NEAR_TIE
    assert_bitwise_glsl(b, gt, rays8, hits)


def test_special_directions_and_windows(ctx):
    tris = scenes.random_triangles(3000, seed=31)
    b, gt, mid = upload(ctx, tris)
    o, d = scenes.sphere_rays(4096, seed=32)
    d = d.copy()
    d[0:512, 0] = 0.0                      # axis-parallel in x
    d[512:1024, 0:2] = 0.0                 # along z only
    d[512:1024, 2] = np.where(o[512:1024, 2] > 0.5, -1.0, 1.0)
    d[1024:1100, 1] = np.nan               # NaN direction: miss
    d[1100:1200] = -d[1100:1200]           # pointing away
    for tmin, tmax in [(1e-4, 10.0), (1.5, 2.5), (0.0, 1.7), (3.0, 3.0)]:
        rays8 = scenes.rays8(o, d, tmin, tmax)
        hits = ctx.trace_closest(mid, packed(rays8), tmin, tmax)
        occ = ctx.trace_any(mid, packed(rays8), tmin, tmax)
        assert_bitwise_glsl(b, gt, rays8, hits, occ)
        assert np.all(hits["triPtr"][1024:1100] == -1)
        assert np.all(occ[1024:1100] == 0)


def test_empty_and_single_meshes(ctx):
    o, d = scenes.sphere_rays(1000, seed=41)
    rays8 = scenes.rays8(o, d, 1e-4, 10.0)
    # a mesh with no nodes: everything misses (BVH.cpp:107)
    mid = ctx.upload_mesh(np.zeros(0, atlas_rt.NODE_DTYPE), np.zeros((0, 12), np.float32))
    hits = ctx.trace_closest(mid, packed(rays8), 1e-4, 10.0)
    assert np.all(hits["triPtr"] == -1) and np.all(hits["t"] == np.float32(10.0))
    assert not ctx.trace_any(mid, packed(rays8), 1e-4, 10.0).any()
    for n in (1, 2, 3):
        tris = scenes.random_triangles(n, seed=40 + n)
        b, gt, mid = upload(ctx, tris)
        hits = ctx.trace_closest(mid, packed(rays8), 1e-4, 10.0)
        assert_bitwise_glsl(b, gt, rays8, hits, ctx.trace_any(mid, packed(rays8), 1e-4, 10.0))
    # zero rays
    out = ctx.trace_closest(mid, np.zeros((0, 12), np.float32), 0.0, 1.0)
    assert len(out) == 0


def test_device_buffers_match_host_buffers(ctx):
    import torch
    tris = scenes.random_triangles(20000, seed=51)
    b, gt, mid = upload(ctx, tris)
    o, d = scenes.sphere_rays(100000, seed=52)
    rays8 = scenes.rays8(o, d, 1e-4, 10.0)
    pr = packed(rays8)
    host_hits = ctx.trace_closest(mid, pr, 1e-4, 10.0)
    host_occ = ctx.trace_any(mid, pr, 1e-4, 10.0)
    dev_rays = torch.from_numpy(pr).cuda()
    dev_hits = torch.zeros((len(pr), 8), dtype=torch.float32, device="cuda")
    dev_occ = torch.zeros(len(pr), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    ctx.trace_closest(mid, dev_rays, 1e-4, 10.0, out=dev_hits, stream=s)
    ctx.trace_any(mid, dev_rays, 1e-4, 10.0, out=dev_occ, stream=s)
    ctx.synchronize(s)
    got = dev_hits.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
    assert np.array_equal(got.view(np.uint32), host_hits.view(np.uint32))
    assert np.array_equal(dev_occ.cpu().numpy(), host_occ)


def test_validator_rejects_bad_bvh(ctx):
    tris = scenes.random_triangles(100, seed=61)
    b = BVH(tris)
    gt = b.pack_triangles()
    bad = b.nodes.copy()
    bad[0]["leftPtr"] = len(bad) + 5           # child out of range
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.upload_mesh(bad, gt)
    assert e.value.status == 2
    bad = b.nodes.copy()
    bad[3]["rightPtr"] = 1                      # points back up: not pre-order (cycle)
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.upload_mesh(bad, gt)
    assert e.value.status == 2
    gt2 = gt.copy()
    gt2[:, 3] = -1.0                            # no leaf terminates
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.upload_mesh(b.nodes, gt2)
    assert e.value.status == 2


def comb_bvh(depth):
    """A valid but degenerate BVH: node i has node i+1 on the left and a leaf
    on the right, every box the same.  A ray through the box sees equal
    entry distances, descends left (hitL <= hitR) and pushes the right leaf,
    so the stack grows by one entry per level."""
    nodes = np.zeros(depth, atlas_rt.NODE_DTYPE)
    box_lo, box_hi = np.zeros(3, np.float32), np.ones(3, np.float32)
    for i in range(depth):
        nodes[i]["leftMin"], nodes[i]["leftMax"] = box_lo, box_hi
        nodes[i]["rightMin"], nodes[i]["rightMax"] = box_lo, box_hi
        nodes[i]["leftPtr"] = i + 1 if i + 1 < depth else ~depth
        nodes[i]["rightPtr"] = ~i
    tris = np.zeros((depth + 1, 12), np.float32)
    tris[:, 0:3] = [5, 5, 5]     # triangles far outside the ray path
    tris[:, 4:7] = [6, 5, 5]
    tris[:, 8:11] = [5, 6, 5]
    tris[:, 3] = 1.0
    return nodes, tris


def chain_bvh(n):
    """A chain-shaped BVH whose traversal needs n - 1 stack entries: triangle
    i lies in the plane z = n - i, node i has the inner node i + 1 (the boxes
    of triangles i+1 .. n-1, nearer to a +z ray from z = -1) on the left and
    the leaf of triangle i (farther) on the right, so every level pushes its
    leaf and descends; the nearest triangle is the last."""
    nodes = np.zeros(n - 1, atlas_rt.NODE_DTYPE)
    tris = np.zeros((n, 12), np.float32)
    for i in range(n):
        z = float(n - i)
        tris[i, 0:4] = (-1.0, -1.0, z, 1.0)
        tris[i, 4:7] = (3.0, -1.0, z)
        tris[i, 8:11] = (-1.0, 3.0, z)
    for i in range(n - 1):
        nodes[i]["leftMin"], nodes[i]["leftMax"] = (-1.0, -1.0, 1.0), (3.0, 3.0, float(n - i - 1))
        nodes[i]["rightMin"], nodes[i]["rightMax"] = (-1.0, -1.0, float(n - i)), (3.0, 3.0, float(n - i))
        nodes[i]["leftPtr"] = i + 1 if i + 1 < n - 1 else ~(n - 1)
        nodes[i]["rightPtr"] = ~i
    return nodes, tris


def test_deep_trees_complete_and_deeper_than_1024_report_overflow(ctx):
    """Meshes whose traversal can need more than the usual kernels' 128 stack
    entries (the upload measures the tree's depth) are traced by the deep
    variants, 1,024 entries per lane in local memory: 200- and 1,000-level
    combs traverse and miss, and a 400-triangle chain (399 entries) returns
    the nearest triangle bit for bit as the oracle's unbounded traversal.
    Beyond 1,024 levels the overflow is still reported (status 6)."""
    rays8 = scenes.rays8(np.array([[0.5, 0.5, -1.0]], np.float32), np.array([[0, 0, 1]], np.float32), 0.0, 10.0)
    for depth in (20, 100, 200, 1000):
        nodes, tris = comb_bvh(depth)
        mid = ctx.upload_mesh(nodes, tris)
        hits = ctx.trace_closest(mid, packed(rays8), 0.0, 10.0)
        assert hits["triPtr"][0] == -1 and (hits["flags"][0] & 0x4) == 0
        assert not ctx.trace_any(mid, packed(rays8), 0.0, 10.0)[0]
    nodes, tris = comb_bvh(1100)
    mid = ctx.upload_mesh(nodes, tris)
    with pytest.raises(atlas_rt.AeRtError) as e:
        ctx.trace_closest(mid, packed(rays8), 0.0, 10.0)
    assert e.value.status == 6
    n = 400
    nodes, tris = chain_bvh(n)
    mid = ctx.upload_mesh(nodes, tris)
    rays8 = scenes.rays8(np.array([[0.5, 0.5, -1.0], [0.2, 0.7, -3.0]], np.float32),
                         np.array([[0, 0, 1], [0.01, -0.02, 1.0]], np.float32), 0.0, 1e4)
    hits = ctx.trace_closest(mid, packed(rays8), 0.0, 1e4)
    ptr, tuv = pyoracle.closest_glsl(nodes.view(np.float32).reshape(-1, 16), tris, rays8)
    assert np.array_equal(hits["triPtr"], ptr) and (ptr == n - 1).all()
    assert np.array_equal(hits["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    assert ctx.trace_any(mid, packed(rays8), 0.0, 1e4).all()
    # the same chain as the one instance of a scene (top level + bottom level)
    sc = atlas_rt.Context(device=0)
    try:
        m2 = sc.upload_mesh(nodes, tris)
        inst = np.array([atlas_rt.make_instance(np.eye(4), m2, atlas_rt.MASK_ALL)])
        sc.scene_build(inst, np.array([[-1.0, -1.0, 1.0, 3.0, 3.0, float(n)]], np.float32))
        sh = sc.trace_scene_closest(packed(rays8), 0.0, 1e4)
        sc.synchronize()
        assert np.array_equal(sh["triPtr"], ptr)
        assert np.array_equal(sh["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    finally:
        sc.close()


def test_step_cap_is_reported():
    c = atlas_rt.Context(device=0, max_steps=3)
    try:
        tris = scenes.random_triangles(5000, seed=71)
        b = BVH(tris)
        mid = c.upload_mesh(b.nodes, b.pack_triangles())
        o, d = scenes.sphere_rays(256, seed=72)
        rays8 = scenes.rays8(o, d, 1e-4, 10.0)
        with pytest.raises(atlas_rt.AeRtError) as e:
            c.trace_closest(mid, packed(rays8), 1e-4, 10.0)
        assert e.value.status == 7
    finally:
        c.close()


def test_fetch_counts_match_oracle():
    c = atlas_rt.Context(device=0, count_fetches=True)
    try:
        tris = scenes.random_triangles(20000, seed=81)
        b = BVH(tris)
        gt = b.pack_triangles()
        mid = c.upload_mesh(b.nodes, gt)
        o, d = scenes.sphere_rays(50000, seed=82)
        rays8 = scenes.rays8(o, d, 1e-4, 10.0)
        c.trace_closest(mid, packed(rays8), 1e-4, 10.0)
        nodes, trisf = c.fetch_counts()
        _, _, nf, tf = pyoracle.closest_glsl(b.nodes_f32, gt, rays8, counters=True)
        assert nodes == int(nf.sum()) and trisf == int(tf.sum())
        c.trace_any(mid, packed(rays8), 1e-4, 10.0)
        nodes, trisf = c.fetch_counts()
        _, nf, tf = pyoracle.any_glsl(b.nodes_f32, gt, rays8, counters=True)
        assert nodes == int(nf.sum()) and trisf == int(tf.sum())
    finally:
        c.close()


def test_divide_free_slab_quotient_is_correctly_rounded(ctx):
    """The traversal kernel's slab quotients come from RN(1/d) and two FMA
    corrections; on the operand window the kernel uses them for, they must
    equal div.rn.f32 bit for bit."""
    for n, seed in ((1 << 31, 12345), (1 << 28, 777)):
        bad = ctx.selftest_division(n, seed=seed)
        assert bad == 0, f"{bad} of {n} quotients differ from div.rn"

