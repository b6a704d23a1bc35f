"""ae_rt_trace_closest_noalloc: the closest-hit trace for hosts that cannot
let a library allocate device memory (engines that pre-allocate every GPU
buffer from their own arenas, frame loops that must not hit cudaMalloc's
implicit synchronisation).  It takes caller-owned device buffers and keeps
its work counter in a static device array.

The test calls it twice in a row through the C ABI on the same buffers and
compares each result with the context-based ae_rt_trace_closest: bit-identical
hit records (the tolerance of every trace test here).  The second call shows
that the shared scratch is re-zeroed: a stale work counter would leave the
hit buffer untouched.  This file is collected last so that a run stopping at
its first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import atlas_rt
from atlas_rt import BVH, _native, scenes

pytestmark = pytest.mark.gpu


def test_noalloc_trace_matches_context_trace_twice():
    import torch
    lib = _native.lib()
    tris = scenes.random_triangles(30000, seed=901)
    bvh = BVH(tris)
    gt = bvh.pack_triangles()
    o, d = scenes.sphere_rays(200000, seed=902)
    packed = scenes.pack_rays(o, d)
    tmin, tmax = 1e-4, 10.0

    ctx = atlas_rt.Context(device=0)
    try:
        mid = ctx.upload_mesh(bvh.nodes, gt)
        expected = ctx.trace_closest(mid, packed, tmin, tmax)
    finally:
        ctx.close()

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nodes_d = torch.from_numpy(bvh.nodes_f32.copy()).to(dev)
    tris_d = torch.from_numpy(gt).to(dev)
    rays_d = torch.from_numpy(packed).to(dev)
    hits_d = torch.empty((len(packed), 8), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        hits_d.fill_(float("nan"))       # a call that wrote nothing cannot pass
        st = lib.ae_rt_trace_closest_noalloc(nodes_d.data_ptr(), len(bvh.nodes), tris_d.data_ptr(), len(gt),
                                             rays_d.data_ptr(), len(packed), C.c_float(tmin), C.c_float(tmax),
                                             hits_d.data_ptr(), stream.cuda_stream)
        assert st == 0, f"call {call}: status {st}"
        torch.cuda.synchronize(dev)
        got = hits_d.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
        assert np.array_equal(got["triPtr"], expected["triPtr"]), f"call {call}: triangle mismatch"
        assert np.array_equal(got.view(np.uint32), expected.view(np.uint32)), f"call {call}: hit records differ"
        assert (got["triPtr"] >= 0).sum() > 0


def _chain_bvh(n):
    """A chain-shaped BVH whose traversal needs n - 1 stack entries: triangle
    i lies in the plane z = n - i, node i has the inner node i + 1 (boxes of
    triangles i+1 .. n-1, nearer to a +z ray from z = -1) as its left child
    and the leaf of triangle i (farther) as its right child, so every level
    pushes its leaf and descends."""
    nodes = np.zeros(n - 1, atlas_rt.NODE_DTYPE)
    tris = np.zeros((n, 12), np.float32)
    for i in range(n):
        z = float(n - i)
        tris[i, 0:4] = (-1.0, -1.0, z, 1.0)     # v0, end of leaf
        tris[i, 4:7] = (3.0, -1.0, z)
        tris[i, 8:11] = (-1.0, 3.0, z)
    for i in range(n - 1):
        nodes[i]["leftMin"] = (-1.0, -1.0, 1.0)
        nodes[i]["leftMax"] = (3.0, 3.0, float(n - i - 1))
        nodes[i]["rightMin"] = (-1.0, -1.0, float(n - i))
        nodes[i]["rightMax"] = (3.0, 3.0, float(n - i))
        nodes[i]["leftPtr"] = i + 1 if i + 1 < n - 1 else ~(n - 1)
        nodes[i]["rightPtr"] = ~i
    return nodes, tris


def _call_noalloc(lib, nodes_d, n_nodes, tris_d, n_tris, rays_d, n, tmin, tmax, hits_d):
    import torch
    st = lib.ae_rt_trace_closest_noalloc(nodes_d.data_ptr(), n_nodes, tris_d.data_ptr(), n_tris, rays_d.data_ptr(),
                                         n, C.c_float(tmin), C.c_float(tmax), hits_d.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
    assert st == 0, f"status {st}"
    torch.cuda.synchronize()
    return hits_d.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)


def test_noalloc_deep_chain_matches_context_trace():
    """A traversal 99 stack entries deep: the allocation-free trace holds the
    same 128 entries per ray as the context trace, so both give the nearest
    triangle with no overflow flag, bit for bit."""
    import torch
    lib = _native.lib()
    n = 100
    nodes, tris = _chain_bvh(n)
    rng = np.random.default_rng(77)
    m = 4096
    o = np.stack([rng.uniform(-0.5, 0.5, m), rng.uniform(-0.5, 0.5, m), np.full(m, -1.0)], 1).astype(np.float32)
    d = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (m, 1))
    d[:, 0:2] = rng.uniform(-1e-3, 1e-3, (m, 2))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    packed = scenes.pack_rays(o, d.astype(np.float32))
    ctx = atlas_rt.Context(device=0)
    try:
        mid = ctx.upload_mesh(nodes, tris)
        expected = ctx.trace_closest(mid, packed, 1e-4, 1e4)
    finally:
        ctx.close()
    assert np.all(expected["triPtr"] == n - 1)
    assert not np.any(expected["flags"] & (atlas_rt.HIT_FLAG_OVERFLOW | atlas_rt.HIT_FLAG_ITER_CAP))
    dev = torch.device("cuda", 0)
    nodes_d = torch.from_numpy(nodes.view(np.float32).reshape(-1, 16).copy()).to(dev)
    tris_d = torch.from_numpy(tris).to(dev)
    rays_d = torch.from_numpy(packed).to(dev)
    hits_d = torch.full((m, 8), float("nan"), dtype=torch.float32, device=dev)
    got = _call_noalloc(lib, nodes_d, len(nodes), tris_d, n, rays_d, m, 1e-4, 1e4, hits_d)
    assert np.array_equal(got.view(np.uint32), expected.view(np.uint32))


def test_noalloc_bounds_check_flags_bad_indices():
    """A BVH that never went through the upload validator: its one node
    points at inner node 5 of a 1-node array and at the leaf of triangle 7
    of a 1-triangle array.  The range check runs before any load, so every
    ray ends with the overflow flag and no hit."""
    import torch
    lib = _native.lib()
    nodes = np.zeros(1, atlas_rt.NODE_DTYPE)
    for side in ("left", "right"):
        nodes[0][side + "Min"] = (-10.0, -10.0, -10.0)
        nodes[0][side + "Max"] = (10.0, 10.0, 10.0)
    nodes[0]["leftPtr"] = 5
    nodes[0]["rightPtr"] = ~7
    tris = np.zeros((1, 12), np.float32)
    tris[0, 0:4] = (0.0, 0.0, 0.0, 1.0)
    tris[0, 4:7] = (1.0, 0.0, 0.0)
    tris[0, 8:11] = (0.0, 1.0, 0.0)
    rng = np.random.default_rng(3)
    m = 1000
    o = rng.uniform(-1.0, 1.0, (m, 3)).astype(np.float32)
    d = rng.normal(size=(m, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    dev = torch.device("cuda", 0)
    nodes_d = torch.from_numpy(nodes.view(np.float32).reshape(-1, 16).copy()).to(dev)
    tris_d = torch.from_numpy(tris).to(dev)
    rays_d = torch.from_numpy(scenes.pack_rays(o, d)).to(dev)
    hits_d = torch.full((m, 8), float("nan"), dtype=torch.float32, device=dev)
    got = _call_noalloc(lib, nodes_d, 1, tris_d, 1, rays_d, m, 0.0, 100.0, hits_d)
    assert np.all(got["flags"] & atlas_rt.HIT_FLAG_OVERFLOW)
    assert np.all(got["triPtr"] == -1)


def test_noalloc_rejects_bad_arguments():
    import torch
    lib = _native.lib()
    rays = torch.zeros((4, 12), dtype=torch.float32, device="cuda")
    hits = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    host = np.zeros((4, 12), np.float32)
    # host pointers are refused
    assert lib.ae_rt_trace_closest_noalloc(None, 0, None, 0, host.ctypes.data, 4, 0.0, 1.0,
                                           hits.data_ptr(), None) == 1
    # beyond the maximum ray count
    assert lib.ae_rt_trace_closest_noalloc(None, 0, None, 0, rays.data_ptr(), (1 << 30) + 1, 0.0, 1.0,
                                           hits.data_ptr(), None) == 1
    # an empty mesh traces fine: every ray misses
    assert lib.ae_rt_trace_closest_noalloc(None, 0, None, 0, rays.data_ptr(), 4, 0.0, 1.0,
                                           hits.data_ptr(), None) == 0
    torch.cuda.synchronize()
    got = hits.cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
    assert np.all(got["triPtr"] == -1)
