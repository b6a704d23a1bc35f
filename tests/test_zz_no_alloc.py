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
