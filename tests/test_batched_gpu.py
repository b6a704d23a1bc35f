"""Batched multi-mesh traces: many meshes, uneven ray batches, mixed
closest-hit and any-hit, one persistent launch (and its CUDA-graph plan).
Every batch must equal the per-mesh launch bit for bit, and the per-mesh
launch equals the oracle (tests/test_trace_gpu.py)."""
import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, scenes

pytestmark = pytest.mark.gpu


def make_workload(ctx, sizes, ray_counts, seed):
    import torch
    meshes, batches, expect = [], [], []
    for i, (nt, nr) in enumerate(zip(sizes, ray_counts)):
        tris = scenes.random_triangles(nt, seed=seed + i) if nt else np.zeros((0, 3, 3), np.float32)
        b = BVH(tris)
        gt = b.pack_triangles()
        mid = ctx.upload_mesh(b.nodes, gt)
        meshes.append((b, gt, mid))
        o, d = scenes.sphere_rays(max(nr, 1), seed=seed + 1000 + i)
        packed = scenes.pack_rays(o, d)[:nr]
        any_q = i % 2 == 1
        tmin, tmax = (1e-4, 10.0) if i % 3 else (1.2, 2.6)
        rays_d = torch.from_numpy(packed.copy()).cuda() if nr else torch.zeros((1, 12), device="cuda")
        out_d = (torch.zeros(max(nr, 1), dtype=torch.uint8, device="cuda") if any_q
                 else torch.zeros((max(nr, 1), 8), dtype=torch.float32, device="cuda"))
        batches.append({"mesh": mid, "any": any_q, "rays": rays_d, "out": out_d, "n_rays": nr,
                        "tmin": tmin, "tmax": tmax})
        if nr:
            ref = (ctx.trace_any(mid, packed, tmin, tmax) if any_q else ctx.trace_closest(mid, packed, tmin, tmax))
        else:
            ref = None
        expect.append(ref)
    return meshes, batches, expect


def check(batches, expect):
    for b, ref in zip(batches, expect):
        if ref is None:
            continue
        got = b["out"].cpu().numpy()
        if b["any"]:
            assert np.array_equal(got[: b["n_rays"]], ref)
        else:
            got = got[: b["n_rays"]].view(atlas_rt.HIT_DTYPE).reshape(-1)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_batched_matches_per_mesh_launches():
    import torch
    ctx = atlas_rt.Context(device=0)
    try:
        rng = np.random.default_rng(5)
        sizes = [int(x) for x in np.exp(rng.uniform(np.log(1000), np.log(60000), 10))] + [0, 1, 3]
        rays = [int(x) for x in np.exp(rng.uniform(np.log(100), np.log(50000), 13))]
        rays[4] = 0                      # an empty batch in the middle
        meshes, batches, expect = make_workload(ctx, sizes, rays, seed=70)
        ctx.trace_batched(batches)
        ctx.synchronize()
        check(batches, expect)
        # one batch against the oracle directly
        b, gt, mid = meshes[0]
        packed = batches[0]["rays"].cpu().numpy()
        r8 = np.empty((len(packed), 8), np.float32)
        r8[:, 0:3], r8[:, 3:6] = packed[:, 0:3], packed[:, 4:7]
        r8[:, 6], r8[:, 7] = batches[0]["tmin"], batches[0]["tmax"]
        ptr, _ = pyoracle.closest_glsl(b.nodes_f32, gt, r8)
        got = batches[0]["out"].cpu().numpy().view(atlas_rt.HIT_DTYPE).reshape(-1)
        assert np.array_equal(got["triPtr"], ptr)
        torch.cuda.synchronize()
    finally:
        ctx.close()


@pytest.mark.parametrize("shape", [(128, 32), (64, 32), (256, 16), (128, 16)])
def test_batch_plan_graph_replays(shape):
    """The captured plan replays with the same buffers; new ray contents give
    new results; every kernel shape the autotuner can pick agrees."""
    import torch
    ctx = atlas_rt.Context(device=0, threads_per_block=shape[0], stack_entries_smem=shape[1], refill_steps=16)
    try:
        meshes, batches, expect = make_workload(ctx, [5000, 20000, 300, 9000], [30000, 7000, 12000, 4096], seed=90)
        plan = ctx.batch_plan(batches)
        for _ in range(2):
            for b in batches:
                b["out"].zero_()
            plan.launch()
            ctx.synchronize()
            check(batches, expect)
        # change the rays of one batch in place and replay
        b0 = batches[0]
        o, d = scenes.sphere_rays(b0["n_rays"], seed=12345)
        new = scenes.pack_rays(o, d)
        b0["rays"].copy_(torch.from_numpy(new))
        expect[0] = ctx.trace_closest(b0["mesh"], new, b0["tmin"], b0["tmax"])
        plan.launch()
        ctx.synchronize()
        check(batches, expect)
        plan.close()
    finally:
        ctx.close()


def test_shapes_agree_on_mesh_traces():
    tris = scenes.random_triangles(30000, seed=111)
    b = BVH(tris)
    gt = b.pack_triangles()
    o, d = scenes.sphere_rays(60000, seed=112)
    packed = scenes.pack_rays(o, d)
    results = []
    for threads, smem, refill in [(128, 32, 0), (64, 32, 8), (256, 16, 128), (128, 16, 32)]:
        c = atlas_rt.Context(device=0, threads_per_block=threads, stack_entries_smem=smem, refill_steps=refill)
        try:
            mid = c.upload_mesh(b.nodes, gt)
            results.append((c.trace_closest(mid, packed, 1e-4, 10.0), c.trace_any(mid, packed, 1e-4, 10.0)))
        finally:
            c.close()
    for h, a in results[1:]:
        assert np.array_equal(h.view(np.uint32), results[0][0].view(np.uint32))
        assert np.array_equal(a, results[0][1])
    with pytest.raises(atlas_rt.AeRtError):
        atlas_rt.Context(device=0, threads_per_block=96)
