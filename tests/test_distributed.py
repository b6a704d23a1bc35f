"""The multi-rank host logic on CPU with gloo (world size 2): sharding of ray
ranges and batches without a data-path collective, and the max-over-ranks
timing the bench divides by."""
import os
import socket

import numpy as np
import pytest

from atlas_rt.distributed import batch_shard, max_over_ranks, ray_shard


def test_ray_shard_tiles_the_range():
    for n in (0, 1, 7, 2073600, 2 ** 30):
        for world in (1, 2, 3, 8):
            ranges = [ray_shard(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        ray_shard(10, 2, 2)


def test_batch_shard_balances_rays():
    rng = np.random.default_rng(3)
    counts = np.exp(rng.uniform(np.log(4096), np.log(1 << 20), 64)).astype(np.int64)
    for world in (1, 2, 4, 8):
        parts = batch_shard(counts, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [int(counts[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= counts.max()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        begin, end = ray_shard(n, rank, world)
        # each rank "traces" its own range: no data crosses ranks
        local_sum = float(np.arange(begin, end, dtype=np.float64).sum())
        dist.barrier()
        times = max_over_ranks([1.0 + rank, 5.0 - rank])
        q.put((rank, begin, end, local_sum, times))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n = 1000003
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, b0, e0, s0, t0), (r1, b1, e1, s1, t1) = res
    assert (b0, e1) == (0, n) and e0 == b1
    assert s0 + s1 == float(np.arange(n, dtype=np.float64).sum())
    assert t0 == t1 == [2.0, 5.0]


def _trace_worker(rank, world, port, q):
    """Each rank traces its ray shard with the oracle's shader-order closest
    query; the shards are gathered on every rank (the test's check only: the
    product path has no collective)."""
    import sys
    from pathlib import Path
    import torch.distributed as dist
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import pyoracle
    from atlas_rt import BVH, scenes
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tris = scenes.random_triangles(4000, seed=31)
        bvh = BVH(tris)
        gt = bvh.pack_triangles()
        o, d = scenes.sphere_rays(20011, seed=32)
        r8 = scenes.rays8(o, d, 1e-4, 10.0)
        begin, end = ray_shard(len(r8), rank, world)
        ptr, tuv = pyoracle.closest_glsl(bvh.nodes_f32, gt, r8[begin:end], threads=2)
        parts = [None] * world
        dist.all_gather_object(parts, (begin, end, ptr, tuv))
        q.put((rank, parts))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shards_equal_unsharded_trace():
    """World size 2 over gloo: the gathered per-rank closest hits of the
    sharded rays equal the unsharded trace bit for bit."""
    import sys
    from pathlib import Path
    import torch.multiprocessing as mp
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import pyoracle
    from atlas_rt import BVH, scenes
    pyoracle.build_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_trace_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tris = scenes.random_triangles(4000, seed=31)
    bvh = BVH(tris)
    o, d = scenes.sphere_rays(20011, seed=32)
    ptr, tuv = pyoracle.closest_glsl(bvh.nodes_f32, bvh.pack_triangles(), scenes.rays8(o, d, 1e-4, 10.0))
    for _, parts in res:
        parts = sorted(parts, key=lambda x: x[0])
        assert parts[0][0] == 0 and parts[-1][1] == len(ptr) and parts[0][1] == parts[1][0]
        assert np.array_equal(np.concatenate([p[2] for p in parts]), ptr)
        assert np.array_equal(np.concatenate([p[3] for p in parts]).view(np.uint32), tuv.view(np.uint32))
    assert (ptr >= 0).sum() > 1000
