"""The library's host BVH builder (atlas_rt.BVH / ae_bvh_build_*) against the
reference builder: byte-identical nodes, primitive order and leaf flags on
the golden small cases and, through SHA-256 digests, on the full-size
workloads.  CPU only."""
import hashlib

import numpy as np
import pytest

import pyoracle
from atlas_rt import BVH, scenes

CASES = ["rand1", "rand2", "rand3", "rand64", "rand2000", "identical9", "flat500", "big300"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("parallel", [True, False])
def test_builder_matches_reference_small(golden, name, parallel):
    g, _ = golden
    b = BVH(g[f"{name}/tris"], parallel=parallel)
    assert np.array_equal(b.nodes_f32.view(np.uint32), g[f"{name}/nodes"].view(np.uint32))
    assert np.array_equal(b.order, g[f"{name}/order"])
    assert np.array_equal(b.end_of_node, g[f"{name}/end_of_node"])


@pytest.mark.parametrize("which", ["random65536", "terrain_boxes"])
def test_builder_matches_reference_full_size(golden, which):
    _, dg = golden
    d = dg[which]
    if which == "random65536":
        tris = scenes.random_triangles()
    else:
        tris, _ = scenes.terrain_boxes()
        assert sha(tris) == d["inputs_sha"]
    b = BVH(tris)
    assert len(b.nodes) == d["nodes"] and len(b.order) == d["primitives"]
    assert sha(b.nodes_f32) == d["nodes_sha"]
    assert sha(b.order) == d["order_sha"]
    assert sha(b.end_of_node) == d["eon_sha"]


def test_builder_empty_and_single():
    e = BVH(np.zeros((0, 3, 3), np.float32))
    assert len(e.nodes) == 0 and len(e.order) == 0
    one = BVH(scenes.random_triangles(1, seed=1))
    assert len(one.order) >= 1 and one.end_of_node[-1] == 1


def test_leaf_structure_and_pointers():
    b = BVH(scenes.random_triangles(3000, seed=3))
    n = len(b.nodes)
    for i, nd in enumerate(b.nodes):
        for p in (int(nd["leftPtr"]), int(nd["rightPtr"])):
            if p >= 0:
                assert i < p < n
            else:
                assert 0 <= ~p < len(b.order)
    # every primitive is referenced exactly once (no duplicates for small random tris)
    assert sorted(b.order.tolist()) == list(range(3000))


def test_pack_triangles_layout():
    tris = scenes.random_triangles(100, seed=5)
    b = BVH(tris)
    mat = np.arange(100, dtype=np.int32) * 3
    opa = np.linspace(0.1, 1.0, 100).astype(np.float32)
    g = b.pack_triangles(mat, opa)
    v = tris.reshape(-1, 9)[b.order]
    assert np.array_equal(g[:, 0:3], v[:, 0:3])
    assert np.array_equal(g[:, 4:7], v[:, 3:6])
    assert np.array_equal(g[:, 8:11], v[:, 6:9])
    assert np.array_equal(g[:, 3] > 0, b.end_of_node > 0)
    assert np.array_equal(g[:, 7].view(np.int32), mat[b.order])
    assert np.array_equal(g[:, 11], opa[b.order])


def test_box_bvh_single_instance_node():
    """One instance: a single node with both pointers ~0 and an empty right
    box at the origin (BVH.cpp:80-88)."""
    b = BVH(boxes_only=np.array([[1, 2, 3, 4, 5, 6]], np.float32))
    assert len(b.nodes) == 1
    nd = b.nodes[0]
    assert nd["leftPtr"] == ~0 and nd["rightPtr"] == ~0
    assert np.array_equal(nd["leftMin"], [1, 2, 3]) and np.array_equal(nd["leftMax"], [4, 5, 6])
    assert np.array_equal(nd["rightMin"], [0, 0, 0]) and np.array_equal(nd["rightMax"], [0, 0, 0])


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference tree not present on this host")
@pytest.mark.parametrize("n", [1, 2, 7, 64, 1000])
def test_box_bvh_matches_reference(n):
    rng = np.random.Generator(np.random.PCG64(n))
    lo = rng.random((n, 3)).astype(np.float32) * 50
    hi = lo + rng.random((n, 3)).astype(np.float32) * 5
    boxes = np.concatenate([lo, hi], axis=1)
    nodes, order = pyoracle.ref_build_aabbs(boxes)
    b = BVH(boxes_only=boxes)
    assert np.array_equal(b.nodes_f32.view(np.uint32), nodes.view(np.uint32))
    assert np.array_equal(b.order, order)


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference tree not present on this host")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_builder_matches_reference_fresh_seeds(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    # mixed sizes: small random triangles plus a few large ones (spatial splits)
    small = scenes.random_triangles(4000, seed=seed)
    big = rng.random((40, 3, 3)).astype(np.float32)
    tris = np.concatenate([small, big])
    r = pyoracle.RefBVH(tris)
    b = BVH(tris)
    assert np.array_equal(b.nodes_f32.view(np.uint32), r.nodes_f32.view(np.uint32))
    assert np.array_equal(b.order, r.order)
    assert np.array_equal(b.end_of_node, r.end_of_node)
