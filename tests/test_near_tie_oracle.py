"""Completeness of the near-tie flag, on the CPU.

The GPU trace flags AE_HIT_NEAR_TIE on a superset of the rays whose two
nearest double-precision hits lie within 1e-6 relative t (a second accepted
triangle within 4e-6, a rejected box entered within that window of the
bound, a triangle rejected within the rounding error of its barycentric
tests, or a hit right child the shader's descent drops at the bound).  The
oracle restates those decisions with the same correctly rounded operations.
Here its flags are checked against the FP64 brute force over every
triangle on 100,000 rays aimed at terrain grid edges and vertices, at box
edges and at the lines where box walls meet the terrain: no ray with a
brute-force gap <= 1e-6 may go unflagged."""
import numpy as np

import near_tie_util as U
import pyoracle
from atlas_rt import scenes


def test_no_false_negatives_on_edge_and_contact_rays():
    tris, obj = U.near_tie_scene()
    r8, lab = U.near_tie_rays(tris, obj)
    assert len(r8) >= 100000
    nodes, order, eon = pyoracle.build_bvh(tris)
    gt = pyoracle.pack_bvh_triangles(tris, order, eon)
    ptr, t1, t2, gap = U.brute_gaps(gt, r8)
    p, tuv, flags, second = pyoracle.closest_glsl_ties(nodes, gt, r8)
    need = gap <= 1e-6
    flagged = (flags & 2) != 0
    assert need.sum() > 20000                      # the rays do produce ties
    for k in range(4):
        m = lab == k
        assert not np.any(need & ~flagged & m), f"class {k}: unflagged near ties"
    # the flag does not change the query: same winners as the plain oracle
    p0, tuv0 = pyoracle.closest_glsl(nodes, gt, r8)
    assert np.array_equal(p, p0) and np.array_equal(tuv.view(np.uint32), tuv0.view(np.uint32))
    # where both precisions hit but name different triangles, the ray is flagged
    # (FP64 misses at the grid's border edges are not ties: nothing to flag)
    assert np.all(flagged[(p != ptr) & (p >= 0) & (ptr >= 0)])


def test_flag_rate_on_ordinary_rays_is_small():
    tris, obj = U.near_tie_scene()
    nodes, order, eon = pyoracle.build_bvh(tris)
    gt = pyoracle.pack_bvh_triangles(tris, order, eon)
    rng = np.random.default_rng(3)
    n = 100000
    o = np.tile(np.array([[50.0, 60.0, -40.0]], np.float32), (n, 1))
    tg = np.stack([rng.uniform(0, 100, n), rng.uniform(0, 5, n), rng.uniform(0, 100, n)], 1)
    d = tg - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p, _, flags, _ = pyoracle.closest_glsl_ties(nodes, gt, scenes.rays8(o, d.astype(np.float32), 1e-4, 1e4))
    assert (p >= 0).mean() > 0.9
    assert ((flags & 2) != 0).mean() < 0.02
