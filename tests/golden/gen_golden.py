"""Generates the golden fixtures in this directory from the reference's OWN
BVH builder and host ray queries (src/engine/volume/BVH.cpp, Ray.cpp,
AABB.cpp, jobsystem/*.cpp), compiled unmodified from the reference tree by
oracle/Makefile into oracle/_ref/libaeref.so.

Run here, where the reference tree exists:
    python tests/golden/gen_golden.py
The GPU host has no reference tree; the tests there read only the committed
outputs:

* ``small_cases.npz`` -- for a set of small seeded scenes: the reference's
  flattened nodes, primitive order and leaf flags, and the reference closest
  / any results for seeded rays (host semantics, BVH.cpp:103-217).
* ``digests.json`` -- for the full-size workloads (65,536 random triangles
  with 1,048,576 sphere rays; the 526,688-triangle terrain + boxes scene):
  SHA-256 of the reference's node and order buffers, and of its closest-hit
  results (original triangle index, t, u, v) and any-hit results.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "atlas-engine_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

from atlas_rt import scenes  # noqa: E402
import pyoracle  # noqa: E402

TMIN, TMAX = 1e-4, 10.0


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def small_cases():
    """Seeded small scenes that cover the builder's branches: tiny meshes,
    identical triangles (median-split fallback), a flat mesh, overlapping
    large triangles (root spatial split) and random clouds."""
    cases = {}
    cases["rand1"] = scenes.random_triangles(1, seed=101)
    cases["rand2"] = scenes.random_triangles(2, seed=102)
    cases["rand3"] = scenes.random_triangles(3, seed=103)
    cases["rand64"] = scenes.random_triangles(64, seed=164)
    cases["rand2000"] = scenes.random_triangles(2000, seed=2000)
    cases["identical9"] = np.tile(scenes.random_triangles(1, seed=9), (9, 1, 1))
    flat = scenes.random_triangles(500, seed=500)
    flat[:, :, 1] = 0.25
    cases["flat500"] = flat
    rng = np.random.Generator(np.random.PCG64(77))
    cases["big300"] = rng.random((300, 3, 3)).astype(np.float32)
    return cases


def small_rays(seed: int, n: int = 2048):
    o, d = scenes.sphere_rays(n, seed=seed)
    return scenes.rays8(o, d, TMIN, TMAX)


def main():
    out = {}
    for name, tris in small_cases().items():
        r = pyoracle.RefBVH(tris)
        rays = small_rays(len(tris) + 17)
        idx, tuv, rbool = r.closest(rays)
        occ = r.any(rays)
        out[f"{name}/tris"] = tris
        out[f"{name}/nodes"] = r.nodes_f32
        out[f"{name}/order"] = r.order
        out[f"{name}/end_of_node"] = r.end_of_node
        out[f"{name}/rays"] = rays
        out[f"{name}/closest_idx"] = idx
        out[f"{name}/closest_tuv"] = tuv
        out[f"{name}/closest_bool"] = rbool
        out[f"{name}/any"] = occ
    np.savez_compressed(HERE / "small_cases.npz", **out)

    digests = {"generator": "tests/golden/gen_golden.py", "tmin": TMIN, "tmax": TMAX}
    # 65,536 random triangles, 1,048,576 sphere rays
    tris = scenes.random_triangles()
    o, d = scenes.sphere_rays()
    rays = scenes.rays8(o, d, TMIN, TMAX)
    r = pyoracle.RefBVH(tris)
    idx, tuv, _ = r.closest(rays)
    occ = r.any(rays)
    digests["random65536"] = {
        "inputs_sha": sha(tris) + ":" + sha(rays),
        "nodes": len(r.nodes_f32), "primitives": len(r.order),
        "nodes_sha": sha(r.nodes_f32), "order_sha": sha(r.order), "eon_sha": sha(r.end_of_node),
        "closest_idx_sha": sha(idx), "closest_tuv_sha": sha(tuv), "any_sha": sha(occ),
        "hits": int((idx >= 0).sum()), "occluded": int(occ.sum()),
    }
    # terrain + boxes
    tb, _ = scenes.terrain_boxes()
    r = pyoracle.RefBVH(tb)
    digests["terrain_boxes"] = {
        "inputs_sha": sha(tb), "nodes": len(r.nodes_f32), "primitives": len(r.order),
        "nodes_sha": sha(r.nodes_f32), "order_sha": sha(r.order), "eon_sha": sha(r.end_of_node),
    }
    (HERE / "digests.json").write_text(json.dumps(digests, indent=1) + "\n")
    print("wrote", HERE / "small_cases.npz", HERE / "digests.json")


if __name__ == "__main__":
    main()
