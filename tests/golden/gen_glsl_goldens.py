"""Writes tests/golden/glsl_shading.npz: golden vectors of the engine's shading
math, produced by the reference's own GLSL (data/shader/brdf/*.hsh,
raytracer/lights.hsh, raytracer/intersections.hsh, common/random.hsh)
compiled on the host by the recipe oracle/glsl/make_ref.py.

Needs the reference tree (this container); the fixture it writes is what the
tests compare the oracle's restatement and the GPU's device functions with.

    python tests/golden/gen_glsl_goldens.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
OUT = REPO / "tests" / "golden" / "glsl_shading.npz"
F32 = np.float32


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _hemi(rng, N, lo=0.02):
    """Unit vectors in the hemisphere around N with cos >= lo."""
    out = np.empty_like(N)
    for i in range(len(N)):
        while True:
            v = rng.normal(size=3)
            v /= np.linalg.norm(v)
            c = v @ N[i]
            if c < 0:
                v, c = -v, -c
            if c >= lo:
                out[i] = v
                break
    return out


def inputs(seed=20261204, n=512):
    """Seeded input rows of every golden set (float32)."""
    rng = np.random.default_rng(seed)
    N = _unit(rng, n)
    V = _hemi(rng, N)
    L = _hemi(rng, N, lo=-0.3)              # a few below the surface: NdotL saturates at 0
    base = rng.uniform(0.0, 1.0, (n, 3))
    rough = np.concatenate([rng.uniform(0.02, 1.0, n - 8), [0.0, 0.001, 0.05, 0.1, 0.3, 0.5, 0.9, 1.0]])
    metal = np.where(rng.random(n) < 0.4, 0.0, np.where(rng.random(n) < 0.5, 1.0, rng.random(n)))
    refl = rng.uniform(0.0, 1.0, n)
    surf = np.concatenate([V, N, L, base, rough[:, None], metal[:, None], refl[:, None]], 1).astype(F32)
    u = rng.uniform(0.0, 1.0, (n, 2)).astype(F32)
    u[:4] = [[0.0, 0.0], [0.999999, 0.5], [0.5, 0.999999], [0.25, 0.0]]
    sample = np.concatenate([surf, u], 1).astype(F32)
    # triangle lights: vertices, normals, area, r0, r1, shaded point
    v = rng.uniform(-5, 5, (n, 9))
    nn = np.concatenate([_unit(rng, n), _unit(rng, n), _unit(rng, n)], 1)
    e0, e1 = v[:, 3:6] - v[:, 0:3], v[:, 6:9] - v[:, 0:3]
    area = 0.5 * np.linalg.norm(np.cross(e0, e1), axis=1)
    light = np.concatenate([v, nn, area[:, None], rng.uniform(0, 1, (n, 2)), rng.uniform(-5, 5, (n, 3))],
                           1).astype(F32)
    # rays against triangles (half aimed inside, some at edges) and boxes
    tri = rng.uniform(-1, 1, (n, 9))
    w = rng.dirichlet([1, 1, 1], n)
    w[: n // 8] = np.stack([rng.uniform(0, 1, n // 8), np.zeros(n // 8), np.zeros(n // 8)], 1)
    w[: n // 8, 1] = 1 - w[: n // 8, 0]
    target = w[:, 0:1] * tri[:, 0:3] + w[:, 1:2] * tri[:, 3:6] + w[:, 2:3] * tri[:, 6:9]
    target[n // 2:] += rng.normal(0, 0.3, (n - n // 2, 3))
    o = rng.uniform(-4, 4, (n, 3))
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    itri = np.concatenate([o, d, tri], 1).astype(F32)
    lo = rng.uniform(-1, 0, (n, 3))
    hi = lo + rng.uniform(0, 1.5, (n, 3))
    hi[: n // 16, 1] = lo[: n // 16, 1]          # flat boxes
    bt = lo + rng.uniform(0, 1, (n, 3)) * (hi - lo)
    bt[n // 2:] += rng.normal(0, 0.5, (n - n // 2, 3))
    ob = rng.uniform(-4, 4, (n, 3))
    db = bt - ob
    db /= np.linalg.norm(db, axis=1, keepdims=True)
    tm = np.stack([np.zeros(n), np.where(rng.random(n) < 0.3, rng.uniform(1, 6, n), 1e4)], 1)
    ibox = np.concatenate([ob, db, lo, hi, tm], 1).astype(F32)
    xs = np.concatenate([np.arange(32, dtype=F32), rng.uniform(0, 4096, 32).astype(F32)])
    return {"eval_in": surf, "sample_in": sample, "light_in": light, "tri_in": itri, "box_in": ibox,
            "random_x": xs}


def evaluate(lib: C.CDLL, ins: dict) -> dict:
    P = C.c_void_p

    def run(fn, x, width, *extra):
        x = np.ascontiguousarray(x, F32)
        out = np.zeros((len(x), width), F32)
        fn(x.ctypes.data_as(P), C.c_int(len(x)), *extra, out.ctypes.data_as(P))
        return out
    out = {"eval_out": run(lib.aeglsl_eval, ins["eval_in"], 16),
           "sample_diffuse_out": run(lib.aeglsl_sample, ins["sample_in"], 8, C.c_int(0)),
           "sample_specular_out": run(lib.aeglsl_sample, ins["sample_in"], 8, C.c_int(1)),
           "light_out": run(lib.aeglsl_triangle_light, ins["light_in"], 7),
           "tri_out": run(lib.aeglsl_intersect_triangle, ins["tri_in"], 4),
           "box_out": run(lib.aeglsl_intersect_aabb, ins["box_in"], 2)}
    xs = np.ascontiguousarray(ins["random_x"], F32)
    r = np.zeros((len(xs), 8), F32)
    lib.aeglsl_random(xs.ctypes.data_as(P), C.c_int(len(xs)), C.c_float(1.0), C.c_int(8), r.ctypes.data_as(P))
    out["random_out"] = r
    return out


def reference_lib():
    """Builds (if needed) and loads the reference's GLSL compiled on the host;
    None where the reference tree is absent."""
    sys.path.insert(0, str(REPO / "oracle"))
    sys.path.insert(0, str(REPO / "oracle" / "glsl"))
    import pyoracle
    import make_ref
    if not (pyoracle.REFERENCE_ROOT / "data" / "shader" / "brdf" / "brdf.hsh").exists():
        return None
    return C.CDLL(str(make_ref.build(pyoracle.REFERENCE_ROOT)))


def main():
    lib = reference_lib()
    if lib is None:
        raise SystemExit("the reference tree is needed to generate the GLSL goldens")
    ins = inputs()
    np.savez_compressed(OUT, **ins, **evaluate(lib, ins))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
