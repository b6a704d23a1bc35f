"""The engine's NEE light list built on the host (ae_lights_*).

* CPU: triangle lights of a mesh (RayTracingWorld.cpp:322-376), their
  placement per instance (:378-407), directional lights, the weight
  normalisation (RayTracingHelper.cpp:481-499) and the per-dispatch selection
  (:72-105, Piecewise.cpp:11-78) equal the oracle's numpy restatement bit for
  bit; argument errors and the capacity overflow return their status.
* GPU: with the area light split into 200 emissive triangles, the path
  tracer with every light in the buffer matches the CPU restatement, and
  rendering each sample with its own 16-light selection (weights scaled as
  the engine scales them) converges to the same image.
"""
import ctypes as C

import numpy as np
import pytest

import atlas_rt
import pyoracle
from atlas_rt import BVH, lights, ptscene, scenes
from atlas_rt._native import lib

F32 = np.float32


def lit_mesh(seed=4, n=300):
    """Random triangles with per-vertex normals and 5 materials, 2 emissive."""
    rng = np.random.default_rng(seed)
    tris = scenes.random_triangles(n, seed=seed)
    nrm = rng.normal(size=(n, 3, 3)).astype(F32)
    mat = rng.integers(0, 5, n).astype(np.int32)
    b = BVH(tris)
    sh = b.pack_shading(nrm, mat)
    emissive = np.zeros((5, 3), F32)
    emissive[1] = (0.9, 0.5, 0.2)
    emissive[3] = (0.05, 0.0, 0.6)
    intensity = np.array([1.0, 4.0, 1.0, 12.5, 1.0], F32)
    return sh, emissive, intensity


def test_triangle_lights_match_restatement():
    sh, em, it = lit_mesh()
    got = lights.from_mesh(sh, em, it)
    want = pyoracle.triangle_lights(sh, em, it)
    mat = sh[:, 15].view(np.int32)
    assert len(got) == np.isin(mat, [1, 3]).sum() > 50
    assert got.tobytes() == want.tobytes()
    # type 1 | triangle index in data.x; the colour converted twice
    data = got[:, 12].view(np.uint32)
    assert np.all(data >> 28 == 1) and np.all(np.isin(mat[data & 0x0FFFFFFF], [1, 3]))


def test_triangle_light_counting_and_overflow():
    sh, em, it = lit_mesh()
    L = lib()
    n = C.c_uint32()
    p = lambda a: C.c_void_p(a.ctypes.data)   # noqa: E731
    assert L.ae_lights_from_mesh(p(sh), len(sh), p(em), p(it), len(em), None, 0, C.byref(n)) == 0
    total = n.value
    out = np.zeros((10, 16), F32)
    assert L.ae_lights_from_mesh(p(sh), len(sh), p(em), p(it), len(em), p(out), 10, C.byref(n)) == 3
    assert n.value == total and out.tobytes() == lights.from_mesh(sh, em, it)[:10].tobytes()
    # a material index past the table
    assert L.ae_lights_from_mesh(p(sh), len(sh), p(em), p(it), 2, None, 0, C.byref(n)) == 1


def test_instance_placement_matches_restatement():
    sh, em, it = lit_mesh()
    base = lights.from_mesh(sh, em, it)
    rng = np.random.default_rng(9)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    M = np.eye(4, dtype=F32)
    M[:3, :3] = (q * rng.uniform(0.5, 2.0, 3)).astype(F32)
    M[:3, 3] = rng.uniform(-10, 10, 3)
    got = lights.instance(base, M, 7)
    want = pyoracle.lights_instance(base, M, 7)
    assert got.tobytes() == want.tobytes()
    assert np.all(got[:, 15].view(np.int32) == 7)
    np.testing.assert_allclose(got[:, 0:3], base[:, 0:3] @ M[:3, :3].T + M[:3, 3], rtol=1e-5, atol=1e-4)


def test_directional_and_normalisation():
    d = lights.directional((1.0, 0.8, 0.6), 3.0, (0.0, -1.0, 0.0), index=0)
    lin = pyoracle._srgb_to_linear([1.0, 0.8, 0.6]) * F32(3.0)
    assert np.array_equal(d[8:11], lin) and d[12].view(np.uint32) == 0
    assert d[13] == pyoracle._dot3(lin, np.full(3, 0.3333, F32))
    sh, em, it = lit_mesh()
    L = np.concatenate([d[None, :], lights.from_mesh(sh, em, it)])
    L[5, 13] = 1e-9                      # below the floor of 0.005 x the largest
    got = lights.normalize(L)
    assert got.tobytes() == pyoracle.lights_normalize(L).tobytes()
    assert abs(float(got[:, 13].sum()) - 1.0) < 1e-5
    assert got[5, 13] == pytest.approx(0.005 * got[:, 13].max(), rel=1e-6)


def test_selection_matches_restatement():
    sh, em, it = lit_mesh()
    L = lights.normalize(lights.from_mesh(sh, em, it))
    # everything fits: all lights, weight 1
    fit = lights.select(L, capacity=len(L))
    assert np.array_equal(fit[:, :13], L[:, :13]) and np.all(fit[:, 13] == 1.0)
    # more lights than slots: draws from the weights, each weight times the capacity
    u = np.random.default_rng(2).random(32, dtype=F32)
    u[0], u[1] = 0.0, np.nextafter(F32(1.0), F32(0.0))
    got = lights.select(L, capacity=32, uniforms=u)
    want = pyoracle.lights_select(L, 32, u)
    assert got.shape == (32, 16) and got.tobytes() == want.tobytes()
    # the draws follow the weights (3,000 selections of 64 slots)
    idx = np.concatenate([lights.select(L, capacity=64, seed=s)[:, 12].view(np.uint32) for s in range(3000)])
    ids = L[:, 12].view(np.uint32)
    counts = np.array([np.sum(idx == i) for i in ids])
    assert counts.sum() == 64 * 3000
    np.testing.assert_allclose(counts / counts.sum(), L[:, 13], atol=2.5e-3)


# ---------------------------------------------------------------------------
# GPU: the path tracer on a light list of 200 triangles
# ---------------------------------------------------------------------------

def split_light_scene(splits=10):
    """The path-traced terrain scene with its 4 x 4 area light cut into
    splits x splits quads (2 * splits^2 emissive triangles, same power)."""
    sc = ptscene.build()
    tris, obj, nrm = sc["tris"][:-2], sc["obj"][:-2], sc["normals"][:-2]
    q = sc["tris"][-2:]
    lo = q.reshape(-1, 3).min(0)
    hi = q.reshape(-1, 3).max(0)
    xs = np.linspace(lo[0], hi[0], splits + 1, dtype=F32)
    zs = np.linspace(lo[2], hi[2], splits + 1, dtype=F32)
    y = lo[1]
    cells = []
    for i in range(splits):
        for j in range(splits):
            a, b = [xs[i], y, zs[j]], [xs[i + 1], y, zs[j]]
            c, d = [xs[i + 1], y, zs[j + 1]], [xs[i], y, zs[j + 1]]
            cells += [[a, b, c], [a, c, d]]
    cells = np.array(cells, F32)
    tris = np.concatenate([tris, cells]).astype(F32)
    obj = np.concatenate([obj, np.full(len(cells), sc["light_obj"], np.int32)])
    cn = np.tile(np.array([0, -1, 0], F32), (len(cells), 3, 1))
    sc.update(tris=tris, obj=obj, normals=np.concatenate([nrm, cn]).astype(F32), bvh=BVH(tris))
    return sc


@pytest.fixture(scope="module")
def split_setup():
    ctx = atlas_rt.Context(device=0)
    sc = split_light_scene()
    mid, shading, _, gt = ptscene.upload(ctx, sc)
    n_mat = len(sc["materials"])
    em = np.zeros((n_mat, 3), F32)
    em[sc["light_obj"]] = 1.0                    # sRGB white: colour pow(pow(1, 2.2), 2.2) * 20 = 20
    it = np.ones(n_mat, F32)
    it[sc["light_obj"]] = 20.0
    L = lights.normalize(lights.instance(lights.from_mesh(shading, em, it), np.eye(4), 0))
    assert len(L) == 200
    bvh = sc["bvh"]
    inst = np.array([atlas_rt.make_instance(np.eye(4), mid, atlas_rt.MASK_ALL | atlas_rt.MASK_SHADOW)])
    lo, hi = atlas_rt.mesh_bounds(bvh)
    top = BVH(boxes_only=np.concatenate([lo, hi])[None, :])
    model = np.tile(np.eye(3, 4, dtype=F32).reshape(-1), (1, 1))
    full = lights.select(L, capacity=len(L))
    osc = (top.nodes_f32, inst[top.order].copy(), model, [(bvh.nodes_f32, gt, shading)], sc["materials"], full)
    yield ctx, L, full, osc
    ctx.close()


def _render(ctx, w, h, spp, offset, seed=1):
    import torch
    cam = atlas_rt.make_camera(scenes.pinhole_camera(w, h))
    acc = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
    ctx.pathtrace(cam, acc, spp=spp, sample_offset=offset, seed=seed)
    ctx.synchronize()
    return acc.cpu().numpy()[:, :3].reshape(h, w, 3).astype(np.float64)


@pytest.mark.gpu
def test_many_lights_match_restatement(split_setup):
    ctx, L, full, osc = split_setup
    w, h, spp = 48, 27, 512
    ctx.set_lights(full)
    g = _render(ctx, w, h, spp, 0) / spp
    camd = scenes.pinhole_camera(w, h)
    camv = np.concatenate([camd["location"], camd["origin"], camd["right"], camd["bottom"]]).astype(F32)
    tl, inst, model, meshes, mats, lts = osc
    c = pyoracle.pathtrace(tl, inst, model, meshes, mats, lts, camv, w, h, spp) / spp
    assert abs(g.mean() - c.mean()) / c.mean() < 0.02, (g.mean(), c.mean())
    gb = g.reshape(h // 9, 9, w // 8, 8, 3).mean(axis=(1, 3))
    cb = c.reshape(h // 9, 9, w // 8, 8, 3).mean(axis=(1, 3))
    assert np.mean(np.abs(gb - cb) > np.maximum(0.08 * cb, 5e-4)) < 0.05


@pytest.mark.gpu
def test_per_dispatch_selection_converges_to_full_list(split_setup):
    """Each sample traced with its own 16 of the 200 lights, drawn by weight
    and weighted by 16 x the normalised weight, as the engine's dispatches
    do: the average over samples equals the all-lights image."""
    ctx, L, full, _ = split_setup
    w, h, spp = 48, 27, 768
    ctx.set_lights(full)
    ref = _render(ctx, w, h, spp, 0) / spp
    acc = np.zeros_like(ref)
    for k in range(spp):
        ctx.set_lights(lights.select(L, capacity=16, seed=1000 + k))
        acc += _render(ctx, w, h, 1, k)
    acc /= spp
    ctx.set_lights(full)
    assert abs(acc.mean() - ref.mean()) / ref.mean() < 0.03, (acc.mean(), ref.mean())
    ab = acc.reshape(h // 9, 9, w // 8, 8, 3).mean(axis=(1, 3))
    rb = ref.reshape(h // 9, 9, w // 8, 8, 3).mean(axis=(1, 3))
    assert np.mean(np.abs(ab - rb) > np.maximum(0.15 * rb, 1e-3)) < 0.1
