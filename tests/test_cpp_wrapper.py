"""The C++ wrapper include/atlas_rt.hpp (atlas::rt::BVH, the drop-in for
Volume::BVH, BVH.h:114-138), compiled with g++ into tests/cpp/bvh_wrapper_check
and linked against libatlas_rt.so.

* CPU: its public members (nodes, data, refs, aabbs) equal the compiled
  reference's member for member, for triangle and AABB-only builds, including
  the single-box duplicate reference (BVH.cpp:58-100) and the Ref::nodeIdx
  stamp of Flatten (BVH.cpp:411-415); the golden small cases where the
  reference is absent.
* GPU: TraceClosest / TraceAny / GetIntersection / GetIntersectionAny equal the
  oracle's restatement of the shader traversal bit for bit, per-ray (tMin,
  tMax) included, and a query before Upload is refused.
* GPU: atlas::rt::PathTracingRenderer driven from engine assets
  (tests/cpp/renderer_check.cpp) equals the direct C ABI calls.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pyoracle
from atlas_rt import build as atlas_build, scenes

REPO = Path(__file__).resolve().parent.parent
SRC = REPO / "tests" / "cpp" / "bvh_wrapper_check.cpp"


@pytest.fixture(scope="module")
def wrapper_bin(tmp_path_factory):
    lib = atlas_build.build()
    out = tmp_path_factory.mktemp("cpp") / "bvh_wrapper_check"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{REPO / 'include'}", str(SRC),
           f"-L{lib.parent}", "-latlas_rt", f"-Wl,-rpath,{lib.parent}", "-Wl,--allow-shlib-undefined", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.fixture(scope="module")
def renderer_bin(tmp_path_factory):
    """tests/cpp/renderer_check.cpp: assets -> light list -> PathTracingRenderer."""
    lib = atlas_build.build()
    cuda = Path(atlas_build._cuda_lib_dir(atlas_build._nvcc())).parent
    out = tmp_path_factory.mktemp("cpp") / "renderer_check"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{REPO / 'include'}", f"-I{cuda / 'include'}",
           str(REPO / "tests" / "cpp" / "renderer_check.cpp"), f"-L{lib.parent}", "-latlas_rt",
           f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda / 'lib64'}",
           "-Wl,--allow-shlib-undefined", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_renderer_program_builds(renderer_bin):
    """The engine-side caller compiles against both headers and links."""
    assert renderer_bin.exists()


@pytest.mark.gpu
def test_path_tracing_renderer_end_to_end(renderer_bin):
    """.aemesh + .aematerial fixtures through the material table, triangle
    assembly, BVH, scene, light list and atlas::rt::PathTracingRenderer:
    progressive tiles, camera-move restart, non-dividing subdivisions and the
    real-time mode each equal the direct C ABI calls."""
    r = subprocess.run([str(renderer_bin), str(REPO / "tests" / "golden" / "assets")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 4, r.stdout


class _Reader:
    def __init__(self, data: bytes):
        self.b, self.p = data, 0

    def arr(self, dt, n):
        dt = np.dtype(dt)
        a = np.frombuffer(self.b, dt, n, self.p).copy()
        self.p += dt.itemsize * n
        return a

    def u32(self):
        return int(self.arr(np.uint32, 1)[0])


def run(binary, mode, payload: bytes, tmp_path, check=True):
    i, o = tmp_path / f"{mode}.in", tmp_path / f"{mode}.out"
    i.write_bytes(payload)
    r = subprocess.run([str(binary), mode, str(i), str(o)], capture_output=True, text=True, timeout=600)
    if check:
        assert r.returncode == 0, r.stderr
    return _Reader(o.read_bytes()) if r.returncode == 0 else r


def members(binary, tmp_path, verts=None, boxes=None):
    if verts is not None:
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        lo = np.minimum(np.minimum(v[:, 0:3], v[:, 3:6]), v[:, 6:9])
        hi = np.maximum(np.maximum(v[:, 0:3], v[:, 3:6]), v[:, 6:9])
        payload = np.array([0, len(v)], np.uint32).tobytes() + v.tobytes() + np.concatenate([lo, hi], 1).tobytes()
    else:
        b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
        payload = np.array([1, len(b)], np.uint32).tobytes() + b.tobytes()
    r = run(binary, "build", payload, tmp_path)
    out = {}
    nn = r.u32()
    out["nodes"] = r.arr(np.float32, nn * 16).reshape(nn, 16)
    nd = r.u32()
    out["data_verts"] = r.arr(np.float32, nd * 9).reshape(nd, 9)
    out["data_idx"] = r.arr(np.uint32, nd)
    out["data_eon"] = r.arr(np.uint8, nd)
    nr = r.u32()
    out["refs_idx"] = r.arr(np.uint32, nr)
    out["refs_node"] = r.arr(np.uint32, nr)
    out["refs_eon"] = r.arr(np.uint8, nr)
    out["refs_aabb"] = r.arr(np.float32, nr * 6).reshape(nr, 6)
    na = r.u32()
    out["aabbs"] = r.arr(np.float32, na * 6).reshape(na, 6)
    return out


def assert_same_members(got, want):
    assert set(got) == set(want)
    for k in want:
        assert got[k].shape == want[k].shape, k
        assert np.array_equal(got[k].view(np.uint8), want[k].view(np.uint8)), f"member {k} differs"


def random_boxes(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = rng.random((n, 3)).astype(np.float32) * 50
    return np.concatenate([lo, lo + rng.random((n, 3)).astype(np.float32) * 5], 1)


def test_members_match_golden_cases(wrapper_bin, golden, tmp_path):
    """nodes and data of the wrapper's triangle build against the fixtures
    made by the compiled reference (no reference tree needed)."""
    g, _ = golden
    for name in ["rand1", "rand64", "rand2000", "identical9", "big300"]:
        tris = g[f"{name}/tris"]
        m = members(wrapper_bin, tmp_path, verts=tris)
        assert np.array_equal(m["nodes"].view(np.uint32), g[f"{name}/nodes"].view(np.uint32)), name
        assert np.array_equal(m["data_idx"], g[f"{name}/order"]), name
        assert np.array_equal(m["data_eon"], g[f"{name}/end_of_node"]), name
        assert np.array_equal(m["data_verts"], np.asarray(tris, np.float32).reshape(-1, 9)[g[f"{name}/order"]])
        assert len(m["refs_idx"]) == 0                      # the reference's member stays empty


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference tree not present on this host")
@pytest.mark.parametrize("case", ["random3000", "mixed_spatial", "single"])
def test_triangle_members_match_reference(wrapper_bin, tmp_path, case):
    if case == "random3000":
        tris = scenes.random_triangles(3000, seed=7)
    elif case == "single":
        tris = scenes.random_triangles(1, seed=8)
    else:
        # small triangles plus large ones across the unit cube: root spatial splits duplicate references
        rng = np.random.Generator(np.random.PCG64(9))
        tris = np.concatenate([scenes.random_triangles(4000, seed=9), rng.random((40, 3, 3)).astype(np.float32)])
    got = members(wrapper_bin, tmp_path, verts=tris)
    want = pyoracle.ref_members(verts=tris)
    assert_same_members(got, want)
    if case == "mixed_spatial":
        assert len(want["data_idx"]) > len(tris)             # the case does exercise spatial splits


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference tree not present on this host")
@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 1000])
def test_box_members_match_reference(wrapper_bin, tmp_path, n):
    boxes = random_boxes(n, seed=100 + n)
    got = members(wrapper_bin, tmp_path, boxes=boxes)
    want = pyoracle.ref_members(boxes=boxes)
    assert_same_members(got, want)
    if n == 1:
        assert len(got["refs_idx"]) == 2                     # the input reference ahead of the flattened one


# ---------------------------------------------------------------------------
# GPU queries through the wrapper
# ---------------------------------------------------------------------------

def trace_payload(tris, rays8):
    v = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays8, np.float32).reshape(-1, 8)
    return (np.array([len(v)], np.uint32).tobytes() + v.tobytes() + np.array([len(r)], np.uint32).tobytes()
            + r.tobytes())


@pytest.mark.gpu
def test_wrapper_queries_match_shader_oracle(wrapper_bin, tmp_path):
    tris = scenes.random_triangles(32768, seed=31)
    o, d = scenes.sphere_rays(6000, seed=32)
    rays8 = scenes.rays8(o, d, 1e-4, 10.0)
    # a second run of rays with a shorter window, and a third with a later start
    rays8[2000:4000, 7] = 1.6
    rays8[4000:, 6] = 1.2
    r = run(wrapper_bin, "trace", trace_payload(tris, rays8), tmp_path)
    n = len(rays8)
    hit = r.arr(np.uint8, n)
    tuv = r.arr(np.float32, 3 * n).reshape(n, 3)
    tri_ptr = r.arr(np.int32, n)
    idx = r.arr(np.uint32, n)
    occ = r.arr(np.uint8, n)
    m = r.u32()
    s_hit, s_idx = r.arr(np.uint8, m), r.arr(np.uint32, m)
    s_xyz, s_any = r.arr(np.float32, 3 * m).reshape(m, 3), r.arr(np.uint8, m)

    from atlas_rt import BVH
    b = BVH(tris)
    gt = b.pack_triangles()
    want_ptr = np.empty(n, np.int32)
    want_tuv = np.empty((n, 3), np.float32)
    want_occ = np.empty(n, np.uint8)
    for lo, hi in ((0, 2000), (2000, 4000), (4000, n)):
        p, t = pyoracle.closest_glsl(b.nodes_f32, gt, rays8[lo:hi])
        want_ptr[lo:hi], want_tuv[lo:hi] = p, t
        want_occ[lo:hi] = pyoracle.any_glsl(b.nodes_f32, gt, rays8[lo:hi])
    h = want_ptr >= 0
    assert 0.3 < h.mean() < 0.6 and h[2000:4000].mean() < 0.5 * h[:2000].mean()   # the windows do cut
    assert np.array_equal(hit.astype(bool), h)
    assert np.array_equal(tri_ptr, np.where(h, want_ptr, -1))
    assert np.array_equal(idx[h], b.order[want_ptr[h]])
    assert np.array_equal(tuv[h].view(np.uint32), want_tuv[h].view(np.uint32))
    assert np.array_equal(occ, want_occ)
    # the one-ray queries: the hit, data[hit].idx and (t, u, v); on a miss x = tMax and data[0]
    assert np.array_equal(s_hit, hit[:m]) and np.array_equal(s_any, occ[:m])
    hm = h[:m]
    assert np.array_equal(s_idx[hm], idx[:m][hm])
    assert np.array_equal(s_xyz[hm].view(np.uint32), tuv[:m][hm].view(np.uint32))
    assert np.all(s_xyz[~hm, 0] == rays8[:m][~hm, 7]) and np.all(s_idx[~hm] == b.order[0])
