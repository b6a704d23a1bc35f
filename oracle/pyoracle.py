"""Python access to the oracle libraries.  TEST INFRASTRUCTURE ONLY.

* ``libaeoracle.so`` (oracle/_build): the C restatement of the engine's BVH
  ray queries (ae_oracle.c), host and shader semantics.  Builds with gcc on
  any host.
* ``libaeref.so`` (oracle/_ref): the reference's own BVH builder and host
  queries compiled from the reference tree (oracle/Makefile target ``ref``).
  Only available where the reference tree is present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
PORT_LIB = ORACLE_DIR / "_build" / "libaeoracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libaeref.so"


def _reference_root() -> Path:
    """Where the reference tree lies: AE_REFERENCE_ROOT, else the location the
    oracle's build recipe (oracle/Makefile, REFERENCE_ROOT) names."""
    env = os.environ.get("AE_REFERENCE_ROOT")
    if env:
        return Path(env)
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", str(ORACLE_DIR), "reference-root"],
                           check=True, capture_output=True, text=True)
        return Path(r.stdout.strip())
    except (OSError, subprocess.CalledProcessError):
        return ORACLE_DIR / "_no_reference"


REFERENCE_ROOT = _reference_root()

P = C.c_void_p
U32 = C.c_uint32

_port = None
_ref = None


def build_port(force: bool = False) -> Path:
    src = [ORACLE_DIR / "ae_oracle.c", ORACLE_DIR / "ae_oracle_build.cpp", ORACLE_DIR / "ae_oracle.h"]
    if force or not PORT_LIB.exists() or any(s.stat().st_mtime > PORT_LIB.stat().st_mtime for s in src):
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "port"], check=True)
    return PORT_LIB


def build_ref(force: bool = False) -> Path | None:
    """Compiles the reference's own sources, if the reference tree exists here."""
    if not (REFERENCE_ROOT / "src" / "engine" / "volume" / "BVH.cpp").exists():
        return None
    if force or not REF_LIB.exists():
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref", f"REFERENCE_ROOT={REFERENCE_ROOT}"],
                       check=True, capture_output=True)
    return REF_LIB


def build_glsl_ref(force: bool = False) -> Path | None:
    """The reference's GLSL shading helpers compiled on the host
    (oracle/glsl/make_ref.py), if the reference tree exists here."""
    if not (REFERENCE_ROOT / "data" / "shader" / "brdf" / "brdf.hsh").exists():
        return None
    lib = ORACLE_DIR / "_ref" / "libglslref.so"
    if force or not lib.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("make_ref", ORACLE_DIR / "glsl" / "make_ref.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build(REFERENCE_ROOT)
    return lib


def port():
    global _port
    if _port is None:
        build_port()
        L = C.CDLL(str(PORT_LIB))
        L.aeo_closest_cpu.argtypes = [P, U32, P, U32, P, U32, C.c_int, P, P]
        L.aeo_any_cpu.argtypes = [P, U32, P, U32, P, U32, C.c_int, P]
        L.aeo_closest_glsl.argtypes = [P, U32, P, U32, P, U32, C.c_int, P, P, P, P]
        L.aeo_any_glsl.argtypes = [P, U32, P, U32, P, U32, C.c_int, P, P, P]
        L.aeo_closest_glsl_ties.argtypes = [P, U32, P, U32, P, U32, C.c_int, P, P, P, P]
        L.aeo_closest_glsl_ties.restype = None
        L.aeo_closest_f64_brute.argtypes = [P, U32, P, U32, C.c_int, P, P, P]
        L.aeo_scene_closest_glsl.argtypes = [P, U32, P, U32, P, U32, P, U32, U32, C.c_int, P, P, P, P, P]
        L.aeo_scene_any_glsl.argtypes = [P, U32, P, U32, P, U32, P, U32, U32, C.c_int, P]
        L.aeo_scene_closest_glsl.restype = None
        L.aeo_pathtrace.argtypes = [P, U32, P, P, U32, P, U32, P, P, U32, P, U32, P, U32, U32, U32, U32, U32, U32,
                                    C.c_float, C.c_int, P]
        L.aeo_pathtrace.restype = None
        L.aeo_pathtrace_env.argtypes = [P, U32, P, P, U32, P, U32, P, U32, P, U32, P, U32, P, U32, U32, U32, U32, U32,
                                        U32, C.c_float, P, C.c_int, P]
        L.aeo_pathtrace_env.restype = None
        L.aeo_scene_any_glsl.restype = None
        L.aeo_scene_closest_transparency_glsl.argtypes = [P, U32, P, U32, P, U32, P, U32, P, U32, P, U32, U32,
                                                          C.c_int, P, P, P]
        L.aeo_scene_closest_transparency_glsl.restype = None
        L.aeo_scene_any_transparency_glsl.argtypes = [P, U32, P, U32, P, U32, P, U32, P, U32, P, U32, U32,
                                                      C.c_int, P]
        L.aeo_scene_any_transparency_glsl.restype = None
        L.aeo_sample_r_bilinear.argtypes = [P, U32, C.c_int32, C.c_float, C.c_float]
        L.aeo_sample_r_bilinear.restype = C.c_float
        L.aeo_build_triangles.argtypes = [P, U32, C.c_int]
        L.aeo_build_triangles.restype = P
        L.aeo_build_aabbs.argtypes = [P, U32, C.c_int]
        L.aeo_build_aabbs.restype = P
        L.aeo_bvh_node_count.argtypes = [P]
        L.aeo_bvh_node_count.restype = U32
        L.aeo_bvh_prim_count.argtypes = [P]
        L.aeo_bvh_prim_count.restype = U32
        L.aeo_bvh_get.argtypes = [P, P, P, P]
        L.aeo_bvh_get.restype = None
        L.aeo_bvh_free.argtypes = [P]
        L.aeo_bvh_free.restype = None
        L.aeo_half_to_float.argtypes = [C.c_uint16]
        L.aeo_half_to_float.restype = C.c_float
        for f in (L.aeo_closest_cpu, L.aeo_any_cpu, L.aeo_closest_glsl, L.aeo_any_glsl, L.aeo_closest_f64_brute):
            f.restype = None
        _port = L
    return _port


def ref_available() -> bool:
    return REF_LIB.exists() or build_ref() is not None


def ref():
    global _ref
    if _ref is None:
        if build_ref() is None and not REF_LIB.exists():
            raise RuntimeError("the reference tree is not available on this host")
        L = C.CDLL(str(REF_LIB))
        L.aeref_build.restype = P
        L.aeref_build.argtypes = [P, U32, C.c_int]
        L.aeref_build_aabbs.restype = P
        L.aeref_build_aabbs.argtypes = [P, U32, C.c_int]
        for f in ("aeref_node_count", "aeref_data_count", "aeref_refs_count"):
            getattr(L, f).restype = U32
            getattr(L, f).argtypes = [P]
        L.aeref_get_nodes.argtypes = [P, P]
        L.aeref_get_data.argtypes = [P, P, P, P]
        L.aeref_get_refs.argtypes = [P, P]
        L.aeref_get_refs_full.argtypes = [P, P, P, P, P]
        L.aeref_aabbs_count.restype = U32
        L.aeref_aabbs_count.argtypes = [P]
        L.aeref_get_aabbs.argtypes = [P, P]
        L.aeref_closest.argtypes = [P, P, U32, C.c_int, P, P, P]
        L.aeref_any.argtypes = [P, P, U32, C.c_int, P]
        L.aeref_free.argtypes = [P]
        L.aeref_jobsystem_init.argtypes = [C.c_int]
        _ref = L
    return _ref


def _c(a, dt):
    return np.ascontiguousarray(a, dt)


# ---------------------------------------------------------------------------
# Restatement (port)
# ---------------------------------------------------------------------------

def closest_cpu(nodes_f32, tris_f32, rays8, threads=os.cpu_count()):
    n = len(rays8)
    nodes_f32, tris_f32, rays8 = _c(nodes_f32, np.float32), _c(tris_f32, np.float32), _c(rays8, np.float32)
    ptr = np.empty(n, np.int32)
    tuv = np.empty((n, 3), np.float32)
    port().aeo_closest_cpu(nodes_f32.ctypes.data, len(nodes_f32), tris_f32.ctypes.data, len(tris_f32),
                           rays8.ctypes.data, n, threads, ptr.ctypes.data, tuv.ctypes.data)
    return ptr, tuv


def any_cpu(nodes_f32, tris_f32, rays8, threads=os.cpu_count()):
    n = len(rays8)
    nodes_f32, tris_f32, rays8 = _c(nodes_f32, np.float32), _c(tris_f32, np.float32), _c(rays8, np.float32)
    occ = np.empty(n, np.uint8)
    port().aeo_any_cpu(nodes_f32.ctypes.data, len(nodes_f32), tris_f32.ctypes.data, len(tris_f32),
                       rays8.ctypes.data, n, threads, occ.ctypes.data)
    return occ


def build_bvh(verts=None, boxes=None, parallel=True):
    """The reference builder restated (oracle/ae_oracle_build.cpp): triangles
    (n, 3, 3) float32, or boxes (n, 6) for the top-level tree.  Returns
    (nodes (m, 16) float32 in the 64-byte node layout, order uint32,
    end_of_node uint8)."""
    L = port()
    if boxes is not None:
        b = _c(np.asarray(boxes, np.float32).reshape(-1, 6), np.float32)
        h = L.aeo_build_aabbs(b.ctypes.data if len(b) else None, len(b), int(parallel))
    else:
        v = _c(np.asarray(verts, np.float32).reshape(-1, 9), np.float32)
        h = L.aeo_build_triangles(v.ctypes.data if len(v) else None, len(v), int(parallel))
    try:
        nn, npr = L.aeo_bvh_node_count(h), L.aeo_bvh_prim_count(h)
        nodes = np.zeros((nn, 16), np.float32)
        order = np.zeros(npr, np.uint32)
        eon = np.zeros(npr, np.uint8)
        L.aeo_bvh_get(h, nodes.ctypes.data if nn else None, order.ctypes.data if npr else None,
                      eon.ctypes.data if npr else None)
    finally:
        L.aeo_bvh_free(h)
    return nodes, order, eon


def pack_bvh_triangles(verts, order, eon):
    """GPUBVHTriangle rows (n, 12) float32 in BVH order, as MeshData.cpp:241-248
    packs them with material 0 and opacity 1."""
    v = np.asarray(verts, np.float32).reshape(-1, 9)[order]
    out = np.zeros((len(order), 12), np.float32)
    out[:, 0:3], out[:, 4:7], out[:, 8:11] = v[:, 0:3], v[:, 3:6], v[:, 6:9]
    out[:, 3] = np.where(eon > 0, 1.0, -1.0)
    out[:, 11] = 1.0
    return out


def closest_glsl(nodes_f32, tris_f32, rays8, threads=os.cpu_count(), counters=False):
    n = len(rays8)
    nodes_f32, tris_f32, rays8 = _c(nodes_f32, np.float32), _c(tris_f32, np.float32), _c(rays8, np.float32)
    ptr = np.empty(n, np.int32)
    tuv = np.empty((n, 3), np.float32)
    nf = np.empty(n, np.uint32) if counters else None
    tf = np.empty(n, np.uint32) if counters else None
    port().aeo_closest_glsl(nodes_f32.ctypes.data, len(nodes_f32), tris_f32.ctypes.data, len(tris_f32),
                            rays8.ctypes.data, n, threads, ptr.ctypes.data, tuv.ctypes.data,
                            None if nf is None else nf.ctypes.data, None if tf is None else tf.ctypes.data)
    if counters:
        return ptr, tuv, nf, tf
    return ptr, tuv


def closest_glsl_ties(nodes_f32, tris_f32, rays8, threads=os.cpu_count()):
    """closest_glsl plus the GPU trace's near-tie flags and second distance:
    (tri_ptr, tuv, flags (bit 0 hit, bit 1 near tie), t_second)."""
    n = len(rays8)
    nodes_f32, tris_f32, rays8 = _c(nodes_f32, np.float32), _c(tris_f32, np.float32), _c(rays8, np.float32)
    ptr = np.empty(n, np.int32)
    tuv = np.empty((n, 3), np.float32)
    flags = np.empty(n, np.uint32)
    second = np.empty(n, np.float32)
    port().aeo_closest_glsl_ties(nodes_f32.ctypes.data, len(nodes_f32), tris_f32.ctypes.data, len(tris_f32),
                                 rays8.ctypes.data, n, threads, ptr.ctypes.data, tuv.ctypes.data, flags.ctypes.data,
                                 second.ctypes.data)
    return ptr, tuv, flags, second


def any_glsl(nodes_f32, tris_f32, rays8, threads=os.cpu_count(), counters=False):
    n = len(rays8)
    nodes_f32, tris_f32, rays8 = _c(nodes_f32, np.float32), _c(tris_f32, np.float32), _c(rays8, np.float32)
    occ = np.empty(n, np.uint8)
    nf = np.empty(n, np.uint32) if counters else None
    tf = np.empty(n, np.uint32) if counters else None
    port().aeo_any_glsl(nodes_f32.ctypes.data, len(nodes_f32), tris_f32.ctypes.data, len(tris_f32),
                        rays8.ctypes.data, n, threads, occ.ctypes.data,
                        None if nf is None else nf.ctypes.data, None if tf is None else tf.ctypes.data)
    if counters:
        return occ, nf, tf
    return occ


def closest_f64_brute(tris_f32, rays8, threads=os.cpu_count()):
    n = len(rays8)
    tris_f32, rays8 = _c(tris_f32, np.float32), _c(rays8, np.float32)
    ptr = np.empty(n, np.int32)
    t = np.empty(n, np.float64)
    t2 = np.empty(n, np.float64)
    port().aeo_closest_f64_brute(tris_f32.ctypes.data, len(tris_f32), rays8.ctypes.data, n, threads,
                                 ptr.ctypes.data, t.ctypes.data, t2.ctypes.data)
    return ptr, t, t2


class _Mesh(C.Structure):
    _fields_ = [("nodes", P), ("n_nodes", U32), ("tris", P), ("n_tris", U32), ("shading", P)]


def _mesh_table(meshes):
    """meshes: list of (nodes_f32 (n,16), tris_f32 (m,12)[, shading (m,24)]);
    keeps the arrays alive."""
    keep = []
    table = (_Mesh * max(1, len(meshes)))()
    for i, m in enumerate(meshes):
        nodes = _c(m[0], np.float32)
        tris = _c(m[1], np.float32)
        keep += [nodes, tris]
        table[i].nodes = nodes.ctypes.data if nodes.size else None
        table[i].n_nodes = len(nodes)
        table[i].tris = tris.ctypes.data if tris.size else None
        table[i].n_tris = len(tris)
        if len(m) > 2 and m[2] is not None:
            sh = _c(m[2], np.float32)
            keep.append(sh)
            table[i].shading = sh.ctypes.data
    return table, keep


class _Texture(C.Structure):
    pass


_Texture._fields_ = [("texels", P), ("width", U32), ("height", U32), ("format", U32), ("row_pitch", U32),
                     ("mips", C.POINTER(_Texture)), ("n_mips", U32)]


def mip_chain(tex: np.ndarray) -> list:
    """Levels 1.. down to 1 x 1 of a texel array: texel (x, y) of level k + 1
    averages texels (2x + {0, 1}, 2y + {0, 1}) of level k, the indices
    clamped to the level; UNORM bytes as (a + b + c + d + 2) // 4, floats as
    ((a + b) + (c + d)) * 0.25 in float32."""
    out = []
    cur = tex
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        h, w = cur.shape[:2]
        nh, nw = max(1, h >> 1), max(1, w >> 1)
        x0 = np.minimum(2 * np.arange(nw), w - 1)
        x1 = np.minimum(2 * np.arange(nw) + 1, w - 1)
        y0 = np.minimum(2 * np.arange(nh), h - 1)
        y1 = np.minimum(2 * np.arange(nh) + 1, h - 1)
        a, b = cur[y0][:, x0], cur[y0][:, x1]
        c, d = cur[y1][:, x0], cur[y1][:, x1]
        if cur.dtype == np.uint8:
            nxt = ((a.astype(np.uint32) + b + c + d + 2) >> 2).astype(np.uint8)
        else:
            nxt = ((a + b) + (c + d)) * np.float32(0.25)
        nxt = np.ascontiguousarray(nxt)
        out.append(nxt)
        cur = nxt
    return out


TEX_FORMATS = {"r8": 0, "rgba8": 1, "r32f": 2}


def texture_format(a: np.ndarray) -> int:
    """AE_TEX_* of a texel array: uint8 (h, w) R8, uint8 (h, w, 4) RGBA8,
    float32 (h, w) R32F."""
    if a.dtype == np.uint8 and a.ndim == 2:
        return 0
    if a.dtype == np.uint8 and a.ndim == 3 and a.shape[2] == 4:
        return 1
    if a.dtype == np.float32 and a.ndim == 2:
        return 2
    raise ValueError(f"unsupported texel array {a.dtype} {a.shape}")


def _texture_table(textures):
    """textures: list of texel arrays (see texture_format); keeps them alive."""
    textures = list(textures or [])
    keep = [np.ascontiguousarray(t) for t in textures]
    table = (_Texture * max(1, len(keep)))()
    extra = []
    for i, t in enumerate(keep):
        table[i].texels = t.ctypes.data
        table[i].height, table[i].width = t.shape[0], t.shape[1]
        table[i].format = texture_format(t)
        table[i].row_pitch = 0
        levels = mip_chain(t)
        mt = (_Texture * max(1, len(levels)))()
        for k, lv in enumerate(levels):
            mt[k].texels = lv.ctypes.data
            mt[k].height, mt[k].width = lv.shape[0], lv.shape[1]
            mt[k].format = table[i].format
        table[i].mips = mt
        table[i].n_mips = len(levels)
        extra += [levels, mt]
    return table, len(keep), keep + extra


def sample_r_bilinear(textures, tex_id, u, v):
    """The traversal's opacity lookup of one texture at (u, v)."""
    table, n, keep = _texture_table(textures)
    return port().aeo_sample_r_bilinear(table, n, tex_id, u, v)


def half_to_float(h: int) -> float:
    return port().aeo_half_to_float(h)


def scene_closest_glsl(tlas_f32, instances, meshes, rays8, cull_mask=0xFFFFFFFF, threads=os.cpu_count(),
                       counters=False):
    """HitClosest over TLAS + instances + BLASes.  instances: structured array
    with the GPUBVHInstance layout (64 bytes each)."""
    n = len(rays8)
    tlas_f32, rays8 = _c(tlas_f32, np.float32), _c(rays8, np.float32)
    inst = np.ascontiguousarray(instances)
    table, keep = _mesh_table(meshes)
    ptr = np.empty(n, np.int32)
    ino = np.empty(n, np.int32)
    tuv = np.empty((n, 3), np.float32)
    nf = np.empty(n, np.uint32) if counters else None
    tf = np.empty(n, np.uint32) if counters else None
    port().aeo_scene_closest_glsl(tlas_f32.ctypes.data if tlas_f32.size else None, len(tlas_f32),
                                  inst.ctypes.data, len(inst), table, len(meshes), rays8.ctypes.data, n,
                                  cull_mask, threads, ptr.ctypes.data, ino.ctypes.data, tuv.ctypes.data,
                                  None if nf is None else nf.ctypes.data, None if tf is None else tf.ctypes.data)
    if counters:
        return ptr, ino, tuv, nf, tf
    return ptr, ino, tuv


def scene_any_glsl(tlas_f32, instances, meshes, rays8, cull_mask=0xFFFFFFFF, threads=os.cpu_count()):
    n = len(rays8)
    tlas_f32, rays8 = _c(tlas_f32, np.float32), _c(rays8, np.float32)
    inst = np.ascontiguousarray(instances)
    table, keep = _mesh_table(meshes)
    occ = np.empty(n, np.uint8)
    port().aeo_scene_any_glsl(tlas_f32.ctypes.data if tlas_f32.size else None, len(tlas_f32),
                              inst.ctypes.data, len(inst), table, len(meshes), rays8.ctypes.data, n,
                              cull_mask, threads, occ.ctypes.data)
    return occ


def scene_closest_transparency_glsl(tlas_f32, instances, meshes, materials, rays8, cull_mask=0xFFFFFFFF,
                                    threads=os.cpu_count(), textures=None):
    """HitClosestTransparency (bvh.hsh:275-357); meshes carry shading
    triangles, materials is the GPUMaterial array, textures the texel arrays
    that the materials' opacityTexture indexes."""
    n = len(rays8)
    tlas_f32, rays8 = _c(tlas_f32, np.float32), _c(rays8, np.float32)
    inst = np.ascontiguousarray(instances)
    mats = np.ascontiguousarray(materials)
    table, keep = _mesh_table(meshes)
    ttab, ntex, tkeep = _texture_table(textures)
    ptr = np.empty(n, np.int32)
    ino = np.empty(n, np.int32)
    tuv = np.empty((n, 3), np.float32)
    port().aeo_scene_closest_transparency_glsl(tlas_f32.ctypes.data if tlas_f32.size else None, len(tlas_f32),
                                               inst.ctypes.data, len(inst), table, len(meshes), mats.ctypes.data,
                                               len(mats), ttab, ntex, rays8.ctypes.data, n, cull_mask, threads,
                                               ptr.ctypes.data, ino.ctypes.data, tuv.ctypes.data)
    return ptr, ino, tuv


def scene_any_transparency_glsl(tlas_f32, instances, meshes, materials, rays8, cull_mask=0xFFFFFFFF,
                                threads=os.cpu_count(), textures=None):
    """HitAnyTransparency (bvh.hsh:443-524): transparency per ray (1 = clear)."""
    n = len(rays8)
    tlas_f32, rays8 = _c(tlas_f32, np.float32), _c(rays8, np.float32)
    inst = np.ascontiguousarray(instances)
    mats = np.ascontiguousarray(materials)
    table, keep = _mesh_table(meshes)
    ttab, ntex, tkeep = _texture_table(textures)
    out = np.empty(n, np.float32)
    port().aeo_scene_any_transparency_glsl(tlas_f32.ctypes.data if tlas_f32.size else None, len(tlas_f32),
                                           inst.ctypes.data, len(inst), table, len(meshes), mats.ctypes.data,
                                           len(mats), ttab, ntex, rays8.ctypes.data, n, cull_mask, threads,
                                           out.ctypes.data)
    return out


def pathtrace(tlas_f32, instances, inst_model, meshes, materials, lights, cam, width, height, spp,
              sample_offset=0, max_bounces=3, seed=1, epsilon=0.1, threads=os.cpu_count(), accum=None,
              textures=None, environment=None):
    """CPU restatement of the path tracer; returns the summed radiance
    (height, width, 3) float64 over spp samples (add to `accum` if given).
    environment: a constant radiance added on a miss (rayHit.csh:166-171)."""
    tlas_f32 = _c(tlas_f32, np.float32)
    inst = np.ascontiguousarray(instances)
    model = _c(inst_model, np.float32)
    mats = np.ascontiguousarray(materials)
    lights = _c(lights, np.float32)
    cam = _c(cam, np.float32)
    table, keep = _mesh_table(meshes)
    out = np.zeros((height, width, 3), np.float64) if accum is None else accum
    ttab, ntex, tkeep = _texture_table(textures)
    env = None if environment is None else _c(environment, np.float32).reshape(3)
    port().aeo_pathtrace_env(tlas_f32.ctypes.data, len(tlas_f32), inst.ctypes.data, model.ctypes.data, len(inst),
                             table, len(meshes), mats.ctypes.data, len(mats), lights.ctypes.data, len(lights), ttab, ntex,
                             cam.ctypes.data, width, height, spp, sample_offset, max_bounces, seed, epsilon,
                             None if env is None else env.ctypes.data, threads, out.ctypes.data)
    return out


# ---------------------------------------------------------------------------
# Compiled reference
# ---------------------------------------------------------------------------

class RefBVH:
    """The reference's Volume::BVH built from triangles, exported to arrays."""

    def __init__(self, verts, parallel=True):
        L = ref()
        v = _c(verts, np.float32).reshape(-1, 9)
        self.h = L.aeref_build(v.ctypes.data if len(v) else None, len(v), int(parallel))
        nn = L.aeref_node_count(self.h)
        nd = L.aeref_data_count(self.h)
        self.nodes_f32 = np.zeros((nn, 16), np.float32)
        if nn:
            L.aeref_get_nodes(self.h, self.nodes_f32.ctypes.data)
        self.data_verts = np.zeros((nd, 9), np.float32)
        self.order = np.zeros(nd, np.uint32)
        self.end_of_node = np.zeros(nd, np.uint8)
        if nd:
            L.aeref_get_data(self.h, self.data_verts.ctypes.data, self.order.ctypes.data,
                             self.end_of_node.ctypes.data)

    def gpu_triangles(self):
        """GPUBVHTriangle packing of the reference data (MeshData.cpp:241-248)."""
        nd = len(self.order)
        t = np.zeros((nd, 12), np.float32)
        t[:, 0:3] = self.data_verts[:, 0:3]
        t[:, 3] = np.where(self.end_of_node > 0, 1.0, -1.0)
        t[:, 4:7] = self.data_verts[:, 3:6]
        t[:, 8:11] = self.data_verts[:, 6:9]
        t[:, 11] = 1.0
        return t

    def closest(self, rays8, threads=os.cpu_count()):
        n = len(rays8)
        rays8 = _c(rays8, np.float32)
        idx = np.empty(n, np.int32)
        tuv = np.empty((n, 3), np.float32)
        rb = np.empty(n, np.uint8)
        ref().aeref_closest(self.h, rays8.ctypes.data, n, threads, idx.ctypes.data, tuv.ctypes.data,
                            rb.ctypes.data)
        return idx, tuv, rb

    def any(self, rays8, threads=os.cpu_count()):
        n = len(rays8)
        rays8 = _c(rays8, np.float32)
        occ = np.empty(n, np.uint8)
        ref().aeref_any(self.h, rays8.ctypes.data, n, threads, occ.ctypes.data)
        return occ

    def __del__(self):
        if getattr(self, "h", None):
            ref().aeref_free(self.h)
            self.h = None


def ref_members(verts=None, boxes=None, parallel=True):
    """Every public member of the reference's Volume::BVH (BVH.h:133-137)
    after the triangle build (verts; boxes are the triangles' bounds) or the
    AABB-only build (boxes): nodes (n, 16) in the GPUBVHNode layout, data
    (verts, idx, endOfNode), refs (idx, nodeIdx, endOfNode, aabb) and aabbs."""
    L = ref()
    if verts is not None:
        v = _c(verts, np.float32).reshape(-1, 9)
        h = L.aeref_build(v.ctypes.data if len(v) else None, len(v), int(parallel))
    else:
        b = _c(boxes, np.float32).reshape(-1, 6)
        h = L.aeref_build_aabbs(b.ctypes.data if len(b) else None, len(b), int(parallel))
    try:
        nn, nd, nr = L.aeref_node_count(h), L.aeref_data_count(h), L.aeref_refs_count(h)
        na = L.aeref_aabbs_count(h)
        out = {"nodes": np.zeros((nn, 16), np.float32), "data_verts": np.zeros((nd, 9), np.float32),
               "data_idx": np.zeros(nd, np.uint32), "data_eon": np.zeros(nd, np.uint8),
               "refs_idx": np.zeros(nr, np.uint32), "refs_node": np.zeros(nr, np.uint32),
               "refs_eon": np.zeros(nr, np.uint8), "refs_aabb": np.zeros((nr, 6), np.float32),
               "aabbs": np.zeros((na, 6), np.float32)}
        if nn:
            L.aeref_get_nodes(h, out["nodes"].ctypes.data)
        if nd:
            L.aeref_get_data(h, out["data_verts"].ctypes.data, out["data_idx"].ctypes.data, out["data_eon"].ctypes.data)
        if nr:
            L.aeref_get_refs_full(h, out["refs_idx"].ctypes.data, out["refs_node"].ctypes.data,
                                  out["refs_eon"].ctypes.data, out["refs_aabb"].ctypes.data)
        if na:
            L.aeref_get_aabbs(h, out["aabbs"].ctypes.data)
        return out
    finally:
        L.aeref_free(h)


def ref_build_aabbs(boxes, parallel=True):
    """The reference's AABB-only BVH: (nodes_f32, refs order)."""
    L = ref()
    b = _c(boxes, np.float32).reshape(-1, 6)
    h = L.aeref_build_aabbs(b.ctypes.data, len(b), int(parallel))
    nn = L.aeref_node_count(h)
    nr = L.aeref_refs_count(h)
    nodes = np.zeros((nn, 16), np.float32)
    if nn:
        L.aeref_get_nodes(h, nodes.ctypes.data)
    order = np.zeros(nr, np.uint32)
    if nr:
        L.aeref_get_refs(h, order.ctypes.data)
    L.aeref_free(h)
    return nodes, order


# ---------------------------------------------------------------------------
# The traversal's other consumers (RTAO, reflections, RTGI, DDGI probe rays)
# ---------------------------------------------------------------------------

class _GBuffer(C.Structure):
    _fields_ = [("depth", P), ("normal", P), ("offset", P), ("roughness", P), ("samples", P), ("width", U32),
                ("height", U32), ("half_res", U32), ("reserved", U32), ("ip_matrix", C.c_float * 16),
                ("iv_matrix", C.c_float * 16), ("scrambling_ranking", P), ("sobol_sequence", P)]


class _PassParams(C.Structure):
    _fields_ = [("radius", C.c_float), ("bias", C.c_float), ("roughness_cutoff", C.c_float),
                ("radiance_limit", C.c_float), ("environment", C.c_float * 3), ("flags", U32),
                ("frame_seed", U32), ("seed", U32), ("texture_level", U32), ("reserved", U32)]


class _DdgiProbes(C.Structure):
    _fields_ = [("probes", P), ("ray_dirs", P), ("ray_dirs_inactive", P), ("rotation", C.c_float * 16),
                ("n_probes", U32), ("ray_count", U32), ("inactive_ray_count", U32), ("reserved", U32)]


class _PassScene(C.Structure):
    _fields_ = [("tlas", P), ("n_tlas", U32), ("inst", P), ("inst_model", P), ("n_inst", U32), ("meshes", P),
                ("n_meshes", U32), ("materials", P), ("n_materials", U32), ("textures", P), ("n_textures", U32),
                ("lights", P), ("n_lights", U32)]


def _pass_fns():
    L = port()
    if not getattr(L, "_pass_ready", False):
        for name in ("aeo_pass_rtao", "aeo_pass_reflections", "aeo_pass_rtgi"):
            getattr(L, name).argtypes = [C.POINTER(_PassScene), C.POINTER(_GBuffer), C.POINTER(_PassParams),
                                         C.c_int, P]
            getattr(L, name).restype = None
        L.aeo_pass_ddgi.argtypes = [C.POINTER(_PassScene), C.POINTER(_DdgiProbes), C.POINTER(_PassParams),
                                    C.c_int, P]
        L.aeo_pass_ddgi.restype = None
        L._pass_ready = True
    return L


def _pass_scene(tlas_f32, instances, inst_model, meshes, materials, lights, textures):
    tlas_f32 = _c(tlas_f32, np.float32)
    inst = np.ascontiguousarray(instances)
    model = _c(inst_model, np.float32)
    mats = np.ascontiguousarray(materials)
    lights = _c(lights, np.float32).reshape(-1, 16)
    table, keep = _mesh_table(meshes)
    ttab, ntex, tkeep = _texture_table(textures)
    s = _PassScene(tlas_f32.ctypes.data, len(tlas_f32), inst.ctypes.data, model.ctypes.data, len(inst), C.cast(table, P),
                   len(meshes), mats.ctypes.data, len(mats), C.cast(ttab, P), ntex,
                   lights.ctypes.data if len(lights) else None, len(lights))
    return s, [tlas_f32, inst, model, mats, lights, table, keep, ttab, tkeep]


def _pass_params(radius=1.0, bias=0.0, roughness_cutoff=1.0, radiance_limit=10.0, environment=(0, 0, 0),
                 opacity_check=False, frame_seed=0, seed=1, texture_level=0):
    return _PassParams(radius, bias, roughness_cutoff, radiance_limit, (C.c_float * 3)(*environment),
                       1 if opacity_check else 0, frame_seed, seed, texture_level, 0)


def _gbuffer(gb):
    """gb: dict of numpy arrays like atlas_rt.Context._gbuffer takes."""
    depth = _c(gb["depth"], np.float32)
    normal = _c(gb["normal"], np.float32)
    keep = [depth, normal]
    g = _GBuffer()
    g.height, g.width = depth.shape[0], depth.shape[1]
    g.depth, g.normal = depth.ctypes.data, normal.ctypes.data
    for name, dt in (("offset", np.uint8), ("roughness", np.float32), ("samples", np.float32),
                     ("scrambling_ranking", np.uint8), ("sobol_sequence", np.uint8)):
        if gb.get(name) is not None:
            a = np.ascontiguousarray(gb[name], dt)
            keep.append(a)
            setattr(g, name, a.ctypes.data)
    g.half_res = int(gb.get("half_res", 0))
    for name in ("ip_matrix", "iv_matrix"):
        getattr(g, name)[:] = list(np.asarray(gb[name], np.float32).reshape(4, 4).T.reshape(-1))
    return g, keep


def blue_noise(ranking, sobol, width, height, sample_index):
    """SampleBlueNoise (common/bluenoise.hsh:9-32) for dimensions 0 and 1 of
    every pixel of a width x height image -> (height, width, 2) float32.
    ranking: (128, 128, 4) and sobol: (256, 4) uint8 RGBA texels, read as the
    shader's sampler returns them (c / 255) and scaled by 256 as it does."""
    def texel(t):
        v = np.asarray(t, np.uint8).astype(np.float32) / np.float32(255.0) * np.float32(256.0)
        return np.clip(v, np.float32(0.0), np.float32(255.0)).astype(np.int32)
    y, x = np.mgrid[0:height, 0:width]
    r = texel(ranking)[y % 128, x % 128]
    s = texel(sobol)[(int(sample_index) % 256) ^ r[..., 2]]
    v = s[..., :2] ^ r[..., :2]
    return ((np.float32(0.5) + v.astype(np.float32)) / np.float32(256.0)).astype(np.float32)


def pass_screen(kind, scene, gbuffer, threads=os.cpu_count(), **params):
    """kind: "rtao" -> (h, w) float32; "reflections" / "rtgi" -> (h, w, 4).
    scene: (tlas_f32, instances, inst_model, meshes, materials, lights[, textures])."""
    s, skeep = _pass_scene(*scene[:6], scene[6] if len(scene) > 6 else None)
    g, gkeep = _gbuffer(gbuffer)
    pp = _pass_params(**params)
    h, w = gbuffer["depth"].shape
    out = np.zeros((h, w) if kind == "rtao" else (h, w, 4), np.float32)
    getattr(_pass_fns(), f"aeo_pass_{kind}")(C.byref(s), C.byref(g), C.byref(pp), threads, out.ctypes.data)
    return out


def pass_ddgi(scene, probes, ray_dirs, rotation, out, ray_dirs_inactive=None, inactive_ray_count=0,
              threads=os.cpu_count(), **params):
    """DDGI probe rays into `out` ((n_probes * ray_count, 4) float32, entries
    beyond a probe's ray count untouched)."""
    s, skeep = _pass_scene(*scene[:6], scene[6] if len(scene) > 6 else None)
    probes = _c(probes, np.float32)
    dirs = _c(ray_dirs, np.float32)
    dirs_in = None if ray_dirs_inactive is None else _c(ray_dirs_inactive, np.float32)
    d = _DdgiProbes()
    d.probes, d.ray_dirs = probes.ctypes.data, dirs.ctypes.data
    d.ray_dirs_inactive = None if dirs_in is None else dirs_in.ctypes.data
    d.rotation[:] = list(np.asarray(rotation, np.float32).reshape(4, 4).T.reshape(-1))
    d.n_probes, d.ray_count, d.inactive_ray_count = len(probes), len(dirs), inactive_ray_count
    assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == len(probes) * len(dirs) * 4
    _pass_fns().aeo_pass_ddgi(C.byref(s), C.byref(d), C.byref(_pass_params(**params)), threads, out.ctypes.data)
    return out


# ---------------------------------------------------------------------------
# The engine's host light list (numpy restatement, float32 operation by operation)
# ---------------------------------------------------------------------------

def _srgb_to_linear(c):
    """ColorConverter::ConvertSRGBToLinear (common/ColorConverter.h:18-23):
    pow(c, 2.2) in float32, rounded once as the C library's powf rounds."""
    return (np.asarray(c, np.float32).astype(np.float64) ** np.float64(np.float32(2.2))).astype(np.float32)


def _dot3(a, b):
    """glm dot of vec3: (x*x' + y*y') + z*z' in float32."""
    p = (np.asarray(a, np.float32) * np.asarray(b, np.float32)).astype(np.float32)
    return ((p[..., 0] + p[..., 1]) + p[..., 2]).astype(np.float32)


def _unpack10(bits):
    """Common::Packing::UnpackSignedVector3x10_1x2 (common/Packing.cpp:37-48), xyz."""
    c = np.asarray(bits, np.float32).view(np.int32)
    f32 = np.float32
    return np.stack([((c >> s) & 1023).astype(f32) / f32(1023.0) * f32(2.0) - f32(1.0) for s in (0, 10, 20)], -1)


def triangle_lights(shading, emissive_srgb, emissive_intensity):
    """RayTracingWorld::BuildTriangleLightsForMesh (RayTracingWorld.cpp:322-376)
    over a GPUTriangle array (n, 24) float32: GPULight records (m, 16)."""
    f32 = np.float32
    sh = np.asarray(shading, f32).reshape(-1, 24)
    mat = sh[:, 15].view(np.int32)
    rad = _srgb_to_linear(np.asarray(emissive_srgb, f32).reshape(-1, 3))[mat]
    bright = _dot3(rad, np.full(3, 0.3333, f32))
    keep = np.nonzero(bright > 0)[0]
    out = np.zeros((len(keep), 16), f32)
    for k, i in enumerate(keep):
        t = sh[i]
        v0, v1, v2 = t[0:3], t[4:7], t[8:11]
        n = _unpack10(np.array([t[3], t[7], t[11]], f32))
        P = ((v0 + v1) + v2) / f32(3.0)
        N = ((n[0] + n[1]) + n[2]) / f32(3.0)
        dist = lambda a, b: np.sqrt(_dot3(a - b, a - b))   # noqa: E731
        a, b, c = dist(v1, v0), dist(v2, v0), dist(v1, v2)
        p = f32(0.5) * ((a + b) + c)
        area = np.sqrt(((p * (p - a)) * (p - b)) * (p - c))
        color = _srgb_to_linear(rad[i]) * f32(np.asarray(emissive_intensity, f32)[mat[i]])
        out[k, 0:3], out[k, 3] = P, 1.0
        out[k, 4:7] = N
        out[k, 8:11] = color
        out[k, 12] = np.uint32((1 << 28) | int(i)).view(f32)
        out[k, 13] = area * bright[i]
        out[k, 14] = area
    return out


def lights_instance(lights, model, instance):
    """RayTracingWorld::UpdateTriangleLights (:378-407): P = M (P, 1), N = M (N, 0)
    with glm's pairwise column sum, data.w = the instance bits."""
    f32 = np.float32
    L = np.asarray(lights, f32).reshape(-1, 16).copy()
    M = np.asarray(model, f32).reshape(4, 4)
    for v, w in ((slice(0, 3), f32(1.0)), (slice(4, 7), f32(0.0))):
        x = L[:, v].copy()
        for r in range(3):
            m = M[r]
            L[:, v.start + r] = (m[0] * x[:, 0] + m[1] * x[:, 1]) + (m[2] * x[:, 2] + m[3] * w)
    L[:, 15] = np.int32(instance).view(f32)
    return L


def lights_normalize(lights):
    """RayTracingHelper::UpdateLights' weights (RayTracingHelper.cpp:481-499)."""
    f32 = np.float32
    L = np.asarray(lights, f32).reshape(-1, 16).copy()
    w = L[:, 13]
    mx = f32(0.0)
    for x in w:
        mx = max(mx, x)
    mn = f32(0.005) * mx
    total = f32(0.0)
    for k in range(len(w)):
        w[k] = max(w[k], mn)
        total = f32(total + w[k])
    L[:, 13] = w / total
    return L


def lights_select(lights, capacity, uniforms):
    """DispatchAndHit's selection (RayTracingHelper.cpp:72-105) with
    Common::Piecewise1D (Piecewise.cpp:11-78) on the given uniforms."""
    f32 = np.float32
    L = np.asarray(lights, f32).reshape(-1, 16)
    n = len(L)
    if n <= capacity:
        out = L.copy()
        out[:, 13] = 1.0
        return out
    cdf = np.zeros(n + 1, f32)
    s = f32(0.0)
    for k in range(n):
        cdf[k] = s
        s = f32(s + f32(L[k, 13] / f32(n)))
    cdf[n] = s
    cdf = (cdf / s).astype(f32)
    out = np.zeros((capacity, 16), f32)
    for j in range(capacity):
        x = f32(uniforms[j])
        lo, hi, found = 0, n, -1
        while lo <= hi:
            m = lo + (hi - lo) // 2
            k = m if m + 1 > n else m + 1
            if cdf[m] <= x <= cdf[k]:
                found = m
                break
            if cdf[m] < x:
                lo = m + 1
            else:
                hi = m - 1
        if found < 0 or found >= n:
            found = n - 1
        out[j] = L[found]
        out[j, 13] = L[found, 13] * f32(capacity)
    return out
