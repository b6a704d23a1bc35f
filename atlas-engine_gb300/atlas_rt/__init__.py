"""Python host binding of the GB300 ray-tracing library (libatlas_rt.so).

Mirrors the engine's host interface for the software ray-tracing path:

* :class:`BVH` -- ``Volume::BVH`` (src/engine/volume/BVH.h:114-138): built
  from triangles or AABBs, exposing ``nodes`` (GPUBVHNode layout), the
  flattened primitive ``order`` (``BVHTriangle::idx``) and leaf flags, and the
  ``GPUBVHTriangle`` packing of ``MeshData::BuildBVH``.
* :class:`Context` -- device context: mesh uploads (``Mesh::BuildBVH``'s
  buffers) and the batched GPU ray queries ``trace_closest`` / ``trace_any``
  (shader ``HitClosest`` / ``HitAny``; the GPU form of
  ``BVH::GetIntersection`` / ``GetIntersectionAny``).

Buffers may be numpy arrays (host memory; copied in and out by the library)
or CUDA tensors / raw device pointers (asynchronous on the given stream).
Every call goes through the C ABI; nothing here computes results itself.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import (AeRtError, BatchDesc, BounceParams, Camera, CastOutputs, Config, DdgiProbes, GBuffer, PassParams,
                      PtRealtime,
                      PtParams, RcConfig, lib)

NODE_DTYPE = np.dtype([("leftMin", "<f4", 3), ("leftMax", "<f4", 3),
                       ("rightMin", "<f4", 3), ("rightMax", "<f4", 3),
                       ("leftPtr", "<i4"), ("rightPtr", "<i4"), ("padding", "<i4", 2)])
HIT_DTYPE = np.dtype([("t", "<f4"), ("triPtr", "<i4"), ("instance", "<i4"), ("flags", "<u4"),
                      ("u", "<f4"), ("v", "<f4"), ("tSecond", "<f4"), ("reserved", "<i4")])
INSTANCE_DTYPE = np.dtype([("inverseMatrix", "<f4", 12), ("meshOffset", "<i4"), ("materialOffset", "<i4"),
                           ("nextInstance", "<i4"), ("mask", "<u4")])
MATERIAL_DTYPE = np.dtype([("ID", "<i4"), ("baseColor", "<f4", 3), ("emissiveColor", "<f4", 3),
                           ("opacity", "<f4"), ("roughness", "<f4"), ("metalness", "<f4"), ("ao", "<f4"),
                           ("reflectance", "<f4"), ("normalScale", "<f4"), ("invertUVs", "<i4"),
                           ("twoSided", "<i4"), ("cullBackFaces", "<i4"), ("useVertexColors", "<i4"),
                           ("baseColorTexture", "<i4"), ("opacityTexture", "<i4"), ("normalTexture", "<i4"),
                           ("roughnessTexture", "<i4"), ("metalnessTexture", "<i4"), ("aoTexture", "<i4")])
assert NODE_DTYPE.itemsize == 64 and HIT_DTYPE.itemsize == 32 and INSTANCE_DTYPE.itemsize == 64
assert MATERIAL_DTYPE.itemsize == 92

HIT_FLAG_HIT = 0x1
HIT_FLAG_NEAR_TIE = 0x2
HIT_FLAG_OVERFLOW = 0x4
HIT_FLAG_ITER_CAP = 0x8
HIT_FLAG_RETESTED = 0x10
HIT64_DTYPE = np.dtype([("t", "<f8"), ("t_second", "<f8"), ("triPtr", "<i4"), ("flags", "<u4"),
                        ("reserved", "<i4", (2,))])
assert HIT64_DTYPE.itemsize == 32

PT_MIS = 0x1
PT_CENTERED = 0x2

MASK_ALL = 1 << 7
MASK_SHADOW = 1 << 6
CFG_COUNT_FETCHES = 0x1
CFG_NO_NEAR_TIES = 0x2
CFG_STAGED_RAYS = 0x4
CFG_APPROXIMATE = 0x8


def _check(status: int, ctx=None):
    if status != 0:
        msg = ""
        if ctx is not None:
            raw = lib().ae_rt_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise AeRtError(status, msg)


def _ptr(x):
    """Raw address of a numpy array, a CUDA tensor or an integer pointer."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("buffer must be C-contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_contiguous") and not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)!r}")


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class BVH:
    """Host BVH with the reference builder's output layout (``Volume::BVH``)."""

    def __init__(self, verts=None, aabbs=None, parallel: bool = True, *, boxes_only=None):
        L = lib()
        h = C.c_void_p()
        if boxes_only is not None:
            b = np.ascontiguousarray(boxes_only, np.float32).reshape(-1, 6)
            self.n_input = len(b)
            _check(L.ae_bvh_build_aabbs(_ptr(b) if len(b) else None, len(b), int(parallel), C.byref(h)))
            self._verts = None
        else:
            v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
            a = None if aabbs is None else np.ascontiguousarray(aabbs, np.float32).reshape(-1, 6)
            self.n_input = len(v)
            _check(L.ae_bvh_build_triangles(_ptr(v) if len(v) else None, _ptr(a), len(v), int(parallel),
                                            C.byref(h)))
            self._verts = v
        self._h = h
        nn = L.ae_bvh_node_count(h)
        npr = L.ae_bvh_primitive_count(h)
        self.nodes = np.zeros(nn, NODE_DTYPE)
        _check(L.ae_bvh_get_nodes(h, _ptr(self.nodes) if nn else None))
        self.order = np.zeros(npr, np.uint32)
        self.end_of_node = np.zeros(npr, np.uint8)
        if npr:
            _check(L.ae_bvh_get_order(h, _ptr(self.order), _ptr(self.end_of_node)))

    def pack_triangles(self, material=None, opacity=None) -> np.ndarray:
        """GPUBVHTriangle array (n, 12) float32 in BVH order (MeshData.cpp:241-248)."""
        out = np.zeros((len(self.order), 12), np.float32)
        m = None if material is None else np.ascontiguousarray(material, np.int32)
        o = None if opacity is None else np.ascontiguousarray(opacity, np.float32)
        if len(self.order):
            _check(lib().ae_bvh_pack_triangles(self._h, _ptr(self._verts), _ptr(m), _ptr(o), _ptr(out)))
        return out

    def pack_shading(self, normals=None, material=None, opacity=None) -> np.ndarray:
        """GPUTriangle array (n, 24) float32 in BVH order (MeshData.cpp:172-239)."""
        out = np.zeros((len(self.order), 24), np.float32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        m = None if material is None else np.ascontiguousarray(material, np.int32)
        o = None if opacity is None else np.ascontiguousarray(opacity, np.float32)
        if len(self.order):
            _check(lib().ae_bvh_pack_shading(self._h, _ptr(self._verts), _ptr(nrm), _ptr(m), _ptr(o), _ptr(out)))
        return out

    def pack_uvs(self, shading: np.ndarray, uvs) -> np.ndarray:
        """Writes per-input-triangle UVs ((n, 3, 2) or (n, 6) float32) into the
        GPUTriangle array from pack_shading as packHalf2x16 (MeshData.cpp:172-239)."""
        uv = np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
        if self._verts is None or len(uv) != self.n_input or shading.shape != (len(self.order), 24) or shading.dtype != np.float32 \
                or not shading.flags.c_contiguous:
            raise ValueError("uvs must hold 6 floats per triangle and shading be the (n, 24) pack_shading array")
        if len(self.order):
            _check(lib().ae_bvh_pack_uvs(self._h, _ptr(uv), _ptr(shading)))
        return shading

    def pack_attributes(self, shading: np.ndarray, uvs, normals=None, colors=None) -> np.ndarray:
        """UVs, the UV-derived tangent frame and vertex colours (RGBA per
        vertex, (n, 3, 4) or (n, 12)) into the GPUTriangle array from
        pack_shading, as MeshData.cpp:172-239 packs them."""
        uv = np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        col = None if colors is None else np.ascontiguousarray(colors, np.float32).reshape(-1, 12)
        if self._verts is None or len(uv) != self.n_input or shading.shape != (len(self.order), 24) \
                or shading.dtype != np.float32 or not shading.flags.c_contiguous \
                or (nrm is not None and len(nrm) != self.n_input) or (col is not None and len(col) != self.n_input):
            raise ValueError("per-input-triangle uvs / normals / colors and the (n, 24) pack_shading array expected")
        if len(self.order):
            _check(lib().ae_bvh_pack_attributes(self._h, _ptr(self._verts), _ptr(nrm), _ptr(uv), _ptr(col),
                                                _ptr(shading)))
        return shading

    @property
    def nodes_f32(self) -> np.ndarray:
        return self.nodes.view(np.float32).reshape(-1, 16)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().ae_bvh_destroy(h)
            self._h = None


class _Texture(C.Structure):
    """ae_texture"""
    _fields_ = [("texels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32),
                ("row_pitch", C.c_uint32)]


TEX_R8_UNORM, TEX_RGBA8_UNORM, TEX_R32_FLOAT = 0, 1, 2
PASS_OPACITY_CHECK = 0x1


def _texture_format(a: np.ndarray) -> int:
    if a.dtype == np.uint8 and a.ndim == 2:
        return TEX_R8_UNORM
    if a.dtype == np.uint8 and a.ndim == 3 and a.shape[2] == 4:
        return TEX_RGBA8_UNORM
    if a.dtype == np.float32 and a.ndim == 2:
        return TEX_R32_FLOAT
    raise ValueError(f"unsupported texel array {a.dtype} {a.shape}: uint8 (h, w), uint8 (h, w, 4) or float32 (h, w)")


class Context:
    """Device context of the library (``ae_rt_ctx``)."""

    def __init__(self, device: int = 0, count_fetches: bool = False, blocks_per_sm: int = 0,
                 max_steps: int = 0, refill_steps: int = 0, threads_per_block: int = 0,
                 stack_entries_smem: int = 0, refill_below: int = 0, leaf_wait: int = 0,
                 near_ties: bool = True, staged_rays: bool = False, approximate: bool = False):
        cfg = Config()
        cfg.device = device
        cfg.blocks_per_sm = blocks_per_sm
        cfg.threads_per_block = threads_per_block
        cfg.stack_entries_smem = stack_entries_smem
        cfg.max_steps = max_steps
        cfg.flags = ((CFG_COUNT_FETCHES if count_fetches else 0) | (0 if near_ties else CFG_NO_NEAR_TIES)
                     | (CFG_STAGED_RAYS if staged_rays else 0) | (CFG_APPROXIMATE if approximate else 0))
        cfg.refill_steps = refill_steps
        cfg.refill_below = refill_below
        cfg.leaf_wait = leaf_wait
        h = C.c_void_p()
        _check(lib().ae_rt_ctx_create(C.byref(cfg), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ae_rt_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def upload_mesh(self, nodes, bvh_tris, shading=None) -> int:
        nodes = np.ascontiguousarray(nodes)
        bvh_tris = np.ascontiguousarray(bvh_tris, np.float32)
        n_nodes = nodes.nbytes // 64
        n_tris = bvh_tris.nbytes // 48
        mid = C.c_int32(-1)
        _check(lib().ae_rt_mesh_upload(self._h, _ptr(nodes) if n_nodes else None, n_nodes,
                                       _ptr(bvh_tris) if n_tris else None,
                                       _ptr(shading), n_tris, C.byref(mid)), self._h)
        return mid.value

    def trace_closest(self, mesh: int, rays, tmin: float, tmax: float, out=None, stream=None,
                      n_rays: int | None = None):
        """rays: PackedRay buffer (n, 12) float32 / 48-byte records.  Returns the
        hit buffer (HIT_DTYPE for host input)."""
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, HIT_DTYPE)
        _check(lib().ae_rt_trace_closest(self._h, mesh, _ptr(rays), n_rays, tmin, tmax, _ptr(out),
                                         _stream_handle(stream)), self._h)
        return out

    def build_mesh(self, verts, material=None, opacity=None, stream=None):
        """GPU BVH build of a triangle mesh (verts (n, 3, 3) float32, host or
        device); returns (mesh_id, order) with order[i] the input index of
        BVH-order triangle i (numpy)."""
        if isinstance(verts, np.ndarray):
            verts = np.ascontiguousarray(verts, np.float32)
            n = verts.size // 9
        else:
            n = verts.numel() // 9
        if material is not None and isinstance(material, np.ndarray):
            material = np.ascontiguousarray(material, np.int32)
        if opacity is not None and isinstance(opacity, np.ndarray):
            opacity = np.ascontiguousarray(opacity, np.float32)
        order = np.zeros(max(n, 2 if n == 1 else 0), np.uint32)
        mid = C.c_int32()
        _check(lib().ae_rt_mesh_build(self._h, _ptr(verts) if n else None, n, _ptr(material), _ptr(opacity),
                                      C.byref(mid), _ptr(order) if len(order) else None, _stream_handle(stream)),
               self._h)
        return mid.value, order

    def mesh_bvh(self, mesh: int):
        """(nodes NODE_DTYPE, bvh_tris (n, 12) float32) of a mesh of this context."""
        nn, nt = C.c_uint32(), C.c_uint32()
        _check(lib().ae_rt_mesh_get_bvh(self._h, mesh, None, None, C.byref(nn), C.byref(nt)), self._h)
        nodes = np.zeros(nn.value, NODE_DTYPE)
        tris = np.zeros((nt.value, 12), np.float32)
        _check(lib().ae_rt_mesh_get_bvh(self._h, mesh, _ptr(nodes) if nn.value else None,
                                        _ptr(tris) if nt.value else None, None, None), self._h)
        return nodes, tris

    def retest_near_ties(self, mesh: int, rays, hits, tmin: float, tmax: float, out, n_rays: int | None = None,
                         stream=None, count: bool = True):
        """FP64 re-test of the rays flagged HIT_FLAG_NEAR_TIE (device buffers:
        rays (n, 12) float32, hits (n, 8) float32, out (n, 8) float32 viewed
        as HIT64_DTYPE).  Returns the number of flagged rays (which waits for
        the stream), or None with count=False (asynchronous)."""
        if n_rays is None:
            n_rays = rays.numel() * rays.element_size() // 48
        cnt = C.c_uint32()
        _check(lib().ae_rt_retest_near_ties(self._h, mesh, _ptr(rays), _ptr(hits), n_rays, tmin, tmax, _ptr(out),
                                            C.byref(cnt) if count else None, _stream_handle(stream)), self._h)
        return cnt.value if count else None

    def trace_any(self, mesh: int, rays, tmin: float, tmax: float, out=None, stream=None,
                  n_rays: int | None = None):
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, np.uint8)
        _check(lib().ae_rt_trace_any(self._h, mesh, _ptr(rays), n_rays, tmin, tmax, _ptr(out),
                                     _stream_handle(stream)), self._h)
        return out

    # ---- two-level scene ----
    def scene_set(self, tlas_nodes, instances):
        tlas_nodes = np.ascontiguousarray(tlas_nodes)
        instances = np.ascontiguousarray(instances, INSTANCE_DTYPE)
        _check(lib().ae_rt_scene_set(self._h, _ptr(tlas_nodes) if tlas_nodes.size else None,
                                     tlas_nodes.nbytes // 64, _ptr(instances) if len(instances) else None,
                                     len(instances)), self._h)

    def scene_build(self, instances, world_aabbs):
        """RayTracingWorld-style top level; returns the input index of each
        ordered instance."""
        instances = np.ascontiguousarray(instances, INSTANCE_DTYPE)
        boxes = np.ascontiguousarray(world_aabbs, np.float32).reshape(-1, 6)
        order = np.zeros(len(instances) + 1, np.uint32)
        n = C.c_uint32()
        _check(lib().ae_rt_scene_build(self._h, _ptr(instances), _ptr(boxes), len(instances), _ptr(order),
                                       C.byref(n)), self._h)
        return order[:n.value]

    def trace_scene_closest(self, rays, tmin, tmax, cull_mask=0xFFFFFFFF, out=None, stream=None,
                            n_rays: int | None = None):
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, HIT_DTYPE)
        _check(lib().ae_rt_trace_scene_closest(self._h, _ptr(rays), n_rays, tmin, tmax, cull_mask, _ptr(out),
                                               _stream_handle(stream)), self._h)
        return out

    def trace_scene_any(self, rays, tmin, tmax, cull_mask=0xFFFFFFFF, out=None, stream=None,
                        n_rays: int | None = None):
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, np.uint8)
        _check(lib().ae_rt_trace_scene_any(self._h, _ptr(rays), n_rays, tmin, tmax, cull_mask, _ptr(out),
                                           _stream_handle(stream)), self._h)
        return out

    def trace_scene_closest_transparency(self, rays, tmin, tmax, cull_mask=0xFFFFFFFF, out=None, stream=None,
                                         n_rays: int | None = None):
        """HitClosestTransparency over the scene (hits with opacity > 0)."""
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, HIT_DTYPE)
        _check(lib().ae_rt_trace_scene_closest_transparency(self._h, _ptr(rays), n_rays, tmin, tmax, cull_mask,
                                                            _ptr(out), _stream_handle(stream)), self._h)
        return out

    def trace_scene_any_transparency(self, rays, tmin, tmax, cull_mask=0xFFFFFFFF, out=None, stream=None,
                                     n_rays: int | None = None):
        """HitAnyTransparency over the scene: transparency per ray (1 = clear)."""
        if n_rays is None:
            n_rays = (rays.nbytes if isinstance(rays, np.ndarray) else rays.numel() * rays.element_size()) // 48
        if out is None:
            out = np.zeros(n_rays, np.float32)
        _check(lib().ae_rt_trace_scene_any_transparency(self._h, _ptr(rays), n_rays, tmin, tmax, cull_mask,
                                                        _ptr(out), _stream_handle(stream)), self._h)
        return out

    def trace_scene_closest_queue(self, rays, count, capacity, tmin, tmax, hits, cull_mask=0xFFFFFFFF,
                                  stream=None):
        _check(lib().ae_rt_trace_scene_closest_queue(self._h, _ptr(rays), _ptr(count), capacity, tmin, tmax,
                                                     cull_mask, _ptr(hits), _stream_handle(stream)), self._h)

    def trace_scene_any_queue(self, rays, count, capacity, tmin, tmax, occluded, cull_mask=0xFFFFFFFF,
                              stream=None):
        _check(lib().ae_rt_trace_scene_any_queue(self._h, _ptr(rays), _ptr(count), capacity, tmin, tmax,
                                                 cull_mask, _ptr(occluded), _stream_handle(stream)), self._h)

    # ---- batched multi-mesh launches ----
    @staticmethod
    def _batch_table(batches):
        """batches: list of dicts {mesh, any, rays, out, n_rays, tmin, tmax}."""
        table = (BatchDesc * len(batches))()
        for i, b in enumerate(batches):
            table[i].mesh_id = b["mesh"]
            table[i].any = 1 if b["any"] else 0
            table[i].rays = _ptr(b["rays"])
            table[i].out = _ptr(b["out"])
            table[i].n_rays = b["n_rays"]
            table[i].tmin = b["tmin"]
            table[i].tmax = b["tmax"]
        return table

    def trace_batched(self, batches, stream=None):
        table = self._batch_table(batches)
        _check(lib().ae_rt_trace_batched(self._h, table, len(batches), _stream_handle(stream)), self._h)

    def batch_plan(self, batches) -> "BatchPlan":
        return BatchPlan(self, batches)

    # ---- wavefront stages (device buffers) ----
    def raygen(self, cam: "Camera", rays, stream=None):
        _check(lib().ae_rt_raygen(self._h, C.byref(cam), _ptr(rays), _stream_handle(stream)), self._h)

    def trace_closest_queue(self, mesh, rays, count, capacity, tmin, tmax, hits, stream=None):
        _check(lib().ae_rt_trace_closest_queue(self._h, mesh, _ptr(rays), _ptr(count), capacity, tmin, tmax,
                                               _ptr(hits), _stream_handle(stream)), self._h)

    def trace_any_queue(self, mesh, rays, count, capacity, tmin, tmax, occluded, stream=None):
        _check(lib().ae_rt_trace_any_queue(self._h, mesh, _ptr(rays), _ptr(count), capacity, tmin, tmax,
                                           _ptr(occluded), _stream_handle(stream)), self._h)

    def spawn_bounce(self, mesh, rays, hits, n, params: "BounceParams", secondary, shadow, counts,
                     count=None, stream=None):
        _check(lib().ae_rt_spawn_bounce(self._h, mesh, _ptr(rays), _ptr(hits), _ptr(count), n, C.byref(params),
                                        _ptr(secondary), _ptr(shadow), _ptr(counts), _stream_handle(stream)),
               self._h)

    def trace_camera_closest(self, mesh, cam: "Camera", hits, tmin=0.0, tmax=float("inf"), stream=None):
        """raygen + trace_closest of the camera's rays without a ray buffer."""
        _check(lib().ae_rt_trace_camera_closest(self._h, mesh, C.byref(cam), tmin, tmax, _ptr(hits),
                                                _stream_handle(stream)), self._h)

    def spawn_bounce_camera(self, mesh, cam: "Camera", hits, params: "BounceParams", secondary, shadow, counts,
                            stream=None):
        """spawn_bounce over the camera's width*height rays."""
        _check(lib().ae_rt_spawn_bounce_camera(self._h, mesh, C.byref(cam), _ptr(hits), C.byref(params),
                                               _ptr(secondary), _ptr(shadow), _ptr(counts),
                                               _stream_handle(stream)), self._h)

    def cast_pass(self, mesh, cam: "Camera", params: "BounceParams", primary_hits=None, secondary_rays=None,
                  secondary_hits=None, shadow_rays=None, shadow_occluded=None, stream=None):
        """One camera pass (primary, bounce and shadow rays).  Returns counts
        (primary, secondary, shadow)."""
        out = CastOutputs()
        out.primary_hits = _ptr(primary_hits)
        out.secondary_rays = _ptr(secondary_rays)
        out.secondary_hits = _ptr(secondary_hits)
        out.shadow_rays = _ptr(shadow_rays)
        out.shadow_occluded = _ptr(shadow_occluded)
        _check(lib().ae_rt_cast_pass(self._h, mesh, C.byref(cam), C.byref(params), C.byref(out),
                                     _stream_handle(stream)), self._h)
        return tuple(out.counts)

    # ---- path tracer ----
    def set_materials(self, materials):
        materials = np.ascontiguousarray(materials, MATERIAL_DTYPE)
        _check(lib().ae_rt_scene_set_materials(self._h, _ptr(materials) if len(materials) else None,
                                               len(materials)), self._h)

    def set_textures(self, textures):
        """The scene's texture table (ae_rt_scene_set_textures): a list of
        texel arrays, uint8 (h, w) = R8 UNORM, uint8 (h, w, 4) = RGBA8 UNORM,
        float32 (h, w) = R32 float; entry i is the materials' texture index i."""
        arrs = [np.ascontiguousarray(t) for t in textures]
        table = (_Texture * max(1, len(arrs)))()
        for i, t in enumerate(arrs):
            table[i].texels = t.ctypes.data
            table[i].height, table[i].width = t.shape[0], t.shape[1]
            table[i].format = _texture_format(t)
            table[i].row_pitch = 0
        _check(lib().ae_rt_scene_set_textures(self._h, table if arrs else None, len(arrs)), self._h)

    def set_environment(self, radiance):
        """ae_rt_scene_set_environment: the constant radiance the path tracer's misses see."""
        r = np.ascontiguousarray(radiance, np.float32).reshape(3)
        _check(lib().ae_rt_scene_set_environment(self._h, _ptr(r)), self._h)

    def set_lights(self, lights):
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 16)
        _check(lib().ae_rt_scene_set_lights(self._h, _ptr(lights) if len(lights) else None, len(lights)),
               self._h)

    @staticmethod
    def _pt_params(spp, max_bounces, sample_offset, seed, epsilon, mis, centered=False):
        p = PtParams()
        p.spp, p.max_bounces, p.sample_offset, p.seed, p.epsilon = spp, max_bounces, sample_offset, seed, epsilon
        p.flags = (PT_MIS if mis else 0) | (PT_CENTERED if centered else 0)
        return p

    def pathtrace(self, cam: "Camera", accum, accum64=None, spp=1, max_bounces=3, sample_offset=0, seed=1,
                  epsilon=0.1, mis=False, centered=False, tile=None, stream=None):
        """ae_rt_pathtrace (whole image) or, with tile = (x0, y0, w, h),
        ae_rt_pathtrace_tile: accumulates into the whole-image buffers."""
        p = self._pt_params(spp, max_bounces, sample_offset, seed, epsilon, mis, centered)
        if tile is None:
            st = lib().ae_rt_pathtrace(self._h, C.byref(cam), C.byref(p), _ptr(accum), _ptr(accum64),
                                       _stream_handle(stream))
        else:
            x0, y0, w, h = (int(v) for v in tile)
            st = lib().ae_rt_pathtrace_tile(self._h, C.byref(cam), C.byref(p), x0, y0, w, h, _ptr(accum),
                                            _ptr(accum64), _stream_handle(stream))
        _check(st, self._h)

    def pathtrace_realtime(self, cam: "Camera", frame_accum, max_radiance=0.0, spp=1, max_bounces=3,
                           sample_offset=0, seed=1, epsilon=0.1, mis=False, gbuffer=None, stream=None):
        """ae_rt_pathtrace_realtime: the engine's real-time accumulation into
        frame_accum, a (3, h, w) 32-bit device tensor (float bits at spp = 1,
        quantised unsigned sums at spp > 1).  gbuffer: a dict with any of the
        device planes depth / material_idx / normal / velocity and the
        matrices view / proj / pv_last (4 x 4) and last_matrices ((n, 3, 4))."""
        p = self._pt_params(spp, max_bounces, sample_offset, seed, epsilon, mis)
        rt = None
        keep = []
        if gbuffer is not None:
            rt = PtRealtime()
            for k in ("depth", "material_idx", "normal", "velocity"):
                setattr(rt, k, _ptr(gbuffer.get(k)))
            for k in ("view", "proj", "pv_last"):
                m = np.ascontiguousarray(gbuffer.get(k, np.eye(4)), np.float32).reshape(16)
                getattr(rt, k)[:] = m.tolist()
            if gbuffer.get("last_matrices") is not None:
                lm = np.ascontiguousarray(gbuffer["last_matrices"], np.float32).reshape(-1, 12)
                keep.append(lm)
                rt.last_matrices, rt.n_last_matrices = _ptr(lm), len(lm)
        _check(lib().ae_rt_pathtrace_realtime(self._h, C.byref(cam), C.byref(p),
                                              None if rt is None else C.byref(rt), _ptr(frame_accum), max_radiance,
                                              _stream_handle(stream)), self._h)

    def tonemap(self, accum, width: int, height: int, samples: int, exposure: float, gamma: float, out,
                stream=None):
        """ae_rt_pt_tonemap: the non-real-time output image into `out` (float4 per pixel)."""
        _check(lib().ae_rt_pt_tonemap(self._h, _ptr(accum), width, height, samples, exposure, gamma, _ptr(out),
                                      _stream_handle(stream)), self._h)

    # -- the traversal's other consumers (RTAO, reflections, RTGI, DDGI) ------

    @staticmethod
    def _gbuffer(gb: dict):
        """ae_gbuffer from a dict of device tensors: depth (h, w), normal
        (h, w, 2), optional offset (h, w) uint8, roughness (h, w), samples
        (h, w, 2), the blue-noise textures scrambling_ranking (128, 128, 4)
        and sobol_sequence (256, 4) uint8; ip_matrix / iv_matrix as 4x4
        row-major arrays (stored column-major, like GLSL); half_res."""
        g = GBuffer()
        depth = gb["depth"]
        g.height, g.width = int(depth.shape[0]), int(depth.shape[1])
        g.depth, g.normal = _ptr(depth), _ptr(gb["normal"])
        g.offset, g.roughness, g.samples = _ptr(gb.get("offset")), _ptr(gb.get("roughness")), _ptr(gb.get("samples"))
        g.half_res = int(gb.get("half_res", 0))
        for name in ("ip_matrix", "iv_matrix"):
            m = np.asarray(gb[name], np.float32).reshape(4, 4)
            getattr(g, name)[:] = list(m.T.reshape(-1))
        for name, shape in (("scrambling_ranking", (128, 128, 4)), ("sobol_sequence", (256, 4))):
            t = gb.get(name)
            if t is not None and tuple(t.shape) != shape:
                raise ValueError(f"{name} must have shape {shape}")
            setattr(g, name, _ptr(t))
        return g

    @staticmethod
    def _pass_params(radius=1.0, bias=0.0, roughness_cutoff=1.0, radiance_limit=10.0, environment=(0, 0, 0),
                     opacity_check=False, frame_seed=0, seed=1, texture_level=0):
        p = PassParams()
        p.texture_level = texture_level
        p.radius, p.bias, p.roughness_cutoff, p.radiance_limit = radius, bias, roughness_cutoff, radiance_limit
        p.environment[:] = [float(x) for x in environment]
        p.flags = PASS_OPACITY_CHECK if opacity_check else 0
        p.frame_seed, p.seed = frame_seed, seed
        return p

    def rtao(self, gbuffer: dict, out, stream=None, **params):
        """ae_rt_rtao: ambient occlusion per pixel into `out` (h, w) float32 (device)."""
        _check(lib().ae_rt_rtao(self._h, C.byref(self._gbuffer(gbuffer)), C.byref(self._pass_params(**params)),
                                _ptr(out), _stream_handle(stream)), self._h)

    def reflections(self, gbuffer: dict, out, stream=None, **params):
        """ae_rt_reflections: reflected radiance per pixel into `out` (h, w, 4) float32 (device)."""
        _check(lib().ae_rt_reflections(self._h, C.byref(self._gbuffer(gbuffer)),
                                       C.byref(self._pass_params(**params)), _ptr(out), _stream_handle(stream)),
               self._h)

    def rtgi(self, gbuffer: dict, out, stream=None, **params):
        """ae_rt_rtgi: one-bounce diffuse radiance per pixel into `out` (h, w, 4) float32 (device)."""
        _check(lib().ae_rt_rtgi(self._h, C.byref(self._gbuffer(gbuffer)), C.byref(self._pass_params(**params)),
                                _ptr(out), _stream_handle(stream)), self._h)

    def ddgi_trace(self, probes, ray_dirs, rotation, out, ray_dirs_inactive=None, inactive_ray_count=0,
                   stream=None, **params):
        """ae_rt_ddgi_trace: PackRayHit per probe ray into `out` (n_probes * ray_count, 4) float32 (device).
        probes (n, 4) float32 with the state's bits in w; ray_dirs (ray_count, 4); rotation 4x4 row-major."""
        d = DdgiProbes()
        d.probes, d.ray_dirs, d.ray_dirs_inactive = _ptr(probes), _ptr(ray_dirs), _ptr(ray_dirs_inactive)
        d.rotation[:] = list(np.asarray(rotation, np.float32).reshape(4, 4).T.reshape(-1))
        d.n_probes, d.ray_count, d.inactive_ray_count = int(probes.shape[0]), int(ray_dirs.shape[0]), inactive_ray_count
        _check(lib().ae_rt_ddgi_trace(self._h, C.byref(d), C.byref(self._pass_params(**params)), _ptr(out),
                                      _stream_handle(stream)), self._h)

    def synchronize(self, stream=None):
        _check(lib().ae_rt_synchronize(self._h, _stream_handle(stream)), self._h)

    def selftest_division(self, n: int, seed: int = 1) -> int:
        m = C.c_uint64()
        _check(lib().ae_rt_selftest_division(self._h, n, seed, C.byref(m)), self._h)
        return m.value

    def fetch_counts(self):
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib().ae_rt_get_fetch_counts(self._h, C.byref(a), C.byref(b)), self._h)
        return a.value, b.value


class BatchPlan:
    """ae_rt_batch_plan: a batched launch captured once in a CUDA graph."""

    def __init__(self, ctx: Context, batches):
        self.ctx = ctx
        table = Context._batch_table(batches)
        h = C.c_void_p()
        _check(lib().ae_rt_batch_plan_create(ctx.handle, table, len(batches), C.byref(h)), ctx.handle)
        self._h = h

    def launch(self, stream=None):
        _check(lib().ae_rt_batch_plan_launch(self._h, _stream_handle(stream)), self.ctx.handle)

    def close(self):
        if getattr(self, "_h", None):
            lib().ae_rt_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class RadianceCache:
    """ae_rc: the learned radiance cache bound to a context's scene."""

    def __init__(self, ctx: Context, aabb_min, aabb_max, log2_table=19, base_resolution=16, max_resolution=2048,
                 learning_rate=1e-2, beta1=0.9, beta2=0.99, epsilon=1e-15, seed=1, radiance_scale=1.0,
                 rough_cut=0.35, glossy_split=4, warp_mma_training=False):
        cfg = RcConfig()
        cfg.flags = 0x1 if warp_mma_training else 0
        cfg.radiance_scale = float(radiance_scale)
        cfg.rough_cut = float(rough_cut)
        cfg.glossy_split = int(glossy_split)
        cfg.log2_table, cfg.base_resolution, cfg.max_resolution = log2_table, base_resolution, max_resolution
        cfg.learning_rate, cfg.beta1, cfg.beta2, cfg.epsilon, cfg.seed = learning_rate, beta1, beta2, epsilon, seed
        for i in range(3):
            cfg.aabb_min[i] = float(aabb_min[i])
            cfg.aabb_max[i] = float(aabb_max[i])
        self.ctx = ctx
        self.cfg = cfg
        h = C.c_void_p()
        _check(lib().ae_rc_create(ctx.handle, C.byref(cfg), C.byref(h)), ctx.handle)
        self._h = h
        nm, ng = C.c_uint32(), C.c_uint64()
        _check(lib().ae_rc_param_counts(h, C.byref(nm), C.byref(ng)), ctx.handle)
        self.n_mlp, self.n_grid = nm.value, ng.value

    def close(self):
        if getattr(self, "_h", None):
            lib().ae_rc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def get_params(self):
        mlp = np.zeros(self.n_mlp, np.float32)
        grid = np.zeros(self.n_grid, np.float32)
        _check(lib().ae_rc_get_params(self._h, _ptr(mlp), _ptr(grid)), self.ctx.handle)
        return mlp, grid

    def set_params(self, mlp, grid):
        mlp = np.ascontiguousarray(mlp, np.float32)
        grid = np.ascontiguousarray(grid, np.float32)
        _check(lib().ae_rc_set_params(self._h, _ptr(mlp), _ptr(grid)), self.ctx.handle)

    def predict(self, queries, out, n=None, stream=None):
        n = len(queries) if n is None else n
        _check(lib().ae_rc_predict(self._h, _ptr(queries), n, _ptr(out), _stream_handle(stream)), self.ctx.handle)

    def gradients(self, samples, grad_mlp, grad_grid, n=None, stream=None):
        n = len(samples) if n is None else n
        loss = C.c_float()
        _check(lib().ae_rc_gradients(self._h, _ptr(samples), n, _ptr(grad_mlp), _ptr(grad_grid), C.byref(loss),
                                     _stream_handle(stream)), self.ctx.handle)
        return loss.value

    def train_batch(self, samples, n=None, stream=None):
        n = len(samples) if n is None else n
        loss = C.c_float()
        _check(lib().ae_rc_train_batch(self._h, _ptr(samples), n, C.byref(loss), _stream_handle(stream)),
               self.ctx.handle)
        return loss.value

    def train_frame(self, cam: Camera, frame: int, n_paths=65536, steps=4, max_bounces=3, want_loss=False,
                    stream=None):
        loss = C.c_float()
        _check(lib().ae_rc_train_frame(self._h, C.byref(cam), frame, n_paths, steps, max_bounces,
                                       C.byref(loss) if want_loss else None, _stream_handle(stream)),
               self.ctx.handle)
        return loss.value if want_loss else None

    def frame(self, cam: Camera, frame: int, accum, n_paths=65536, steps=2, max_bounces=3, last_bounce=2,
              want_loss=False, stream=None):
        """ae_rc_frame: render one sample per pixel with the current cache while
        the frame's training paths are traced beside it, then train."""
        loss = C.c_float()
        _check(lib().ae_rc_frame(self._h, C.byref(cam), frame, n_paths, steps, max_bounces, last_bounce, _ptr(accum),
                                 C.byref(loss) if want_loss else None, _stream_handle(stream)), self.ctx.handle)
        return loss.value if want_loss else None

    def selftest_wait_timeout(self) -> bool:
        """ae_rc_selftest_wait_timeout: True when the tensor-memory kernel's
        bounded wait ran out and was reported as a timeout."""
        t = C.c_uint32()
        _check(lib().ae_rc_selftest_wait_timeout(self._h, C.byref(t)), self.ctx.handle)
        return bool(t.value)

    def render(self, cam: Camera, frame: int, accum, last_bounce=2, stream=None):
        _check(lib().ae_rc_render(self._h, C.byref(cam), frame, last_bounce, _ptr(accum), _stream_handle(stream)),
               self.ctx.handle)


def make_camera(cam: dict) -> Camera:
    """ae_camera from the dict of scenes.pinhole_camera."""
    c = Camera()
    for name in ("location", "origin", "right", "bottom"):
        v = getattr(c, name)
        for i in range(3):
            v[i] = float(cam[name][i])
    c.width, c.height = cam["width"], cam["height"]
    j = cam.get("jitter", (0.5, 0.5))
    c.jitter[0], c.jitter[1] = j
    return c


def make_bounce_params(light_dir=(0.4, 1.0, 0.3), epsilon=0.1, seed=1) -> BounceParams:
    p = BounceParams()
    L = np.asarray(light_dir, np.float64)
    L = L / np.linalg.norm(L)
    for i in range(3):
        p.light_dir[i] = float(L[i])
    p.epsilon = epsilon
    p.seed = seed
    return p


def make_instance(model, mesh_id: int, mask: int = MASK_ALL | MASK_SHADOW, material_offset: int = 0):
    """GPUBVHInstance for an object-to-world affine `model` (3x4 or 4x4): the
    mat3x4 columns are the rows of the inverse model matrix
    (RayTracingWorld.cpp:100), computed in double and stored as float."""
    M = np.eye(4)
    m = np.asarray(model, np.float64)
    M[: m.shape[0], : m.shape[1]] = m
    inv = np.linalg.inv(M)
    rec = np.zeros((), INSTANCE_DTYPE)
    rec["inverseMatrix"] = inv[:3, :4].reshape(-1).astype(np.float32)
    rec["meshOffset"] = mesh_id
    rec["materialOffset"] = material_offset
    rec["nextInstance"] = -1
    rec["mask"] = mask
    return rec


def transform_aabb(lo, hi, model):
    """AABB::Transform (AABB.cpp:33-56): the box of the 8 transformed corners."""
    M = np.asarray(model, np.float64)
    corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])],
                       np.float64)
    w = corners @ M[:3, :3].T + M[:3, 3]
    return np.concatenate([w.min(0), w.max(0)]).astype(np.float32)


def mesh_bounds(bvh: "BVH"):
    """Root box of a mesh BVH: the union of the root's two child boxes."""
    if len(bvh.nodes) == 0:
        v = bvh._verts.reshape(-1, 3)
        return v.min(0), v.max(0)
    r = bvh.nodes[0]
    lo = np.minimum(r["leftMin"], r["rightMin"])
    hi = np.maximum(r["leftMax"], r["rightMax"])
    return lo, hi
