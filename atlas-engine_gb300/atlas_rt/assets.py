"""Engine assets into the library's buffers.

``MeshAsset`` reads a .aemesh file (Loader::MeshLoader::LoadMesh,
src/engine/loader/MeshLoader.cpp:6-36) and ``MaterialAsset`` a .aematerial
file (Material from_json, src/engine/mesh/MeshSerializer.cpp:212-256), both
through libatlas_rt.so's decoders.  ``build_mesh`` takes them the way
MeshData::BuildBVH (src/engine/mesh/MeshData.cpp:62-268) and
RayTracingWorld::UpdateMaterials (src/engine/raytracing/RayTracingWorld.cpp:171-240)
do: triangle assembly, the reference BVH build, GPUBVHTriangle and
GPUTriangle packing, GPUMaterial flattening.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from ._native import AeRtError, MeshAssetInfo, MeshSub, lib

MAP_SLOTS = ("baseColor", "opacity", "normal", "roughness", "metalness", "ao", "displacement")


def _raise(status: int):
    raw = lib().ae_asset_last_error()
    raise AeRtError(status, raw.decode() if raw else "")


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _load(loader_bytes, loader_file, source):
    h = C.c_void_p()
    if isinstance(source, (bytes, bytearray, memoryview)):
        buf = bytes(source)
        st = loader_bytes(buf, len(buf), C.byref(h))
    else:
        st = loader_file(str(Path(source)).encode(), C.byref(h))
    if st != 0:
        _raise(st)
    return h


class MeshAsset:
    """A decoded .aemesh document (MessagePack or JSON text), from a path or bytes."""

    def __init__(self, source):
        L = lib()
        self._h = _load(L.ae_mesh_asset_load, L.ae_mesh_asset_load_file, source)
        info = MeshAssetInfo()
        if (st := L.ae_mesh_asset_get_info(self._h, C.byref(info))) != 0:
            _raise(st)
        self.info = {k: (list(getattr(info, k)) if k == "aabb" else getattr(info, k)) for k, _ in info._fields_}
        self.name = L.ae_mesh_asset_name(self._h).decode()
        self.material_paths = [L.ae_mesh_asset_material_path(self._h, i).decode()
                                for i in range(info.material_count)]
        self.subs = []
        for i in range(info.sub_count):
            s = MeshSub()
            if (st := L.ae_mesh_asset_get_sub(self._h, i, C.byref(s))) != 0:
                _raise(st)
            self.subs.append({"indices_offset": s.indices_offset, "indices_count": s.indices_count,
                              "material_idx": s.material_idx, "aabb": list(s.aabb)})

    def arrays(self) -> dict:
        """The file's components: indices (u32), vertices (n, 3), texCoords (n, 2),
        normals / tangents / colors (n, 4), float32."""
        i = self.info
        out = {"indices": np.zeros(i["index_count"], np.uint32),
               "vertices": np.zeros((i["vertex_count"], 3), np.float32),
               "texCoords": np.zeros((i["tex_coord_count"], 2), np.float32),
               "normals": np.zeros((i["normal_count"], 4), np.float32),
               "tangents": np.zeros((i["tangent_count"], 4), np.float32),
               "colors": np.zeros((i["color_count"], 4), np.float32)}
        st = lib().ae_mesh_asset_get_arrays(self._h, *(_ptr(out[k]) for k in
                                                        ("indices", "vertices", "texCoords", "normals", "tangents",
                                                         "colors")))
        if st != 0:
            _raise(st)
        return out

    def triangles(self, materials: np.ndarray | None = None) -> dict:
        """MeshData::BuildBVH's per-triangle arrays (MeshData.cpp:89-155):
        verts (n, 9), normals (n, 9), uvs (n, 6), colors (n, 12), material,
        opacity.  `materials` is the mesh's GPUMaterial table (MATERIAL_DTYPE)."""
        n = self.info["triangle_count"]
        out = {"verts": np.zeros((n, 9), np.float32), "normals": np.zeros((n, 9), np.float32),
               "uvs": np.zeros((n, 6), np.float32), "colors": np.zeros((n, 12), np.float32),
               "material": np.zeros(n, np.int32), "opacity": np.zeros(n, np.float32)}
        m = None if materials is None else np.ascontiguousarray(materials)
        st = lib().ae_mesh_asset_triangles(self._h, _ptr(m), 0 if m is None else len(m),
                                           *(_ptr(out[k]) for k in ("verts", "normals", "uvs", "colors", "material",
                                                                    "opacity")))
        if st != 0:
            _raise(st)
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().ae_mesh_asset_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class MaterialAsset:
    """A decoded .aematerial document (JSON text), from a path or bytes."""

    def __init__(self, source):
        L = lib()
        self._h = _load(L.ae_material_asset_load, L.ae_material_asset_load_file, source)
        self.name = L.ae_material_asset_name(self._h).decode()
        self.maps = {k: L.ae_material_asset_map_path(self._h, i).decode() for i, k in enumerate(MAP_SLOTS)}

    def to_gpu(self, mesh: MeshAsset | None = None, texture_ids=None, material_id: int = 0) -> np.ndarray:
        """GPUMaterial (one MATERIAL_DTYPE record) as RayTracingWorld::UpdateMaterials fills it."""
        from . import MATERIAL_DTYPE
        out = np.zeros(1, MATERIAL_DTYPE)
        ids = None
        if texture_ids is not None:
            ids = np.full(6, -1, np.int32)
            for i, k in enumerate(MAP_SLOTS[:6]):
                if isinstance(texture_ids, dict):
                    ids[i] = texture_ids.get(k, -1)
                else:
                    ids[i] = texture_ids[i]
        st = lib().ae_material_asset_to_gpu(self._h, None if mesh is None else mesh._h, _ptr(ids), material_id,
                                            _ptr(out))
        if st != 0:
            _raise(st)
        return out[0]

    def close(self):
        if getattr(self, "_h", None):
            lib().ae_material_asset_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


@dataclass
class BuiltMesh:
    bvh: object              # atlas_rt.BVH
    bvh_triangles: np.ndarray
    shading: np.ndarray
    materials: np.ndarray
    triangles: dict


def build_mesh(mesh: MeshAsset, materials: list | None = None, material_root=None, texture_ids=None,
               parallel: bool = True) -> BuiltMesh:
    """The engine's path from a mesh file to the ray tracer's buffers: the
    materials (MaterialAsset objects, or loaded from the mesh's paths under
    `material_root`) flattened to GPUMaterial, the triangles assembled, the
    BVH built, GPUBVHTriangle and GPUTriangle (UVs, UV tangent frame,
    vertex colours) packed in BVH order.  texture_ids: per material, the
    ids handed to MaterialAsset.to_gpu."""
    from . import BVH, MATERIAL_DTYPE
    if materials is None and material_root is not None:
        materials = [MaterialAsset(Path(material_root) / p) for p in mesh.material_paths]
    table = None
    if materials:
        table = np.zeros(len(materials), MATERIAL_DTYPE)
        for i, m in enumerate(materials):
            table[i] = m.to_gpu(mesh, None if texture_ids is None else texture_ids[i], material_id=i)
    tri = mesh.triangles(table)
    bvh = BVH(tri["verts"], parallel=parallel)
    gt = bvh.pack_triangles(tri["material"], tri["opacity"])
    sh = bvh.pack_shading(tri["normals"] if mesh.info["normal_count"] else None, tri["material"], tri["opacity"])
    if mesh.info["tex_coord_count"] or mesh.info["color_count"]:
        sh = bvh.pack_attributes(sh, tri["uvs"], tri["normals"] if mesh.info["normal_count"] else None,
                                 tri["colors"] if mesh.info["color_count"] else None)
    return BuiltMesh(bvh, gt, sh, table if table is not None else np.zeros(0, MATERIAL_DTYPE), tri)
