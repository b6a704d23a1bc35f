"""Generates the engine-asset fixtures in tests/golden/assets/ and their
expected decodings in tests/golden/assets_expected.npz.

The files follow the documents the engine writes (no file of the engine is
copied): a mesh is Mesh / MeshData / MeshSubData / DataComponent as
src/engine/mesh/MeshSerializer.cpp:7-156 and MeshSerializer.h:29-72 lay them
out, with nlohmann::json's sorted object keys, saved as MessagePack the way
Loader::MeshLoader::SaveMesh does with binaryJson = true
(src/engine/loader/MeshLoader.cpp:38-63), or as JSON text with byte arrays
(binaryJson = false, "binary": false); a material is the JSON text of
MeshSerializer.cpp:174-210.

The expected arrays are restated here with numpy, independently of the
library: MeshData::BuildBVH's triangle assembly (MeshData.cpp:89-155) and
RayTracingWorld::UpdateMaterials' GPUMaterial flattening
(RayTracingWorld.cpp:186-240, ColorConverter.h:18-23).

Needs the `msgpack` package (present where the fixtures are made, not on the
GPU host, which reads only the committed files):
    python tests/golden/gen_assets.py
"""
from __future__ import annotations

import json
from pathlib import Path

import msgpack
import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "assets"
F32 = np.float32

# ComponentFormat values (mesh/DataComponent.h:18-25) as the engine's files carry them
FMT_UINT, FMT_FLOAT, FMT_HALF, FMT_PACKED_NORMAL, FMT_PACKED_COLOR = 0, 2, 3, 4, 5


def component(arr, fmt, binary):
    raw = np.ascontiguousarray(arr).tobytes()
    return {"data": raw if binary else list(raw), "format": fmt}


def vec3(v):
    return {"x": float(v[0]), "y": float(v[1]), "z": float(v[2])}


def aabb(lo, hi):
    return {"max": vec3(hi), "min": vec3(lo)}


def sphere(center, radius, seg, rings):
    """UV sphere: positions, unit normals (w = 0), uvs, per-vertex colours, indices."""
    th = np.linspace(0, np.pi, rings + 1)
    ph = np.linspace(0, 2 * np.pi, seg + 1)
    T, Pp = np.meshgrid(th, ph, indexing="ij")
    n = np.stack([np.sin(T) * np.cos(Pp), np.cos(T), np.sin(T) * np.sin(Pp)], -1).reshape(-1, 3)
    pos = (np.asarray(center) + radius * n).astype(F32)
    nrm = np.concatenate([n, np.zeros((len(n), 1))], 1).astype(F32)
    uv = np.stack([Pp / (2 * np.pi), T / np.pi], -1).reshape(-1, 2).astype(F32)
    col = np.concatenate([0.5 + 0.5 * n, np.ones((len(n), 1))], 1).astype(F32)
    idx = []
    for r in range(rings):
        for s in range(seg):
            a, b = r * (seg + 1) + s, (r + 1) * (seg + 1) + s
            idx += [a, b, a + 1, a + 1, b, b + 1]
    return pos, nrm, uv, col, np.asarray(idx, np.uint32)


def mesh_doc(name, pos, nrm, uv, col, idx, subs, materials, binary, cull=True, invert_uvs=False):
    lo, hi = pos.min(0), pos.max(0)
    data = {
        "aabb": aabb(lo, hi),
        "binary": binary,
        "colors": component(col, FMT_PACKED_COLOR, binary),
        "indexCount": int(len(idx)),
        "indices": component(idx, FMT_UINT, binary),
        "materials": materials,
        "name": name,
        "normals": component(nrm, FMT_PACKED_NORMAL, binary),
        "primitiveType": 0,
        "radius": float(np.linalg.norm(hi - lo) * 0.5),
        "subData": [{"aabb": aabb((0, 0, 0), (0, 0, 0)), "indicesCount": c, "indicesOffset": o, "materialIdx": m,
                     "name": f"part{k}"} for k, (o, c, m) in enumerate(subs)],
        "tangents": component(np.zeros((0, 4), F32), FMT_PACKED_NORMAL, binary),
        "texCoords": component(uv, FMT_HALF, binary),
        "vertexCount": int(len(pos)),
        "vertices": component(pos, FMT_FLOAT, binary),
    }
    return {
        "allowedShadowCascades": 6, "castShadow": True, "cullBackFaces": cull, "data": data,
        "distanceCulling": 10000.0, "impostorDistance": 300.0, "impostorShadowDistance": 100.0,
        "invertUVs": invert_uvs, "mobility": 0, "name": name, "shadowDistanceCulling": 10000.0, "usage": 0,
        "vegetation": False, "windBendScale": 1.0, "windNoiseTextureLod": 2.0, "windWiggleScale": 1.0,
    }


MATERIALS = {
    "red": {"ao": 0.9, "baseColor": vec3((0.8, 0.1, 0.1)), "baseColorMapPath": "textures/checker.png",
            "displacementScale": 0.01, "emissiveColor": vec3((0, 0, 0)), "emissiveIntensity": 1.0, "metalness": 0.0,
            "name": "red", "normalScale": 0.5, "opacity": 1.0, "reflectance": 0.5, "roughness": 0.4, "tiling": 1.0,
            "transmissiveColor": vec3((0, 0, 0)), "twoSided": False, "uvChannel": 0, "vertexColors": True},
    "floor": {"ao": 1.0, "baseColor": vec3((0.5, 0.5, 0.5)), "displacementScale": 0.01,
              "emissiveColor": vec3((0.2, 0.1, 0.0)), "emissiveIntensity": 3.0, "metalness": 0.25, "name": "floor",
              "normalScale": 1.0, "opacity": 0.7, "opacityMapPath": "textures/leaf_mask.png",
              "normalMapPath": "textures/floor_normal.png", "reflectance": 0.5, "roughness": 0.8, "tiling": 2.0,
              "transmissiveColor": vec3((0, 0, 0)), "twoSided": True, "uvChannel": 0, "vertexColors": False},
}
MAP_KEYS = ["baseColorMapPath", "opacityMapPath", "normalMapPath", "roughnessMapPath", "metalnessMapPath",
            "aoMapPath"]


def expected_triangles(pos, nrm, uv, col, idx, subs, table):
    """MeshData.cpp:89-155 restated: triangle k over the sub-meshes in order
    reads indices 3k .. 3k + 2."""
    n = sum(c // 3 for _, c, _ in subs)
    tri_idx = idx[: 3 * n].reshape(n, 3)
    mat = np.concatenate([np.full(c // 3, m, np.int32) for _, c, m in subs])
    opa = np.where(table["opacityTexture"][mat] >= 0, F32(-1.0), table["opacity"][mat]).astype(F32)
    return {"verts": pos[tri_idx].reshape(n, 9), "normals": nrm[tri_idx][..., :3].reshape(n, 9),
            "uvs": uv[tri_idx].reshape(n, 6), "colors": col[tri_idx].reshape(n, 12), "material": mat,
            "opacity": opa}


def srgb_to_linear(c):
    """ColorConverter::ConvertSRGBToLinear (common/ColorConverter.h:18-23)."""
    x = np.asarray(c, F32).astype(np.float64)
    return (x ** np.float64(F32(2.2))).astype(F32)


def expected_material(doc, ids, cull, invert_uvs, mid):
    """RayTracingWorld.cpp:186-240 restated: pow(c, 2.2) of float32 inputs,
    rounded once to float32 (the engine's glm::pow calls the C library's
    powf, which rounds correctly; numpy's float32 power may not)."""
    base = srgb_to_linear([doc["baseColor"][k] for k in "xyz"])
    emis = srgb_to_linear([doc["emissiveColor"][k] for k in "xyz"]) * F32(doc["emissiveIntensity"])
    tex = [(ids[i] if (MAP_KEYS[i] in doc and ids[i] >= 0) else -1) for i in range(6)]
    return (mid, base, emis, doc["opacity"], doc["roughness"], doc["metalness"], doc["ao"], doc["reflectance"],
            doc["normalScale"], int(invert_uvs), int(doc["twoSided"]), int(cull), int(doc["vertexColors"]), *tex)


def main():
    import sys
    sys.path.insert(0, str(HERE.parent.parent / "atlas-engine_gb300"))
    from atlas_rt import MATERIAL_DTYPE

    (OUT / "meshes").mkdir(parents=True, exist_ok=True)
    (OUT / "materials").mkdir(parents=True, exist_ok=True)
    for name, doc in MATERIALS.items():
        (OUT / "materials" / f"{name}.aematerial").write_text(json.dumps(doc, sort_keys=True))

    # two sub-meshes: a UV sphere (material 0) and a floor quad (material 1)
    sp = sphere((0.0, 1.2, 0.0), 1.0, 16, 8)
    fl_pos = np.array([[-3, 0, -3], [3, 0, -3], [3, 0, 3], [-3, 0, 3]], F32)
    fl_nrm = np.tile(np.array([[0, 1, 0, 0]], F32), (4, 1))
    fl_uv = np.array([[0, 0], [2, 0], [2, 2], [0, 2]], F32)
    fl_col = np.ones((4, 4), F32)
    base = len(sp[0])
    fl_idx = np.array([0, 2, 1, 0, 3, 2], np.uint32) + base
    pos = np.concatenate([sp[0], fl_pos])
    nrm = np.concatenate([sp[1], fl_nrm])
    uv = np.concatenate([sp[2], fl_uv])
    col = np.concatenate([sp[3], fl_col])
    idx = np.concatenate([sp[4], fl_idx])
    subs = [(0, len(sp[4]), 0), (len(sp[4]), 6, 1)]
    mats = ["materials/red.aematerial", "materials/floor.aematerial"]
    doc = mesh_doc("two_part", pos, nrm, uv, col, idx, subs, mats, binary=True)
    (OUT / "meshes" / "two_part.aemesh").write_bytes(msgpack.packb(doc, use_bin_type=True))

    # a small JSON-text mesh (binaryJson = false): three triangles in two
    # sub-meshes, no normals or colours, inverted UVs, back faces not culled
    q_pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [2, 0, 1]], F32)
    q_uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [0.5, 0.5]], F32)
    q_idx = np.array([0, 1, 2, 0, 2, 3, 1, 4, 2], np.uint32)
    q_subs = [(0, 6, 0), (6, 3, 0)]
    qdoc = mesh_doc("quad_text", q_pos, np.zeros((0, 4), F32), q_uv, np.zeros((0, 4), F32), q_idx, q_subs,
                    ["materials/red.aematerial"], binary=False, cull=False, invert_uvs=True)
    (OUT / "meshes" / "quad_text.aemesh").write_text(json.dumps(qdoc))

    # expected decodings
    ids = {"red": [3, -1, -1, -1, -1, -1], "floor": [-1, 5, 6, -1, -1, -1]}
    table = np.zeros(2, MATERIAL_DTYPE)
    for i, name in enumerate(["red", "floor"]):
        table[i] = expected_material(MATERIALS[name], ids[name], True, False, i)
    q_table = np.zeros(1, MATERIAL_DTYPE)
    q_table[0] = expected_material(MATERIALS["red"], [-1] * 6, False, True, 0)
    out = {"two_part/table": table, "quad_text/table": q_table,
           "two_part/indices": idx, "two_part/vertices": pos, "two_part/normals": nrm, "two_part/texCoords": uv,
           "two_part/colors": col, "quad_text/indices": q_idx, "quad_text/vertices": q_pos,
           "quad_text/texCoords": q_uv}
    for k, v in expected_triangles(pos, nrm, uv, col, idx, subs, table).items():
        out[f"two_part/tri_{k}"] = v
    q_nrm = np.zeros((len(q_pos), 4), F32)
    q_col = np.ones((len(q_pos), 4), F32)
    for k, v in expected_triangles(q_pos, q_nrm, q_uv, q_col, q_idx, q_subs, q_table).items():
        out[f"quad_text/tri_{k}"] = v
    np.savez_compressed(HERE / "assets_expected.npz", **out)
    print("wrote", sorted(p.name for p in OUT.rglob("*") if p.is_file()))


if __name__ == "__main__":
    main()
