"""Engine assets (.aemesh, .aematerial) through the library's decoders.

* The committed fixtures (tests/golden/gen_assets.py): components, sub-meshes,
  MeshData::BuildBVH's triangle assembly and RayTracingWorld's GPUMaterial
  flattening equal the numpy restatement bit for bit, for the MessagePack and
  the JSON-text form.
* Where the reference tree is present: its own engine assets
  (data/meshes/*.aemesh, data/materials/*.aematerial) decode to what an
  independent MessagePack decoder reads, and the BVH built from a real mesh's
  triangles equals the compiled reference builder's.
* Malformed documents (truncated, too deep, oversized counts, missing
  fields, out-of-range indices) are refused with a message, never read past.
* GPU: a mesh built from a fixture traces bit-identically to the shader
  traversal restatement.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle
from atlas_rt import BVH, AeRtError, scenes
from atlas_rt.assets import MaterialAsset, MeshAsset, build_mesh

GOLDEN = Path(__file__).resolve().parent / "golden"
ASSETS = GOLDEN / "assets"
REF_DATA = pyoracle.REFERENCE_ROOT / "data"
REAL_MESHES = ["metallicwall", "capsule", "chromesphere"]


def srgb_to_linear(c):
    """pow(c, 2.2) of float32 inputs rounded once to float32, as a correctly
    rounded powf gives it (ColorConverter.h:18-23)."""
    return (np.asarray(c, np.float32).astype(np.float64) ** np.float64(np.float32(2.2))).astype(np.float32)


@pytest.fixture(scope="module")
def expected():
    return np.load(GOLDEN / "assets_expected.npz")


TEX_IDS = {"red": [3, -1, -1, -1, -1, -1], "floor": [-1, 5, 6, -1, -1, -1]}


def fixture_materials():
    return [MaterialAsset(ASSETS / "materials" / f"{n}.aematerial") for n in ("red", "floor")]


def test_fixture_mesh_components(expected):
    m = MeshAsset(ASSETS / "meshes" / "two_part.aemesh")
    assert m.name == "two_part"
    assert m.material_paths == ["materials/red.aematerial", "materials/floor.aematerial"]
    assert m.info["cull_back_faces"] == 1 and m.info["invert_uvs"] == 0 and m.info["tangent_count"] == 0
    a = m.arrays()
    for k in ("indices", "vertices", "normals", "texCoords", "colors"):
        assert np.array_equal(a[k], expected[f"two_part/{k}"]), k
    assert [s["material_idx"] for s in m.subs] == [0, 1]
    assert m.subs[0]["indices_offset"] == 0 and m.subs[1]["indices_count"] == 6
    assert m.info["triangle_count"] == len(expected["two_part/tri_verts"])


@pytest.mark.parametrize("name", ["two_part", "quad_text"])
def test_triangle_assembly_and_materials(expected, name):
    m = MeshAsset(ASSETS / "meshes" / f"{name}.aemesh")
    mats = fixture_materials() if name == "two_part" else fixture_materials()[:1]
    ids = [TEX_IDS["red"], TEX_IDS["floor"]] if name == "two_part" else [[-1] * 6]
    table = np.zeros(len(mats), expected[f"{name}/table"].dtype)
    for i, mat in enumerate(mats):
        table[i] = mat.to_gpu(m, ids[i], material_id=i)
    assert table.tobytes() == expected[f"{name}/table"].tobytes()
    t = m.triangles(table)
    for k in ("verts", "normals", "uvs", "colors", "material", "opacity"):
        assert t[k].tobytes() == expected[f"{name}/tri_{k}"].tobytes(), k


def test_json_text_mesh():
    m = MeshAsset(ASSETS / "meshes" / "quad_text.aemesh")
    assert m.info["normal_count"] == 0 and m.info["color_count"] == 0
    assert m.info["cull_back_faces"] == 0 and m.info["invert_uvs"] == 1
    assert m.info["triangle_count"] == 3 and len(m.subs) == 2
    # the same document as MessagePack decodes identically
    msgpack = pytest.importorskip("msgpack")
    doc = json.loads((ASSETS / "meshes" / "quad_text.aemesh").read_text())
    for k in ("indices", "vertices", "texCoords", "normals", "tangents", "colors"):
        doc["data"][k]["data"] = bytes(doc["data"][k]["data"])
    doc["data"]["binary"] = True
    m2 = MeshAsset(msgpack.packb(doc, use_bin_type=True))
    a, b = m.arrays(), m2.arrays()
    assert all(np.array_equal(a[k], b[k]) for k in a)
    assert m.triangles()["verts"].tobytes() == m2.triangles()["verts"].tobytes()


def test_material_maps_and_flags():
    red, floor = fixture_materials()
    assert red.maps["baseColor"] == "textures/checker.png" and red.maps["opacity"] == ""
    assert floor.maps["opacity"] == "textures/leaf_mask.png" and floor.maps["normal"] == "textures/floor_normal.png"
    g = floor.to_gpu(None)
    # no mesh: invertUVs / cullBackFaces 0; no texture ids: every slot -1
    assert g["cullBackFaces"] == 0 and g["invertUVs"] == 0 and g["twoSided"] == 1
    assert all(g[k] == -1 for k in ("baseColorTexture", "opacityTexture", "normalTexture"))
    # an id given for a slot the material has no map in stays -1
    g = red.to_gpu(None, [3, 4, 4, 4, 4, 4])
    assert g["baseColorTexture"] == 3 and g["opacityTexture"] == -1 and g["aoTexture"] == -1


def test_build_mesh_packs_in_bvh_order():
    m = MeshAsset(ASSETS / "meshes" / "two_part.aemesh")
    built = build_mesh(m, material_root=ASSETS, texture_ids=[TEX_IDS["red"], TEX_IDS["floor"]])
    order = built.bvh.order
    t = built.triangles
    assert np.array_equal(built.bvh_triangles[:, 7].view(np.int32), t["material"][order])
    assert np.array_equal(built.bvh_triangles[:, 11], t["opacity"][order])
    assert np.all(t["opacity"][t["material"] == 1] == -1.0)       # floor: opacity texture
    assert built.shading.shape == (len(order), 24)
    # the UVs went into d0 as half floats: the first vertex's u of the first triangle
    u0 = np.frombuffer(built.shading[0, 12:13].tobytes(), np.float16)[0]
    assert u0 == np.float16(t["uvs"][order[0], 0])


# ---------------------------------------------------------------------------
# The reference's own assets
# ---------------------------------------------------------------------------

real = pytest.mark.skipif(not (REF_DATA / "meshes" / "capsule.aemesh").exists(),
                          reason="reference tree not present on this host")


@real
@pytest.mark.parametrize("name", REAL_MESHES)
def test_real_engine_mesh_matches_independent_decoder(name):
    msgpack = pytest.importorskip("msgpack")
    path = REF_DATA / "meshes" / f"{name}.aemesh"
    doc = msgpack.unpackb(path.read_bytes(), raw=False)
    d = doc["data"]
    m = MeshAsset(path)
    assert m.name == doc["name"] and m.material_paths == d.get("materials", [])
    a = m.arrays()
    widths = {"indices": (np.uint32, 1), "vertices": (np.float32, 3), "texCoords": (np.float32, 2),
              "normals": (np.float32, 4), "tangents": (np.float32, 4), "colors": (np.float32, 4)}
    for k, (dt, w) in widths.items():
        want = np.frombuffer(d[k]["data"], dt).reshape(-1, w) if w > 1 else np.frombuffer(d[k]["data"], dt)
        assert np.array_equal(a[k], want), k
    assert m.info["cull_back_faces"] == int(doc["cullBackFaces"])
    assert m.info["radius"] == np.float32(d["radius"])
    # the triangle assembly of MeshData.cpp:89-155 over the real buffers
    t = m.triangles()
    n = sum(s["indicesCount"] // 3 for s in d["subData"])
    tri = a["indices"][: 3 * n].reshape(n, 3)
    assert np.array_equal(t["verts"], a["vertices"][tri].reshape(n, 9))
    assert np.array_equal(t["normals"], a["normals"][tri][..., :3].reshape(n, 9))
    assert np.array_equal(t["uvs"], a["texCoords"][tri].reshape(n, 6))


@real
@pytest.mark.parametrize("name", REAL_MESHES)
def test_real_engine_mesh_bvh_matches_reference_builder(name):
    if not pyoracle.ref_available():
        pytest.skip("compiled reference not available")
    t = MeshAsset(REF_DATA / "meshes" / f"{name}.aemesh").triangles()
    r = pyoracle.RefBVH(t["verts"])
    b = BVH(t["verts"])
    assert np.array_equal(b.nodes_f32.view(np.uint32), r.nodes_f32.view(np.uint32))
    assert np.array_equal(b.order, r.order) and np.array_equal(b.end_of_node, r.end_of_node)


@real
def test_real_engine_materials():
    """Every material the real meshes name, flattened as RayTracingWorld.cpp:186-240 does."""
    for name in REAL_MESHES:
        mesh = MeshAsset(REF_DATA / "meshes" / f"{name}.aemesh")
        for p in mesh.material_paths:
            path = REF_DATA / p
            doc = json.loads(path.read_text())
            g = MaterialAsset(path).to_gpu(mesh)
            base = srgb_to_linear([doc["baseColor"][k] for k in "xyz"])
            emis = srgb_to_linear([doc["emissiveColor"][k] for k in "xyz"]) * np.float32(doc["emissiveIntensity"])
            assert np.array_equal(g["baseColor"], base) and np.array_equal(g["emissiveColor"], emis)
            assert g["roughness"] == np.float32(doc["roughness"]) and g["metalness"] == np.float32(doc["metalness"])
            assert g["twoSided"] == int(doc["twoSided"]) and g["cullBackFaces"] == mesh.info["cull_back_faces"]


# ---------------------------------------------------------------------------
# Malformed input
# ---------------------------------------------------------------------------

def refused(source, fragment=""):
    with pytest.raises(AeRtError) as e:
        MeshAsset(source)
    assert e.value.status == 1 and fragment in str(e.value)


def test_truncated_documents_are_refused():
    data = (ASSETS / "meshes" / "two_part.aemesh").read_bytes()
    for n in list(range(0, 64)) + list(range(64, len(data), 97)):
        refused(data[:n])
    text = (ASSETS / "meshes" / "quad_text.aemesh").read_bytes()
    for n in range(1, len(text), 53):
        refused(text[:n])


def test_hostile_documents_are_refused():
    refused(b"\x91" * 200 + b"\xc0", "nested too deeply")
    refused(b"\xdd\xff\xff\xff\xff\x00", "truncated")                 # a 4-billion-element array in 6 bytes
    refused(b"\xdf\xff\xff\xff\xff", "truncated")
    refused(b"\xc6\xff\xff\xff\xff\x00", "truncated")                 # a 4 GB binary blob
    refused(b"[" * 500 + b"]" * 500, "")
    refused(b'{"a":' + b"[" * 100 + b"]" * 100 + b"}", "nested too deeply")
    refused(b"\x80\x00", "trailing")
    doc = json.loads((ASSETS / "meshes" / "quad_text.aemesh").read_text())
    del doc["data"]["vertexCount"]
    refused(json.dumps(doc).encode(), "vertexCount")
    doc = json.loads((ASSETS / "meshes" / "quad_text.aemesh").read_text())
    doc["data"]["vertices"]["data"] = doc["data"]["vertices"]["data"][:-1]
    refused(json.dumps(doc).encode(), "whole number")
    with pytest.raises(AeRtError):
        MeshAsset(ASSETS / "meshes" / "no_such_file.aemesh")
    with pytest.raises(AeRtError):
        MaterialAsset(b'{"name": "x"}')


def test_out_of_range_indices_are_refused_before_writing():
    doc = json.loads((ASSETS / "meshes" / "quad_text.aemesh").read_text())
    idx = np.frombuffer(bytes(doc["data"]["indices"]["data"]), np.uint32).copy()
    idx[4] = 5                                                        # one past the five vertices
    doc["data"]["indices"]["data"] = list(idx.tobytes())
    m = MeshAsset(json.dumps(doc).encode())
    with pytest.raises(AeRtError, match="out of range"):
        m.triangles()
    doc["data"]["subData"][1]["indicesCount"] = 30                    # more triangles than indices
    with pytest.raises(AeRtError, match="index buffer"):
        MeshAsset(json.dumps(doc).encode()).triangles()


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
def test_asset_mesh_traces_like_the_shader_restatement(ctx):
    m = MeshAsset(ASSETS / "meshes" / "two_part.aemesh")
    built = build_mesh(m, material_root=ASSETS)
    mid = ctx.upload_mesh(built.bvh.nodes, built.bvh_triangles, built.shading)
    rng = np.random.default_rng(5)
    n = 20000
    o = np.tile(np.array([[0.3, 2.0, 4.0]], np.float32), (n, 1))
    target = rng.uniform([-2.8, 0.0, -2.8], [2.8, 0.0, 2.8], (n, 3)).astype(np.float32)    # points on the floor
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays8 = scenes.rays8(o, d.astype(np.float32), 1e-3, 100.0)
    pr = scenes.pack_rays(o, d.astype(np.float32))
    hits = ctx.trace_closest(mid, pr, 1e-3, 100.0)
    occ = ctx.trace_any(mid, pr, 1e-3, 100.0)
    ptr, tuv = pyoracle.closest_glsl(built.bvh.nodes_f32, built.bvh_triangles, rays8)
    assert (ptr >= 0).mean() > 0.8
    assert np.array_equal(hits["triPtr"], ptr)
    assert np.array_equal(hits["t"].view(np.uint32), tuv[:, 0].view(np.uint32))
    assert np.array_equal(occ, pyoracle.any_glsl(built.bvh.nodes_f32, built.bvh_triangles, rays8))
    # the material of the hit triangle: the sphere (0) or the floor (1)
    mat = built.bvh_triangles[np.maximum(ptr, 0), 7].view(np.int32)
    assert set(np.unique(mat[ptr >= 0]).tolist()) == {0, 1}
