/*
 * atlas_rt.h -- C ABI of the GB300 ray-tracing library for Atlas Engine.
 *
 * Drop-in boundary for the engine's software ray-tracing path: the host BVH
 * builder and ray query (src/engine/volume/BVH.h:114-138), the GPU buffer
 * layouts the engine uploads (src/engine/raytracing/RTStructures.h:14-110),
 * and the traversal / path-tracing dispatches that the engine records today
 * as Vulkan compute shaders (data/shader/raytracer/bvh.hsh,
 * src/engine/renderer/helper/RayTracingHelper.cpp).
 *
 * Conventions
 *  - Every struct below is byte-identical to the engine's struct of the same
 *    role; the engine's host arrays can be passed without repacking.
 *  - Every call returns ae_rt_status; no C++ exception crosses this boundary.
 *  - Buffer arguments of trace calls may live in host memory (pageable or
 *    pinned) or in device memory of the context's GPU.  With device buffers a
 *    call is asynchronous on `stream` (a cudaStream_t, NULL = the legacy
 *    default stream); with host buffers it returns after the results have
 *    been copied back.
 *  - One context is driven by one host thread at a time; independent
 *    contexts may be used concurrently.
 */
#ifndef ATLAS_RT_H
#define ATLAS_RT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AE_RT_ABI_VERSION 1

typedef enum ae_rt_status {
    AE_RT_OK = 0,
    AE_RT_INVALID_ARG = 1,      /* null pointer, bad id, size out of range */
    AE_RT_BAD_BVH = 2,          /* the BVH validator rejected an upload */
    AE_RT_OUT_OF_MEMORY = 3,
    AE_RT_CUDA_ERROR = 4,       /* a CUDA call failed; see ae_rt_last_error */
    AE_RT_TIMEOUT = 5,          /* a bounded device wait gave up */
    AE_RT_STACK_OVERFLOW = 6,   /* a ray needed more traversal stack than its launch holds
                                   (trees deeper than 1,024 levels; batched launches: 128) */
    AE_RT_ITERATION_LIMIT = 7,  /* a ray exceeded the traversal step cap (cyclic BVH?) */
    AE_RT_NO_DEVICE = 8,
    AE_RT_NOT_BUILT = 9         /* the library was built without the requested feature */
} ae_rt_status;

/* ------------------------------------------------------------------------ */
/* Engine buffer layouts                                                     */
/* ------------------------------------------------------------------------ */

/* GPUAABB (RTStructures.h:80-83) */
typedef struct ae_aabb {
    float min[3];
    float max[3];
} ae_aabb;

/* GPUBVHNode (RTStructures.h:95-103).  Pointer >= 0: inner node index;
 * pointer < 0: leaf, ~pointer = first triangle (BLAS) or instance (TLAS). */
typedef struct ae_bvh_node {
    ae_aabb leftAABB;
    ae_aabb rightAABB;
    int32_t leftPtr;
    int32_t rightPtr;
    int32_t padding0;
    int32_t padding1;
} ae_bvh_node;

/* GPUBVHTriangle (RTStructures.h:23-27), packed by MeshData.cpp:241-248:
 * v0.w > 0 marks the last triangle of a leaf, v1.w = material index bits,
 * v2.w = opacity (-1: opacity texture). */
typedef struct ae_bvh_triangle {
    float v0[4];
    float v1[4];
    float v2[4];
} ae_bvh_triangle;

/* GPUTriangle (RTStructures.h:14-21), packed by MeshData.cpp:172-239:
 * v*.w = 10:10:10:2 normal bits, d0 = half2 UVs x3 + material index bits,
 * d1 = tangent, bitangent, endOfNode (+1/-1), 0; d2 = unorm4x8 colours x3 + opacity. */
typedef struct ae_triangle {
    float v0[4];
    float v1[4];
    float v2[4];
    float d0[4];
    float d1[4];
    float d2[4];
} ae_triangle;

/* GPUBVHInstance (RTStructures.h:85-93): mat3x4 (three vec4 columns) holding
 * the transposed inverse model matrix, so that
 * objectPos[i] = dot(vec4(worldPos, 1), inverseMatrix[i]). */
typedef struct ae_bvh_instance {
    float inverseMatrix[12];
    int32_t meshOffset;
    int32_t materialOffset;
    int32_t nextInstance;
    uint32_t mask;
} ae_bvh_instance;

/* GPUMaterial (RTStructures.h:51-78) */
typedef struct ae_material {
    int32_t ID;
    float baseColor[3];
    float emissiveColor[3];
    float opacity;
    float roughness;
    float metalness;
    float ao;
    float reflectance;
    float normalScale;
    int32_t invertUVs;
    int32_t twoSided;
    int32_t cullBackFaces;
    int32_t useVertexColors;
    int32_t baseColorTexture;
    int32_t opacityTexture;
    int32_t normalTexture;
    int32_t roughnessTexture;
    int32_t metalnessTexture;
    int32_t aoTexture;
} ae_material;

/* GPULight (RTStructures.h:105-110): data.x = (type << 28) | triangle index
 * bits, data.y = selection weight, data.z = area, data.w = instance bits. */
typedef struct ae_light {
    float P[4];
    float N[4];
    float color[4];
    float data[4];
} ae_light;

/* PackedRay (data/shader/raytracer/structures.hsh:9-13): origin.w = ray ID
 * bits; hit = (t, hitID bits, instance bits, unused). */
typedef struct ae_packed_ray {
    float origin[4];
    float direction[4];
    float hit[4];
} ae_packed_ray;

/* Instance cull masks (RTStructures.h:9-12, common.hsh:14-15) */
#define AE_RT_MASK_ALL    (1u << 7)
#define AE_RT_MASK_SHADOW (1u << 6)

/* Result of a closest-hit query.  triPtr is the BVH-order triangle index the
 * shader writes as ray.hitID (bvh.hsh:65); u, v are the barycentric weights
 * of v1 and v2 (surface.hsh:80-88), which the shader re-derives at shading
 * time.  tSecond is the second-smallest accepted t the traversal met (used to
 * flag near ties). */
typedef struct ae_hit {
    float t;
    int32_t triPtr;       /* -1: miss */
    int32_t instance;     /* -1: miss or single-mesh query */
    uint32_t flags;       /* AE_HIT_* */
    float u;
    float v;
    float tSecond;
    int32_t reserved;
} ae_hit;

#define AE_HIT_HIT       0x1u
#define AE_HIT_NEAR_TIE  0x2u  /* the nearest triangle may be decided by FP32 rounding: set on
                                  every ray whose two nearest hits lie within 1e-6 relative t
                                  (a superset: a second hit within 4e-6, a box or triangle
                                  rejected within rounding of the window; misses included);
                                  ae_rt_retest_near_ties decides them in double */
#define AE_HIT_OVERFLOW  0x4u  /* traversal stack overflowed; result invalid */
#define AE_HIT_ITER_CAP  0x8u  /* traversal step cap hit; result invalid */
#define AE_HIT_RETESTED  0x10u /* ae_hit_f64 only: the double-precision re-test decided it */

/* ------------------------------------------------------------------------ */
/* Host BVH builder -- replaces Volume::BVH::BVH (BVH.cpp:14, :58)           */
/* ------------------------------------------------------------------------ */

typedef struct ae_bvh ae_bvh;

/* Triangle BVH.  verts: n * 9 floats (v0, v1, v2).  aabbs: optional n * 6
 * floats (min, max); when NULL each is the triangle's vertex bound, as
 * MeshData::BuildBVH forms it (MeshData.cpp:143-146).  parallel != 0 builds
 * sub-trees on worker threads (the result is identical).  An empty input gives
 * an empty BVH (the reference dereferences a missing child there).
 * Replaces Volume::BVH::BVH(aabbs, data, parallelBuild)  BVH.cpp:14-56. */
ae_rt_status ae_bvh_build_triangles(const float* verts, const float* aabbs, uint32_t n,
                                    int parallel, ae_bvh** out);

/* AABB-only BVH (the top level over instances, 64 bins).
 * Replaces Volume::BVH::BVH(aabbs, parallelBuild)  BVH.cpp:58-100. */
ae_rt_status ae_bvh_build_aabbs(const float* aabbs, uint32_t n, int parallel, ae_bvh** out);

void ae_bvh_destroy(ae_bvh* bvh);

/* Sizes of BVH::nodes and BVH::data / BVH::refs (BVH.h:133-137). */
uint32_t ae_bvh_node_count(const ae_bvh* bvh);
uint32_t ae_bvh_primitive_count(const ae_bvh* bvh);

/* Nodes in the GPUBVHNode layout, as MeshData.cpp:256-268 copies them. */
ae_rt_status ae_bvh_get_nodes(const ae_bvh* bvh, ae_bvh_node* out);

/* Flattened primitive order: order[i] = input index of primitive i
 * (BVHTriangle::idx / Ref::idx), end_of_node[i] = leaf terminator flag. */
ae_rt_status ae_bvh_get_order(const ae_bvh* bvh, uint32_t* order, uint8_t* end_of_node);

/* GPUBVHTriangle packing in BVH order (MeshData.cpp:241-248).  material and
 * opacity are per input triangle and optional (0 and 1.0). */
ae_rt_status ae_bvh_pack_triangles(const ae_bvh* bvh, const float* verts, const int32_t* material,
                                   const float* opacity, ae_bvh_triangle* out);

/* GPUTriangle packing in BVH order (MeshData.cpp:172-239) for meshes without
 * texture coordinates or vertex colours: normals (n * 9 floats, per vertex;
 * NULL = face normals) normalised and packed 10:10:10:2, UVs 0, colours
 * white, tangent frame from the first edge; material and opacity per input
 * triangle (optional: 0, 1.0). */
ae_rt_status ae_bvh_pack_shading(const ae_bvh* bvh, const float* verts, const float* normals,
                                 const int32_t* material, const float* opacity, ae_triangle* out);

/* Texture coordinates into GPUTriangle d0.xyz (MeshData.cpp:172-239:
 * packHalf2x16 of the three vertices' UVs, round to nearest even): uvs is
 * n * 6 floats per input triangle (u0, v0, u1, v1, u2, v2), `inout` the
 * GPUTriangle array in BVH order that ae_bvh_pack_shading filled. */
ae_rt_status ae_bvh_pack_uvs(const ae_bvh* bvh, const float* uvs, ae_triangle* inout);

/* The rest of MeshData's GPUTriangle packing (MeshData.cpp:172-239) for
 * meshes with texture coordinates: UVs into d0.xyz as ae_bvh_pack_uvs; the
 * tangent frame from the UVs into d1.xy (tangent = the UV-space s direction
 * made orthogonal to the normalised vertex-normal sum, bitangent = +-
 * normalize(cross(tangent, normal)) by the handedness of the t direction,
 * both packed 10:10:10:2); vertex colours (optional, n * 12 floats, RGBA per
 * vertex) into d2.xyz as packUnorm4x8.  normals: n * 9 floats per vertex, or
 * NULL for the face normal.  `inout` is the GPUTriangle array in BVH order
 * that ae_bvh_pack_shading filled. */
ae_rt_status ae_bvh_pack_attributes(const ae_bvh* bvh, const float* verts, const float* normals, const float* uvs,
                                    const float* colors, ae_triangle* inout);

/* ------------------------------------------------------------------------ */
/* Engine assets: .aemesh and .aematerial                                    */
/* ------------------------------------------------------------------------ */

/* A mesh file as Loader::MeshLoader::LoadMesh reads it
 * (src/engine/loader/MeshLoader.cpp:6-36; layout MeshSerializer.cpp:7-134):
 * the MessagePack document the engine's importer saves (binaryJson = true)
 * or the same document as JSON text.  Per-vertex components keep their file
 * form: vertices 3 floats, texCoords 2, normals / tangents / colors 4. */
typedef struct ae_mesh_asset ae_mesh_asset;

typedef struct ae_mesh_asset_info {
    uint32_t vertex_count;     /* elements of each component actually present */
    uint32_t index_count;
    uint32_t triangle_count;   /* sum over sub-meshes of indicesCount / 3 (MeshData.cpp:91-93) */
    uint32_t sub_count;
    uint32_t material_count;   /* material paths in the file */
    uint32_t tex_coord_count;
    uint32_t normal_count;
    uint32_t tangent_count;
    uint32_t color_count;
    int32_t cull_back_faces;   /* Mesh::cullBackFaces */
    int32_t invert_uvs;        /* Mesh::invertUVs */
    int32_t cast_shadow;
    int32_t primitive_type;
    int32_t mobility;
    int32_t usage;
    float radius;
    float aabb[6];             /* min, max */
} ae_mesh_asset_info;

/* MeshSubData (MeshSerializer.cpp:136-156) */
typedef struct ae_mesh_sub {
    uint32_t indices_offset;
    uint32_t indices_count;
    int32_t material_idx;
    float aabb[6];
} ae_mesh_sub;

/* Message of the last failed asset call on this thread ("" when none). */
const char* ae_asset_last_error(void);

/* Decodes a mesh document (size bytes, MessagePack or JSON text).  A
 * malformed, truncated or incomplete document is AE_RT_INVALID_ARG with a
 * message; the reference throws from nlohmann::json there. */
ae_rt_status ae_mesh_asset_load(const void* bytes, size_t size, ae_mesh_asset** out);
ae_rt_status ae_mesh_asset_load_file(const char* path, ae_mesh_asset** out);
void ae_mesh_asset_destroy(ae_mesh_asset* asset);
ae_rt_status ae_mesh_asset_get_info(const ae_mesh_asset* asset, ae_mesh_asset_info* info);
const char* ae_mesh_asset_name(const ae_mesh_asset* asset);
/* The i-th material path (MeshSerializer.cpp:89-93), NULL past the end. */
const char* ae_mesh_asset_material_path(const ae_mesh_asset* asset, uint32_t i);
ae_rt_status ae_mesh_asset_get_sub(const ae_mesh_asset* asset, uint32_t i, ae_mesh_sub* out);
/* Copies the components out (any pointer may be NULL); sizes from
 * ae_mesh_asset_info. */
ae_rt_status ae_mesh_asset_get_arrays(const ae_mesh_asset* asset, uint32_t* indices, float* vertices,
                                      float* tex_coords, float* normals, float* tangents, float* colors);

/* MeshData::BuildBVH's triangle assembly (MeshData.cpp:89-155): triangle k
 * (counted over the sub-meshes in order) takes indices 3k .. 3k + 2; per
 * triangle verts (9 floats), normals (9: the file's xyz, which the shading
 * packer normalises; engine files store w = 0), uvs (6; 0 without
 * texCoords), colors (12; 1.0 without colors), material (the sub-mesh's
 * materialIdx) and opacity (-1 where materials[materialIdx] has an opacity
 * texture, else its opacity; 1.0 with no material table).  Every index is
 * checked against the component buffers first: out-of-range input is
 * AE_RT_INVALID_ARG, where the reference reads past its arrays.  Any output
 * may be NULL.  The outputs feed ae_bvh_build_triangles, ae_bvh_pack_triangles,
 * ae_bvh_pack_shading and ae_bvh_pack_attributes in that order. */
ae_rt_status ae_mesh_asset_triangles(const ae_mesh_asset* asset, const ae_material* materials, uint32_t n_materials,
                                     float* verts, float* normals, float* uvs, float* colors, int32_t* material,
                                     float* opacity);

/* A material file (JSON text, Material from_json, MeshSerializer.cpp:212-256). */
typedef struct ae_material_asset ae_material_asset;

/* Texture slots of a material, in GPUMaterial's order */
#define AE_MAP_BASE_COLOR   0u
#define AE_MAP_OPACITY      1u
#define AE_MAP_NORMAL       2u
#define AE_MAP_ROUGHNESS    3u
#define AE_MAP_METALNESS    4u
#define AE_MAP_AO           5u
#define AE_MAP_DISPLACEMENT 6u

ae_rt_status ae_material_asset_load(const void* bytes, size_t size, ae_material_asset** out);
ae_rt_status ae_material_asset_load_file(const char* path, ae_material_asset** out);
void ae_material_asset_destroy(ae_material_asset* material);
const char* ae_material_asset_name(const ae_material_asset* material);
/* The texture path of one AE_MAP_* slot ("" when the material has none). */
const char* ae_material_asset_map_path(const ae_material_asset* material, uint32_t which);

/* The material's emissiveColor (sRGB, as in the file) and emissiveIntensity:
 * the inputs of ae_lights_from_mesh. */
ae_rt_status ae_material_asset_get_emissive(const ae_material_asset* material, float srgb[3], float* intensity);

/* GPUMaterial of this material the way RayTracingWorld::UpdateMaterials
 * fills it (RayTracingWorld.cpp:186-240): baseColor = pow(c, 2.2),
 * emissiveColor = pow(c, 2.2) * emissiveIntensity (ColorConverter.h:18-23),
 * opacity / roughness / metalness / ao / reflectance / normalScale /
 * twoSided / useVertexColors from the material, invertUVs and cullBackFaces
 * from `mesh` (NULL: 0).  texture_ids (6 entries in AE_MAP_* order, or
 * NULL) are the texture-table indices the caller gave the material's maps
 * (the engine's textureToBindlessIdx); a slot without a map, or with a
 * negative id, is -1.  ID is the caller's `id` (the engine hashes its mesh
 * id there). */
ae_rt_status ae_material_asset_to_gpu(const ae_material_asset* material, const ae_mesh_asset* mesh,
                                      const int32_t* texture_ids, int32_t id, ae_material* out);

/* ------------------------------------------------------------------------ */
/* Device context                                                            */
/* ------------------------------------------------------------------------ */

typedef struct ae_rt_ctx ae_rt_ctx;

/* Launch shape of the traversal kernels; the project's autotuner
 * (atlas_rt.autotune) picks these per workload.  Supported
 * (threads_per_block, stack_entries_smem) pairs: (128, 32) default, (64, 32),
 * (256, 16), (128, 16); each lane has 128 stack entries in total, the rest in
 * local memory.  Meshes and scenes whose trees can need more (the upload
 * measures each tree's depth) are traced by a variant with 1,024 entries
 * per lane (128 threads, 32 in shared memory). */
typedef struct ae_rt_config {
    int32_t device;               /* CUDA device ordinal */
    uint32_t blocks_per_sm;       /* persistent CTAs per SM (0 = the kernel's occupancy) */
    uint32_t threads_per_block;   /* 0 = 128 */
    uint32_t max_steps;           /* traversal step cap per ray (0 = 4 x nodes + 64) */
    uint32_t flags;               /* AE_RT_CFG_COUNT_FETCHES, _NO_NEAR_TIES, _STAGED_RAYS, _APPROXIMATE */
    uint32_t refill_steps;        /* traversal steps between warp refills (0 = 32) */
    uint32_t stack_entries_smem;  /* shared-memory stack entries per lane (0 = 32) */
    uint32_t refill_below;        /* also refill as soon as fewer than this many lanes of a warp
                                     are still traversing (1..32; 0 = the default; > 32 = never) */
    uint32_t leaf_wait;           /* closest-hit traces: a lane that reaches a leaf waits until this
                                     many lanes of its warp are at leaves (or no lane is at an inner
                                     node), so that leaf tests run together (0 = never wait;
                                     scheduling only, results are unchanged) */
} ae_rt_config;

ae_rt_status ae_rt_ctx_create(const ae_rt_config* cfg, ae_rt_ctx** out);
void ae_rt_ctx_destroy(ae_rt_ctx* ctx);

/* Text of the last error on this context ("" when none). */
const char* ae_rt_last_error(const ae_rt_ctx* ctx);

/* Uploads one mesh's BLAS: nodes, BVH triangles and (optional) shading
 * triangles, deep-copied into device memory the context owns.  The host
 * validator checks pointer ranges, leaf termination and pre-order child
 * indices (which rules out cycles) and returns AE_RT_BAD_BVH otherwise.
 * Replaces Mesh::BuildBVH's uploads (src/engine/mesh/Mesh.cpp:97-108). */
ae_rt_status ae_rt_mesh_upload(ae_rt_ctx* ctx, const ae_bvh_node* nodes, uint32_t n_nodes,
                               const ae_bvh_triangle* tris, const ae_triangle* shading,
                               uint32_t n_tris, int32_t* mesh_id);

/* Closest hit of every ray against one mesh: HitClosest (bvh.hsh:191-273)
 * over one BLAS, i.e. the engine's traversal with an identity instance.
 * tmin/tmax as HitClosest's arguments.  Also the batched GPU form of
 * Volume::BVH::GetIntersection (BVH.cpp:103). */
ae_rt_status ae_rt_trace_closest(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                 uint32_t n_rays, float tmin, float tmax, ae_hit* hits,
                                 void* stream);

/* Occlusion of every ray against one mesh: HitAny (bvh.hsh:359-441); the
 * batched GPU form of Volume::BVH::GetIntersectionAny (BVH.cpp:176).
 * occluded[i] = 1 when a triangle is hit with tmin < t < tmax. */
ae_rt_status ae_rt_trace_any(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                             uint32_t n_rays, float tmin, float tmax, uint8_t* occluded,
                             void* stream);

/* ------------------------------------------------------------------------ */
/* Two-level scene: top level over instances                                 */
/* ------------------------------------------------------------------------ */

/* Sets the scene traced by ae_rt_trace_scene_*: the top-level nodes (GPUBVHNode
 * layout, leaves ~index into `instances`) and the instances in top-level
 * order (GPUBVHInstance; meshOffset = a mesh id from ae_rt_mesh_upload).
 * Validated (pointer ranges, pre-order, mesh ids) and deep-copied.  Replaces
 * the tlasNodeBuffer / bvhInstanceBuffer uploads of RayTracingWorld
 * (RayTracingWorld.cpp:150-160, :297-301). */
ae_rt_status ae_rt_scene_set(ae_rt_ctx* ctx, const ae_bvh_node* tlas, uint32_t n_tlas,
                             const ae_bvh_instance* instances, uint32_t n_instances);

/* Builds the top level the way RayTracingWorld::UpdateForSoftwareRayTracing
 * does (RayTracingWorld.cpp:267-307): an AABB-only BVH over the instances'
 * world boxes (BVH.cpp:58-100), instances reordered to its reference order
 * with nextInstance linking each leaf, then ae_rt_scene_set.  order_out
 * (optional, capacity n_instances + 1) receives the input index of each
 * ordered instance; n_ordered their count (n_instances, or 2 for a single
 * instance, which the reference lists twice). */
ae_rt_status ae_rt_scene_build(ae_rt_ctx* ctx, const ae_bvh_instance* instances, const ae_aabb* world_aabbs,
                               uint32_t n_instances, uint32_t* order_out, uint32_t* n_ordered);

/* HitClosest / HitAny over the scene (bvh.hsh:191-273, :359-441): instances
 * whose mask shares no bit with cull_mask are skipped; ae_hit.instance is the
 * hit instance's top-level index. */
ae_rt_status ae_rt_trace_scene_closest(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays, float tmin,
                                       float tmax, uint32_t cull_mask, ae_hit* hits, void* stream);
ae_rt_status ae_rt_trace_scene_any(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays, float tmin,
                                   float tmax, uint32_t cull_mask, uint8_t* occluded, void* stream);
ae_rt_status ae_rt_trace_scene_closest_queue(ae_rt_ctx* ctx, const ae_packed_ray* rays, const uint32_t* count,
                                             uint32_t capacity, float tmin, float tmax, uint32_t cull_mask,
                                             ae_hit* hits, void* stream);
ae_rt_status ae_rt_trace_scene_any_queue(ae_rt_ctx* ctx, const ae_packed_ray* rays, const uint32_t* count,
                                         uint32_t capacity, float tmin, float tmax, uint32_t cull_mask,
                                         uint8_t* occluded, void* stream);

/* The transparency variants over the scene (every mesh needs its shading
 * triangles; materials from ae_rt_scene_set_materials, or opacity 1 when
 * none are set).  Opacity = GPUTriangle d2.w, or, when negative, GetOpacity
 * (surface.hsh:147-159): the material's opacity times its opacity texture
 * (ae_rt_scene_set_textures) sampled at the hit's interpolated UV, with v
 * flipped when the material's invertUVs > 0; a material index outside the
 * material array counts as opacity 1.
 * Replace HitClosestTransparency (bvh.hsh:275-357: only hits with opacity > 0
 * count) and HitAnyTransparency (bvh.hsh:443-524: `transparency` receives
 * the shader's return value, 1 = unoccluded, including its per-leaf
 * re-multiplication, bvh.hsh:500).  Host or device buffers. */
ae_rt_status ae_rt_trace_scene_closest_transparency(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays,
                                                    float tmin, float tmax, uint32_t cull_mask, ae_hit* out,
                                                    void* stream);
ae_rt_status ae_rt_trace_scene_any_transparency(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays,
                                                float tmin, float tmax, uint32_t cull_mask, float* transparency,
                                                void* stream);

/* ------------------------------------------------------------------------ */
/* Batched multi-mesh traces in one persistent launch                        */
/* ------------------------------------------------------------------------ */

/* One batch: rays against one uploaded mesh, closest hit (out = ae_hit[n]) or
 * any hit (out = uint8_t[n]); device buffers.  This is the engine's bindless
 * per-mesh array indexing (blasNodes[meshIdx], buffers.hsh:3-7, :45-61)
 * turned into a launch table. */
typedef struct ae_batch_desc {
    int32_t mesh_id;
    uint32_t any;
    const ae_packed_ray* rays;
    void* out;
    uint32_t n_rays;
    float tmin;
    float tmax;
    uint32_t reserved;
} ae_batch_desc;

/* All batches in one persistent launch: warps pull rays from one global
 * numbering; each lane looks up its ray's batch.  Asynchronous on `stream`. */
ae_rt_status ae_rt_trace_batched(ae_rt_ctx* ctx, const ae_batch_desc* batches, uint32_t n_batches, void* stream);

/* A reusable plan of a batched launch: the batch table lives in device
 * memory and the launch (counter reset + kernel) is captured once in a CUDA
 * graph; ae_rt_batch_plan_launch replays it.  The plan keeps the buffer
 * pointers of `batches`, so their contents may change between launches but
 * not their addresses or sizes. */
typedef struct ae_rt_batch_plan ae_rt_batch_plan;
ae_rt_status ae_rt_batch_plan_create(ae_rt_ctx* ctx, const ae_batch_desc* batches, uint32_t n_batches,
                                     ae_rt_batch_plan** out);
ae_rt_status ae_rt_batch_plan_launch(ae_rt_batch_plan* plan, void* stream);
void ae_rt_batch_plan_destroy(ae_rt_batch_plan* plan);

/* Closest hit against one mesh without any device allocation.  This entry
 * point has no counterpart in the reference.  It is for hosts that own all
 * device memory and do not let a library call cudaMalloc / cudaFree -- an
 * engine that carves every GPU buffer out of its own arenas at load time, or
 * a frame loop that must not hit the implicit device synchronisation those
 * calls bring -- and so cannot create an ae_rt_ctx.
 *  - nodes, tris, rays and hits are device pointers the caller owns; the BVH
 *    need not have passed the upload validator: node and triangle indices are
 *    range-checked on the device, and a bad one ends that ray with
 *    AE_HIT_OVERFLOW in its flags.
 *  - Results and semantics are those of ae_rt_trace_closest for trees of up
 *    to 128 levels, with the same 128-entry traversal stack per ray.  The
 *    call does not measure the tree, so a ray that needs more entries ends
 *    with AE_HIT_OVERFLOW (ae_rt_trace_closest, which knows each uploaded
 *    mesh's depth, runs 1,024-entry kernels for deeper trees).  The call is
 *    asynchronous on `stream` (NULL = legacy default stream) and reports
 *    device-side failures per ray in ae_hit.flags (AE_HIT_OVERFLOW,
 *    AE_HIT_ITER_CAP) rather than through a status.
 *  - Its only scratch is a 256-byte static device array per GPU (work
 *    counter and error word), which each call re-zeroes; calls that overlap
 *    on the GPU race on it, so issue them in one stream or order them.
 *  - The first call on a device looks up that array's device address and
 *    the kernel's occupancy; make it before any stream capture.
 *  - n_rays above AE_RT_NOALLOC_MAX_RAYS is rejected with AE_RT_INVALID_ARG
 *    (the work counter is 32 bits wide), as are host pointers and device
 *    pointers of a GPU other than the current one. */
#define AE_RT_NOALLOC_MAX_RAYS (1u << 30)
ae_rt_status ae_rt_trace_closest_noalloc(const ae_bvh_node* nodes, uint32_t n_nodes,
                                         const ae_bvh_triangle* tris, uint32_t n_tris,
                                         const ae_packed_ray* rays, uint32_t n_rays, float tmin, float tmax,
                                         ae_hit* hits, void* stream);

/* ------------------------------------------------------------------------ */
/* Wavefront stages (device buffers, asynchronous on `stream`)               */
/* ------------------------------------------------------------------------ */

/* Pinhole camera in the form of the engine's ray-gen uniforms
 * (PathTracingRenderer.h:49-57, PathTracingRenderer.cpp:157-160): `origin`
 * is the image-plane corner of pixel (0,0) at unit distance, `right` and
 * `bottom` span the image, `location` is the eye. */
typedef struct ae_camera {
    float location[4];
    float origin[4];
    float right[4];
    float bottom[4];
    uint32_t width;
    uint32_t height;
    float jitter[2];     /* sub-pixel offset in [0,1) */
} ae_camera;

/* Bounce / shadow ray spawn after a closest-hit trace. */
typedef struct ae_bounce_params {
    float light_dir[4];  /* unit direction towards the directional light */
    float epsilon;       /* origin offset (the engine's EPSILON = 0.1, common.hsh:9) */
    uint32_t seed;       /* random stream of the bounce directions */
    uint32_t reserved[2];
} ae_bounce_params;

/* Writes width*height primary rays (8x8 tile order, ID = pixel index) into
 * the device buffer `rays`.  Replaces the ray-gen dispatch
 * RayTracingHelper::DispatchRayGen (RayTracingHelper.cpp:147-221) running
 * rayGen.csh. */
ae_rt_status ae_rt_raygen(ae_rt_ctx* ctx, const ae_camera* cam, ae_packed_ray* rays, void* stream);

/* Queue-driven traces: the ray count is read on the device from `count`
 * (written by an earlier kernel), at most `capacity`.  These replace the
 * indirect-dispatch pair traceDispatch.csh + traceClosest.csh
 * (RayTracingHelper.cpp:224-363) without a host round trip. */
ae_rt_status ae_rt_trace_closest_queue(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                       const uint32_t* count, uint32_t capacity, float tmin, float tmax,
                                       ae_hit* hits, void* stream);
ae_rt_status ae_rt_trace_any_queue(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                   const uint32_t* count, uint32_t capacity, float tmin, float tmax,
                                   uint8_t* occluded, void* stream);

/* For every hit among the first min(*count, n) rays (count may be NULL):
 * appends one cosine-weighted bounce ray to `secondary` and, when the light
 * is above the surface, one shadow ray to `shadow`; counts[0] / counts[1]
 * are incremented (the caller zeroes them).  Ray IDs are carried over.
 * The hit-shader step of rayHit.csh:160-338 reduced to ray spawning. */
ae_rt_status ae_rt_spawn_bounce(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays, const ae_hit* hits,
                                const uint32_t* count, uint32_t n, const ae_bounce_params* params,
                                ae_packed_ray* secondary, ae_packed_ray* shadow, uint32_t* counts,
                                void* stream);

/* ae_rt_raygen followed by ae_rt_trace_closest of its width*height rays,
 * with the same hits, but the rays are made inside the traversal kernel
 * and never stored (the 32-byte ray write and read per ray saved).  `hits`
 * is host or device memory, as for ae_rt_trace_closest.  Meshes deeper than 128 levels, and contexts with
 * AE_RT_CFG_APPROXIMATE or fetch counting, run raygen and the plain trace
 * on context scratch instead.  Replaces the rayGen.csh dispatch of
 * RayTracingHelper::DispatchRayGen (RayTracingHelper.cpp:147-221) and the
 * closest-hit trace of its rays. */
ae_rt_status ae_rt_trace_camera_closest(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam, float tmin,
                                        float tmax, ae_hit* hits, void* stream);

/* ae_rt_spawn_bounce over the width*height camera rays of `cam` (as
 * ae_rt_raygen makes them) and their hits, without a primary ray buffer. */
ae_rt_status ae_rt_spawn_bounce_camera(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam, const ae_hit* hits,
                                       const ae_bounce_params* params, ae_packed_ray* secondary,
                                       ae_packed_ray* shadow, uint32_t* counts, void* stream);

/* One ray-cast pass of a camera over a mesh: primary closest-hit, bounce and
 * shadow spawn, secondary closest-hit, shadow any-hit.  Output buffers may be
 * host or device memory (any may be NULL); counts receives the number of
 * primary, secondary and shadow rays.  Returns after the results are in
 * place. */
typedef struct ae_cast_outputs {
    ae_hit* primary_hits;            /* width*height */
    ae_packed_ray* secondary_rays;   /* up to width*height */
    ae_hit* secondary_hits;
    ae_packed_ray* shadow_rays;
    uint8_t* shadow_occluded;
    uint32_t counts[3];
} ae_cast_outputs;

ae_rt_status ae_rt_cast_pass(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam,
                             const ae_bounce_params* params, ae_cast_outputs* out, void* stream);

/* ------------------------------------------------------------------------ */
/* Path tracer                                                               */
/* ------------------------------------------------------------------------ */

/* Materials (GPUMaterial, indexed by GPUTriangle material index +
 * GPUBVHInstance::materialOffset) and lights (GPULight; type 1 = triangle
 * light: data.x = (1 << 28) | BVH-order triangle index, data.z = area,
 * data.w = instance index bits; type 0 = directional: N = direction).
 * Replaces RayTracingWorld::UpdateMaterials (RayTracingWorld.cpp:171-251)
 * and RayTracingHelper::UpdateLights (RayTracingHelper.cpp:436-500). */
ae_rt_status ae_rt_scene_set_materials(ae_rt_ctx* ctx, const ae_material* materials, uint32_t n);

/* Texel formats of ae_texture; sampling reads the first channel. */
#define AE_TEX_R8_UNORM    0u
#define AE_TEX_RGBA8_UNORM 1u
#define AE_TEX_R32_FLOAT   2u

/* One texture's base level in host memory: `height` rows of `row_pitch`
 * bytes (0 = tightly packed), 1 <= width, height <= 65536. */
typedef struct ae_texture {
    const void* texels;
    uint32_t width;
    uint32_t height;
    uint32_t format;
    uint32_t row_pitch;
} ae_texture;

/* The scene's textures: the bindless texture array (globals.hsh:33) that
 * RayTracingWorld::UpdateMaterials indexes through
 * Scene::textureToBindlessIdx (RayTracingWorld.cpp:217-237); texture i is
 * what a material's *Texture field i names, and a negative or out-of-range
 * index samples as 1.0 (texture.hsh:18-25 for negative ones).  The
 * traversal's opacity lookups sample level 0 (bvh.hsh:127, :163); surface
 * shading samples the level its pass reads (0 for the path tracer, 4 for
 * DDGI, ae_rt_pass_params.texture_level for reflections and RTGI).
 * Sampling follows the engine's bindless sampler (linear filter, repeat
 * addressing, MainRenderer.cpp:922-929) in FP32, one rounding per
 * operation: x = u * width - 0.5, i = floor(x), a = x - i, texels i and i+1
 * modulo width (likewise y with v and height), value = ((w00*c00 + w10*c10)
 * + w01*c01) + w11*c11 with w00 = (1-a)(1-b), w10 = a(1-b), w01 = (1-a)b,
 * w11 = ab; UNORM texels are byte / 255; a non-finite x (or y) becomes 0,
 * which reads texel 0 of that axis alone.  Copies the texels into device
 * memory together with their mip chain down to 1 x 1 (level k + 1 = the
 * 2 x 2 box filter of level k, indices clamped at odd edges; UNORM bytes
 * as (a + b + c + d + 2) / 4, floats as ((a + b) + (c + d)) * 0.25) and
 * replaces the previous table (n = 0 clears it).  An integer level samples
 * that one level, as textureLod does. */
ae_rt_status ae_rt_scene_set_textures(ae_rt_ctx* ctx, const ae_texture* textures, uint32_t n);
ae_rt_status ae_rt_scene_set_lights(ae_rt_ctx* ctx, const ae_light* lights, uint32_t n);

/* The environment the path tracer's misses see: a constant radiance (rgb,
 * finite, >= 0; initially black), added as min(radiance * throughput, 10) per
 * channel on every miss, the camera's included (EvaluateBounce,
 * rayHit.csh:166-171, where the engine samples its sky cubemap).  The
 * radiance cache models no environment: its calls refuse a non-black one,
 * and a scene with a mesh that is not opaque (shading opacity other than 1). */
ae_rt_status ae_rt_scene_set_environment(ae_rt_ctx* ctx, const float radiance[3]);

/* The light list the engine builds on the host before each path-tracing
 * dispatch.  Arithmetic follows the reference in float32, operation by
 * operation; pow is the C library's powf, as glm::pow calls it.
 *
 * ae_lights_from_mesh: RayTracingWorld::BuildTriangleLightsForMesh
 * (RayTracingWorld.cpp:322-376).  One GPULight per triangle of `shading` (the
 * mesh's GPUTriangle array, BVH order) whose material (d0.w, an index into
 * the mesh's materials) has brightness = dot(pow(emissive, 2.2), 0.3333) > 0:
 * P = the vertex mean, N = the mean of the unpacked 10:10:10:2 vertex normals
 * (not normalised), area by Heron's formula, colour = pow(pow(emissive, 2.2),
 * 2.2) * emissiveIntensity (the reference converts twice), data = (type 1 |
 * triangle index, area * brightness, area, 0).  emissive_srgb (3 floats per
 * material) and emissive_intensity are the engine Material's sRGB
 * emissiveColor and emissiveIntensity.  *n_out = the number of emissive
 * triangles; out may be NULL to count them; more than `capacity` fills
 * `capacity` and returns AE_RT_OUT_OF_MEMORY. */
ae_rt_status ae_lights_from_mesh(const ae_triangle* shading, uint32_t n_tris, const float* emissive_srgb,
                                 const float* emissive_intensity, uint32_t n_materials, ae_light* out,
                                 uint32_t capacity, uint32_t* n_out);

/* RayTracingWorld::UpdateTriangleLights (RayTracingWorld.cpp:378-407): a
 * mesh's lights placed by one instance.  P = model * (P, 1), N = model *
 * (N, 0) with `model` the 4 x 4 world matrix in row-major order (glm's
 * pairwise column sum), data.w = the instance index bits. */
ae_rt_status ae_lights_instance(const ae_light* mesh_lights, uint32_t n, const float* model, int32_t instance,
                                ae_light* out);

/* The directional branch of RayTracingHelper::UpdateLights
 * (RayTracingHelper.cpp:440-474): colour = pow(color, 2.2) * intensity,
 * N = direction (the light travels along it), data = (type 0 | index,
 * brightness, 0, 0). */
ae_rt_status ae_light_directional(const float color_srgb[3], float intensity, const float direction[3],
                                  uint32_t index, ae_light* out);

/* UpdateLights' weights (RayTracingHelper.cpp:481-499): data.y raised to at
 * least 0.005 x the largest, then divided by their sum. */
ae_rt_status ae_lights_normalize(ae_light* lights, uint32_t n);

/* DispatchAndHit's selection (RayTracingHelper.cpp:72-105): when n <=
 * capacity (the engine's light buffer holds 128), every light with data.y =
 * 1; otherwise `capacity` draws with replacement from the piecewise-constant
 * distribution over data.y (Common::Piecewise1D, Piecewise.cpp:11-78, one
 * draw per entry of `uniforms`, each in [0, 1)), each drawn light's data.y
 * multiplied by capacity.  The engine draws from an unseeded std::mt19937;
 * the caller supplies the uniforms here.  *n_out = min(n, capacity). */
ae_rt_status ae_lights_select(const ae_light* lights, uint32_t n, uint32_t capacity, const float* uniforms,
                              ae_light* out, uint32_t* n_out);

typedef struct ae_pt_params {
    uint32_t spp;            /* samples per pixel in this call */
    uint32_t max_bounces;    /* the engine's `bounces`: bounces + 1 hit evaluations */
    uint32_t sample_offset;  /* index of the first sample (random streams continue across calls) */
    uint32_t seed;
    float epsilon;           /* ray origin offset (EPSILON = 0.1, common.hsh:9) */
    uint32_t flags;          /* AE_PT_MIS: not the engine's estimator (below) */
    uint32_t reserved[2];
} ae_pt_params;

/* Next-event estimation combined with BRDF sampling by the power heuristic
 * (BRDF-sampled light hits at bounces >= 1 count, weighted).  Same expected
 * image as the engine's estimator, fewer outliers on glossy surfaces. */
#define AE_PT_MIS 0x1u

/* Primary rays through the pixel centres offset by ae_camera.jitter * 0.25
 * (the engine's TAA jitter, globalData.jitterCurrent) instead of a random
 * sub-pixel offset per sample: the real-time ray generation
 * (rayGen.csh:37-38), which ae_rt_pathtrace_realtime always uses. */
#define AE_PT_CENTERED 0x2u

/* The call's pixels (the whole image, or the tile) start a new accumulation:
 * their accum / accum64 entries are cleared before the first sample, as the
 * engine's rayHit overwrites its accumulation image at sampleCount 0
 * (rayHit.csh:121-122). */
#define AE_PT_RESTART 0x4u

/* Path-traces spp samples of every pixel of `cam` over the scene (which needs
 * shading triangles, materials and lights) and adds the radiance of each
 * sample into accum (float4 per pixel, rgb) and, if given, accum64 (double x3
 * per pixel).  Device buffers, asynchronous on `stream`; divide by the
 * number of samples for the image.  Replaces PathTracingRenderer::Render's
 * ray-gen + bounce loop (PathTracingRenderer.cpp:29-192) for the
 * non-real-time mode, without the indirect radiance clamp (rayHit.csh:196-201). */
ae_rt_status ae_rt_pathtrace(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params, float* accum,
                             double* accum64, void* stream);

/* The same over one tile of the image: the pixels x0 <= x < x0 + width,
 * y0 <= y < y0 + height of cam's resolution, as PathTracingRenderer::Render
 * traces one of imageSubdivisions tiles per call (rayGen.csh:25-30,
 * pixelOffset and tileSize).  accum / accum64 are whole-image buffers; the
 * other pixels are left alone.  A pixel's samples do not depend on the
 * tiling. */
ae_rt_status ae_rt_pathtrace_tile(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params, uint32_t x0,
                                  uint32_t y0, uint32_t width, uint32_t height, float* accum, double* accum64,
                                  void* stream);

/* The real-time G-buffer that the first sample's first hit writes for the
 * temporal pass (rayHit.csh:76-116); every plane is optional device memory
 * of one entry per pixel. */
typedef struct ae_pt_realtime {
    float* depth;              /* view-space z of the hit (view * (P, 1)).z, INF = 1e12 on a miss */
    uint32_t* material_idx;    /* GPUMaterial.ID of the hit, 65535 on a miss */
    float* normal;             /* 2 floats: EncodeNormal of the world-space geometry normal, (1, 0, 0) on a miss */
    float* velocity;           /* 2 floats: (ndcLast - ndcCurrent) * 0.5 */
    float view[16];            /* globalData.vMatrix, row-major */
    float proj[16];            /* globalData.pMatrix */
    float pv_last[16];         /* globalData.pvMatrixLast */
    /* previous frame's object-to-world matrix of every scene instance (12
     * floats, 3 rows of 4), indexed like the instances on the device (the
     * order given to ae_rt_scene_set, or the order ae_rt_scene_build
     * reports); NULL: the current ones.  A miss moves with the camera only
     * (position = origin + direction * 100). */
    const float* last_matrices;
    uint32_t n_last_matrices;
} ae_pt_realtime;

/* The engine's real-time accumulation of the same estimator
 * (rayHit.csh:134-150, REALTIME): params->spp samples per pixel into
 * frame_accum, a [3][height][width] uint32 image (one layer per channel,
 * the engine's frameAccumImage), cleared by the call.  At spp = 1 each
 * pixel holds the float bits of its radiance; at spp > 1 every radiance
 * contribution is divided by max_radiance, clamped to [0, 1], scaled to
 * 0xFFFFFFFF / spp and added as an unsigned integer.  The engine quantises
 * a path's total; here each contribution (emission, each light sample) is
 * quantised, which differs only where the clamp or the rounding bites.
 * Primary rays go through the pixel centres offset by cam->jitter * 0.25
 * (AE_PT_CENTERED).  rt (optional) names the G-buffer planes the first
 * sample writes.  Device memory. */
ae_rt_status ae_rt_pathtrace_realtime(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params,
                                      const ae_pt_realtime* rt, uint32_t* frame_accum, float max_radiance,
                                      void* stream);

/* The non-real-time output image (rayHit.csh:124-130): for every pixel of
 * accum (float4, the sum of `samples` samples), colour = accum.rgb *
 * exposure / samples (in that order), out = (pow(1 - exp(-colour), gamma),
 * 1).  Device memory, float4 per pixel. */
ae_rt_status ae_rt_pt_tonemap(ae_rt_ctx* ctx, const float* accum, uint32_t width, uint32_t height, uint32_t samples,
                              float exposure, float gamma, float* out, void* stream);

/* The same over the pixels x0 <= x < x0 + tile_width, y0 <= y < y0 +
 * tile_height of the width x height images accum and out (the engine writes
 * the output image of the tile it traced). */
ae_rt_status ae_rt_pt_tonemap_tile(ae_rt_ctx* ctx, const float* accum, uint32_t width, uint32_t height, uint32_t x0,
                                   uint32_t y0, uint32_t tile_width, uint32_t tile_height, uint32_t samples,
                                   float exposure, float gamma, float* out, void* stream);

/* ------------------------------------------------------------------------ */
/* The traversal's other consumers: RTAO, reflections, RTGI, DDGI probe rays  */
/* ------------------------------------------------------------------------ */

/* The G-buffer that a screen-space pass reads, all device memory, `width` x
 * `height` pixels row by row:
 *   depth      one float per pixel, NDC depth (>= 1: nothing drawn);
 *   normal     two floats per pixel, the octahedral view-space normal
 *              (DecodeNormal, common/normalencode.hsh:18-30);
 *   offset     optional byte per pixel, 0..3: which pixel of its 2x2 block a
 *              half-resolution depth sample came from (offsets[],
 *              ao/rtao.csh:27-32); NULL = 0;
 *   roughness  one float per pixel, the material roughness after its map
 *              (reflections only; rtreflection.csh:92-96);
 *   samples    optional two floats per pixel in [0, 1): the shader's
 *              blue-noise vector; NULL = drawn as below;
 *   ip_matrix, iv_matrix  inverse projection and inverse view, column-major
 *              like GLSL's mat4 (globalData.ipMatrix / ivMatrix);
 *   half_res   1: this buffer has half the depth buffer's resolution, and
 *              positions are reconstructed at 2*pixel + offset + 0.5 of the
 *              full one (ao/rtao.csh:66, rtreflection.csh:75-79).
 *   scrambling_ranking, sobol_sequence  optional, both or neither: the
 *              engine's blue-noise textures as RGBA8 texels, 128 x 128 and
 *              256 x 1 (the scramblingRankingTexture / sobolSequenceTexture
 *              that rtao.csh, rtreflection.csh and rtgi.csh bind).  When
 *              `samples` is NULL and these are given, the pixel's vector is
 *              (SampleBlueNoise(pixel, frame_seed, 0), SampleBlueNoise(pixel,
 *              frame_seed, 1)) of common/bluenoise.hsh:9-32 (Heitz et al.
 *              2019): pixel mod 128, sample index mod 256, ranked index =
 *              index ^ ranking.b, value = sobol[ranked][dim] ^
 *              ranking[dim], (value + 0.5) / 256; without them, the
 *              library's PCG hash of (pixel, frame_seed).
 * World position = iv * (ConvertDepthToViewSpace: ip * (2*tc - 1, depth, 1),
 * divided by w); world normal = normalize(iv * (DecodeNormal(normal), 0)). */
typedef struct ae_gbuffer {
    const float* depth;
    const float* normal;
    const uint8_t* offset;
    const float* roughness;
    const float* samples;
    uint32_t width;
    uint32_t height;
    uint32_t half_res;
    uint32_t reserved;
    float ip_matrix[16];
    float iv_matrix[16];
    const uint8_t* scrambling_ranking;
    const uint8_t* sobol_sequence;
} ae_gbuffer;

#define AE_PASS_OPACITY_CHECK 0x1u   /* trace with the transparency variants (OPACITY_CHECK) */

/* Uniforms of the passes. */
typedef struct ae_rt_pass_params {
    float radius;            /* RTAO: length of the occlusion rays */
    float bias;              /* reflections: sample.y *= 1 - bias; RTGI: sample.x *= 1 - bias */
    float roughness_cutoff;  /* reflections: rougher pixels trace nothing (radiance 0) */
    float radiance_limit;    /* reflections, RTGI: colours scaled so no channel exceeds it */
    float environment[3];    /* radiance of rays that hit nothing (the environment map's place) */
    uint32_t flags;          /* AE_PASS_OPACITY_CHECK */
    uint32_t frame_seed;     /* uniforms.frameSeed: the sample index of the random streams */
    uint32_t seed;           /* random stream of light choices (and of samples when none are given) */
    uint32_t texture_level;  /* reflections, RTGI: mip level of the hit's surface textures
                                (uniforms.textureLevel); DDGI always reads level 4 (ddgi/rayHit.csh:79) */
    uint32_t reserved;
} ae_rt_pass_params;

/* Ray-traced ambient occlusion, ao/rtao.csh:40-112: per pixel with depth < 1
 * one cosine-weighted ray (SampleDiffuseBRDF, brdf/brdfSample.hsh:8-32) from
 * P + L*EPSILON + N*EPSILON, HitAny (or, with AE_PASS_OPACITY_CHECK,
 * 1 - HitAnyTransparency) over [0, radius], mask ALL; ao = 1 - occlusion,
 * 1 where nothing was drawn.  ao: one float per pixel, device memory. */
ae_rt_status ae_rt_rtao(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params, float* ao,
                        void* stream);

/* Ray-traced reflections, reflection/rtreflection.csh:60-245: per pixel with
 * depth < 1 and roughness <= 1, a GGX VNDF sample (roughness > 0.01) or the
 * mirror direction, from P offset by EPSILON * 0.1 * max(1, |viewPos|) * 0.1
 * along L and N; pixels with roughness <= roughness_cutoff trace HitClosest
 * (HitClosestTransparency) over [0, INF] and shade the hit: emission + one
 * light sample with the Disney diffuse + GGX specular BRDF times opacity,
 * visible through HitAnyTransparency (mask SHADOW, up to the light distance
 * - 2*EPSILON); misses return `environment`; no DDGI term.  Then the
 * radiance limit.  radiance: four floats per pixel (rgb, 1), device memory. */
ae_rt_status ae_rt_reflections(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params,
                               float* radiance, void* stream);

/* Ray-traced diffuse GI, rtgi/rtgi.csh:100-234: a cosine-weighted sample
 * (ImportanceSampleCosDir, brdf/importanceSample.hsh:82-101) from P offset by
 * EPSILON * max(1, |viewPos|) * 0.01 along L and N, traced and shaded like
 * the reflections.  radiance: four floats per pixel, device memory. */
ae_rt_status ae_rt_rtgi(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params, float* radiance,
                        void* stream);

/* DDGI probe rays, ddgi/rayGen.csh:39-81 + ddgi/rayHit.csh:37-151.
 *   probes    n_probes x 4 floats: probe position + offset (xyz) and the
 *             probe state's bits in w (0 new, 1 active, 2 inactive);
 *   ray_dirs / ray_dirs_inactive  ray_count / inactive_ray_count x 4 floats;
 *   rotation  the frame's random rotation (mat4, column-major; its 3x3 part
 *             turns every direction).
 * Probe p traces ray_count rays (inactive probes: inactive_ray_count, along
 * ray_dirs_inactive) with HitClosest (HitClosestTransparency) and shades
 * each like rayHit.csh: a miss returns `environment`; a backface hit on a
 * one-sided material that culls back faces has radiance 0 and a negative
 * distance; otherwise emission + one light sample with the diffuse BRDF
 * times opacity, visible through HitAny (mask SHADOW).  The irradiance
 * volume's indirect term is not added.  Output: PackRayHit (ddgi.hsh:85-98)
 * at hits[p * ray_count + i] (4 floats: half2 direction.xy, half2
 * radiance.xy, half2 (direction.z, radiance.z), distance; radiance clamped
 * to 3200); entries beyond a probe's ray count are left as they were.  All
 * buffers are device memory. */
typedef struct ae_ddgi_probes {
    const float* probes;
    const float* ray_dirs;
    const float* ray_dirs_inactive;
    float rotation[16];
    uint32_t n_probes;
    uint32_t ray_count;
    uint32_t inactive_ray_count;
    uint32_t reserved;
} ae_ddgi_probes;
ae_rt_status ae_rt_ddgi_trace(ae_rt_ctx* ctx, const ae_ddgi_probes* probes, const ae_rt_pass_params* params,
                              float* hits, void* stream);

/* ------------------------------------------------------------------------ */
/* Learned radiance cache (no counterpart in the reference engine)           */
/* ------------------------------------------------------------------------ */

/* A neural radiance cache bound to a context's scene: a 16-level hash grid
 * (2 FP16 features per entry, 2^log2_table entries per level, resolutions
 * from base_resolution to max_resolution in a geometric progression) over
 * the world box aabb_min..aabb_max, 16 spherical-harmonic coefficients of
 * the outgoing direction, the normal and the roughness feed a 5 x 64 ReLU
 * MLP (BF16 weights, FP32 accumulation) that predicts the indirect radiance
 * leaving a surface point (what the path tracer adds after the point's own
 * next-event estimate, within its bounce budget), divided by the point's base
 * colour and times radiance_scale.  Trained online with Adam on a relative L2
 * loss. */
typedef struct ae_rc ae_rc;

typedef struct ae_rc_config {
    uint32_t log2_table;        /* 19 */
    uint32_t base_resolution;   /* 16 */
    uint32_t max_resolution;    /* 2048 */
    float learning_rate;        /* 1e-2 */
    float beta1;                /* 0.9 */
    float beta2;                /* 0.99 */
    float epsilon;              /* 1e-15 */
    uint32_t seed;
    float aabb_min[3];
    float aabb_max[3];
    float radiance_scale;       /* stored value = radiance x scale (0: 1) */
    float rough_cut;            /* rendering: metals at least this rough end in the cache (0: 0.35) */
    uint32_t glossy_split;      /* rendering: paths per glossier metal at the first vertex (0: 4; max 4) */
    uint32_t flags;             /* AE_RC_TRAIN_WARP_MMA */
} ae_rc_config;

/* Training runs on the warp-level mma.sync kernel instead of the default
 * tensor-memory (tcgen05) kernel; both compute the same gradients up to the
 * order of FP32 additions. */
#define AE_RC_TRAIN_WARP_MMA 0x1u

ae_rt_status ae_rc_create(ae_rt_ctx* ctx, const ae_rc_config* cfg, ae_rc** out);
void ae_rc_destroy(ae_rc* rc);

/* Parameter counts: MLP weights (21,504: 5 matrices of 64 x 64 and a 16 x 64
 * output matrix of which 3 rows are used, rows = output neurons) and grid
 * features (16 x 2^log2_table x 2). */
ae_rt_status ae_rc_param_counts(const ae_rc* rc, uint32_t* n_mlp, uint64_t* n_grid);

/* FP32 master parameters to / from host memory (checkpoint and resume; a
 * set also resets the optimizer state). */
ae_rt_status ae_rc_get_params(ae_rc* rc, float* mlp, float* grid);
ae_rt_status ae_rc_set_params(ae_rc* rc, const float* mlp, const float* grid);

/* Query / training records, 16 floats each: position xyz, roughness;
 * outgoing direction xyz (unit, towards the viewer), pixel index bits;
 * normal xyz, vertex depth (bounces from the camera); target (training) or
 * render weight rgb, 1. */

/* Predictions for n query records (device buffers; out: 4 floats each). */
ae_rt_status ae_rc_predict(ae_rc* rc, const float* queries, uint32_t n, float* out, void* stream);

/* Diagnostic of the tensor-memory kernels' bounded waits: runs the inference
 * kernel on one CTA with no MMA issued, so that nothing ever completes the
 * mbarrier it waits on; the wait gives up after ~200 ms, the kernel frees its
 * tensor memory and returns, and the error word reports the timeout.
 * *timed_out = 1 when ae_rt_synchronize reported AE_RT_TIMEOUT as expected;
 * the context remains usable.  Synchronous. */
ae_rt_status ae_rc_selftest_wait_timeout(ae_rc* rc, uint32_t* timed_out);

/* Loss gradients of n training records without an optimizer step (device
 * records; grad_mlp / grad_grid may be host or device memory or NULL). */
ae_rt_status ae_rc_gradients(ae_rc* rc, const float* samples, uint32_t n, float* grad_mlp, float* grad_grid,
                             float* loss_out, void* stream);

/* One Adam step on n training records (device). */
ae_rt_status ae_rc_train_batch(ae_rc* rc, const float* samples, uint32_t n, float* loss_out, void* stream);

/* One frame of online training: n_paths self-generated paths from random
 * pixels of `cam`, each traced with the path tracer's estimator up to
 * max_bounces bounces (1..16); every vertex at depth < min(max_bounces, 3)
 * gives one record of its indirect radiance, and the records train the cache
 * in `steps` Adam steps (equal slices).  The render uses the same bounce
 * budget.  loss_out (optional, mean loss of the last step) synchronises. */
ae_rt_status ae_rc_train_frame(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t n_paths, uint32_t steps,
                               uint32_t max_bounces, float* loss_out, void* stream);

/* One sample per pixel with paths terminated into the cache: the first hit's
 * emission and next-event estimation at every vertex, as the path tracer;
 * at the first diffuse vertex or metal with roughness >= rough_cut (or at
 * bounce last_bounce, or depth 2) the cache's indirect radiance times path
 * throughput x base colour ends the path; glossier metals before it continue,
 * their light combining next-event estimation and BRDF sampling (power
 * heuristic); at the first vertex they split into glossy_split paths of
 * weight 1/glossy_split.  Adds into accum (float4 per pixel, device;
 * atomically).  At most 2^24 pixels. */
ae_rt_status ae_rc_render(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t last_bounce, float* accum,
                          void* stream);

/* One online frame: renders one sample per pixel as ae_rc_render with the
 * cache as it stands at the call (a device-side snapshot of its FP16 grid
 * and BF16 weights), while on a second stream the frame's n_paths training
 * paths are traced (they read the scene only) and trained on in `steps`
 * Adam steps (ae_rc_train_frame).  Same work as train + render, with the
 * render one training step behind and the training overlapped with it; the
 * call's stream waits for both. */
ae_rt_status ae_rc_frame(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t n_paths, uint32_t steps,
                         uint32_t max_bounces, uint32_t last_bounce, float* accum, float* loss_out, void* stream);

/* GPU BVH build: a linear BVH (Morton order of triangle centroids, Karras's
 * parallel hierarchy, bounds bottom-up) built on the device and registered
 * as a mesh of the context, in the engine's GPUBVHNode / GPUBVHTriangle
 * layouts (one triangle per leaf; root = node 0; n - 1 nodes for n >= 2).
 * verts: n * 9 floats (v0, v1, v2); material / opacity: optional, per input
 * triangle; order_out (optional, n entries, or 2 for n == 1) receives the
 * input index of each BVH-order triangle.  Host or device buffers; returns
 * after the build.  The engine builds on the CPU (Volume::BVH, BVH.cpp:14;
 * MeshData::BuildBVH, MeshData.cpp:63-271): this is the GPU alternative, not
 * a reproduction of that tree -- traces on it return the same nearest
 * distance for every ray, and the same triangle except between triangles at
 * exactly equal distance. */
ae_rt_status ae_rt_mesh_build(ae_rt_ctx* ctx, const float* verts, uint32_t n, const int32_t* material,
                              const float* opacity, int32_t* mesh_id, uint32_t* order_out, void* stream);

/* The BVH of a mesh of the context (uploaded or built) back into host or
 * device memory; n_nodes / n_tris (optional) receive the counts; nodes / tris
 * may be NULL to query them. */
ae_rt_status ae_rt_mesh_get_bvh(ae_rt_ctx* ctx, int32_t mesh, ae_bvh_node* nodes, ae_bvh_triangle* tris,
                                uint32_t* n_nodes, uint32_t* n_tris);

/* Double-precision re-test of near ties.  For every ray whose ae_hit (from
 * ae_rt_trace_closest / _queue on the same mesh, tmin and tmax) carries
 * AE_HIT_NEAR_TIE, the nearest triangle is searched again in double precision:
 * a closest-hit traversal of the same BVH with conservative double slab
 * tests and the double form of the shader's triangle test (tmin < t < tmax);
 * equal double distances resolve to the lower BVH-order index (entries with
 * the same vertices, the copies a spatial split makes, count as one triangle:
 * triPtr is one of them), t_second is the second smallest accepted distance
 * when it is at most t + |t| 1e-5 (each operation rounded separately), else
 * +inf: the search prunes at that window.  Other rays are passed through (t,
 * triPtr, tSecond, AE_HIT_HIT).  Device buffers; n_retested (optional, host)
 * receives the number of flagged rays and synchronises.  The engine has no
 * counterpart: its shader keeps the FP32 winner (bvh.hsh:62-63). */
typedef struct ae_hit_f64 {
    double t;             /* +inf: no hit */
    double t_second;      /* within t + |t| 1e-5, else +inf (re-tested rays) */
    int32_t triPtr;       /* BVH order, -1: miss */
    uint32_t flags;       /* AE_HIT_HIT, AE_HIT_RETESTED, AE_HIT_OVERFLOW */
    int32_t reserved[2];
} ae_hit_f64;
ae_rt_status ae_rt_retest_near_ties(ae_rt_ctx* ctx, int32_t mesh, const ae_packed_ray* rays, const ae_hit* hits,
                                    uint32_t n_rays, float tmin, float tmax, ae_hit_f64* out,
                                    uint32_t* n_retested, void* stream);

/* Waits for `stream` and reports device-side errors of the context's
 * preceding asynchronous calls (stack overflow, step cap, timeouts). */
ae_rt_status ae_rt_synchronize(ae_rt_ctx* ctx, void* stream);

/* Per-launch statistics of the most recent trace on this context (counted
 * only when the context was created with AE_RT_CFG_COUNT_FETCHES in
 * ae_rt_config.flags): inner-node fetches and triangle fetches summed over
 * rays. */
#define AE_RT_CFG_COUNT_FETCHES 0x1u
/* Closest-hit traces of the context skip the complete near-tie detection
 * (AE_HIT_NEAR_TIE): the flag then marks only rays whose second accepted
 * triangle lies within 1e-6 relative t of the nearest, a subset of the near
 * ties, and ae_rt_retest_near_ties re-tests only those.  Hits are unchanged;
 * the detection costs about a tenth of the closest-hit time of the terrain
 * camera pass. */
#define AE_RT_CFG_NO_NEAR_TIES  0x2u
/* Single-mesh and scene traces of the context hand out rays in tiles of 16
 * consecutive rays that each warp copies into shared memory with one bulk
 * copy (TMA), the next tile in flight while the current one is used.  Ray
 * buffers must be 16-byte aligned (as for the plain loads).  Results are
 * unchanged. */
#define AE_RT_CFG_STAGED_RAYS   0x4u
/* Every closest- and any-hit trace of the context over one mesh or the scene
 * (also those of the library's path tracer and passes on it) uses the
 * approximate traversal, for consumers whose results are Monte Carlo
 * estimates rather than the shader's bit for bit: child boxes are tested with
 * RN(RN(c - o) * RN(1/d)) instead of the correctly rounded quotient, with a
 * margin of 2^-20 relative that never rejects a box the exact test accepts,
 * and triangles with one reciprocal of the denominator.  The nearest
 * triangle is the exact traversal's except where two triangles tie in t or
 * a ray grazes a triangle edge within a few units in the last place of its
 * barycentrics; for the same triangle t, u and v are within 1.5 units of
 * 2^-24 (relative) of the exact ones; the near-tie flag marks only rays whose
 * second accepted triangle lies within 1e-6 relative t (as with
 * AE_RT_CFG_NO_NEAR_TIES).  (The radiance cache's training paths always
 * trace this way; its render follows the context.)  The transparency
 * variants, the batched launch and the FP64
 * re-test stay exact, and so do launches with AE_RT_CFG_STAGED_RAYS or
 * AE_RT_CFG_COUNT_FETCHES. */
#define AE_RT_CFG_APPROXIMATE   0x8u
ae_rt_status ae_rt_get_fetch_counts(ae_rt_ctx* ctx, uint64_t* node_fetches, uint64_t* tri_fetches);

/* Device self-test of the traversal kernel's divide-free slab arithmetic:
 * compares it bit for bit with div.rn.f32 on n generated operand pairs from
 * the kernel's fast window (coordinates 0 or of magnitude 2^-40..2^40, ray
 * directions of magnitude 2^-40..2^40) and returns the mismatch count
 * (0 expected).  Diagnostic only; uses the context's fetch-count scratch. */
ae_rt_status ae_rt_selftest_division(ae_rt_ctx* ctx, uint64_t n, uint32_t seed, uint64_t* mismatches);

/* Device self-test of the path tracer's shading and intersection functions:
 * evaluates the very device functions the path tracer and the traversal use
 * on n host rows of inputs and copies the n output rows back (synchronous;
 * diagnostic only).  Row layouts (floats), the same as the golden vectors of
 * the reference's GLSL helpers:
 *   EVAL            in 15: V N L baseColor roughness metalness reflectance
 *                   out 16: diffuse(3) specular(3) NdotL NdotV NdotH LdotH F0(3) F90 H.x H.y
 *                   (UpdateSurface, EvaluateDiffuseBRDF / EvaluateSpecularBRDF,
 *                   brdf/surface.hsh:25-41, brdf/brdfEval.hsh:8-32)
 *   SAMPLE_DIFFUSE, SAMPLE_SPECULAR
 *                   in 17: the EVAL row (L ignored) + u0 u1
 *                   out 8: L(3) pdf reflectance(3) NdotL (brdf/brdfSample.hsh:8-90)
 *   TRIANGLE_LIGHT  in 24: v0 v1 v2 n0 n1 n2 area r0 r1 P(3)
 *                   out 7: P(3) N(3) pdf (raytracer/lights.hsh:11-29)
 *   EVAL_TERMS      in 13: NdotL NdotV NdotH LdotH F0(3) F90 baseColor(3) roughness metalness
 *                   out 6: diffuse(3) specular(3)
 *   TRIANGLE        in 15: origin direction v0 v1 v2; out 4: hit t u v
 *                   (IntersectTriangle, raytracer/intersections.hsh:36-57)
 *   AABB            in 14: origin direction min max tmin tmax; out 2: hit dist
 *                   (IntersectAABB, raytracer/intersections.hsh:18-34) */
#define AE_SELFTEST_EVAL 0u
#define AE_SELFTEST_SAMPLE_DIFFUSE 1u
#define AE_SELFTEST_SAMPLE_SPECULAR 2u
#define AE_SELFTEST_TRIANGLE_LIGHT 3u
#define AE_SELFTEST_EVAL_TERMS 4u
#define AE_SELFTEST_TRIANGLE 5u
#define AE_SELFTEST_AABB 6u
ae_rt_status ae_rt_selftest_shading(ae_rt_ctx* ctx, uint32_t kind, const float* in, uint32_t n, float* out);

#ifdef __cplusplus
}
#endif

#endif /* ATLAS_RT_H */
