/*
 * CPU restatement of Atlas Engine's BVH ray queries -- the ORACLE.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm load this library, and only to
 * check or time against; the product path (libatlas_rt.so) never links it.
 *
 * Two traversal semantics are restated, both over the engine's GPU buffer
 * layouts (64-byte GPUBVHNode, 48-byte GPUBVHTriangle, see
 * src/engine/raytracing/RTStructures.h:23-27, :95-103):
 *
 *   *_cpu   the host query  Volume::BVH::GetIntersection / GetIntersectionAny
 *           (src/engine/volume/BVH.cpp:103-217, Ray.cpp:28-76): slab test by
 *           multiplication with 1/dir, triangle accepted for t >= 0, glm
 *           min/max semantics.
 *   *_glsl  the shader query HitClosest / HitAny on one BLAS
 *           (data/shader/raytracer/bvh.hsh:44-104, :191-273, :359-441;
 *           intersections.hsh:3-57): slab test by division, near-child-first
 *           descent, triangle accepted for tmin < t < tmax.
 *
 * Rays are rows of 8 floats: origin.xyz, direction.xyz, tmin, tmax.
 */
#ifndef AE_ORACLE_H
#define AE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aeo_node {
    float lmin[3], lmax[3];
    float rmin[3], rmax[3];
    int32_t left, right, pad0, pad1;
} aeo_node;

typedef struct aeo_tri {
    float v0[4];  /* w > 0: last triangle of its leaf */
    float v1[4];
    float v2[4];
} aeo_tri;

/* The reference builder restated (oracle/ae_oracle_build.cpp, BVH.cpp:14-100,
 * :249-870): the triangle BVH (triangle i gets original index i) and the
 * AABB-only BVH of the top level (boxes: n * 6 floats, min then max).  The
 * handle holds the 64-byte nodes and, per BVH-order primitive, its original
 * index and end-of-leaf flag.  Empty input gives an empty tree. */
typedef struct aeo_bvh aeo_bvh;
aeo_bvh* aeo_build_triangles(const float* verts, uint32_t n_tris, int parallel);
aeo_bvh* aeo_build_aabbs(const float* boxes, uint32_t n, int parallel);
uint32_t aeo_bvh_node_count(const aeo_bvh* h);
uint32_t aeo_bvh_prim_count(const aeo_bvh* h);
void aeo_bvh_get(const aeo_bvh* h, aeo_node* nodes, uint32_t* order, uint8_t* end_of_node);
void aeo_bvh_free(aeo_bvh* h);

/* Host closest-hit query (BVH.cpp:103-174).  tri_ptr = BVH-order index of the
 * closest triangle or -1; tuv = (t, u, v) of that hit. */
void aeo_closest_cpu(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                     const float* rays, uint32_t n_rays, int threads,
                     int32_t* tri_ptr, float* tuv);

/* aeo_closest_glsl plus the GPU trace's near-tie flags (bit 0 hit, bit 1
 * near tie: a second accepted triangle within 4e-6 relative t, a rejected
 * box entered within that window of the bound, or a triangle rejected
 * within the rounding error of its barycentric tests) and its second
 * distance (the second smallest accepted t, tmax if none). */
void aeo_closest_glsl_ties(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                           const float* rays, uint32_t n_rays, int threads,
                           int32_t* tri_ptr, float* tuv, uint32_t* flags, float* t_second);

/* The restatement's shading and intersection functions on rows of inputs,
 * in the layouts of the golden vectors the reference's GLSL writes when
 * compiled on the host (oracle/glsl/glsl_capi.cpp). */
void aeo_shade_eval(const float* in, int n, float* out);
void aeo_shade_eval_terms(const float* in, int n, float* out);
void aeo_shade_sample(const float* in, int n, int specular, float* out);
void aeo_shade_triangle_light(const float* in, int n, float* out);
void aeo_shade_intersect_triangle(const float* in, int n, float* out);
void aeo_shade_intersect_aabb(const float* in, int n, float* out);

/* Host any-hit query (BVH.cpp:176-217); occluded[i] = 0/1. */
void aeo_any_cpu(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                 const float* rays, uint32_t n_rays, int threads, uint8_t* occluded);

/* Shader closest-hit query on one BLAS (bvh.hsh:191-273 with the TLAS level
 * collapsed to a single identity instance).  Outputs as aeo_closest_cpu plus
 * per-ray counts of inner nodes fetched and triangles tested (any counter
 * pointer may be NULL). */
void aeo_closest_glsl(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                      const float* rays, uint32_t n_rays, int threads,
                      int32_t* tri_ptr, float* tuv, uint32_t* node_fetches, uint32_t* tri_fetches);

/* Shader any-hit query on one BLAS (bvh.hsh:359-441). */
void aeo_any_glsl(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                  const float* rays, uint32_t n_rays, int threads, uint8_t* occluded,
                  uint32_t* node_fetches, uint32_t* tri_fetches);

/* Two-level scene (top level over instances): GPUBVHInstance
 * (RTStructures.h:85-93): m = mat3x4 columns = rows of the inverse model
 * matrix, objectPos[i] = dot(vec4(worldPos, 1), m[i]). */
typedef struct aeo_instance {
    float m[12];
    int32_t meshOffset, materialOffset, nextInstance;
    uint32_t mask;
} aeo_instance;

typedef struct aeo_mesh {
    const aeo_node* nodes;
    uint32_t n_nodes;
    const aeo_tri* tris;
    uint32_t n_tris;
    const float* shading;     /* GPUTriangle, 24 floats each (path tracer only) */
} aeo_mesh;

/* Shader closest-hit over TLAS + BLASes: HitClosest with CheckInstance
 * (bvh.hsh:172-273).  inst_out = hitInstanceID (-1 on a miss). */
void aeo_scene_closest_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, uint32_t n_inst,
                            const aeo_mesh* meshes, uint32_t n_meshes, const float* rays, uint32_t n_rays,
                            uint32_t cull_mask, int threads, int32_t* tri_ptr, int32_t* inst_out, float* tuv,
                            uint32_t* node_fetches, uint32_t* tri_fetches);

/* Shader any-hit over TLAS + BLASes: HitAny (bvh.hsh:359-441). */
void aeo_scene_any_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, uint32_t n_inst,
                        const aeo_mesh* meshes, uint32_t n_meshes, const float* rays, uint32_t n_rays,
                        uint32_t cull_mask, int threads, uint8_t* occluded);

/* One texture's level 0 (the layout of the library's ae_texture): `height`
 * rows of `row_pitch` bytes (0 = tight); format 0 = R8 UNORM, 1 = RGBA8
 * UNORM, 2 = R32 float; the first channel is sampled. */
typedef struct aeo_texture {
    const void* texels;
    uint32_t width, height, format, row_pitch;
    /* levels 1, 2, ... of the mip chain (tight rows), for the surface
     * lookups at a level > 0; NULL / 0 when only level 0 is given */
    const struct aeo_texture* mips;
    uint32_t n_mips;
} aeo_texture;

/* Path tracer -- the restatement of the engine's non-real-time estimator
 * (pathtracer/rayGen.csh, rayHit.csh, raytracer/direct.hsh, lights.hsh,
 * brdf/*.hsh) without the indirect radiance clamp, accumulating every sample's
 * radiance in double precision.  materials: GPUMaterial (23 words), lights:
 * GPULight (16 floats), inst_model: object-to-world 3x4 rows per instance,
 * textures: the materials' texture table (vertex colours, base colour,
 * opacity, roughness, metalness, ao, normal maps at level 0).
 * cam: location[3], origin[3], right[3], bottom[3].  accum: w * h * 3. */
void aeo_pathtrace(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, const float* inst_model,
                   uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes, const float* materials,
                   const float* lights, uint32_t n_lights, const aeo_texture* textures, uint32_t n_textures,
                   const float* cam, uint32_t width, uint32_t height,
                   uint32_t spp, uint32_t sample_offset, uint32_t max_bounces, uint32_t seed, float epsilon,
                   int threads, double* accum);
/* The same with a constant environment radiance env[3] added on a miss,
 * min(env * throughput, 10) per channel (rayHit.csh:166-171; NULL = none),
 * and the material count that the opacity check (used when a shading
 * triangle's opacity is not 1) bounds its material reads with. */
void aeo_pathtrace_env(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, const float* inst_model,
                       uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes, const float* materials,
                       uint32_t n_materials, const float* lights, uint32_t n_lights, const aeo_texture* textures,
                       uint32_t n_textures, const float* cam, uint32_t width, uint32_t height,
                       uint32_t spp, uint32_t sample_offset, uint32_t max_bounces, uint32_t seed, float epsilon,
                       const float* env, int threads, double* accum);


/* textureLod(sampler2D(bindlessTextures[id], bindlessSampler), (u, v), 0).r
 * (texture.hsh:18-25) with the engine's bindless sampler (linear filter,
 * repeat addressing, MainRenderer.cpp:922-929), in FP32 with one rounding
 * per operation: x = u * width - 0.5, i = floor(x), a = x - i, texels i and
 * i + 1 modulo width (likewise v), ((w00 c00 + w10 c10) + w01 c01) + w11 c11
 * with w00 = (1-a)(1-b), w10 = a(1-b), w01 = (1-a)b, w11 = ab; UNORM texels
 * are byte / 255; a non-finite x (or y) becomes 0 (texel 0 alone); a negative or
 * out-of-range id samples as 1.0. */
float aeo_sample_r_bilinear(const aeo_texture* textures, uint32_t n_textures, int32_t id, float u, float v);

/* IEEE binary16 bits to float (unpackHalf2x16 of one half). */
float aeo_half_to_float(uint16_t h);

/* The transparency variants over TLAS + BLASes (meshes need `shading`):
 * HitClosestTransparency (bvh.hsh:275-357: a hit counts only where the
 * triangle's opacity is > 0) and HitAnyTransparency (bvh.hsh:443-524: the
 * returned transparency, 1 = unoccluded).  Opacity: GPUTriangle d2.w, or,
 * when negative, GetOpacity (surface.hsh:147-159): the material's opacity
 * (materials: GPUMaterial, 23 words, indexed by the triangle's material
 * index + the instance's materialOffset; outside [0, n_materials) the
 * opacity is 1) times its opacity texture sampled at the UV interpolated
 * from the triangle's half2 UVs, v flipped when invertUVs > 0. */
void aeo_scene_closest_transparency_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst,
                                         uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes,
                                         const float* materials, uint32_t n_materials,
                                         const aeo_texture* textures, uint32_t n_textures, const float* rays,
                                         uint32_t n_rays, uint32_t cull_mask, int threads, int32_t* tri_ptr,
                                         int32_t* inst_out, float* tuv);
void aeo_scene_any_transparency_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst,
                                     uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes,
                                     const float* materials, uint32_t n_materials, const aeo_texture* textures,
                                     uint32_t n_textures, const float* rays, uint32_t n_rays, uint32_t cull_mask,
                                     int threads, float* transparency);

/* The traversal's other consumers -- ao/rtao.csh, reflection/rtreflection.csh,
 * rtgi/rtgi.csh, ddgi/rayGen.csh + rayHit.csh -- restated per pixel / probe
 * ray with the library's random streams (pixel samples: `samples` if given,
 * else the engine's SampleBlueNoise over the two blue-noise textures if
 * given, else PCG hash slot 13 of (pixel, frame_seed); light choices: slot 14 keyed
 * by the pixel or probe-ray index).  Structs mirror the library's
 * ae_gbuffer, ae_rt_pass_params and ae_ddgi_probes (host memory here). */
typedef struct aeo_gbuffer {
    const float* depth;
    const float* normal;
    const uint8_t* offset;
    const float* roughness;
    const float* samples;
    uint32_t width, height, half_res, reserved;
    float ip_matrix[16], iv_matrix[16];
    const uint8_t* scrambling_ranking;   /* blue-noise textures, RGBA8: 128 x 128 */
    const uint8_t* sobol_sequence;       /* and 256 x 1 (used when samples is NULL) */
} aeo_gbuffer;

typedef struct aeo_pass_params {
    float radius, bias, roughness_cutoff, radiance_limit;
    float environment[3];
    uint32_t flags;        /* 1: opacity check (transparency traversals) */
    uint32_t frame_seed, seed;
    uint32_t texture_level, reserved;   /* reflections / RTGI surface textures; DDGI reads level 4 */
} aeo_pass_params;

typedef struct aeo_ddgi_probes {
    const float* probes;
    const float* ray_dirs;
    const float* ray_dirs_inactive;
    float rotation[16];
    uint32_t n_probes, ray_count, inactive_ray_count, reserved;
} aeo_ddgi_probes;

/* The scene of the passes: TLAS, instances (+ object-to-world 3x4 rows),
 * meshes with shading triangles, materials, opacity textures, lights. */
typedef struct aeo_pass_scene {
    const aeo_node* tlas; uint32_t n_tlas;
    const aeo_instance* inst; const float* inst_model; uint32_t n_inst;
    const aeo_mesh* meshes; uint32_t n_meshes;
    const float* materials; uint32_t n_materials;
    const aeo_texture* textures; uint32_t n_textures;
    const float* lights; uint32_t n_lights;
} aeo_pass_scene;

void aeo_pass_rtao(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                   float* ao);
void aeo_pass_reflections(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                          float* rgba);
void aeo_pass_rtgi(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                   float* rgba);
void aeo_pass_ddgi(const aeo_pass_scene* s, const aeo_ddgi_probes* dp, const aeo_pass_params* pp, int threads,
                   float* hits);

/* Exact-as-possible nearest hit in double precision by brute force over every
 * triangle (for small cases and for re-testing near ties): the double-precision
 * form of the same triangle test, accepting tmin < t < tmax.  t2 = second
 * smallest accepted t (or +inf). */
void aeo_closest_f64_brute(const aeo_tri* tris, uint32_t n_tris, const float* rays, uint32_t n_rays,
                           int threads, int32_t* tri_ptr, double* t, double* t2);

#ifdef __cplusplus
}
#endif

#endif
