// C entry points over the reference's GLSL shading helpers compiled on the
// host (oracle/glsl/make_ref.py) -- TEST INFRASTRUCTURE ONLY: the golden
// generator calls them; nothing on the product path links this.
//
// Each function takes n packed input rows and writes n packed output rows of
// floats, evaluating the reference's own code:
//   CreateSurface / UpdateSurface            brdf/surface.hsh:25-57
//   EvaluateDiffuseBRDF / EvaluateSpecularBRDF  brdf/brdfEval.hsh:8-32
//   SampleDiffuseBRDF / SampleSpecularBRDF   brdf/brdfSample.hsh:8-90
//   SampleTriangleLight                      raytracer/lights.hsh:11-29
//   IntersectAABB / IntersectTriangle        raytracer/intersections.hsh:18-57
//   random(x, inout seed)                    common/random.hsh:5-54
//   HitClosest / HitAny / HitClosestTransparency / HitAnyTransparency over a
//   two-level scene (TLAS, instances, per-mesh BLAS, materials, opacity
//   textures)                                raytracer/bvh.hsh:44-524
//   the path tracer's ray generation, every invocation of one dispatch
//                                            pathtracer/rayGen.csh:25-91
//   the engine's path tracer, sample by sample: rayGen.csh, the trace
//   dispatch (traceClosest.csh:12-36) and the hit shader, bounce by bounce
//                                            pathtracer/rayHit.csh:54-338
//   the ambient-occlusion pass, one dispatch over a G-buffer (with and
//   without OPACITY_CHECK), and its blue-noise sampler
//                                            ao/rtao.csh:40-112,
//                                            common/bluenoise.hsh:9-32
//   the reflection and diffuse GI passes, one dispatch each (with and
//   without OPACITY_CHECK)              reflection/rtreflection.csh:60-245,
//                                            rtgi/rtgi.csh:60-234
//   the DDGI probe rays: ray generation, the trace dispatch and the hit
//   shader                               ddgi/rayGen.csh:39-81,
//                                            ddgi/rayHit.csh:37-151
#include "glsl.hpp"
#include "glsl_ref.inc"
#include "glsl_raygen.inc"
#include "glsl_pt.inc"
#include "glsl_rtao.inc"
#include "glsl_rtao_opacity.inc"
#include "glsl_rtr.inc"
#include "glsl_rtr_opacity.inc"
#include "glsl_rtgi.inc"
#include "glsl_rtgi_opacity.inc"
#include "glsl_ddgi_raygen.inc"
#include "glsl_ddgi.inc"

using namespace aeg_glsl;

#include <vector>

namespace {

// Row layout of a surface: V(3) N(3) L(3) baseColor(3) roughness metalness reflectance
constexpr int kSurfaceIn = 15;

Material MakeMaterial(const float* r) {
    Material m;
    m.baseColor = vec3(r[9], r[10], r[11]);
    m.roughness = r[12];
    m.metalness = r[13];
    m.reflectance = r[14];
    m.opacity = 1.0f;
    m.ao = 1.0f;
    return m;
}

vec3 V3(const float* p) { return vec3(p[0], p[1], p[2]); }
void Put(float* o, const vec3& v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

}  // namespace

extern "C" {

// in: kSurfaceIn floats per row.  out per row (16): diffuse(3) specular(3)
// NdotL NdotV NdotH LdotH F0(3) F90 H.xy
void aeglsl_eval(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + i * kSurfaceIn;
        Surface s = CreateSurface(V3(r), V3(r + 3), V3(r + 6), MakeMaterial(r));
        float* o = out + i * 16;
        Put(o, EvaluateDiffuseBRDF(s));
        Put(o + 3, EvaluateSpecularBRDF(s));
        o[6] = s.NdotL; o[7] = s.NdotV; o[8] = s.NdotH; o[9] = s.LdotH;
        Put(o + 10, s.F0);
        o[13] = s.F90;
        o[14] = s.H.x; o[15] = s.H.y;
    }
}

// in: kSurfaceIn floats (L ignored) + u0 u1 per row.  out per row (8):
// L(3) pdf reflectance(3) NdotL.  specular: SampleSpecularBRDF, else diffuse.
void aeglsl_sample(const float* in, int n, int specular, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + i * (kSurfaceIn + 2);
        Surface s = CreateSurface(V3(r), V3(r + 3), V3(r + 3), MakeMaterial(r));
        const vec2 u(r[kSurfaceIn], r[kSurfaceIn + 1]);
        BRDFSample b = specular ? SampleSpecularBRDF(s, u) : SampleDiffuseBRDF(s, u);
        float* o = out + i * 8;
        Put(o, s.L);
        o[3] = b.pdf;
        Put(o + 4, b.reflectance);
        o[7] = s.NdotL;
    }
}

// in per row (24): v0 v1 v2 n0 n1 n2 (18) area r0 r1 P(3, the shaded point,
// unused by the sample).  out per row (7): P(3) N(3) pdf.
void aeglsl_triangle_light(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + i * 24;
        Triangle t;
        t.v0 = V3(r); t.v1 = V3(r + 3); t.v2 = V3(r + 6);
        t.n0 = V3(r + 9); t.n1 = V3(r + 12); t.n2 = V3(r + 15);
        Light l;
        l.area = r[18];
        Surface s;
        s.P = V3(r + 21);
        LightSample ls = SampleTriangleLight(l, t, s, r[19], r[20]);
        float* o = out + i * 7;
        Put(o, ls.P);
        Put(o + 3, ls.N);
        o[6] = ls.pdf;
    }
}

// in per row (15): origin(3) direction(3) v0(3) v1(3) v2(3); out (4): hit, t, u, v.
void aeglsl_intersect_triangle(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + i * 15;
        Ray ray;
        ray.origin = V3(r);
        ray.direction = V3(r + 3);
        vec3 sol;
        const bool hit = IntersectTriangle(ray, V3(r + 6), V3(r + 9), V3(r + 12), sol);
        float* o = out + i * 4;
        o[0] = hit ? 1.0f : 0.0f;
        o[1] = sol.x; o[2] = sol.y; o[3] = sol.z;
    }
}

// in per row (14): origin(3) direction(3) min(3) max(3) tmin tmax; out (2): hit, dist.
void aeglsl_intersect_aabb(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + i * 14;
        Ray ray;
        ray.origin = V3(r);
        ray.direction = V3(r + 3);
        AABB box;
        box.min = V3(r + 6);
        box.max = V3(r + 9);
        float dist = 0.0f;
        const bool hit = IntersectAABB(ray, box, r[12], r[13], dist);
        out[i * 2] = hit ? 1.0f : 0.0f;
        out[i * 2 + 1] = dist;
    }
}

// The scene the traversals read, in the engine's GPU layouts (64-byte
// nodes and instances, 48-byte BVH triangles, 96-byte triangles, 92-byte
// materials), and its opacity textures as RGBA float texels (width, height
// per texture in wh).  The arrays stay owned by the caller.
static std::vector<glsl_texture2D> g_textures;

void aeglsl_scene(const void* tlas, const void* instances, int n_meshes, const void* const* nodes,
                  const void* const* bvh_tris, const void* const* tris, const void* mats, int n_textures,
                  const float* const* texels, const int* wh) {
    tlasNodes = (PackedBVHNode*)tlas;
    bvhInstances = (Instance*)instances;
    for (int m = 0; m < n_meshes; m++) {
        blasNodes[m].data = (PackedBVHNode*)nodes[m];
        bvhTriangles[m].data = (PackedBVHTriangle*)bvh_tris[m];
        triangles[m].data = (PackedTriangle*)tris[m];
    }
    materials = (RaytraceMaterial*)mats;
    g_textures.assign(size_t(n_textures), glsl_texture2D());
    for (int i = 0; i < n_textures; i++) {
        g_textures[i].texels = texels[i];
        g_textures[i].width = wh[2 * i];
        g_textures[i].height = wh[2 * i + 1];
    }
    bindlessTextures = g_textures.data();
    // the ambient-occlusion programs trace the same scene
#define AEG_SCENE_INTO(T)                                                  \
    T::tlasNodes = (T::PackedBVHNode*)tlas;                                \
    T::bvhInstances = (T::Instance*)instances;                             \
    for (int m = 0; m < n_meshes; m++) {                                   \
        T::blasNodes[m].data = (T::PackedBVHNode*)nodes[m];                \
        T::bvhTriangles[m].data = (T::PackedBVHTriangle*)bvh_tris[m];      \
        T::triangles[m].data = (T::PackedTriangle*)tris[m];                \
    }                                                                      \
    T::materials = (T::RaytraceMaterial*)mats;                             \
    T::bindlessTextures = g_textures.data();
    AEG_SCENE_INTO(aeg_rtao)
    AEG_SCENE_INTO(aeg_rtao_opacity)
    AEG_SCENE_INTO(aeg_rtr)
    AEG_SCENE_INTO(aeg_rtr_opacity)
    AEG_SCENE_INTO(aeg_rtgi)
    AEG_SCENE_INTO(aeg_rtgi_opacity)
    AEG_SCENE_INTO(aeg_ddgi)
#undef AEG_SCENE_INTO
}

// The light list (GPULight, 64 bytes each) of the shading passes' programs.
void aeglsl_scene_lights(const void* lights, int n_lights) {
#define AEG_LIGHTS_INTO(T)                                                 \
    T::lights = (T::PackedLight*)lights;                                   \
    T::PushConstants.lightCount = n_lights;
    AEG_LIGHTS_INTO(aeg_rtr)
    AEG_LIGHTS_INTO(aeg_rtr_opacity)
    AEG_LIGHTS_INTO(aeg_rtgi)
    AEG_LIGHTS_INTO(aeg_rtgi_opacity)
    AEG_LIGHTS_INTO(aeg_ddgi)
#undef AEG_LIGHTS_INTO
}

// kind 0 HitClosest, 1 HitAny, 2 HitClosestTransparency, 3 HitAnyTransparency
// over rows origin(3) direction(3) tmin tmax; out per row (4): hitID and
// hitInstanceID (int bits), hitDistance, and HitAny's result (0 / 1) or
// HitAnyTransparency's transparency.  A ray starts with hitID and
// hitInstanceID -1, as the engine's ray queue writes them (tracing.hsh).
void aeglsl_scene_trace(int kind, const float* rays, int n, uint cull, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = rays + i * 8;
        Ray ray;
        ray.ID = i;
        ray.origin = V3(r);
        ray.direction = V3(r + 3);
        ray.hitID = -1;
        ray.hitInstanceID = -1;
        ray.currentInstanceID = -1;
        ray.hitDistance = 0.0f;
        float value = 0.0f;
        switch (kind) {
        case 0: HitClosest(ray, cull, r[6], r[7]); break;
        case 1: value = HitAny(ray, cull, r[6], r[7]) ? 1.0f : 0.0f; break;
        case 2: HitClosestTransparency(ray, cull, r[6], r[7]); break;
        default: value = HitAnyTransparency(ray, cull, r[6], r[7]); break;
        }
        float* o = out + i * 4;
        o[0] = intBitsToFloat(ray.hitID);
        o[1] = intBitsToFloat(ray.hitInstanceID);
        o[2] = ray.hitDistance;
        o[3] = value;
    }
}

// One dispatch of rayGen.csh (not REALTIME) over a tile of the image, the
// engine's 8 x 8 work groups run invocation by invocation.  cam: origin(4)
// right(4) bottom(4) location(4); ints: resolution(2) pixelOffset(2)
// tileSize(2) sampleCount.  out: capacity PackedRays (12 floats each),
// written where the shader writes them; returns the rays written (the
// shader's write counter).
int aeglsl_raygen(const float* cam, const int* ints, float* out, int capacity) {
    namespace R = aeg_raygen;
    R::Uniforms.origin = vec4(cam[0], cam[1], cam[2], cam[3]);
    R::Uniforms.right = vec4(cam[4], cam[5], cam[6], cam[7]);
    R::Uniforms.bottom = vec4(cam[8], cam[9], cam[10], cam[11]);
    R::globalData.cameraLocation = vec4(cam[12], cam[13], cam[14], cam[15]);
    R::Uniforms.resolution = ivec2(ints[0], ints[1]);
    R::Uniforms.pixelOffset = ivec2(ints[2], ints[3]);
    R::Uniforms.tileSize = ivec2(ints[4], ints[5]);
    R::Uniforms.sampleCount = ints[6];
    R::PushConstants.rayBufferOffset = 0;
    R::PushConstants.rayBufferSize = uint(capacity);
    R::PushConstants.useRayBinning = 0;
    R::rays = reinterpret_cast<R::PackedRay*>(out);
    static uint counter[1];
    counter[0] = 0u;
    R::writeAtomic = counter;
    const uint gx = uint((ints[4] + 7) / 8), gy = uint((ints[5] + 7) / 8);
    gl_NumWorkGroups = uvec3(gx, gy, 1u);
    for (uint wy = 0; wy < gy; wy++)
        for (uint wx = 0; wx < gx; wx++)
            for (uint ly = 0; ly < 8u; ly++)
                for (uint lx = 0; lx < 8u; lx++) {
                    gl_WorkGroupID = uvec3(wx, wy, 0u);
                    gl_LocalInvocationID = uvec3(lx, ly, 0u);
                    gl_GlobalInvocationID = uvec3(wx * 8u + lx, wy * 8u + ly, 0u);
                    gl_LocalInvocationIndex = ly * 8u + lx;
                    R::aeg_raygen_main();
                }
    return int(counter[0]);
}

// random(vec2(x, y)) of common/random.hsh: the per-frame sub-pixel jitter of
// rayGen.csh is random(vec2(sampleCount, 0)), random(vec2(sampleCount, 1)).
float aeglsl_random2(float x, float y) { return random(vec2(x, y)); }

// The scene of the reference's hit shader (rayHit.csh's program): the same
// layouts as aeglsl_scene, plus the light list (GPULight, 64 bytes each).
// No textures (every material's texture indices must be -1) and a black
// environment.  The arrays stay owned by the caller.
void aeglsl_pt_scene(const void* tlas, const void* instances, int n_meshes, const void* const* nodes,
                     const void* const* bvh_tris, const void* const* tris, const void* mats, const void* lights,
                     int n_lights) {
    namespace T = aeg_pt;
    T::tlasNodes = (T::PackedBVHNode*)tlas;
    T::bvhInstances = (T::Instance*)instances;
    for (int m = 0; m < n_meshes; m++) {
        T::blasNodes[m].data = (T::PackedBVHNode*)nodes[m];
        T::bvhTriangles[m].data = (T::PackedBVHTriangle*)bvh_tris[m];
        T::triangles[m].data = (T::PackedTriangle*)tris[m];
    }
    T::materials = (T::RaytraceMaterial*)mats;
    T::lights = (T::PackedLight*)lights;
    T::PushConstants.lightCount = n_lights;
}

// `spp` samples of the engine's path tracer (not REALTIME) over a w x h image:
// per sample, rayGen.csh (sampleCount = first_sample + s), then per bounce the
// trace dispatch (traceClosest.csh: hitID = -1, HitClosest -- or
// HitClosestTransparency with opacity_check -- from 0 to INF) and the hit
// shader over the queue, the two ray / payload halves swapping as the
// engine's buffers do.  seeds: the hit shader's Uniforms.seed per sample and
// bounce ((max_bounces + 1) per sample; the engine draws them uniformly).
// accum: w * h float4, the radiance sums and sample counts (outAccumImage);
// it must hold the previous samples' sums when first_sample > 0.
void aeglsl_pt_render(const float* cam, int w, int h, int spp, int first_sample, int max_bounces,
                      int opacity_check, const float* seeds, float* accum) {
    namespace T = aeg_pt;
    const int n_pix = w * h;
    std::vector<T::PackedRay> ray_buf(size_t(2) * n_pix);
    std::vector<T::PackedRayPayload> pay_buf(size_t(2) * n_pix);
    std::vector<vec4> out_image(static_cast<size_t>(n_pix));
    static uint read_count[1], write_count[1];
    T::rays = ray_buf.data();
    T::rayPayloads = pay_buf.data();
    T::readAtomic = read_count;
    T::writeAtomic = write_count;
    T::inAccumImage.texels = reinterpret_cast<vec4*>(accum);
    T::inAccumImage.width = w;
    T::outAccumImage = T::inAccumImage;
    T::outputImage.texels = out_image.data();
    T::outputImage.width = w;
    for (int s = 0; s < spp; s++) {
        const int sample = first_sample + s;
        const int ints[7] = { w, h, 0, 0, w, h, sample };
        aeglsl_raygen(cam, ints, reinterpret_cast<float*>(ray_buf.data()), n_pix);
        int cur = 0;
        uint n = uint(n_pix);
        for (int b = 0; b <= max_bounces && n > 0; b++) {
            for (uint i = 0; i < n; i++) {
                T::Ray r = T::UnpackRay(ray_buf[size_t(cur) * n_pix + i]);
                r.hitID = -1;
                r.hitDistance = 0.0f;
                if (r.ID >= 0) {
                    if (opacity_check) T::HitClosestTransparency(r, INSTANCE_MASK_ALL, 0.0f, INF);
                    else T::HitClosest(r, INSTANCE_MASK_ALL, 0.0f, INF);
                }
                ray_buf[size_t(cur) * n_pix + i] = T::PackRay(r);
            }
            T::Uniforms.resolution = ivec2(w, h);
            T::Uniforms.maxBounces = max_bounces;
            T::Uniforms.sampleCount = sample;
            T::Uniforms.bounceCount = b;
            T::Uniforms.seed = seeds[s * (max_bounces + 1) + b];
            T::Uniforms.exposure = 1.0f;
            T::Uniforms.samplesPerFrame = 1;
            T::Uniforms.maxRadiance = 1.0f;
            T::PushConstants.rayBufferOffset = uint(1 - cur);
            T::PushConstants.rayPayloadBufferOffset = uint(1 - cur);
            T::PushConstants.rayBufferSize = uint(n_pix);
            T::PushConstants.useRayBinning = 0;
            read_count[0] = n;
            write_count[0] = 0u;
            for (uint i = 0; i < n; i++) {
                gl_GlobalInvocationID = uvec3(i, 0u, 0u);
                T::aeg_pt_main();
            }
            n = write_count[0];
            cur = 1 - cur;
        }
    }
}

namespace {

// A texture of RGBA float texels holding one or two channels per pixel.
glsl_texture2D Plane(std::vector<float>& texels, const float* src, int channels, int w, int h) {
    texels.assign(size_t(w) * h * 4, 0.0f);
    for (size_t i = 0; i < size_t(w) * h; i++) {
        for (int c = 0; c < channels; c++) texels[i * 4 + c] = src[i * channels + c];
        texels[i * 4 + 3] = 1.0f;
    }
    glsl_texture2D t;
    t.texels = texels.data();
    t.width = w;
    t.height = h;
    return t;
}

glsl_texture2D Rgba(const float* texels, int w, int h) {
    glsl_texture2D t;
    t.texels = texels;
    t.width = w;
    t.height = h;
    return t;
}

mat4 ColumnMajor(const float* m) {
    mat4 r(1.0f);
    for (int c = 0; c < 4; c++) r.c[c] = vec4(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
    return r;
}

}  // namespace

// One dispatch of ao/rtao.csh over a w x h G-buffer, as AORenderer.cpp:85-114
// issues it: ceil(w / 8) * ceil(h / 4) work groups of 8 x 4 invocations in a
// row, which the shader lays onto tiles four groups wide; pixels that no
// invocation reaches keep their value in `ao`.  Over the scene aeglsl_scene
// set (HitAny, or HitAnyTransparency with opacity_check).
//   depth   w * h floats (the depth texture's r; read with texelFetch)
//   normal  w * h * 2 floats, octahedral (the normal texture's rg; read with
//           textureLod at the texel's centre through the render target's
//           sampler: clamp to edge, 8-bit sub-texel filter weights)
//   offset  w * h ints, 0..3 (the offset texture; texelFetch)
//   ranking 128 * 128 and sobol 256 RGBA float texels (c / 255 of the
//           engine's RGBA8 blue-noise textures)
//   ip, iv  column-major inverse projection and inverse view
//   ao      w * h floats, in / out
void aeglsl_rtao(int opacity_check, int w, int h, const float* depth, const float* normal, const int* offset,
                 const float* ranking, const float* sobol, const float* ip, const float* iv, float radius,
                 int frame_seed, float* ao) {
    std::vector<float> depth_texels, normal_texels;
    const glsl_texture2D depth_tex = Plane(depth_texels, depth, 1, w, h);
    const glsl_texture2D normal_tex = Plane(normal_texels, normal, 2, w, h);
    const glsl_texture2D rank_tex = Rgba(ranking, 128, 128), sobol_tex = Rgba(sobol, 256, 1);
    std::vector<vec4> image(size_t(w) * h);
    for (size_t i = 0; i < image.size(); i++) image[i] = vec4(ao[i], 0.0f, 0.0f, 0.0f);
    const int gx = (w + 7) / 8, gy = (h + 3) / 4;
#define AEG_RTAO_RUN(T)                                                                    \
    T::rtaoImage.texels = image.data();                                                    \
    T::rtaoImage.width = w;                                                                \
    T::rtaoImage.height = h;                                                               \
    T::normalTexture.tex = &normal_tex;                                                    \
    T::normalTexture.clamp_to_edge = true;                                                 \
    T::normalTexture.subtexel_bits = 8;                                                    \
    T::shadowMap.tex = &depth_tex;                                                         \
    T::offsetTexture.texels = offset;                                                      \
    T::offsetTexture.width = w;                                                            \
    T::offsetTexture.height = h;                                                           \
    T::scramblingRankingTexture.tex = &rank_tex;                                           \
    T::sobolSequenceTexture.tex = &sobol_tex;                                              \
    T::uniforms.radius = radius;                                                           \
    T::uniforms.frameSeed = frame_seed;                                                    \
    T::globalData.ipMatrix = ColumnMajor(ip);                                              \
    T::globalData.ivMatrix = ColumnMajor(iv);                                              \
    gl_NumWorkGroups = uvec3(uint(gx * gy), 1u, 1u);                                       \
    for (int g = 0; g < gx * gy; g++)                                                      \
        for (uint ly = 0; ly < 4u; ly++)                                                   \
            for (uint lx = 0; lx < 8u; lx++) {                                             \
                gl_WorkGroupID = uvec3(uint(g), 0u, 0u);                                   \
                gl_LocalInvocationID = uvec3(lx, ly, 0u);                                  \
                gl_LocalInvocationIndex = ly * 8u + lx;                                    \
                gl_GlobalInvocationID = uvec3(uint(g) * 8u + lx, ly, 0u);                  \
                T::T##_main();                                                             \
            }
    if (opacity_check) {
        AEG_RTAO_RUN(aeg_rtao_opacity)
    } else {
        AEG_RTAO_RUN(aeg_rtao)
    }
#undef AEG_RTAO_RUN
    for (size_t i = 0; i < image.size(); i++) ao[i] = image[i].x;
}

// One dispatch of reflection/rtreflection.csh (kind 0) or rtgi/rtgi.csh
// (kind 1) over a w x h G-buffer, as RTReflectionRenderer.cpp:107-135 issues
// it: ceil(w / 8) x ceil(h / 4) work groups of 8 x 4 over the pixels; over the
// scene and lights of aeglsl_scene / aeglsl_scene_lights (HitClosest, or
// HitClosestTransparency with opacity_check; shadows by HitAnyTransparency).
// The G-buffer planes as in aeglsl_rtao, plus roughness (w * h floats: the
// r channel of roughnessMetallicAoTexture); the pixel's material is a packed
// material of roughness 1 with a roughness map, so its roughness is the
// plane's (rtreflection.csh:92-96).  params: radianceLimit, bias,
// roughnessCutoff and the environment's colour (r, g, b).  out: w * h * 4
// floats (rtrImage), in / out.
void aeglsl_screen_pass(int kind, int opacity_check, int w, int h, int half_res, const float* depth,
                        const float* normal, const int* offset, const float* roughness, const float* ranking,
                        const float* sobol, const float* ip, const float* iv, const float* params, uint frame_seed,
                        float* out) {
    std::vector<float> depth_texels, normal_texels, rough_texels;
    const glsl_texture2D depth_tex = Plane(depth_texels, depth, 1, w, h);
    const glsl_texture2D normal_tex = Plane(normal_texels, normal, 2, w, h);
    const glsl_texture2D rough_tex = Plane(rough_texels, roughness, 1, w, h);
    const glsl_texture2D rank_tex = Rgba(ranking, 128, 128), sobol_tex = Rgba(sobol, 256, 1);
    std::vector<uint> material_idx(size_t(w) * h, 0u);
    // packUnorm 10:10:10:2 of (opacity 0, roughness 1, metalness 0) and the
    // roughness-map feature bit (common/material.hsh:52-92)
    static uint packed_material[8];
    packed_material[4] = 1023u << 10;
    packed_material[7] = 1u << 4;
    std::vector<vec4> image(size_t(w) * h);
    for (size_t i = 0; i < image.size(); i++) image[i] = vec4(out[4 * i], out[4 * i + 1], out[4 * i + 2], out[4 * i + 3]);
    const int gx = (w + 7) / 8, gy = (h + 3) / 4;
#define AEG_SCREEN_RUN(T)                                                                  \
    T::rtrImage.texels = image.data();                                                     \
    T::rtrImage.width = w;                                                                 \
    T::rtrImage.height = h;                                                                \
    T::normalTexture.tex = &normal_tex;                                                    \
    T::normalTexture.clamp_to_edge = true;                                                 \
    T::normalTexture.subtexel_bits = 8;                                                    \
    T::depthTexture.tex = &depth_tex;                                                      \
    T::roughnessMetallicAoTexture.tex = &rough_tex;                                        \
    T::offsetTexture.texels = offset;                                                      \
    T::offsetTexture.width = w;                                                            \
    T::offsetTexture.height = h;                                                           \
    T::materialIdxTexture.texels = material_idx.data();                                    \
    T::materialIdxTexture.width = w;                                                       \
    T::materialIdxTexture.height = h;                                                      \
    T::packedMaterials = reinterpret_cast<T::PackedMaterial*>(packed_material);            \
    T::scramblingRankingTexture.tex = &rank_tex;                                           \
    T::sobolSequenceTexture.tex = &sobol_tex;                                              \
    T::environmentMap.constant = vec4(params[3], params[4], params[5], 1.0f);              \
    T::uniforms.radianceLimit = params[0];                                                 \
    T::uniforms.bias = params[1];                                                          \
    T::uniforms.roughnessCutoff = params[2];                                               \
    T::uniforms.frameSeed = frame_seed;                                                    \
    T::uniforms.textureLevel = 0;                                                          \
    T::uniforms.halfRes = half_res;                                                        \
    T::uniforms.resolution = ivec2(w, h);                                                  \
    T::globalData.ipMatrix = ColumnMajor(ip);                                              \
    T::globalData.ivMatrix = ColumnMajor(iv);                                              \
    gl_NumWorkGroups = uvec3(uint(gx), uint(gy), 1u);                                      \
    for (int by = 0; by < gy; by++)                                                        \
        for (int bx = 0; bx < gx; bx++)                                                    \
            for (uint ly = 0; ly < 4u; ly++)                                               \
                for (uint lx = 0; lx < 8u; lx++) {                                         \
                    gl_WorkGroupID = uvec3(uint(bx), uint(by), 0u);                        \
                    gl_LocalInvocationID = uvec3(lx, ly, 0u);                              \
                    gl_LocalInvocationIndex = ly * 8u + lx;                                \
                    gl_GlobalInvocationID = uvec3(uint(bx) * 8u + lx, uint(by) * 4u + ly, 0u); \
                    T::T##_main();                                                         \
                }
    if (kind == 0) {
        if (opacity_check) { AEG_SCREEN_RUN(aeg_rtr_opacity) } else { AEG_SCREEN_RUN(aeg_rtr) }
    } else {
        if (opacity_check) { AEG_SCREEN_RUN(aeg_rtgi_opacity) } else { AEG_SCREEN_RUN(aeg_rtgi) }
    }
#undef AEG_SCREEN_RUN
    for (size_t i = 0; i < image.size(); i++)
        for (int c = 0; c < 4; c++) out[4 * i + c] = image[i].v[c];
}

// One DDGI probe-ray pass as DDGIRenderer.cpp:93-175 issues it, one cascade:
// ddgi/rayGen.csh over grid[0] x grid[1] x grid[2] work groups of 32, the
// trace dispatch (traceClosest.csh:12-36: HitClosest, or HitClosestTransparency
// with opacity_check, from 0 to INF) and ddgi/rayHit.csh over every ray slot,
// over the scene and lights of aeglsl_scene / aeglsl_scene_lights.  The
// hit shader's irradiance volume is given an empty box (volumeMax below
// volumeMin), so IsInsideVolume is false and no indirect term is added.
//   volume_min, cell_size  3 floats each (cascade 0)
//   states     one PROBE_STATE_* per probe, offsets 4 floats per probe (the
//              history buffers; probes in the engine's order,
//              Flatten3D(probe.xzy))
//   dirs / dirs_inactive  ray_count / inactive_count x 4 floats
//   rotation   16 floats, column-major (Uniforms.randomRotation)
//   env        the environment's colour; seed: the hit shader's Uniforms.seed
//   origins    out: 4 floats per probe, the origin of its rays
//   hits       n_probes * ray_count x 4 floats (PackedRayHit), in / out;
//              slots past a probe's ray count keep their value
void aeglsl_ddgi(const int* grid, const float* volume_min, const float* cell_size, uint ray_count,
                 uint inactive_count, const uint* states, const float* offsets, const float* dirs,
                 const float* dirs_inactive, const float* rotation, int opacity_check, const float* env, float seed,
                 float* origins, float* hits) {
    namespace R = aeg_ddgi_rg;
    namespace H = aeg_ddgi;
    const int nx = grid[0], ny = grid[1], nz = grid[2], n = nx * ny * nz;
    const uint total = uint(n) * ray_count;
    std::vector<R::PackedRay> rays(size_t(2) * total);
    std::vector<vec4> history_states(static_cast<size_t>(n)), zeros(static_cast<size_t>(n), vec4(0.0f));
    for (int p = 0; p < n; p++) history_states[p] = vec4(uintBitsToFloat(states[p]), 0.0f, 0.0f, 0.0f);
    static uint read_count[1], write_count[1];
    auto volume = [&](auto& d, bool empty) {
        d.cascades[0].volumeMin = vec4(volume_min[0], volume_min[1], volume_min[2], 0.0f);
        d.cascades[0].cellSize = vec4(cell_size[0], cell_size[1], cell_size[2], 0.0f);
        d.cascades[0].volumeMax = empty ? vec4(volume_min[0] - 1.0f, volume_min[1] - 1.0f, volume_min[2] - 1.0f, 0.0f)
                                        : vec4(volume_min[0] + cell_size[0] * float(nx - 1),
                                               volume_min[1] + cell_size[1] * float(ny - 1),
                                               volume_min[2] + cell_size[2] * float(nz - 1), 0.0f);
        d.cascades[0].offsetDifference = ivec4(0, 0, 0, 0);
        d.volumeProbeCount = ivec4(nx, ny, nz, n);
        d.cascadeCount = 1;
        d.rayCount = ray_count;
        d.inactiveRayCount = inactive_count;
    };
    // ray generation into the first half of the ray buffer
    volume(R::ddgiData, false);
    R::rayDirs = reinterpret_cast<vec4*>(const_cast<float*>(dirs));
    R::rayDirsInactiveProbes = reinterpret_cast<vec4*>(const_cast<float*>(dirs_inactive));
    R::historyProbeStates = history_states.data();
    R::historyProbeOffsets = reinterpret_cast<vec4*>(const_cast<float*>(offsets));
    R::Uniforms.randomRotation = ColumnMajor(rotation);
    R::rays = rays.data();
    R::readAtomic = read_count;
    R::writeAtomic = write_count;
    R::PushConstants.rayBufferOffset = 0u;
    R::PushConstants.rayBufferSize = total;
    R::PushConstants.useRayBinning = 0;
    write_count[0] = 0u;
    gl_NumWorkGroups = uvec3(uint(nx), uint(ny), uint(nz));
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++)
                for (uint l = 0; l < 32u; l++) {
                    gl_WorkGroupID = uvec3(uint(x), uint(y), uint(z));
                    gl_LocalInvocationID = uvec3(l, 0u, 0u);
                    gl_LocalInvocationIndex = l;
                    gl_GlobalInvocationID = uvec3(uint(x) * 32u + l, uint(y), uint(z));
                    R::aeg_ddgi_rg_main();
                }
    for (int p = 0; p < n; p++) {
        const R::Ray r = R::UnpackRay(rays[size_t(p) * ray_count]);
        origins[4 * p] = r.origin.x;
        origins[4 * p + 1] = r.origin.y;
        origins[4 * p + 2] = r.origin.z;
        origins[4 * p + 3] = 0.0f;
    }
    // the trace dispatch, then the hit shader over every slot
    H::PackedRay* hr = reinterpret_cast<H::PackedRay*>(rays.data());
    for (uint i = 0; i < total; i++) {
        H::Ray r = H::UnpackRay(hr[i]);
        r.hitID = -1;
        r.hitDistance = 0.0f;
        if (r.ID >= 0) {
            if (opacity_check) H::HitClosestTransparency(r, INSTANCE_MASK_ALL, 0.0f, INF);
            else H::HitClosest(r, INSTANCE_MASK_ALL, 0.0f, INF);
        }
        hr[i] = H::PackRay(r);
    }
    volume(H::ddgiData, true);
    H::probeStates = zeros.data();
    H::probeOffsets = zeros.data();
    H::rays = hr;
    H::readAtomic = read_count;
    H::writeAtomic = write_count;
    H::hits = reinterpret_cast<H::PackedRayHit*>(hits);
    H::Uniforms.seed = seed;
    H::environmentMap.constant = vec4(env[0], env[1], env[2], 1.0f);
    H::PushConstants.rayBufferOffset = 1u;
    H::PushConstants.rayBufferSize = total;
    H::PushConstants.useRayBinning = 0;
    read_count[0] = total;
    for (uint i = 0; i < total; i++) {
        gl_GlobalInvocationID = uvec3(i, 0u, 0u);
        gl_LocalInvocationID = uvec3(i % 32u, 0u, 0u);
        gl_LocalInvocationIndex = i % 32u;
        gl_WorkGroupID = uvec3(i / 32u, 0u, 0u);
        H::aeg_ddgi_main();
    }
}

// SampleBlueNoise(pixel, sample_index, 0 and 1) for every pixel of a w x h
// image: out w * h * 2 floats (the blueNoiseVec of rtao.csh:82-86).
void aeglsl_blue_noise(int w, int h, const float* ranking, const float* sobol, int sample_index, float* out) {
    const glsl_texture2D rank_tex = Rgba(ranking, 128, 128), sobol_tex = Rgba(sobol, 256, 1);
    sampler2D rank_s, sobol_s;
    rank_s.tex = &rank_tex;
    sobol_s.tex = &sobol_tex;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            for (int d = 0; d < 2; d++)
                out[(size_t(y) * w + x) * 2 + d] = aeg_rtao::SampleBlueNoise(ivec2(x, y), sample_index, d, rank_s, sobol_s);
}

// count draws of random(x, seed) from the seed, per x; out: n * count floats.
void aeglsl_random(const float* x, int n, float seed0, int count, float* out) {
    for (int i = 0; i < n; i++) {
        float seed = seed0;
        for (int k = 0; k < count; k++) out[i * count + k] = random(x[i], seed);
    }
}

}  // extern "C"
