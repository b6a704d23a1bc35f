// Wavefront path tracer: ray generation, the hit/shade bounce kernel and the
// shadow-ray resolve, around the traversal kernels.
//
// Estimator: the engine's non-real-time path tracer
// (data/shader/pathtracer/rayGen.csh, rayHit.csh) --
//   * emission of the first hit only (rayHit.csh:180-183);
//   * next-event estimation at every vertex: one light picked by streaming
//     weighted selection (raytracer/direct.hsh:12-49; weight =
//     brightness*area*cos/d^2 for triangle lights, clamped to [1e-7, 1]), a
//     uniform point on the light triangle (raytracer/lights.hsh:11-29), the
//     Disney-diffuse + GGX BRDF (brdf/brdfEval.hsh:8-32, brdf/brdf.hsh), a
//     shadow ray from P + N*EPSILON to the light (rayHit.csh:327-338);
//   * the continuation: lobe picked by Fresnel (spec probability clamped to
//     [0.1, 0.9]), cosine-weighted diffuse or GGX VNDF specular sampling
//     (brdf/brdfSample.hsh), origin pushed back along V by EPSILON, ambient
//     occlusion factor, Russian roulette with p = clamp(max(throughput),
//     0.01, 0.99), tripled before bounce 3, and termination below the
//     geometric surface (rayHit.csh:237-325);
//   * a constant environment radiance on a miss (the engine samples its sky cubemap there), and -- deliberately --
//     without the engine's clamp of indirect radiance at 10 (rayHit.csh:
//     196-201), which biases the estimate; this renderer is the unbiased
//     reference the radiance cache is compared against.
// Shadow rays are not traced inline: the shade kernel appends them, with the
// contribution they would add, to a shadow queue that the any-hit kernel
// traces and the resolve kernel adds into the accumulation buffers (FP32,
// and FP64 for converged images).
// Random numbers: the PCG hash of Jarzynski & Olano (JCGT 2020) keyed by
// (pixel, sample, bounce, dimension).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cast_kernels.cuh"
#include "texture.cuh"

namespace atlas::rt::dev {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;

struct PtScene {
    const float4* instances;      // GPUBVHInstance (4 float4)
    const float4* inst_model;     // object-to-world 3x4 rows per instance (3 float4)
    const MeshDesc* meshes;
    const float* materials;       // GPUMaterial, 23 words each
    uint32_t n_materials;
    const float4* lights;         // GPULight (4 float4)
    uint32_t n_lights;
    TexTable tex;                 // the scene's textures (texture.cuh)
    uint32_t tex_level;           // mip level of the surface textures (GetSurfaceParameters' textureLevel)
    float env_r, env_g, env_b;    // constant environment radiance a miss adds (rayHit.csh:166-171)
};

struct PtParams {
    PtScene sc;
    uint32_t width, height;
    uint32_t sample;              // sample index (RNG stream)
    uint32_t bounce;              // bounce of the rays being shaded
    uint32_t max_bounces;
    float epsilon;
    uint32_t seed;
    uint32_t mis;                 // 1: next-event estimation combined with BRDF sampling (power heuristic)
    // queues
    const float4* rays_in;        // PackedRay
    const float4* hits_in;        // ae_hit
    const float4* pay_in;         // throughput.xyz, pixel bits
    const uint32_t* n_in;
    float4* rays_out;
    float4* pay_out;
    uint32_t* n_out;
    float4* shadow_rays;
    float4* shadow_pay;           // contribution.rgb, pixel bits
    uint32_t* n_shadow;
    const uint8_t* shadow_occ;
    const float* shadow_vis;      // with transparent surfaces: the visibility prod(1 - opacity) per shadow ray
    float4* accum;                // W*H float4 (rgb, sample count in .w from raygen)
    double* accum64;              // W*H*3 or null
    uint32_t atomic_accum;        // several contributions per pixel and pass: add atomically
    uint32_t capacity;            // queue capacity in rays (0: width * height)
    uint32_t* overflow;           // set when an append would pass the capacity (ray dropped)
    // real-time mode (rayHit.csh:134-150): radiance into a [3][H][W] uint32
    // frame accumulation instead of accum / accum64
    uint32_t* frame_accum;
    float rt_max_radiance;
    uint32_t rt_max_per_sample;   // 0: one sample per frame, float bits
    // primary rays: the pixels of one tile (pixelOffset / tileSize of
    // rayGen.csh:27-30); centred = through pixel centres + jitter * 0.25 as the
    // real-time ray generation does (rayGen.csh:37-38), else a random sub-pixel offset
    uint32_t tile_x0, tile_y0, tile_w, tile_h;
    uint32_t centered;
    float jitter_x, jitter_y;
    // real-time G-buffer of the frame's first sample (rayHit.csh:76-116),
    // written by the bounce-0 shading when gb_write is set
    uint32_t gb_write;
    float* gb_depth;              // view-space z of the hit, INF on a miss
    uint32_t* gb_material;        // GPUMaterial.ID, 65535 on a miss
    float2* gb_normal;            // EncodeNormal(geometry normal)
    float2* gb_velocity;          // (ndc last - ndc current) * 0.5
    const float4* gb_mats;        // rows of the view, projection and last view-projection matrices
    const float4* gb_last_model;  // previous object-to-world rows per instance; null: the current ones
};

// Pixel keys carried by rays and payloads: the pixel index in the low 24
// bits; the radiance-cache renderer's path splits keep their split index in
// bits 24-26, which gives every split its own random streams.
constexpr uint32_t kPixelMask = 0x00FFFFFFu;

// ---- small vector helpers (fast math is fine here: statistics, not parity) ----
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{ x, y, z }; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 normalize(V3 a) {
    const float l2 = dot(a, a);
    return a * (l2 > 0.0f ? rsqrtf(l2) : 0.0f);
}
__device__ __forceinline__ float saturate(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
__device__ __forceinline__ V3 ld3(const float4& f) { return v3(f.x, f.y, f.z); }

// 10:10:10:2 signed unit vector (common/packing.hsh unpackUnitVector)
__device__ __forceinline__ V3 unpack_unit(float bits) {
    const int32_t c = __float_as_int(bits);
    return v3(float((c >> 0) & 1023) / 1023.0f * 2.0f - 1.0f, float((c >> 10) & 1023) / 1023.0f * 2.0f - 1.0f,
              float((c >> 20) & 1023) / 1023.0f * 2.0f - 1.0f);
}

__device__ __forceinline__ float rng(uint32_t pixel, uint32_t sample, uint32_t bounce, uint32_t dim, uint32_t seed) {
    return rand01(pixel, sample * 16u + bounce + (seed << 12), dim * 0x9E3779B9u + 0x7F4A7C15u);
}

struct Mat {
    int id;                     // GPUMaterial.ID
    V3 base, emissive;
    float opacity, roughness, metalness, ao, reflectance, normalScale;
    int twoSided, cullBackFaces, invertUVs, useVertexColors;
    int baseTex, opacityTex, normalTex, roughTex, metalTex, aoTex;
};

__device__ __forceinline__ Mat load_material(const float* m) {
    Mat r;
    r.id = __float_as_int(m[0]);
    r.base = v3(m[1], m[2], m[3]);
    r.emissive = v3(m[4], m[5], m[6]);
    r.opacity = m[7];
    r.roughness = m[8];
    r.metalness = m[9];
    r.ao = m[10];
    r.reflectance = m[11];
    r.normalScale = m[12];
    r.invertUVs = __float_as_int(m[13]);
    r.twoSided = __float_as_int(m[14]);
    r.cullBackFaces = __float_as_int(m[15]);
    r.useVertexColors = __float_as_int(m[16]);
    r.baseTex = __float_as_int(m[17]);
    r.opacityTex = __float_as_int(m[18]);
    r.normalTex = __float_as_int(m[19]);
    r.roughTex = __float_as_int(m[20]);
    r.metalTex = __float_as_int(m[21]);
    r.aoTex = __float_as_int(m[22]);
    return r;
}

struct Surf {
    V3 P, V, N, L, H, geoN;
    float NdotL, LdotH, NdotH, NdotV;
    V3 F0;
    float F90;
    Mat mat;
    bool backface;      // backfaceHit of GetSurfaceParameters (surface.hsh:99)
};

// UpdateSurface (brdf/surface.hsh:25-41)
__device__ __forceinline__ void update_surface(Surf& s) {
    s.L = normalize(s.L);
    s.V = normalize(s.V);
    s.N = normalize(s.N);
    s.H = normalize(s.L + s.V);
    s.NdotL = saturate(dot(s.N, s.L));
    s.LdotH = saturate(dot(s.L, s.H));
    s.NdotH = saturate(dot(s.N, s.H));
    s.NdotV = saturate(dot(s.N, s.V));
    const float f0 = 0.16f * s.mat.reflectance * s.mat.reflectance;
    s.F0 = v3(f0, f0, f0) * (1.0f - s.mat.metalness) + s.mat.base * s.mat.metalness;
    s.F90 = saturate(50.0f * (s.F0.x * 0.333f + s.F0.y * 0.333f + s.F0.z * 0.333f));
}

__device__ __forceinline__ float pow5(float x) { return x * x * x * x * x; }

__device__ __forceinline__ V3 fresnel(V3 F0, float F90, float c) {
    const float k = pow5(1.0f - c);
    return v3(F0.x + (F90 - F0.x) * k, F0.y + (F90 - F0.y) * k, F0.z + (F90 - F0.z) * k);
}

// brdf.hsh: RenormalizedDisneyDiffuse, visibility terms, GGX distribution
__device__ __forceinline__ float disney_diffuse(float NdotV, float NdotL, float LdotH, float lr) {
    const float energyBias = 0.5f * lr;
    const float energyFactor = 1.0f + (1.0f / 1.51f - 1.0f) * lr;
    const float FD90 = energyBias + 2.0f * LdotH * LdotH * lr;
    const float ls = 1.0f + (FD90 - 1.0f) * pow5(1.0f - NdotL);
    const float vs = 1.0f + (FD90 - 1.0f) * pow5(1.0f - NdotV);
    return ls * vs * energyFactor;
}
__device__ __forceinline__ float vis_separable(float c, float a) {
    const float a2 = a * a;
    return 2.0f * c / (c + sqrtf(a2 + (1.0f - a2) * c * c));
}
__device__ __forceinline__ float vis_correlated(float NdotL, float NdotV, float a) {
    const float a2 = a * a;
    const float gl = NdotV * sqrtf((-NdotL * a2 + NdotL) * NdotL + a2);
    const float gv = NdotL * sqrtf((-NdotV * a2 + NdotV) * NdotV + a2);
    return 0.5f / (gl + gv + 0.0000001f);
}
__device__ __forceinline__ float ggx_d(float NdotH, float a) {
    const float a2 = a * a;
    const float f = (NdotH * a2 - NdotH) * NdotH + 1.0f;
    return a2 / (f * f + 0.0000001f) * kInvPi;
}

// brdfEval.hsh:8-32
__device__ __forceinline__ V3 eval_diffuse(const Surf& s) {
    const float r = fmaxf(s.mat.roughness * s.mat.roughness, 0.00001f);
    return s.mat.base * ((1.0f - s.mat.metalness) * disney_diffuse(s.NdotV, s.NdotL, s.LdotH, r) * kInvPi);
}
__device__ __forceinline__ V3 eval_specular(const Surf& s) {
    const float r = fmaxf(s.mat.roughness * s.mat.roughness, 0.00001f);
    return fresnel(s.F0, s.F90, s.LdotH) * (ggx_d(s.NdotH, r) * vis_correlated(s.NdotV, s.NdotL, r));
}

__device__ __forceinline__ void basis_from(V3 N, V3& t, V3& b) {
    const V3 up = fabsf(N.z) < 0.999f ? v3(0, 0, 1) : v3(1, 0, 0);
    t = normalize(cross(up, N));
    b = cross(N, t);
}

// brdfSample.hsh:8-30 -- returns pdf, sets s.L
__device__ __forceinline__ float sample_diffuse(Surf& s, float u0, float u1, V3& refl) {
    const float th = sqrtf(u0);
    float sp, cp;
    sincospif(2.0f * u1, &sp, &cp);
    V3 t, b;
    basis_from(s.N, t, b);
    s.L = normalize(t * (th * cp) + b * (th * sp) + s.N * sqrtf(fmaxf(0.0f, 1.0f - u0)));
    update_surface(s);
    refl = eval_diffuse(s);
    return s.NdotL * kInvPi;
}

// brdfSample.hsh:32-90 (Dupuy & Benyoub spherical-cap VNDF sampling)
__device__ __forceinline__ float sample_specular(Surf& s, float u0, float u1, V3& refl) {
    const float alpha = s.mat.roughness * s.mat.roughness;
    s.V = normalize(s.V);
    const V3 N = normalize(s.N);
    const V3 up = fabsf(N.z) < 0.999f ? v3(0, 0, 1) : v3(1, 0, 0);
    const V3 t = normalize(cross(up, N));
    const V3 b = normalize(cross(N, t));
    // V in the tangent frame (V * TBN)
    V3 Vl = normalize(v3(dot(s.V, t), dot(s.V, b), dot(s.V, N)));
    Vl = normalize(v3(Vl.x * alpha, Vl.y * alpha, Vl.z));
    float sp, cp;
    sincospif(2.0f * u0, &sp, &cp);
    const float z = (1.0f - u1) * (1.0f + Vl.z) - Vl.z;
    const float rr = sqrtf(saturate(1.0f - z * z));
    const V3 c = v3(cp * rr, sp * rr, z);
    const V3 Hh = c + Vl;
    const V3 Ml = v3(Hh.x * alpha, Hh.y * alpha, fmaxf(Hh.z, 0.0f));
    const V3 M = normalize(t * Ml.x + b * Ml.y + N * Ml.z);
    s.L = M * (2.0f * dot(s.V, M)) - s.V;
    update_surface(s);
    refl = v3(0, 0, 0);
    float pdf = 1.0f;
    if (s.NdotL > 0.0f && s.LdotH > 0.0f) {
        const V3 F = fresnel(s.F0, s.F90, s.LdotH);
        const float Vis = vis_correlated(s.NdotV, s.NdotL, alpha);
        const float G1 = vis_separable(s.NdotV, alpha);
        pdf = G1 / (4.0f * fabsf(dot(s.V, s.N)));
        refl = F * Vis;
    }
    return pdf;
}

__device__ __forceinline__ V3 xform_point(const float4* m, V3 p) {
    return v3(m[0].x * p.x + m[0].y * p.y + m[0].z * p.z + m[0].w, m[1].x * p.x + m[1].y * p.y + m[1].z * p.z + m[1].w,
              m[2].x * p.x + m[2].y * p.y + m[2].z * p.z + m[2].w);
}
__device__ __forceinline__ V3 xform_dir(const float4* m, V3 p) {
    return v3(m[0].x * p.x + m[0].y * p.y + m[0].z * p.z, m[1].x * p.x + m[1].y * p.y + m[1].z * p.z,
              m[2].x * p.x + m[2].y * p.y + m[2].z * p.z);
}

struct Tri {
    V3 v0, v1, v2, n0, n1, n2;
    int material;
};

// GPUTriangle (common.hsh:17-44) in world space (TransformTriangle, surface.hsh:46-61)
__device__ __forceinline__ Tri load_triangle(const PtScene& sc, int32_t inst, int32_t tri) {
    const float4* ip = sc.instances + size_t(inst) * 4;
    const float4 c3 = __ldg(ip + 3);
    const MeshDesc m = sc.meshes[__float_as_int(c3.x)];
    const float4* tp = m.shading + size_t(tri) * 6;
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2), d0 = __ldg(tp + 3);
    const float4* M = sc.inst_model + size_t(inst) * 3;
    float4 mm[3] = { __ldg(M), __ldg(M + 1), __ldg(M + 2) };
    Tri t;
    t.v0 = xform_point(mm, ld3(a));
    t.v1 = xform_point(mm, ld3(b));
    t.v2 = xform_point(mm, ld3(c));
    t.n0 = normalize(xform_dir(mm, unpack_unit(a.w)));
    t.n1 = normalize(xform_dir(mm, unpack_unit(b.w)));
    t.n2 = normalize(xform_dir(mm, unpack_unit(c.w)));
    t.material = __float_as_int(d0.w) + __float_as_int(c3.y);
    return t;
}

struct Light {
    V3 P, N, radiance;
    uint32_t type;
    int32_t tri, inst;
    float pdf, area, brightness;
};

__device__ __forceinline__ Light load_light(const float4* l) {
    const float4 P = __ldg(l), N = __ldg(l + 1), C = __ldg(l + 2), D = __ldg(l + 3);
    Light r;
    r.P = ld3(P);
    r.N = ld3(N);
    r.radiance = ld3(C);
    const uint32_t data = __float_as_uint(D.x);
    r.type = data >> 28;
    r.tri = int32_t(data & 0x0FFFFFFFu);
    r.inst = __float_as_int(D.w);
    r.pdf = D.y;
    r.area = D.z;
    r.brightness = (r.radiance.x + r.radiance.y + r.radiance.z) * 0.33333f;
    return r;
}

static __global__ void pt_raygen_kernel(CameraParams c, PtParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = p.tile_w * p.tile_h;
    if (i >= n) return;
    const uint32_t t = slot_to_pixel(i, p.tile_w, p.tile_h);
    const uint32_t px = p.tile_x0 + t % p.tile_w, py = p.tile_y0 + t / p.tile_w;
    const uint32_t pix = py * c.width + px;
    float u, v;
    if (p.centered) {
        u = p.jitter_x * 0.25f + (float(px) + 0.5f) / float(c.width);
        v = p.jitter_y * 0.25f + (float(py) + 0.5f) / float(c.height);
    } else {
        const float jx = rng(pix, p.sample, 15, 0, p.seed), jy = rng(pix, p.sample, 15, 1, p.seed);
        u = (float(px) + jx) / float(c.width);
        v = (float(py) + jy) / float(c.height);
    }
    V3 d = v3(c.ox + c.rx * u + c.bx * v - c.lx, c.oy + c.ry * u + c.by * v - c.ly, c.oz + c.rz * u + c.bz * v - c.lz);
    d = normalize(d);
    float4* r = p.rays_out + size_t(i) * 3;
    r[0] = make_float4(c.lx, c.ly, c.lz, __int_as_float(int32_t(pix)));
    r[1] = make_float4(d.x, d.y, d.z, 0.0f);
    r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
    p.pay_out[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pix));
    if (i == 0) *p.n_out = n;
}

__device__ __forceinline__ void add_radiance(const PtParams& p, uint32_t key, V3 L) {
    const uint32_t pix = key & kPixelMask;
    if (p.frame_accum) {
        // real-time accumulation: the float itself at one sample per frame,
        // else radiance / maxRadiance clamped to [0, 1] and quantised to
        // 0xFFFFFFFF / samplesPerFrame steps, added atomically per channel
        const size_t plane = size_t(p.width) * p.height;
        const float c[3] = { L.x, L.y, L.z };
#pragma unroll
        for (int k = 0; k < 3; k++) {
            uint32_t* d = p.frame_accum + k * plane + pix;
            if (!p.rt_max_per_sample) {
                atomicAdd(reinterpret_cast<float*>(d), c[k]);
            } else {
                const float nr = fminf(fmaxf(c[k] / p.rt_max_radiance, 0.0f), 1.0f);
                const uint32_t q = min(uint32_t(nr * float(p.rt_max_per_sample)), p.rt_max_per_sample);
                if (q) atomicAdd(d, q);
            }
        }
        return;
    }
    float4* a = p.accum + pix;
    if (p.atomic_accum) {
        atomicAdd(&a->x, L.x);
        atomicAdd(&a->y, L.y);
        atomicAdd(&a->z, L.z);
    } else {
        a->x += L.x;
        a->y += L.y;
        a->z += L.z;
    }
    if (p.accum64) {
        double* d = p.accum64 + size_t(pix) * 3;
        if (p.atomic_accum) {
            atomicAdd(d, double(L.x));
            atomicAdd(d + 1, double(L.y));
            atomicAdd(d + 2, double(L.z));
        } else {
            d[0] += double(L.x);
            d[1] += double(L.y);
            d[2] += double(L.z);
        }
    }
}

__device__ __forceinline__ uint32_t queue_capacity(const PtParams& p) {
    return p.capacity ? p.capacity : p.width * p.height;
}

// GetSurfaceParameters (raytracer/surface.hsh:63-140) at a closest hit:
// position, interpolated shading normal, geometric normal (both flipped
// towards the ray on two-sided materials), material.
// unpackUnorm4x8 (one vertex colour of GPUTriangle d2)
__device__ __forceinline__ float4 unpack_unorm4(float bits) {
    const uint32_t c = __float_as_uint(bits);
    return make_float4(float(c & 255u) / 255.0f, float((c >> 8) & 255u) / 255.0f, float((c >> 16) & 255u) / 255.0f,
                       float(c >> 24) / 255.0f);
}

// The material terms of GetSurfaceParameters (surface.hsh:83-124) at the
// hit's barycentrics: vertex colours, base colour / opacity / roughness /
// metalness / ao textures and the normal map, all at mip level sc.tex_level
// (0 for the path tracer, rayHit.csh:177; 4 for DDGI probe rays,
// ddgi/rayHit.csh:79).  N is the interpolated normal (in and out).
__device__ __forceinline__ void surface_textures(const PtScene& sc, int32_t inst, int32_t triPtr, float r, float s,
                                                 float t, Mat& mat, V3& N) {
    const float4* ip = sc.instances + size_t(inst) * 4;
    const MeshDesc m = sc.meshes[__float_as_int(__ldg(ip + 3).x)];
    const float4* tp = m.shading + size_t(triPtr) * 6;
    const float4 d0 = __ldg(tp + 3), d1 = __ldg(tp + 4), d2 = __ldg(tp + 5);
    const float2 uv0 = unpack_half2(d0.x), uv1 = unpack_half2(d0.y), uv2 = unpack_half2(d0.z);
    const float tu = r * uv0.x + s * uv1.x + t * uv2.x;
    float tv = r * uv0.y + s * uv1.y + t * uv2.y;
    if (mat.invertUVs > 0) tv = 1.0f - tv;
    if (mat.useVertexColors > 0) {
        const float4 c0 = unpack_unorm4(d2.x), c1 = unpack_unorm4(d2.y), c2 = unpack_unorm4(d2.z);
        mat.base = mat.base * v3(r * c0.x + s * c1.x + t * c2.x, r * c0.y + s * c1.y + t * c2.y,
                                 r * c0.z + s * c1.z + t * c2.z);
    }
    const uint32_t lv = sc.tex_level;
    const float4 bc = sample_rgba_bilinear(sc.tex, mat.baseTex, tu, tv, lv);
    mat.base = mat.base * v3(bc.x, bc.y, bc.z);
    mat.opacity *= sample_r_bilinear(sc.tex, mat.opacityTex, tu, tv, lv);
    mat.roughness *= sample_r_bilinear(sc.tex, mat.roughTex, tu, tv, lv);
    mat.metalness *= sample_r_bilinear(sc.tex, mat.metalTex, tu, tv, lv);
    mat.ao *= sample_r_bilinear(sc.tex, mat.aoTex, tu, tv, lv);
    if (mat.normalTex >= 0) {
        // TBN = (tangent, +-bitangent, normal) in world space (TransformTriangle)
        const float4* M = sc.inst_model + size_t(inst) * 3;
        float4 mm[3] = { __ldg(M), __ldg(M + 1), __ldg(M + 2) };
        const V3 T = normalize(xform_dir(mm, unpack_unit(d1.x)));
        V3 B = normalize(xform_dir(mm, unpack_unit(d1.y)));
        if (!(mat.invertUVs > 0)) B = B * -1.0f;
        const float4 tn = sample_rgba_bilinear(sc.tex, mat.normalTex, tu, tv, lv);
        V3 n = T * (2.0f * tn.x - 1.0f) + B * (2.0f * tn.y - 1.0f) + N * (2.0f * tn.z - 1.0f);
        n = n * (1.0f / fmaxf(sqrtf(dot(n, n)), 0.00001f));
        const float w = saturate(mat.normalScale);
        N = N * (1.0f - w) + n * w;
    }
}

__device__ __forceinline__ bool has_surface_textures(const Mat& m) {
    // some index is >= 0 exactly when the AND of all of them has its sign bit clear
    return m.useVertexColors > 0 || (m.baseTex & m.opacityTex & m.normalTex & m.roughTex & m.metalTex & m.aoTex) >= 0;
}

__device__ __forceinline__ Surf make_surface(const PtScene& sc, V3 ro, V3 rd, float t, int32_t inst, int32_t triPtr,
                                             float bu, float bv) {
    const Tri tri = load_triangle(sc, inst, triPtr);
    const float r = 1.0f - bu - bv;
    Surf sf;
    sf.mat = load_material(sc.materials + size_t(tri.material) * 23);
    sf.P = ro + rd * t;
    V3 N = normalize(tri.n0 * r + tri.n1 * bu + tri.n2 * bv);
    V3 triN = normalize(cross(tri.v0 - tri.v1, tri.v0 - tri.v2));
    const bool flip = dot(triN, rd) > 0.0f;
    sf.backface = sf.mat.twoSided > 0 || sf.mat.cullBackFaces == 0 ? false : flip;
    if (flip && sf.mat.twoSided > 0) triN = triN * -1.0f;
    if (has_surface_textures(sf.mat)) surface_textures(sc, inst, triPtr, r, bu, bv, sf.mat, N);
    if (dot(N, triN) < 0.0f && sf.mat.twoSided > 0) N = N * -1.0f;
    sf.V = rd * -1.0f;
    sf.N = normalize(N);
    sf.geoN = triN;
    sf.L = sf.N;
    // NdotV, F0 and F90 do not depend on L: set them here, as the light
    // sample's UpdateSurface would, so that the lobe choice of the
    // continuation (which reads them) is defined in a scene without lights
    update_surface(sf);
    return sf;
}

// SampleTriangleLight (raytracer/lights.hsh:11-29): the point and normal of
// a triangle light at (r0, r1), uniform over its area.
__device__ __forceinline__ void triangle_light_point(const Tri& lt, float r0, float r1, V3& P, V3& N) {
    const float lu = 1.0f - sqrtf(r0), lv = r1 * sqrtf(r0), lw = 1.0f - lu - lv;
    P = lt.v0 * lu + lt.v1 * lv + lt.v2 * lw;
    N = lt.n0 * lu + lt.n1 * lv + lt.n2 * lw;
}

// Selection weight of a light seen from P (raytracer/direct.hsh:12-49).
__device__ __forceinline__ float light_weight(const Light& L, V3 P) {
    float w = 1.0f;
    if (L.type == 1u) {
        const V3 toL = L.P - P;
        const float d2 = dot(toL, toL);
        const float NdotL = fmaxf(dot(L.N, normalize(toL) * -1.0f), 0.0f);
        w = L.brightness * L.area * NdotL / d2;
    } else {
        w = L.brightness;
    }
    return fminf(fmaxf(w, 0.0000001f), 1.0f);
}

// EvaluateDirectLight (rayHit.csh:209-235) up to the visibility test: picks a
// light, samples it, evaluates the BRDF.  Returns false when nothing needs a
// shadow ray; otherwise the contribution (already scaled by the path
// throughput) and the shadow ray (origin, direction, tmax).
// GetLight + SampleLight (raytracer/direct.hsh:12-86): picks one light by
// streaming weighted selection, samples a point on it (triangle lights) and
// points sf.L at it (UpdateSurface).  False when the scene has no lights.
struct LightSample {
    V3 radiance;
    float pdf, solidAngle, dist;
    uint32_t type;
};
__device__ __forceinline__ bool sample_light(const PtScene& sc, Surf& sf, uint32_t pix, uint32_t sample,
                                             uint32_t bounce, uint32_t seed, LightSample& ls) {
    if (sc.n_lights == 0) return false;
    Light sel{};
    float selW = 0.0f, total = 0.0f;
    for (uint32_t li = 0; li < sc.n_lights; li++) {
        const Light L = load_light(sc.lights + size_t(li) * 4);
        const float w = light_weight(L, sf.P);
        total += w;
        if (rng(pix, sample, bounce, 16u + li, seed) < w / total) {
            selW = w;
            sel = L;
        }
    }
    ls.pdf = selW / total * sel.pdf;
    ls.solidAngle = 1.0f;
    ls.dist = 1e12f;
    ls.type = sel.type;
    ls.radiance = sel.radiance;
    if (sel.type == 1u) {
        const float r0 = rng(pix, sample, bounce, 1, seed);
        const float r1 = rng(pix, sample, bounce, 2, seed);
        const Tri lt = load_triangle(sc, sel.inst, sel.tri);
        V3 LP, LN;
        triangle_light_point(lt, r0, r1, LP, LN);
        const V3 toL = LP - sf.P;
        const float d2 = dot(toL, toL);
        ls.dist = sqrtf(d2);
        sf.L = toL * (1.0f / ls.dist);
        update_surface(sf);
        const float NdotLl = fmaxf(dot(LN, sf.L * -1.0f), 0.0f);
        ls.solidAngle = NdotLl / (d2 * (1.0f / sel.area));
    } else {
        sf.L = normalize(sel.N * -1.0f);
        update_surface(sf);
    }
    return true;
}

__device__ __forceinline__ bool direct_light(const PtScene& sc, Surf& sf, V3 thr, uint32_t pix, uint32_t sample,
                                             uint32_t bounce, uint32_t seed, float eps, V3& contrib, V3& so,
                                             V3& sd, float& stmax, float* pdf_sa = nullptr) {
    LightSample ls;
    if (!sample_light(sc, sf, pix, sample, bounce, seed, ls)) return false;
    const float lightPdf = ls.pdf, solidAngle = ls.solidAngle, dist = ls.dist;
    const V3 refl = (eval_diffuse(sf) + eval_specular(sf)) * sf.mat.opacity;
    contrib = thr * sf.mat.opacity * (refl * ls.radiance) * (solidAngle * sf.NdotL / lightPdf);
    if (pdf_sa) *pdf_sa = ls.type == 1u ? (solidAngle > 0.0f ? lightPdf / solidAngle : 0.0f) : 0.0f;
    if (!(sf.NdotL > 0.0f && lightPdf > 0.0f && contrib.x + contrib.y + contrib.z > 0.0f)) return false;
    so = sf.P + sf.N * eps;         // CheckVisibility, rayHit.csh:327-338
    sd = sf.L;
    stmax = dist - 2.0f * eps;
    return true;
}

// Chance that EvaluateIndirectLight passes straight through a partially
// opaque surface (rayHit.csh:252-253): clamp(1 - opacity, 0.1, 0.9), 0 for
// an opaque one.
__device__ __forceinline__ float refract_chance(float opacity) {
    return opacity == 1.0f ? 0.0f : fminf(fmaxf(1.0f - opacity, 0.1f), 0.9f);
}

// EvaluateIndirectLight (rayHit.csh:237-325): the pass-through of a partially
// opaque surface or a reflection lobe, BRDF sample, throughput update,
// Russian roulette, termination below the surface.  Returns true when the
// path continues with (o, d) and throughput thr; *passed tells a
// pass-through (which keeps the ray's direction).
__device__ __forceinline__ bool continue_path(Surf& sf, V3& thr, uint32_t pix, uint32_t sample, uint32_t bounce,
                                              uint32_t seed, float eps, V3& o, V3& d, bool* spec_lobe = nullptr,
                                              bool* passed = nullptr) {
    const Mat& mat = sf.mat;
    const float refractChance = refract_chance(mat.opacity);
    V3 refl;
    float pdf;
    bool through = false;
    if (spec_lobe) *spec_lobe = false;
    if (rng(pix, sample, bounce, 3, seed) >= refractChance) {
        const V3 F = fresnel(sf.F0, sf.F90, sf.NdotV);
        const float specChance = fminf(fmaxf((F.x + F.y + F.z) * 0.33333f, 0.1f), 0.9f);
        const float rnd = rng(pix, sample, bounce, 4, seed);
        const float u0 = rng(pix, sample, bounce, 5, seed);
        const float u1 = rng(pix, sample, bounce, 6, seed);
        if (spec_lobe) *spec_lobe = rnd < specChance;
        if (rnd < specChance) {
            pdf = sample_specular(sf, u0, u1, refl);
            refl = refl * mat.opacity;
            pdf *= specChance;
        } else {
            pdf = sample_diffuse(sf, u0, u1, refl);
            refl = refl * ((1.0f - mat.metalness) * mat.opacity);
            pdf *= (1.0f - specChance);
        }
        pdf *= (1.0f - refractChance);
        o = sf.P + sf.V * eps;
    } else {
        // straight through with reflectance 1 - opacity at full throughput
        // (NdotL = 1), the origin pushed behind the surface (rayHit.csh:282-291)
        sf.L = sf.V * -1.0f;
        pdf = refractChance;
        refl = v3(1.0f - mat.opacity, 1.0f - mat.opacity, 1.0f - mat.opacity);
        sf.NdotL = 1.0f;
        o = sf.P - sf.N * eps;
        through = true;
    }
    if (passed) *passed = through;
    if (pdf > 0.0f && refl.x + refl.y + refl.z > 0.0f) thr = thr * refl * (sf.NdotL / pdf);
    else thr = v3(0, 0, 0);
    d = normalize(sf.L);
    thr = thr * mat.ao;
    float prob = fminf(fmaxf(fmaxf(thr.x, fmaxf(thr.y, thr.z)), 0.01f), 0.99f);
    prob = bounce < 3 ? fminf(3.0f * prob, 1.0f) : prob;
    // a pass-through is exempt from the below-surface termination (rayHit.csh:318)
    const bool alive = thr.x + thr.y + thr.z > 0.0f && rng(pix, sample, bounce, 7, seed) <= prob &&
                       (through || dot(d, sf.geoN) > 0.0f);
    if (alive) thr = thr * (1.0f / prob);
    return alive;
}

// ---- combining next-event estimation with BRDF sampling (power heuristic) ----
// Not part of the engine's estimator: used by the radiance-cache renderer and
// its training paths, and by the path tracer when PtParams::mis is set.  Both
// strategies estimate the engine's direct-light integral: the GGX term the
// engine evaluates for lights carries a 1e-7 in its denominator (ggx_d), which
// caps it below roughness ~0.2, while the VNDF continuation follows the
// uncapped lobe; a BRDF-sampled light hit is therefore scaled by
// D_capped / D_true, and by opacity / ao for the engine's opacity^2 and ao
// factors, so that the sum stays unbiased with respect to the engine.

__device__ __forceinline__ float ggx_d_true(float NdotH, float a) {
    const float a2 = a * a;
    const float f = (NdotH * a2 - NdotH) * NdotH + 1.0f;
    return a2 / fmaxf(kPi * f * f, 1e-30f);
}

// Density (per solid angle) of continue_path's direction sampling towards L.
__device__ __forceinline__ float bsdf_pdf(Surf s, V3 L) {
    s.L = L;
    update_surface(s);
    if (!(s.NdotL > 0.0f)) return 0.0f;
    const V3 F = fresnel(s.F0, s.F90, s.NdotV);
    const float specChance = fminf(fmaxf((F.x + F.y + F.z) * 0.33333f, 0.1f), 0.9f);
    const float a = s.mat.roughness * s.mat.roughness;
    const float nv = fmaxf(s.NdotV, 1e-4f);
    const float ps = vis_separable(nv, a) * ggx_d_true(s.NdotH, a) / (4.0f * nv);
    const float pd = s.NdotL * kInvPi * (1.0f - s.mat.metalness);
    return (1.0f - refract_chance(s.mat.opacity)) * (specChance * ps + (1.0f - specChance) * pd);
}

// Density (per solid angle) with which direct_light at P samples the first
// emissive triangle along (P, d); 0 when the ray meets none or its back.
__device__ __forceinline__ float light_pdf_dir(const PtScene& sc, V3 P, V3 d) {
    float total = 0.0f, best = 1e30f, bw = 0.0f, bpdf = 0.0f, barea = 0.0f, bcos = 0.0f;
    for (uint32_t li = 0; li < sc.n_lights; li++) {
        const Light L = load_light(sc.lights + size_t(li) * 4);
        const float w = light_weight(L, P);
        total += w;
        if (L.type != 1u) continue;
        const Tri lt = load_triangle(sc, L.inst, L.tri);
        // Moller-Trumbore
        const V3 e1 = lt.v1 - lt.v0, e2 = lt.v2 - lt.v0;
        const V3 pv = cross(d, e2);
        const float det = dot(e1, pv);
        if (fabsf(det) < 1e-20f) continue;
        const float inv = 1.0f / det;
        const V3 tv = P - lt.v0;
        const float u = dot(tv, pv) * inv;
        if (u < 0.0f || u > 1.0f) continue;
        const V3 qv = cross(tv, e1);
        const float v = dot(d, qv) * inv;
        if (v < 0.0f || u + v > 1.0f) continue;
        const float t = dot(e2, qv) * inv;
        if (t <= 0.0f || t >= best) continue;
        const V3 LN = lt.n0 * (1.0f - u - v) + lt.n1 * u + lt.n2 * v;
        best = t;
        bw = w;
        bpdf = L.pdf;
        barea = L.area;
        bcos = fmaxf(dot(LN, d * -1.0f), 0.0f);
    }
    if (best >= 1e30f || bcos <= 0.0f || total <= 0.0f) return 0.0f;
    return bw / total * bpdf * best * best / (bcos * barea);
}

__device__ __forceinline__ float power_weight(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

// Multiplier of the emission found by the continuation (sf after
// continue_path: sf.L is the sampled direction, sf.H its half vector).
__device__ __forceinline__ float mis_hit_factor(const PtScene& sc, const Surf& sf, V3 d, bool spec_lobe) {
    const float pl = light_pdf_dir(sc, sf.P, d);
    if (pl <= 0.0f) return 0.0f;
    float m = power_weight(bsdf_pdf(sf, d), pl);
    if (spec_lobe) {
        // the engine's capped D over the sampled (true) D
        const float a = sf.mat.roughness * sf.mat.roughness;
        const float a2 = a * a;
        const float f = (sf.NdotH * a2 - sf.NdotH) * sf.NdotH + 1.0f;
        m *= f * f / (f * f + 0.0000001f);
    }
    return sf.mat.ao > 0.0f ? m * sf.mat.opacity / sf.mat.ao : 0.0f;
}

// rayHit.csh:55-325 for one bounce of the wavefront.
// The real-time G-buffer entry of one pixel (rayHit.csh:76-116): the hit's
// world position (or origin + direction * 100 on a miss) carried into the
// previous frame through the instance's inverse and last matrices, projected
// with the current and the last view-projection; view-space depth, material
// id and the encoded geometry normal.
__device__ __forceinline__ float dot4(float4 r, V3 v, float w) {
    return r.x * v.x + r.y * v.y + r.z * v.z + r.w * w;
}
__device__ __forceinline__ float dot4(float4 r, float4 v) {
    return r.x * v.x + r.y * v.y + r.z * v.z + r.w * v.w;
}
__device__ __forceinline__ void write_gbuffer(const PtParams& p, uint32_t pix, bool hit, V3 P, V3 geoN, int mat_id, int inst) {
    V3 last = P;
    if (hit) {
        const float4* im = p.sc.instances + size_t(inst) * 4;   // transposed inverse: object = (P, 1) . column
        const V3 obj = v3(dot4(__ldg(im + 0), P, 1.0f), dot4(__ldg(im + 1), P, 1.0f), dot4(__ldg(im + 2), P, 1.0f));
        const float4* lm = (p.gb_last_model ? p.gb_last_model : p.sc.inst_model) + size_t(inst) * 3;
        last = v3(dot4(__ldg(lm + 0), obj, 1.0f), dot4(__ldg(lm + 1), obj, 1.0f), dot4(__ldg(lm + 2), obj, 1.0f));
    }
    const float4* M = p.gb_mats;   // rows 0-3 view, 4-7 projection, 8-11 last view-projection
    const float4 vs = make_float4(dot4(M[0], P, 1.0f), dot4(M[1], P, 1.0f), dot4(M[2], P, 1.0f), dot4(M[3], P, 1.0f));
    const float4 pc = make_float4(dot4(M[4], vs), dot4(M[5], vs), dot4(M[6], vs), dot4(M[7], vs));
    const float4 pl = make_float4(dot4(M[8], last, 1.0f), dot4(M[9], last, 1.0f), dot4(M[10], last, 1.0f),
                                  dot4(M[11], last, 1.0f));
    if (p.gb_velocity)
        p.gb_velocity[pix] = make_float2((pl.x / pl.w - pc.x / pc.w) * 0.5f, (pl.y / pl.w - pc.y / pc.w) * 0.5f);
    if (p.gb_depth) p.gb_depth[pix] = hit ? vs.z : 1e12f;
    if (p.gb_material) p.gb_material[pix] = hit ? uint32_t(mat_id) : 65535u;
    if (p.gb_normal) {
        // EncodeNormal (common/normalencode.hsh:3-16): octahedral xz, lower hemisphere folded
        const V3 n = hit ? geoN : v3(1.0f, 0.0f, 0.0f);
        const float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
        float x = n.x / s, z = n.z / s;
        if (n.y < 0.0f) {
            const float ox = x, oz = z;
            x = (ox >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(oz));
            z = (oz >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(ox));
        }
        p.gb_normal[pix] = make_float2(x, z);
    }
}

static __global__ void pt_shade_kernel(PtParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = min(*p.n_in, queue_capacity(p));
    bool emitRay = false, emitShadow = false;
    float4 outRay0{}, outRay1{}, outPay{}, shRay0{}, shRay1{}, shPay{};
    if (i < n) {
        const float4 h0 = p.hits_in[size_t(i) * 2];
        const int32_t triPtr = __float_as_int(h0.y);
        const float4 pay = p.pay_in[i];
        const uint32_t pix = __float_as_uint(pay.w);
        V3 thr = v3(pay.x, pay.y, pay.z);
        const bool gbuffer = p.gb_write && p.bounce == 0;
        if (gbuffer && triPtr < 0) {
            const float4 o4 = p.rays_in[size_t(i) * 3], d4 = p.rays_in[size_t(i) * 3 + 1];
            write_gbuffer(p, pix & kPixelMask, false, ld3(o4) + ld3(d4) * 100.0f, v3(1.0f, 0.0f, 0.0f), 0, 0);
        }
        if (triPtr < 0 && p.sc.env_r + p.sc.env_g + p.sc.env_b > 0.0f) {
            // EvaluateBounce's miss: the environment times the throughput, clamped per channel
            add_radiance(p, pix, v3(fminf(p.sc.env_r * thr.x, 10.0f), fminf(p.sc.env_g * thr.y, 10.0f),
                                    fminf(p.sc.env_b * thr.z, 10.0f)));
        }
        if (triPtr >= 0) {
            const float4 o4 = p.rays_in[size_t(i) * 3], d4 = p.rays_in[size_t(i) * 3 + 1];
            const float4 h1 = p.hits_in[size_t(i) * 2 + 1];
            Surf sf = make_surface(p.sc, ld3(o4), ld3(d4), h0.x, __float_as_int(h0.z), triPtr, h1.x, h1.y);
            if (gbuffer) write_gbuffer(p, pix & kPixelMask, true, sf.P, sf.geoN, sf.mat.id, __float_as_int(h0.z));
            // emission of the first hit (rayHit.csh:180-183); with MIS, also
            // the emission a continuation finds, weighted by its factor (ray dir.w)
            const bool emissive = sf.mat.emissive.x + sf.mat.emissive.y + sf.mat.emissive.z > 0.0f;
            if (p.bounce == 0 && emissive) add_radiance(p, pix, sf.mat.emissive);
            if (p.bounce > 0 && emissive && d4.w > 0.0f) add_radiance(p, pix, thr * sf.mat.emissive * d4.w);
            const bool cont = p.bounce < p.max_bounces;
            V3 c, so, sd;
            float st, pl = 0.0f;
            if (direct_light(p.sc, sf, thr, pix, p.sample, p.bounce, p.seed, p.epsilon, c, so, sd, st, &pl)) {
                if (p.mis && cont) c = c * power_weight(pl, bsdf_pdf(sf, sf.L));
                emitShadow = true;
                shRay0 = make_float4(so.x, so.y, so.z, __uint_as_float(pix));
                shRay1 = make_float4(sd.x, sd.y, sd.z, st);
                shPay = make_float4(c.x, c.y, c.z, __uint_as_float(pix));
            }
            if (cont) {
                V3 o, d;
                bool spec = false, passed = false;
                if (continue_path(sf, thr, pix, p.sample, p.bounce, p.seed, p.epsilon, o, d, &spec, &passed)) {
                    emitRay = true;
                    outRay0 = make_float4(o.x, o.y, o.z, __uint_as_float(pix));
                    // a light seen through a pass-through is not part of the
                    // engine's direct light (its NEE evaluates reflection only)
                    outRay1 = make_float4(d.x, d.y, d.z,
                                          p.mis && !passed ? mis_hit_factor(p.sc, sf, d, spec) : 0.0f);
                    outPay = make_float4(thr.x, thr.y, thr.z, __uint_as_float(pix));
                }
            }
        }
    }
    uint32_t* const counters[2] = { p.n_out, p.n_shadow };
    const bool want[2] = { emitRay, emitShadow };
    uint32_t slot[2];
    block_append<2>(counters, want, slot);
    const uint32_t ri = slot[0], si = slot[1];
    if (emitRay) {
        float4* r = p.rays_out + size_t(ri) * 3;
        r[0] = outRay0;
        r[1] = outRay1;
        r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
        p.pay_out[ri] = outPay;
    }
    if (emitShadow) {
        float4* r = p.shadow_rays + size_t(si) * 3;
        r[0] = shRay0;
        r[1] = make_float4(shRay1.x, shRay1.y, shRay1.z, 0.0f);
        r[2] = make_float4(shRay1.w, __int_as_float(-1), __int_as_float(-1), 0.0f);   // hit.x = tmax
        p.shadow_pay[si] = shPay;
    }
}

// Adds the contributions of the unoccluded shadow rays.
static __global__ void pt_resolve_kernel(PtParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = min(*p.n_shadow, queue_capacity(p));
    if (i >= n) return;
    float vis = 1.0f;
    if (p.shadow_vis) {
        vis = p.shadow_vis[i];            // CheckVisibility's HitAnyTransparency (rayHit.csh:327-338)
        if (!(vis > 0.0f)) return;
    } else if (p.shadow_occ[i]) {
        return;
    }
    const float4 c = p.shadow_pay[i];
    add_radiance(p, __float_as_uint(c.w), v3(c.x, c.y, c.z) * vis);
}

}  // namespace atlas::rt::dev

namespace atlas::rt::dev {

// The non-real-time output image (rayHit.csh:124-130): colour = accum.rgb *
// exposure / samples, mapped by 1 - exp(-colour) and raised to gamma.
// The output image of rayHit.csh:126-132 over the rectangle (x0, y0, tw, th)
// of a width-wide image: colour = accum.rgb * exposure / samples, out =
// (pow(1 - exp(-colour), gamma), 1).
static __global__ void pt_tonemap_kernel(const float4* accum, uint32_t width, uint32_t x0, uint32_t y0, uint32_t tw,
                                         uint32_t th, float exposure, float samples, float gamma, float4* out) {
    const uint32_t n = tw * th;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t pix = size_t(y0 + i / tw) * width + x0 + i % tw;
        const float4 a = accum[pix];
        out[pix] = make_float4(powf(1.0f - expf(-(a.x * exposure / samples)), gamma),
                               powf(1.0f - expf(-(a.y * exposure / samples)), gamma),
                               powf(1.0f - expf(-(a.z * exposure / samples)), gamma), 1.0f);
    }
}

}  // namespace atlas::rt::dev
