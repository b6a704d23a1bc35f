// The traversal's other consumers (include/atlas_rt.h): ray-traced ambient
// occlusion (data/shader/ao/rtao.csh), reflections
// (reflection/rtreflection.csh), diffuse GI (rtgi/rtgi.csh) and DDGI probe
// rays (ddgi/rayGen.csh + ddgi/rayHit.csh).
//
// Each pass is a short wavefront over the library's traversal kernels:
//   1. ray generation from the G-buffer (or the probe grid) into a compact
//      queue -- 48-byte rays plus the pixel (or probe-ray) index -- with the
//      output of pixels that trace nothing written at once;
//   2. the closest- or any-hit trace of the queue (the opaque persistent
//      kernel, or the transparency variants with AE_PASS_OPACITY_CHECK);
//   3. RTAO: the occlusion lands in the output; the others shade every hit
//      like the shaders' EvaluateHit -- emission plus one light sample --
//      and append one shadow ray per lit hit to a second queue;
//   4. the shadow trace (HitAnyTransparency for reflections and GI,
//      HitAny for DDGI, mask SHADOW, per-ray tmax = light distance -
//      2 EPSILON), a resolve that adds the visible light, and the output
//      (radiance limit, or PackRayHit for DDGI).
// Random numbers: the caller's per-pixel samples (the shaders' blue-noise
// vector) where given, else the PCG hash of (pixel, frame_seed); light
// choices always use the PCG hash keyed by the pixel / probe-ray index.
#include "atlas_rt.h"
#include "context.cuh"
#include "pt_kernels.cuh"

#include <cuda_fp16.h>

using namespace atlas::rt::host;
using namespace atlas::rt::dev;

namespace {

constexpr float kEps = 0.1f;            // EPSILON, raytracer/common.hsh:9
constexpr float kInfT = 1e12f;          // INF, raytracer/common.hsh:8
constexpr uint32_t kSampleSlot = 13u;   // RNG bounce slot of the pixel samples
constexpr uint32_t kLightSlot = 14u;    // RNG bounce slot of the light choices

enum PassKind : int { kPassAO = 0, kPassRefl = 1, kPassGI = 2, kPassDDGI = 3 };

struct GbParams {
    const float* depth;
    const float2* normal;
    const uint8_t* offset;
    const float* rough;
    const float2* samples;
    const uchar4* ranking;   // blue-noise scrambling / ranking texture, 128 x 128
    const uchar4* sobol;     // blue-noise Sobol sequence, 256 x 1
    uint32_t w, h, half_res;
    float ip[16], iv[16];
};

// SampleBlueNoise of common/bluenoise.hsh:9-32 (Heitz, Belcour, Ostromoukhov,
// Coeurjolly, Iehl 2019) for dimensions 0 and 1 of one pixel.  The shader
// reads the RGBA8 texels as unorm floats c / 255 and takes
// int(clamp(c / 255 * 256, 0, 255)); c / 255 * 256 = c + c / 255 lies in
// [c, c + 1) for c <= 254 and clamps to 255 for c = 255, so that integer is
// the byte itself, which is what this reads.
__device__ __forceinline__ void blue_noise(const GbParams& g, uint32_t px, uint32_t py, uint32_t index,
                                           float& u0, float& u1) {
    const uchar4 r = g.ranking[(py & 127u) * 128u + (px & 127u)];
    const uchar4 s = g.sobol[(index & 255u) ^ r.z];
    u0 = (0.5f + float(uint32_t(s.x) ^ r.x)) / 256.0f;
    u1 = (0.5f + float(uint32_t(s.y) ^ r.y)) / 256.0f;
}

struct PassP {
    float radius, bias, cutoff, limit;
    float env[3];
    uint32_t frame_seed, seed, tex_level;
};

struct Queue {
    float4* rays;        // PackedRay
    uint32_t* key;       // pixel or probe-ray index per ray
    uint32_t* count;
    uint32_t capacity;
};

// column-major mat4 times (x, y, z, w), summed in column order
__device__ __forceinline__ float4 mat4_mul(const float* m, float x, float y, float z, float w) {
    return make_float4(m[0] * x + m[4] * y + m[8] * z + m[12] * w, m[1] * x + m[5] * y + m[9] * z + m[13] * w,
                       m[2] * x + m[6] * y + m[10] * z + m[14] * w, m[3] * x + m[7] * y + m[11] * z + m[15] * w);
}

// DecodeNormal, common/normalencode.hsh:18-30 (octahedral, y up)
__device__ __forceinline__ V3 decode_normal(float cx, float cy) {
    const float y = 1.0f - (fabsf(cx) + fabsf(cy));
    if (y < 0.0f) {
        const float ox = cx, oy = cy;
        cx = (ox >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(oy));
        cy = (oy >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(ox));
    }
    return normalize(v3(cx, y, cy));
}

__device__ __forceinline__ void tangent_frame(V3 N, V3& t, V3& b, bool normalize_b) {
    const V3 up = fabsf(N.z) < 0.999f ? v3(0, 0, 1) : v3(1, 0, 0);
    t = normalize(cross(up, N));
    b = normalize_b ? normalize(cross(N, t)) : cross(N, t);
}

// ImportanceSampleCosDir (brdf/importanceSample.hsh:82-101), the same
// mapping as SampleDiffuseBRDF (brdf/brdfSample.hsh:8-32)
__device__ __forceinline__ V3 cos_dir(V3 N, float u0, float u1) {
    const float th = sqrtf(u0);
    float sp, cp;
    sincospif(2.0f * u1, &sp, &cp);
    V3 t, b;
    tangent_frame(N, t, b, false);
    return normalize(t * (th * cp) + b * (th * sp) + N * sqrtf(1.0f - u0));
}

// ImportanceSampleGGXVNDF (brdf/importanceSample.hsh:37-80), `alpha` =
// roughness^2 as the reflection shader passes it
__device__ __forceinline__ V3 ggx_vndf_dir(V3 N, V3 V, float alpha, float u0, float u1) {
    V3 t, b;
    tangent_frame(N, t, b, true);
    const V3 Vl = normalize(v3(dot(V, t) * alpha, dot(V, b) * alpha, dot(V, N)));
    float sp, cp;
    sincospif(2.0f * u0, &sp, &cp);
    const float z = (1.0f - u1) * (1.0f + Vl.z) + -Vl.z;
    const float s = sqrtf(fminf(fmaxf(1.0f - z * z, 0.0f), 1.0f));
    const V3 Hh = v3(cp * s + Vl.x, sp * s + Vl.y, z + Vl.z);
    const V3 H = normalize(t * (Hh.x * alpha) + b * (Hh.y * alpha) + N * fmaxf(Hh.z, 0.0f));
    return normalize(H * (2.0f * dot(V, H)) - V);
}

template <int KIND>
__global__ void gb_raygen_kernel(GbParams g, PassP pp, Queue q, float* ao_out, float4* rad_out) {
    const uint32_t n = g.w * g.h;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t pix = base + threadIdx.x;
        bool emit = false;
        V3 O = v3(0, 0, 0), L = v3(0, 0, 0);
        if (pix < n) {
            const uint32_t px = pix % g.w, py = pix / g.w;
            const float depth = g.depth[pix];
            bool traced = depth < 1.0f;
            float rough = 1.0f;
            if (KIND == kPassRefl) {
                rough = g.rough[pix];
                traced = traced && rough <= 1.0f;
            }
            if (traced) {
                float tx, ty;
                if (g.half_res) {
                    const uint32_t off = g.offset ? (g.offset[pix] & 3u) : 0u;
                    tx = (2.0f * float(px) + float(off & 1u) + 0.5f) / (2.0f * float(g.w));
                    ty = (2.0f * float(py) + float(off >> 1) + 0.5f) / (2.0f * float(g.h));
                } else {
                    tx = (float(px) + 0.5f) / float(g.w);
                    ty = (float(py) + 0.5f) / float(g.h);
                }
                // ConvertDepthToViewSpace (common/convert.hsh) and the world transforms
                const float4 vs = mat4_mul(g.ip, tx * 2.0f - 1.0f, ty * 2.0f - 1.0f, depth, 1.0f);
                const V3 viewPos = v3(vs.x / vs.w, vs.y / vs.w, vs.z / vs.w);
                const float4 wp = mat4_mul(g.iv, viewPos.x, viewPos.y, viewPos.z, 1.0f);
                const float4 vv = mat4_mul(g.iv, viewPos.x, viewPos.y, viewPos.z, 0.0f);
                const float2 en = g.normal[pix];
                const V3 vn = decode_normal(en.x, en.y);
                const float4 wn = mat4_mul(g.iv, vn.x, vn.y, vn.z, 0.0f);
                const V3 P = v3(wp.x, wp.y, wp.z), N = normalize(v3(wn.x, wn.y, wn.z));
                float u0, u1;
                if (g.samples) {
                    const float2 s = g.samples[pix];
                    u0 = s.x;
                    u1 = s.y;
                } else if (g.ranking) {
                    blue_noise(g, px, py, pp.frame_seed, u0, u1);
                } else {
                    u0 = rng(pix, pp.frame_seed, kSampleSlot, 0, pp.seed);
                    u1 = rng(pix, pp.frame_seed, kSampleSlot, 1, pp.seed);
                }
                const float viewLen = sqrtf(dot(viewPos, viewPos));
                if (KIND == kPassAO) {
                    // SampleDiffuseBRDF normalises L once more in UpdateSurface
                    L = normalize(cos_dir(N, u0, u1));
                    O = P + L * kEps + N * kEps;
                    emit = true;
                } else {
                    if (KIND == kPassRefl) {
                        u1 *= (1.0f - pp.bias);
                        const V3 V = normalize(v3(-vv.x, -vv.y, -vv.z));
                        if (rough > 0.01f) {
                            L = ggx_vndf_dir(N, V, rough * rough, u0, u1);
                        } else {
                            const V3 I = V * -1.0f;   // reflect(-V, N)
                            L = normalize(I - N * (2.0f * dot(N, I)));
                        }
                    } else {
                        u0 *= (1.0f - pp.bias);
                        L = cos_dir(N, u0, u1);
                    }
                    // isRayValid: false only when every component is NaN
                    const bool valid = !(isnan(L.x) && isnan(L.y) && isnan(L.z));
                    if (KIND == kPassRefl) {
                        const float viewOffset = fmaxf(1.0f, viewLen) * 0.1f;
                        O = P + L * kEps * 0.1f * viewOffset + N * kEps * viewOffset * 0.1f;
                        emit = valid && rough <= pp.cutoff;
                    } else {
                        const float viewOffset = fmaxf(1.0f, viewLen);
                        O = P + L * kEps * viewOffset * 0.01f + N * kEps * 0.01f * viewOffset;
                        emit = valid;
                    }
                }
            }
            if (!emit) {
                // nothing traced: ao 1, reflection / GI 0 (a valid untraced
                // reflection scales radiance 0 by the limit: still 0)
                if (KIND == kPassAO) ao_out[pix] = 1.0f;
                else rad_out[pix] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            }
        }
        uint32_t* const counters[1] = { q.count };
        const bool want[1] = { emit };
        uint32_t slots[1];
        block_append<1>(counters, want, slots);
        const uint32_t slot = slots[0];
        if (emit && slot < q.capacity) {
            float4* r = q.rays + size_t(slot) * 3;
            r[0] = make_float4(O.x, O.y, O.z, 0.0f);
            r[1] = make_float4(L.x, L.y, L.z, 0.0f);
            r[2] = make_float4(KIND == kPassAO ? pp.radius : kInfT, __int_as_float(-1), __int_as_float(-1), 0.0f);
            q.key[slot] = pix;
        }
    }
}

struct DdgiP {
    const float4* probes;
    const float4* dirs;
    const float4* dirs_inactive;
    float rot[9];
    uint32_t n_probes, ray_count, inactive_count;
};

// ddgi/rayGen.csh:39-81.  The queue is filled direction-major: the 32 rays
// of a warp share one direction of the set and start from 32 neighbouring
// probes, so they cross the scene side by side (probe-major order would give
// every warp 32 directions spread over the sphere).  Results still land at
// probe * ray_count + i through the key.
__global__ void ddgi_raygen_kernel(DdgiP d, Queue q) {
    const uint32_t total = d.n_probes * d.ray_count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t t = base + threadIdx.x;
        bool emit = false;
        V3 O = v3(0, 0, 0), D = v3(0, 0, 0);
        uint32_t idx = 0;
        if (t < total) {
            const uint32_t probe = t % d.n_probes, i = t / d.n_probes;
            idx = probe * d.ray_count + i;
            const float4 pr = d.probes[probe];
            const bool inactive = __float_as_uint(pr.w) == 2u;
            if (i < (inactive ? d.inactive_count : d.ray_count)) {
                const float4 v = inactive ? d.dirs_inactive[i] : d.dirs[i];
                D = normalize(v3(d.rot[0] * v.x + d.rot[3] * v.y + d.rot[6] * v.z,
                                 d.rot[1] * v.x + d.rot[4] * v.y + d.rot[7] * v.z,
                                 d.rot[2] * v.x + d.rot[5] * v.y + d.rot[8] * v.z));
                O = v3(pr.x, pr.y, pr.z);
                emit = true;
            }
        }
        uint32_t* const counters[1] = { q.count };
        const bool want[1] = { emit };
        uint32_t slots[1];
        block_append<1>(counters, want, slots);
        const uint32_t slot = slots[0];
        if (emit && slot < q.capacity) {
            float4* r = q.rays + size_t(slot) * 3;
            r[0] = make_float4(O.x, O.y, O.z, 0.0f);
            r[1] = make_float4(D.x, D.y, D.z, 0.0f);
            r[2] = make_float4(kInfT, __int_as_float(-1), __int_as_float(-1), 0.0f);
            q.key[slot] = idx;
        }
    }
}

// RTAO output: ao = 1 - occlusion (rtao.csh:93-106)
__global__ void ao_resolve_kernel(Queue q, const uint8_t* occ, const float* transparency, float* ao_out) {
    const uint32_t n = min(*q.count, q.capacity);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float hit = transparency ? __fsub_rn(1.0f, transparency[e]) : (occ[e] ? 1.0f : 0.0f);
        ao_out[q.key[e]] = __fsub_rn(1.0f, hit);
    }
}

struct ShadeP {
    PtScene sc;
    PassP pp;
    Queue q;                 // primary rays
    const float4* hits;      // ae_hit per queue entry
    float4* rad;             // per queue entry: radiance so far, hit distance
    Queue sq;                // shadow rays
    float4* shadow_pay;      // per shadow ray: contribution, primary entry
};

// EvaluateHit of rtreflection.csh:152-182 / rtgi.csh:155-185 (reflections,
// GI) and ddgi/rayHit.csh:62-95 (DDGI), up to the visibility test.
template <int KIND>
__global__ void pass_shade_kernel(ShadeP p) {
    const uint32_t n = min(*p.q.count, p.q.capacity);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        bool emit = false;
        float4 sr0{}, sr1{}, sr2{}, pay{};
        if (e < n) {
            const float4 h0 = p.hits[size_t(e) * 2], h1 = p.hits[size_t(e) * 2 + 1];
            const int32_t triPtr = __float_as_int(h0.y);
            V3 rad = v3(p.pp.env[0], p.pp.env[1], p.pp.env[2]);
            float dist = h0.x;
            if (triPtr >= 0) {
                const float4 o4 = p.q.rays[size_t(e) * 3], d4 = p.q.rays[size_t(e) * 3 + 1];
                Surf sf = make_surface(p.sc, ld3(o4), ld3(d4), h0.x, __float_as_int(h0.z), triPtr, h1.x, h1.y);
                if (KIND == kPassDDGI && sf.backface) {
                    rad = v3(0, 0, 0);
                    dist = -dist;
                } else {
                    rad = sf.mat.emissive;
                    LightSample ls;
                    const uint32_t key = p.q.key[e];
                    if (sample_light(p.sc, sf, key, p.pp.frame_seed, kLightSlot, p.pp.seed, ls)) {
                        V3 refl = KIND == kPassDDGI ? eval_diffuse(sf) : eval_diffuse(sf) + eval_specular(sf);
                        refl = refl * sf.mat.opacity;
                        const V3 c = refl * (ls.radiance * ls.solidAngle) * (sf.NdotL / ls.pdf);
                        // CheckVisibility traces whenever NdotL > 0; the light term can be
                        // negative (a one-sided back face seen from behind gives NdotV < 0),
                        // and the shaders add it as it is
                        if (sf.NdotL > 0.0f && (c.x != 0.0f || c.y != 0.0f || c.z != 0.0f)) {
                            const V3 so = sf.P + sf.N * kEps;
                            sr0 = make_float4(so.x, so.y, so.z, 0.0f);
                            sr1 = make_float4(sf.L.x, sf.L.y, sf.L.z, 0.0f);
                            sr2 = make_float4(ls.dist - 2.0f * kEps, __int_as_float(-1), __int_as_float(-1), 0.0f);
                            pay = make_float4(c.x, c.y, c.z, __uint_as_float(e));
                            emit = true;
                        }
                    }
                }
            }
            p.rad[e] = make_float4(rad.x, rad.y, rad.z, dist);
        }
        uint32_t* const counters[1] = { p.sq.count };
        const bool want[1] = { emit };
        uint32_t slots[1];
        block_append<1>(counters, want, slots);
        const uint32_t slot = slots[0];
        if (emit && slot < p.sq.capacity) {
            float4* r = p.sq.rays + size_t(slot) * 3;
            r[0] = sr0;
            r[1] = sr1;
            r[2] = sr2;
            p.shadow_pay[slot] = pay;
        }
    }
}

// the light a shadow ray carries, times its visibility
__global__ void pass_shadow_resolve_kernel(Queue sq, const float4* shadow_pay, const uint8_t* occ,
                                           const float* transparency, float4* rad) {
    const uint32_t n = min(*sq.count, sq.capacity);
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const float vis = transparency ? transparency[s] : (occ[s] ? 0.0f : 1.0f);
        if (vis == 0.0f) continue;
        const float4 c = shadow_pay[s];
        float4& r = rad[__float_as_uint(c.w)];
        r.x += c.x * vis;
        r.y += c.y * vis;
        r.z += c.z * vis;
    }
}

__device__ __forceinline__ uint32_t half_bits(float x) { return __half_as_ushort(__float2half_rn(x)); }

template <int KIND>
__global__ void pass_output_kernel(Queue q, const float4* rad, float limit, float4* out) {
    const uint32_t n = min(*q.count, q.capacity);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float4 r = rad[e];
        if (KIND == kPassDDGI) {
            // PackRayHit, ddgi/ddgi.hsh:85-98
            const float4 d = q.rays[size_t(e) * 3 + 1];
            const float rx = fminf(r.x, 3200.0f), ry = fminf(r.y, 3200.0f), rz = fminf(r.z, 3200.0f);
            out[q.key[e]] = make_float4(__uint_as_float(half_bits(d.x) | (half_bits(d.y) << 16)),
                                        __uint_as_float(half_bits(rx) | (half_bits(ry) << 16)),
                                        __uint_as_float(half_bits(d.z) | (half_bits(rz) << 16)), r.w);
        } else {
            // radiance limit, rtreflection.csh:140-142
            const float m = fmaxf(fmaxf(fmaxf(r.x, fmaxf(r.y, r.z)), limit), 0.01f);
            const float s = limit / m;
            out[q.key[e]] = make_float4(r.x * s, r.y * s, r.z * s, 1.0f);
        }
    }
}

PtScene Scene(ae_rt_ctx* ctx) {
    PtScene sc{};
    sc.instances = ctx->d_instances;
    sc.inst_model = ctx->d_inst_model;
    sc.meshes = ctx->d_mesh_table;
    sc.materials = ctx->d_materials;
    sc.n_materials = ctx->n_materials;
    sc.lights = ctx->d_lights;
    sc.n_lights = ctx->n_lights;
    sc.tex.pool = ctx->d_tex_pool;
    sc.tex.desc = static_cast<const atlas::rt::dev::TexDesc*>(ctx->d_tex_desc);
    sc.tex.n = ctx->n_textures;
    return sc;
}

uint32_t Blocks(ae_rt_ctx* ctx, uint32_t n) {
    const uint32_t want = (n + 255u) / 256u, cap = uint32_t(ctx->sm_count) * 8u;
    return want == 0 ? 1u : (want < cap ? want : cap);
}

ae_rt_status CheckScene(ae_rt_ctx* ctx, const ae_rt_pass_params* params, bool shading) {
    if (!ctx || !params) return AE_RT_INVALID_ARG;
    if (!ctx->scene_ready) return Fail(ctx, AE_RT_INVALID_ARG, "no scene has been set");
    if ((params->flags & AE_PASS_OPACITY_CHECK) || shading) {
        for (const DeviceMesh& m : ctx->meshes)
            if (m.n_nodes > 0 && !m.shading)
                return Fail(ctx, AE_RT_INVALID_ARG, "these passes need the meshes' shading triangles");
    }
    if (shading && !ctx->d_materials) return Fail(ctx, AE_RT_INVALID_ARG, "no materials have been set");
    return AE_RT_OK;
}

ae_rt_status CheckGBuffer(ae_rt_ctx* ctx, const ae_gbuffer* gb, bool need_rough) {
    if (!gb) return Fail(ctx, AE_RT_INVALID_ARG, "null G-buffer");
    if (!gb->depth || !gb->normal || (need_rough && !gb->roughness))
        return Fail(ctx, AE_RT_INVALID_ARG, need_rough ? "the G-buffer needs depth, normal and roughness"
                                                       : "the G-buffer needs depth and normal");
    if (uint64_t(gb->width) * gb->height > (1u << 26))
        return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^26 pixels");
    for (const void* ptr : { static_cast<const void*>(gb->depth), static_cast<const void*>(gb->normal),
                             static_cast<const void*>(gb->offset), static_cast<const void*>(gb->roughness),
                             static_cast<const void*>(gb->samples), static_cast<const void*>(gb->scrambling_ranking),
                             static_cast<const void*>(gb->sobol_sequence) })
        if (ptr && !IsDevicePointer(ptr)) return Fail(ctx, AE_RT_INVALID_ARG, "G-buffer planes must be device memory");
    if (!gb->scrambling_ranking != !gb->sobol_sequence)
        return Fail(ctx, AE_RT_INVALID_ARG, "the blue-noise ranking and Sobol textures come together");
    if ((reinterpret_cast<uintptr_t>(gb->scrambling_ranking) | reinterpret_cast<uintptr_t>(gb->sobol_sequence)) & 3u)
        return Fail(ctx, AE_RT_INVALID_ARG, "the blue-noise textures must be 4-byte aligned");
    return AE_RT_OK;
}

PassP Pass(const ae_rt_pass_params* params) {
    PassP pp{};
    pp.radius = params->radius;
    pp.bias = params->bias;
    pp.cutoff = params->roughness_cutoff;
    pp.limit = params->radiance_limit;
    for (int k = 0; k < 3; k++) pp.env[k] = params->environment[k];
    pp.frame_seed = params->frame_seed;
    pp.seed = params->seed;
    pp.tex_level = params->texture_level;
    return pp;
}

GbParams GBuffer(const ae_gbuffer* gb) {
    GbParams g{};
    g.depth = gb->depth;
    g.normal = reinterpret_cast<const float2*>(gb->normal);
    g.offset = gb->offset;
    g.rough = gb->roughness;
    g.samples = reinterpret_cast<const float2*>(gb->samples);
    g.ranking = reinterpret_cast<const uchar4*>(gb->scrambling_ranking);
    g.sobol = reinterpret_cast<const uchar4*>(gb->sobol_sequence);
    g.w = gb->width;
    g.h = gb->height;
    g.half_res = gb->half_res ? 1u : 0u;
    for (int k = 0; k < 16; k++) {
        g.ip[k] = gb->ip_matrix[k];
        g.iv[k] = gb->iv_matrix[k];
    }
    return g;
}

// Scratch of the passes for `cap` primary rays: queue, hits, per-entry
// radiance, shadow queue.
ae_rt_status EnsurePassScratch(ae_rt_ctx* ctx, uint32_t cap, Queue& q, Queue& sq) {
    AE_CUDA(ctx, ctx->pass_rays.ensure(size_t(cap) * sizeof(ae_packed_ray)));
    AE_CUDA(ctx, ctx->pass_key.ensure(size_t(cap) * sizeof(uint32_t)));
    AE_CUDA(ctx, ctx->pass_hits.ensure(size_t(cap) * sizeof(ae_hit)));
    AE_CUDA(ctx, ctx->pass_rad.ensure(size_t(cap) * sizeof(float4)));
    AE_CUDA(ctx, ctx->pass_shadow.ensure(size_t(cap) * sizeof(ae_packed_ray)));
    AE_CUDA(ctx, ctx->pass_shadow_pay.ensure(size_t(cap) * sizeof(float4)));
    AE_CUDA(ctx, ctx->pass_vis.ensure(size_t(cap) * sizeof(float)));
    AE_CUDA(ctx, ctx->pass_counts.ensure(2 * sizeof(uint32_t)));
    uint32_t* counts = static_cast<uint32_t*>(ctx->pass_counts.ptr);
    q = Queue{ static_cast<float4*>(ctx->pass_rays.ptr), static_cast<uint32_t*>(ctx->pass_key.ptr), counts, cap };
    sq = Queue{ static_cast<float4*>(ctx->pass_shadow.ptr), nullptr, counts + 1, cap };
    return AE_RT_OK;
}

// Trace of the primary queue (closest or any) with or without transparency.
ae_rt_status TracePrimary(ae_rt_ctx* ctx, bool any, bool opacity, const Queue& q, float tmax, void* out,
                          void* stream) {
    const ae_packed_ray* rays = reinterpret_cast<const ae_packed_ray*>(q.rays);
    if (opacity) return TraceTransparency(ctx, any, rays, q.capacity, 0.0f, tmax, AE_RT_MASK_ALL, out, stream, q.count);
    return TraceSceneQueue(ctx, any, rays, q.capacity, 0.0f, tmax, out, stream, q.count, AE_RT_MASK_ALL, false);
}

// Steps 3-4 of the shading passes: shade, shadow trace, resolve, output.
template <int KIND>
ae_rt_status ShadeAndResolve(ae_rt_ctx* ctx, const PassP& pp, const Queue& q, const Queue& sq, float4* out,
                             cudaStream_t s) {
    ShadeP sp{};
    sp.sc = Scene(ctx);
    sp.sc.tex_level = KIND == kPassDDGI ? 4u : pp.tex_level;   // ddgi/rayHit.csh:79
    sp.pp = pp;
    sp.q = q;
    sp.hits = static_cast<const float4*>(ctx->pass_hits.ptr);
    sp.rad = static_cast<float4*>(ctx->pass_rad.ptr);
    sp.sq = sq;
    sp.shadow_pay = static_cast<float4*>(ctx->pass_shadow_pay.ptr);
    const uint32_t blocks = Blocks(ctx, q.capacity);
    pass_shade_kernel<KIND><<<blocks, 256, 0, s>>>(sp);
    AE_CUDA(ctx, cudaGetLastError());
    const ae_packed_ray* srays = reinterpret_cast<const ae_packed_ray*>(sq.rays);
    ae_rt_status st;
    if (KIND == kPassDDGI)   // CheckVisibility, ddgi/rayHit.csh:140-151
        st = TraceSceneQueue(ctx, true, srays, sq.capacity, 0.0f, kInfT, ctx->pass_vis.ptr, s, sq.count,
                             AE_RT_MASK_SHADOW, true);
    else                     // CheckVisibility, rtreflection.csh:232-245 / rtgi.csh:222-234
        st = TraceTransparency(ctx, true, srays, sq.capacity, 0.0f, kInfT, AE_RT_MASK_SHADOW, ctx->pass_vis.ptr, s,
                               sq.count, true);
    if (st != AE_RT_OK) return st;
    const bool opaqueVis = KIND == kPassDDGI;
    pass_shadow_resolve_kernel<<<blocks, 256, 0, s>>>(
        sq, sp.shadow_pay, opaqueVis ? static_cast<const uint8_t*>(ctx->pass_vis.ptr) : nullptr,
        opaqueVis ? nullptr : static_cast<const float*>(ctx->pass_vis.ptr), sp.rad);
    AE_CUDA(ctx, cudaGetLastError());
    pass_output_kernel<KIND><<<blocks, 256, 0, s>>>(q, sp.rad, pp.limit, out);
    AE_CUDA(ctx, cudaGetLastError());
    return AE_RT_OK;
}

template <int KIND>
ae_rt_status ScreenPass(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params, void* out,
                        void* stream) {
    ae_rt_status st = CheckScene(ctx, params, KIND != kPassAO);
    if (st != AE_RT_OK) return st;
    if (!gb) return Fail(ctx, AE_RT_INVALID_ARG, "null G-buffer");
    if (gb->width == 0 || gb->height == 0) return AE_RT_OK;
    st = CheckGBuffer(ctx, gb, KIND == kPassRefl);
    if (st != AE_RT_OK) return st;
    if (!out || !IsDevicePointer(out)) return Fail(ctx, AE_RT_INVALID_ARG, "the output must be device memory");
    const uint32_t n = gb->width * gb->height;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Queue q, sq;
    st = EnsurePassScratch(ctx, n, q, sq);
    if (st != AE_RT_OK) return st;
    AE_CUDA(ctx, cudaMemsetAsync(q.count, 0, 2 * sizeof(uint32_t), s));
    const PassP pp = Pass(params);
    const bool opacity = (params->flags & AE_PASS_OPACITY_CHECK) != 0;
    gb_raygen_kernel<KIND><<<Blocks(ctx, n), 256, 0, s>>>(GBuffer(gb), pp, q, static_cast<float*>(out),
                                                          static_cast<float4*>(out));
    AE_CUDA(ctx, cudaGetLastError());
    if (KIND == kPassAO) {
        st = TracePrimary(ctx, true, opacity, q, params->radius, ctx->pass_vis.ptr, stream);
        if (st != AE_RT_OK) return st;
        ao_resolve_kernel<<<Blocks(ctx, n), 256, 0, s>>>(
            q, opacity ? nullptr : static_cast<const uint8_t*>(ctx->pass_vis.ptr),
            opacity ? static_cast<const float*>(ctx->pass_vis.ptr) : nullptr, static_cast<float*>(out));
        AE_CUDA(ctx, cudaGetLastError());
        return AE_RT_OK;
    }
    st = TracePrimary(ctx, false, opacity, q, kInfT, ctx->pass_hits.ptr, stream);
    if (st != AE_RT_OK) return st;
    return ShadeAndResolve<KIND>(ctx, pp, q, sq, static_cast<float4*>(out), s);
}

}  // namespace

extern "C" {

ae_rt_status ae_rt_rtao(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params, float* ao,
                        void* stream) {
    return ScreenPass<kPassAO>(ctx, gb, params, ao, stream);
}

ae_rt_status ae_rt_reflections(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params,
                               float* radiance, void* stream) {
    return ScreenPass<kPassRefl>(ctx, gb, params, radiance, stream);
}

ae_rt_status ae_rt_rtgi(ae_rt_ctx* ctx, const ae_gbuffer* gb, const ae_rt_pass_params* params, float* radiance,
                        void* stream) {
    return ScreenPass<kPassGI>(ctx, gb, params, radiance, stream);
}

ae_rt_status ae_rt_ddgi_trace(ae_rt_ctx* ctx, const ae_ddgi_probes* probes, const ae_rt_pass_params* params,
                              float* hits, void* stream) {
    ae_rt_status st = CheckScene(ctx, params, true);
    if (st != AE_RT_OK) return st;
    if (!probes || !hits) return Fail(ctx, AE_RT_INVALID_ARG, "null probes or hit buffer");
    const uint64_t total = uint64_t(probes->n_probes) * probes->ray_count;
    if (total == 0) return AE_RT_OK;
    if (total > (1u << 26)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^26 probe rays");
    if (!probes->probes || !probes->ray_dirs || (probes->inactive_ray_count && !probes->ray_dirs_inactive))
        return Fail(ctx, AE_RT_INVALID_ARG, "null probe or direction buffer");
    for (const void* ptr : { static_cast<const void*>(probes->probes), static_cast<const void*>(probes->ray_dirs),
                             static_cast<const void*>(probes->ray_dirs_inactive), static_cast<const void*>(hits) })
        if (ptr && !IsDevicePointer(ptr)) return Fail(ctx, AE_RT_INVALID_ARG, "probe buffers must be device memory");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Queue q, sq;
    st = EnsurePassScratch(ctx, uint32_t(total), q, sq);
    if (st != AE_RT_OK) return st;
    AE_CUDA(ctx, cudaMemsetAsync(q.count, 0, 2 * sizeof(uint32_t), s));
    DdgiP d{};
    d.probes = reinterpret_cast<const float4*>(probes->probes);
    d.dirs = reinterpret_cast<const float4*>(probes->ray_dirs);
    d.dirs_inactive = reinterpret_cast<const float4*>(probes->ray_dirs_inactive);
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) d.rot[c * 3 + r] = probes->rotation[c * 4 + r];
    d.n_probes = probes->n_probes;
    d.ray_count = probes->ray_count;
    d.inactive_count = probes->inactive_ray_count < probes->ray_count ? probes->inactive_ray_count
                                                                     : probes->ray_count;
    ddgi_raygen_kernel<<<Blocks(ctx, uint32_t(total)), 256, 0, s>>>(d, q);
    AE_CUDA(ctx, cudaGetLastError());
    const bool opacity = (params->flags & AE_PASS_OPACITY_CHECK) != 0;
    st = TracePrimary(ctx, false, opacity, q, kInfT, ctx->pass_hits.ptr, stream);
    if (st != AE_RT_OK) return st;
    return ShadeAndResolve<kPassDDGI>(ctx, Pass(params), q, sq, reinterpret_cast<float4*>(hits), s);
}

}  // extern "C"
