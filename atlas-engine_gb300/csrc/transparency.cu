// The transparency traversal variants (include/atlas_rt.h,
// ae_rt_trace_scene_*_transparency):
//   HitClosestTransparency  data/shader/raytracer/bvh.hsh:275-357
//                           (+ CheckLeafClosestTransparency :106-138)
//   HitAnyTransparency      data/shader/raytracer/bvh.hsh:443-524
//                           (+ CheckLeafTransparency :140-170)
// over the context's two-level scene.  The box tests, the triangle test and
// the instance transform are the bit-exact ones of the opaque traversal
// (trace_kernels.cuh); the leaves read the 96-byte shading triangle
// (UnpackTriangle, common.hsh:17-44): its vertices, endOfNode = d1.z > 0 and
// opacity = d2.w, or, when that is negative, GetOpacity (surface.hsh:147-159,
// texture.cuh): the material's opacity times its opacity texture sampled at
// the hit's interpolated UV, 1.0 when absent (texture.hsh:18-25).
//  * closest: a triangle hit counts only where its opacity is > 0;
//  * any: every accepted triangle multiplies the leaf's running
//    transparency, which starts from the current value; the leaf's result
//    multiplies the current value again (`transparency *=
//    CheckLeafTransparency(..., transparency)`, bvh.hsh:500), values below
//    1e-6 become 0, and the traversal ends at 0.
// These queries are off the configs' hot path (every material there is
// opaque): one thread per ray, a local stack, no persistent scheduling.
#include "atlas_rt.h"
#include "context.cuh"
#include "trace_kernels.cuh"
#include "texture.cuh"

using namespace atlas::rt::host;
using namespace atlas::rt::dev;

namespace {

constexpr uint32_t kTransStack = 128;

struct TransParams {
    const float4* tlas;
    uint32_t n_tlas;
    const float4* instances;
    const MeshDesc* meshes;
    const float* materials;      // GPUMaterial (23 words), may be null (opacity 1)
    uint32_t n_materials;
    TexTable textures;
    const float4* rays;
    uint32_t n;                  // rays, or the queue's capacity when count is set
    const uint32_t* count;       // device-side ray count (queues), or null
    uint32_t per_ray_tmax;       // tmax of ray i = its third vector's x
    float tmin, tmax;
    uint32_t cull_mask;
    uint32_t max_steps;
    float4* hits;                // closest: ae_hit (2 float4)
    float* transparency;         // any
    uint32_t* error_word;
};

// `tri.opacity < 0.0 ? GetOpacity(tri, sol.yz, materialOffset, 0) : tri.opacity`
__device__ __forceinline__ float shading_opacity(const TransParams& p, float4 d0, float4 d2, int32_t matOffset,
                                                 float u, float v) {
    if (!(d2.w < 0.0f)) return d2.w;
    return get_opacity(p.materials, p.n_materials, p.textures, d0, matOffset, u, v);
}

template <bool ANY>
__global__ void transparency_kernel(TransParams p) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const uint32_t n = p.count ? min(*p.count, p.n) : p.n;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 o4 = p.rays[i * 3], d4 = p.rays[i * 3 + 1];
        TRay wr{};
        wr.ox = o4.x; wr.oy = o4.y; wr.oz = o4.z;
        wr.dx = d4.x; wr.dy = d4.y; wr.dz = d4.z;
        wr.prepare();
        TRay r = wr;
        const float tMin = p.tmin, tMax = p.per_ray_tmax ? p.rays[i * 3 + 2].x : p.tmax;
        float hitDist = tMax, hu = 0.0f, hv = 0.0f, transparency = 1.0f;
        int32_t hitID = -1, hitInst = -1, curInst = -1, matOffset = 0;
        uint32_t flags = 0;
        const float4* blasNodes = nullptr;
        const float4* shading = nullptr;
        const bool nanDir = isnan(d4.x) || isnan(d4.y) || isnan(d4.z);
        if (p.n_tlas > 0 && !nanDir) {
            int32_t stack[kTransStack];
            uint32_t sp = 1, tlasIndex = kTlasInvalid, steps = 0;
            int32_t nodePtr = 0;
            stack[0] = 0;
            while (sp != 0 && (!ANY || transparency > 0.0f)) {
                if (++steps > p.max_steps) {
                    flags |= kHitFlagIterCap;
                    atomicOr(p.error_word, kErrIterationCap);
                    break;
                }
                int32_t next = 0;
                bool pop = false;
                if (sp < tlasIndex) {
                    r = wr;
                    tlasIndex = kTlasInvalid;
                    if (nodePtr < 0) {
                        // CheckInstance -- bvh.hsh:172-189
                        const uint32_t ii = uint32_t(~nodePtr);
                        const float4* ip = p.instances + size_t(ii) * 4;
                        const float4 c0 = __ldg(ip), c1 = __ldg(ip + 1), c2 = __ldg(ip + 2), c3 = __ldg(ip + 3);
                        curInst = int32_t(ii);
                        const MeshDesc m = p.meshes[__float_as_int(c3.x)];
                        matOffset = __float_as_int(c3.y);
                        r.ox = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c0);
                        r.oy = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c1);
                        r.oz = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c2);
                        r.dx = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c0);
                        r.dy = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c1);
                        r.dz = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c2);
                        r.prepare();
                        blasNodes = m.nodes;
                        shading = m.shading;
                        if ((__float_as_uint(c3.w) & p.cull_mask) != 0u && m.n_nodes > 0 && shading) {
                            nodePtr = 0;
                            tlasIndex = sp;
                            continue;
                        }
                        pop = true;
                    } else {
                        const float4* np = p.tlas + size_t(nodePtr) * 4;
                        const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
                        bool il, ir, leftFirst;
                        bool nearCullUnused;   // near-tie detection is the closest-hit trace's alone
                        test_children<false>(r, n0, n1, n2, n3, tMin, ANY ? tMax : hitDist, !ANY, false, il, ir,
                                             leftFirst, nearCullUnused);
                        const int32_t l = __float_as_int(n3.x), rr = __float_as_int(n3.y);
                        if (ANY) {
                            next = il ? l : rr;
                            if (il && ir) {
                                if (sp >= kTransStack) { flags |= kHitFlagOverflow; atomicOr(p.error_word, kErrStackOverflow); break; }
                                stack[sp++] = rr;
                            }
                        } else {
                            next = leftFirst ? l : rr;
                            if (il && ir) {
                                if (sp >= kTransStack) { flags |= kHitFlagOverflow; atomicOr(p.error_word, kErrStackOverflow); break; }
                                stack[sp++] = leftFirst ? rr : l;
                            }
                        }
                        pop = !il && !ir;
                    }
                } else if (nodePtr < 0) {
                    int32_t tp = ~nodePtr;
                    bool end = false;
                    float leaf = transparency;
                    do {
                        const float4* sp4 = shading + size_t(tp) * 6;
                        const float4 a = __ldg(sp4), b = __ldg(sp4 + 1), c = __ldg(sp4 + 2);
                        const float4 d0 = __ldg(sp4 + 3), d1 = __ldg(sp4 + 4), d2 = __ldg(sp4 + 5);
                        end = d1.z > 0.0f;
                        float t, u, v;
                        const bool hit = tri_test(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, a, b, c, t, u, v);
                        if (ANY) {
                            if (hit && t > tMin && t < tMax)
                                leaf = __fmul_rn(leaf, __fsub_rn(1.0f, shading_opacity(p, d0, d2, matOffset, u, v)));
                        } else if (hit && t > tMin && t < hitDist && shading_opacity(p, d0, d2, matOffset, u, v) > 0.0f) {
                            hitDist = t; hitID = tp; hu = u; hv = v; hitInst = curInst;
                        }
                        tp++;
                    } while (!end);
                    if (ANY) {
                        transparency = __fmul_rn(transparency, leaf);
                        if (transparency < 0.000001f) transparency = 0.0f;
                    }
                    pop = true;
                } else {
                    const float4* np = blasNodes + size_t(nodePtr) * 4;
                    const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
                    bool il, ir, leftFirst;
                    bool nearCullUnused;   // near-tie detection is the closest-hit trace's alone
                    test_children<false>(r, n0, n1, n2, n3, tMin, ANY ? tMax : hitDist, !ANY, false, il, ir, leftFirst,
                                         nearCullUnused);
                    const int32_t l = __float_as_int(n3.x), rr = __float_as_int(n3.y);
                    if (ANY) {
                        next = il ? l : rr;
                        if (il && ir) {
                            if (sp >= kTransStack) { flags |= kHitFlagOverflow; atomicOr(p.error_word, kErrStackOverflow); break; }
                            stack[sp++] = rr;
                        }
                    } else {
                        next = leftFirst ? l : rr;
                        if (il && ir) {
                            if (sp >= kTransStack) { flags |= kHitFlagOverflow; atomicOr(p.error_word, kErrStackOverflow); break; }
                            stack[sp++] = leftFirst ? rr : l;
                        }
                    }
                    pop = !il && !ir;
                }
                nodePtr = pop ? stack[--sp] : next;
            }
        }
        if (ANY) {
            p.transparency[i] = transparency;
        } else {
            if (hitID >= 0) flags |= kHitFlagHit;
            float4* h = p.hits + i * 2;
            h[0] = make_float4(hitDist, __int_as_float(hitID), __int_as_float(hitInst), __uint_as_float(flags));
            h[1] = make_float4(hu, hv, tMax, 0.0f);
        }
    }
}

}  // namespace

ae_rt_status atlas::rt::host::TraceTransparency(ae_rt_ctx* ctx, bool any, const ae_packed_ray* rays, uint32_t n,
                                                float tmin, float tmax, uint32_t cull_mask, void* out, void* stream,
                                                const uint32_t* count_dev, bool per_ray_tmax) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!ctx->scene_ready) return Fail(ctx, AE_RT_INVALID_ARG, "no scene has been set");
    if (n == 0) return AE_RT_OK;
    if (!rays || !out) return Fail(ctx, AE_RT_INVALID_ARG, "null ray or result buffer");
    if (n > (1u << 30)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^30 rays in one call");
    if (count_dev && (!IsDevicePointer(rays) || !IsDevicePointer(out)))
        return Fail(ctx, AE_RT_INVALID_ARG, "queue traces take device buffers");
    for (const DeviceMesh& m : ctx->meshes)
        if (m.n_nodes > 0 && !m.shading)
            return Fail(ctx, AE_RT_INVALID_ARG, "transparency queries need the meshes' shading triangles");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t rb = size_t(n) * sizeof(ae_packed_ray), ob = size_t(n) * (any ? sizeof(float) : sizeof(ae_hit));
    const bool rays_dev = IsDevicePointer(rays), out_dev = IsDevicePointer(out);
    const void* d_rays = rays;
    void* d_out = out;
    if (!rays_dev) {
        AE_CUDA(ctx, ctx->rays_in.ensure(rb));
        AE_CUDA(ctx, cudaMemcpyAsync(ctx->rays_in.ptr, rays, rb, cudaMemcpyHostToDevice, s));
        d_rays = ctx->rays_in.ptr;
    }
    if (!out_dev) {
        AE_CUDA(ctx, ctx->results_out.ensure(ob));
        d_out = ctx->results_out.ptr;
    }
    TransParams p{};
    p.tlas = ctx->d_tlas;
    p.n_tlas = ctx->n_tlas;
    p.instances = ctx->d_instances;
    p.meshes = ctx->d_mesh_table;
    p.materials = ctx->d_materials;
    p.n_materials = ctx->n_materials;
    p.textures.pool = ctx->d_tex_pool;
    p.textures.desc = static_cast<const TexDesc*>(ctx->d_tex_desc);
    p.textures.n = ctx->n_textures;
    p.rays = static_cast<const float4*>(d_rays);
    p.n = n;
    p.count = count_dev;
    p.per_ray_tmax = per_ray_tmax ? 1u : 0u;
    p.tmin = tmin;
    p.tmax = tmax;
    p.cull_mask = cull_mask;
    p.max_steps = ctx->max_steps_cfg ? ctx->max_steps_cfg : ctx->scene_steps;
    p.hits = any ? nullptr : static_cast<float4*>(d_out);
    p.transparency = any ? static_cast<float*>(d_out) : nullptr;
    p.error_word = ctx->d_counter + 1;
    const uint32_t want = (n + 127) / 128, cap = uint32_t(ctx->sm_count) * 16u;
    const uint32_t blocks = want < cap ? want : cap;
    if (any) transparency_kernel<true><<<blocks, 128, 0, s>>>(p);
    else transparency_kernel<false><<<blocks, 128, 0, s>>>(p);
    AE_CUDA(ctx, cudaGetLastError());
    if (!out_dev) AE_CUDA(ctx, cudaMemcpyAsync(out, d_out, ob, cudaMemcpyDeviceToHost, s));
    if (!out_dev || !rays_dev) return ae_rt_synchronize(ctx, stream);
    return AE_RT_OK;
}

extern "C" {

ae_rt_status ae_rt_trace_scene_closest_transparency(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays,
                                                    float tmin, float tmax, uint32_t cull_mask, ae_hit* out,
                                                    void* stream) {
    return TraceTransparency(ctx, false, rays, n_rays, tmin, tmax, cull_mask, out, stream);
}

ae_rt_status ae_rt_trace_scene_any_transparency(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays,
                                                float tmin, float tmax, uint32_t cull_mask, float* transparency,
                                                void* stream) {
    return TraceTransparency(ctx, true, rays, n_rays, tmin, tmax, cull_mask, transparency, stream);
}

}  // extern "C"
