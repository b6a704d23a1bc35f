// Wavefront stages around the traversal kernels: primary ray generation and
// the bounce/shadow ray spawn that follows a closest-hit trace.
//
//  * raygen_kernel: pinhole camera rays from the frustum description of the
//    engine's ray-gen pass (data/shader/pathtracer/rayGen.csh:25-91,
//    PathTracingRenderer.cpp:157-160): dir = normalize(origin + right*u +
//    bottom*v - location), u,v = (pixel + jitter) / resolution.  Rays are
//    written in rayGen.csh's queue order (8 x 8 work groups, then the
//    partial groups; :53-80) so that neighbouring lanes trace neighbouring
//    pixels; ray.ID = pixel index.
//    Arithmetic is explicitly rounded in a fixed order, so a host can
//    regenerate the same rays bit for bit.
//  * spawn_kernel: for every hit, one cosine-weighted diffuse bounce ray
//    (origin pushed back along the view direction by EPSILON, as
//    rayHit.csh:282) and, when the light is above the surface, one shadow
//    ray towards a directional light (origin lifted along the normal by
//    EPSILON, rayHit.csh:327-338).  Queue appends are warp-aggregated: one
//    atomic per warp and queue (the reference takes one per ray,
//    tracing.hsh:70-77).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "camera.cuh"

namespace atlas::rt::dev {

struct SpawnParams {
    const float4* rays;        // primary rays, or null: made from `cam` (the camera trace)
    CameraParams cam;
    const float4* hits;        // 2 float4 per ae_hit
    const uint32_t* n_dev;     // optional device count
    uint32_t n;
    const float4* tris;        // GPUBVHTriangle
    float4* secondary;         // PackedRay queue
    float4* shadow;            // PackedRay queue
    uint32_t* counts;          // [0] secondary, [1] shadow
    float lightx, lighty, lightz;
    float epsilon;
    uint32_t seed;
};

static __global__ void raygen_kernel(CameraParams c, float4* rays) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = c.width * c.height;
    if (i >= n) return;
    float4 o, d;
    camera_ray(c, i, o, d);
    float4* r = rays + size_t(i) * 3;
    r[0] = o;
    r[1] = d;
    r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
}

// Integer hash of Jarzynski & Olano, "Hash Functions for GPU Rendering"
// (JCGT 2020), PCG variant.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
    const uint32_t state = x * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

__device__ __forceinline__ float rand01(uint32_t a, uint32_t b, uint32_t c) {
    const uint32_t h = pcg_hash(a ^ pcg_hash(b ^ pcg_hash(c)));
    return float(h >> 8) * (1.0f / 16777216.0f);
}

// Orthonormal basis around a unit normal: Duff et al., "Building an
// Orthonormal Basis, Revisited" (JCGT 2017).
__device__ __forceinline__ void onb(float nx, float ny, float nz, float3& t, float3& b) {
    const float sign = copysignf(1.0f, nz);
    const float a = -1.0f / (sign + nz);
    const float bb = nx * ny * a;
    t = make_float3(1.0f + sign * nx * nx * a, sign * bb, -sign * nx);
    b = make_float3(bb, sign + ny * ny * a, -ny);
}

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want, uint32_t lane) {
    const uint32_t mask = __ballot_sync(0xffffffffu, want);
    uint32_t base = 0;
    const uint32_t leader = mask ? (__ffs(mask) - 1) : 0;
    if (mask && lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    uint32_t lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return base + __popc(mask & lt);
}

// Queue appends aggregated over the block: one atomicAdd per block and
// queue.  Appending per warp instead puts 8k-65k atomics on one address for
// a full-screen queue, and they serialise in L2.  Every thread of the block
// must call this the same number of times (it synchronises the block), with
// blockDim.x a multiple of 32 and at most 1024.  slot[q] is valid where
// want[q] is set.
template <int NQ>
__device__ __forceinline__ void block_append(uint32_t* const (&counters)[NQ], const bool (&want)[NQ],
                                             uint32_t (&slot)[NQ]) {
    __shared__ uint32_t sm[NQ][33];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    uint32_t mask[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        mask[q] = __ballot_sync(0xffffffffu, want[q]);
        if (lane == 0) sm[q][warp] = __popc(mask[q]);
    }
    __syncthreads();
    if (threadIdx.x < uint32_t(NQ)) {
        const uint32_t q = threadIdx.x;
        uint32_t total = 0;
        for (uint32_t w = 0; w < warps; w++) {
            const uint32_t c = sm[q][w];
            sm[q][w] = total;
            total += c;
        }
        sm[q][32] = total ? atomicAdd(counters[q], total) : 0u;
    }
    __syncthreads();
    uint32_t lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
#pragma unroll
    for (int q = 0; q < NQ; q++) slot[q] = sm[q][32] + sm[q][warp] + __popc(mask[q] & lt);
    __syncthreads();
}

// Append to one queue in an order sorted by a small key within the block:
// a counting sort over KEYS buckets in shared memory, one atomicAdd per block
// on the global counter.  Rays of one bucket (e.g. one direction octant)
// land next to each other, so a warp of the tracing kernel gets rays that
// cross the BVH the same way.  Every thread of the block must call it.
template <int KEYS>
__device__ __forceinline__ uint32_t block_append_sorted(uint32_t* counter, bool want, uint32_t key) {
    __shared__ uint32_t hist[KEYS + 1];
    if (threadIdx.x <= uint32_t(KEYS)) hist[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t rank = want ? atomicAdd(&hist[key], 1u) : 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int k = 0; k < KEYS; k++) {
            const uint32_t c = hist[k];
            hist[k] = total;
            total += c;
        }
        hist[KEYS] = total ? atomicAdd(counter, total) : 0u;
    }
    __syncthreads();
    const uint32_t slot = hist[KEYS] + hist[want ? key : 0u] + rank;
    __syncthreads();
    return slot;
}

static __global__ void spawn_kernel(SpawnParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = p.n_dev ? min(*p.n_dev, p.n) : p.n;
    bool sec = false, shd = false;
    float3 P = make_float3(0, 0, 0), N = make_float3(0, 0, 0), D = make_float3(0, 0, 0), S = make_float3(0, 0, 0);
    int32_t id = 0;
    if (i < n) {
        const float4 h0 = p.hits[size_t(i) * 2];
        const int32_t tp = __float_as_int(h0.y);
        if (tp >= 0) {
            float4 o4, d4;
            if (p.rays) {
                o4 = p.rays[size_t(i) * 3];
                d4 = p.rays[size_t(i) * 3 + 1];
            } else {
                camera_ray(p.cam, i, o4, d4);
            }
            id = __float_as_int(o4.w);
            const float t = h0.x;
            P = make_float3(o4.x + t * d4.x, o4.y + t * d4.y, o4.z + t * d4.z);
            const float4 a = __ldg(p.tris + size_t(tp) * 3), b = __ldg(p.tris + size_t(tp) * 3 + 1),
                         c = __ldg(p.tris + size_t(tp) * 3 + 2);
            const float3 e0 = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
            const float3 e1 = make_float3(c.x - a.x, c.y - a.y, c.z - a.z);
            float3 n = make_float3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x);
            const float inv = rsqrtf(fmaxf(n.x * n.x + n.y * n.y + n.z * n.z, 1e-30f));
            n = make_float3(n.x * inv, n.y * inv, n.z * inv);
            if (n.x * d4.x + n.y * d4.y + n.z * d4.z > 0.0f) n = make_float3(-n.x, -n.y, -n.z);
            N = n;
            // cosine-weighted bounce direction
            const float r1 = rand01(uint32_t(id), p.seed, 0x68bc21ebu);
            const float r2 = rand01(uint32_t(id), p.seed, 0x02e5be93u);
            float sp, cp;
            sincospif(2.0f * r1, &sp, &cp);
            const float rad = sqrtf(r2);
            const float lz = sqrtf(fmaxf(0.0f, 1.0f - r2));
            float3 tg, bt;
            onb(N.x, N.y, N.z, tg, bt);
            D = make_float3(rad * cp * tg.x + rad * sp * bt.x + lz * N.x,
                            rad * cp * tg.y + rad * sp * bt.y + lz * N.y,
                            rad * cp * tg.z + rad * sp * bt.z + lz * N.z);
            S = make_float3(P.x - d4.x * p.epsilon, P.y - d4.y * p.epsilon, P.z - d4.z * p.epsilon);
            sec = true;
            shd = N.x * p.lightx + N.y * p.lighty + N.z * p.lightz > 0.0f;
        }
    }
    // bounce rays sorted by direction octant within the block; shadow rays
    // all share the light's direction
    const uint32_t octant = (D.x < 0.0f ? 1u : 0u) | (D.y < 0.0f ? 2u : 0u) | (D.z < 0.0f ? 4u : 0u);
    const uint32_t si = block_append_sorted<8>(p.counts, sec, octant);
    uint32_t* const counters[1] = { p.counts + 1 };
    const bool want[1] = { shd };
    uint32_t slot[1];
    block_append<1>(counters, want, slot);
    const uint32_t hi = slot[0];
    if (sec) {
        float4* r = p.secondary + size_t(si) * 3;
        r[0] = make_float4(S.x, S.y, S.z, __int_as_float(id));
        r[1] = make_float4(D.x, D.y, D.z, 0.0f);
        r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
    }
    if (shd) {
        float4* r = p.shadow + size_t(hi) * 3;
        r[0] = make_float4(P.x + N.x * p.epsilon, P.y + N.y * p.epsilon, P.z + N.z * p.epsilon, __int_as_float(id));
        r[1] = make_float4(p.lightx, p.lighty, p.lightz, 0.0f);
        r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
    }
}

}  // namespace atlas::rt::dev
