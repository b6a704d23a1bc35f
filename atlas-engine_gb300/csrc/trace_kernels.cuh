// Persistent wavefront BVH traversal kernels for sm_103a.
//
// Semantics: the engine's shader traversal on one BLAS --
//   HitClosest  data/shader/raytracer/bvh.hsh:191-273 (+ CheckLeafClosest :44-72)
//   HitAny      data/shader/raytracer/bvh.hsh:359-441 (+ CheckLeaf :74-104)
//   IntersectAABB / IntersectTriangle  data/shader/raytracer/intersections.hsh:18-57
// reproduced bit for bit: every multiply, add and divide is an explicitly
// rounded IEEE operation in the shader's order (no FMA contraction), GLSL
// min/max are min.f32/max.f32 (a NaN operand loses), the descent goes to the
// nearer child first (hitL <= hitR) and pushes the farther one.
//
// Execution model (not the shader's):
//  * persistent CTAs, a few per SM; each warp pulls rays from a global
//    counter.  A lane that finishes its ray takes a fresh one at the next
//    refill point: the idle lanes are found by a warp ballot and served with
//    one atomic per warp, so live rays stay packed in the warp;
//  * the traversal stack of each lane lives in shared memory, lane-interleaved
//    (entry k of lane l at [k][l], conflict-free), with a local-memory spill
//    area behind it;
//  * nodes (4 x 16 B) and triangles (3 x 16 B) are fetched with 128-bit
//    read-only loads;
//  * every ray carries a step cap and a stack bound; exceeding either sets a
//    flag on the ray and in the context's error word instead of faulting.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "camera.cuh"

namespace atlas::rt::dev {

constexpr uint32_t kErrStackOverflow = 0x1u;
constexpr uint32_t kErrIterationCap = 0x2u;
constexpr uint32_t kErrQueueOverflow = 0x8u;   // a wavefront queue append found the queue full

constexpr uint32_t kHitFlagHit = 0x1u;
constexpr uint32_t kHitFlagNearTie = 0x2u;
constexpr uint32_t kHitFlagOverflow = 0x4u;
constexpr uint32_t kHitFlagIterCap = 0x8u;

// One uploaded mesh (BLAS): the bindless blasNodes[mesh] / bvhTriangles[mesh]
// pair of the engine (data/shader/raytracer/buffers.hsh:45-57).
struct MeshDesc {
    const float4* nodes;
    const float4* tris;
    const float4* shading;       // GPUTriangle (6 float4), may be null
    uint32_t n_nodes;
    uint32_t n_tris;
};

struct TraceParams {
    const float4* nodes;         // 4 float4 per GPUBVHNode
    const float4* tris;          // 3 float4 per GPUBVHTriangle
    uint32_t n_nodes;
    uint32_t n_tris;
    const float4* rays;          // 3 float4 per PackedRay
    uint32_t n_rays;             // ray count, or the queue capacity when n_rays_dev is set
    const uint32_t* n_rays_dev;  // optional: ray count written by an earlier kernel
    float tmin;
    float tmax;
    float4* hits;                // 2 float4 per ae_hit (closest)
    uint8_t* occluded;           // 1 byte per ray (any)
    uint32_t* work_counter;      // rays handed out so far (zeroed before launch)
    uint32_t* error_word;        // kErr* bits
    unsigned long long* fetch_counts;  // [0] nodes, [1] triangles (optional)
    uint32_t max_steps;
    // two-level scenes (TLAS instantiation only)
    const float4* tlas;          // TLAS nodes, 4 float4 each
    uint32_t n_tlas;
    const float4* instances;     // GPUBVHInstance, 4 float4 each
    uint32_t n_instances;
    const MeshDesc* meshes;      // indexed by GPUBVHInstance::meshOffset
    uint32_t n_meshes;
    uint32_t cull_mask;
    // batched multi-mesh launches (MODE_BATCH): n_rays = total over batches
    const struct BatchDesc* batches;
    uint32_t n_batches;
    uint32_t refill_steps;       // traversal steps between warp refills
    uint32_t refill_below;       // refill early when fewer lanes than this still traverse (0: never)
    uint32_t per_ray_tmax;       // nonzero: a ray's tmax is its PackedRay hit.x (shadow queues)
    uint32_t leaf_wait;          // closest hit: a lane at a leaf waits for this many leaf lanes (0: never)
    CameraParams cam;            // the camera variant: ray i is camera_ray(cam, i), `rays` unused
};

// One ray batch of a batched launch: its mesh, its rays and results, its
// query kind, and its first index in the launch's global ray numbering.
struct BatchDesc {
    const float4* nodes;
    const float4* tris;
    const float4* rays;
    void* out;                   // ae_hit[] (closest) or uint8_t[] (any)
    uint32_t n_nodes;
    uint32_t n_tris;
    uint32_t n_rays;
    uint32_t any;
    float tmin;
    float tmax;
    uint32_t first;              // global index of the batch's first ray
    uint32_t max_steps;
};
static_assert(sizeof(BatchDesc) == 64, "batch descriptor layout");

// Default per-ray step cap of a BVH with n_nodes nodes: a valid tree visits
// each node at most once per ray, so 4 n + 64 never cuts a correct traversal
// short.  Computed in 64 bits and saturated, so that arrays of 2^30 nodes and
// more (64 GB of nodes fits in HBM) do not wrap to a small cap.
__host__ __device__ constexpr uint32_t default_step_cap(uint32_t n_nodes) {
    return 4ull * n_nodes + 64ull > 0xffffffffull ? 0xffffffffu : uint32_t(4ull * n_nodes + 64ull);
}

// ae_rt_config::refill_below when left 0 (lanes; 0 = never refill early):
// measured best with a 32-step burst on the terrain + boxes camera pass
// (0.913 against 0.974 ms for 64 steps and no early refill).
constexpr uint32_t kDefaultRefillBelow = 8;

constexpr int MODE_MESH = 0;     // one BLAS
constexpr int MODE_SCENE = 1;    // TLAS over instances
constexpr int MODE_BATCH = 2;    // many BLASes, one per batch

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// A 64-byte node as two 32-byte read-only loads, one L1 sector each: every lane
// gathers its own node, so four 16-byte loads would look each sector up twice
// (the L1 pipeline is the limiter of incoherent rays).  Needs the node at a
// 32-byte boundary: node arrays are cudaMalloc'ed by the library (256-byte
// aligned) and 64-byte strided.  Caller-owned arrays (the bounds-checked
// instance) use ldg4.
__device__ __forceinline__ void ldg_node(const float4* p, float4& n0, float4& n1, float4& n2, float4& n3) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(n0.x), "=f"(n0.y), "=f"(n0.z), "=f"(n0.w), "=f"(n1.x), "=f"(n1.y), "=f"(n1.z), "=f"(n1.w)
        : "l"(p));
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8+32];"
        : "=f"(n2.x), "=f"(n2.y), "=f"(n2.z), "=f"(n2.w), "=f"(n3.x), "=f"(n3.y), "=f"(n3.z), "=f"(n3.w)
        : "l"(p));
}

// IEEE single operations with explicit rounding (no contraction into FMA).
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Correctly rounded a / b from y = RN(1/b) without a divide instruction:
// q0 = RN(a*y) is within 1.5 ulp of a/b; one residual correction
// q1 = RN(q0 + RN(a - b*q0)*y) makes it faithful; with a faithful quotient the
// residual a - b*q1 is exact (computed by FMA) and Markstein's theorem
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990) gives RN(q1 + r1*y) = RN(a/b).
// Valid while no intermediate under- or overflows, which the callers ensure
// by range (see kFastLo / kFastHi); everything else takes div.rn.
__device__ __forceinline__ float div_rn_from_rcp(float a, float b, float y) {
    float q = __fmul_rn(a, y);
    float r = __fmaf_rn(-q, b, a);
    q = __fmaf_rn(r, y, q);
    r = __fmaf_rn(-q, b, a);
    return __fmaf_rn(r, y, q);
}

// Exponent window of the fast quotient: every |origin|, |box coordinate| is 0
// or in [2^-40, 2^40] and every |direction| in [2^-40, 2^40], so |a| = |c - o|
// is 0 or in [2^-63, 2^41] and all intermediates stay normal.
constexpr float kFastLo = 9.094947017729282e-13f;   // 2^-40
constexpr float kFastHi = 1.099511627776e12f;       // 2^40

__device__ __forceinline__ bool in_fast_range(float v, bool zero_ok) {
    const float m = fabsf(v);
    return (zero_ok && m == 0.0f) || (m >= kFastLo && m <= kFastHi);
}

// Near ties.  The nearest triangle of a closest-hit ray is decided by FP32
// rounding when a second triangle lies within 1e-6 relative t of it; such
// rays carry kHitFlagNearTie and are re-tested in double.  The flag must
// cover every ray whose two nearest double-precision hits are that close,
// including hits the FP32 traversal never sees, so it is set (a superset)
// when any of these holds:
//  * a second accepted triangle lies within kTieWindow relative t of the
//    nearest (1e-6 plus the FP32 error of the two distances);
//  * a child box rejected by the shader's test had its entry within
//    kTieWindow of the bound it was tested against (its triangles could tie
//    with the final hit, which is at most that bound);
//  * a triangle rejected by the FP32 test lies within the rounding error of
//    its barycentric tests (tri_test's nearMiss) at a distance up to
//    kTieWindow past the current nearest hit -- a shared edge, where either
//    side's FP32 test may fail;
//  * the shader's descent dropped a hit right child whose entry equals the
//    bound (bvh.hsh:234-236: a missed left child reports the bound too, and
//    hitL <= hitR then picks it).
// None of this changes which triangle the traversal returns.
constexpr float kTieWindow = 4e-6f;
constexpr float kTieWiden = 1.0f + kTieWindow;
constexpr float kNearMissScale = 9.5367431640625e-07f;   // 2^-20

// IntersectAABB(ray, aabb, tmin, tmax, out dist) -- intersections.hsh:18-34.
// FAST: quotients through div_rn_from_rcp with (yx, yy, yz) = RN(1/d); the
// result is bit-identical to the div.rn form.  nearCull: the box was
// rejected but its entry lies within kTieWindow of the exit bound.
template <bool FAST>
__device__ __forceinline__ bool box_test(float ox, float oy, float oz, float dx, float dy, float dz,
                                         float yx, float yy, float yz,
                                         float lx, float ly, float lz, float hx, float hy, float hz,
                                         float tmin, float tmax, float& dist, bool& nearCull) {
    float t0x, t0y, t0z, t1x, t1y, t1z;
    if (FAST) {
        t0x = div_rn_from_rcp(fsub(lx, ox), dx, yx);
        t0y = div_rn_from_rcp(fsub(ly, oy), dy, yy);
        t0z = div_rn_from_rcp(fsub(lz, oz), dz, yz);
        t1x = div_rn_from_rcp(fsub(hx, ox), dx, yx);
        t1y = div_rn_from_rcp(fsub(hy, oy), dy, yy);
        t1z = div_rn_from_rcp(fsub(hz, oz), dz, yz);
    } else {
        t0x = fdiv(fsub(lx, ox), dx); t0y = fdiv(fsub(ly, oy), dy); t0z = fdiv(fsub(lz, oz), dz);
        t1x = fdiv(fsub(hx, ox), dx); t1y = fdiv(fsub(hy, oy), dy); t1z = fdiv(fsub(hz, oz), dz);
    }
    const float sx = fminf(t0x, t1x), sy = fminf(t0y, t1y), sz = fminf(t0z, t1z);
    const float bx = fmaxf(t0x, t1x), by = fmaxf(t0y, t1y), bz = fmaxf(t0z, t1z);
    const float tminf = fmaxf(fmaxf(tmin, sx), fmaxf(sy, sz));
    const float tmaxf = fminf(fminf(tmax, bx), fminf(by, bz));
    const bool hit = tminf <= tmaxf;
    dist = hit ? tminf : tmax;
    nearCull = !hit && tminf <= fmul(tmaxf, kTieWiden);
    return hit;
}

// IntersectTriangle -- intersections.hsh:36-57.  Returns the shader's accept
// test; (t, u, v) = sol.  NEAR: *nearMiss tells whether (u, v) lie within the
// rounding error of the barycentric bounds.  With the L1 norms Sd, S0, S1, Ss
// of d, e0, e1 and s = o - v0, every operation of the formula contributes at
// most a few ulps of products bounded by Sd (S0+S1) (Ss+S0+S1), so
// |error(u)|, |error(v)| < beta = m / |den| with
// m = 2^-20 Sd (S0+S1) (Ss+S0+S1) (2^-20 = 16 ulps of 1).  The tests are
// taken multiplied by |den| (u |den| + m >= 0, ...), one correctly rounded
// FMA each, so the oracle reproduces them.  slack (optional) receives |den| and m.
template <bool NEAR = false>
__device__ __forceinline__ bool tri_test(float ox, float oy, float oz, float dx, float dy, float dz,
                                         const float4& a, const float4& b, const float4& c,
                                         float& t, float& u, float& v, bool* nearMiss = nullptr,
                                         float* slack = nullptr) {
    const float e0x = fsub(b.x, a.x), e0y = fsub(b.y, a.y), e0z = fsub(b.z, a.z);
    const float e1x = fsub(c.x, a.x), e1y = fsub(c.y, a.y), e1z = fsub(c.z, a.z);
    const float sx = fsub(ox, a.x), sy = fsub(oy, a.y), sz = fsub(oz, a.z);
    // the slack's scale, folded at once so that one value stays live
    float m = 0.0f;
    if (NEAR) {
        const float s01 = fadd(fadd(fadd(fabsf(e0x), fabsf(e0y)), fabsf(e0z)),
                               fadd(fadd(fabsf(e1x), fabsf(e1y)), fabsf(e1z)));
        const float ss = fadd(fadd(fabsf(sx), fabsf(sy)), fabsf(sz));
        const float sd = fadd(fadd(fabsf(dx), fabsf(dy)), fabsf(dz));
        m = fmul(fmul(fmul(sd, s01), fadd(ss, s01)), kNearMissScale);
    }
    // p = cross(s, e0), q = cross(d, e1)
    const float px = fsub(fmul(sy, e0z), fmul(e0y, sz));
    const float py = fsub(fmul(sz, e0x), fmul(e0z, sx));
    const float pz = fsub(fmul(sx, e0y), fmul(e0x, sy));
    const float qx = fsub(fmul(dy, e1z), fmul(e1y, dz));
    const float qy = fsub(fmul(dz, e1x), fmul(e1z, dx));
    const float qz = fsub(fmul(dx, e1y), fmul(e1x, dy));
    const float den = fadd(fadd(fmul(qx, e0x), fmul(qy, e0y)), fmul(qz, e0z));
    t = fdiv(fadd(fadd(fmul(px, e1x), fmul(py, e1y)), fmul(pz, e1z)), den);
    u = fdiv(fadd(fadd(fmul(qx, sx), fmul(qy, sy)), fmul(qz, sz)), den);
    v = fdiv(fadd(fadd(fmul(px, dx), fmul(py, dy)), fmul(pz, dz)), den);
    if (NEAR) {
        const float ad = fabsf(den);
        *nearMiss = __fmaf_rn(u, ad, m) >= 0.0f && __fmaf_rn(v, ad, m) >= 0.0f &&
                    __fmaf_rn(fsub(1.0f, fadd(u, v)), ad, fadd(m, m)) >= 0.0f;
        if (slack) { slack[0] = ad; slack[1] = m; }
    }
    return t >= 0.0f && u >= 0.0f && v >= 0.0f && fadd(u, v) <= 1.0f;
}

// IntersectTriangle with one reciprocal of the denominator instead of three
// divisions, for traversals whose results are statistical (the radiance
// cache, AE_RT_CFG_APPROXIMATE): the numerators and the denominator are the
// shader's, operation by operation (no contraction: the dot products of
// nearly edge-on triangles cancel), and each of t, u, v is RN(RN(n) *
// RN(1/den)), within 1.5 units of 2^-24 (relative) of the shader's RN(n / den);
// the same accept test.
__device__ __forceinline__ bool tri_test_fast(float ox, float oy, float oz, float dx, float dy, float dz,
                                              const float4& a, const float4& b, const float4& c,
                                              float& t, float& u, float& v) {
    const float e0x = fsub(b.x, a.x), e0y = fsub(b.y, a.y), e0z = fsub(b.z, a.z);
    const float e1x = fsub(c.x, a.x), e1y = fsub(c.y, a.y), e1z = fsub(c.z, a.z);
    const float sx = fsub(ox, a.x), sy = fsub(oy, a.y), sz = fsub(oz, a.z);
    const float px = fsub(fmul(sy, e0z), fmul(e0y, sz));
    const float py = fsub(fmul(sz, e0x), fmul(e0z, sx));
    const float pz = fsub(fmul(sx, e0y), fmul(e0x, sy));
    const float qx = fsub(fmul(dy, e1z), fmul(e1y, dz));
    const float qy = fsub(fmul(dz, e1x), fmul(e1z, dx));
    const float qz = fsub(fmul(dx, e1y), fmul(e1x, dy));
    const float inv = __frcp_rn(fadd(fadd(fmul(qx, e0x), fmul(qy, e0y)), fmul(qz, e0z)));
    t = fmul(fadd(fadd(fmul(px, e1x), fmul(py, e1y)), fmul(pz, e1z)), inv);
    u = fmul(fadd(fadd(fmul(qx, sx), fmul(qy, sy)), fmul(qz, sz)), inv);
    v = fmul(fadd(fadd(fmul(px, dx), fmul(py, dy)), fmul(pz, dz)), inv);
    return t >= 0.0f && u >= 0.0f && v >= 0.0f && fadd(u, v) <= 1.0f;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- staged ray queue: 1-D bulk copies (TMA) of ray tiles into shared memory ----
constexpr uint32_t kErrWaitTimeout = 0x4u;     // a bounded device wait gave up
constexpr int kStageRays = 16;                 // rays per staged tile (768 bytes)

__device__ __forceinline__ uint32_t shared_addr(const void* ptr) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void stage_barrier_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
}

// One bulk copy of `bytes` (a multiple of 16, both addresses 16-byte
// aligned) from global into this CTA's shared memory; the barrier's phase
// completes when the bytes have landed.  The proxy fence orders the warp's
// earlier reads of the buffer before the copy's writes.
__device__ __forceinline__ void stage_bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t stage_clock_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the completion of the barrier phase of parity `parity`; false
// after ~200 ms of the global timer, or after 2^25 polls whatever it says.
__device__ __forceinline__ bool stage_wait(uint32_t bar, uint32_t parity) {
    const uint64_t start = stage_clock_ns();
    for (uint32_t it = 0; it < (1u << 25); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}"
            : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 63u) == 63u && stage_clock_ns() - start > 200000000ull) return false;
    }
    return false;
}

// Per-lane traversal stack: SMEM entries in shared memory (lane-interleaved),
// then SPILL entries in local memory.
template <int SMEM, int SPILL>
struct LaneStack {
    int32_t* sh;           // &shared[warp][0][lane]; entry k at sh[k * 32]
    int32_t spill[SPILL];
    __device__ __forceinline__ void put(uint32_t k, int32_t v) {
        if (k < SMEM) sh[k * 32] = v;
        else spill[k - SMEM] = v;
    }
    __device__ __forceinline__ int32_t get(uint32_t k) const {
        return k < SMEM ? sh[k * 32] : spill[k - SMEM];
    }
    static constexpr uint32_t capacity = SMEM + SPILL;
};

// One traversal ray in the space of the structure being traversed, with
// the reciprocals of its direction and the fast-division window flag.
struct TRay {
    float ox, oy, oz, dx, dy, dz, yx, yy, yz;
    bool fast;
    __device__ __forceinline__ void prepare() {
        yx = __frcp_rn(dx); yy = __frcp_rn(dy); yz = __frcp_rn(dz);
        fast = in_fast_range(ox, true) && in_fast_range(oy, true) && in_fast_range(oz, true) &&
               in_fast_range(dx, false) && in_fast_range(dy, false) && in_fast_range(dz, false);
    }
};

// Approximate IntersectAABB for the screening below: the six quotients as
// RN(RN(c - o) * RN(1/d)) instead of the shader's RN((c - o) / d).  Each
// lies within 3 units of 2^-24 (relative) of the shader's quotient and has
// its sign (zero exactly when c == o), and min / max carry that bound over
// to the entry lo and exit hi.
__device__ __forceinline__ void box_approx(const TRay& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                           float tmin, float tmax, float& lo, float& hi) {
    const float t0x = fmul(fsub(lx, r.ox), r.yx), t0y = fmul(fsub(ly, r.oy), r.yy), t0z = fmul(fsub(lz, r.oz), r.yz);
    const float t1x = fmul(fsub(hx, r.ox), r.yx), t1y = fmul(fsub(hy, r.oy), r.yy), t1z = fmul(fsub(hz, r.oz), r.yz);
    lo = fmaxf(fmaxf(tmin, fminf(t0x, t1x)), fmaxf(fminf(t0y, t1y), fminf(t0z, t1z)));
    hi = fminf(fminf(tmax, fmaxf(t0x, t1x)), fminf(fmaxf(t0y, t1y), fmaxf(t0z, t1z)));
}

// x <= y decided from approximations x', y' >= 0 that are each within 8 units
// of 2^-24 (relative) of x and y: x' <= y' * kSure proves x <= y, and
// x' * kSure > y' proves x > y (kSure = 1 - 2^-20 leaves room for the rounding
// of the product); anything between is a close call.
constexpr float kSure = 0.99999904632568359375f;

// Both child boxes of a node (IntersectAABB x 2, bvh.hsh:229-232 / :253-256)
// as the traversal uses them: il / ir whether each box is hit;
// leftFirst = (distL <= distR) for the descent order (only read when
// `ordered`), with a missed box reporting the bound as the shader's does;
// nearCull (only when `ties`): a box was rejected with its entry within
// kTieWindow of the bound (see kTieWindow).
// Inside the fast-division window (node.padding0 == 0 marks a node whose
// coordinates are in it, set by the upload; the ray's own flag; tmin >= 0)
// the quotients are correctly rounded from the reciprocal (div_rn_from_rcp);
// outside it and for the BOUNDS variant (whose nodes did not go through the
// upload) they divide with div.rn.  A traversal that needs only il / ir (any
// hit: neither ordered nor ties) first screens the boxes with box_approx:
// every hit decision that the approximations settle with a margin of 16
// units of 2^-24 is the shader's, and only a lane with a close call (a
// grazing ray) computes the quotients exactly.  Closest-hit traversals
// compare entry distances, which are often exactly equal (sibling boxes
// with a common face), so they take the exact quotients at once.
template <bool BOUNDS>
__device__ __forceinline__ void test_children(const TRay& r, const float4& n0, const float4& n1, const float4& n2,
                                              const float4& n3, float tmin, float bound, bool ordered, bool ties,
                                              bool& il, bool& ir, bool& leftFirst, bool& nearCull) {
    const bool fast = !BOUNDS && r.fast && __float_as_int(n3.z) == 0;
    if (fast && !ordered && !ties && tmin >= 0.0f) {
        float lol, hil, lor, hir;
        box_approx(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, bound, lol, hil);
        box_approx(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, bound, lor, hir);
        // lo >= tmin >= 0, so a negative exit is a sure miss
        il = hil >= 0.0f && lol <= fmul(hil, kSure);
        ir = hir >= 0.0f && lor <= fmul(hir, kSure);
        const bool close = (!il && hil >= 0.0f && !(fmul(lol, kSure) > hil)) ||
                           (!ir && hir >= 0.0f && !(fmul(lor, kSure) > hir));
        leftFirst = true;
        nearCull = false;
        if (!close) return;
    }
    bool nl, nr;
    float hl, hr;
    if (fast) {
        il = box_test<true>(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.yx, r.yy, r.yz, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y,
                            tmin, bound, hl, nl);
        ir = box_test<true>(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.yx, r.yy, r.yz, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w,
                            tmin, bound, hr, nr);
    } else {
        il = box_test<false>(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.yx, r.yy, r.yz, n0.x, n0.y, n0.z, n0.w, n1.x,
                             n1.y, tmin, bound, hl, nl);
        ir = box_test<false>(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.yx, r.yy, r.yz, n1.z, n1.w, n2.x, n2.y, n2.z,
                             n2.w, tmin, bound, hr, nr);
    }
    leftFirst = hl <= hr;
    nearCull = nl || nr;
}

// Both child boxes for traversals whose results are statistical rather than
// the shader's bit for bit (the radiance cache's training paths): the
// approximate quotients of box_approx with no exact re-test.  A box counts
// as hit when its entry is at most its exit times 1 + 2^-20, so the test
// never rejects a box that the exact test accepts (it may accept a grazed
// one); the order follows the approximate entries.  Outside the
// fast-division window it is test_children.
constexpr float kLoose = 1.00000095367431640625f;   // 1 + 2^-20

__device__ __forceinline__ void test_children_loose(const TRay& r, const float4& n0, const float4& n1,
                                                    const float4& n2, const float4& n3, float tmin, float bound,
                                                    bool& il, bool& ir, bool& leftFirst) {
    if (r.fast && __float_as_int(n3.z) == 0 && tmin >= 0.0f) {
        float lol, hil, lor, hir;
        box_approx(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, bound, lol, hil);
        box_approx(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, bound, lor, hir);
        il = lol <= fmul(hil, kLoose);
        ir = lor <= fmul(hir, kLoose);
        leftFirst = (il ? lol : bound) <= (ir ? lor : bound);
        return;
    }
    bool unused;
    test_children<false>(r, n0, n1, n2, n3, tmin, bound, true, false, il, ir, leftFirst, unused);
}

// vec4(v, w) * inverseMatrix (bvh.hsh:179-180): component i = dot(vec4(v, w),
// column i), summed left to right with separate roundings.
__device__ __forceinline__ float xform_row(float x, float y, float z, float w, const float4& c) {
    return fadd(fadd(fadd(fmul(x, c.x), fmul(y, c.y)), fmul(z, c.z)), fmul(w, c.w));
}

constexpr uint32_t kTlasInvalid = 0xffffffffu;

// Batch holding global ray index g: the last descriptor whose first <= g.
__device__ __forceinline__ uint32_t find_batch(const BatchDesc* b, uint32_t n, uint32_t g) {
    uint32_t lo = 0, hi = n;            // invariant: b[lo].first <= g < b[hi].first
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&b[mid].first) <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ANY: HitAny instead of HitClosest.  COUNT: per-launch node / triangle fetch
// totals.  MODE_SCENE: two-level traversal over instances (CheckInstance,
// bvh.hsh:172-189, with the TLAS/BLAS switch keyed on the stack depth at which
// the instance was entered, bvh.hsh:212-223).  MODE_BATCH: every lane finds
// its ray's batch (mesh, query kind, t range, result buffer) when it takes a
// ray, so one launch serves many meshes and both query kinds.
// BOUNDS = true adds range checks of every node and triangle index against
// n_nodes / n_tris (for callers whose BVH did not pass the host validator);
// an out-of-range index ends the ray with the overflow flag set.
// TIES: closest-hit rays get the complete near-tie flag (kTieWindow); the
// library's own consumers that discard the flag (path tracer, passes,
// radiance cache) launch TIES = false.
//
// STAGE > 0: each warp claims its rays in tiles of STAGE consecutive rays and
// copies every tile into shared memory with one bulk copy (TMA, 1-D) on an
// mbarrier, the next tile in flight while the current one is handed out
// (double-buffered); refills then read rays from shared memory.  Single-mesh
// and scene launches only.  A copy that does not complete within the bounded
// wait sets kErrWaitTimeout and ends the warp's refills.
//
// LOOSE: the conservative approximate box test (test_children_loose) and
// tri_test_fast, for consumers whose results are Monte Carlo estimates
// (AE_RT_CFG_APPROXIMATE), not the shader's bit for bit.
//
// CAMERA: ray i is the camera ray of queue slot i (camera_ray), made by the
// lane that takes it, instead of a load from a ray buffer written by a
// separate ray-generation launch.
template <bool ANY, bool COUNT, int MODE, int WARPS, int SMEM_STACK, int SPILL_STACK, int MIN_BLOCKS,
          bool BOUNDS = false, bool TIES = true, int STAGE = 0, bool LOOSE = false, bool CAMERA = false>
__global__ void __launch_bounds__(WARPS * 32, MIN_BLOCKS) trace_kernel(TraceParams p) {
    constexpr bool TLAS = MODE == MODE_SCENE;
    constexpr bool BATCH = MODE == MODE_BATCH;
    static_assert(STAGE == 0 || (!BATCH && !BOUNDS), "staged rays: single-mesh and scene launches only");
    static_assert(!LOOSE || (!TIES && !BOUNDS), "loose traversal: no near-tie flag, uploaded nodes");
    static_assert(!CAMERA || (MODE == MODE_MESH && STAGE == 0 && !ANY), "camera rays: single-mesh closest hits");
    __shared__ int32_t s_stack[WARPS][SMEM_STACK][32];
    __shared__ __align__(128) float4 s_rays[STAGE > 0 ? WARPS : 1][2][STAGE > 0 ? STAGE * 3 : 1];
    __shared__ __align__(8) uint64_t s_rbar[STAGE > 0 ? WARPS : 1][2];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    constexpr unsigned kFull = 0xffffffffu;

    LaneStack<SMEM_STACK, SPILL_STACK> st;
    st.sh = &s_stack[warp][0][lane];

    bool live = false;
    bool queueDry = false;          // warp-uniform
    uint32_t rid = 0;
    TRay wr{};                      // world-space ray (TLAS level)
    TRay r{};                       // ray in the space of the current BLAS
    float hitDist = 0, second = 0, hu = 0, hv = 0;
    int32_t hitID = -1, hitInst = -1, curInst = -1;
    int32_t node = 0;
    uint32_t sp = 0, steps = 0, flags = 0, tlasIndex = kTlasInvalid;
    const float4* blasNodes = p.nodes;
    const float4* blasTris = p.tris;
    bool occl = false;
    bool tieSuspect = false;        // closest hit: a near tie the second distance cannot show (kTieWindow)
    bool laneAny = ANY;             // batched: the lane's query kind
    float tmin = p.tmin, tmax = p.tmax;
    uint32_t maxSteps = p.max_steps;
    void* out = nullptr;            // batched: the lane's result array
    unsigned long long nodeCount = 0, triCount = 0;
    const uint32_t nRays = p.n_rays_dev ? min(*p.n_rays_dev, p.n_rays) : p.n_rays;
    const uint32_t nTop = TLAS ? p.n_tlas : p.n_nodes;
    const int refill = p.refill_steps ? int(p.refill_steps) : 32;
    const uint32_t refillBelow = p.refill_below;
    const uint32_t leafWait = ANY ? 0u : p.leaf_wait;

    // a ray's traversal state from its origin and direction (tmax already set)
    auto beginRay = [&](const float4& o4, const float4& d4, uint32_t nodesHere) {
        r.ox = o4.x; r.oy = o4.y; r.oz = o4.z;
        r.dx = d4.x; r.dy = d4.y; r.dz = d4.z;
        r.prepare();
        if (TLAS) wr = r;
        hitDist = tmax; second = tmax; hu = 0.0f; hv = 0.0f;
        hitID = -1; hitInst = -1; curInst = -1;
        node = 0; sp = 0; steps = 0; flags = 0; occl = false; tieSuspect = false;
        tlasIndex = kTlasInvalid;
        if (MODE == MODE_MESH) { blasNodes = p.nodes; blasTris = p.tris; }
        live = true;
        // NaN direction or an empty BVH: miss (bvh.hsh:204, BVH.cpp:107)
        if (isnan(r.dx) || isnan(r.dy) || isnan(r.dz) || nodesHere == 0) node = INT32_MIN;
    };

    // staged queue of the warp, kept in shared memory between refills (no
    // registers during traversal): word 0 the current tile's first ray,
    // word 1 the next tile's (in flight while kStPending), word 2 the rays of
    // the current tile handed out (bits 0-7) and the flags below; the current
    // tile sits in buffer kStCur's value, the next in the other one
    constexpr uint32_t kStUsed = 0xffu, kStCur = 1u << 8, kStPhase0 = 1u << 9, kStPending = 1u << 11,
                       kStDry = 1u << 12, kStFault = 1u << 13, kStEmpty = 1u << 14;
    __shared__ uint32_t s_rstate[STAGE > 0 ? WARPS : 1][3];
    if constexpr (STAGE > 0) {
        if (lane == 0) {
            stage_barrier_init(shared_addr(&s_rbar[warp][0]));
            stage_barrier_init(shared_addr(&s_rbar[warp][1]));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            s_rstate[warp][0] = 0;
            s_rstate[warp][1] = 0;
            s_rstate[warp][2] = kStEmpty;     // no current tile yet
        }
        __syncwarp();
    }

    for (;;) {
        // ---- refill idle lanes (one atomic per warp) ----
        if (!queueDry) {
            const uint32_t idle = __ballot_sync(kFull, !live);
            if (STAGE > 0 && idle) {
                uint32_t base = s_rstate[warp][0], nxt = s_rstate[warp][1], bits = s_rstate[warp][2];
                // the rays of a tile starting at b
                auto tileRays = [&](uint32_t b) { return min(uint32_t(STAGE), nRays - b); };
                // claims the next tile and starts its copy into the free buffer
                auto issue = [&]() {
                    __syncwarp();
                    uint32_t b = 0;
                    if (lane == 0) b = atomicAdd(p.work_counter, uint32_t(STAGE));
                    b = __shfl_sync(kFull, b, 0);
                    if (b >= nRays) { bits |= kStDry; return; }
                    if (b + uint32_t(STAGE) >= nRays) bits |= kStDry;
                    const uint32_t nb = (bits & kStCur) ? 0u : 1u;
                    if (lane == 0)
                        stage_bulk_load(shared_addr(&s_rays[warp][nb][0]), p.rays + size_t(b) * 3,
                                        tileRays(b) * 48u, shared_addr(&s_rbar[warp][nb]));
                    nxt = b;
                    bits |= kStPending;
                };
                uint32_t need = idle;
                while (need && !(bits & kStFault)) {
                    if ((bits & kStEmpty) || (bits & kStUsed) == tileRays(base)) {
                        if (!(bits & kStPending)) {
                            if (bits & kStDry) break;
                            issue();
                            if (!(bits & kStPending)) break;
                        }
                        const uint32_t nb = (bits & kStCur) ? 0u : 1u;
                        const uint32_t parity = (bits >> (9 + nb)) & 1u;
                        if (!__all_sync(kFull, stage_wait(shared_addr(&s_rbar[warp][nb]), parity))) {
                            if (lane == 0) atomicOr(p.error_word, kErrWaitTimeout);
                            bits |= kStFault;      // the copy stays pending: waited for again at exit
                            break;
                        }
                        bits ^= kStPhase0 << nb;
                        bits = (bits & ~(kStUsed | kStPending | kStEmpty | kStCur)) | (nb ? kStCur : 0u);
                        base = nxt;
                        if (!(bits & kStDry)) issue();
                    }
                    const uint32_t used = bits & kStUsed;
                    const uint32_t rank = __popc(need & lanemask_lt());
                    const uint32_t k = min(uint32_t(__popc(need)), tileRays(base) - used);
                    const bool mine = ((need >> lane) & 1u) && rank < k;
                    if (mine) {
                        const float4* src = &s_rays[warp][(bits & kStCur) ? 1 : 0][(used + rank) * 3];
                        rid = base + used + rank;
                        if (p.per_ray_tmax) tmax = src[2].x;
                        beginRay(src[0], src[1], nTop);
                    }
                    need &= ~__ballot_sync(kFull, mine);
                    bits += k;
                }
                if ((bits & kStFault) ||
                    ((bits & kStDry) && !(bits & kStPending) &&
                     ((bits & kStEmpty) || (bits & kStUsed) == tileRays(base))))
                    queueDry = true;
                __syncwarp();
                if (lane == 0) {
                    s_rstate[warp][0] = base;
                    s_rstate[warp][1] = nxt;
                    s_rstate[warp][2] = bits;
                }
                __syncwarp();
            } else if (idle) {
                const uint32_t leader = __ffs(idle) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(p.work_counter, __popc(idle));
                base = __shfl_sync(kFull, base, leader);
                if (base + __popc(idle) >= nRays) queueDry = true;
                if (!live) {
                    const uint32_t gi = base + __popc(idle & lanemask_lt());
                    if (gi < nRays) {
                        const float4* raySrc = p.rays;
                        uint32_t ri = gi;
                        uint32_t nodesHere = nTop;
                        if (BATCH) {
                            const BatchDesc& bd = p.batches[find_batch(p.batches, p.n_batches, gi)];
                            ri = gi - bd.first;
                            raySrc = bd.rays;
                            blasNodes = bd.nodes;
                            blasTris = bd.tris;
                            nodesHere = bd.n_nodes;
                            laneAny = bd.any != 0;
                            tmin = bd.tmin;
                            tmax = bd.tmax;
                            maxSteps = bd.max_steps;
                            out = bd.out;
                        }
                        rid = ri;
                        float4 o4, d4;
                        if (CAMERA) {
                            // the ray made where it is traced (no ray buffer)
                            camera_ray(p.cam, ri, o4, d4);
                        } else {
                            o4 = ldg4(raySrc + size_t(ri) * 3);
                            d4 = ldg4(raySrc + size_t(ri) * 3 + 1);
                            if (p.per_ray_tmax) tmax = ldg4(raySrc + size_t(ri) * 3 + 2).x;
                        }
                        beginRay(o4, d4, nodesHere);
                    }
                }
            }
        }
        if (!__any_sync(kFull, live)) break;

        // ---- traverse: a bounded number of steps, then refill again ----
        if (live) {
            const bool anyQ = ANY || (BATCH && laneAny);
            bool done = node == INT32_MIN;
            for (int k = 0; k < refill && !done; k++) {
                // dynamic fetch: leave the burst for a refill once too few lanes
                // are still traversing (while the queue still has rays)
                if (refillBelow && !queueDry && uint32_t(__popc(__activemask())) < refillBelow) break;
                // postponed leaves: a lane at a leaf skips this step while fewer
                // than leafWait lanes are at leaves and others still descend, so
                // that the warp's triangle tests run together instead of beside
                // every node step (the order of each lane's own steps is kept)
                if (leafWait) {
                    const bool atLeaf = node < 0 && !(TLAS && sp < tlasIndex);
                    const uint32_t act = __activemask();
                    const uint32_t leaves = __ballot_sync(act, atLeaf);
                    if (atLeaf && uint32_t(__popc(leaves)) < leafWait && leaves != act) continue;
                }
                if (++steps > maxSteps) {
                    flags |= kHitFlagIterCap;
                    atomicOr(p.error_word, kErrIterationCap);
                    done = true;
                    break;
                }
                const bool top = TLAS && sp < tlasIndex;
                if (top) {
                    tlasIndex = kTlasInvalid;
                    if (node < 0) {
                        // CheckInstance: object-space ray, mesh, cull mask
                        const uint32_t ii = uint32_t(~node);
                        const float4* ip = p.instances + size_t(ii) * 4;
                        const float4 c0 = ldg4(ip), c1 = ldg4(ip + 1), c2 = ldg4(ip + 2), c3 = ldg4(ip + 3);
                        curInst = int32_t(ii);
                        bool enter = (__float_as_uint(c3.w) & p.cull_mask) != 0u;
                        MeshDesc m{};
                        if (enter) {
                            m = p.meshes[__float_as_int(c3.x)];
                            enter = m.n_nodes > 0;     // an empty BLAS has no root to visit
                        }
                        if (enter) {
                            r.ox = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c0);
                            r.oy = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c1);
                            r.oz = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c2);
                            r.dx = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c0);
                            r.dy = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c1);
                            r.dz = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c2);
                            r.prepare();
                            blasNodes = m.nodes;
                            blasTris = m.tris;
                            node = 0;
                            tlasIndex = sp;
                        } else {
                            if (sp == 0) { done = true; break; }
                            node = st.get(--sp);
                        }
                        continue;
                    }
                }
                const float4* nodesArr = top ? p.tlas : blasNodes;
                const TRay& cr = top ? wr : r;
                if (BOUNDS && (node < 0 ? uint32_t(~node) >= p.n_tris : uint32_t(node) >= p.n_nodes)) {
                    flags |= kHitFlagOverflow;
                    atomicOr(p.error_word, kErrStackOverflow);
                    done = true;
                    break;
                }
                if (node < 0) {
                    // Leaf: contiguous triangles up to the end-of-node flag.
                    int32_t tp = ~node;
                    bool end = false;
                    do {
                        if (BOUNDS && uint32_t(tp) >= p.n_tris) {
                            flags |= kHitFlagOverflow;
                            atomicOr(p.error_word, kErrStackOverflow);
                            break;
                        }
                        const float4 a = ldg4(blasTris + size_t(tp) * 3);
                        const float4 b = ldg4(blasTris + size_t(tp) * 3 + 1);
                        const float4 c = ldg4(blasTris + size_t(tp) * 3 + 2);
                        end = a.w > 0.0f;
                        if (COUNT) triCount++;
                        float t, u, v;
                        bool nearMiss = false;
                        const bool hit = LOOSE ? tri_test_fast(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, a, b, c, t, u, v)
                                               : tri_test<TIES && !ANY>(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, a, b, c, t,
                                                                        u, v, &nearMiss);
                        if (anyQ) {
                            if (hit && t > tmin && t < tmax) { occl = true; end = true; }
                        } else if (hit && t > tmin && t < tmax) {
                            if (t < hitDist) {
                                second = hitDist;
                                hitDist = t; hitID = tp; hu = u; hv = v; hitInst = curInst;
                            } else if (t < second) {
                                second = t;
                            }
                        } else if (TIES && nearMiss && t > tmin && t < tmax && t <= fmul(hitDist, kTieWiden)) {
                            tieSuspect = true;
                        }
                        tp++;
                    } while (!end);
                    if (BOUNDS && (flags & kHitFlagOverflow)) { done = true; break; }
                    if (anyQ && occl) { done = true; break; }
                    if (sp == 0) { done = true; break; }
                    node = st.get(--sp);
                } else {
                    const float4* np = nodesArr + size_t(node) * 4;
                    float4 n0, n1, n2, n3;
                    if (BOUNDS) {
                        n0 = ldg4(np); n1 = ldg4(np + 1); n2 = ldg4(np + 2); n3 = ldg4(np + 3);
                    } else {
                        ldg_node(np, n0, n1, n2, n3);
                    }
                    if (COUNT) nodeCount++;
                    const int32_t lptr = __float_as_int(n3.x), rptr = __float_as_int(n3.y);
                    bool il, ir, leftFirst, nearCull = false;
                    if (LOOSE)
                        test_children_loose(cr, n0, n1, n2, n3, tmin, anyQ ? tmax : hitDist, il, ir, leftFirst);
                    else
                        // the batched launch decides the query kind per lane at run time; with
                        // both box tests compiled into it, it ran 8 % slower (11.85 against
                        // 10.99 ms on 64 meshes), so every lane takes the exact test there
                        test_children<BOUNDS>(cr, n0, n1, n2, n3, tmin, anyQ ? tmax : hitDist, BATCH || !anyQ,
                                              TIES && !anyQ, il, ir, leftFirst, nearCull);
                    if (TIES && !anyQ) tieSuspect = tieSuspect || nearCull;
                    int32_t next, far;
                    if (anyQ) {
                        next = il ? lptr : rptr;
                        far = rptr;
                    } else {
                        next = leftFirst ? lptr : rptr;
                        far = leftFirst ? rptr : lptr;
                        // bvh.hsh:234-236: with only the right box hit and its
                        // entry equal to the bound, the missed left box also
                        // reports the bound, so the shader descends left and
                        // drops the right subtree, whose triangles may tie
                        if (TIES) tieSuspect = tieSuspect || (!il && ir && leftFirst);
                    }
                    if (il && ir) {
                        if (sp >= st.capacity) {
                            flags |= kHitFlagOverflow;
                            atomicOr(p.error_word, kErrStackOverflow);
                            done = true;
                            break;
                        }
                        st.put(sp++, far);
                    } else if (!il && !ir) {
                        if (sp == 0) { done = true; break; }
                        next = st.get(--sp);
                    }
                    node = next;
                }
            }
            if (done) {
                if (anyQ) {
                    uint8_t* occOut = BATCH ? static_cast<uint8_t*>(out) : p.occluded;
                    occOut[rid] = (occl && !(flags & (kHitFlagOverflow | kHitFlagIterCap))) ? 1 : 0;
                } else {
                    const bool hit = hitID >= 0;
                    uint32_t f = flags | (hit ? kHitFlagHit : 0u);
                    if (TIES ? (hit && fsub(second, hitDist) <= fmul(kTieWindow, hitDist)) || tieSuspect
                             : hit && fsub(second, hitDist) <= fmul(1e-6f, hitDist))
                        f |= kHitFlagNearTie;
                    float4* hp = (BATCH ? static_cast<float4*>(out) : p.hits) + size_t(rid) * 2;
                    hp[0] = make_float4(hitDist, __int_as_float(hitID), __int_as_float(hitInst), __uint_as_float(f));
                    hp[1] = make_float4(hu, hv, second, 0.0f);
                }
                live = false;
            }
        }
    }

    if constexpr (STAGE > 0) {
        // a copy left in flight by a timed-out wait must land before the CTA exits
        const uint32_t bits = s_rstate[warp][2];
        if (bits & kStPending) {
            const uint32_t nb = (bits & kStCur) ? 0u : 1u;
            (void)__all_sync(kFull, stage_wait(shared_addr(&s_rbar[warp][nb]), (bits >> (9 + nb)) & 1u));
        }
    }

    if (COUNT) {
        unsigned long long nc = nodeCount, tc = triCount;
        for (int off = 16; off > 0; off >>= 1) {
            nc += __shfl_down_sync(kFull, nc, off);
            tc += __shfl_down_sync(kFull, tc, off);
        }
        if (lane == 0) {
            atomicAdd(p.fetch_counts, nc);
            atomicAdd(p.fetch_counts + 1, tc);
        }
    }
}

}  // namespace atlas::rt::dev
