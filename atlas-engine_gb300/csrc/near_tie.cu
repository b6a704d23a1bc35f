// FP64 re-test of near ties (include/atlas_rt.h, ae_rt_retest_near_ties).
//
// The FP32 traversal reproduces the engine's shader bit for bit, and flags a
// ray whose second-nearest accepted hit lies within 1e-6 relative t of the
// nearest (AE_HIT_NEAR_TIE): for those rays the FP32 winner is decided by
// rounding and traversal order.  This kernel finds, for each flagged ray, the
// nearest triangle in double precision: a closest-hit traversal of the same
// BVH with conservative slab tests (single precision, every box widened by a
// relative 1e-5 so that no triangle the double test accepts is culled by
// rounding) and
// the double form of the shader's triangle test (intersections.hsh:36-57),
// accepting tmin < t < tmax.  Exactly equal double distances resolve to the
// lower BVH-order triangle index, and t_second is the second smallest
// accepted distance over distinct triangles (two triangles at the same
// distance make t_second equal to t) when it lies within kSecondWindow
// relative of t, else +inf: the traversal prunes at that window once it has
// a hit, so it visits about what the FP32 closest-hit traversal visits
// instead of every box up to a far second surface.  An entry with the winner's vertices
// is the winner itself (the root's spatial split stores a straddling
// triangle twice), so the reported entry is one of its copies; the oracle's
// brute-force pass over every entry gives the same triangle and pair.
#include "atlas_rt.h"
#include "context.cuh"
#include "trace_kernels.cuh"

#include <cmath>

using namespace atlas::rt::host;

namespace {

constexpr uint32_t kRetestStack = 128;
constexpr double kSecondWindow = 1e-5;     // ten times the 1e-6 of a near tie

// The farthest distance that can still matter: best + |best| kSecondWindow
// (each operation rounded separately), or +inf before the first hit.
__device__ __forceinline__ double second_limit(double best) {
    return isinf(best) ? best : __dadd_rn(best, __dmul_rn(fabs(best), kSecondWindow));
}

struct RetestParams {
    const float4* nodes;
    const float4* tris;
    uint32_t n_nodes;
    uint32_t n_tris;
    const float4* rays;      // PackedRay (3 float4)
    const float4* hits;      // ae_hit (2 float4)
    uint32_t n;
    double tmin, tmax;
    uint32_t max_steps;
    ae_hit_f64* out;
    uint32_t* n_retested;    // flagged rays found by the compaction pass
    uint32_t* list;          // their indices, in no particular order
    uint32_t* error_word;
};

// Conservative slab test in single precision: [tn, tf] of the ray inside the
// box, widened by 1e-5 relative (+1e-30): each slab distance fl(fl(c - o) y)
// with y = RN(1/d) is within 3 units of 2^-24 of (c - o) / d unless it
// under- or overflows; an underflow stays inside the absolute term, and an
// overflowed distance lies beyond every float tmax (entry) or below every
// tmin (exit), where culling is right anyway; a NaN (0 times an infinite
// reciprocal) is dropped by fminf / fmaxf, which only widens.  An axis with
// zero direction constrains only by whether the origin lies in the (equally
// widened) slab.  tmin / tmax are rounded outwards to float.  Double
// precision is kept for the triangle test, which decides the result; the
// boxes only have to keep every triangle that test can accept.
__device__ __forceinline__ bool box32(const float o[3], const float d[3], const float y[3], float lx, float ly,
                                      float lz, float hx, float hy, float hz, float tmin, float tmax) {
    const float lo[3] = { lx, ly, lz }, hi[3] = { hx, hy, hz };
    float tn = tmin, tf = tmax;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (d[k] == 0.0f) {
            const float w = 1e-5f * (fabsf(lo[k]) + fabsf(hi[k])) + 1e-30f;
            if (o[k] < lo[k] - w || o[k] > hi[k] + w) return false;
            continue;
        }
        float a = (lo[k] - o[k]) * y[k], b = (hi[k] - o[k]) * y[k];
        if (a > b) { const float t = a; a = b; b = t; }
        const float w = 1e-5f * (fabsf(a) + fabsf(b)) + 1e-30f;
        tn = fmaxf(tn, a - w);
        tf = fminf(tf, b + w);
    }
    return tn <= tf;
}

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double cr(double a, double b, double c, double d) { return ds(dm(a, b), dm(c, d)); }
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
    return da(da(dm(a[0], b[0]), dm(a[1], b[1])), dm(a[2], b[2]));
}

// intersections.hsh:36-57 in double, every operation rounded separately in
// the formula's order (no contraction), so that exactly equal distances are
// decided as the double-precision restatement decides them.  Returns the
// accept test; t out.  A triangle whose quotients would fall clearly outside
// the accept test, or beyond `bound` (a distance past which no candidate
// changes the result), is rejected from the signs and sizes of the
// numerators and the denominator, without the three divisions: the margins
// (1e-12 of |den|) dwarf the rounding of a quotient (2^-53 relative), so
// such a triangle fails the exact test too.
__device__ __forceinline__ bool tri64(const double o[3], const double d[3], const float4& A, const float4& B,
                                      const float4& C, double bound, double& t) {
    const double v0[3] = { A.x, A.y, A.z };
    const double e0[3] = { ds(B.x, v0[0]), ds(B.y, v0[1]), ds(B.z, v0[2]) };
    const double e1[3] = { ds(C.x, v0[0]), ds(C.y, v0[1]), ds(C.z, v0[2]) };
    const double s[3] = { ds(o[0], v0[0]), ds(o[1], v0[1]), ds(o[2], v0[2]) };
    const double p[3] = { cr(s[1], e0[2], e0[1], s[2]), cr(s[2], e0[0], e0[2], s[0]), cr(s[0], e0[1], e0[0], s[1]) };
    const double q[3] = { cr(d[1], e1[2], e1[1], d[2]), cr(d[2], e1[0], e1[2], d[0]), cr(d[0], e1[1], e1[0], d[1]) };
    const double den = dot3(q, e0);
    const double nt = dot3(p, e1), nu = dot3(q, s), nv = dot3(p, d);
    const double ad = fabs(den);
    if (ad > 1e-200 && ad < 1e200) {
        const double sg = den < 0.0 ? -1.0 : 1.0;
        const double wt = nt * sg, wu = nu * sg, wv = nv * sg;      // exact: sign flips
        const double m = 1e-12 * ad;
        if (wu < -m || wv < -m || wt < -m || (wu >= 0.0 && wv >= 0.0 && wu + wv > ad + m) || wt > bound * (ad + m))
            return false;
    }
    t = __ddiv_rn(nt, den);
    const double u = __ddiv_rn(nu, den);
    const double v = __ddiv_rn(nv, den);
    return t >= 0.0 && u >= 0.0 && v >= 0.0 && da(u, v) <= 1.0;
}

// Two BVH entries with the same vertices are one triangle: the root spatial
// split stores a straddling triangle in both children, each copy under a box
// clipped to its side, so a traversal may find either copy but not both.
__device__ __forceinline__ bool same_triangle(const float4* q, const float4& A, const float4& B, const float4& C) {
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    return a.x == A.x && a.y == A.y && a.z == A.z && b.x == B.x && b.y == B.y && b.z == B.z && c.x == C.x &&
           c.y == C.y && c.z == C.z;
}

// Pass 1: every ray's result as the FP32 trace left it, and the list of the
// flagged rays (warp-aggregated appends), so that the double-precision pass
// runs one flagged ray per thread with full warps.
__global__ void retest_compact_kernel(RetestParams p) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const size_t n_iter = (size_t(p.n) + stride - 1) / stride * stride;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n_iter; i += stride) {
        bool flagged = false;
        if (i < p.n) {
            const float4 h0 = p.hits[i * 2], h1 = p.hits[i * 2 + 1];
            const uint32_t flags = __float_as_uint(h0.w);
            ae_hit_f64 r;
            r.t = double(h0.x);
            r.t_second = double(h1.z);
            r.triPtr = __float_as_int(h0.y);
            r.flags = flags & AE_HIT_HIT;
            r.reserved[0] = r.reserved[1] = 0;
            p.out[i] = r;
            flagged = (flags & AE_HIT_NEAR_TIE) && p.n_nodes != 0;
        }
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t want = __ballot_sync(0xffffffffu, flagged);
        uint32_t base = 0;
        if (want) {
            const uint32_t leader = __ffs(want) - 1;
            if (lane == leader) base = atomicAdd(p.n_retested, __popc(want));
            base = __shfl_sync(0xffffffffu, base, leader);
        }
        if (flagged) p.list[base + __popc(want & ((1u << lane) - 1u))] = uint32_t(i);
    }
}

// Pass 2: the double-precision search for every listed ray.
__global__ void retest_kernel(RetestParams p) {
    const uint32_t count = *p.n_retested;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        const uint32_t i = p.list[j];
        ae_hit_f64 r;
        r.reserved[0] = r.reserved[1] = 0;
        const float4 o4 = p.rays[size_t(i) * 3], d4 = p.rays[size_t(i) * 3 + 1];
        const double o[3] = { o4.x, o4.y, o4.z }, d[3] = { d4.x, d4.y, d4.z };
        const float of[3] = { o4.x, o4.y, o4.z }, df[3] = { d4.x, d4.y, d4.z };
        const float yf[3] = { __frcp_rn(d4.x), __frcp_rn(d4.y), __frcp_rn(d4.z) };
        const float tminf = __double2float_rd(p.tmin);
        double best = INFINITY, second = INFINITY;
        int32_t bi = -1;
        int32_t stack[kRetestStack];
        uint32_t sp = 0, steps = 0;
        int32_t node = 0;
        bool bad = false;
        while (true) {
            if (++steps > p.max_steps) { bad = true; atomicOr(p.error_word, atlas::rt::dev::kErrIterationCap); break; }
            if (node < 0) {
                int32_t tp = ~node;
                bool end = false;
                do {
                    if (uint32_t(tp) >= p.n_tris) { bad = true; break; }
                    const float4 A = __ldg(p.tris + size_t(tp) * 3), B = __ldg(p.tris + size_t(tp) * 3 + 1),
                                 C = __ldg(p.tris + size_t(tp) * 3 + 2);
                    end = A.w > 0.0f;
                    // single-precision screen: the FP32 barycentrics are within m / |den|
                    // of the exact ones (the near-tie slack), so a triangle outside its
                    // bounds by twice that, with |den| well above m, fails the exact test
                    // by more than m / |den| -- far more than the double test's rounding
                    float t32, u32, v32, sl[2];
                    bool near32 = true;
                    (void)atlas::rt::dev::tri_test<true>(of[0], of[1], of[2], df[0], df[1], df[2], A, B, C, t32, u32,
                                                         v32, &near32, sl);
                    const float ad = sl[0], m2 = 2.0f * sl[1];
                    const bool outside = ad > 2.0f * m2 && isfinite(u32) && isfinite(v32) &&
                                         !(__fmaf_rn(u32, ad, m2) >= 0.0f && __fmaf_rn(v32, ad, m2) >= 0.0f &&
                                           __fmaf_rn(1.0f - (u32 + v32), ad, 2.0f * m2) >= 0.0f);
                    double t;
                    if (!outside && tri64(o, d, A, B, C, fmin(fmin(p.tmax, second), second_limit(best)), t) && t > p.tmin &&
                        t < p.tmax &&
                        !(bi >= 0 && t == best && same_triangle(p.tris + size_t(bi) * 3, A, B, C))) {
                        if (t < best || (t == best && tp < bi)) {
                            if (tp != bi) second = best;
                            best = t;
                            bi = tp;
                        } else if (t < second && tp != bi) {
                            second = t;
                        }
                    }
                    tp++;
                } while (!end);
                if (bad || sp == 0) break;
                node = stack[--sp];
                continue;
            }
            if (uint32_t(node) >= p.n_nodes) { bad = true; break; }
            const float4* np = p.nodes + size_t(node) * 4;
            float4 n0, n1, n2, n3;
            atlas::rt::dev::ldg_node(np, n0, n1, n2, n3);
            // prune by the second distance, and by the window past the nearest
            // beyond which a second distance is not reported
            const double bound = fmin(fmin(p.tmax, second), second_limit(best));
            const float boundf = __double2float_ru(bound);
            const bool il = box32(of, df, yf, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tminf, boundf);
            const bool ir = box32(of, df, yf, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tminf, boundf);
            const int32_t l = __float_as_int(n3.x), rr = __float_as_int(n3.y);
            if (il && ir) {
                if (sp >= kRetestStack) { bad = true; atomicOr(p.error_word, atlas::rt::dev::kErrStackOverflow); break; }
                stack[sp++] = rr;
                node = l;
            } else if (il) {
                node = l;
            } else if (ir) {
                node = rr;
            } else {
                if (sp == 0) break;
                node = stack[--sp];
            }
        }
        r.flags = AE_HIT_RETESTED | (bi >= 0 ? AE_HIT_HIT : 0u) | (bad ? AE_HIT_OVERFLOW : 0u);
        r.triPtr = bi;
        r.t = best;
        r.t_second = second <= second_limit(best) ? second : INFINITY;
        p.out[i] = r;
    }
}

}  // namespace

extern "C" ae_rt_status ae_rt_retest_near_ties(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                               const ae_hit* hits, uint32_t n_rays, float tmin, float tmax,
                                               ae_hit_f64* out, uint32_t* n_retested, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (mesh_id < 0 || size_t(mesh_id) >= ctx->meshes.size())
        return Fail(ctx, AE_RT_INVALID_ARG, "unknown mesh id " + std::to_string(mesh_id));
    if (n_retested) *n_retested = 0;
    if (n_rays == 0) return AE_RT_OK;
    if (!rays || !hits || !out) return Fail(ctx, AE_RT_INVALID_ARG, "null ray, hit or result buffer");
    if (!IsDevicePointer(rays) || !IsDevicePointer(hits) || !IsDevicePointer(out))
        return Fail(ctx, AE_RT_INVALID_ARG, "ae_rt_retest_near_ties takes device buffers");
    if (n_rays > (1u << 30)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^30 rays in one call");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const DeviceMesh& m = ctx->meshes[size_t(mesh_id)];
    RetestParams p{};
    p.nodes = m.nodes;
    p.tris = m.tris;
    p.n_nodes = m.n_nodes;
    p.n_tris = m.n_tris;
    p.rays = reinterpret_cast<const float4*>(rays);
    p.hits = reinterpret_cast<const float4*>(hits);
    p.n = n_rays;
    p.tmin = tmin;
    p.tmax = tmax;
    p.max_steps = atlas::rt::dev::default_step_cap(m.n_nodes);
    p.out = out;
    // word 0: the count of flagged rays; then their indices
    AE_CUDA(ctx, ctx->retest_count.ensure(sizeof(uint32_t) * (size_t(n_rays) + 1)));
    p.n_retested = static_cast<uint32_t*>(ctx->retest_count.ptr);
    p.list = p.n_retested + 1;
    p.error_word = ctx->d_counter + 1;
    AE_CUDA(ctx, cudaMemsetAsync(p.n_retested, 0, sizeof(uint32_t), s));
    const uint32_t cap = uint32_t(ctx->sm_count) * 8u;
    const uint32_t blocks = (n_rays + 255) / 256 < cap ? (n_rays + 255) / 256 : cap;
    retest_compact_kernel<<<blocks, 256, 0, s>>>(p);
    AE_CUDA(ctx, cudaGetLastError());
    // one listed ray per thread: enough threads for every ray being flagged
    const uint32_t cap2 = uint32_t(ctx->sm_count) * 16u;
    const uint32_t blocks2 = (n_rays + 127) / 128 < cap2 ? (n_rays + 127) / 128 : cap2;
    retest_kernel<<<blocks2, 128, 0, s>>>(p);
    AE_CUDA(ctx, cudaGetLastError());
    if (n_retested) {
        AE_CUDA(ctx, cudaMemcpyAsync(n_retested, p.n_retested, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        return ae_rt_synchronize(ctx, stream);
    }
    return AE_RT_OK;
}
