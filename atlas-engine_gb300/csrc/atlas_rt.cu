// Device context, uploads and trace entry points of the C ABI (include/atlas_rt.h).
#include "atlas_rt.h"
#include "context.cuh"
#include "trace_kernels.cuh"
#include "cast_kernels.cuh"
#include "pt_kernels.cuh"
#include "texture.cuh"
#include "bvh_builder.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

using namespace atlas::rt::host;

namespace {

using atlas::rt::dev::TraceParams;

// Kernel shapes the context can run (chosen by ae_rt_config, tuned by the
// project's autotuner): warps per CTA and the shared-memory part of each
// lane's 128-entry traversal stack (the rest spills to local memory).  The
// register budget follows from the minimum resident CTAs per SM.
constexpr int kStackEntries = 128;
// Stack entries of the deep variants, launched for meshes and scenes whose
// trees can need more than kStackEntries (local memory, 4 KB per lane).
constexpr int kDeepStackEntries = 1024;
struct Shape {
    int warps;
    int smem;
};
constexpr Shape kShapes[] = { { 4, 32 }, { 2, 32 }, { 8, 16 }, { 4, 16 } };
constexpr int kNumShapes = 4;

using atlas::rt::dev::MODE_BATCH;
using atlas::rt::dev::MODE_MESH;
using atlas::rt::dev::MODE_SCENE;

template <bool ANY, bool COUNT, int MODE, int W, int S, bool TIES = true, int STAGE = 0, bool LOOSE = false,
          bool DEEP = false, bool CAMERA = false>
void* KernelFor() {
    // single-mesh kernels keep <= 64 registers; scene / batched kernels carry
    // more per-lane state and get ~73
    constexpr int minBlocks = MODE == MODE_MESH ? 32 / W : (28 / W > 0 ? 28 / W : 1);
    return reinterpret_cast<void*>(
        &atlas::rt::dev::trace_kernel<ANY, COUNT, MODE, W, S, (DEEP ? kDeepStackEntries : kStackEntries) - S,
                                      minBlocks, false, TIES && !ANY, STAGE, LOOSE, CAMERA>);
}

// ties = false: the caller discards the near-tie flag (the library's path
// tracer, passes and radiance cache) or the context was created with
// AE_RT_CFG_NO_NEAR_TIES, so the kernel skips its detection.
// staged: the ray tiles go through shared memory by bulk copy
// (AE_RT_CFG_STAGED_RAYS; single-mesh and scene launches without counters).
// loose: the approximate traversal (AE_RT_CFG_APPROXIMATE): single-mesh and
// scene launches without counters or staged rays, no near-tie flag.
template <int W, int S>
void* PickShape(bool any, bool count, int mode, bool ties, bool staged, bool loose, bool camera) {
    constexpr int T = atlas::rt::dev::kStageRays;
    if (camera)
        return ties ? KernelFor<false, false, MODE_MESH, W, S, true, 0, false, false, true>()
                    : KernelFor<false, false, MODE_MESH, W, S, false, 0, false, false, true>();
    if (loose && mode == MODE_SCENE && !count && !staged)
        return any ? KernelFor<true, false, MODE_SCENE, W, S, false, 0, true>()
                   : KernelFor<false, false, MODE_SCENE, W, S, false, 0, true>();
    if (loose && mode == MODE_MESH && !count && !staged)
        return any ? KernelFor<true, false, MODE_MESH, W, S, false, 0, true>()
                   : KernelFor<false, false, MODE_MESH, W, S, false, 0, true>();
    if (staged && !count && mode != MODE_BATCH) {
        if (mode == MODE_SCENE) {
            if (any) return KernelFor<true, false, MODE_SCENE, W, S, true, T>();
            return ties ? KernelFor<false, false, MODE_SCENE, W, S, true, T>()
                        : KernelFor<false, false, MODE_SCENE, W, S, false, T>();
        }
        if (any) return KernelFor<true, false, MODE_MESH, W, S, true, T>();
        return ties ? KernelFor<false, false, MODE_MESH, W, S, true, T>()
                    : KernelFor<false, false, MODE_MESH, W, S, false, T>();
    }
    if (mode == MODE_BATCH) {
        if (!ties)
            return count ? KernelFor<false, true, MODE_BATCH, W, S, false>() : KernelFor<false, false, MODE_BATCH, W, S, false>();
        return count ? KernelFor<false, true, MODE_BATCH, W, S>() : KernelFor<false, false, MODE_BATCH, W, S>();
    }
    if (mode == MODE_SCENE) {
        if (any) return count ? KernelFor<true, true, MODE_SCENE, W, S>() : KernelFor<true, false, MODE_SCENE, W, S>();
        if (!ties)
            return count ? KernelFor<false, true, MODE_SCENE, W, S, false>() : KernelFor<false, false, MODE_SCENE, W, S, false>();
        return count ? KernelFor<false, true, MODE_SCENE, W, S>() : KernelFor<false, false, MODE_SCENE, W, S>();
    }
    if (any) return count ? KernelFor<true, true, MODE_MESH, W, S>() : KernelFor<true, false, MODE_MESH, W, S>();
    if (!ties)
        return count ? KernelFor<false, true, MODE_MESH, W, S, false>() : KernelFor<false, false, MODE_MESH, W, S, false>();
    return count ? KernelFor<false, true, MODE_MESH, W, S>() : KernelFor<false, false, MODE_MESH, W, S>();
}

// The deep variants (kDeepStackEntries, exact traversal, the default shape)
// for single-mesh and scene launches whose tree can need more than
// kStackEntries entries.
void* PickDeep(bool any, int mode, bool ties) {
    if (mode == MODE_SCENE) {
        if (any) return KernelFor<true, false, MODE_SCENE, 4, 32, true, 0, false, true>();
        return ties ? KernelFor<false, false, MODE_SCENE, 4, 32, true, 0, false, true>()
                    : KernelFor<false, false, MODE_SCENE, 4, 32, false, 0, false, true>();
    }
    if (any) return KernelFor<true, false, MODE_MESH, 4, 32, true, 0, false, true>();
    return ties ? KernelFor<false, false, MODE_MESH, 4, 32, true, 0, false, true>()
                : KernelFor<false, false, MODE_MESH, 4, 32, false, 0, false, true>();
}

void* PickKernelShape(int shape, bool any, bool count, int mode, bool ties = true, bool staged = false,
                      bool loose = false, bool camera = false) {
    switch (shape) {
    case 1: return PickShape<2, 32>(any, count, mode, ties, staged, loose, camera);
    case 2: return PickShape<8, 16>(any, count, mode, ties, staged, loose, camera);
    case 3: return PickShape<4, 16>(any, count, mode, ties, staged, loose, camera);
    default: return PickShape<4, 32>(any, count, mode, ties, staged, loose, camera);
    }
}

int ShapeIndex(uint32_t threads, uint32_t smem) {
    if (threads == 0) threads = 128;
    if (smem == 0) smem = 32;
    for (int i = 0; i < kNumShapes; i++)
        if (uint32_t(kShapes[i].warps * 32) == threads && uint32_t(kShapes[i].smem) == smem) return i;
    return -1;
}

}  // namespace


namespace {

// Copy of `nodes` with padding0 = 1 on nodes holding a coordinate outside the
// traversal kernel's fast-division window (0 or 2^-40..2^40), 0 elsewhere.
std::vector<ae_bvh_node> FlagNodes(const ae_bvh_node* nodes, uint32_t n) {
    std::vector<ae_bvh_node> out(nodes, nodes + n);
    for (auto& nd : out) {
        const float* c = nd.leftAABB.min;
        bool ok = true;
        for (int k = 0; k < 12; k++) {
            const float a = std::fabs(c[k]);
            ok = ok && (a == 0.0f || (a >= 9.094947017729282e-13f && a <= 1.099511627776e12f));
        }
        nd.padding0 = ok ? 0 : 1;
        nd.padding1 = 0;
    }
    return out;
}

// Host-side BVH validation before upload: child pointers in range, inner
// children after their parent (pre-order, which rules out cycles), and every
// referenced leaf terminated by an end-of-node flag inside the buffer.
ae_rt_status ValidateBlas(ae_rt_ctx* ctx, const ae_bvh_node* nodes, uint32_t n_nodes,
                          const ae_bvh_triangle* tris, uint32_t n_tris) {
    // leafEnd[i] = first index >= i carrying the end flag (n_tris if none)
    std::vector<uint32_t> leafEnd(n_tris + 1, n_tris);
    for (int64_t i = int64_t(n_tris) - 1; i >= 0; i--)
        leafEnd[i] = tris[i].v0[3] > 0.0f ? uint32_t(i) : leafEnd[i + 1];
    for (uint32_t i = 0; i < n_nodes; i++) {
        const int32_t ptrs[2] = { nodes[i].leftPtr, nodes[i].rightPtr };
        for (int32_t ptr : ptrs) {
            if (ptr >= 0) {
                if (uint32_t(ptr) >= n_nodes || uint32_t(ptr) <= i)
                    return Fail(ctx, AE_RT_BAD_BVH, "node " + std::to_string(i) + " has child pointer " +
                                                    std::to_string(ptr) + " out of range or not after its parent");
            } else {
                const uint32_t first = uint32_t(~ptr);
                if (first >= n_tris)
                    return Fail(ctx, AE_RT_BAD_BVH, "node " + std::to_string(i) + " points at triangle " +
                                                    std::to_string(first) + " beyond " + std::to_string(n_tris));
                if (leafEnd[first] >= n_tris)
                    return Fail(ctx, AE_RT_BAD_BVH, "leaf starting at triangle " + std::to_string(first) +
                                                    " has no end-of-node flag");
            }
        }
    }
    return AE_RT_OK;
}

// Inner-node levels on the longest root-to-leaf path of a validated tree
// (children after their parents, so one pass from the back): the most stack
// entries its traversal can hold.
uint32_t TreeDepth(const ae_bvh_node* nodes, uint32_t n_nodes) {
    if (n_nodes == 0) return 0;
    std::vector<uint32_t> d(n_nodes, 1);
    for (int64_t i = int64_t(n_nodes) - 1; i >= 0; i--) {
        uint32_t below = 0;
        for (int32_t ptr : { nodes[i].leftPtr, nodes[i].rightPtr })
            if (ptr >= 0) below = std::max(below, d[size_t(ptr)]);
        d[size_t(i)] = 1 + below;
    }
    return d[0];
}

uint32_t MaxSteps(const ae_rt_ctx* ctx, const DeviceMesh& m) {
    if (ctx->max_steps_cfg) return ctx->max_steps_cfg;
    return atlas::rt::dev::default_step_cap(m.n_nodes);
}

// Persistent grid for `fn`: SMs x resident CTAs (the configured count, or the
// kernel's occupancy), never more warps than rays.
// threads: the block size when it is not the context's (the deep variants,
// sized by their occupancy alone).
uint32_t GridFor(const ae_rt_ctx* ctx, const void* fn, uint32_t n_rays, uint32_t threads = 0) {
    uint32_t per_sm = threads ? 0u : ctx->blocks_per_sm;
    if (threads == 0) threads = ctx->threads;
    if (per_sm == 0) {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, int(threads), 0) != cudaSuccess) {
            cudaGetLastError();
            occ = 1;
        }
        per_sm = uint32_t(occ > 0 ? occ : 1);
    }
    uint32_t grid = uint32_t(ctx->sm_count) * per_sm;
    const uint32_t needed = (n_rays + threads - 1) / threads;
    if (needed < grid) grid = needed;
    return grid == 0 ? 1 : grid;
}

// Work-counter words of the context's launches, used in rotation so that
// launches on different streams (up to kWorkSlots at a time) can overlap.
constexpr uint32_t kWorkSlots = 6;
uint32_t* WorkCounter(ae_rt_ctx* ctx) {
    const uint32_t k = ctx->next_work_slot++ % kWorkSlots;
    return ctx->d_counter + (k == 0 ? 0u : k + 1u);          // word 1 is the error word
}

// depth: stack entries the launch's tree can need (0: the batched launch,
// whose meshes keep to kStackEntries or report overflow).
// camera: the rays are p.cam's camera rays (single mesh, closest hit, a tree
// within kStackEntries, exact, no counters: Trace checks this).
ae_rt_status Launch(ae_rt_ctx* ctx, bool any, int mode, TraceParams& p, cudaStream_t s, bool ties = true,
                    uint32_t depth = 0, bool camera = false) {
    if (p.work_counter == ctx->d_counter) p.work_counter = WorkCounter(ctx);
    AE_CUDA(ctx, cudaMemsetAsync(p.work_counter, 0, sizeof(uint32_t), s));
    if (ctx->count_fetches) AE_CUDA(ctx, cudaMemsetAsync(ctx->d_fetch, 0, 2 * sizeof(unsigned long long), s));
    p.refill_steps = ctx->refill_steps;
    p.refill_below = ctx->refill_below;
    p.leaf_wait = ctx->leaf_wait;
    const bool deep = depth > uint32_t(kStackEntries) && mode != MODE_BATCH;
    void* fn = deep ? PickDeep(any, mode, ties && ctx->near_ties)
                    : PickKernelShape(ctx->shape, any, ctx->count_fetches, mode, ties && ctx->near_ties,
                                      ctx->staged_rays, ctx->approximate, camera);
    const uint32_t threads = deep ? 128u : ctx->threads;
    const uint32_t grid = GridFor(ctx, fn, p.n_rays, threads);
    void* args[] = { &p };
    AE_CUDA(ctx, cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, 0, s));
    return AE_RT_OK;
}

constexpr int32_t kSceneTarget = -1;   // Trace() target: the two-level scene

// The camera of ae_rt_raygen and the camera traces.
atlas::rt::dev::CameraParams CameraFrom(const ae_camera* cam) {
    atlas::rt::dev::CameraParams c{};
    c.lx = cam->location[0]; c.ly = cam->location[1]; c.lz = cam->location[2];
    c.ox = cam->origin[0]; c.oy = cam->origin[1]; c.oz = cam->origin[2];
    c.rx = cam->right[0]; c.ry = cam->right[1]; c.rz = cam->right[2];
    c.bx = cam->bottom[0]; c.by = cam->bottom[1]; c.bz = cam->bottom[2];
    c.width = cam->width; c.height = cam->height;
    c.jx = cam->jitter[0]; c.jy = cam->jitter[1];
    return c;
}

// cam: trace the camera rays of `cam` (rays null, n_rays = its pixel
// count), made in the traversal kernel where it can (one mesh, closest hit,
// a tree within kStackEntries, and none of the approximate, counting or
// staged launches), else written by raygen_kernel into scratch first.
ae_rt_status Trace(ae_rt_ctx* ctx, bool any, int32_t mesh_id, const ae_packed_ray* rays, uint32_t n_rays,
                   float tmin, float tmax, void* out, void* stream, const uint32_t* count_dev = nullptr,
                   uint32_t cull_mask = 0xffffffffu, bool per_ray_tmax = false, bool ties = true,
                   const atlas::rt::dev::CameraParams* cam = nullptr) {
    if (!ctx) return AE_RT_INVALID_ARG;
    const bool scene = mesh_id == kSceneTarget;
    if (scene && !ctx->scene_ready) return Fail(ctx, AE_RT_INVALID_ARG, "no scene has been set");
    if (!scene && (mesh_id < 0 || size_t(mesh_id) >= ctx->meshes.size()))
        return Fail(ctx, AE_RT_INVALID_ARG, "unknown mesh id " + std::to_string(mesh_id));
    if (n_rays == 0) return AE_RT_OK;
    if ((!rays && !cam) || !out) return Fail(ctx, AE_RT_INVALID_ARG, "null ray or result buffer");
    if (n_rays > (1u << 30)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^30 rays in one call");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    static const DeviceMesh kNoMesh;
    const DeviceMesh& m = scene ? kNoMesh : ctx->meshes[size_t(mesh_id)];

    const size_t ray_bytes = size_t(n_rays) * sizeof(ae_packed_ray);
    const size_t out_bytes = size_t(n_rays) * (any ? 1 : sizeof(ae_hit));
    const bool camera = cam && !scene && !any && count_dev == nullptr && m.depth <= uint32_t(kStackEntries) &&
                        !ctx->approximate && !ctx->count_fetches && !ctx->staged_rays;
    if (cam && !camera) {
        // the general path: the camera's rays into scratch, then a plain trace
        AE_CUDA(ctx, ctx->rays_in.ensure(ray_bytes));
        atlas::rt::dev::raygen_kernel<<<(n_rays + 255) / 256, 256, 0, s>>>(*cam,
                                                                        static_cast<float4*>(ctx->rays_in.ptr));
        AE_CUDA(ctx, cudaGetLastError());
        rays = static_cast<const ae_packed_ray*>(ctx->rays_in.ptr);
    }
    const bool rays_dev = camera || IsDevicePointer(rays);
    const bool out_dev = IsDevicePointer(out);

    const void* d_rays = camera ? nullptr : rays;
    void* d_out = out;
    if (!rays_dev) {
        AE_CUDA(ctx, ctx->rays_in.ensure(ray_bytes));
        AE_CUDA(ctx, cudaMemcpyAsync(ctx->rays_in.ptr, rays, ray_bytes, cudaMemcpyHostToDevice, s));
        d_rays = ctx->rays_in.ptr;
    }
    if (!out_dev) {
        AE_CUDA(ctx, ctx->results_out.ensure(out_bytes));
        d_out = ctx->results_out.ptr;
    }

    TraceParams p{};
    p.nodes = m.nodes;
    p.tris = m.tris;
    p.n_nodes = m.n_nodes;
    p.n_tris = m.n_tris;
    p.rays = static_cast<const float4*>(d_rays);
    p.n_rays = n_rays;
    p.n_rays_dev = count_dev;
    p.tmin = tmin;
    p.tmax = tmax;
    p.hits = any ? nullptr : static_cast<float4*>(d_out);
    p.occluded = any ? static_cast<uint8_t*>(d_out) : nullptr;
    p.work_counter = ctx->d_counter;
    p.error_word = ctx->d_counter + 1;
    p.fetch_counts = ctx->d_fetch;
    p.max_steps = scene ? (ctx->max_steps_cfg ? ctx->max_steps_cfg : ctx->scene_steps) : MaxSteps(ctx, m);
    if (scene) {
        p.tlas = ctx->d_tlas;
        p.n_tlas = ctx->n_tlas;
        p.instances = ctx->d_instances;
        p.n_instances = ctx->n_instances;
        p.meshes = ctx->d_mesh_table;
        p.n_meshes = ctx->n_mesh_table;
        p.cull_mask = cull_mask;
    }
    p.per_ray_tmax = per_ray_tmax ? 1u : 0u;
    if (camera) p.cam = *cam;
    ae_rt_status st = Launch(ctx, any, scene ? MODE_SCENE : MODE_MESH, p, s, ties, scene ? ctx->scene_depth : m.depth,
                             camera);
    if (st != AE_RT_OK) return st;

    if (!out_dev) {
        AE_CUDA(ctx, cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, s));
    }
    if (!out_dev || !rays_dev) return ae_rt_synchronize(ctx, stream);
    return AE_RT_OK;
}

}  // namespace

ae_rt_status atlas::rt::host::EnsureBounceQueues(ae_rt_ctx* ctx, uint32_t capacity) {
    for (int k = 0; k < 2; k++) {
        AE_CUDA(ctx, ctx->pt_rays[k].ensure(size_t(capacity) * sizeof(ae_packed_ray)));
        AE_CUDA(ctx, ctx->pt_pay[k].ensure(size_t(capacity) * sizeof(float4)));
    }
    AE_CUDA(ctx, ctx->pt_hits.ensure(size_t(capacity) * sizeof(ae_hit)));
    for (Scratch* sc : { &ctx->pt_shadow, &ctx->pt_shadow2 })
        AE_CUDA(ctx, sc->ensure(size_t(capacity) * sizeof(ae_packed_ray)));
    for (Scratch* sc : { &ctx->pt_shadow_pay, &ctx->pt_shadow_pay2 })
        AE_CUDA(ctx, sc->ensure(size_t(capacity) * sizeof(float4)));
    for (Scratch* sc : { &ctx->pt_occ, &ctx->pt_occ2 })
        AE_CUDA(ctx, sc->ensure(capacity));
    if (!ctx->d_pt_counts) AE_CUDA(ctx, cudaMalloc(&ctx->d_pt_counts, 4 * sizeof(uint32_t)));
    if (!ctx->trace_stream) AE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->trace_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ctx->pt_events)
        if (!e) AE_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return AE_RT_OK;
}

ae_rt_status atlas::rt::host::TraceSceneQueue(ae_rt_ctx* ctx, bool any, const ae_packed_ray* rays, uint32_t capacity,
                                             float tmin, float tmax, void* out, void* stream,
                                             const uint32_t* count_dev, uint32_t cull_mask, bool per_ray_tmax) {
    return Trace(ctx, any, kSceneTarget, rays, capacity, tmin, tmax, out, stream, count_dev, cull_mask, per_ray_tmax,
                 false);
}

namespace {

// Random float with |v| in [2^lo, 2^hi] (random sign, mantissa, exponent), or
// a structured special case (power of two, all-ones mantissa, zero).
__device__ __forceinline__ float selftest_float(uint32_t h1, uint32_t h2, int lo, int hi, bool allow_zero) {
    const uint32_t kind = h2 & 15u;
    if (allow_zero && kind == 0) return (h1 & 1u) ? -0.0f : 0.0f;
    const int e = lo + int((h2 >> 4) % uint32_t(hi - lo + 1));
    uint32_t mant = h1 & 0x7fffffu;
    if (kind == 1) mant = 0;                 // power of two
    if (kind == 2) mant = 0x7fffffu;         // just below the next power of two
    if (kind == 3) mant = 1;                 // just above a power of two
    const uint32_t bits = ((h1 >> 31) << 31) | (uint32_t(e + 127) << 23) | mant;
    return __uint_as_float(bits);
}

__global__ void selftest_division_kernel(uint64_t n, uint32_t seed, unsigned long long* mismatches) {
    using namespace atlas::rt::dev;
    unsigned long long bad = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t k = uint32_t(i) ^ uint32_t(i >> 32) * 0x9E3779B9u;
        const uint32_t h0 = pcg_hash(k ^ seed), h1 = pcg_hash(h0), h2 = pcg_hash(h1), h3 = pcg_hash(h2);
        const uint32_t h4 = pcg_hash(h3), h5 = pcg_hash(h4);
        // a = c - o with c, o in the coordinate window, d in the direction window
        const float c = selftest_float(h0, h1, -40, 39, true);
        float o = selftest_float(h2, h3, -40, 39, true);
        // nearly equal pair (a tiny difference); c = 0 would make o subnormal, outside the window
        if ((h5 & 7u) == 0 && c != 0.0f) o = __uint_as_float(__float_as_uint(c) ^ (h5 & 0xffu));
        const float d = selftest_float(h4, h5, -40, 39, false);
        const float a = __fsub_rn(c, o);
        const float ref = __fdiv_rn(a, d);
        const float got = div_rn_from_rcp(a, d, __frcp_rn(d));
        if (__float_as_uint(ref) != __float_as_uint(got) && !(ref == 0.0f && got == 0.0f)) bad++;
    }
    for (int off = 16; off > 0; off >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, off);
    if ((threadIdx.x & 31u) == 0 && bad) atomicAdd(mismatches, bad);
}

}  // namespace

extern "C" {

ae_rt_status ae_rt_ctx_create(const ae_rt_config* cfg, ae_rt_ctx** out) {
    if (!out) return AE_RT_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return AE_RT_NO_DEVICE;
    }
    ae_rt_ctx* ctx = new (std::nothrow) ae_rt_ctx;
    if (!ctx) return AE_RT_OUT_OF_MEMORY;
    ae_rt_config c{};
    if (cfg) c = *cfg;
    if (c.device < 0 || c.device >= count) {
        delete ctx;
        return AE_RT_INVALID_ARG;
    }
    ctx->device = c.device;
    ctx->max_steps_cfg = c.max_steps;
    ctx->count_fetches = (c.flags & AE_RT_CFG_COUNT_FETCHES) != 0;
    ctx->near_ties = (c.flags & AE_RT_CFG_NO_NEAR_TIES) == 0;
    ctx->staged_rays = (c.flags & AE_RT_CFG_STAGED_RAYS) != 0;
    ctx->approximate = (c.flags & AE_RT_CFG_APPROXIMATE) != 0;
    ctx->refill_steps = c.refill_steps;
    ctx->refill_below = c.refill_below == 0 ? atlas::rt::dev::kDefaultRefillBelow
                                            : (c.refill_below > 32 ? 0u : c.refill_below);
    ctx->leaf_wait = c.leaf_wait > 32 ? 32u : c.leaf_wait;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counter, 8 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_counter, 0, 8 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_fetch, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_fetch, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_cast_counts, 4 * sizeof(uint32_t));
    if (e != cudaSuccess) {
        ae_rt_ctx_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? AE_RT_OUT_OF_MEMORY : AE_RT_CUDA_ERROR;
    }
    ctx->shape = ShapeIndex(c.threads_per_block, c.stack_entries_smem);
    if (ctx->shape < 0) {
        ae_rt_ctx_destroy(ctx);
        return AE_RT_INVALID_ARG;
    }
    ctx->threads = uint32_t(kShapes[ctx->shape].warps * 32);
    ctx->blocks_per_sm = c.blocks_per_sm;
    *out = ctx;
    return AE_RT_OK;
}

void ae_rt_ctx_destroy(ae_rt_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (auto& m : ctx->meshes) {
        cudaFree(m.nodes);
        cudaFree(m.tris);
        cudaFree(m.shading);
    }
    cudaFree(ctx->d_counter);
    cudaFree(ctx->d_fetch);
    cudaFree(ctx->d_cast_counts);
    cudaFree(ctx->d_tlas);
    cudaFree(ctx->d_instances);
    cudaFree(ctx->d_mesh_table);
    cudaFree(ctx->d_inst_model);
    cudaFree(ctx->d_materials);
    cudaFree(ctx->d_tex_pool);
    cudaFree(ctx->d_tex_desc);
    cudaFree(ctx->d_lights);
    cudaFree(ctx->d_pt_counts);
    for (Scratch* sc : { &ctx->pt_rays[0], &ctx->pt_rays[1], &ctx->pt_pay[0], &ctx->pt_pay[1], &ctx->pt_hits,
                         &ctx->pt_shadow, &ctx->pt_shadow_pay, &ctx->pt_occ, &ctx->pt_shadow2, &ctx->pt_shadow_pay2,
                         &ctx->pt_occ2, &ctx->pass_rays, &ctx->pass_key, &ctx->pass_hits, &ctx->pass_rad,
                         &ctx->pass_shadow, &ctx->pass_shadow_pay, &ctx->pass_vis, &ctx->pass_counts })
        sc->release();
    for (cudaEvent_t e : ctx->pt_events)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->cast_events)
        if (e) cudaEventDestroy(e);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->trace_stream) cudaStreamDestroy(ctx->trace_stream);
    if (ctx->h_cast_counts) cudaFreeHost(ctx->h_cast_counts);
    if (ctx->h_error) cudaFreeHost(ctx->h_error);
    for (Scratch* sc : { &ctx->rays_in, &ctx->results_out, &ctx->batch_table, &ctx->retest_count, &ctx->cast_primary, &ctx->cast_primary_hits,
                         &ctx->cast_secondary, &ctx->cast_secondary_hits, &ctx->cast_shadow, &ctx->cast_occluded })
        sc->release();
    delete ctx;
}

const char* ae_rt_last_error(const ae_rt_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

ae_rt_status ae_rt_mesh_upload(ae_rt_ctx* ctx, const ae_bvh_node* nodes, uint32_t n_nodes,
                               const ae_bvh_triangle* tris, const ae_triangle* shading, uint32_t n_tris,
                               int32_t* mesh_id) {
    if (!ctx || !mesh_id) return AE_RT_INVALID_ARG;
    if ((n_nodes && !nodes) || (n_tris && !tris)) return Fail(ctx, AE_RT_INVALID_ARG, "null mesh buffer");
    if (n_tris >= (1u << 31) - 1 || n_nodes >= (1u << 31) - 1) return Fail(ctx, AE_RT_INVALID_ARG, "mesh too large");
    ae_rt_status v = ValidateBlas(ctx, nodes, n_nodes, tris, n_tris);
    if (v != AE_RT_OK) return v;
    std::lock_guard<std::mutex> g(ctx->upload_mutex);
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    DeviceMesh m;
    m.n_nodes = n_nodes;
    m.n_tris = n_tris;
    m.depth = TreeDepth(nodes, n_nodes);
    if (shading)
        for (uint32_t i = 0; i < n_tris && !m.transparent; i++) m.transparent = shading[i].d2[3] != 1.0f;
    auto upload = [&](float4** dst, const void* src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        return e;
    };
    std::vector<ae_bvh_node> flagged = FlagNodes(nodes, n_nodes);
    cudaError_t e = upload(&m.nodes, flagged.data(), size_t(n_nodes) * sizeof(ae_bvh_node));
    if (e == cudaSuccess) e = upload(&m.tris, tris, size_t(n_tris) * sizeof(ae_bvh_triangle));
    if (e == cudaSuccess && shading) e = upload(&m.shading, shading, size_t(n_tris) * sizeof(ae_triangle));
    if (e != cudaSuccess) {
        cudaFree(m.nodes);
        cudaFree(m.tris);
        cudaFree(m.shading);
        return CudaFail(ctx, e, "mesh upload");
    }
    *mesh_id = int32_t(ctx->meshes.size());
    ctx->meshes.push_back(m);
    return AE_RT_OK;
}

ae_rt_status ae_rt_trace_closest(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays, uint32_t n_rays,
                                 float tmin, float tmax, ae_hit* hits, void* stream) {
    return Trace(ctx, false, mesh_id, rays, n_rays, tmin, tmax, hits, stream);
}

ae_rt_status ae_rt_trace_any(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays, uint32_t n_rays,
                             float tmin, float tmax, uint8_t* occluded, void* stream) {
    return Trace(ctx, true, mesh_id, rays, n_rays, tmin, tmax, occluded, stream);
}

ae_rt_status ae_rt_scene_set(ae_rt_ctx* ctx, const ae_bvh_node* tlas, uint32_t n_tlas,
                             const ae_bvh_instance* instances, uint32_t n_instances) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if ((n_tlas && !tlas) || (n_instances && !instances)) return Fail(ctx, AE_RT_INVALID_ARG, "null scene buffer");
    if (n_tlas >= (1u << 31) - 1 || n_instances >= (1u << 31) - 1) return Fail(ctx, AE_RT_INVALID_ARG, "scene too large");
    // top-level pointers: inner nodes after their parent, leaves name an instance
    for (uint32_t i = 0; i < n_tlas; i++) {
        const int32_t ptrs[2] = { tlas[i].leftPtr, tlas[i].rightPtr };
        for (int32_t ptr : ptrs) {
            if (ptr >= 0 ? (uint32_t(ptr) >= n_tlas || uint32_t(ptr) <= i) : uint32_t(~ptr) >= n_instances)
                return Fail(ctx, AE_RT_BAD_BVH, "top-level node " + std::to_string(i) + " has pointer " +
                                                std::to_string(ptr) + " out of range");
        }
    }
    uint64_t steps = uint64_t(n_tlas) + n_instances;
    uint32_t blas_depth = 0;
    for (uint32_t i = 0; i < n_instances; i++) {
        const int32_t m = instances[i].meshOffset;
        if (m < 0 || size_t(m) >= ctx->meshes.size())
            return Fail(ctx, AE_RT_INVALID_ARG, "instance " + std::to_string(i) + " names unknown mesh " +
                                                std::to_string(m));
        steps += ctx->meshes[size_t(m)].n_nodes + ctx->meshes[size_t(m)].n_tris;
        blas_depth = std::max(blas_depth, ctx->meshes[size_t(m)].depth);
    }
    const uint32_t scene_depth = TreeDepth(tlas, n_tlas) + blas_depth;
    std::lock_guard<std::mutex> g(ctx->upload_mutex);
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<atlas::rt::dev::MeshDesc> table(ctx->meshes.size());
    for (size_t i = 0; i < table.size(); i++) {
        table[i].nodes = ctx->meshes[i].nodes;
        table[i].tris = ctx->meshes[i].tris;
        table[i].shading = ctx->meshes[i].shading;
        table[i].n_nodes = ctx->meshes[i].n_nodes;
        table[i].n_tris = ctx->meshes[i].n_tris;
    }
    std::vector<ae_bvh_node> flagged = FlagNodes(tlas, n_tlas);
    // object-to-world matrices: the inverse of each instance's world-to-object
    // affine map (the engine's TransformTriangle, surface.hsh:46-61)
    std::vector<float> model(size_t(n_instances) * 12);
    for (uint32_t i = 0; i < n_instances; i++) {
        const float* m = instances[i].inverseMatrix;
        double a[3][4];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) a[r][c] = m[r * 4 + c];
        const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                           a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                           a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
        if (det == 0.0 || !std::isfinite(det))
            return Fail(ctx, AE_RT_INVALID_ARG, "instance " + std::to_string(i) + " has a singular matrix");
        double inv[3][3];
        inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
        inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
        inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
        inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
        inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
        inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
        inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
        inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
        inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
        for (int r = 0; r < 3; r++) {
            double t = 0.0;
            for (int c = 0; c < 3; c++) {
                model[size_t(i) * 12 + r * 4 + c] = float(inv[r][c]);
                t -= inv[r][c] * a[c][3];
            }
            model[size_t(i) * 12 + r * 4 + 3] = float(t);
        }
    }
    cudaFree(ctx->d_tlas);
    cudaFree(ctx->d_instances);
    cudaFree(ctx->d_mesh_table);
    cudaFree(ctx->d_inst_model);
    ctx->d_tlas = nullptr;
    ctx->d_instances = nullptr;
    ctx->d_mesh_table = nullptr;
    ctx->d_inst_model = nullptr;
    ctx->scene_ready = false;
    auto up = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up(reinterpret_cast<void**>(&ctx->d_tlas), flagged.data(), flagged.size() * sizeof(ae_bvh_node));
    if (e == cudaSuccess)
        e = up(reinterpret_cast<void**>(&ctx->d_instances), instances, size_t(n_instances) * sizeof(ae_bvh_instance));
    if (e == cudaSuccess)
        e = up(reinterpret_cast<void**>(&ctx->d_mesh_table), table.data(), table.size() * sizeof(table[0]));
    if (e == cudaSuccess)
        e = up(reinterpret_cast<void**>(&ctx->d_inst_model), model.data(), model.size() * sizeof(float));
    if (e != cudaSuccess) return CudaFail(ctx, e, "scene upload");
    ctx->n_tlas = n_tlas;
    ctx->n_instances = n_instances;
    ctx->scene_depth = scene_depth;
    ctx->n_mesh_table = uint32_t(table.size());
    steps = 4 * steps + 64;
    ctx->scene_steps = steps > 0xffffffffull ? 0xffffffffu : uint32_t(steps);
    ctx->scene_ready = true;
    return AE_RT_OK;
}

ae_rt_status ae_rt_scene_build(ae_rt_ctx* ctx, const ae_bvh_instance* instances, const ae_aabb* world_aabbs,
                               uint32_t n_instances, uint32_t* order_out, uint32_t* n_ordered) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (n_instances == 0 || !instances || !world_aabbs)
        return Fail(ctx, AE_RT_INVALID_ARG, "a scene needs at least one instance");
    atlas::rt::BuiltBVH b;
    try {
        b = atlas::rt::BuildBoxBVH(reinterpret_cast<const float*>(world_aabbs), n_instances, false);
    } catch (...) {
        return Fail(ctx, AE_RT_OUT_OF_MEMORY, "top-level build failed");
    }
    // instances in reference order, nextInstance linking the members of a leaf
    std::vector<ae_bvh_instance> ordered(b.order.size());
    for (size_t i = 0; i < b.order.size(); i++) {
        ordered[i] = instances[b.order[i]];
        ordered[i].nextInstance = b.endOfNode[i] ? -1 : int32_t(i) + 1;
    }
    if (order_out)
        for (size_t i = 0; i < b.order.size(); i++) order_out[i] = b.order[i];
    if (n_ordered) *n_ordered = uint32_t(b.order.size());
    static_assert(sizeof(atlas::rt::BuiltNode) == sizeof(ae_bvh_node), "node layout");
    return ae_rt_scene_set(ctx, reinterpret_cast<const ae_bvh_node*>(b.nodes.data()), uint32_t(b.nodes.size()),
                           ordered.data(), uint32_t(ordered.size()));
}

ae_rt_status ae_rt_trace_scene_closest(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays, float tmin,
                                       float tmax, uint32_t cull_mask, ae_hit* hits, void* stream) {
    return Trace(ctx, false, kSceneTarget, rays, n_rays, tmin, tmax, hits, stream, nullptr, cull_mask);
}

ae_rt_status ae_rt_trace_scene_any(ae_rt_ctx* ctx, const ae_packed_ray* rays, uint32_t n_rays, float tmin,
                                   float tmax, uint32_t cull_mask, uint8_t* occluded, void* stream) {
    return Trace(ctx, true, kSceneTarget, rays, n_rays, tmin, tmax, occluded, stream, nullptr, cull_mask);
}

ae_rt_status ae_rt_trace_scene_closest_queue(ae_rt_ctx* ctx, const ae_packed_ray* rays, const uint32_t* count,
                                             uint32_t capacity, float tmin, float tmax, uint32_t cull_mask,
                                             ae_hit* hits, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!count || !IsDevicePointer(count) || (capacity && (!IsDevicePointer(rays) || !IsDevicePointer(hits))))
        return Fail(ctx, AE_RT_INVALID_ARG, "queue traces take device buffers");
    return Trace(ctx, false, kSceneTarget, rays, capacity, tmin, tmax, hits, stream, count, cull_mask);
}

ae_rt_status ae_rt_trace_scene_any_queue(ae_rt_ctx* ctx, const ae_packed_ray* rays, const uint32_t* count,
                                         uint32_t capacity, float tmin, float tmax, uint32_t cull_mask,
                                         uint8_t* occluded, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!count || !IsDevicePointer(count) || (capacity && (!IsDevicePointer(rays) || !IsDevicePointer(occluded))))
        return Fail(ctx, AE_RT_INVALID_ARG, "queue traces take device buffers");
    return Trace(ctx, true, kSceneTarget, rays, capacity, tmin, tmax, occluded, stream, count, cull_mask);
}

struct ae_rt_batch_plan {
    ae_rt_ctx* ctx = nullptr;
    atlas::rt::dev::BatchDesc* d_batches = nullptr;
    uint32_t* d_counter = nullptr;
    uint32_t n_batches = 0;
    uint32_t total = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// Device batch table for a launch; returns the total ray count.
ae_rt_status MakeBatchTable(ae_rt_ctx* ctx, const ae_batch_desc* batches, uint32_t n,
                            std::vector<atlas::rt::dev::BatchDesc>& table, uint32_t& total) {
    table.resize(n);
    uint64_t first = 0;
    for (uint32_t i = 0; i < n; i++) {
        const ae_batch_desc& b = batches[i];
        if (b.mesh_id < 0 || size_t(b.mesh_id) >= ctx->meshes.size())
            return Fail(ctx, AE_RT_INVALID_ARG, "batch " + std::to_string(i) + ": unknown mesh id");
        if (b.n_rays && (!IsDevicePointer(b.rays) || !IsDevicePointer(b.out)))
            return Fail(ctx, AE_RT_INVALID_ARG, "batch " + std::to_string(i) + ": batched traces take device buffers");
        const DeviceMesh& m = ctx->meshes[size_t(b.mesh_id)];
        atlas::rt::dev::BatchDesc& d = table[i];
        d.nodes = m.nodes;
        d.tris = m.tris;
        d.rays = reinterpret_cast<const float4*>(b.rays);
        d.out = b.out;
        d.n_nodes = m.n_nodes;
        d.n_tris = m.n_tris;
        d.n_rays = b.n_rays;
        d.any = b.any ? 1u : 0u;
        d.tmin = b.tmin;
        d.tmax = b.tmax;
        d.first = uint32_t(first);
        d.max_steps = ctx->max_steps_cfg ? ctx->max_steps_cfg : MaxSteps(ctx, m);
        first += b.n_rays;
        if (first > (1u << 30)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^30 rays in one batched launch");
    }
    total = uint32_t(first);
    return AE_RT_OK;
}

TraceParams BatchParams(ae_rt_ctx* ctx, const atlas::rt::dev::BatchDesc* d_batches, uint32_t n, uint32_t total,
                        uint32_t* counter) {
    TraceParams p{};
    p.n_rays = total;
    p.work_counter = counter;
    p.error_word = ctx->d_counter + 1;
    p.fetch_counts = ctx->d_fetch;
    p.batches = d_batches;
    p.n_batches = n;
    p.refill_steps = ctx->refill_steps;
    p.refill_below = ctx->refill_below;
    p.leaf_wait = ctx->leaf_wait;
    p.max_steps = 0xffffffffu;
    return p;
}

}  // namespace

ae_rt_status ae_rt_trace_batched(ae_rt_ctx* ctx, const ae_batch_desc* batches, uint32_t n_batches, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (n_batches == 0) return AE_RT_OK;
    if (!batches) return Fail(ctx, AE_RT_INVALID_ARG, "null batch table");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<atlas::rt::dev::BatchDesc> table;
    uint32_t total = 0;
    ae_rt_status st = MakeBatchTable(ctx, batches, n_batches, table, total);
    if (st != AE_RT_OK) return st;
    if (total == 0) return AE_RT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    AE_CUDA(ctx, ctx->batch_table.ensure(table.size() * sizeof(table[0])));
    AE_CUDA(ctx, cudaMemcpyAsync(ctx->batch_table.ptr, table.data(), table.size() * sizeof(table[0]),
                                 cudaMemcpyHostToDevice, s));
    TraceParams p = BatchParams(ctx, static_cast<atlas::rt::dev::BatchDesc*>(ctx->batch_table.ptr), n_batches,
                                total, ctx->d_counter);
    return Launch(ctx, false, MODE_BATCH, p, s);
}

ae_rt_status ae_rt_batch_plan_create(ae_rt_ctx* ctx, const ae_batch_desc* batches, uint32_t n_batches,
                                     ae_rt_batch_plan** out) {
    if (!ctx || !out) return AE_RT_INVALID_ARG;
    *out = nullptr;
    if (n_batches == 0 || !batches) return Fail(ctx, AE_RT_INVALID_ARG, "a plan needs at least one batch");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<atlas::rt::dev::BatchDesc> table;
    uint32_t total = 0;
    ae_rt_status st = MakeBatchTable(ctx, batches, n_batches, table, total);
    if (st != AE_RT_OK) return st;
    auto* plan = new (std::nothrow) ae_rt_batch_plan;
    if (!plan) return AE_RT_OUT_OF_MEMORY;
    plan->ctx = ctx;
    plan->n_batches = n_batches;
    plan->total = total;
    cudaStream_t cap = nullptr;
    cudaError_t e = cudaMalloc(&plan->d_batches, table.size() * sizeof(table[0]));
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->d_batches, table.data(), table.size() * sizeof(table[0]), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_counter, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        TraceParams p = BatchParams(ctx, plan->d_batches, n_batches, total, plan->d_counter);
        cudaError_t le = cudaMemsetAsync(plan->d_counter, 0, sizeof(uint32_t), cap);
        void* args[] = { &p };
        void* fn = PickKernelShape(ctx->shape, false, false, MODE_BATCH, ctx->near_ties);
        if (le == cudaSuccess)
            le = cudaLaunchKernel(fn, dim3(GridFor(ctx, fn, total)), dim3(ctx->threads), args, 0, cap);
        e = cudaStreamEndCapture(cap, &plan->graph);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (cap) cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        ae_rt_batch_plan_destroy(plan);
        return CudaFail(ctx, e, "batch plan");
    }
    *out = plan;
    return AE_RT_OK;
}

ae_rt_status ae_rt_batch_plan_launch(ae_rt_batch_plan* plan, void* stream) {
    if (!plan) return AE_RT_INVALID_ARG;
    ae_rt_ctx* ctx = plan->ctx;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    AE_CUDA(ctx, cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream)));
    return AE_RT_OK;
}

void ae_rt_batch_plan_destroy(ae_rt_batch_plan* plan) {
    if (!plan) return;
    cudaSetDevice(plan->ctx->device);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    cudaFree(plan->d_batches);
    cudaFree(plan->d_counter);
    delete plan;
}

ae_rt_status ae_rt_scene_set_materials(ae_rt_ctx* ctx, const ae_material* materials, uint32_t n) {
    if (!ctx || (n && !materials)) return AE_RT_INVALID_ARG;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaFree(ctx->d_materials);
    ctx->d_materials = nullptr;
    ctx->n_materials = 0;
    if (n) {
        AE_CUDA(ctx, cudaMalloc(&ctx->d_materials, size_t(n) * sizeof(ae_material)));
        AE_CUDA(ctx, cudaMemcpy(ctx->d_materials, materials, size_t(n) * sizeof(ae_material), cudaMemcpyHostToDevice));
    }
    ctx->n_materials = n;
    return AE_RT_OK;
}

namespace {

// One level of a texture's mip chain down from `src` (w x h texels of `texel`
// bytes): texel (x, y) of the next level averages texels (2x + {0, 1},
// 2y + {0, 1}), the indices clamped to the level; UNORM bytes as
// (a + b + c + d + 2) / 4 in integers, floats as ((a + b) + (c + d)) * 0.25.
void DownsampleLevel(const uint8_t* src, uint32_t w, uint32_t h, uint32_t format, uint8_t* dst) {
    const uint32_t texel = format == AE_TEX_R8_UNORM ? 1u : 4u, nw = w > 1 ? w >> 1 : 1u, nh = h > 1 ? h >> 1 : 1u;
    for (uint32_t y = 0; y < nh; y++)
        for (uint32_t x = 0; x < nw; x++) {
            const uint32_t x0 = std::min(2 * x, w - 1), x1 = std::min(2 * x + 1, w - 1);
            const uint32_t y0 = std::min(2 * y, h - 1), y1 = std::min(2 * y + 1, h - 1);
            const uint8_t* a = src + (size_t(y0) * w + x0) * texel;
            const uint8_t* b = src + (size_t(y0) * w + x1) * texel;
            const uint8_t* c = src + (size_t(y1) * w + x0) * texel;
            const uint8_t* d = src + (size_t(y1) * w + x1) * texel;
            uint8_t* o = dst + (size_t(y) * nw + x) * texel;
            if (format == AE_TEX_R32_FLOAT) {
                float fa, fb, fc, fd;
                std::memcpy(&fa, a, 4); std::memcpy(&fb, b, 4); std::memcpy(&fc, c, 4); std::memcpy(&fd, d, 4);
                const float f = ((fa + fb) + (fc + fd)) * 0.25f;
                std::memcpy(o, &f, 4);
            } else {
                for (uint32_t k = 0; k < texel; k++)
                    o[k] = uint8_t((uint32_t(a[k]) + b[k] + c[k] + d[k] + 2u) >> 2);
            }
        }
}

}  // namespace

ae_rt_status ae_rt_scene_set_textures(ae_rt_ctx* ctx, const ae_texture* textures, uint32_t n) {
    if (!ctx || (n && !textures)) return AE_RT_INVALID_ARG;
    std::vector<atlas::rt::dev::TexDesc> desc(n);
    size_t total = 0;
    for (uint32_t i = 0; i < n; i++) {
        const ae_texture& t = textures[i];
        const std::string what = "texture " + std::to_string(i) + ": ";
        if (!t.texels) return Fail(ctx, AE_RT_INVALID_ARG, what + "null texels");
        if (t.width == 0 || t.height == 0 || t.width > 65536u || t.height > 65536u)
            return Fail(ctx, AE_RT_INVALID_ARG, what + "width and height must lie in [1, 65536]");
        if (t.format > AE_TEX_R32_FLOAT) return Fail(ctx, AE_RT_INVALID_ARG, what + "unknown format");
        const uint32_t texel = t.format == AE_TEX_R8_UNORM ? 1u : 4u;
        const uint32_t row = t.width * texel;
        if (t.row_pitch != 0 && t.row_pitch < row) return Fail(ctx, AE_RT_INVALID_ARG, what + "row pitch below a row");
        desc[i] = atlas::rt::dev::TexDesc{};
        desc[i].offset = total;
        desc[i].width = t.width;
        desc[i].height = t.height;
        desc[i].format = t.format;
        desc[i].row_pitch = row;
        // the full mip chain down to 1 x 1, every level 16-byte aligned
        uint32_t levels = 0, w = t.width, h = t.height;
        for (;;) {
            total += (size_t(w) * texel * h + 15u) & ~size_t(15);
            levels++;
            if (w == 1 && h == 1) break;
            w = w > 1 ? w >> 1 : 1u;
            h = h > 1 ? h >> 1 : 1u;
        }
        desc[i].levels = levels;
    }
    std::vector<uint8_t> pool(total);
    for (uint32_t i = 0; i < n; i++) {
        const ae_texture& t = textures[i];
        const uint32_t texel = t.format == AE_TEX_R8_UNORM ? 1u : 4u;
        const size_t pitch = t.row_pitch ? t.row_pitch : desc[i].row_pitch;
        uint8_t* lv = pool.data() + desc[i].offset;
        for (uint32_t y = 0; y < t.height; y++)
            std::memcpy(lv + size_t(y) * desc[i].row_pitch, static_cast<const uint8_t*>(t.texels) + size_t(y) * pitch,
                        desc[i].row_pitch);
        uint32_t w = t.width, h = t.height;
        for (uint32_t k = 1; k < desc[i].levels; k++) {
            uint8_t* next = lv + ((size_t(w) * texel * h + 15u) & ~size_t(15));
            DownsampleLevel(lv, w, h, t.format, next);
            lv = next;
            w = w > 1 ? w >> 1 : 1u;
            h = h > 1 ? h >> 1 : 1u;
        }
    }
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaFree(ctx->d_tex_pool);
    cudaFree(ctx->d_tex_desc);
    ctx->d_tex_pool = nullptr;
    ctx->d_tex_desc = nullptr;
    ctx->n_textures = 0;
    if (n) {
        AE_CUDA(ctx, cudaMalloc(&ctx->d_tex_pool, total));
        AE_CUDA(ctx, cudaMalloc(&ctx->d_tex_desc, desc.size() * sizeof(desc[0])));
        AE_CUDA(ctx, cudaMemcpy(ctx->d_tex_pool, pool.data(), total, cudaMemcpyHostToDevice));
        AE_CUDA(ctx, cudaMemcpy(ctx->d_tex_desc, desc.data(), desc.size() * sizeof(desc[0]), cudaMemcpyHostToDevice));
    }
    ctx->n_textures = n;
    return AE_RT_OK;
}

ae_rt_status ae_rt_scene_set_environment(ae_rt_ctx* ctx, const float radiance[3]) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!radiance) return Fail(ctx, AE_RT_INVALID_ARG, "null environment radiance");
    for (int c = 0; c < 3; c++)
        if (!(radiance[c] >= 0.0f) || !std::isfinite(radiance[c]))
            return Fail(ctx, AE_RT_INVALID_ARG, "the environment radiance must be finite and non-negative");
    for (int c = 0; c < 3; c++) ctx->env[c] = radiance[c];
    return AE_RT_OK;
}

ae_rt_status ae_rt_scene_set_lights(ae_rt_ctx* ctx, const ae_light* lights, uint32_t n) {
    if (!ctx || (n && !lights)) return AE_RT_INVALID_ARG;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t data;
        std::memcpy(&data, &lights[i].data[0], 4);
        const uint32_t type = data >> 28;
        int32_t inst;
        std::memcpy(&inst, &lights[i].data[3], 4);
        if (type > 1) return Fail(ctx, AE_RT_INVALID_ARG, "light " + std::to_string(i) + ": unknown type");
        if (type == 1 && (inst < 0 || uint32_t(inst) >= ctx->n_instances))
            return Fail(ctx, AE_RT_INVALID_ARG, "light " + std::to_string(i) + ": instance out of range");
    }
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaFree(ctx->d_lights);
    ctx->d_lights = nullptr;
    ctx->n_lights = 0;
    if (n) {
        AE_CUDA(ctx, cudaMalloc(&ctx->d_lights, size_t(n) * sizeof(ae_light)));
        AE_CUDA(ctx, cudaMemcpy(ctx->d_lights, lights, size_t(n) * sizeof(ae_light), cudaMemcpyHostToDevice));
    }
    ctx->n_lights = n;
    return AE_RT_OK;
}

}  // extern "C"

namespace {

// The path tracer's sample loop (ae_rt_pathtrace / ae_rt_pathtrace_realtime):
// radiance into accum (+ accum64), or, with frame_accum, into the real-time
// [3][H][W] uint32 frame accumulation.
// What one path-tracing call writes: the non-real-time accumulation (accum,
// accum64) or the real-time frame image (frame_accum) and G-buffer (rt), over
// the whole image or one tile of it.
struct PtCall {
    float* accum = nullptr;
    double* accum64 = nullptr;
    uint32_t* frame_accum = nullptr;
    float max_radiance = 0.0f;
    const ae_pt_realtime* rt = nullptr;
    bool tiled = false;
    uint32_t x0 = 0, y0 = 0, w = 0, h = 0;
};

ae_rt_status PathTrace(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params, const PtCall& call,
                       void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    float* const accum = call.accum;
    double* const accum64 = call.accum64;
    uint32_t* const frame_accum = call.frame_accum;
    const float max_radiance = call.max_radiance;
    if (!cam || !params || (!accum && !frame_accum)) return Fail(ctx, AE_RT_INVALID_ARG, "null argument");
    if (!ctx->scene_ready) return Fail(ctx, AE_RT_INVALID_ARG, "no scene has been set");
    if (!ctx->d_materials) return Fail(ctx, AE_RT_INVALID_ARG, "no materials have been set");
    for (const auto& m : ctx->meshes)
        if (!m.shading && m.n_tris) return Fail(ctx, AE_RT_INVALID_ARG, "path tracing needs shading triangles");
    if (cam->width == 0 || cam->height == 0 || uint64_t(cam->width) * cam->height > (1ull << 28))
        return Fail(ctx, AE_RT_INVALID_ARG, "camera resolution out of range");
    if ((accum && !IsDevicePointer(accum)) || (accum64 && !IsDevicePointer(accum64)) ||
        (frame_accum && !IsDevicePointer(frame_accum)))
        return Fail(ctx, AE_RT_INVALID_ARG, "accumulation buffers must be device memory");
    if (frame_accum && !(max_radiance > 0.0f) && params->spp > 1)
        return Fail(ctx, AE_RT_INVALID_ARG, "the quantised real-time accumulation needs max_radiance > 0");
    const uint32_t tx0 = call.tiled ? call.x0 : 0u, ty0 = call.tiled ? call.y0 : 0u;
    const uint32_t tw = call.tiled ? call.w : cam->width, th = call.tiled ? call.h : cam->height;
    if (tw == 0 || th == 0 || tx0 > cam->width - tw || ty0 > cam->height - th || tw > cam->width || th > cam->height)
        return Fail(ctx, AE_RT_INVALID_ARG, "the tile does not lie inside the image");
    const ae_pt_realtime* rt = call.rt;
    if (rt) {
        const void* outs[4] = { rt->depth, rt->material_idx, rt->normal, rt->velocity };
        for (const void* o : outs)
            if (o && !IsDevicePointer(o)) return Fail(ctx, AE_RT_INVALID_ARG, "G-buffer planes must be device memory");
        if (rt->last_matrices && rt->n_last_matrices != ctx->n_instances)
            return Fail(ctx, AE_RT_INVALID_ARG, "last_matrices must hold one matrix per scene instance");
    }
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t n = cam->width * cam->height;
    const uint32_t n_tile = tw * th;
    ae_rt_status qs = EnsureBounceQueues(ctx, n);
    if (qs != AE_RT_OK) return qs;

    atlas::rt::dev::CameraParams c{};
    c.lx = cam->location[0]; c.ly = cam->location[1]; c.lz = cam->location[2];
    c.ox = cam->origin[0]; c.oy = cam->origin[1]; c.oz = cam->origin[2];
    c.rx = cam->right[0]; c.ry = cam->right[1]; c.rz = cam->right[2];
    c.bx = cam->bottom[0]; c.by = cam->bottom[1]; c.bz = cam->bottom[2];
    c.width = cam->width; c.height = cam->height;

    atlas::rt::dev::PtParams p{};
    p.sc.instances = ctx->d_instances;
    p.sc.inst_model = ctx->d_inst_model;
    p.sc.meshes = ctx->d_mesh_table;
    p.sc.materials = ctx->d_materials;
    p.sc.n_materials = ctx->n_materials;
    p.sc.lights = ctx->d_lights;
    p.sc.n_lights = ctx->n_lights;
    p.sc.tex.pool = ctx->d_tex_pool;
    p.sc.tex.desc = static_cast<const atlas::rt::dev::TexDesc*>(ctx->d_tex_desc);
    p.sc.tex.n = ctx->n_textures;
    p.width = cam->width;
    p.height = cam->height;
    p.max_bounces = params->max_bounces;
    p.epsilon = params->epsilon;
    p.seed = params->seed;
    p.mis = (params->flags & AE_PT_MIS) ? 1u : 0u;
    p.sc.env_r = ctx->env[0];
    p.sc.env_g = ctx->env[1];
    p.sc.env_b = ctx->env[2];
    const bool env = ctx->env[0] + ctx->env[1] + ctx->env[2] > 0.0f;
    // The engine traces with its opacity check (PathTracingRenderer.cpp:186;
    // rayHit.csh:327-338): closest hits skip surfaces of opacity 0, shadow
    // rays see the product of (1 - opacity).  With every opacity 1 that is
    // the opaque traversal, which runs here unless a mesh is not opaque.
    bool transparent = false;
    for (const auto& m : ctx->meshes) transparent = transparent || m.transparent;
    // with MIS (light hits) or an environment (misses) a later bounce's
    // shading adds into the pixels that the previous bounce's resolve,
    // running beside it, adds into
    p.atomic_accum = (p.mis || env) ? 1u : 0u;
    if (frame_accum) {
        // cleared here; the engine's renderer clears its frame image before
        // the dispatch (one store per pixel at one sample, atomics otherwise)
        AE_CUDA(ctx, cudaMemsetAsync(frame_accum, 0, size_t(n) * 3 * sizeof(uint32_t), s));
        p.frame_accum = frame_accum;
        p.rt_max_radiance = max_radiance;
        p.rt_max_per_sample = params->spp > 1 ? 0xFFFFFFFFu / params->spp : 0u;
        p.atomic_accum = 1;
    }
    p.hits_in = static_cast<const float4*>(ctx->pt_hits.ptr);
    p.accum = reinterpret_cast<float4*>(accum);
    p.accum64 = accum64;
    p.tile_x0 = tx0;
    p.tile_y0 = ty0;
    p.tile_w = tw;
    p.tile_h = th;
    p.centered = (frame_accum || (params->flags & AE_PT_CENTERED)) ? 1u : 0u;
    p.jitter_x = cam->jitter[0];
    p.jitter_y = cam->jitter[1];
    if (rt && (rt->depth || rt->material_idx || rt->normal || rt->velocity)) {
        // view, projection and last view-projection rows, then the previous
        // object-to-world rows of every instance
        std::vector<float> m(48 + (rt->last_matrices ? size_t(ctx->n_instances) * 12 : 0));
        std::memcpy(m.data(), rt->view, 16 * sizeof(float));
        std::memcpy(m.data() + 16, rt->proj, 16 * sizeof(float));
        std::memcpy(m.data() + 32, rt->pv_last, 16 * sizeof(float));
        if (rt->last_matrices) std::memcpy(m.data() + 48, rt->last_matrices, size_t(ctx->n_instances) * 12 * sizeof(float));
        AE_CUDA(ctx, ctx->pt_gb.ensure(m.size() * sizeof(float)));
        AE_CUDA(ctx, cudaMemcpyAsync(ctx->pt_gb.ptr, m.data(), m.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        p.gb_depth = rt->depth;
        p.gb_material = rt->material_idx;
        p.gb_normal = reinterpret_cast<float2*>(rt->normal);
        p.gb_velocity = reinterpret_cast<float2*>(rt->velocity);
        p.gb_mats = static_cast<const float4*>(ctx->pt_gb.ptr);
        p.gb_last_model = rt->last_matrices ? static_cast<const float4*>(ctx->pt_gb.ptr) + 12 : nullptr;
    }
    if (params->flags & AE_PT_RESTART) {
        // the first sample replaces the tile's accumulation (rayHit.csh:121-122
        // loads it only when sampleCount > 0)
        if (accum)
            AE_CUDA(ctx, cudaMemset2DAsync(accum + (size_t(ty0) * cam->width + tx0) * 4, size_t(cam->width) * 16, 0,
                                           size_t(tw) * 16, th, s));
        if (accum64)
            AE_CUDA(ctx, cudaMemset2DAsync(accum64 + (size_t(ty0) * cam->width + tx0) * 3, size_t(cam->width) * 24, 0,
                                           size_t(tw) * 24, th, s));
    }
    // every queue holds at most one ray per pixel of the tile
    const uint32_t blocks = (n_tile + 255) / 256;
    const float kInf = 1e12f;   // INF of common.hsh:8
    // Shadow queues alternate between two buffers: a bounce's shadow trace and
    // resolve run on the side stream while the next bounce is traced and shaded
    // on `s` (the plain estimator's later bounces add nothing into accum, so
    // only the resolves write it).  Events: [0], [1] shade done per queue,
    // [2], [3] resolve done per queue.
    Scratch* shadowRays[2] = { &ctx->pt_shadow, &ctx->pt_shadow2 };
    Scratch* shadowPay[2] = { &ctx->pt_shadow_pay, &ctx->pt_shadow_pay2 };
    Scratch* shadowOcc[2] = { &ctx->pt_occ, &ctx->pt_occ2 };
    cudaStream_t side = ctx->trace_stream;
    bool pending[2] = { false, false };
    for (uint32_t smp = 0; smp < params->spp; smp++) {
        p.sample = params->sample_offset + smp;
        p.gb_write = (smp == 0 && p.gb_mats) ? 1u : 0u;
        // ray generation into queue 0
        p.rays_out = static_cast<float4*>(ctx->pt_rays[0].ptr);
        p.pay_out = static_cast<float4*>(ctx->pt_pay[0].ptr);
        p.n_out = ctx->d_pt_counts + 0;
        atlas::rt::dev::pt_raygen_kernel<<<blocks, 256, 0, s>>>(c, p);
        AE_CUDA(ctx, cudaGetLastError());
        for (uint32_t b = 0; b <= params->max_bounces; b++) {
            const int in = int(b & 1), out = 1 - in, q = int(b & 1);
            p.bounce = b;
            p.rays_in = static_cast<const float4*>(ctx->pt_rays[in].ptr);
            p.pay_in = static_cast<const float4*>(ctx->pt_pay[in].ptr);
            p.n_in = ctx->d_pt_counts + in;
            p.rays_out = static_cast<float4*>(ctx->pt_rays[out].ptr);
            p.pay_out = static_cast<float4*>(ctx->pt_pay[out].ptr);
            p.n_out = ctx->d_pt_counts + out;
            p.shadow_rays = static_cast<float4*>(shadowRays[q]->ptr);
            p.shadow_pay = static_cast<float4*>(shadowPay[q]->ptr);
            p.n_shadow = ctx->d_pt_counts + 2 + q;
            p.shadow_occ = static_cast<const uint8_t*>(shadowOcc[q]->ptr);
            const ae_packed_ray* rays_in = static_cast<const ae_packed_ray*>(ctx->pt_rays[in].ptr);
            ae_rt_status st = transparent
                ? TraceTransparency(ctx, false, rays_in, n, 0.0f, kInf, AE_RT_MASK_ALL, ctx->pt_hits.ptr, stream,
                                    ctx->d_pt_counts + in)
                : Trace(ctx, false, kSceneTarget, rays_in, n, 0.0f, kInf, ctx->pt_hits.ptr, stream,
                        ctx->d_pt_counts + in, AE_RT_MASK_ALL, false, false);
            if (st != AE_RT_OK) return st;
            // this shadow queue's previous resolve must be done before it is refilled
            if (pending[q]) AE_CUDA(ctx, cudaStreamWaitEvent(s, ctx->pt_events[2 + q], 0));
            AE_CUDA(ctx, cudaMemsetAsync(ctx->d_pt_counts + out, 0, sizeof(uint32_t), s));
            AE_CUDA(ctx, cudaMemsetAsync(p.n_shadow, 0, sizeof(uint32_t), s));
            atlas::rt::dev::pt_shade_kernel<<<blocks, 256, 0, s>>>(p);
            AE_CUDA(ctx, cudaGetLastError());
            AE_CUDA(ctx, cudaEventRecord(ctx->pt_events[q], s));
            AE_CUDA(ctx, cudaStreamWaitEvent(side, ctx->pt_events[q], 0));
            const ae_packed_ray* shadow_in = static_cast<const ae_packed_ray*>(shadowRays[q]->ptr);
            if (transparent) {
                AE_CUDA(ctx, ctx->pt_vis[q].ensure(size_t(n) * sizeof(float)));
                p.shadow_vis = static_cast<const float*>(ctx->pt_vis[q].ptr);
                st = TraceTransparency(ctx, true, shadow_in, n, 0.0f, kInf, AE_RT_MASK_SHADOW, ctx->pt_vis[q].ptr, side,
                                       p.n_shadow, true);
            } else {
                p.shadow_vis = nullptr;
                st = Trace(ctx, true, kSceneTarget, shadow_in, n, 0.0f, kInf, shadowOcc[q]->ptr, side, p.n_shadow,
                           AE_RT_MASK_SHADOW, true);
            }
            if (st != AE_RT_OK) return st;
            atlas::rt::dev::pt_resolve_kernel<<<blocks, 256, 0, side>>>(p);
            AE_CUDA(ctx, cudaGetLastError());
            AE_CUDA(ctx, cudaEventRecord(ctx->pt_events[2 + q], side));
            pending[q] = true;
        }
        // the sample's resolves finish before the next sample's first hits
        // (whose emission goes into accum) are shaded
        for (int q = 0; q < 2; q++)
            if (pending[q]) AE_CUDA(ctx, cudaStreamWaitEvent(s, ctx->pt_events[2 + q], 0));
    }
    return AE_RT_OK;
}

}  // namespace

extern "C" {

ae_rt_status ae_rt_pathtrace(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params, float* accum,
                             double* accum64, void* stream) {
    if (ctx && !accum) return Fail(ctx, AE_RT_INVALID_ARG, "null accumulation buffer");
    PtCall call;
    call.accum = accum;
    call.accum64 = accum64;
    return PathTrace(ctx, cam, params, call, stream);
}

ae_rt_status ae_rt_pathtrace_tile(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params, uint32_t x0,
                                  uint32_t y0, uint32_t width, uint32_t height, float* accum, double* accum64,
                                  void* stream) {
    if (ctx && !accum) return Fail(ctx, AE_RT_INVALID_ARG, "null accumulation buffer");
    PtCall call;
    call.accum = accum;
    call.accum64 = accum64;
    call.tiled = true;
    call.x0 = x0;
    call.y0 = y0;
    call.w = width;
    call.h = height;
    return PathTrace(ctx, cam, params, call, stream);
}

ae_rt_status ae_rt_pathtrace_realtime(ae_rt_ctx* ctx, const ae_camera* cam, const ae_pt_params* params,
                                      const ae_pt_realtime* rt, uint32_t* frame_accum, float max_radiance,
                                      void* stream) {
    if (ctx && !frame_accum) return Fail(ctx, AE_RT_INVALID_ARG, "null frame accumulation buffer");
    PtCall call;
    call.frame_accum = frame_accum;
    call.max_radiance = max_radiance;
    call.rt = rt;
    return PathTrace(ctx, cam, params, call, stream);
}

ae_rt_status ae_rt_pt_tonemap_tile(ae_rt_ctx* ctx, const float* accum, uint32_t width, uint32_t height, uint32_t x0,
                                   uint32_t y0, uint32_t tile_width, uint32_t tile_height, uint32_t samples,
                                   float exposure, float gamma, float* out, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    const uint64_t n = uint64_t(tile_width) * tile_height;
    if (uint64_t(width) * height > (1ull << 28) || tile_width > width || tile_height > height ||
        x0 > width - tile_width || y0 > height - tile_height)
        return Fail(ctx, AE_RT_INVALID_ARG, "the tile does not lie inside the image");
    if (n == 0) return AE_RT_OK;
    if (!accum || !out || !IsDevicePointer(accum) || !IsDevicePointer(out))
        return Fail(ctx, AE_RT_INVALID_ARG, "ae_rt_pt_tonemap takes device buffers");
    if (samples == 0) return Fail(ctx, AE_RT_INVALID_ARG, "the sample count must be positive");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    const uint32_t blocks = uint32_t(std::min<uint64_t>((n + 255) / 256, uint64_t(ctx->sm_count) * 8u));
    atlas::rt::dev::pt_tonemap_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(accum), width, x0, y0, tile_width, tile_height, exposure, float(samples),
        gamma, reinterpret_cast<float4*>(out));
    AE_CUDA(ctx, cudaGetLastError());
    return AE_RT_OK;
}

ae_rt_status ae_rt_pt_tonemap(ae_rt_ctx* ctx, const float* accum, uint32_t width, uint32_t height, uint32_t samples,
                              float exposure, float gamma, float* out, void* stream) {
    return ae_rt_pt_tonemap_tile(ctx, accum, width, height, 0, 0, width, height, samples, exposure, gamma, out, stream);
}

ae_rt_status ae_rt_raygen(ae_rt_ctx* ctx, const ae_camera* cam, ae_packed_ray* rays, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!cam || !rays) return Fail(ctx, AE_RT_INVALID_ARG, "null camera or ray buffer");
    if (cam->width == 0 || cam->height == 0 || uint64_t(cam->width) * cam->height > (1ull << 30))
        return Fail(ctx, AE_RT_INVALID_ARG, "camera resolution out of range");
    if (!IsDevicePointer(rays)) return Fail(ctx, AE_RT_INVALID_ARG, "ae_rt_raygen writes device memory only");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    const atlas::rt::dev::CameraParams c = CameraFrom(cam);
    const uint32_t n = cam->width * cam->height;
    atlas::rt::dev::raygen_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        c, reinterpret_cast<float4*>(rays));
    AE_CUDA(ctx, cudaGetLastError());
    return AE_RT_OK;
}

ae_rt_status ae_rt_trace_closest_queue(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                       const uint32_t* count, uint32_t capacity, float tmin, float tmax,
                                       ae_hit* hits, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!count || !IsDevicePointer(count) || (capacity && (!IsDevicePointer(rays) || !IsDevicePointer(hits))))
        return Fail(ctx, AE_RT_INVALID_ARG, "queue traces take device buffers");
    return Trace(ctx, false, mesh_id, rays, capacity, tmin, tmax, hits, stream, count);
}

ae_rt_status ae_rt_trace_any_queue(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays,
                                   const uint32_t* count, uint32_t capacity, float tmin, float tmax,
                                   uint8_t* occluded, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!count || !IsDevicePointer(count) || (capacity && (!IsDevicePointer(rays) || !IsDevicePointer(occluded))))
        return Fail(ctx, AE_RT_INVALID_ARG, "queue traces take device buffers");
    return Trace(ctx, true, mesh_id, rays, capacity, tmin, tmax, occluded, stream, count);
}

namespace {
// The bounce spawn over primary rays in a buffer, or (rays null) over the
// camera rays of `cam`.
ae_rt_status Spawn(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays, const ae_camera* cam,
                   const ae_hit* hits, const uint32_t* count, uint32_t n, const ae_bounce_params* params,
                   ae_packed_ray* secondary, ae_packed_ray* shadow, uint32_t* counts, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (mesh_id < 0 || size_t(mesh_id) >= ctx->meshes.size())
        return Fail(ctx, AE_RT_INVALID_ARG, "unknown mesh id " + std::to_string(mesh_id));
    if (!params || !counts) return Fail(ctx, AE_RT_INVALID_ARG, "null parameters");
    if (n == 0) return AE_RT_OK;
    if ((rays && !IsDevicePointer(rays)) || !IsDevicePointer(hits) || !IsDevicePointer(secondary) ||
        !IsDevicePointer(shadow) || !IsDevicePointer(counts) || (count && !IsDevicePointer(count)))
        return Fail(ctx, AE_RT_INVALID_ARG, "the bounce spawn takes device buffers");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    atlas::rt::dev::SpawnParams sp{};
    sp.rays = reinterpret_cast<const float4*>(rays);
    if (!rays) sp.cam = CameraFrom(cam);
    sp.hits = reinterpret_cast<const float4*>(hits);
    sp.n_dev = count;
    sp.n = n;
    sp.tris = ctx->meshes[size_t(mesh_id)].tris;
    sp.secondary = reinterpret_cast<float4*>(secondary);
    sp.shadow = reinterpret_cast<float4*>(shadow);
    sp.counts = counts;
    sp.lightx = params->light_dir[0]; sp.lighty = params->light_dir[1]; sp.lightz = params->light_dir[2];
    sp.epsilon = params->epsilon;
    sp.seed = params->seed;
    atlas::rt::dev::spawn_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(sp);
    AE_CUDA(ctx, cudaGetLastError());
    return AE_RT_OK;
}
}  // namespace

ae_rt_status ae_rt_spawn_bounce(ae_rt_ctx* ctx, int32_t mesh_id, const ae_packed_ray* rays, const ae_hit* hits,
                                const uint32_t* count, uint32_t n, const ae_bounce_params* params,
                                ae_packed_ray* secondary, ae_packed_ray* shadow, uint32_t* counts,
                                void* stream) {
    if (ctx && !rays) return Fail(ctx, AE_RT_INVALID_ARG, "null ray buffer");
    return Spawn(ctx, mesh_id, rays, nullptr, hits, count, n, params, secondary, shadow, counts, stream);
}

ae_rt_status ae_rt_trace_camera_closest(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam, float tmin,
                                        float tmax, ae_hit* hits, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!cam) return Fail(ctx, AE_RT_INVALID_ARG, "null camera");
    if (cam->width == 0 || cam->height == 0 || uint64_t(cam->width) * cam->height > (1ull << 30))
        return Fail(ctx, AE_RT_INVALID_ARG, "camera resolution out of range");
    const atlas::rt::dev::CameraParams c = CameraFrom(cam);
    return Trace(ctx, false, mesh_id, nullptr, cam->width * cam->height, tmin, tmax, hits, stream, nullptr,
                 0xffffffffu, false, true, &c);
}

ae_rt_status ae_rt_spawn_bounce_camera(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam, const ae_hit* hits,
                                       const ae_bounce_params* params, ae_packed_ray* secondary,
                                       ae_packed_ray* shadow, uint32_t* counts, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!cam) return Fail(ctx, AE_RT_INVALID_ARG, "null camera");
    if (cam->width == 0 || cam->height == 0 || uint64_t(cam->width) * cam->height > (1ull << 30))
        return Fail(ctx, AE_RT_INVALID_ARG, "camera resolution out of range");
    return Spawn(ctx, mesh_id, nullptr, cam, hits, nullptr, cam->width * cam->height, params, secondary, shadow,
                 counts, stream);
}

namespace {
__global__ void publish_counts_kernel(const uint32_t* counts, uint32_t* host_mapped) {
    if (threadIdx.x < 2) host_mapped[threadIdx.x] = counts[threadIdx.x];
    __threadfence_system();
}

// The error word, taken (and cleared) in stream order and written to mapped
// host memory: a synchronising call then reads it without a blocking copy.
__global__ void publish_error_kernel(uint32_t* error_word, uint32_t* host_mapped) {
    *host_mapped = atomicExch(error_word, 0u);
    __threadfence_system();
}
}  // namespace

ae_rt_status ae_rt_cast_pass(ae_rt_ctx* ctx, int32_t mesh_id, const ae_camera* cam,
                             const ae_bounce_params* params, ae_cast_outputs* out, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (!cam || !params || !out) return Fail(ctx, AE_RT_INVALID_ARG, "null argument");
    if (mesh_id < 0 || size_t(mesh_id) >= ctx->meshes.size())
        return Fail(ctx, AE_RT_INVALID_ARG, "unknown mesh id " + std::to_string(mesh_id));
    if (cam->width == 0 || cam->height == 0 || uint64_t(cam->width) * cam->height > (1ull << 30))
        return Fail(ctx, AE_RT_INVALID_ARG, "camera resolution out of range");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t n = cam->width * cam->height;
    const size_t rb = size_t(n) * sizeof(ae_packed_ray), hb = size_t(n) * sizeof(ae_hit);
    AE_CUDA(ctx, ctx->cast_primary_hits.ensure(hb));
    AE_CUDA(ctx, ctx->cast_secondary.ensure(rb));
    AE_CUDA(ctx, ctx->cast_secondary_hits.ensure(hb));
    AE_CUDA(ctx, ctx->cast_shadow.ensure(rb));
    AE_CUDA(ctx, ctx->cast_occluded.ensure(n));
    auto* primHits = static_cast<ae_hit*>(ctx->cast_primary_hits.ptr);
    auto* sec = static_cast<ae_packed_ray*>(ctx->cast_secondary.ptr);
    auto* secHits = static_cast<ae_hit*>(ctx->cast_secondary_hits.ptr);
    auto* shd = static_cast<ae_packed_ray*>(ctx->cast_shadow.ptr);
    auto* occ = static_cast<uint8_t*>(ctx->cast_occluded.ptr);
    uint32_t* counts = ctx->d_cast_counts;
    const float kInf = 1e12f;   // INF of common.hsh:8
    // The result copies run on a second stream, each as soon as the stage
    // that produced it is done, so they overlap the later stages: primary hits
    // during the spawn and bounce trace, bounce rays and hits during the
    // shadow trace.  The host learns the queue lengths from a pinned word
    // written right after the spawn, while the bounce trace runs.
    if (!ctx->copy_stream) AE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ctx->cast_events)
        if (!e) AE_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!ctx->h_cast_counts) {
        AE_CUDA(ctx, cudaHostAlloc(&ctx->h_cast_counts, 2 * sizeof(uint32_t), cudaHostAllocMapped));
        AE_CUDA(ctx, cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->d_cast_counts_mapped),
                                              ctx->h_cast_counts, 0));
    }
    cudaStream_t cs = ctx->copy_stream;
    cudaEvent_t evPrim = ctx->cast_events[0], evCounts = ctx->cast_events[1], evSec = ctx->cast_events[2],
                evShd = ctx->cast_events[3];
    auto copy = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        if (!dst || !bytes) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, cs);
    };
    ae_rt_status st;
    // the primary rays are made in the traversal kernel (no ray buffer)
    if ((st = ae_rt_trace_camera_closest(ctx, mesh_id, cam, 0.0f, kInf, primHits, stream)) != AE_RT_OK) return st;
    AE_CUDA(ctx, cudaEventRecord(evPrim, s));
    AE_CUDA(ctx, cudaStreamWaitEvent(cs, evPrim, 0));
    AE_CUDA(ctx, copy(out->primary_hits, primHits, hb));
    AE_CUDA(ctx, cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s));
    if ((st = ae_rt_spawn_bounce_camera(ctx, mesh_id, cam, primHits, params, sec, shd, counts, stream)) != AE_RT_OK)
        return st;
    // the queue lengths reach the host through mapped memory, written by a
    // kernel: a copy here would queue on the copy engine behind the primary
    // hits and hold back the bounce trace that follows in stream order
    publish_counts_kernel<<<1, 32, 0, s>>>(counts, ctx->d_cast_counts_mapped);
    AE_CUDA(ctx, cudaGetLastError());
    AE_CUDA(ctx, cudaEventRecord(evCounts, s));
    const float shadowMax = kInf - 2.0f * params->epsilon;   // rayHit.csh:333
    const bool secToHost = (out->secondary_hits && !IsDevicePointer(out->secondary_hits)) ||
                           (out->secondary_rays && !IsDevicePointer(out->secondary_rays));
    if (!ctx->trace_stream) AE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->trace_stream, cudaStreamNonBlocking));
    if (secToHost) {
        // the bounce hits' copy to the host runs during the shadow trace (a
        // shadow trace beside the bounce trace delays the bounce hits and
        // measured slower end to end: 3.95 against 4.14 Grays/s)
        if ((st = Trace(ctx, false, mesh_id, sec, n, 0.0f, kInf, secHits, stream, counts)) != AE_RT_OK) return st;
        AE_CUDA(ctx, cudaEventRecord(evSec, s));
        if ((st = Trace(ctx, true, mesh_id, shd, n, 0.0f, shadowMax, occ, stream, counts + 1)) != AE_RT_OK)
            return st;
        AE_CUDA(ctx, cudaEventRecord(evShd, s));
    } else {
        // the shadow trace beside the bounce trace (both read only the spawn's
        // queues; separate work counters), each hiding the other's tail
        AE_CUDA(ctx, cudaStreamWaitEvent(ctx->trace_stream, evCounts, 0));
        if ((st = Trace(ctx, true, mesh_id, shd, n, 0.0f, shadowMax, occ, ctx->trace_stream, counts + 1)) !=
            AE_RT_OK)
            return st;
        AE_CUDA(ctx, cudaEventRecord(evShd, ctx->trace_stream));
        if ((st = Trace(ctx, false, mesh_id, sec, n, 0.0f, kInf, secHits, stream, counts)) != AE_RT_OK) return st;
        AE_CUDA(ctx, cudaEventRecord(evSec, s));
        AE_CUDA(ctx, cudaStreamWaitEvent(s, evShd, 0));
    }
    AE_CUDA(ctx, cudaEventSynchronize(evCounts));
    const volatile uint32_t* hc = ctx->h_cast_counts;
    const uint32_t nSec = hc[0], nShd = hc[1];
    out->counts[0] = n;
    out->counts[1] = nSec;
    out->counts[2] = nShd;
    AE_CUDA(ctx, cudaStreamWaitEvent(cs, evSec, 0));
    AE_CUDA(ctx, copy(out->secondary_rays, sec, size_t(nSec) * sizeof(ae_packed_ray)));
    AE_CUDA(ctx, copy(out->secondary_hits, secHits, size_t(nSec) * sizeof(ae_hit)));
    AE_CUDA(ctx, copy(out->shadow_rays, shd, size_t(nShd) * sizeof(ae_packed_ray)));
    AE_CUDA(ctx, cudaStreamWaitEvent(cs, evShd, 0));
    AE_CUDA(ctx, copy(out->shadow_occluded, occ, nShd));
    AE_CUDA(ctx, cudaStreamSynchronize(cs));
    return ae_rt_synchronize(ctx, stream);
}

ae_rt_status ae_rt_synchronize(ae_rt_ctx* ctx, void* stream) {
    if (!ctx) return AE_RT_INVALID_ARG;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->h_error) {
        AE_CUDA(ctx, cudaHostAlloc(&ctx->h_error, sizeof(uint32_t), cudaHostAllocMapped));
        AE_CUDA(ctx, cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->d_error_mapped), ctx->h_error, 0));
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    publish_error_kernel<<<1, 1, 0, s>>>(ctx->d_counter + 1, ctx->d_error_mapped);
    AE_CUDA(ctx, cudaGetLastError());
    AE_CUDA(ctx, cudaStreamSynchronize(s));
    const uint32_t err = *static_cast<volatile uint32_t*>(ctx->h_error);
    if (err) {
        if (err & 0x4u)   // kErrTimeout of the tensor-memory kernels
            return Fail(ctx, AE_RT_TIMEOUT, "a bounded device wait gave up");
        if (err & atlas::rt::dev::kErrQueueOverflow)
            return Fail(ctx, AE_RT_OUT_OF_MEMORY, "a wavefront queue was full; rays were dropped");
        if (err & atlas::rt::dev::kErrStackOverflow)
            return Fail(ctx, AE_RT_STACK_OVERFLOW,
                        "a ray needed more stack entries than its kernel holds (" + std::to_string(kStackEntries) +
                            "; " + std::to_string(kDeepStackEntries) + " for trees deeper than " +
                            std::to_string(kStackEntries) + " levels)");
        return Fail(ctx, AE_RT_ITERATION_LIMIT, "a ray exceeded the traversal step cap");
    }
    return AE_RT_OK;
}

namespace {

// The path tracer's own device functions on rows of inputs (the layouts of
// ae_rt_selftest_shading in include/atlas_rt.h).
__global__ void selftest_shading_kernel(uint32_t kind, const float* in, uint32_t n, float* out) {
    using namespace atlas::rt::dev;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto surf = [](const float* r, bool withL) {
        Surf s{};
        s.V = v3(r[0], r[1], r[2]);
        s.N = v3(r[3], r[4], r[5]);
        s.L = withL ? v3(r[6], r[7], r[8]) : s.N;
        s.mat.base = v3(r[9], r[10], r[11]);
        s.mat.roughness = r[12];
        s.mat.metalness = r[13];
        s.mat.reflectance = r[14];
        s.mat.opacity = 1.0f;
        s.mat.ao = 1.0f;
        update_surface(s);
        return s;
    };
    switch (kind) {
    case AE_SELFTEST_EVAL: {
        const Surf s = surf(in + size_t(i) * 15, true);
        const V3 d = eval_diffuse(s), sp = eval_specular(s);
        float* o = out + size_t(i) * 16;
        const float v[16] = { d.x, d.y, d.z, sp.x, sp.y, sp.z, s.NdotL, s.NdotV, s.NdotH, s.LdotH,
                              s.F0.x, s.F0.y, s.F0.z, s.F90, s.H.x, s.H.y };
        for (int k = 0; k < 16; k++) o[k] = v[k];
        break;
    }
    case AE_SELFTEST_SAMPLE_DIFFUSE:
    case AE_SELFTEST_SAMPLE_SPECULAR: {
        const float* r = in + size_t(i) * 17;
        Surf s = surf(r, false);
        V3 refl;
        const float pdf = kind == AE_SELFTEST_SAMPLE_DIFFUSE ? sample_diffuse(s, r[15], r[16], refl)
                                                              : sample_specular(s, r[15], r[16], refl);
        float* o = out + size_t(i) * 8;
        const float v[8] = { s.L.x, s.L.y, s.L.z, pdf, refl.x, refl.y, refl.z, s.NdotL };
        for (int k = 0; k < 8; k++) o[k] = v[k];
        break;
    }
    case AE_SELFTEST_TRIANGLE_LIGHT: {
        const float* r = in + size_t(i) * 24;
        Tri lt{};
        lt.v0 = v3(r[0], r[1], r[2]); lt.v1 = v3(r[3], r[4], r[5]); lt.v2 = v3(r[6], r[7], r[8]);
        lt.n0 = v3(r[9], r[10], r[11]); lt.n1 = v3(r[12], r[13], r[14]); lt.n2 = v3(r[15], r[16], r[17]);
        V3 P, N;
        triangle_light_point(lt, r[19], r[20], P, N);
        float* o = out + size_t(i) * 7;
        const float v[7] = { P.x, P.y, P.z, N.x, N.y, N.z, 1.0f / r[18] };
        for (int k = 0; k < 7; k++) o[k] = v[k];
        break;
    }
    case AE_SELFTEST_EVAL_TERMS: {
        // NdotL NdotV NdotH LdotH F0(3) F90 baseColor(3) roughness metalness
        const float* r = in + size_t(i) * 13;
        Surf s{};
        s.NdotL = r[0]; s.NdotV = r[1]; s.NdotH = r[2]; s.LdotH = r[3];
        s.F0 = v3(r[4], r[5], r[6]);
        s.F90 = r[7];
        s.mat.base = v3(r[8], r[9], r[10]);
        s.mat.roughness = r[11];
        s.mat.metalness = r[12];
        const V3 d = eval_diffuse(s), sp = eval_specular(s);
        float* o = out + size_t(i) * 6;
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = sp.x; o[4] = sp.y; o[5] = sp.z;
        break;
    }
    case AE_SELFTEST_TRIANGLE: {
        const float* r = in + size_t(i) * 15;
        const float4 a = make_float4(r[6], r[7], r[8], 0.0f), b = make_float4(r[9], r[10], r[11], 0.0f),
                     c = make_float4(r[12], r[13], r[14], 0.0f);
        float t, u, v;
        const bool hit = tri_test(r[0], r[1], r[2], r[3], r[4], r[5], a, b, c, t, u, v);
        float* o = out + size_t(i) * 4;
        o[0] = hit ? 1.0f : 0.0f; o[1] = t; o[2] = u; o[3] = v;
        break;
    }
    case AE_SELFTEST_AABB: {
        const float* r = in + size_t(i) * 14;
        float dist;
        bool nearCull;
        const bool hit = box_test<false>(r[0], r[1], r[2], r[3], r[4], r[5], 0.0f, 0.0f, 0.0f, r[6], r[7], r[8],
                                         r[9], r[10], r[11], r[12], r[13], dist, nearCull);
        out[size_t(i) * 2] = hit ? 1.0f : 0.0f;
        out[size_t(i) * 2 + 1] = dist;
        break;
    }
    default:
        break;
    }
}

}  // namespace

ae_rt_status ae_rt_selftest_shading(ae_rt_ctx* ctx, uint32_t kind, const float* in, uint32_t n, float* out) {
    static const uint32_t kIn[] = { 15, 17, 17, 24, 13, 15, 14 }, kOut[] = { 16, 8, 8, 7, 6, 4, 2 };
    if (!ctx || (n && (!in || !out))) return AE_RT_INVALID_ARG;
    if (kind > AE_SELFTEST_AABB) return Fail(ctx, AE_RT_INVALID_ARG, "unknown self-test kind");
    if (n == 0) return AE_RT_OK;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t ib = size_t(n) * kIn[kind] * sizeof(float), ob = size_t(n) * kOut[kind] * sizeof(float);
    float* d = nullptr;
    AE_CUDA(ctx, cudaMalloc(&d, ib + ob));
    cudaError_t e = cudaMemcpy(d, in, ib, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        selftest_shading_kernel<<<(n + 127) / 128, 128>>>(kind, d, n, d + size_t(n) * kIn[kind]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + size_t(n) * kIn[kind], ob, cudaMemcpyDeviceToHost);
    cudaFree(d);
    AE_CUDA(ctx, e);
    return AE_RT_OK;
}

ae_rt_status ae_rt_selftest_division(ae_rt_ctx* ctx, uint64_t n, uint32_t seed, uint64_t* mismatches) {
    if (!ctx || !mismatches) return AE_RT_INVALID_ARG;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    AE_CUDA(ctx, cudaMemset(ctx->d_fetch, 0, sizeof(unsigned long long)));
    selftest_division_kernel<<<uint32_t(ctx->sm_count) * 8u, 256>>>(n, seed, ctx->d_fetch);
    AE_CUDA(ctx, cudaGetLastError());
    unsigned long long h = 0;
    AE_CUDA(ctx, cudaMemcpy(&h, ctx->d_fetch, sizeof(h), cudaMemcpyDeviceToHost));
    *mismatches = h;
    return AE_RT_OK;
}

ae_rt_status ae_rt_get_fetch_counts(ae_rt_ctx* ctx, uint64_t* node_fetches, uint64_t* tri_fetches) {
    if (!ctx || !node_fetches || !tri_fetches) return AE_RT_INVALID_ARG;
    if (!ctx->count_fetches) return Fail(ctx, AE_RT_NOT_BUILT, "context created without AE_RT_CFG_COUNT_FETCHES");
    unsigned long long h[2] = { 0, 0 };
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    AE_CUDA(ctx, cudaMemcpy(h, ctx->d_fetch, sizeof(h), cudaMemcpyDeviceToHost));
    *node_fetches = h[0];
    *tri_fetches = h[1];
    return AE_RT_OK;
}

}  // extern "C"
