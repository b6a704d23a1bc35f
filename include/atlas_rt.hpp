/* atlas_rt.hpp -- C++ face of the traversal library for code written against
 * Atlas Engine's Volume::BVH (src/engine/volume/BVH.h:114-138) and
 * Volume::Ray (src/engine/volume/Ray.h:21-51).
 *
 * Header only, over the C ABI of atlas_rt.h; link libatlas_rt.so.
 *
 *   atlas::rt::BVH      same constructors and public members as Volume::BVH:
 *                       nodes, data (BVH order, endOfNode set), refs, aabbs,
 *                       GetTree(), Clear(), built by the library's host
 *                       builder, whose output equals the reference builder's.
 *   BVH::Upload         copies the BVH to a device context (GPUBVHNode and
 *                       GPUBVHTriangle layouts, MeshData.cpp:241-268).
 *   BVH::TraceClosest   batched closest hit on the GPU (ae_rt_trace_closest).
 *   BVH::TraceAny       batched occlusion on the GPU (ae_rt_trace_any).
 *   GetIntersection / GetIntersectionAny
 *                       the reference's one-ray host queries
 *                       (BVH.cpp:103-217), answered by the same GPU traversal.
 *   atlas::rt::PathTracingRenderer
 *                       the engine's path-tracing renderer (fields bounces,
 *                       realTime, realTimeSamplesPerFrame, maxRadiance; Render,
 *                       ResetSampleCount, GetSampleCount) over the library's
 *                       path tracer, tiles and real-time mode included.
 *
 * Query semantics are those of the engine's shader traversal (HitClosest /
 * HitAny, bvh.hsh:191-273, :359-441), which every GPU consumer of the BVH
 * sees: a triangle counts when tMin < t < tMax.  The reference's host query
 * differs in two places, both kept apart here on purpose:
 *   - it takes triangles at 0 <= t <= tMin too (Ray.cpp:53-76 tests t >= 0
 *     only), so results differ for triangles nearer than tMin;
 *   - its returned bool compares against the ray's tMax after the traversal
 *     lowered it (BVH.cpp:141, :172), so it reads false for many hits; the
 *     bool returned here is the hit itself.
 * There is no CPU path: every query needs an uploaded BVH and a CUDA device,
 * and a failing call throws atlas::rt::Error with the library's message. */
#pragma once

#include "atlas_rt.h"

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace atlas {
namespace rt {

struct vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    vec3() = default;
    constexpr vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

/* Volume::AABB (AABB.h): min and max corner. */
struct AABB {
    vec3 min, max;
    AABB() = default;
    AABB(vec3 mn, vec3 mx) : min(mn), max(mx) {}
};

/* Volume::BVHNode (BVH.h): ptr >= 0 is an inner node, ~ptr the first
 * primitive of a leaf. */
struct BVHNode {
    AABB leftAABB;
    AABB rightAABB;
    int32_t leftPtr = 0;
    int32_t rightPtr = 0;
};

/* Volume::BVHTriangle (BVH.h): idx is the caller's index, copied through the
 * build; endOfNode marks the last triangle of a leaf. */
struct BVHTriangle {
    vec3 v0, v1, v2;
    uint32_t idx = 0;
    bool endOfNode = false;
};

/* Volume::BVHBuilder::Ref (BVH.h): a leaf reference of the flattened tree;
 * nodeIdx is the last node created before the leaf was flattened
 * (BVH.cpp:411-415). */
struct Ref {
    uint32_t idx = 0;
    uint32_t nodeIdx = 0;
    bool endOfNode = false;
    AABB aabb;
};

/* Volume::Ray (Ray.h:21-51). */
struct Ray {
    Ray() = default;
    Ray(vec3 o, vec3 d, float tMin_ = 0.0f, float tMax_ = 2048.0f)
        : origin(o), direction(d), tMin(tMin_), tMax(tMax_) {}
    vec3 origin = vec3(0.0f);
    vec3 direction = vec3(0.0f, 1.0f, 0.0f);
    float tMin = 0.0f;
    float tMax = 2048.0f;
};

/* One closest-hit answer: t and the barycentric weights u (of v1) and v (of
 * v2), triPtr = the BVH-order triangle (index into BVH::data, -1 on a miss),
 * idx = data[triPtr].idx, flags = AE_HIT_* of the traversal. */
struct Hit {
    bool hit = false;
    float t = 0.0f, u = 0.0f, v = 0.0f;
    int32_t triPtr = -1;
    uint32_t idx = 0;
    uint32_t flags = 0;
};

class Error : public std::runtime_error {
public:
    Error(ae_rt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    ae_rt_status status;
};

/* A device context (ae_rt_ctx): one CUDA device, the meshes uploaded to it. */
class Context {
public:
    explicit Context(int device = 0) {
        ae_rt_config cfg;
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.device = device;
        Create(cfg);
    }
    explicit Context(const ae_rt_config& cfg) { Create(cfg); }
    ~Context() {
        if (ctx_) ae_rt_ctx_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    Context(Context&& o) noexcept : ctx_(o.ctx_) { o.ctx_ = nullptr; }
    Context& operator=(Context&& o) noexcept {
        std::swap(ctx_, o.ctx_);
        return *this;
    }

    ae_rt_ctx* get() const { return ctx_; }

    /* Throws Error for any status but AE_RT_OK, with the context's message. */
    void Check(ae_rt_status st, const char* call) const {
        if (st == AE_RT_OK) return;
        const char* msg = ctx_ ? ae_rt_last_error(ctx_) : "";
        throw Error(st, std::string(call) + ": " + (msg && *msg ? msg : "status " + std::to_string(int(st))));
    }

    void Synchronize(void* stream = nullptr) const { Check(ae_rt_synchronize(ctx_, stream), "ae_rt_synchronize"); }

private:
    void Create(const ae_rt_config& cfg) {
        const ae_rt_status st = ae_rt_ctx_create(&cfg, &ctx_);
        if (st != AE_RT_OK) {
            ctx_ = nullptr;
            throw Error(st, "ae_rt_ctx_create failed with status " + std::to_string(int(st)));
        }
    }
    ae_rt_ctx* ctx_ = nullptr;
};

class BVH {
public:
    BVH() = default;

    /* Volume::BVH::BVH(aabbs, data, parallelBuild), BVH.cpp:14-56: a
     * triangle BVH; data is reordered into BVH order with endOfNode set, and
     * aabbs follows it.  Unequal sizes leave the BVH empty, as in the
     * reference.  refs stays empty (the reference flattens into a local). */
    BVH(const std::vector<AABB>& aabbs_, const std::vector<BVHTriangle>& data_, bool parallelBuild = true) {
        if (aabbs_.size() != data_.size()) return;
        const size_t n = data_.size();
        verts_.resize(n * 9);
        std::vector<float> boxes(n * 6);
        for (size_t i = 0; i < n; i++) {
            const BVHTriangle& t = data_[i];
            const vec3* v[3] = { &t.v0, &t.v1, &t.v2 };
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) verts_[i * 9 + k * 3 + c] = (*v[k])[c];
            for (int c = 0; c < 3; c++) {
                boxes[i * 6 + c] = aabbs_[i].min[c];
                boxes[i * 6 + 3 + c] = aabbs_[i].max[c];
            }
        }
        ae_bvh* h = nullptr;
        CheckBuild(ae_bvh_build_triangles(n ? verts_.data() : nullptr, n ? boxes.data() : nullptr, uint32_t(n),
                                          parallelBuild ? 1 : 0, &h),
                   "ae_bvh_build_triangles");
        handle_.reset(h, ae_bvh_destroy);
        std::vector<uint32_t> order;
        std::vector<uint8_t> eon;
        ReadBack(order, eon);
        data.resize(order.size());
        aabbs.resize(order.size());
        for (size_t i = 0; i < order.size(); i++) {
            data[i] = data_[order[i]];
            data[i].endOfNode = eon[i] != 0;
            aabbs[i] = aabbs_[order[i]];
        }
        triangles_ = true;
    }

    /* Volume::BVH::BVH(aabbs, parallelBuild), BVH.cpp:58-100: the AABB-only
     * tree of the top level (64 bins).  refs holds the leaf references in
     * flattened order, aabbs the boxes in the same order; for a single box the
     * reference's list holds it twice (the input reference ahead of the
     * flattened one) and so does this one. */
    explicit BVH(const std::vector<AABB>& aabbs_, bool parallelBuild = true) {
        const size_t n = aabbs_.size();
        std::vector<float> boxes(n * 6);
        for (size_t i = 0; i < n; i++)
            for (int c = 0; c < 3; c++) {
                boxes[i * 6 + c] = aabbs_[i].min[c];
                boxes[i * 6 + 3 + c] = aabbs_[i].max[c];
            }
        ae_bvh* h = nullptr;
        CheckBuild(ae_bvh_build_aabbs(n ? boxes.data() : nullptr, uint32_t(n), parallelBuild ? 1 : 0, &h),
                   "ae_bvh_build_aabbs");
        handle_.reset(h, ae_bvh_destroy);
        std::vector<uint32_t> order;
        std::vector<uint8_t> eon;
        ReadBack(order, eon);
        refs.resize(order.size());
        aabbs.resize(order.size());
        const std::vector<uint32_t> leafNode = LeafNodeIndices(eon);
        for (size_t i = 0; i < order.size(); i++) {
            refs[i].idx = order[i];
            refs[i].endOfNode = eon[i] != 0;
            refs[i].nodeIdx = leafNode[i];
            refs[i].aabb = aabbs_[order[i]];
            aabbs[i] = aabbs_[order[i]];
        }
    }

    std::vector<BVHNode>& GetTree() { return nodes; }

    void Clear() {
        aabbs.clear();
        data.clear();
        refs.clear();
        nodes.clear();
        handle_.reset();
        verts_.clear();
        ctx_ = nullptr;
        mesh_ = -1;
    }

    /* Copies the triangle BVH to `ctx` as one mesh (GPUBVHNode + GPUBVHTriangle
     * arrays; material index and opacity per input triangle, optional: 0 and
     * 1.0).  Returns the mesh id; the queries below then run on that context,
     * which must outlive them. */
    int32_t Upload(Context& ctx, const int32_t* material = nullptr, const float* opacity = nullptr) {
        if (!triangles_ || !handle_)
            throw Error(AE_RT_INVALID_ARG, "BVH::Upload needs a triangle BVH");
        const uint32_t nn = ae_bvh_node_count(handle_.get());
        const uint32_t nt = ae_bvh_primitive_count(handle_.get());
        std::vector<ae_bvh_node> gnodes(nn);
        std::vector<ae_bvh_triangle> gtris(nt);
        ctx.Check(ae_bvh_get_nodes(handle_.get(), gnodes.data()), "ae_bvh_get_nodes");
        if (nt)
            ctx.Check(ae_bvh_pack_triangles(handle_.get(), verts_.data(), material, opacity, gtris.data()),
                      "ae_bvh_pack_triangles");
        int32_t id = -1;
        ctx.Check(ae_rt_mesh_upload(ctx.get(), gnodes.data(), nn, gtris.data(), nullptr, nt, &id), "ae_rt_mesh_upload");
        ctx_ = &ctx;
        mesh_ = id;
        return id;
    }

    int32_t MeshId() const { return mesh_; }

    /* Closest hit of n rays (host memory), each within its own (tMin, tMax);
     * rays sharing bounds go to the GPU in one call. */
    void TraceClosest(const Ray* rays, size_t n, Hit* hits, void* stream = nullptr) const {
        RequireUpload("BVH::TraceClosest");
        std::vector<ae_packed_ray> packed;
        std::vector<ae_hit> out;
        ForEachRun(rays, n, [&](size_t begin, size_t end) {
            Pack(rays + begin, end - begin, packed);
            out.resize(end - begin);
            ctx_->Check(ae_rt_trace_closest(ctx_->get(), mesh_, packed.data(), uint32_t(end - begin), rays[begin].tMin,
                                            rays[begin].tMax, out.data(), stream),
                        "ae_rt_trace_closest");
            for (size_t i = begin; i < end; i++) hits[i] = ToHit(out[i - begin]);
        });
    }

    std::vector<Hit> TraceClosest(const std::vector<Ray>& rays, void* stream = nullptr) const {
        std::vector<Hit> hits(rays.size());
        TraceClosest(rays.data(), rays.size(), hits.data(), stream);
        return hits;
    }

    /* Occlusion of n rays (host memory): occluded[i] = 1 when a triangle lies
     * at tMin < t < tMax. */
    void TraceAny(const Ray* rays, size_t n, uint8_t* occluded, void* stream = nullptr) const {
        RequireUpload("BVH::TraceAny");
        std::vector<ae_packed_ray> packed;
        ForEachRun(rays, n, [&](size_t begin, size_t end) {
            Pack(rays + begin, end - begin, packed);
            ctx_->Check(ae_rt_trace_any(ctx_->get(), mesh_, packed.data(), uint32_t(end - begin), rays[begin].tMin,
                                        rays[begin].tMax, occluded + begin, stream),
                        "ae_rt_trace_any");
        });
    }

    std::vector<uint8_t> TraceAny(const std::vector<Ray>& rays, void* stream = nullptr) const {
        std::vector<uint8_t> occ(rays.size());
        TraceAny(rays.data(), rays.size(), occ.data(), stream);
        return occ;
    }

    /* Volume::BVH::GetIntersection (BVH.cpp:103-174) for one ray.  On a hit:
     * closest = data[hit triangle], intersection = (t, u, v).  On a miss:
     * intersection.x = ray.tMax and closest = data[0], as the reference
     * leaves them.  Returns whether the ray hit.  `stack` is unused (the GPU
     * traversal keeps its own). */
    bool GetIntersection(std::vector<std::pair<int32_t, float>>& stack, Ray ray, BVHTriangle& closest,
                         vec3& intersection) {
        (void)stack;
        intersection.x = ray.tMax;
        if (nodes.empty()) return false;
        Hit h;
        TraceClosest(&ray, 1, &h);
        if (!h.hit) {
            closest = data[0];
            return false;
        }
        closest = data[size_t(h.triPtr)];
        intersection = vec3(h.t, h.u, h.v);
        return true;
    }

    /* Volume::BVH::GetIntersectionAny (BVH.cpp:176-217) for one ray. */
    bool GetIntersectionAny(std::vector<std::pair<int32_t, float>>& stack, Ray ray) {
        (void)stack;
        if (nodes.empty()) return false;
        uint8_t occ = 0;
        TraceAny(&ray, 1, &occ);
        return occ != 0;
    }

    std::vector<AABB> aabbs;
    std::vector<BVHTriangle> data;
    std::vector<Ref> refs;
    std::vector<BVHNode> nodes;

private:
    static void CheckBuild(ae_rt_status st, const char* call) {
        if (st != AE_RT_OK) throw Error(st, std::string(call) + " failed with status " + std::to_string(int(st)));
    }

    void ReadBack(std::vector<uint32_t>& order, std::vector<uint8_t>& eon) {
        const uint32_t nn = ae_bvh_node_count(handle_.get());
        const uint32_t np = ae_bvh_primitive_count(handle_.get());
        std::vector<ae_bvh_node> g(nn);
        if (nn) CheckBuild(ae_bvh_get_nodes(handle_.get(), g.data()), "ae_bvh_get_nodes");
        nodes.resize(nn);
        for (uint32_t i = 0; i < nn; i++) {
            nodes[i].leftAABB = AABB(vec3(g[i].leftAABB.min[0], g[i].leftAABB.min[1], g[i].leftAABB.min[2]),
                                     vec3(g[i].leftAABB.max[0], g[i].leftAABB.max[1], g[i].leftAABB.max[2]));
            nodes[i].rightAABB = AABB(vec3(g[i].rightAABB.min[0], g[i].rightAABB.min[1], g[i].rightAABB.min[2]),
                                      vec3(g[i].rightAABB.max[0], g[i].rightAABB.max[1], g[i].rightAABB.max[2]));
            nodes[i].leftPtr = g[i].leftPtr;
            nodes[i].rightPtr = g[i].rightPtr;
        }
        order.resize(np);
        eon.resize(np);
        if (np) CheckBuild(ae_bvh_get_order(handle_.get(), order.data(), eon.data()), "ae_bvh_get_order");
    }

    /* Ref::nodeIdx of each flattened reference.  Flatten creates nodes in
     * pre-order and stamps a leaf's references with the index of the last
     * node created so far (BVH.cpp:411-415): the parent for a left leaf, the
     * last node of the left sub-tree for a right leaf.  References ahead of
     * the first leaf pointer (the duplicate of a single-box build) keep 0. */
    std::vector<uint32_t> LeafNodeIndices(const std::vector<uint8_t>& eon) const {
        const size_t n_refs = eon.size();
        std::vector<uint32_t> out(n_refs, 0);
        if (nodes.empty()) return out;
        uint32_t last = 0;
        std::vector<std::pair<int32_t, int>> todo;  // (node, 0 = enter, 1 = right child)
        todo.push_back({ 0, 0 });
        auto stamp = [&](int32_t ptr) {
            for (size_t r = size_t(~ptr); r < n_refs; r++) {
                out[r] = last;
                if (eon[r]) break;
            }
        };
        while (!todo.empty()) {
            const auto [i, phase] = todo.back();
            todo.pop_back();
            const BVHNode& node = nodes[size_t(i)];
            if (phase == 0) {
                if (uint32_t(i) > last) last = uint32_t(i);
                todo.push_back({ i, 1 });
                if (node.leftPtr < 0)
                    stamp(node.leftPtr);
                else
                    todo.push_back({ node.leftPtr, 0 });
            } else if (node.rightPtr < 0) {
                stamp(node.rightPtr);
            } else {
                todo.push_back({ node.rightPtr, 0 });
            }
        }
        return out;
    }

    void RequireUpload(const char* call) const {
        if (!ctx_ || mesh_ < 0) throw Error(AE_RT_INVALID_ARG, std::string(call) + " needs BVH::Upload first");
    }

    template <class F>
    static void ForEachRun(const Ray* rays, size_t n, F&& f) {
        size_t begin = 0;
        while (begin < n) {
            size_t end = begin + 1;
            while (end < n && end - begin < (size_t(1) << 30) && rays[end].tMin == rays[begin].tMin &&
                   rays[end].tMax == rays[begin].tMax)
                end++;
            f(begin, end);
            begin = end;
        }
    }

    /* PackedRay (structures.hsh:9-13): origin.w = the ray's index bits. */
    static void Pack(const Ray* rays, size_t n, std::vector<ae_packed_ray>& out) {
        out.resize(n);
        for (size_t i = 0; i < n; i++) {
            ae_packed_ray& p = out[i];
            std::memset(&p, 0, sizeof(p));
            p.origin[0] = rays[i].origin.x;
            p.origin[1] = rays[i].origin.y;
            p.origin[2] = rays[i].origin.z;
            const int32_t id = int32_t(i);
            std::memcpy(&p.origin[3], &id, 4);
            p.direction[0] = rays[i].direction.x;
            p.direction[1] = rays[i].direction.y;
            p.direction[2] = rays[i].direction.z;
        }
    }

    Hit ToHit(const ae_hit& a) const {
        Hit h;
        h.flags = a.flags;
        h.hit = (a.flags & AE_HIT_HIT) != 0 && a.triPtr >= 0;
        h.t = a.t;
        h.u = a.u;
        h.v = a.v;
        h.triPtr = h.hit ? a.triPtr : -1;
        h.idx = h.hit && size_t(a.triPtr) < data.size() ? data[size_t(a.triPtr)].idx : 0;
        return h;
    }

    std::shared_ptr<ae_bvh> handle_;
    std::vector<float> verts_;
    bool triangles_ = false;
    Context* ctx_ = nullptr;
    int32_t mesh_ = -1;
};

/* The images PathTracingRenderer writes, as device buffers the caller owns
 * (the engine's PathTracerRenderTarget textures): the accumulation image
 * (float4 per pixel; FP64 copy optional), the tonemapped output image
 * (float4, optional) and, for the real-time mode, the [3][height][width]
 * frame image and the G-buffer planes. */
struct PathTracerRenderTarget {
    uint32_t width = 0, height = 0;
    float* accum = nullptr;
    double* accum64 = nullptr;
    float* output = nullptr;
    uint32_t* frameAccum = nullptr;
    ae_pt_realtime* gbuffer = nullptr;
};

/* PathTracingRenderer (src/engine/renderer/PathTracingRenderer.h:16-50,
 * PathTracingRenderer.cpp:29-306) over the library's path tracer, with the
 * engine's public fields and counters.  The scene (meshes with shading
 * triangles, instances, materials, lights) is the context's. */
class PathTracingRenderer {
public:
    explicit PathTracingRenderer(Context& ctx) : ctx_(&ctx) {}

    /* Render (PathTracingRenderer.cpp:29-192, :266-281).  A camera that moved
     * (location or frustum by more than 1e-3) or a new image size restarts the
     * accumulation.  Non-real-time: traces one sample of one tile of
     * imageSubdivisions per call (tile = resolution / subdivisions, at
     * tile * imageOffset; the remainder rows and columns of a resolution
     * that does not divide are not traced, as in the engine), adds it to the
     * accumulation (replacing it at sample 0) and writes the tile's output
     * image (exposure, gamma 1 / 2.2); after the last tile the sample count
     * advances.  Real-time: traces realTimeSamplesPerFrame samples of every
     * pixel into the frame image (and the G-buffer), the frame count
     * advances and the sample count reads 1. */
    void Render(PathTracerRenderTarget& target, const ae_camera& camera, float exposure = 1.0f,
                int32_t subdivisionsX = 1, int32_t subdivisionsY = 1, void* stream = nullptr) {
        if (target.width != camera.width || target.height != camera.height || subdivisionsX < 1 ||
            subdivisionsY < 1 || uint32_t(subdivisionsX) > camera.width || uint32_t(subdivisionsY) > camera.height)
            throw Error(AE_RT_INVALID_ARG, "PathTracingRenderer::Render: target, camera and subdivisions disagree");
        if (Moved(camera) || target.width != width_ || target.height != height_) {
            camera_ = camera;
            width_ = target.width;
            height_ = target.height;
            sampleCount_ = 0;
            offsetX_ = offsetY_ = 0;
        }
        ae_pt_params p;
        std::memset(&p, 0, sizeof(p));
        p.max_bounces = uint32_t(bounces);
        p.seed = seed;
        p.epsilon = epsilon;
        if (realTime) {
            subdivisionsX = subdivisionsY = 1;
            sampleCount_ = 0;
            frameCount_++;
            if (!target.frameAccum) throw Error(AE_RT_INVALID_ARG, "the real-time mode writes target.frameAccum");
            p.spp = uint32_t(realTimeSamplesPerFrame);
            p.sample_offset = uint32_t(frameCount_) * p.spp;
            ctx_->Check(ae_rt_pathtrace_realtime(ctx_->get(), &camera, &p, target.gbuffer, target.frameAccum,
                                                 maxRadiance, stream),
                        "ae_rt_pathtrace_realtime");
        } else {
            const uint32_t tw = camera.width / uint32_t(subdivisionsX), th = camera.height / uint32_t(subdivisionsY);
            const uint32_t x0 = tw * uint32_t(offsetX_), y0 = th * uint32_t(offsetY_);
            p.spp = 1;
            p.sample_offset = uint32_t(sampleCount_);
            p.flags = sampleCount_ == 0 ? AE_PT_RESTART : 0u;
            ctx_->Check(ae_rt_pathtrace_tile(ctx_->get(), &camera, &p, x0, y0, tw, th, target.accum, target.accum64,
                                             stream),
                        "ae_rt_pathtrace_tile");
            if (target.output)
                ctx_->Check(ae_rt_pt_tonemap_tile(ctx_->get(), target.accum, camera.width, camera.height, x0, y0, tw,
                                                  th, uint32_t(sampleCount_) + 1u, exposure, 1.0f / 2.2f,
                                                  target.output, stream),
                            "ae_rt_pt_tonemap_tile");
        }
        if (++offsetX_ == subdivisionsX) {
            offsetX_ = 0;
            offsetY_++;
        }
        if (offsetY_ >= subdivisionsY) {
            offsetY_ = 0;
            sampleCount_++;
        }
    }

    void ResetSampleCount() { sampleCount_ = 0; }
    int32_t GetSampleCount() const { return sampleCount_; }
    int32_t GetFrameCount() const { return frameCount_; }

    int32_t bounces = 10;
    bool realTime = true;
    int32_t realTimeSamplesPerFrame = 4;
    float maxRadiance = 65535.0f;
    uint32_t seed = 1;
    float epsilon = 0.1f;   /* EPSILON, raytracer/common.hsh:9 */

private:
    bool Moved(const ae_camera& c) const {
        auto dist = [](const float* a, const float* b) {
            const float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
            return std::sqrt(x * x + y * y + z * z);
        };
        return dist(c.location, camera_.location) > 1e-3f || dist(c.origin, camera_.origin) > 1e-3f ||
               dist(c.right, camera_.right) > 1e-3f || dist(c.bottom, camera_.bottom) > 1e-3f;
    }

    Context* ctx_;
    ae_camera camera_{};
    uint32_t width_ = 0, height_ = 0;
    int32_t sampleCount_ = 0, frameCount_ = 0;
    int32_t offsetX_ = 0, offsetY_ = 0;
};

}  // namespace rt
}  // namespace atlas
