// C wrapper over the reference's own BVH builder and host ray queries,
// compiled unmodified from the reference tree into oracle/_ref/libaeref.so.
//
// TEST INFRASTRUCTURE ONLY: used by the CPU tests in this container to pin the
// CPU restatement (oracle/ae_oracle.c) and the library's builder against the
// real reference, and to generate the committed golden fixtures.  The GPU machine
// has no reference tree, so nothing on the product path links this.
//
// Wrapped reference entry points:
//   Volume::BVH::BVH(aabbs, data, parallel)   src/engine/volume/BVH.cpp:14
//   Volume::BVH::BVH(aabbs, parallel)         src/engine/volume/BVH.cpp:58
//   Volume::BVH::GetIntersection              src/engine/volume/BVH.cpp:103
//   Volume::BVH::GetIntersectionAny           src/engine/volume/BVH.cpp:176
//   JobSystem::Init / Shutdown                src/engine/jobsystem/JobSystem.cpp:17,45
#include "volume/BVH.h"
#include "jobsystem/JobSystem.h"

#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

using namespace Atlas;

namespace {

bool g_jobsInit = false;

void ShutdownJobs() {
    if (g_jobsInit) {
        JobSystem::Shutdown();
        g_jobsInit = false;
    }
}

// Triangle AABB exactly as MeshData::BuildBVH forms it (src/engine/mesh/MeshData.cpp:143-146).
Volume::AABB TriangleAABB(const vec3& v0, const vec3& v1, const vec3& v2) {
    auto mn = glm::min(glm::min(v0, v1), v2);
    auto mx = glm::max(glm::max(v0, v1), v2);
    return Volume::AABB(mn, mx);
}

}  // namespace

extern "C" {

// Starts the reference job system with `threads` workers per priority pool
// (<= 0 keeps the reference's defaults, JobSystem.h:17-21).  Needed only for
// parallel builds.
void aeref_jobsystem_init(int threads) {
    if (g_jobsInit) return;
    JobSystemConfig cfg;
    if (threads > 0) {
        cfg.highPriorityThreadCount = threads;
        cfg.mediumPriorityThreadCount = threads;
        cfg.lowPriorityThreadCount = threads;
    }
    JobSystem::Init(cfg);
    g_jobsInit = true;
    std::atexit(ShutdownJobs);
}

void aeref_jobsystem_shutdown(void) { ShutdownJobs(); }

// Builds the triangle BVH.  verts: n_tris * 9 floats (v0, v1, v2 per triangle),
// triangle i gets idx = i (as MeshData.cpp:140).
void* aeref_build(const float* verts, uint32_t n_tris, int parallel) {
    std::vector<Volume::AABB> aabbs(n_tris);
    std::vector<Volume::BVHTriangle> tris(n_tris);
    for (uint32_t i = 0; i < n_tris; i++) {
        const float* t = verts + size_t(i) * 9;
        tris[i].v0 = vec3(t[0], t[1], t[2]);
        tris[i].v1 = vec3(t[3], t[4], t[5]);
        tris[i].v2 = vec3(t[6], t[7], t[8]);
        tris[i].idx = i;
        aabbs[i] = TriangleAABB(tris[i].v0, tris[i].v1, tris[i].v2);
    }
    if (parallel && !g_jobsInit) aeref_jobsystem_init(0);
    return new Volume::BVH(aabbs, tris, parallel != 0);
}

// Builds the AABB-only BVH used for the top level (BVH.cpp:58).
void* aeref_build_aabbs(const float* boxes /* n * 6: min, max */, uint32_t n, int parallel) {
    std::vector<Volume::AABB> aabbs(n);
    for (uint32_t i = 0; i < n; i++) {
        const float* b = boxes + size_t(i) * 6;
        aabbs[i] = Volume::AABB(vec3(b[0], b[1], b[2]), vec3(b[3], b[4], b[5]));
    }
    if (parallel && !g_jobsInit) aeref_jobsystem_init(0);
    return new Volume::BVH(aabbs, parallel != 0);
}

void aeref_free(void* h) { delete static_cast<Volume::BVH*>(h); }

uint32_t aeref_node_count(void* h) { return uint32_t(static_cast<Volume::BVH*>(h)->nodes.size()); }
uint32_t aeref_data_count(void* h) { return uint32_t(static_cast<Volume::BVH*>(h)->data.size()); }
uint32_t aeref_refs_count(void* h) { return uint32_t(static_cast<Volume::BVH*>(h)->refs.size()); }

// Nodes in the 64-byte GPUBVHNode layout (raytracing/RTStructures.h:95-103),
// copied field by field as MeshData.cpp:256-268 does.
void aeref_get_nodes(void* h, void* out) {
    auto& nodes = static_cast<Volume::BVH*>(h)->nodes;
    auto* o = static_cast<unsigned char*>(out);
    for (size_t i = 0; i < nodes.size(); i++) {
        float f[12] = {
            nodes[i].leftAABB.min.x, nodes[i].leftAABB.min.y, nodes[i].leftAABB.min.z,
            nodes[i].leftAABB.max.x, nodes[i].leftAABB.max.y, nodes[i].leftAABB.max.z,
            nodes[i].rightAABB.min.x, nodes[i].rightAABB.min.y, nodes[i].rightAABB.min.z,
            nodes[i].rightAABB.max.x, nodes[i].rightAABB.max.y, nodes[i].rightAABB.max.z };
        int32_t p[4] = { nodes[i].leftPtr, nodes[i].rightPtr, 0, 0 };
        std::memcpy(o + i * 64, f, 48);
        std::memcpy(o + i * 64 + 48, p, 16);
    }
}

// BVH-ordered triangle data: vertices (9 floats each), original index, endOfNode.
void aeref_get_data(void* h, float* verts, uint32_t* idx, uint8_t* end_of_node) {
    auto& data = static_cast<Volume::BVH*>(h)->data;
    for (size_t i = 0; i < data.size(); i++) {
        const auto& t = data[i];
        float f[9] = { t.v0.x, t.v0.y, t.v0.z, t.v1.x, t.v1.y, t.v1.z, t.v2.x, t.v2.y, t.v2.z };
        std::memcpy(verts + i * 9, f, sizeof(f));
        idx[i] = t.idx;
        end_of_node[i] = t.endOfNode ? 1 : 0;
    }
}

// Leaf references of the AABB-only build, in flattened order (BVH.cpp:92-97).
void aeref_get_refs(void* h, uint32_t* idx) {
    auto& refs = static_cast<Volume::BVH*>(h)->refs;
    for (size_t i = 0; i < refs.size(); i++) idx[i] = refs[i].idx;
}

// Every field of BVH::refs (BVHBuilder::Ref, BVH.h): idx, nodeIdx, endOfNode
// and the reference box (min, max) per reference, in list order.
void aeref_get_refs_full(void* h, uint32_t* idx, uint32_t* node_idx, uint8_t* end_of_node, float* aabb) {
    auto& refs = static_cast<Volume::BVH*>(h)->refs;
    for (size_t i = 0; i < refs.size(); i++) {
        idx[i] = refs[i].idx;
        node_idx[i] = refs[i].nodeIdx;
        end_of_node[i] = refs[i].endOfNode ? 1 : 0;
        const float f[6] = { refs[i].aabb.min.x, refs[i].aabb.min.y, refs[i].aabb.min.z,
                             refs[i].aabb.max.x, refs[i].aabb.max.y, refs[i].aabb.max.z };
        std::memcpy(aabb + i * 6, f, sizeof(f));
    }
}

// BVH::aabbs (min, max per entry), in list order.
uint32_t aeref_aabbs_count(void* h) { return uint32_t(static_cast<Volume::BVH*>(h)->aabbs.size()); }
void aeref_get_aabbs(void* h, float* out) {
    auto& a = static_cast<Volume::BVH*>(h)->aabbs;
    for (size_t i = 0; i < a.size(); i++) {
        const float f[6] = { a[i].min.x, a[i].min.y, a[i].min.z, a[i].max.x, a[i].max.y, a[i].max.z };
        std::memcpy(out + i * 6, f, sizeof(f));
    }
}

// Closest-hit host query over a batch of rays on `threads` std::threads.
// rays: n * 8 floats (origin.xyz, dir.xyz, tMin, tMax).
// Outputs per ray: orig_idx = data[closestPtr].idx, or -1 when the hit test
// intersection.x < original tMax fails (the reference's returned bool compares
// against the mutated ray.tMax, BVH.cpp:141/:172, so it is reported apart in
// ret_bool); tuv = (t, u, v) from the reference (u weights v1, v weights v2).
void aeref_closest(void* h, const float* rays, uint32_t n, int threads,
                   int32_t* orig_idx, float* tuv, uint8_t* ret_bool) {
    auto* bvh = static_cast<Volume::BVH*>(h);
    if (threads < 1) threads = 1;
    const size_t stackSize = bvh->nodes.size() + 64;
    auto work = [&](uint32_t begin, uint32_t end) {
        std::vector<std::pair<int32_t, float>> stack(stackSize);
        for (uint32_t i = begin; i < end; i++) {
            const float* r = rays + size_t(i) * 8;
            Volume::Ray ray(vec3(r[0], r[1], r[2]), vec3(r[3], r[4], r[5]), r[6], r[7]);
            Volume::BVHTriangle closest;
            glm::vec3 inter(0.0f);
            bool b = bvh->GetIntersection(stack, ray, closest, inter);
            bool hit = inter.x < r[7];
            orig_idx[i] = hit ? int32_t(closest.idx) : -1;
            tuv[size_t(i) * 3 + 0] = inter.x;
            tuv[size_t(i) * 3 + 1] = inter.y;
            tuv[size_t(i) * 3 + 2] = inter.z;
            if (ret_bool) ret_bool[i] = b ? 1 : 0;
        }
    };
    std::vector<std::thread> pool;
    uint32_t chunk = (n + uint32_t(threads) - 1) / uint32_t(threads);
    for (int t = 0; t < threads; t++) {
        uint32_t b = uint32_t(t) * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back(work, b, e);
    }
    for (auto& t : pool) t.join();
}

// Any-hit host query (BVH.cpp:176); out[i] = 1 when occluded.
void aeref_any(void* h, const float* rays, uint32_t n, int threads, uint8_t* out) {
    auto* bvh = static_cast<Volume::BVH*>(h);
    if (threads < 1) threads = 1;
    const size_t stackSize = bvh->nodes.size() + 64;
    auto work = [&](uint32_t begin, uint32_t end) {
        std::vector<std::pair<int32_t, float>> stack(stackSize);
        for (uint32_t i = begin; i < end; i++) {
            const float* r = rays + size_t(i) * 8;
            Volume::Ray ray(vec3(r[0], r[1], r[2]), vec3(r[3], r[4], r[5]), r[6], r[7]);
            out[i] = bvh->GetIntersectionAny(stack, ray) ? 1 : 0;
        }
    };
    std::vector<std::thread> pool;
    uint32_t chunk = (n + uint32_t(threads) - 1) / uint32_t(threads);
    for (int t = 0; t < threads; t++) {
        uint32_t b = uint32_t(t) * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back(work, b, e);
    }
    for (auto& t : pool) t.join();
}

}  // extern "C"
