// C ABI of the host BVH builder and the GPU-layout packing (include/atlas_rt.h).
#include "atlas_rt.h"
#include "bvh_builder.h"

#include <cstring>
#include <new>

struct ae_bvh {
    atlas::rt::BuiltBVH built;
    uint32_t primitives = 0;
};

extern "C" {

ae_rt_status ae_bvh_build_triangles(const float* verts, const float* aabbs, uint32_t n, int parallel,
                                    ae_bvh** out) {
    if (!out || (n && !verts)) return AE_RT_INVALID_ARG;
    *out = nullptr;
    try {
        auto* b = new ae_bvh;
        atlas::rt::TriangleInput in;
        in.verts = verts;
        in.boxes = aabbs;
        in.count = n;
        b->built = atlas::rt::BuildTriangleBVH(in, parallel != 0);
        b->primitives = uint32_t(b->built.order.size());
        *out = b;
        return AE_RT_OK;
    } catch (const std::bad_alloc&) {
        return AE_RT_OUT_OF_MEMORY;
    } catch (...) {
        return AE_RT_INVALID_ARG;
    }
}

ae_rt_status ae_bvh_build_aabbs(const float* aabbs, uint32_t n, int parallel, ae_bvh** out) {
    if (!out || (n && !aabbs)) return AE_RT_INVALID_ARG;
    *out = nullptr;
    try {
        auto* b = new ae_bvh;
        b->built = atlas::rt::BuildBoxBVH(aabbs, n, parallel != 0);
        b->primitives = uint32_t(b->built.order.size());
        *out = b;
        return AE_RT_OK;
    } catch (const std::bad_alloc&) {
        return AE_RT_OUT_OF_MEMORY;
    } catch (...) {
        return AE_RT_INVALID_ARG;
    }
}

void ae_bvh_destroy(ae_bvh* bvh) { delete bvh; }

uint32_t ae_bvh_node_count(const ae_bvh* bvh) { return bvh ? uint32_t(bvh->built.nodes.size()) : 0; }

uint32_t ae_bvh_primitive_count(const ae_bvh* bvh) { return bvh ? bvh->primitives : 0; }

ae_rt_status ae_bvh_get_nodes(const ae_bvh* bvh, ae_bvh_node* out) {
    if (!bvh || (!out && !bvh->built.nodes.empty())) return AE_RT_INVALID_ARG;
    static_assert(sizeof(ae_bvh_node) == sizeof(atlas::rt::BuiltNode), "node layout");
    if (!bvh->built.nodes.empty())
        std::memcpy(out, bvh->built.nodes.data(), bvh->built.nodes.size() * sizeof(ae_bvh_node));
    return AE_RT_OK;
}

ae_rt_status ae_bvh_get_order(const ae_bvh* bvh, uint32_t* order, uint8_t* end_of_node) {
    if (!bvh) return AE_RT_INVALID_ARG;
    const size_t n = bvh->built.order.size();
    if (order && n) std::memcpy(order, bvh->built.order.data(), n * sizeof(uint32_t));
    if (end_of_node && n) std::memcpy(end_of_node, bvh->built.endOfNode.data(), n);
    return AE_RT_OK;
}

// MeshData::BuildBVH's GPUBVHTriangle packing (MeshData.cpp:241-248).
ae_rt_status ae_bvh_pack_triangles(const ae_bvh* bvh, const float* verts, const int32_t* material,
                                   const float* opacity, ae_bvh_triangle* out) {
    if (!bvh || !verts || (!out && bvh->primitives)) return AE_RT_INVALID_ARG;
    for (uint32_t i = 0; i < bvh->primitives; i++) {
        const uint32_t src = bvh->built.order[i];
        const float* t = verts + size_t(src) * 9;
        ae_bvh_triangle& o = out[i];
        o.v0[0] = t[0]; o.v0[1] = t[1]; o.v0[2] = t[2];
        o.v0[3] = bvh->built.endOfNode[i] ? 1.0f : -1.0f;
        o.v1[0] = t[3]; o.v1[1] = t[4]; o.v1[2] = t[5];
        int32_t m = material ? material[src] : 0;
        std::memcpy(&o.v1[3], &m, 4);
        o.v2[0] = t[6]; o.v2[1] = t[7]; o.v2[2] = t[8];
        o.v2[3] = opacity ? opacity[src] : 1.0f;
    }
    return AE_RT_OK;
}

}  // extern "C"
