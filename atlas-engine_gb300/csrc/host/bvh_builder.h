// Host BVH builder emitting Atlas Engine's flattened BVH layout.
//
// Behaviour follows Volume::BVH (src/engine/volume/BVH.cpp:14-100, :249-870):
// binned SAH with 256 / (depth + 1) bins (at least 16), SBVH-style spatial
// splits considered at the root only, 1-reference leaves below the root,
// median-split fallback, children flattened in pre-order with the child of
// larger surface area on the left.  For the same input it produces the same
// nodes, the same triangle order and the same leaf flags as the reference,
// byte for byte (this is checked against the compiled reference).  Sub-trees
// down to depth 6 are built on worker threads; the result does not depend on
// the thread count.
#pragma once

#include <cstdint>
#include <vector>

namespace atlas::rt {

struct Box {
    float lo[3];
    float hi[3];
};

struct BuiltNode {           // identical to GPUBVHNode (RTStructures.h:95-103)
    Box left;
    Box right;
    int32_t leftPtr = 0;
    int32_t rightPtr = 0;
    int32_t padding0 = 0;
    int32_t padding1 = 0;
};
static_assert(sizeof(BuiltNode) == 64, "GPUBVHNode is 64 bytes");

struct BuiltBVH {
    std::vector<BuiltNode> nodes;
    std::vector<uint32_t> order;       // order[i] = input index of flattened primitive i
    std::vector<uint8_t> endOfNode;    // 1 on the last primitive of each leaf
};

struct TriangleInput {
    const float* verts = nullptr;      // n * 9 floats: v0, v1, v2
    const float* boxes = nullptr;      // optional n * 6 floats (min, max); derived from verts if null
    uint32_t count = 0;
};

// Triangle BVH (BVH::BVH(aabbs, data, parallel), BVH.cpp:14).
BuiltBVH BuildTriangleBVH(const TriangleInput& in, bool parallel);

// AABB-only BVH used for the top level (BVH::BVH(aabbs, parallel), BVH.cpp:58).
BuiltBVH BuildBoxBVH(const float* boxes, uint32_t count, bool parallel);

// The triangle bounding box as MeshData::BuildBVH forms it (MeshData.cpp:143-146).
Box TriangleBox(const float* v9);

}  // namespace atlas::rt
