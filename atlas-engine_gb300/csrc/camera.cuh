// Pinhole camera rays of the engine's ray-gen pass (data/shader/pathtracer/
// rayGen.csh:25-91, PathTracingRenderer.cpp:157-160): dir = normalize(origin +
// right*u + bottom*v - location), u,v = (pixel + jitter) / resolution, in
// rayGen.csh's queue order (8 x 8 work groups, then the partial groups;
// :53-80); ray.ID = pixel index.  Arithmetic is explicitly rounded in a fixed
// order, so a host can regenerate the same rays bit for bit.  Shared by the
// ray-generation kernel, the traversal kernel's camera variant (rays made
// where they are traced) and the bounce spawn.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace atlas::rt::dev {

struct CameraParams {
    float lx, ly, lz;       // location
    float ox, oy, oz;       // top-left corner of the image plane
    float rx, ry, rz;       // right span
    float bx, by, bz;       // bottom span
    uint32_t width, height;
    float jx, jy;           // sub-pixel jitter
};

// Pixel index (within a w x h tile) of queue slot i, in rayGen.csh's order
// (:57-80): the complete 8 x 8 work groups first, row-major, each row-major
// inside; then the columns of the partial groups on the right (w % 8 wide,
// as tall as the complete groups), row-major; then the partial rows at the
// bottom (h % 8 tall, the full width), column-major.
__device__ __forceinline__ uint32_t slot_to_pixel(uint32_t i, uint32_t w, uint32_t h) {
    const uint32_t px = w >> 3, py = h >> 3, ox = w & 7u, oy = h & 7u;
    const uint32_t a = px * py * 64u, b = a + ox * py * 8u;
    uint32_t x, y;
    if (i < a) {
        const uint32_t tile = i >> 6, local = i & 63u;
        x = (tile % px) * 8u + (local & 7u);
        y = (tile / px) * 8u + (local >> 3);
    } else if (i < b) {
        const uint32_t j = i - a;
        x = px * 8u + j % ox;
        y = j / ox;
    } else {
        const uint32_t j = i - b;
        x = j / oy;
        y = py * 8u + j % oy;
    }
    return y * w + x;
}

// The camera ray of queue slot i: origin (the pixel index's bits in w) and
// direction, as raygen_kernel writes them.
__device__ __forceinline__ void camera_ray(const CameraParams& c, uint32_t i, float4& o, float4& d) {
    const uint32_t pix = slot_to_pixel(i, c.width, c.height);
    const float px = float(pix % c.width), py = float(pix / c.width);
    const float u = __fdiv_rn(__fadd_rn(px, c.jx), float(c.width));
    const float v = __fdiv_rn(__fadd_rn(py, c.jy), float(c.height));
    const float qx = __fsub_rn(__fadd_rn(__fadd_rn(c.ox, __fmul_rn(c.rx, u)), __fmul_rn(c.bx, v)), c.lx);
    const float qy = __fsub_rn(__fadd_rn(__fadd_rn(c.oy, __fmul_rn(c.ry, u)), __fmul_rn(c.by, v)), c.ly);
    const float qz = __fsub_rn(__fadd_rn(__fadd_rn(c.oz, __fmul_rn(c.rz, u)), __fmul_rn(c.bz, v)), c.lz);
    const float len2 = __fadd_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy)), __fmul_rn(qz, qz));
    const float inv = __frcp_rn(__fsqrt_rn(len2));
    o = make_float4(c.lx, c.ly, c.lz, __int_as_float(int32_t(pix)));
    d = make_float4(__fmul_rn(qx, inv), __fmul_rn(qy, inv), __fmul_rn(qz, inv), 0.0f);
}

}  // namespace atlas::rt::dev
