// C ABI of the host BVH builder and the GPU-layout packing (include/atlas_rt.h).
#include "atlas_rt.h"
#include "bvh_builder.h"

#include <cmath>
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

namespace {

// Common::Packing::PackSignedVector3x10_1x2 (src/engine/common/Packing.cpp:24-35)
int32_t PackSigned10(float x, float y, float z, float w) {
    int32_t p = 0;
    p |= int32_t((x * 0.5f + 0.5f) * 1023.0f) << 0;
    p |= int32_t((y * 0.5f + 0.5f) * 1023.0f) << 10;
    p |= int32_t((z * 0.5f + 0.5f) * 1023.0f) << 20;
    p |= int32_t((w * 0.5f + 0.5f) * 2.0f) << 30;
    return p;
}

float Bits(int32_t v) {
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

// IEEE binary16 bits of f, rounded to nearest even (glm::packHalf2x16):
// overflow to infinity, NaN payloads keep their top mantissa bits.
uint16_t HalfBits(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) {
        const uint32_t m = (ax & 0x7FFFFFu) >> 13;
        return uint16_t(sign | 0x7C00u | (ax > 0x7F800000u ? (m ? m : 1u) : 0u));
    }
    if (ax >= 0x477FF000u) return uint16_t(sign | 0x7C00u);   // rounds to 65520 or more
    uint32_t r, rem, halfway;
    if (ax < 0x38800000u) {                                      // half subnormal (or zero)
        if (ax < 0x33000000u) return uint16_t(sign);
        const uint32_t e = ax >> 23, m = (ax & 0x7FFFFFu) | 0x800000u, shift = 126u - e;
        r = m >> shift;
        rem = m & ((1u << shift) - 1u);
        halfway = 1u << (shift - 1u);
    } else {
        r = (ax - 0x38000000u) >> 13;                            // exponent rebiased by -112
        rem = ax & 0x1FFFu;
        halfway = 0x1000u;
    }
    if (rem > halfway || (rem == halfway && (r & 1u))) r++;
    return uint16_t(sign | r);
}

void Normalize3(const float* in, float* out) {
    const float l = std::sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
    const float s = l > 0.0f ? 1.0f / l : 0.0f;
    out[0] = in[0] * s;
    out[1] = in[1] * s;
    out[2] = in[2] * s;
}

// glm::packUnorm4x8: round(clamp(c, 0, 1) * 255) per channel, x lowest
uint32_t PackUnorm4(const float* c) {
    uint32_t out = 0;
    for (int k = 0; k < 4; k++) {
        const float v = std::fmin(std::fmax(c[k], 0.0f), 1.0f);
        out |= uint32_t(std::lround(v * 255.0f)) << (8 * k);
    }
    return out;
}

}  // namespace

// GPUTriangle packing in BVH order (MeshData.cpp:172-239), without texture
// coordinates and vertex colours (UVs 0, colours white, tangent frame from
// the face): normals are normalised and stored 10:10:10:2.
ae_rt_status ae_bvh_pack_shading(const ae_bvh* bvh, const float* verts, const float* normals,
                                 const int32_t* material, const float* opacity, ae_triangle* out) {
    if (!bvh || !verts || (!out && bvh->primitives)) return AE_RT_INVALID_ARG;
    for (uint32_t i = 0; i < bvh->primitives; i++) {
        const uint32_t src = bvh->built.order[i];
        const float* t = verts + size_t(src) * 9;
        float n[3][3];
        if (normals) {
            for (int k = 0; k < 3; k++) Normalize3(normals + size_t(src) * 9 + 3 * k, n[k]);
        } else {
            const float e0[3] = { t[3] - t[0], t[4] - t[1], t[5] - t[2] };
            const float e1[3] = { t[6] - t[0], t[7] - t[1], t[8] - t[2] };
            const float c[3] = { e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0] };
            Normalize3(c, n[0]);
            for (int k = 0; k < 3; k++) n[1][k] = n[2][k] = n[0][k];
        }
        // tangent frame from the face (there are no texture coordinates)
        float e0[3] = { t[3] - t[0], t[4] - t[1], t[5] - t[2] };
        float tan[3], bit[3];
        Normalize3(e0, tan);
        const float* nn = n[0];
        const float b[3] = { nn[1] * tan[2] - nn[2] * tan[1], nn[2] * tan[0] - nn[0] * tan[2], nn[0] * tan[1] - nn[1] * tan[0] };
        Normalize3(b, bit);
        ae_triangle& o = out[i];
        for (int k = 0; k < 3; k++) {
            float* v = k == 0 ? o.v0 : (k == 1 ? o.v1 : o.v2);
            v[0] = t[3 * k]; v[1] = t[3 * k + 1]; v[2] = t[3 * k + 2];
            v[3] = Bits(PackSigned10(n[k][0], n[k][1], n[k][2], 0.0f));
        }
        const int32_t m = material ? material[src] : 0;
        o.d0[0] = 0.0f; o.d0[1] = 0.0f; o.d0[2] = 0.0f; o.d0[3] = Bits(m);
        o.d1[0] = Bits(PackSigned10(tan[0], tan[1], tan[2], 0.0f));
        o.d1[1] = Bits(PackSigned10(bit[0], bit[1], bit[2], 0.0f));
        o.d1[2] = bvh->built.endOfNode[i] ? 1.0f : -1.0f;
        o.d1[3] = 0.0f;
        const int32_t white = int32_t(0xFFFFFFFFu);
        o.d2[0] = Bits(white); o.d2[1] = Bits(white); o.d2[2] = Bits(white);
        o.d2[3] = opacity ? opacity[src] : 1.0f;
    }
    return AE_RT_OK;
}

ae_rt_status ae_bvh_pack_uvs(const ae_bvh* bvh, const float* uvs, ae_triangle* inout) {
    if (!bvh || (bvh->primitives && (!uvs || !inout))) return AE_RT_INVALID_ARG;
    for (uint32_t i = 0; i < bvh->primitives; i++) {
        const float* uv = uvs + size_t(bvh->built.order[i]) * 6;
        for (int k = 0; k < 3; k++) {
            // packHalf2x16: x in the low half, y in the high half
            const uint32_t bits = uint32_t(HalfBits(uv[2 * k])) | (uint32_t(HalfBits(uv[2 * k + 1])) << 16);
            inout[i].d0[k] = Bits(int32_t(bits));
        }
    }
    return AE_RT_OK;
}

ae_rt_status ae_bvh_pack_attributes(const ae_bvh* bvh, const float* verts, const float* normals, const float* uvs,
                                    const float* colors, ae_triangle* inout) {
    if (!bvh || (bvh->primitives && (!verts || !uvs || !inout))) return AE_RT_INVALID_ARG;
    ae_rt_status st = ae_bvh_pack_uvs(bvh, uvs, inout);
    if (st != AE_RT_OK) return st;
    for (uint32_t i = 0; i < bvh->primitives; i++) {
        const uint32_t src = bvh->built.order[i];
        const float* v = verts + size_t(src) * 9;
        const float* uv = uvs + size_t(src) * 6;
        float n[3][3];
        if (normals) {
            for (int k = 0; k < 3; k++) Normalize3(normals + size_t(src) * 9 + 3 * k, n[k]);
        } else {
            const float a[3] = { v[3] - v[0], v[4] - v[1], v[5] - v[2] }, b[3] = { v[6] - v[0], v[7] - v[1], v[8] - v[2] };
            const float c[3] = { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
            Normalize3(c, n[0]);
            for (int k = 0; k < 3; k++) n[1][k] = n[2][k] = n[0][k];
        }
        // MeshData.cpp:176-197: UV-space derivatives of position
        const float e1[3] = { v[3] - v[0], v[4] - v[1], v[5] - v[2] }, e2[3] = { v[6] - v[0], v[7] - v[1], v[8] - v[2] };
        const float du1 = uv[2] - uv[0], dv1 = uv[3] - uv[1], du2 = uv[4] - uv[0], dv2 = uv[5] - uv[1];
        const float r = 1.0f / (du1 * dv2 - du2 * dv1);
        float sdir[3], tdir[3], nsum[3], nn[3];
        for (int k = 0; k < 3; k++) {
            sdir[k] = (dv2 * e1[k] - dv1 * e2[k]) * r;
            tdir[k] = (du1 * e2[k] - du2 * e1[k]) * r;
            nsum[k] = n[0][k] + n[1][k] + n[2][k];
        }
        Normalize3(nsum, nn);
        const float ns = nn[0] * sdir[0] + nn[1] * sdir[1] + nn[2] * sdir[2];
        const float tg0[3] = { sdir[0] - nn[0] * ns, sdir[1] - nn[1] * ns, sdir[2] - nn[2] * ns };
        float tg[3];
        Normalize3(tg0, tg);
        const float cr[3] = { tg[1] * nn[2] - tg[2] * nn[1], tg[2] * nn[0] - tg[0] * nn[2], tg[0] * nn[1] - tg[1] * nn[0] };
        const float hand = (cr[0] * tdir[0] + cr[1] * tdir[1] + cr[2] * tdir[2]) < 0.0f ? 1.0f : -1.0f;
        float bt[3];
        Normalize3(cr, bt);
        for (int k = 0; k < 3; k++) bt[k] *= hand;
        inout[i].d1[0] = Bits(PackSigned10(tg[0], tg[1], tg[2], 0.0f));
        inout[i].d1[1] = Bits(PackSigned10(bt[0], bt[1], bt[2], 0.0f));
        if (colors) {
            for (int k = 0; k < 3; k++) inout[i].d2[k] = Bits(int32_t(PackUnorm4(colors + size_t(src) * 12 + 4 * k)));
        }
    }
    return AE_RT_OK;
}

}  // extern "C"
