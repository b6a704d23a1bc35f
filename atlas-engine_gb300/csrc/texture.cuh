// Texture lookups of the software traversal: the engine's bindless sampler
// (linear filter, repeat addressing; MainRenderer.cpp:922-929) at level 0
// (texture.hsh:18-25), written out in FP32 with one rounding per operation so
// that a CPU restatement reproduces every sample bit for bit.  Hardware
// filtering is not used: its interpolation weights have 8 fractional bits.
//
// Layout: every texture's mip chain lies tightly packed (row pitch = width x
// texel bytes) in one pool, level after level, each level starting on a
// 16-byte boundary; TexDesc gives level 0's offset, size and format.  Level
// k + 1 is the 2 x 2 box filter of level k (indices clamped at odd edges;
// built on the host when the textures are set).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

namespace atlas::rt::dev {

struct TexDesc {
    unsigned long long offset;   // bytes into the pool (level 0)
    uint32_t width, height;      // level 0
    uint32_t format;             // AE_TEX_*
    uint32_t row_pitch;          // bytes (level 0)
    uint32_t levels;             // mip levels stored after level 0, down to 1 x 1
    uint32_t pad;
};
static_assert(sizeof(TexDesc) == 32, "TexDesc is 32 bytes");

struct TexTable {
    const uint8_t* pool;
    const TexDesc* desc;
    uint32_t n;
};

// The first channel of texel (x, y).
__device__ __forceinline__ float texel_r(const TexTable& tt, const TexDesc& t, uint32_t x, uint32_t y) {
    const uint8_t* row = tt.pool + t.offset + size_t(y) * t.row_pitch;
    if (t.format == 0u) return __fdiv_rn(float(__ldg(row + x)), 255.0f);
    if (t.format == 1u) return __fdiv_rn(float(__ldg(row + size_t(x) * 4u)), 255.0f);
    return __ldg(reinterpret_cast<const float*>(row) + x);
}

// One axis of the bilinear footprint: texels i0 and i1 = i0 + 1, both
// wrapped into [0, n) (repeat addressing), and the weight a of i1.
__device__ __forceinline__ void tex_axis(float s, uint32_t n, uint32_t& i0, uint32_t& i1, float& a) {
    float x = __fsub_rn(__fmul_rn(s, float(n)), 0.5f);
    if (!(fabsf(x) < 9.0e18f)) x = 0.0f;   // non-finite (or beyond int64): texel 0 alone
    const float fx = floorf(x);
    a = __fsub_rn(x, fx);
    long long i = static_cast<long long>(fx) % static_cast<long long>(n);
    if (i < 0) i += n;
    i0 = uint32_t(i);
    i1 = i0 + 1u == n ? 0u : i0 + 1u;
}

// The descriptor of mip level `level` (clamped to the chain) of texture t.
__device__ __forceinline__ TexDesc tex_level(TexDesc t, uint32_t level) {
    const uint32_t texel = t.format == 0u ? 1u : 4u;
    const uint32_t last = t.levels ? t.levels - 1u : 0u;
    for (uint32_t k = 0; k < level && k < last; k++) {
        t.offset += ((unsigned long long)(t.width * texel) * t.height + 15ull) & ~15ull;
        t.width = t.width > 1u ? t.width >> 1 : 1u;
        t.height = t.height > 1u ? t.height >> 1 : 1u;
        t.row_pitch = t.width * texel;
    }
    return t;
}

// textureLod(sampler2D(bindlessTextures[id], bindlessSampler), uv, level).r
// for an integer level (one mip level, no blending between levels); 1.0
// for a negative or out-of-range id.
__device__ __forceinline__ float sample_r_bilinear(const TexTable& tt, int32_t id, float u, float v,
                                                   uint32_t level = 0) {
    if (id < 0 || uint32_t(id) >= tt.n) return 1.0f;
    const TexDesc t = tex_level(tt.desc[id], level);
    uint32_t x0, x1, y0, y1;
    float a, b;
    tex_axis(u, t.width, x0, x1, a);
    tex_axis(v, t.height, y0, y1, b);
    const float c00 = texel_r(tt, t, x0, y0), c10 = texel_r(tt, t, x1, y0);
    const float c01 = texel_r(tt, t, x0, y1), c11 = texel_r(tt, t, x1, y1);
    const float ia = __fsub_rn(1.0f, a), ib = __fsub_rn(1.0f, b);
    float r = __fmul_rn(__fmul_rn(ia, ib), c00);
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(a, ib), c10));
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(ia, b), c01));
    return __fadd_rn(r, __fmul_rn(__fmul_rn(a, b), c11));
}

// All four channels of texel (x, y) as the sampler returns them: R8 gives
// (r, 0, 0, 1), RGBA8 (r, g, b, a), R32F (r, 0, 0, 1).
__device__ __forceinline__ float4 texel_rgba(const TexTable& tt, const TexDesc& t, uint32_t x, uint32_t y) {
    const uint8_t* row = tt.pool + t.offset + size_t(y) * t.row_pitch;
    if (t.format == 0u) return make_float4(__fdiv_rn(float(__ldg(row + x)), 255.0f), 0.0f, 0.0f, 1.0f);
    if (t.format == 1u) {
        const uchar4 c = __ldg(reinterpret_cast<const uchar4*>(row) + x);
        return make_float4(__fdiv_rn(float(c.x), 255.0f), __fdiv_rn(float(c.y), 255.0f),
                           __fdiv_rn(float(c.z), 255.0f), __fdiv_rn(float(c.w), 255.0f));
    }
    return make_float4(__ldg(reinterpret_cast<const float*>(row) + x), 0.0f, 0.0f, 1.0f);
}

__device__ __forceinline__ float bilerp(float ia, float ib, float a, float b, float c00, float c10, float c01,
                                        float c11) {
    float r = __fmul_rn(__fmul_rn(ia, ib), c00);
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(a, ib), c10));
    r = __fadd_rn(r, __fmul_rn(__fmul_rn(ia, b), c01));
    return __fadd_rn(r, __fmul_rn(__fmul_rn(a, b), c11));
}

// textureLod(sampler2D(bindlessTextures[id], bindlessSampler), uv, 0) with
// every channel filtered as sample_r_bilinear filters the first; (1, 1, 1, 1)
// for a negative or out-of-range id (SampleBaseColorBilinear and friends,
// texture.hsh:9-60).
__device__ __forceinline__ float4 sample_rgba_bilinear(const TexTable& tt, int32_t id, float u, float v,
                                                     uint32_t level = 0) {
    if (id < 0 || uint32_t(id) >= tt.n) return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    const TexDesc t = tex_level(tt.desc[id], level);
    uint32_t x0, x1, y0, y1;
    float a, b;
    tex_axis(u, t.width, x0, x1, a);
    tex_axis(v, t.height, y0, y1, b);
    const float4 c00 = texel_rgba(tt, t, x0, y0), c10 = texel_rgba(tt, t, x1, y0);
    const float4 c01 = texel_rgba(tt, t, x0, y1), c11 = texel_rgba(tt, t, x1, y1);
    const float ia = __fsub_rn(1.0f, a), ib = __fsub_rn(1.0f, b);
    return make_float4(bilerp(ia, ib, a, b, c00.x, c10.x, c01.x, c11.x), bilerp(ia, ib, a, b, c00.y, c10.y, c01.y, c11.y),
                       bilerp(ia, ib, a, b, c00.z, c10.z, c01.z, c11.z), bilerp(ia, ib, a, b, c00.w, c10.w, c01.w, c11.w));
}

__device__ __forceinline__ float2 unpack_half2(float bits) {
    const uint32_t u = __float_as_uint(bits);
    return make_float2(__half2float(__ushort_as_half(uint16_t(u & 0xFFFFu))),
                       __half2float(__ushort_as_half(uint16_t(u >> 16))));
}

// GetOpacity (surface.hsh:147-159) for the shading triangle's d0 (half2 UVs
// x3 + material index) at barycentrics (s, t) = the triangle test's (u, v);
// materials are GPUMaterial (23 words: opacity at 7, invertUVs at 13,
// opacityTexture at 18).  The interpolated vertex alpha of the shader is
// computed there but unused, so it is not computed here.
__device__ __forceinline__ float get_opacity(const float* materials, uint32_t n_materials, const TexTable& tt,
                                             float4 d0, int32_t mat_offset, float s, float t) {
    const int32_t mi = __float_as_int(d0.w) + mat_offset;
    if (!materials || mi < 0 || uint32_t(mi) >= n_materials) return 1.0f;
    const float* m = materials + size_t(mi) * 23;
    const float r = __fsub_rn(__fsub_rn(1.0f, s), t);
    const float2 uv0 = unpack_half2(d0.x), uv1 = unpack_half2(d0.y), uv2 = unpack_half2(d0.z);
    const float tu = __fadd_rn(__fadd_rn(__fmul_rn(r, uv0.x), __fmul_rn(s, uv1.x)), __fmul_rn(t, uv2.x));
    float tv = __fadd_rn(__fadd_rn(__fmul_rn(r, uv0.y), __fmul_rn(s, uv1.y)), __fmul_rn(t, uv2.y));
    if (__float_as_int(m[13]) > 0) tv = __fsub_rn(1.0f, tv);
    return __fmul_rn(sample_r_bilinear(tt, __float_as_int(m[18]), tu, tv), m[7]);
}

}  // namespace atlas::rt::dev
