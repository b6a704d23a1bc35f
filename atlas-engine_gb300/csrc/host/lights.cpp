// The engine's light list for next-event estimation, built on the host the
// way it builds it before every path-tracing dispatch:
//
//   ae_lights_from_mesh     RayTracingWorld::BuildTriangleLightsForMesh
//                           (src/engine/raytracing/RayTracingWorld.cpp:322-376)
//   ae_lights_instance      RayTracingWorld::UpdateTriangleLights (:378-407)
//   ae_light_directional    the directional branch of RayTracingHelper::UpdateLights
//                           (src/engine/renderer/helper/RayTracingHelper.cpp:440-474)
//   ae_lights_normalize     UpdateLights' weight floor and normalisation (:481-499)
//   ae_lights_select        DispatchAndHit's light selection (:72-105) with
//                           Common::Piecewise1D (src/engine/common/Piecewise.cpp:11-78)
//
// Arithmetic follows the reference operation by operation in float32
// (glm's vec3 dot as (x*a + y*b) + z*c, distance as sqrt of that dot), with
// this file compiled without contraction.  pow is the C library's powf, as
// glm::pow calls it.
#include "atlas_rt.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct F3 {
    float x, y, z;
};

F3 Load3(const float* p) { return F3{ p[0], p[1], p[2] }; }
F3 Add(F3 a, F3 b) { return F3{ a.x + b.x, a.y + b.y, a.z + b.z }; }
F3 Sub(F3 a, F3 b) { return F3{ a.x - b.x, a.y - b.y, a.z - b.z }; }
F3 Div(F3 a, float s) { return F3{ a.x / s, a.y / s, a.z / s }; }
float Dot(F3 a, F3 b) {
    const float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (x + y) + z;
}
float Distance(F3 a, F3 b) {
    const F3 d = Sub(a, b);
    return std::sqrt(Dot(d, d));
}
F3 SrgbToLinear(F3 c) {  // ColorConverter::ConvertSRGBToLinear, common/ColorConverter.h:18-23
    return F3{ std::pow(c.x, 2.2f), std::pow(c.y, 2.2f), std::pow(c.z, 2.2f) };
}
int32_t Bits(float f) {
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
}
float AsFloat(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
// Common::Packing::UnpackSignedVector3x10_1x2 (common/Packing.cpp:37-48), xyz
F3 Unpack10(int32_t packed) {
    auto c = [](int32_t v) { return float(v & 1023) / 1023.0f * 2.0f - 1.0f; };
    return F3{ c(packed >> 0), c(packed >> 10), c(packed >> 20) };
}
void Set4(float* dst, F3 v, float w) {
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
    dst[3] = w;
}

constexpr uint32_t kTriangleLight = 1u;     // RayTracingHelper.cpp:10
constexpr uint32_t kDirectionalLight = 0u;  // RayTracingHelper.cpp:9

}  // namespace

extern "C" {

ae_rt_status ae_lights_from_mesh(const ae_triangle* shading, uint32_t n_tris, const float* emissive_srgb,
                                 const float* emissive_intensity, uint32_t n_materials, ae_light* out,
                                 uint32_t capacity, uint32_t* n_out) {
    if (!n_out || (n_tris && !shading) || (n_materials && (!emissive_srgb || !emissive_intensity)))
        return AE_RT_INVALID_ARG;
    if (n_tris >= (1u << 28)) return AE_RT_INVALID_ARG;  // the index shares data.x with the type
    uint32_t count = 0;
    for (uint32_t i = 0; i < n_tris; i++) {
        const ae_triangle& t = shading[i];
        const int32_t idx = Bits(t.d0[3]);
        if (idx < 0 || uint32_t(idx) >= n_materials) return AE_RT_INVALID_ARG;
        const F3 radiance = SrgbToLinear(Load3(emissive_srgb + size_t(idx) * 3));
        const float brightness = Dot(radiance, F3{ 0.3333f, 0.3333f, 0.3333f });
        if (!(brightness > 0.0f)) continue;
        if (count < capacity && out) {
            const F3 v0 = Load3(t.v0), v1 = Load3(t.v1), v2 = Load3(t.v2);
            const F3 n0 = Unpack10(Bits(t.v0[3])), n1 = Unpack10(Bits(t.v1[3])), n2 = Unpack10(Bits(t.v2[3]));
            const F3 P = Div(Add(Add(v0, v1), v2), 3.0f);
            const F3 N = Div(Add(Add(n0, n1), n2), 3.0f);
            const float a = Distance(v1, v0), b = Distance(v2, v0), c = Distance(v1, v2);
            const float p = 0.5f * ((a + b) + c);
            const float area = std::sqrt(((p * (p - a)) * (p - b)) * (p - c));
            const float weight = area * brightness;
            // the colour converts the already converted radiance once more (RayTracingWorld.cpp:368)
            const F3 lin = SrgbToLinear(radiance);
            const float intensity = emissive_intensity[idx];
            ae_light& L = out[count];
            Set4(L.P, P, 1.0f);
            Set4(L.N, N, 0.0f);
            Set4(L.color, F3{ lin.x * intensity, lin.y * intensity, lin.z * intensity }, 0.0f);
            L.data[0] = AsFloat((kTriangleLight << 28) | i);
            L.data[1] = weight;
            L.data[2] = area;
            L.data[3] = 0.0f;
        }
        count++;
    }
    *n_out = count;
    return count > capacity && out ? AE_RT_OUT_OF_MEMORY : AE_RT_OK;
}

ae_rt_status ae_lights_instance(const ae_light* mesh_lights, uint32_t n, const float* model, int32_t instance,
                                ae_light* out) {
    if ((n && (!mesh_lights || !out)) || !model) return AE_RT_INVALID_ARG;
    for (uint32_t k = 0; k < n; k++) {
        const ae_light& L = mesh_lights[k];
        ae_light r = L;
        // matrix * vec4 (P with w = 1, N with w = 0): row r of the row-major model
        // matrix against (x, y, z, w), summed as glm's mat4 * vec4 sums the
        // columns, pairwise: (m0 x + m1 y) + (m2 z + m3 w)
        for (int row = 0; row < 3; row++) {
            const float* m = model + row * 4;
            r.P[row] = (m[0] * L.P[0] + m[1] * L.P[1]) + (m[2] * L.P[2] + m[3] * 1.0f);
            r.N[row] = (m[0] * L.N[0] + m[1] * L.N[1]) + (m[2] * L.N[2] + m[3] * 0.0f);
        }
        std::memcpy(&r.data[3], &instance, 4);
        out[k] = r;
    }
    return AE_RT_OK;
}

ae_rt_status ae_light_directional(const float color_srgb[3], float intensity, const float direction[3],
                                  uint32_t index, ae_light* out) {
    if (!color_srgb || !direction || !out || index >= (1u << 28)) return AE_RT_INVALID_ARG;
    const F3 lin = SrgbToLinear(Load3(color_srgb));
    const F3 radiance{ lin.x * intensity, lin.y * intensity, lin.z * intensity };
    const float brightness = Dot(radiance, F3{ 0.3333f, 0.3333f, 0.3333f });
    std::memset(out, 0, sizeof(*out));
    Set4(out->P, F3{ 0, 0, 0 }, 1.0f);
    Set4(out->N, Load3(direction), 0.0f);
    Set4(out->color, radiance, 0.0f);
    out->data[0] = AsFloat((kDirectionalLight << 28) | index);
    out->data[1] = brightness;
    return AE_RT_OK;
}

ae_rt_status ae_lights_normalize(ae_light* lights, uint32_t n) {
    if (n && !lights) return AE_RT_INVALID_ARG;
    float max_w = 0.0f;
    for (uint32_t k = 0; k < n; k++) max_w = lights[k].data[1] > max_w ? lights[k].data[1] : max_w;
    const float min_w = 0.005f * max_w;
    float total = 0.0f;
    for (uint32_t k = 0; k < n; k++) {
        lights[k].data[1] = lights[k].data[1] > min_w ? lights[k].data[1] : min_w;
        total += lights[k].data[1];
    }
    for (uint32_t k = 0; k < n; k++) lights[k].data[1] /= total;
    return AE_RT_OK;
}

ae_rt_status ae_lights_select(const ae_light* lights, uint32_t n, uint32_t capacity, const float* uniforms,
                              ae_light* out, uint32_t* n_out) {
    if (!n_out || (n && (!lights || !out)) || capacity == 0) return AE_RT_INVALID_ARG;
    if (n <= capacity) {
        for (uint32_t k = 0; k < n; k++) {
            out[k] = lights[k];
            out[k].data[1] = 1.0f;
        }
        *n_out = n;
        return AE_RT_OK;
    }
    if (!uniforms) return AE_RT_INVALID_ARG;
    // Piecewise1D(weights): cdf[k] = running sum of weight / count, divided by the total
    std::vector<float> cdf(size_t(n) + 1);
    float sum = 0.0f;
    for (uint32_t k = 0; k < n; k++) {
        cdf[k] = sum;
        sum += lights[k].data[1] / float(n);
    }
    cdf[n] = sum;
    if (!(sum > 0.0f)) return AE_RT_INVALID_ARG;
    for (float& c : cdf) c /= sum;
    for (uint32_t s = 0; s < capacity; s++) {
        const float x = uniforms[s];
        // Piecewise1D::BinarySearch: the first interval [cdf[m], cdf[m + 1]] the search meets holding x
        int l = 0, r = int(n), found = -1;
        while (l <= r) {
            const int m = l + (r - l) / 2;
            const int k = m + 1 > int(n) ? m : m + 1;
            if (cdf[size_t(m)] <= x && x <= cdf[size_t(k)]) {
                found = m;
                break;
            }
            if (cdf[size_t(m)] < x) l = m + 1;
            else r = m - 1;
        }
        // x in [0, 1) always lands in an interval; m == n (a zero-width last
        // interval) names no light, so take the last one
        if (found < 0 || found >= int(n)) found = int(n) - 1;
        out[s] = lights[found];
        out[s].data[1] = lights[found].data[1] * float(capacity);
    }
    *n_out = capacity;
    return AE_RT_OK;
}

}  // extern "C"
