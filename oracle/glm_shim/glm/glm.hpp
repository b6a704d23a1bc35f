// Minimal stand-in for the glm vector/matrix library, covering only what the
// reference's BVH builder, ray queries, AABB and job system use.
//
// TEST INFRASTRUCTURE ONLY: this header exists so the reference's own sources
// (volume/BVH.cpp, volume/Ray.cpp, volume/AABB.cpp, jobsystem/*.cpp) compile
// unmodified into the checker library under oracle/_ref/.  The reference pins
// glm 0.9.8.0 (vcpkg.json:46-48), which is not vendored and not installed.
//
// Written from the documented GLSL / glm semantics, not from glm's source:
//   min(x, y)   = (y < x) ? y : x            (GLSL spec 8.3)
//   max(x, y)   = (x < y) ? y : x
//   clamp(x,a,b)= min(max(x, a), b)
//   mix(x,y,a)  = x * (1 - a) + y * a
//   dot(a, b)   = (a.x*b.x + a.y*b.y) + a.z*b.z   (left-to-right sum)
//   cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   normalize(v)= v * (1 / sqrt(dot(v, v)))
// Rounding at this boundary (association of dot, NaN behaviour of min/max,
// FMA contraction) is therefore a property of this shim; everything here is
// compiled with -ffp-contract=off so x86-64 and aarch64 agree bit for bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstddef>

namespace glm {

struct vec4;

struct vec2 {
    float x = 0.0f, y = 0.0f;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
};

struct vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec4& v);  // drops w, like glm's converting constructor
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct vec4 {
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct ivec2 { int32_t x = 0, y = 0; };
struct ivec3 { int32_t x = 0, y = 0, z = 0; };
struct ivec4 { int32_t x = 0, y = 0, z = 0, w = 0; };

// vec3 arithmetic (component-wise, IEEE single precision)
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }

inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, const vec4& a) { return a * s; }

// Scalar min/max/clamp with the GLSL definition (the second operand wins only
// when it is strictly smaller / larger).
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int32_t min(int32_t x, int32_t y) { return (y < x) ? y : x; }
inline int32_t max(int32_t x, int32_t y) { return (x < y) ? y : x; }

inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 min(const vec3& a, float b) { return vec3(min(a.x, b), min(a.y, b), min(a.z, b)); }
inline vec3 max(const vec3& a, float b) { return vec3(max(a.x, b), max(a.y, b), max(a.z, b)); }
inline vec3 clamp(const vec3& x, const vec3& lo, const vec3& hi) { return min(max(x, lo), hi); }
inline vec3 clamp(const vec3& x, float lo, float hi) { return min(max(x, lo), hi); }

inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }

inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec4& a, const vec4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }

inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(b - a); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline float pow(float b, float e) { return std::pow(b, e); }
inline float abs(float x) { return std::fabs(x); }

// Column-major matrices (columns are vectors), as in GLSL.
struct mat3 {
    vec3 c[3];
    mat3() { c[0] = vec3(1, 0, 0); c[1] = vec3(0, 1, 0); c[2] = vec3(0, 0, 1); }
    explicit mat3(float s) { c[0] = vec3(s, 0, 0); c[1] = vec3(0, s, 0); c[2] = vec3(0, 0, s); }
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};

struct mat4 {
    vec4 c[4];
    mat4() { c[0] = vec4(1, 0, 0, 0); c[1] = vec4(0, 1, 0, 0); c[2] = vec4(0, 0, 1, 0); c[3] = vec4(0, 0, 0, 1); }
    explicit mat4(float s) { c[0] = vec4(s, 0, 0, 0); c[1] = vec4(0, s, 0, 0); c[2] = vec4(0, 0, s, 0); c[3] = vec4(0, 0, 0, s); }
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};

// 4 columns x 3 rows and 3 columns x 4 rows; only their names and sizes are
// needed by the compiled sources.
struct mat4x3 { vec3 c[4]; };
struct mat3x4 { vec4 c[3]; };

inline vec4 operator*(const mat4& m, const vec4& v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w;
}

inline float determinant(const mat3& m) {
    // Cofactor expansion along the first column.
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2])
         - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2])
         + m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

struct quat { float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f; };

}  // namespace glm
