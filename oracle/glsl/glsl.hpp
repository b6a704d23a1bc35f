// A subset of GLSL 4.60 for host C++ -- TEST INFRASTRUCTURE ONLY.
//
// oracle/glsl/make_ref.py compiles the reference's own GLSL helper files
// (brdf/*.hsh, raytracer/lights.hsh, raytracer/intersections.hsh,
// common/random.hsh, ...) unmodified on the host against this header, to
// produce golden vectors of the engine's shading math.  Written from the
// GLSL specification (OpenGL Shading Language 4.60, chapters 5 and 8):
//
//  * vec2/3/4, ivec, uvec with the component names x y z w / r g b a, the
//    two-component swizzles xy / rg (read, assign, *=), constructors from
//    scalars and shorter vectors, component-wise arithmetic;
//  * mat3 (column-major; mat3(c0, c1, c2), mat3 * vec3, vec3 * mat3);
//  * the built-ins the helpers call, with the specification's definitions:
//    min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x,
//    clamp(x, a, b) = min(max(x, a), b), mix(x, y, a) = x * (1 - a) + y * a,
//    dot as a left-to-right sum, normalize(x) = x / length(x).
//
// All arithmetic is single precision (the recipe suffixes GLSL's float
// literals with f) and is compiled with -ffp-contract=off, so every
// operation rounds as the GLSL expression's would.  No C math header is
// included: the built-ins call the compiler's single-precision builtins, so
// that GLSL's names (sqrt, pow, atan2 ...) are free for these overloads.
#pragma once

#include <cstdint>
#include <cstring>

typedef unsigned int uint;

inline float glsl_sqrt(float x) { return __builtin_sqrtf(x); }

template <int N, int A, int B>
struct Swz2;

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        float v[2];
    };
    vec2() : x(0.0f), y(0.0f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};

// Two components of a vecN, read as a vec2 and assigned or scaled in place.
template <int N, int A, int B>
struct Swz2 {
    float v[N];
    operator vec2() const { return vec2(v[A], v[B]); }
    Swz2& operator=(const vec2& o) { v[A] = o.x; v[B] = o.y; return *this; }
    Swz2& operator*=(float s) { v[A] = v[A] * s; v[B] = v[B] * s; return *this; }
    Swz2& operator*=(const vec2& o) { v[A] = v[A] * o.x; v[B] = v[B] * o.y; return *this; }
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        Swz2<3, 0, 1> xy;
        Swz2<3, 0, 1> rg;
        float v[3];
    };
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& a, float c) : x(a.x), y(a.y), z(c) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    explicit vec3(const struct vec4& o);
    vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    float& operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        Swz2<4, 0, 1> xy;
        Swz2<4, 0, 1> rg;
        float v[4];
    };
    vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    vec4(const vec2& a, float c, float d) : x(a.x), y(a.y), z(c), w(d) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    float& operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};
inline vec3::vec3(const vec4& o) : x(o.x), y(o.y), z(o.z) {}

#define GLSL_VEC_OPS(T, N)                                                                          \
    inline T operator+(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] + b.v[i]; return r; } \
    inline T operator-(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] - b.v[i]; return r; } \
    inline T operator*(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] * b.v[i]; return r; } \
    inline T operator/(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] / b.v[i]; return r; } \
    inline T operator*(const T& a, float s) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] * s; return r; }      \
    inline T operator*(float s, const T& a) { T r; for (int i = 0; i < N; i++) r.v[i] = s * a.v[i]; return r; }      \
    inline T operator/(const T& a, float s) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] / s; return r; }      \
    inline T operator+(const T& a, float s) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] + s; return r; }      \
    inline T operator-(const T& a, float s) { T r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] - s; return r; }      \
    inline T operator-(float s, const T& a) { T r; for (int i = 0; i < N; i++) r.v[i] = s - a.v[i]; return r; }      \
    inline T operator-(const T& a) { T r; for (int i = 0; i < N; i++) r.v[i] = -a.v[i]; return r; }                \
    inline T& operator+=(T& a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] + b.v[i]; return a; }      \
    inline T& operator-=(T& a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] - b.v[i]; return a; }      \
    inline T& operator*=(T& a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * b.v[i]; return a; }      \
    inline T& operator*=(T& a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * s; return a; }              \
    inline T& operator/=(T& a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] / s; return a; }
GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)

// Integer vectors (the hash functions of common/random.hsh take uvec).
struct uvec2 { uint x, y; uvec2(uint a, uint b) : x(a), y(b) {} };
struct uvec3 { uint x, y, z; uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {} };
struct uvec4 { uint x, y, z, w; uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {} };
struct ivec2 { int x, y; };
struct ivec3 { int x, y, z; };
struct ivec4 { int x, y, z, w; };

// mat3: three columns.
struct mat3 {
    vec3 c[3];
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
struct mat4 { vec4 c[4]; };
struct mat3x4 { vec4 c[3]; };

// ---- scalar built-ins (GLSL 4.60 section 8) ----
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline int min(int x, int y) { return (y < x) ? y : x; }
inline int max(int x, int y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float abs(float x) { return __builtin_fabsf(x); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float sin(float x) { return __builtin_sinf(x); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float atan(float y, float x) { return __builtin_atan2f(y, x); }
inline float atan(float x) { return __builtin_atanf(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline bool isnan(float x) { return __builtin_isnan(x); }
inline bool isinf(float x) { return __builtin_isinf(x); }
inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline int floatBitsToInt(float f) { int u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float intBitsToFloat(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uvec2 floatBitsToUint(const vec2& v) { return uvec2(floatBitsToUint(v.x), floatBitsToUint(v.y)); }
inline uvec3 floatBitsToUint(const vec3& v) {
    return uvec3(floatBitsToUint(v.x), floatBitsToUint(v.y), floatBitsToUint(v.z));
}
inline uvec4 floatBitsToUint(const vec4& v) {
    return uvec4(floatBitsToUint(v.x), floatBitsToUint(v.y), floatBitsToUint(v.z), floatBitsToUint(v.w));
}

// ---- vector built-ins ----
#define GLSL_VEC_FUNCS(T, N)                                                                                \
    inline T min(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = min(a.v[i], b.v[i]); return r; } \
    inline T max(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) r.v[i] = max(a.v[i], b.v[i]); return r; } \
    inline T clamp(const T& x, const T& a, const T& b) { return min(max(x, a), b); }                          \
    inline T clamp(const T& x, float a, float b) { return min(max(x, T(a)), T(b)); }                          \
    inline T mix(const T& x, const T& y, float a) { return x * (1.0f - a) + y * a; }                          \
    inline T abs(const T& a) { T r; for (int i = 0; i < N; i++) r.v[i] = abs(a.v[i]); return r; }            \
    inline T sqrt(const T& a) { T r; for (int i = 0; i < N; i++) r.v[i] = sqrt(a.v[i]); return r; }          \
    inline float dot(const T& a, const T& b) { float s = a.v[0] * b.v[0]; for (int i = 1; i < N; i++) s = s + a.v[i] * b.v[i]; return s; } \
    inline float length(const T& a) { return sqrt(dot(a, a)); }                                                \
    inline T normalize(const T& a) { return a / length(a); }
GLSL_VEC_FUNCS(vec2, 2)
GLSL_VEC_FUNCS(vec3, 3)
GLSL_VEC_FUNCS(vec4, 4)

inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// row vector times matrix: the dot products with the columns
inline vec3 operator*(const vec3& v, const mat3& m) { return vec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }

// half2 packing (GLSL 4.60 section 8.4), the IEEE binary16 conversions
inline vec2 unpackHalf2x16(uint u) {
    auto h2f = [](uint h) {
        const uint s = (h >> 15) & 1u, e = (h >> 10) & 31u, m = h & 1023u;
        float f;
        if (e == 0) f = float(m) * (1.0f / 16777216.0f);
        else if (e == 31) f = m ? __builtin_nanf("") : __builtin_inff();
        else f = uintBitsToFloat(((e + 112u) << 23) | (m << 13));
        return s ? -f : f;
    };
    return vec2(h2f(u & 0xffffu), h2f(u >> 16));
}

// Resource access the helpers mention but the goldens never evaluate
// (EvaluateIndirect*BRDF reads the DFG lookup texture).
struct glsl_sampler2D {};
inline vec4 texture(const glsl_sampler2D&, const vec2&) { return vec4(0.0f); }
#define nonuniformEXT(x) (x)
