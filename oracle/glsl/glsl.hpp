// A subset of GLSL 4.60 for host C++ -- TEST INFRASTRUCTURE ONLY.
//
// oracle/glsl/make_ref.py compiles the reference's own GLSL (the BRDF,
// light, intersection, traversal and path-tracer files) unmodified on the
// host against this header, to produce golden vectors of the engine's
// shading and traversal.  Written from the GLSL specification (OpenGL
// Shading Language 4.60, chapters 5 and 8):
//
//  * vec2/3/4, ivec2/3/4, uvec2/3/4 with the component names x y z w /
//    r g b a and the swizzles the engine's files use (xy xz yz zw xyz rg rgb;
//    read, assign, compound-assign), constructors from scalars and shorter
//    vectors, component-wise arithmetic;
//  * mat3, mat4 (column-major), mat3x4 (three vec4 columns, the engine's
//    instance matrix) and mat4x3, with the products, transpose, the mat4
//    constructor from a mat4x3 (the missing row taken from the identity) and
//    inverse (by cofactors);
//  * the built-ins, with the specification's definitions:
//    min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x,
//    clamp(x, a, b) = min(max(x, a), b), mix(x, y, a) = x * (1 - a) + y * a,
//    dot as a left-to-right sum, normalize(x) = x / length(x);
//  * textures as arrays of RGBA float texels: texelFetch, textureSize, and
//    textureLod with the engine's bindless sampler (linear filtering, repeat
//    addressing) evaluated with exact weights, or a render target's sampler
//    (clamp to edge, weights rounded to the filter's sub-texel precision);
//    integer textures (isampler2D); images and atomics as plain memory, for
//    the one invocation the goldens run.
//
// All arithmetic is single precision (the recipe suffixes GLSL's float
// literals with f) and is compiled with -ffp-contract=off, so every
// operation rounds as the GLSL expression's would.  No C math header is
// included: the built-ins call the compiler's single-precision builtins, so
// that GLSL's names (sqrt, pow, atan2 ...) are free for these overloads.
#pragma once

#include <cstdint>
#include <cstring>
#include <type_traits>

typedef unsigned int uint;

// ---- swizzles: N components of type T, read as V, written component-wise ----
// (a vector constructed from a swizzle, such as ivec3(v.xzy), converts the
// swizzled vector, not the storage under it)
template <typename V, typename T, int N, int... I>
struct Swz {
    T v[N];
    operator V() const { return V(v[I]...); }
    Swz& operator=(const V& o) { int k = 0; ((v[I] = o.v[k++]), ...); return *this; }
    Swz& operator*=(T s) { ((v[I] = v[I] * s), ...); return *this; }
    Swz& operator/=(T s) { ((v[I] = v[I] / s), ...); return *this; }
    Swz& operator*=(const V& o) { int k = 0; ((v[I] = v[I] * o.v[k++]), ...); return *this; }
    Swz& operator+=(const V& o) { int k = 0; ((v[I] = v[I] + o.v[k++]), ...); return *this; }
    Swz& operator-=(const V& o) { int k = 0; ((v[I] = v[I] - o.v[k++]), ...); return *this; }
};

#define GLSL_VEC2(V, T)                                                                   \
    struct V {                                                                            \
        union {                                                                           \
            struct { T x, y; };                                                           \
            struct { T r, g; };                                                           \
            Swz<V, T, 2, 1, 0> yx;                                                        \
            T v[2];                                                                       \
        };                                                                                \
        V() : x(0), y(0) {}                                                               \
        explicit V(T s) : x(s), y(s) {}                                                   \
        V(T a, T b) : x(a), y(b) {}                                                       \
        template <typename U, typename = decltype(static_cast<const U*>(nullptr)->v)>        \
        explicit V(const U& o) : x(T(o.v[0])), y(T(o.v[1])) {}                            \
        template <typename SV, typename ST, int SN, int... SI>                            \
        explicit V(const Swz<SV, ST, SN, SI...>& s) : V(s.operator SV()) {}               \
        template <typename U, typename = typename std::enable_if<std::is_arithmetic<U>::value>::type, \
                  typename = void>                                                        \
        explicit V(U s) : x(T(s)), y(T(s)) {}                                             \
        T& operator[](int i) { return v[i]; }                                             \
        T operator[](int i) const { return v[i]; }                                        \
    };
#define GLSL_VEC3(V, T, V2)                                                               \
    struct V {                                                                            \
        union {                                                                           \
            struct { T x, y, z; };                                                        \
            struct { T r, g, b; };                                                        \
            Swz<V2, T, 3, 0, 1> xy;                                                       \
            Swz<V2, T, 3, 0, 1> rg;                                                       \
            Swz<V2, T, 3, 0, 2> xz;                                                       \
            Swz<V2, T, 3, 1, 2> yz;                                                       \
            Swz<V, T, 3, 0, 1, 2> xyz;                                                    \
            Swz<V, T, 3, 0, 2, 1> xzy;                                                    \
            Swz<V, T, 3, 0, 1, 2> rgb;                                                    \
            T v[3];                                                                       \
        };                                                                                \
        V() : x(0), y(0), z(0) {}                                                         \
        explicit V(T s) : x(s), y(s), z(s) {}                                             \
        V(T a, T b, T c) : x(a), y(b), z(c) {}                                            \
        V(const V2& a, T c) : x(a.x), y(a.y), z(c) {}                                     \
        V(const V& o) : x(o.x), y(o.y), z(o.z) {}                                         \
        template <typename U, typename = decltype(static_cast<const U*>(nullptr)->v)>        \
        explicit V(const U& o) : x(T(o.v[0])), y(T(o.v[1])), z(T(o.v[2])) {}              \
        template <typename SV, typename ST, int SN, int... SI>                            \
        explicit V(const Swz<SV, ST, SN, SI...>& s) : V(s.operator SV()) {}               \
        template <typename U, typename = typename std::enable_if<std::is_arithmetic<U>::value>::type, \
                  typename = void>                                                        \
        explicit V(U s) : x(T(s)), y(T(s)), z(T(s)) {}                                    \
        V& operator=(const V& o) { x = o.x; y = o.y; z = o.z; return *this; }            \
        T& operator[](int i) { return v[i]; }                                             \
        T operator[](int i) const { return v[i]; }                                        \
    };
#define GLSL_VEC4(V, T, V2, V3)                                                           \
    struct V {                                                                            \
        union {                                                                           \
            struct { T x, y, z, w; };                                                     \
            struct { T r, g, b, a; };                                                     \
            Swz<V2, T, 4, 0, 1> xy;                                                       \
            Swz<V2, T, 4, 0, 1> rg;                                                       \
            Swz<V2, T, 4, 2, 3> zw;                                                       \
            Swz<V2, T, 4, 0, 2> xz;                                                       \
            Swz<V3, T, 4, 0, 1, 2> xyz;                                                   \
            Swz<V3, T, 4, 0, 2, 1> xzy;                                                   \
            Swz<V3, T, 4, 0, 1, 2> rgb;                                                   \
            T v[4];                                                                       \
        };                                                                                \
        V() : x(0), y(0), z(0), w(0) {}                                                   \
        explicit V(T s) : x(s), y(s), z(s), w(s) {}                                       \
        V(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}                                 \
        template <typename A, typename B, typename C, typename D>                         \
        V(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}                     \
        V(const V3& a, T d) : x(a.x), y(a.y), z(a.z), w(d) {}                             \
        V(const V2& a, T c, T d) : x(a.x), y(a.y), z(c), w(d) {}                          \
        V(const V2& a, const V2& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}                   \
        V(const V& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}                                 \
        template <typename SV, typename ST, int SN, int... SI>                            \
        explicit V(const Swz<SV, ST, SN, SI...>& s) : V(s.operator SV()) {}               \
        V& operator=(const V& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }   \
        T& operator[](int i) { return v[i]; }                                             \
        T operator[](int i) const { return v[i]; }                                        \
    };

GLSL_VEC2(vec2, float)
GLSL_VEC3(vec3, float, vec2)
GLSL_VEC4(vec4, float, vec2, vec3)
GLSL_VEC2(ivec2, int)
GLSL_VEC3(ivec3, int, ivec2)
GLSL_VEC4(ivec4, int, ivec2, ivec3)
GLSL_VEC2(uvec2, uint)
GLSL_VEC3(uvec3, uint, uvec2)
GLSL_VEC4(uvec4, uint, uvec2, uvec3)

#define GLSL_VEC_OPS(V, T, N)                                                                              \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] + b.v[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] - b.v[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] * b.v[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] / b.v[i]; return r; } \
    inline V operator*(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] * s; return r; }      \
    inline V operator*(T s, const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = s * a.v[i]; return r; }      \
    inline V operator/(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] / s; return r; }      \
    inline V operator+(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] + s; return r; }      \
    inline V operator+(T s, const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = s + a.v[i]; return r; }      \
    inline V operator-(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = a.v[i] - s; return r; }      \
    inline V operator-(T s, const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = s - a.v[i]; return r; }      \
    inline V operator/(T s, const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = s / a.v[i]; return r; }      \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = -a.v[i]; return r; }                \
    inline V& operator+=(V& a, const V& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] + b.v[i]; return a; }      \
    inline V& operator-=(V& a, const V& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] - b.v[i]; return a; }      \
    inline V& operator*=(V& a, const V& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * b.v[i]; return a; }      \
    inline V& operator/=(V& a, const V& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] / b.v[i]; return a; }      \
    inline V& operator*=(V& a, T s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * s; return a; }              \
    inline V& operator/=(V& a, T s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] / s; return a; }              \
    inline V& operator+=(V& a, T s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] + s; return a; }
GLSL_VEC_OPS(vec2, float, 2)
GLSL_VEC_OPS(vec3, float, 3)
GLSL_VEC_OPS(vec4, float, 4)
GLSL_VEC_OPS(ivec2, int, 2)
GLSL_VEC_OPS(ivec3, int, 3)
GLSL_VEC_OPS(ivec4, int, 4)
GLSL_VEC_OPS(uvec2, uint, 2)
GLSL_VEC_OPS(uvec3, uint, 3)
GLSL_VEC_OPS(uvec4, uint, 4)
// GLSL's implicit int -> float conversion of an operand (section 4.1.10)
inline vec2 operator+(const vec2& a, const ivec2& b) { return a + vec2(b); }
inline ivec2 operator%(const ivec2& a, const ivec2& b) { return ivec2(a.x % b.x, a.y % b.y); }
inline ivec2 operator%(const ivec2& a, int b) { return ivec2(a.x % b, a.y % b); }
inline ivec3 operator&(const ivec3& a, const ivec3& b) { return ivec3(a.x & b.x, a.y & b.y, a.z & b.z); }

// ---- boolean vectors and the component-wise relations (section 8.7) ----
struct bvec2 { bool x, y; };
struct bvec3 { bool x, y, z; };
inline bvec2 lessThan(const ivec2& a, const ivec2& b) { return bvec2{ a.x < b.x, a.y < b.y }; }
#define GLSL_REL3(V)                                                                                       \
    inline bvec3 lessThan(const V& a, const V& b) { return bvec3{ a.x < b.x, a.y < b.y, a.z < b.z }; }      \
    inline bvec3 greaterThan(const V& a, const V& b) { return bvec3{ a.x > b.x, a.y > b.y, a.z > b.z }; }   \
    inline bvec3 greaterThanEqual(const V& a, const V& b) { return bvec3{ a.x >= b.x, a.y >= b.y, a.z >= b.z }; }
GLSL_REL3(vec3)
GLSL_REL3(ivec3)
inline bool all(const bvec2& b) { return b.x && b.y; }
inline bool any(const bvec2& b) { return b.x || b.y; }
inline bool all(const bvec3& b) { return b.x && b.y && b.z; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }

// ---- scalar built-ins (GLSL 4.60 section 8) ----
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline int min(int x, int y) { return (y < x) ? y : x; }
inline int max(int x, int y) { return (x < y) ? y : x; }
inline uint min(uint x, uint y) { return (y < x) ? y : x; }
inline uint max(uint x, uint y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float abs(float x) { return __builtin_fabsf(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float exp(float x) { return __builtin_expf(x); }
inline float acos(float x) { return __builtin_acosf(x); }
inline float sin(float x) { return __builtin_sinf(x); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float atan(float y, float x) { return __builtin_atan2f(y, x); }
inline float atan(float x) { return __builtin_atanf(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float fract(float x) { return x - __builtin_floorf(x); }
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
#define GLSL_VEC_FUNCS(V, N)                                                                                \
    inline V min(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = min(a.v[i], b.v[i]); return r; } \
    inline V max(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = max(a.v[i], b.v[i]); return r; } \
    inline V clamp(const V& x, const V& a, const V& b) { return min(max(x, a), b); }                          \
    inline V abs(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = abs(a.v[i]); return r; }
GLSL_VEC_FUNCS(vec2, 2)
GLSL_VEC_FUNCS(vec3, 3)
GLSL_VEC_FUNCS(vec4, 4)
GLSL_VEC_FUNCS(ivec2, 2)
GLSL_VEC_FUNCS(ivec3, 3)
// min / max of a vector and a scalar (genType min(genType, float))
#define GLSL_VEC_SCALAR(V, T, N)                                                                            \
    inline V min(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = min(a.v[i], s); return r; }   \
    inline V max(const V& a, T s) { V r; for (int i = 0; i < N; i++) r.v[i] = max(a.v[i], s); return r; }
GLSL_VEC_SCALAR(vec2, float, 2)
GLSL_VEC_SCALAR(vec3, float, 3)
GLSL_VEC_SCALAR(vec4, float, 4)
#define GLSL_FVEC_FUNCS(V, N)                                                                               \
    inline V clamp(const V& x, float a, float b) { return min(max(x, V(a)), V(b)); }                          \
    inline V mix(const V& x, const V& y, float a) { return x * (1.0f - a) + y * a; }                          \
    inline V mix(const V& x, const V& y, const V& a) { return x * (1.0f - a) + y * a; }                       \
    inline V sqrt(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = sqrt(a.v[i]); return r; }          \
    inline V floor(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = floor(a.v[i]); return r; }        \
    inline V fract(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = fract(a.v[i]); return r; }        \
    inline V pow(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.v[i] = pow(a.v[i], b.v[i]); return r; } \
    inline V exp(const V& a) { V r; for (int i = 0; i < N; i++) r.v[i] = exp(a.v[i]); return r; }            \
    inline float dot(const V& a, const V& b) { float s = a.v[0] * b.v[0]; for (int i = 1; i < N; i++) s = s + a.v[i] * b.v[i]; return s; } \
    inline float length(const V& a) { return sqrt(dot(a, a)); }                                                \
    inline float distance(const V& a, const V& b) { return length(a - b); }                                    \
    inline V normalize(const V& a) { return a / length(a); }
GLSL_FVEC_FUNCS(vec2, 2)
GLSL_FVEC_FUNCS(vec3, 3)
GLSL_FVEC_FUNCS(vec4, 4)

// reflect(I, N) = I - 2 * dot(N, I) * N (section 8.5)
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }

inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---- matrices (column-major) ----
struct mat3 {
    vec3 c[3];
    mat3() {}
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit mat3(const struct mat4& m);   // the upper-left 3 x 3 (section 5.4.2)
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4x3 { vec3 c[4]; };                  // four columns of three rows
struct mat3x4 {                                // three columns of four rows
    vec4 c[3];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    mat4() {}
    explicit mat4(float s) { for (int i = 0; i < 4; i++) c[i] = vec4(0.0f); for (int i = 0; i < 4; i++) c[i].v[i] = s; }
    mat4(const vec4& a, const vec4& b, const vec4& d, const vec4& e) { c[0] = a; c[1] = b; c[2] = d; c[3] = e; }
    // from a mat4x3: the fourth row taken from the identity
    explicit mat4(const mat4x3& m) { for (int i = 0; i < 4; i++) c[i] = vec4(m.c[i], i == 3 ? 1.0f : 0.0f); }
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3::mat3(const mat4& m) { for (int i = 0; i < 3; i++) c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z); }
inline vec3 operator*(const mat3& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline vec3 operator*(const vec3& v, const mat3& m) { return vec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }
inline vec4 operator*(const mat4& m, const vec4& v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w;
}
// row vector times a 3-column matrix: the dot products with its columns
inline vec3 operator*(const vec4& v, const mat3x4& m) { return vec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }
inline mat4x3 transpose(const mat3x4& m) {
    mat4x3 r;
    for (int i = 0; i < 4; i++) r.c[i] = vec3(m.c[0].v[i], m.c[1].v[i], m.c[2].v[i]);
    return r;
}
inline mat4 transpose(const mat4& m) {
    mat4 r;
    for (int i = 0; i < 4; i++) r.c[i] = vec4(m.c[0].v[i], m.c[1].v[i], m.c[2].v[i], m.c[3].v[i]);
    return r;
}
// The inverse by cofactors (adjugate over the determinant), in single
// precision; the specification leaves the method to the implementation.
inline mat4 inverse(const mat4& m) {
    float a[16], inv[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) a[i * 4 + j] = m.c[i].v[j];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] +
             a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] -
             a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] +
             a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] -
              a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] -
             a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] +
             a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] -
             a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] +
              a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] +
             a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] -
             a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] +
              a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] -
              a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] -
             a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] +
             a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] -
              a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] +
              a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    mat4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.c[i].v[j] = inv[i * 4 + j] / det;
    return r;
}

// ---- packing (GLSL 4.60 section 8.4) ----
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
// binary32 -> binary16, rounded to nearest even (the conversion rounds
// half-way cases to even, as IEEE 754 does)
inline uint glsl_float_to_half(float f) {
    const uint u = floatBitsToUint(f);
    const uint s = (u >> 16) & 0x8000u;
    const uint e = (u >> 23) & 0xffu;
    uint m = u & 0x7fffffu;
    if (e == 0xffu) return s | 0x7c00u | (m ? 0x200u : 0u);
    int he = int(e) - 127 + 15;
    if (he >= 31) return s | 0x7c00u;
    if (he <= 0) {
        if (he < -10) return s;
        m |= 0x800000u;
        const uint shift = uint(14 - he);
        uint h = m >> shift;
        const uint rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) h++;
        return s | h;
    }
    uint h = (uint(he) << 10) | (m >> 13);
    const uint rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return s | h;
}
inline uint packHalf2x16(const vec2& v) { return glsl_float_to_half(v.x) | (glsl_float_to_half(v.y) << 16); }
inline vec4 unpackUnorm4x8(uint u) {
    return vec4(float(u & 255u) / 255.0f, float((u >> 8) & 255u) / 255.0f, float((u >> 16) & 255u) / 255.0f,
                float(u >> 24) / 255.0f);
}

// ---- textures: RGBA float texels, row-major, one level per texture ----
struct glsl_texture2D {
    const float* texels = nullptr;   // width * height * 4
    int width = 0, height = 0;
};
struct glsl_sampler {};
struct glsl_sampler2D {
    const glsl_texture2D* tex = nullptr;
    // addressing and filter precision of a bound sampler: repeat and exact
    // weights by default; a render target's sampler clamps to the edge, and
    // filtering hardware weighs neighbours with subtexel_bits of fraction
    bool clamp_to_edge = false;
    int subtexel_bits = 0;
    glsl_sampler2D() {}
    glsl_sampler2D(const glsl_texture2D& t, const glsl_sampler&) : tex(&t) {}
};
typedef glsl_texture2D texture2D;
typedef glsl_sampler sampler;
typedef glsl_sampler2D sampler2D;
struct sampler2DArray { int width = 0, height = 0, layers = 0; };
struct samplerCube { vec4 constant; };   // a constant environment (the goldens' sky)
inline ivec2 textureSize(const sampler2D& s, int) { return s.tex ? ivec2(s.tex->width, s.tex->height) : ivec2(0); }
inline ivec3 textureSize(const sampler2DArray& s, int) { return ivec3(s.width, s.height, s.layers); }
inline vec4 texelFetch(const sampler2D& s, const ivec2& p, int) {
    const float* t = s.tex->texels + (size_t(p.y) * s.tex->width + p.x) * 4;
    return vec4(t[0], t[1], t[2], t[3]);
}
inline vec4 texelFetch(const sampler2DArray&, const ivec3&, int) { return vec4(0.0f); }
// layered and shadow samplers of the DDGI volume and the shadow cascades, which
// the goldens leave unbound (the programs are compiled without DDGI and
// without USE_SHADOW_MAP): they sample as zero
inline vec4 textureLod(const sampler2DArray&, const vec3&, float) { return vec4(0.0f); }
inline vec4 texture(const sampler2DArray&, const vec3&) { return vec4(0.0f); }
struct sampler2DArrayShadow { int width = 0, height = 0, layers = 0; };
inline float texture(const sampler2DArrayShadow&, const vec4&) { return 0.0f; }
inline ivec3 textureSize(const sampler2DArrayShadow& s, int) { return ivec3(s.width, s.height, s.layers); }
// The bindless sampler of the engine (linear filtering, repeat addressing,
// MainRenderer.cpp:922-929) at one level: the specification's bilinear
// filter (OpenGL 4.6 section 8.14.2) with exact weights.
inline vec4 textureLod(const sampler2D& s, const vec2& uv, float) {
    const int w = s.tex->width, h = s.tex->height;
    const float x = uv.x * float(w) - 0.5f, y = uv.y * float(h) - 0.5f;
    const float fx = floor(x), fy = floor(y);
    float ax = x - fx, ay = y - fy;
    if (s.subtexel_bits > 0) {
        const float q = float(1 << s.subtexel_bits);
        ax = __builtin_nearbyintf(ax * q) / q;
        ay = __builtin_nearbyintf(ay * q) / q;
    }
    const bool clamp_edge = s.clamp_to_edge;
    auto wrap = [clamp_edge](int i, int n) {
        if (clamp_edge) return i < 0 ? 0 : (i >= n ? n - 1 : i);
        int m = i % n;
        return m < 0 ? m + n : m;
    };
    const int x0 = wrap(int(fx), w), x1 = wrap(int(fx) + 1, w), y0 = wrap(int(fy), h), y1 = wrap(int(fy) + 1, h);
    const vec4 t00 = texelFetch(s, ivec2(x0, y0), 0), t10 = texelFetch(s, ivec2(x1, y0), 0);
    const vec4 t01 = texelFetch(s, ivec2(x0, y1), 0), t11 = texelFetch(s, ivec2(x1, y1), 0);
    return t00 * ((1.0f - ax) * (1.0f - ay)) + t10 * (ax * (1.0f - ay)) + t01 * ((1.0f - ax) * ay) + t11 * (ax * ay);
}
inline vec4 textureLod(const samplerCube& s, const vec3&, float) { return s.constant; }
// an integer texture, one channel per texel (r; g, b = 0, a = 1)
struct isampler2D {
    const int* texels = nullptr;
    int width = 0, height = 0;
};
inline ivec4 texelFetch(const isampler2D& s, const ivec2& p, int) { return ivec4(s.texels[p.y * s.width + p.x], 0, 0, 1); }
struct usampler2D {
    const uint* texels = nullptr;
    int width = 0, height = 0;
};
inline uvec4 texelFetch(const usampler2D& s, const ivec2& p, int) { return uvec4(s.texels[p.y * s.width + p.x], 0u, 0u, 1u); }
inline vec4 texture(const sampler2D& s, const vec2& uv) { return s.tex ? textureLod(s, uv, 0.0f) : vec4(0.0f); }

// ---- images, atomics and invocation ids, for one invocation ----
struct image2D { vec4* texels = nullptr; int width = 0, height = 0; };
inline ivec2 imageSize(const image2D& im) { return ivec2(im.width, im.height); }
struct uimage2D { uvec4* texels = nullptr; int width = 0; };
struct uimage2DArray { uint* texels = nullptr; int width = 0, height = 0; };
inline void imageStore(image2D& im, const ivec2& p, const vec4& v) { if (im.texels) im.texels[p.y * im.width + p.x] = v; }
inline vec4 imageLoad(const image2D& im, const ivec2& p) { return im.texels ? im.texels[p.y * im.width + p.x] : vec4(0.0f); }
inline void imageStore(uimage2D& im, const ivec2& p, const uvec4& v) { if (im.texels) im.texels[p.y * im.width + p.x] = v; }
inline void imageStore(uimage2DArray& im, const ivec3& p, const uvec4& v) {
    if (im.texels) im.texels[(size_t(p.z) * im.height + p.y) * im.width + p.x] = v.x;
}
inline uint imageAtomicAdd(uimage2DArray& im, const ivec3& p, uint v) {
    if (!im.texels) return 0u;
    uint& t = im.texels[(size_t(p.z) * im.height + p.y) * im.width + p.x];
    const uint old = t;
    t += v;
    return old;
}
inline uint atomicAdd(uint& mem, uint v) { const uint old = mem; mem += v; return old; }
inline int atomicAdd(int& mem, int v) { const int old = mem; mem += v; return old; }
// compute-shader built-ins, set per invocation by the caller (section 7.1.3)
static uvec3 gl_GlobalInvocationID;
static uvec3 gl_WorkGroupID;
static uvec3 gl_NumWorkGroups;
static uvec3 gl_LocalInvocationID;
static uint gl_LocalInvocationIndex = 0;
#define nonuniformEXT(x) (x)
// one invocation runs at a time, each to its end, in invocation order: a
// barrier() after which the group reads only what invocation 0 wrote before
// it (ddgi/rayGen.csh) holds without waiting
inline void barrier() {}
