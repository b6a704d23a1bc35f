/*
 * CPU restatement of Atlas Engine's BVH ray queries -- the ORACLE.
 * TEST INFRASTRUCTURE ONLY (see ae_oracle.h).  Compiled with
 * -ffp-contract=off so every multiply and add rounds separately, in the
 * order written, on x86-64 and aarch64 alike.
 */
#include "ae_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } float4_t;

static inline v3 mk(float x, float y, float z) { v3 r = { x, y, z }; return r; }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
/* dot as (x + y) + z, cross in the GLSL component formula. */
static inline float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

/* glm scalar min/max as the GLSL specification defines them. */
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }

/* ---------------------------------------------------------------------- */
/* Triangle test shared by both semantics: Ray.cpp:53-76 and               */
/* intersections.hsh:36-57 are the same formula.  u weights v1, v weights v2. */
/* ---------------------------------------------------------------------- */
static inline int tri_test(v3 o, v3 d, const aeo_tri* t, float* st, float* su, float* sv) {
    v3 v0 = ld3(t->v0), v1 = ld3(t->v1), v2 = ld3(t->v2);
    v3 e0 = sub(v1, v0);
    v3 e1 = sub(v2, v0);
    v3 s = sub(o, v0);
    v3 p = cross3(s, e0);
    v3 q = cross3(d, e1);
    float den = dot3(q, e0);
    float x = dot3(p, e1) / den;
    float y = dot3(q, s) / den;
    float z = dot3(p, d) / den;
    *st = x; *su = y; *sv = z;
    return x >= 0.0f && y >= 0.0f && z >= 0.0f && y + z <= 1.0f;
}

/* ---------------------------------------------------------------------- */
/* Host semantics (BVH.cpp / Ray.cpp)                                      */
/* ---------------------------------------------------------------------- */

/* Ray::Intersects(const AABB&, float&) -- Ray.cpp:28-43. */
static inline int box_cpu(v3 o, v3 inv, float tmin, float tmax, const float* bmin, const float* bmax, float* t) {
    float t0x = (bmin[0] - o.x) * inv.x, t0y = (bmin[1] - o.y) * inv.y, t0z = (bmin[2] - o.z) * inv.z;
    float t1x = (bmax[0] - o.x) * inv.x, t1y = (bmax[1] - o.y) * inv.y, t1z = (bmax[2] - o.z) * inv.z;
    float sx = gmin(t0x, t1x), sy = gmin(t0y, t1y), sz = gmin(t0z, t1z);
    float bx = gmax(t0x, t1x), by = gmax(t0y, t1y), bz = gmax(t0z, t1z);
    float tminf = gmax(tmin, gmax(sx, gmax(sy, sz)));
    float tmaxf = gmin(tmax, gmin(bx, gmin(by, bz)));
    *t = tminf;
    return tminf <= tmaxf;
}

typedef struct { int32_t ptr; float dist; } cpu_entry;

/* BVH::GetIntersection -- BVH.cpp:103-174. */
static void closest_cpu_one(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris,
                            const float* r, cpu_entry* stack, int32_t* out_ptr, float* out_tuv) {
    v3 o = ld3(r), d = ld3(r + 3);
    v3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float tMin = r[6], tMax = r[7];
    float ix = tMax, iy = 0.0f, iz = 0.0f;   /* intersection.x starts at tMax */
    int32_t closest = -1;
    if (n_nodes) {
        uint32_t sp = 1;
        stack[0].ptr = 0; stack[0].dist = 0.0f;
        float rayTMax = tMax;
        while (sp != 0) {
            cpu_entry e = stack[--sp];
            if (e.dist > ix) continue;
            if (e.ptr < 0) {
                int32_t tp = ~e.ptr;
                int end = 0;
                while (!end) {
                    int32_t ptr = tp++;
                    const aeo_tri* t = &tris[ptr];
                    end = t->v0[3] > 0.0f;
                    float st, su, sv;
                    int hit = tri_test(o, d, t, &st, &su, &sv);
                    if (hit && st < ix) { closest = ptr; ix = st; iy = su; iz = sv; }
                }
            } else {
                rayTMax = ix;
                const aeo_node* nd = &nodes[e.ptr];
                float hl = 0.0f, hr = 0.0f;
                int il = box_cpu(o, inv, tMin, rayTMax, nd->lmin, nd->lmax, &hl);
                int ir = box_cpu(o, inv, tMin, rayTMax, nd->rmin, nd->rmax, &hr);
                if (ir && il) {
                    if (hl < hr) {
                        stack[sp].ptr = nd->right; stack[sp++].dist = hr;
                        stack[sp].ptr = nd->left;  stack[sp++].dist = hl;
                    } else {
                        stack[sp].ptr = nd->left;  stack[sp++].dist = hl;
                        stack[sp].ptr = nd->right; stack[sp++].dist = hr;
                    }
                } else if (ir) {
                    stack[sp].ptr = nd->right; stack[sp++].dist = hr;
                } else if (il) {
                    stack[sp].ptr = nd->left;  stack[sp++].dist = hl;
                }
            }
        }
    }
    /* Hit predicate: intersection.x < the caller's tMax (the returned bool of
     * the reference compares against the mutated ray.tMax, BVH.cpp:141/:172). */
    *out_ptr = (ix < tMax) ? closest : -1;
    out_tuv[0] = ix; out_tuv[1] = iy; out_tuv[2] = iz;
}

/* BVH::GetIntersectionAny -- BVH.cpp:176-217. */
static int any_cpu_one(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris,
                       const float* r, int32_t* stack) {
    if (!n_nodes) return 0;
    v3 o = ld3(r), d = ld3(r + 3);
    v3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float tMin = r[6], tMax = r[7];
    uint32_t sp = 1;
    stack[0] = 0;
    while (sp != 0) {
        int32_t ptr = stack[--sp];
        if (ptr < 0) {
            int32_t tp = ~ptr;
            int end = 0;
            while (!end) {
                const aeo_tri* t = &tris[tp++];
                end = t->v0[3] > 0.0f;
                float st, su, sv;
                if (tri_test(o, d, t, &st, &su, &sv) && st < tMax) return 1;
            }
        } else {
            const aeo_node* nd = &nodes[ptr];
            float dummy;
            int il = box_cpu(o, inv, tMin, tMax, nd->lmin, nd->lmax, &dummy);
            int ir = box_cpu(o, inv, tMin, tMax, nd->rmin, nd->rmax, &dummy);
            if (ir) stack[sp++] = nd->right;
            if (il) stack[sp++] = nd->left;
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Shader semantics (bvh.hsh / intersections.hsh)                          */
/* ---------------------------------------------------------------------- */

/* IntersectAABB(ray, aabb, tmin, tmax, out dist) -- intersections.hsh:18-34.
 * GLSL min/max are taken as IEEE minNum/maxNum (fminf/fmaxf): a NaN operand
 * loses, as it does for the GPU min/max instructions. */
static inline int box_glsl(v3 o, v3 d, float tmin, float tmax, const float* bmin, const float* bmax, float* dist) {
    float t0x = (bmin[0] - o.x) / d.x, t0y = (bmin[1] - o.y) / d.y, t0z = (bmin[2] - o.z) / d.z;
    float t1x = (bmax[0] - o.x) / d.x, t1y = (bmax[1] - o.y) / d.y, t1z = (bmax[2] - o.z) / d.z;
    float sx = fminf(t0x, t1x), sy = fminf(t0y, t1y), sz = fminf(t0z, t1z);
    float bx = fmaxf(t0x, t1x), by = fmaxf(t0y, t1y), bz = fmaxf(t0z, t1z);
    float tminf = fmaxf(fmaxf(tmin, sx), fmaxf(sy, sz));
    float tmaxf = fminf(fminf(tmax, bx), fminf(by, bz));
    int hit = tminf <= tmaxf;
    *dist = hit ? tminf : tmax;
    return hit;
}

static inline int isnan3(v3 d) { return isnan(d.x) || isnan(d.y) || isnan(d.z); }

/* Near-tie detection of the GPU closest-hit trace (trace_kernels.cuh,
 * kTieWindow / near_miss), restated with the same correctly rounded
 * operations so that both flag the same rays.  It does not change the
 * traversal's result. */
#define TIE_WINDOW 4e-6f
static const float TIE_WIDEN = 1.0f + TIE_WINDOW;
#define NEAR_MISS_SCALE 9.5367431640625e-07f   /* 2^-20 */

/* The box test of box_glsl, also reporting a rejected box whose entry lies
 * within TIE_WINDOW of the exit bound. */
static inline int box_glsl_tie(v3 o, v3 d, float tmin, float tmax, const float* bmin, const float* bmax, float* dist,
                               int* near_cull) {
    float t0x = (bmin[0] - o.x) / d.x, t0y = (bmin[1] - o.y) / d.y, t0z = (bmin[2] - o.z) / d.z;
    float t1x = (bmax[0] - o.x) / d.x, t1y = (bmax[1] - o.y) / d.y, t1z = (bmax[2] - o.z) / d.z;
    float sx = fminf(t0x, t1x), sy = fminf(t0y, t1y), sz = fminf(t0z, t1z);
    float bx = fmaxf(t0x, t1x), by = fmaxf(t0y, t1y), bz = fmaxf(t0z, t1z);
    float tminf = fmaxf(fmaxf(tmin, sx), fmaxf(sy, sz));
    float tmaxf = fminf(fminf(tmax, bx), fminf(by, bz));
    int hit = tminf <= tmaxf;
    *dist = hit ? tminf : tmax;
    *near_cull = !hit && tminf <= tmaxf * TIE_WIDEN;
    return hit;
}

/* A triangle rejected within the rounding error of its barycentric tests:
 * |error(u)|, |error(v)| < m / |den| with m = 2^-20 Sd (S0+S1) (Ss+S0+S1)
 * (the L1 norms of d, e0, e1 and s = o - v0); the tests are taken multiplied
 * by |den|, one correctly rounded fmaf each, as tri_test<NEAR> does. */
static inline int near_miss(v3 o, v3 d, const aeo_tri* t, float u, float v) {
    v3 v0 = ld3(t->v0), v1 = ld3(t->v1), v2 = ld3(t->v2);
    v3 e0 = sub(v1, v0), e1 = sub(v2, v0), s = sub(o, v0);
    v3 q = cross3(d, e1);
    float den = dot3(q, e0);
    float s01 = ((fabsf(e0.x) + fabsf(e0.y)) + fabsf(e0.z)) + ((fabsf(e1.x) + fabsf(e1.y)) + fabsf(e1.z));
    float ss = (fabsf(s.x) + fabsf(s.y)) + fabsf(s.z);
    float sd = (fabsf(d.x) + fabsf(d.y)) + fabsf(d.z);
    float m = ((sd * s01) * (ss + s01)) * NEAR_MISS_SCALE;
    float ad = fabsf(den);
    return fmaf(u, ad, m) >= 0.0f && fmaf(v, ad, m) >= 0.0f && fmaf(1.0f - (u + v), ad, m + m) >= 0.0f;
}

/* HitClosest -- bvh.hsh:191-273 on one BLAS, CheckLeafClosest :44-72.
 * The stack is unbounded here (the shader's holds 32 entries with no check). */
static void closest_glsl_one(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris,
                             const float* r, int32_t* stack, int32_t* out_ptr, float* out_tuv,
                             uint32_t* nf, uint32_t* tf, uint32_t* out_flags, float* out_second) {
    v3 o = ld3(r), d = ld3(r + 3);
    float tMin = r[6], tMax = r[7];
    float hitDist = tMax, hu = 0.0f, hv = 0.0f, second = tMax;
    int32_t hitID = -1;
    int suspect = 0;
    uint32_t nodeFetches = 0, triFetches = 0;
    if (n_nodes && !isnan3(d)) {
        uint32_t sp = 1;
        int32_t nodePtr = 0;
        stack[0] = 0;
        while (sp != 0) {
            if (nodePtr < 0) {
                int32_t tp = ~nodePtr;
                int end = 0;
                while (!end) {
                    const aeo_tri* t = &tris[tp];
                    end = t->v0[3] > 0.0f;
                    triFetches++;
                    float st, su, sv;
                    int hit = tri_test(o, d, t, &st, &su, &sv);
                    /* tmax of CheckLeafClosest is ray.hitDistance (bvh.hsh:246) */
                    if (hit && st > tMin && st < tMax) {
                        if (st < hitDist) { second = hitDist; hitDist = st; hitID = tp; hu = su; hv = sv; }
                        else if (st < second) second = st;
                    } else if (st > tMin && st < tMax && st <= hitDist * TIE_WIDEN && near_miss(o, d, t, su, sv)) {
                        suspect = 1;
                    }
                    tp++;
                }
                nodePtr = stack[--sp];
            } else {
                const aeo_node* nd = &nodes[nodePtr];
                nodeFetches++;
                float hl = 0.0f, hr = 0.0f;
                int nl = 0, nr = 0;
                int il = box_glsl_tie(o, d, tMin, hitDist, nd->lmin, nd->lmax, &hl, &nl);
                int ir = box_glsl_tie(o, d, tMin, hitDist, nd->rmin, nd->rmax, &hr, &nr);
                suspect |= nl | nr;
                /* bvh.hsh:234-236 drops a hit right child entered exactly at the bound */
                suspect |= !il && ir && hl <= hr;
                int none = !il && !ir;
                int32_t next = (hl <= hr) ? nd->left : nd->right;
                if (none) next = stack[--sp];
                if (ir && il) stack[sp++] = (hl <= hr) ? nd->right : nd->left;
                nodePtr = next;
            }
        }
    }
    *out_ptr = hitID;
    out_tuv[0] = hitDist; out_tuv[1] = hu; out_tuv[2] = hv;
    if (nf) *nf = nodeFetches;
    if (tf) *tf = triFetches;
    if (out_flags) {
        uint32_t f = hitID >= 0 ? 1u : 0u;
        if ((hitID >= 0 && second - hitDist <= TIE_WINDOW * hitDist) || suspect) f |= 2u;
        *out_flags = f;
    }
    if (out_second) *out_second = second;
}

/* HitAny -- bvh.hsh:359-441 on one BLAS, CheckLeaf :74-104. */
static int any_glsl_one(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris,
                        const float* r, int32_t* stack, uint32_t* nf, uint32_t* tf) {
    v3 o = ld3(r), d = ld3(r + 3);
    float tMin = r[6], tMax = r[7];
    uint32_t nodeFetches = 0, triFetches = 0;
    int hit = 0;
    if (n_nodes && !isnan3(d)) {
        uint32_t sp = 1;
        int32_t nodePtr = 0;
        stack[0] = 0;
        while (sp != 0 && !hit) {
            if (nodePtr < 0) {
                int32_t tp = ~nodePtr;
                int end = 0;
                while (!end && !hit) {
                    const aeo_tri* t = &tris[tp];
                    end = t->v0[3] > 0.0f;
                    triFetches++;
                    float st, su, sv;
                    if (tri_test(o, d, t, &st, &su, &sv) && st > tMin && st < tMax) hit = 1;
                    tp++;
                }
                nodePtr = stack[--sp];
            } else {
                const aeo_node* nd = &nodes[nodePtr];
                nodeFetches++;
                float dl, dr;
                int il = box_glsl(o, d, tMin, tMax, nd->lmin, nd->lmax, &dl);
                int ir = box_glsl(o, d, tMin, tMax, nd->rmin, nd->rmax, &dr);
                int32_t next = il ? nd->left : nd->right;
                if (!ir && !il) next = stack[--sp];
                if (ir && il) stack[sp++] = nd->right;
                nodePtr = next;
            }
        }
    }
    if (nf) *nf = nodeFetches;
    if (tf) *tf = triFetches;
    return hit;
}


/* ---------------------------------------------------------------------- */
/* Two-level shader traversal (TLAS + instances + BLAS)                    */
/* ---------------------------------------------------------------------- */

/* vec4(v, w) * inverseMatrix (bvh.hsh:179-180): component i is
 * dot(vec4(v, w), column i), summed left to right. */
static inline v3 xform(const aeo_instance* in, v3 v, float w) {
    const float* m = in->m;
    v3 r;
    r.x = ((v.x * m[0] + v.y * m[1]) + v.z * m[2]) + w * m[3];
    r.y = ((v.x * m[4] + v.y * m[5]) + v.z * m[6]) + w * m[7];
    r.z = ((v.x * m[8] + v.y * m[9]) + v.z * m[10]) + w * m[11];
    return r;
}

#define TLAS_INVALID 0xFFFFFFFFu

typedef struct {
    const aeo_node* tlas; uint32_t n_tlas;
    const aeo_instance* inst; uint32_t n_inst;
    const aeo_mesh* meshes; uint32_t n_meshes;
    const float* materials;   /* transparency variants: GPUMaterial (23 words); NULL: opaque queries */
    uint32_t n_materials;
    const aeo_texture* textures; uint32_t n_textures;
} scene_t;

/* Leaf triangle of the transparency variants: UnpackTriangle of the shading
 * triangle (common.hsh:17-44) -- vertices, endOfNode = d1.z > 0, opacity =
 * d2.w -- and GetOpacity (surface.hsh:147-159) when the stored opacity is
 * negative: the material's opacity times its opacity texture, which samples
 * as 1.0 when absent (texture.hsh:18-25); bound textures are not sampled and
 * count as 1.0 as well. */
float aeo_half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    uint32_t bits;
    if (e == 0x1Fu) {
        bits = sign | 0x7F800000u | (m << 13);
    } else if (e != 0) {
        bits = sign | ((e + 112u) << 23) | (m << 13);
    } else {
        /* zero or subnormal: m * 2^-24, exact in float */
        float f = (float)m * 5.9604644775390625e-8f;
        memcpy(&bits, &f, 4);
        bits |= sign;
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

static float texel_r(const aeo_texture* t, uint32_t x, uint32_t y) {
    const uint32_t texel = t->format == 0 ? 1u : 4u;
    const uint32_t pitch = t->row_pitch ? t->row_pitch : t->width * texel;
    const uint8_t* row = (const uint8_t*)t->texels + (size_t)y * pitch;
    if (t->format == 0) return (float)row[x] / 255.0f;
    if (t->format == 1) return (float)row[(size_t)x * 4] / 255.0f;
    float f;
    memcpy(&f, row + (size_t)x * 4, 4);
    return f;
}

static void tex_axis(float s, uint32_t n, uint32_t* i0, uint32_t* i1, float* a) {
    float x = s * (float)n - 0.5f;
    if (!(fabsf(x) < 9.0e18f)) x = 0.0f;
    const float fx = floorf(x);
    *a = x - fx;
    long long i = (long long)fx % (long long)n;
    if (i < 0) i += n;
    *i0 = (uint32_t)i;
    *i1 = *i0 + 1u == n ? 0u : *i0 + 1u;
}

float aeo_sample_r_bilinear(const aeo_texture* textures, uint32_t n_textures, int32_t id, float u, float v) {
    if (id < 0 || (uint32_t)id >= n_textures) return 1.0f;
    const aeo_texture* t = &textures[id];
    uint32_t x0, x1, y0, y1;
    float a, b;
    tex_axis(u, t->width, &x0, &x1, &a);
    tex_axis(v, t->height, &y0, &y1, &b);
    const float c00 = texel_r(t, x0, y0), c10 = texel_r(t, x1, y0), c01 = texel_r(t, x0, y1), c11 = texel_r(t, x1, y1);
    const float ia = 1.0f - a, ib = 1.0f - b;
    float r = (ia * ib) * c00;
    r = r + (a * ib) * c10;
    r = r + (ia * b) * c01;
    return r + (a * b) * c11;
}

static inline void half2_of(float bits, float* x, float* y) {
    uint32_t u;
    memcpy(&u, &bits, 4);
    *x = aeo_half_to_float((uint16_t)(u & 0xFFFFu));
    *y = aeo_half_to_float((uint16_t)(u >> 16));
}

/* `tri.opacity < 0.0 ? GetOpacity(tri, sol.yz, materialOffset, 0) : tri.opacity`
 * (bvh.hsh:127, :163; GetOpacity surface.hsh:147-159, whose interpolated
 * vertex alpha is unused). */
static inline float shading_opacity(const scene_t* sc, const float* s, int32_t materialOffset, float bs, float bt) {
    if (!(s[23] < 0.0f)) return s[23];
    int32_t idx;
    memcpy(&idx, &s[15], 4);
    idx += materialOffset;
    if (idx < 0 || (uint32_t)idx >= sc->n_materials) return 1.0f;
    const float* m = sc->materials + (size_t)idx * 23;
    const float r = (1.0f - bs) - bt;
    float u0, v0, u1, v1, u2, v2;
    half2_of(s[12], &u0, &v0);
    half2_of(s[13], &u1, &v1);
    half2_of(s[14], &u2, &v2);
    const float tu = (r * u0 + bs * u1) + bt * u2;
    float tv = (r * v0 + bs * v1) + bt * v2;
    int32_t invert, tex;
    memcpy(&invert, &m[13], 4);
    memcpy(&tex, &m[18], 4);
    if (invert > 0) tv = 1.0f - tv;
    return aeo_sample_r_bilinear(sc->textures, sc->n_textures, tex, tu, tv) * m[7];
}

static inline aeo_tri shading_tri(const float* s) {
    aeo_tri t;
    memset(&t, 0, sizeof(t));
    for (int k = 0; k < 3; k++) { t.v0[k] = s[k]; t.v1[k] = s[4 + k]; t.v2[k] = s[8 + k]; }
    return t;
}

/* HitClosest -- bvh.hsh:191-273.  The TLAS/BLAS switch is keyed on the stack
 * depth at which the instance was entered (tlasIndex). */
static void scene_closest_one(const scene_t* sc, const float* r, uint32_t cull, int32_t* stack,
                              int32_t* out_ptr, int32_t* out_inst, float* out_tuv, uint32_t* nf, uint32_t* tf) {
    v3 wo = ld3(r), wd = ld3(r + 3);
    float tMin = r[6], tMax = r[7];
    float hitDist = tMax, hu = 0.0f, hv = 0.0f;
    int32_t hitID = -1, hitInst = -1, curInst = -1;
    uint32_t nodeFetches = 0, triFetches = 0;
    if (sc->n_tlas && !isnan3(wd)) {
        v3 o = wo, d = wd;
        const aeo_mesh* mesh = NULL;
        uint32_t sp = 1, tlasIndex = TLAS_INVALID;
        int32_t nodePtr = 0;
        stack[0] = 0;
        while (sp != 0) {
            if (sp < tlasIndex) {
                o = wo; d = wd;
                tlasIndex = TLAS_INVALID;
                if (nodePtr < 0) {
                    /* CheckInstance -- bvh.hsh:172-189 */
                    const aeo_instance* in = &sc->inst[~nodePtr];
                    o = xform(in, wo, 1.0f);
                    d = xform(in, wd, 0.0f);
                    curInst = ~nodePtr;
                    mesh = &sc->meshes[in->meshOffset];
                    if ((in->mask & cull) > 0 && mesh->n_nodes > 0) {
                        nodePtr = 0;
                        tlasIndex = sp;
                    } else {
                        nodePtr = stack[--sp];
                    }
                } else {
                    const aeo_node* nd = &sc->tlas[nodePtr];
                    nodeFetches++;
                    float hl = 0.0f, hr = 0.0f;
                    int il = box_glsl(o, d, tMin, hitDist, nd->lmin, nd->lmax, &hl);
                    int ir = box_glsl(o, d, tMin, hitDist, nd->rmin, nd->rmax, &hr);
                    int none = !il && !ir;
                    int32_t next = (hl <= hr) ? nd->left : nd->right;
                    if (none) next = stack[--sp];
                    if (ir && il) stack[sp++] = (hl <= hr) ? nd->right : nd->left;
                    nodePtr = next;
                }
            } else {
                if (nodePtr < 0) {
                    int32_t tp = ~nodePtr;
                    int end = 0;
                    while (!end) {
                        float st, su, sv;
                        int hit;
                        triFetches++;
                        if (sc->materials) {
                            /* CheckLeafClosestTransparency -- bvh.hsh:106-138 */
                            const float* sh = mesh->shading + (size_t)tp * 24;
                            const aeo_tri t = shading_tri(sh);
                            end = sh[18] > 0.0f;
                            hit = tri_test(o, d, &t, &st, &su, &sv);
                            if (hit && st > tMin && st < hitDist &&
                                shading_opacity(sc, sh, sc->inst[curInst].materialOffset, su, sv) > 0.0f) {
                                hitDist = st; hitID = tp; hu = su; hv = sv; hitInst = curInst;
                            }
                        } else {
                            const aeo_tri* t = &mesh->tris[tp];
                            end = t->v0[3] > 0.0f;
                            hit = tri_test(o, d, t, &st, &su, &sv);
                            if (hit && st > tMin && st < hitDist) {
                                hitDist = st; hitID = tp; hu = su; hv = sv; hitInst = curInst;
                            }
                        }
                        tp++;
                    }
                    nodePtr = stack[--sp];
                } else {
                    const aeo_node* nd = &mesh->nodes[nodePtr];
                    nodeFetches++;
                    float hl = 0.0f, hr = 0.0f;
                    int il = box_glsl(o, d, tMin, hitDist, nd->lmin, nd->lmax, &hl);
                    int ir = box_glsl(o, d, tMin, hitDist, nd->rmin, nd->rmax, &hr);
                    int none = !il && !ir;
                    int32_t next = (hl <= hr) ? nd->left : nd->right;
                    if (none) next = stack[--sp];
                    if (ir && il) stack[sp++] = (hl <= hr) ? nd->right : nd->left;
                    nodePtr = next;
                }
            }
        }
    }
    *out_ptr = hitID;
    *out_inst = hitInst;
    out_tuv[0] = hitDist; out_tuv[1] = hu; out_tuv[2] = hv;
    if (nf) *nf = nodeFetches;
    if (tf) *tf = triFetches;
}

/* HitAny -- bvh.hsh:359-441. */
static int scene_any_one(const scene_t* sc, const float* r, uint32_t cull, int32_t* stack) {
    v3 wo = ld3(r), wd = ld3(r + 3);
    float tMin = r[6], tMax = r[7];
    if (!sc->n_tlas || isnan3(wd)) return 0;
    v3 o = wo, d = wd;
    const aeo_mesh* mesh = NULL;
    uint32_t sp = 1, tlasIndex = TLAS_INVALID;
    int32_t nodePtr = 0;
    int hit = 0;
    stack[0] = 0;
    while (sp != 0 && !hit) {
        if (sp < tlasIndex) {
            o = wo; d = wd;
            tlasIndex = TLAS_INVALID;
            if (nodePtr < 0) {
                const aeo_instance* in = &sc->inst[~nodePtr];
                o = xform(in, wo, 1.0f);
                d = xform(in, wd, 0.0f);
                mesh = &sc->meshes[in->meshOffset];
                if ((in->mask & cull) > 0 && mesh->n_nodes > 0) {
                    nodePtr = 0;
                    tlasIndex = sp;
                } else {
                    nodePtr = stack[--sp];
                }
            } else {
                const aeo_node* nd = &sc->tlas[nodePtr];
                float dl, dr;
                int il = box_glsl(o, d, tMin, tMax, nd->lmin, nd->lmax, &dl);
                int ir = box_glsl(o, d, tMin, tMax, nd->rmin, nd->rmax, &dr);
                int32_t next = il ? nd->left : nd->right;
                if (!ir && !il) next = stack[--sp];
                if (ir && il) stack[sp++] = nd->right;
                nodePtr = next;
            }
        } else {
            if (nodePtr < 0) {
                int32_t tp = ~nodePtr;
                int end = 0;
                while (!end && !hit) {
                    const aeo_tri* t = &mesh->tris[tp];
                    end = t->v0[3] > 0.0f;
                    float st, su, sv;
                    if (tri_test(o, d, t, &st, &su, &sv) && st > tMin && st < tMax) hit = 1;
                    tp++;
                }
                nodePtr = stack[--sp];
            } else {
                const aeo_node* nd = &mesh->nodes[nodePtr];
                float dl, dr;
                int il = box_glsl(o, d, tMin, tMax, nd->lmin, nd->lmax, &dl);
                int ir = box_glsl(o, d, tMin, tMax, nd->rmin, nd->rmax, &dr);
                int32_t next = il ? nd->left : nd->right;
                if (!ir && !il) next = stack[--sp];
                if (ir && il) stack[sp++] = nd->right;
                nodePtr = next;
            }
        }
    }
    return hit;
}

/* HitAnyTransparency -- bvh.hsh:443-524 with CheckLeafTransparency :140-170.
 * Every accepted triangle multiplies the leaf's running transparency, which
 * starts from the current value; the leaf's result multiplies the current
 * value again (transparency *= CheckLeafTransparency(..., transparency)),
 * and values below 1e-6 become 0, which ends the traversal. */
static float scene_any_transparency_one(const scene_t* sc, const float* r, uint32_t cull, int32_t* stack) {
    v3 wo = ld3(r), wd = ld3(r + 3);
    float tMin = r[6], tMax = r[7];
    if (isnan3(wd)) return 1.0f;
    float transparency = 1.0f;
    if (!sc->n_tlas) return transparency;
    v3 o = wo, d = wd;
    const aeo_mesh* mesh = NULL;
    int32_t matOffset = 0;
    uint32_t sp = 1, tlasIndex = TLAS_INVALID;
    int32_t nodePtr = 0;
    stack[0] = 0;
    while (sp != 0 && transparency > 0.0f) {
        if (sp < tlasIndex) {
            o = wo; d = wd;
            tlasIndex = TLAS_INVALID;
            if (nodePtr < 0) {
                const aeo_instance* in = &sc->inst[~nodePtr];
                o = xform(in, wo, 1.0f);
                d = xform(in, wd, 0.0f);
                mesh = &sc->meshes[in->meshOffset];
                matOffset = in->materialOffset;
                if ((in->mask & cull) > 0 && mesh->n_nodes > 0) {
                    nodePtr = 0;
                    tlasIndex = sp;
                } else {
                    nodePtr = stack[--sp];
                }
            } else {
                const aeo_node* nd = &sc->tlas[nodePtr];
                float dl, dr;
                int il = box_glsl(o, d, tMin, tMax, nd->lmin, nd->lmax, &dl);
                int ir = box_glsl(o, d, tMin, tMax, nd->rmin, nd->rmax, &dr);
                int32_t next = il ? nd->left : nd->right;
                if (!ir && !il) next = stack[--sp];
                if (ir && il) stack[sp++] = nd->right;
                nodePtr = next;
            }
        } else {
            if (nodePtr < 0) {
                int32_t tp = ~nodePtr;
                int end = 0;
                float leaf = transparency;
                while (!end) {
                    const float* sh = mesh->shading + (size_t)tp * 24;
                    const aeo_tri t = shading_tri(sh);
                    end = sh[18] > 0.0f;
                    float st, su, sv;
                    if (tri_test(o, d, &t, &st, &su, &sv) && st > tMin && st < tMax)
                        leaf = leaf * (1.0f - shading_opacity(sc, sh, matOffset, su, sv));
                    tp++;
                }
                transparency = transparency * leaf;
                if (transparency < 0.000001f) transparency = 0.0f;
                nodePtr = stack[--sp];
            } else {
                const aeo_node* nd = &mesh->nodes[nodePtr];
                float dl, dr;
                int il = box_glsl(o, d, tMin, tMax, nd->lmin, nd->lmax, &dl);
                int ir = box_glsl(o, d, tMin, tMax, nd->rmin, nd->rmax, &dr);
                int32_t next = il ? nd->left : nd->right;
                if (!ir && !il) next = stack[--sp];
                if (ir && il) stack[sp++] = nd->right;
                nodePtr = next;
            }
        }
    }
    return transparency;
}

typedef struct {
    const scene_t* sc; const float* rays; uint32_t begin, end; uint32_t cull; int any;
    int32_t* ptr; int32_t* inst; float* tuv; uint8_t* occ; float* transparency; uint32_t* nf; uint32_t* tf;
    size_t stack_cap;
} scene_job_t;

static void* run_scene_job(void* arg) {
    scene_job_t* j = (scene_job_t*)arg;
    int32_t* stack = (int32_t*)malloc(j->stack_cap * sizeof(int32_t));
    for (uint32_t i = j->begin; i < j->end; i++) {
        const float* r = j->rays + (size_t)i * 8;
        if (j->transparency) j->transparency[i] = scene_any_transparency_one(j->sc, r, j->cull, stack);
        else if (j->any) j->occ[i] = (uint8_t)scene_any_one(j->sc, r, j->cull, stack);
        else scene_closest_one(j->sc, r, j->cull, stack, &j->ptr[i], &j->inst[i], &j->tuv[(size_t)i * 3],
                               j->nf ? &j->nf[i] : NULL, j->tf ? &j->tf[i] : NULL);
    }
    free(stack);
    return NULL;
}

static void run_scene(scene_job_t proto, uint32_t n, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    scene_job_t jobs[256];
    uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    int started = 0;
    for (int t = 0; t < threads; t++) {
        uint32_t b = (uint32_t)t * chunk;
        if (b >= n) break;
        jobs[t] = proto; jobs[t].begin = b; jobs[t].end = b + chunk < n ? b + chunk : n;
        pthread_create(&th[t], NULL, run_scene_job, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

static size_t scene_stack_cap(const scene_t* sc) {
    size_t cap = sc->n_tlas + 64;
    for (uint32_t i = 0; i < sc->n_meshes; i++) cap += sc->meshes[i].n_nodes;
    return cap;
}

void aeo_scene_closest_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, uint32_t n_inst,
                            const aeo_mesh* meshes, uint32_t n_meshes, const float* rays, uint32_t n_rays,
                            uint32_t cull_mask, int threads, int32_t* tri_ptr, int32_t* inst_out, float* tuv,
                            uint32_t* node_fetches, uint32_t* tri_fetches) {
    scene_t sc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, NULL };
    scene_job_t p; memset(&p, 0, sizeof(p));
    p.sc = &sc; p.rays = rays; p.cull = cull_mask; p.any = 0; p.ptr = tri_ptr; p.inst = inst_out; p.tuv = tuv;
    p.nf = node_fetches; p.tf = tri_fetches; p.stack_cap = scene_stack_cap(&sc);
    run_scene(p, n_rays, threads);
}

void aeo_scene_any_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, uint32_t n_inst,
                        const aeo_mesh* meshes, uint32_t n_meshes, const float* rays, uint32_t n_rays,
                        uint32_t cull_mask, int threads, uint8_t* occluded) {
    scene_t sc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, NULL };
    scene_job_t p; memset(&p, 0, sizeof(p));
    p.sc = &sc; p.rays = rays; p.cull = cull_mask; p.any = 1; p.occ = occluded; p.stack_cap = scene_stack_cap(&sc);
    run_scene(p, n_rays, threads);
}

void aeo_scene_closest_transparency_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst,
                                         uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes,
                                         const float* materials, uint32_t n_materials,
                                         const aeo_texture* textures, uint32_t n_textures, const float* rays,
                                         uint32_t n_rays, uint32_t cull_mask, int threads, int32_t* tri_ptr,
                                         int32_t* inst_out, float* tuv) {
    scene_t sc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, materials, n_materials, textures, n_textures };
    scene_job_t p; memset(&p, 0, sizeof(p));
    p.sc = &sc; p.rays = rays; p.cull = cull_mask; p.any = 0; p.ptr = tri_ptr; p.inst = inst_out; p.tuv = tuv;
    p.stack_cap = scene_stack_cap(&sc);
    run_scene(p, n_rays, threads);
}

void aeo_scene_any_transparency_glsl(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst,
                                     uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes,
                                     const float* materials, uint32_t n_materials, const aeo_texture* textures,
                                     uint32_t n_textures, const float* rays, uint32_t n_rays, uint32_t cull_mask,
                                     int threads, float* transparency) {
    scene_t sc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, materials, n_materials, textures, n_textures };
    scene_job_t p; memset(&p, 0, sizeof(p));
    p.sc = &sc; p.rays = rays; p.cull = cull_mask; p.any = 1; p.transparency = transparency;
    p.stack_cap = scene_stack_cap(&sc);
    run_scene(p, n_rays, threads);
}

/* ---------------------------------------------------------------------- */
/* Double-precision brute force                                            */
/* ---------------------------------------------------------------------- */
/* The vertex positions of two BVH entries are equal (the w fields hold the
 * leaf flag, material and opacity, which may differ between the copies). */
static int same_vertices(const aeo_tri* a, const aeo_tri* b) {
    for (int k = 0; k < 3; k++)
        if (a->v0[k] != b->v0[k] || a->v1[k] != b->v1[k] || a->v2[k] != b->v2[k]) return 0;
    return 1;
}

static void closest_f64_one(const aeo_tri* tris, uint32_t n_tris, const float* r,
                            int32_t* out_ptr, double* out_t, double* out_t2) {
    double o[3] = { r[0], r[1], r[2] }, d[3] = { r[3], r[4], r[5] };
    double tMin = r[6], tMax = r[7];
    double best = INFINITY, second = INFINITY;
    int32_t bi = -1;
    for (uint32_t i = 0; i < n_tris; i++) {
        const aeo_tri* t = &tris[i];
        double v0[3] = { t->v0[0], t->v0[1], t->v0[2] };
        double e0[3] = { t->v1[0] - v0[0], t->v1[1] - v0[1], t->v1[2] - v0[2] };
        double e1[3] = { t->v2[0] - v0[0], t->v2[1] - v0[1], t->v2[2] - v0[2] };
        double s[3] = { o[0] - v0[0], o[1] - v0[1], o[2] - v0[2] };
        double p[3] = { s[1] * e0[2] - e0[1] * s[2], s[2] * e0[0] - e0[2] * s[0], s[0] * e0[1] - e0[0] * s[1] };
        double q[3] = { d[1] * e1[2] - e1[1] * d[2], d[2] * e1[0] - e1[2] * d[0], d[0] * e1[1] - e1[0] * d[1] };
        double den = q[0] * e0[0] + q[1] * e0[1] + q[2] * e0[2];
        double x = (p[0] * e1[0] + p[1] * e1[1] + p[2] * e1[2]) / den;
        double y = (q[0] * s[0] + q[1] * s[1] + q[2] * s[2]) / den;
        double z = (p[0] * d[0] + p[1] * d[1] + p[2] * d[2]) / den;
        if (x >= 0.0 && y >= 0.0 && z >= 0.0 && y + z <= 1.0 && x > tMin && x < tMax) {
            /* an entry with the winner's vertices is the same triangle (a
             * spatial split stores it in two leaves): not a second hit */
            if (bi >= 0 && x == best && same_vertices(t, &tris[bi])) continue;
            if (x < best) { second = best; best = x; bi = (int32_t)i; }
            else if (x < second) second = x;
        }
    }
    *out_ptr = bi; *out_t = best; *out_t2 = second;
}

/* ---------------------------------------------------------------------- */
/* Batch drivers on pthreads                                               */
/* ---------------------------------------------------------------------- */
enum { K_CLOSEST_CPU, K_ANY_CPU, K_CLOSEST_GLSL, K_ANY_GLSL, K_F64 };

typedef struct {
    int kind;
    const aeo_node* nodes; uint32_t n_nodes;
    const aeo_tri* tris; uint32_t n_tris;
    const float* rays; uint32_t begin, end;
    int32_t* ptr; float* tuv; uint8_t* occ; uint32_t* nf; uint32_t* tf;
    double* t64; double* t64b;
    uint32_t* flags; float* second;
} job_t;

static void* run_job(void* arg) {
    job_t* j = (job_t*)arg;
    size_t cap = (size_t)j->n_nodes + 64;
    void* stack = malloc(cap * sizeof(cpu_entry));
    for (uint32_t i = j->begin; i < j->end; i++) {
        const float* r = j->rays + (size_t)i * 8;
        switch (j->kind) {
        case K_CLOSEST_CPU:
            closest_cpu_one(j->nodes, j->n_nodes, j->tris, r, (cpu_entry*)stack, &j->ptr[i], &j->tuv[(size_t)i * 3]);
            break;
        case K_ANY_CPU:
            j->occ[i] = (uint8_t)any_cpu_one(j->nodes, j->n_nodes, j->tris, r, (int32_t*)stack);
            break;
        case K_CLOSEST_GLSL:
            closest_glsl_one(j->nodes, j->n_nodes, j->tris, r, (int32_t*)stack, &j->ptr[i], &j->tuv[(size_t)i * 3],
                             j->nf ? &j->nf[i] : NULL, j->tf ? &j->tf[i] : NULL,
                             j->flags ? &j->flags[i] : NULL, j->second ? &j->second[i] : NULL);
            break;
        case K_ANY_GLSL:
            j->occ[i] = (uint8_t)any_glsl_one(j->nodes, j->n_nodes, j->tris, r, (int32_t*)stack,
                                              j->nf ? &j->nf[i] : NULL, j->tf ? &j->tf[i] : NULL);
            break;
        case K_F64:
            closest_f64_one(j->tris, j->n_tris, r, &j->ptr[i], &j->t64[i], &j->t64b[i]);
            break;
        }
    }
    free(stack);
    return NULL;
}

static void run_batch(job_t proto, uint32_t n, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    job_t jobs[256];
    uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    int started = 0;
    for (int t = 0; t < threads; t++) {
        uint32_t b = (uint32_t)t * chunk;
        if (b >= n) break;
        uint32_t e = b + chunk < n ? b + chunk : n;
        jobs[t] = proto; jobs[t].begin = b; jobs[t].end = e;
        if (threads == 1) { run_job(&jobs[t]); continue; }
        pthread_create(&th[t], NULL, run_job, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

void aeo_closest_cpu(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                     const float* rays, uint32_t n_rays, int threads, int32_t* tri_ptr, float* tuv) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_CLOSEST_CPU; p.nodes = nodes; p.n_nodes = n_nodes; p.tris = tris; p.n_tris = n_tris;
    p.rays = rays; p.ptr = tri_ptr; p.tuv = tuv;
    run_batch(p, n_rays, threads);
}

void aeo_any_cpu(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                 const float* rays, uint32_t n_rays, int threads, uint8_t* occluded) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_ANY_CPU; p.nodes = nodes; p.n_nodes = n_nodes; p.tris = tris; p.n_tris = n_tris;
    p.rays = rays; p.occ = occluded;
    run_batch(p, n_rays, threads);
}

void aeo_closest_glsl(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                      const float* rays, uint32_t n_rays, int threads,
                      int32_t* tri_ptr, float* tuv, uint32_t* node_fetches, uint32_t* tri_fetches) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_CLOSEST_GLSL; p.nodes = nodes; p.n_nodes = n_nodes; p.tris = tris; p.n_tris = n_tris;
    p.rays = rays; p.ptr = tri_ptr; p.tuv = tuv; p.nf = node_fetches; p.tf = tri_fetches;
    run_batch(p, n_rays, threads);
}

void aeo_closest_glsl_ties(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                           const float* rays, uint32_t n_rays, int threads,
                           int32_t* tri_ptr, float* tuv, uint32_t* flags, float* t_second) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_CLOSEST_GLSL; p.nodes = nodes; p.n_nodes = n_nodes; p.tris = tris; p.n_tris = n_tris;
    p.rays = rays; p.ptr = tri_ptr; p.tuv = tuv; p.flags = flags; p.second = t_second;
    run_batch(p, n_rays, threads);
}

void aeo_any_glsl(const aeo_node* nodes, uint32_t n_nodes, const aeo_tri* tris, uint32_t n_tris,
                  const float* rays, uint32_t n_rays, int threads, uint8_t* occluded,
                  uint32_t* node_fetches, uint32_t* tri_fetches) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_ANY_GLSL; p.nodes = nodes; p.n_nodes = n_nodes; p.tris = tris; p.n_tris = n_tris;
    p.rays = rays; p.occ = occluded; p.nf = node_fetches; p.tf = tri_fetches;
    run_batch(p, n_rays, threads);
}

void aeo_closest_f64_brute(const aeo_tri* tris, uint32_t n_tris, const float* rays, uint32_t n_rays,
                           int threads, int32_t* tri_ptr, double* t, double* t2) {
    job_t p; memset(&p, 0, sizeof(p));
    p.kind = K_F64; p.tris = tris; p.n_tris = n_tris; p.rays = rays; p.ptr = tri_ptr; p.t64 = t; p.t64b = t2;
    run_batch(p, n_rays, threads);
}

/* ---------------------------------------------------------------------- */
/* Path tracer restatement (statistical oracle of the GPU path tracer)     */
/* ---------------------------------------------------------------------- */

static inline uint32_t pcg_hash(uint32_t x) {
    uint32_t state = x * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
static inline float rand01(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = pcg_hash(a ^ pcg_hash(b ^ pcg_hash(c)));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}
static inline float prng(uint32_t pix, uint32_t sample, uint32_t bounce, uint32_t dim, uint32_t seed) {
    return rand01(pix, sample * 16u + bounce + (seed << 12), dim * 0x9E3779B9u + 0x7F4A7C15u);
}

static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vmul(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vmulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline v3 vnorm(v3 a) {
    float l2 = vdot(a, a);
    return vmul(a, l2 > 0.0f ? 1.0f / sqrtf(l2) : 0.0f);
}
static inline float sat(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
static inline float p5(float x) { return x * x * x * x * x; }

static v3 unpack10(float bits) {
    int32_t c;
    memcpy(&c, &bits, 4);
    return mk((float)((c >> 0) & 1023) / 1023.0f * 2.0f - 1.0f, (float)((c >> 10) & 1023) / 1023.0f * 2.0f - 1.0f,
              (float)((c >> 20) & 1023) / 1023.0f * 2.0f - 1.0f);
}

typedef struct {
    v3 base, emissive;
    float opacity, roughness, metalness, ao, reflectance;
    int twoSided;
} pt_mat;

typedef struct {
    v3 P, V, N, L, H, geoN, F0;
    float NdotL, LdotH, NdotH, NdotV, F90;
    pt_mat m;
} pt_surf;

static void pt_update(pt_surf* s) {   /* UpdateSurface, brdf/surface.hsh:25-41 */
    s->L = vnorm(s->L);
    s->V = vnorm(s->V);
    s->N = vnorm(s->N);
    s->H = vnorm(vadd(s->L, s->V));
    s->NdotL = sat(vdot(s->N, s->L));
    s->LdotH = sat(vdot(s->L, s->H));
    s->NdotH = sat(vdot(s->N, s->H));
    s->NdotV = sat(vdot(s->N, s->V));
    float f0 = 0.16f * s->m.reflectance * s->m.reflectance;
    s->F0 = vadd(vmul(mk(f0, f0, f0), 1.0f - s->m.metalness), vmul(s->m.base, s->m.metalness));
    s->F90 = sat(50.0f * (s->F0.x * 0.333f + s->F0.y * 0.333f + s->F0.z * 0.333f));
}

static v3 pt_fresnel(v3 F0, float F90, float c) {
    float k = p5(1.0f - c);
    return mk(F0.x + (F90 - F0.x) * k, F0.y + (F90 - F0.y) * k, F0.z + (F90 - F0.z) * k);
}
static float pt_disney(float NdotV, float NdotL, float LdotH, float lr) {
    float bias = 0.5f * lr, factor = 1.0f + (1.0f / 1.51f - 1.0f) * lr;
    float FD90 = bias + 2.0f * LdotH * LdotH * lr;
    return (1.0f + (FD90 - 1.0f) * p5(1.0f - NdotL)) * (1.0f + (FD90 - 1.0f) * p5(1.0f - NdotV)) * factor;
}
static float pt_vis_sep(float c, float a) { float a2 = a * a; return 2.0f * c / (c + sqrtf(a2 + (1.0f - a2) * c * c)); }
static float pt_vis_cor(float NdotL, float NdotV, float a) {
    float a2 = a * a;
    float gl = NdotV * sqrtf((-NdotL * a2 + NdotL) * NdotL + a2);
    float gv = NdotL * sqrtf((-NdotV * a2 + NdotV) * NdotV + a2);
    return 0.5f / (gl + gv + 0.0000001f);
}
static float pt_ggx(float NdotH, float a) {
    float a2 = a * a, f = (NdotH * a2 - NdotH) * NdotH + 1.0f;
    return a2 / (f * f + 0.0000001f) * 0.31830988618379067154f;
}
static v3 pt_eval_diffuse(const pt_surf* s) {
    float r = fmaxf(s->m.roughness * s->m.roughness, 0.00001f);
    return vmul(s->m.base, (1.0f - s->m.metalness) * pt_disney(s->NdotV, s->NdotL, s->LdotH, r) * 0.31830988618379067154f);
}
static v3 pt_eval_specular(const pt_surf* s) {
    float r = fmaxf(s->m.roughness * s->m.roughness, 0.00001f);
    return vmul(pt_fresnel(s->F0, s->F90, s->LdotH), pt_ggx(s->NdotH, r) * pt_vis_cor(s->NdotV, s->NdotL, r));
}
static float pt_sample_diffuse(pt_surf* s, float u0, float u1, v3* refl) {
    float th = sqrtf(u0), phi = 6.28318530717958647692f * u1;
    v3 up = fabsf(s->N.z) < 0.999f ? mk(0, 0, 1) : mk(1, 0, 0);
    v3 t = vnorm(vcross(up, s->N)), b = vcross(s->N, t);
    s->L = vnorm(vadd(vadd(vmul(t, th * cosf(phi)), vmul(b, th * sinf(phi))), vmul(s->N, sqrtf(fmaxf(0.0f, 1.0f - u0)))));
    pt_update(s);
    *refl = pt_eval_diffuse(s);
    return s->NdotL * 0.31830988618379067154f;
}
static float pt_sample_specular(pt_surf* s, float u0, float u1, v3* refl) {
    float alpha = s->m.roughness * s->m.roughness;
    s->V = vnorm(s->V);
    v3 N = vnorm(s->N);
    v3 up = fabsf(N.z) < 0.999f ? mk(0, 0, 1) : mk(1, 0, 0);
    v3 t = vnorm(vcross(up, N)), b = vnorm(vcross(N, t));
    v3 Vl = vnorm(mk(vdot(s->V, t), vdot(s->V, b), vdot(s->V, N)));
    Vl = vnorm(mk(Vl.x * alpha, Vl.y * alpha, Vl.z));
    float phi = 6.28318530717958647692f * u0;
    float z = (1.0f - u1) * (1.0f + Vl.z) - Vl.z;
    float rr = sqrtf(sat(1.0f - z * z));
    v3 c = mk(cosf(phi) * rr, sinf(phi) * rr, z);
    v3 Hh = vadd(c, Vl);
    v3 Ml = mk(Hh.x * alpha, Hh.y * alpha, fmaxf(Hh.z, 0.0f));
    v3 M = vnorm(vadd(vadd(vmul(t, Ml.x), vmul(b, Ml.y)), vmul(N, Ml.z)));
    s->L = vadd(vmul(M, 2.0f * vdot(s->V, M)), vmul(s->V, -1.0f));
    pt_update(s);
    *refl = mk(0, 0, 0);
    float pdf = 1.0f;
    if (s->NdotL > 0.0f && s->LdotH > 0.0f) {
        v3 F = pt_fresnel(s->F0, s->F90, s->LdotH);
        float Vis = pt_vis_cor(s->NdotV, s->NdotL, alpha);
        float G1 = pt_vis_sep(s->NdotV, alpha);
        pdf = G1 / (4.0f * fabsf(vdot(s->V, s->N)));
        *refl = vmul(F, Vis);
    }
    return pdf;
}

/* The shading functions above on rows of inputs, in the layouts of the
 * golden vectors written by the reference's own GLSL compiled on the host
 * (oracle/glsl/glsl_capi.cpp): surface rows V N L baseColor roughness
 * metalness reflectance. */
static pt_surf shade_surface(const float* r, int with_l) {
    pt_surf s;
    memset(&s, 0, sizeof(s));
    s.V = ld3(r);
    s.N = ld3(r + 3);
    s.L = with_l ? ld3(r + 6) : ld3(r + 3);
    s.m.base = ld3(r + 9);
    s.m.roughness = r[12];
    s.m.metalness = r[13];
    s.m.reflectance = r[14];
    s.m.opacity = 1.0f;
    s.m.ao = 1.0f;
    pt_update(&s);
    return s;
}

void aeo_shade_eval(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        pt_surf s = shade_surface(in + (size_t)i * 15, 1);
        float* o = out + (size_t)i * 16;
        v3 d = pt_eval_diffuse(&s), sp = pt_eval_specular(&s);
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = sp.x; o[4] = sp.y; o[5] = sp.z;
        o[6] = s.NdotL; o[7] = s.NdotV; o[8] = s.NdotH; o[9] = s.LdotH;
        o[10] = s.F0.x; o[11] = s.F0.y; o[12] = s.F0.z; o[13] = s.F90; o[14] = s.H.x; o[15] = s.H.y;
    }
}

void aeo_shade_sample(const float* in, int n, int specular, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + (size_t)i * 17;
        pt_surf s = shade_surface(r, 0);
        v3 refl;
        float pdf = specular ? pt_sample_specular(&s, r[15], r[16], &refl) : pt_sample_diffuse(&s, r[15], r[16], &refl);
        float* o = out + (size_t)i * 8;
        o[0] = s.L.x; o[1] = s.L.y; o[2] = s.L.z; o[3] = pdf;
        o[4] = refl.x; o[5] = refl.y; o[6] = refl.z; o[7] = s.NdotL;
    }
}

/* The BRDF evaluation from given surface terms: rows NdotL NdotV NdotH LdotH
 * F0(3) F90 baseColor(3) roughness metalness -> diffuse(3) specular(3). */
void aeo_shade_eval_terms(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + (size_t)i * 13;
        pt_surf s;
        memset(&s, 0, sizeof(s));
        s.NdotL = r[0]; s.NdotV = r[1]; s.NdotH = r[2]; s.LdotH = r[3];
        s.F0 = ld3(r + 4); s.F90 = r[7];
        s.m.base = ld3(r + 8); s.m.roughness = r[11]; s.m.metalness = r[12];
        v3 d = pt_eval_diffuse(&s), sp = pt_eval_specular(&s);
        float* o = out + (size_t)i * 6;
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = sp.x; o[4] = sp.y; o[5] = sp.z;
    }
}

/* The point and normal of a triangle light at (r0, r1) as pt_sample_light
 * forms them (SampleTriangleLight, lights.hsh:11-29), pdf = 1 / area. */
void aeo_shade_triangle_light(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + (size_t)i * 24;
        float lu = 1.0f - sqrtf(r[19]), lv = r[20] * sqrtf(r[19]), lw = 1.0f - lu - lv;
        v3 P = vadd(vadd(vmul(ld3(r), lu), vmul(ld3(r + 3), lv)), vmul(ld3(r + 6), lw));
        v3 N = vadd(vadd(vmul(ld3(r + 9), lu), vmul(ld3(r + 12), lv)), vmul(ld3(r + 15), lw));
        float* o = out + (size_t)i * 7;
        o[0] = P.x; o[1] = P.y; o[2] = P.z; o[3] = N.x; o[4] = N.y; o[5] = N.z; o[6] = 1.0f / r[18];
    }
}

/* The triangle and slab tests of the shader query on rows: origin direction
 * v0 v1 v2 -> hit t u v; origin direction min max tmin tmax -> hit dist. */
void aeo_shade_intersect_triangle(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + (size_t)i * 15;
        aeo_tri t;
        memcpy(t.v0, r + 6, 12); memcpy(t.v1, r + 9, 12); memcpy(t.v2, r + 12, 12);
        float st, su, sv;
        int hit = tri_test(ld3(r), ld3(r + 3), &t, &st, &su, &sv);
        float* o = out + (size_t)i * 4;
        o[0] = hit ? 1.0f : 0.0f; o[1] = st; o[2] = su; o[3] = sv;
    }
}

void aeo_shade_intersect_aabb(const float* in, int n, float* out) {
    for (int i = 0; i < n; i++) {
        const float* r = in + (size_t)i * 14;
        float dist;
        int hit = box_glsl(ld3(r), ld3(r + 3), r[12], r[13], r + 6, r + 9, &dist);
        out[(size_t)i * 2] = hit ? 1.0f : 0.0f;
        out[(size_t)i * 2 + 1] = dist;
    }
}

typedef struct {
    v3 v0, v1, v2, n0, n1, n2;
    int material;
} pt_tri;

static v3 xpoint(const float* m, v3 p) {
    return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
static v3 xdir(const float* m, v3 p) {
    return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z, m[4] * p.x + m[5] * p.y + m[6] * p.z,
              m[8] * p.x + m[9] * p.y + m[10] * p.z);
}

typedef struct {
    scene_t sc;
    const float* inst_model;
    const float* materials;
    const float* lights;
    uint32_t n_lights;
    const aeo_texture* textures; uint32_t n_textures;   /* surface textures (GetSurfaceParameters) */
    uint32_t tex_level;                                  /* their mip level (textureLevel) */
    const float* cam;
    uint32_t width, height, spp, sample_offset, max_bounces, seed;
    float epsilon;
    const float* env;      /* constant environment radiance of a miss (rayHit.csh:166-171), or NULL */
    scene_t tsc;           /* the scene with its materials: the transparency variants */
    int transparent;       /* a shading triangle's opacity is not 1: trace with the opacity check */
    double* accum;
    uint32_t begin, end;
    size_t stack_cap;
} pt_job_t;

static pt_tri pt_load_tri(const pt_job_t* j, int32_t inst, int32_t tri) {
    const aeo_instance* in = &j->sc.inst[inst];
    const aeo_mesh* mesh = &j->sc.meshes[in->meshOffset];
    const float* t = mesh->shading + (size_t)tri * 24;
    const float* m = j->inst_model + (size_t)inst * 12;
    pt_tri r;
    r.v0 = xpoint(m, ld3(t));
    r.v1 = xpoint(m, ld3(t + 4));
    r.v2 = xpoint(m, ld3(t + 8));
    r.n0 = vnorm(xdir(m, unpack10(t[3])));
    r.n1 = vnorm(xdir(m, unpack10(t[7])));
    r.n2 = vnorm(xdir(m, unpack10(t[11])));
    int32_t mi;
    memcpy(&mi, &t[15], 4);
    r.material = mi + in->materialOffset;
    return r;
}

static pt_mat pt_load_mat(const float* m) {
    pt_mat r;
    r.base = mk(m[1], m[2], m[3]);
    r.emissive = mk(m[4], m[5], m[6]);
    r.opacity = m[7]; r.roughness = m[8]; r.metalness = m[9]; r.ao = m[10]; r.reflectance = m[11];
    memcpy(&r.twoSided, &m[14], 4);
    return r;
}

/* All four channels of a texel as the sampler returns them: R8 (r, 0, 0, 1),
 * RGBA8 (r, g, b, a), R32F (r, 0, 0, 1). */
static void texel_rgba(const aeo_texture* t, uint32_t x, uint32_t y, float c[4]) {
    const uint32_t texel = t->format == 0 ? 1u : 4u;
    const uint32_t pitch = t->row_pitch ? t->row_pitch : t->width * texel;
    const uint8_t* row = (const uint8_t*)t->texels + (size_t)y * pitch;
    c[1] = c[2] = 0.0f;
    c[3] = 1.0f;
    if (t->format == 0) {
        c[0] = (float)row[x] / 255.0f;
    } else if (t->format == 1) {
        for (int k = 0; k < 4; k++) c[k] = (float)row[(size_t)x * 4 + k] / 255.0f;
    } else {
        memcpy(&c[0], row + (size_t)x * 4, 4);
    }
}

/* textureLod(...) with all channels filtered like aeo_sample_r_bilinear's
 * first; (1, 1, 1, 1) for a negative or out-of-range id (texture.hsh:9-60). */
/* Mip level `level` of texture t, clamped to the levels given. */
static const aeo_texture* tex_at_level(const aeo_texture* t, uint32_t level) {
    if (level == 0 || t->n_mips == 0) return t;
    return &t->mips[(level < t->n_mips ? level : t->n_mips) - 1];
}

/* aeo_sample_r_bilinear at mip level `level` */
static float sample_r_level(const aeo_texture* textures, uint32_t n_textures, int32_t id, float u, float v,
                            uint32_t level) {
    if (id < 0 || (uint32_t)id >= n_textures) return 1.0f;
    return aeo_sample_r_bilinear(tex_at_level(&textures[id], level), 1, 0, u, v);
}

static void sample_rgba_bilinear(const aeo_texture* textures, uint32_t n_textures, int32_t id, float u, float v,
                                 uint32_t level, float out[4]) {
    if (id < 0 || (uint32_t)id >= n_textures) {
        out[0] = out[1] = out[2] = out[3] = 1.0f;
        return;
    }
    const aeo_texture* t = tex_at_level(&textures[id], level);
    uint32_t x0, x1, y0, y1;
    float a, b;
    tex_axis(u, t->width, &x0, &x1, &a);
    tex_axis(v, t->height, &y0, &y1, &b);
    float c00[4], c10[4], c01[4], c11[4];
    texel_rgba(t, x0, y0, c00);
    texel_rgba(t, x1, y0, c10);
    texel_rgba(t, x0, y1, c01);
    texel_rgba(t, x1, y1, c11);
    const float ia = 1.0f - a, ib = 1.0f - b;
    for (int k = 0; k < 4; k++) {
        float r = (ia * ib) * c00[k];
        r = r + (a * ib) * c10[k];
        r = r + (ia * b) * c01[k];
        out[k] = r + (a * b) * c11[k];
    }
}

static float unorm8(uint32_t c, int k) { return (float)((c >> (8 * k)) & 255u) / 255.0f; }

/* The material terms of GetSurfaceParameters (surface.hsh:83-124) at
 * barycentrics (r, s, t): vertex colours, base colour / opacity / roughness /
 * metalness / ao textures and the normal map, level 0.  N: the interpolated
 * normal, in and out. */
static void pt_surface_textures(const pt_job_t* j, int32_t inst, int32_t tp, const float* mw, float r, float s,
                                float t, pt_mat* m, v3* N) {
    const aeo_instance* in = &j->sc.inst[inst];
    const float* g = j->sc.meshes[in->meshOffset].shading + (size_t)tp * 24;
    float u0, v0, u1, v1, u2, v2;
    half2_of(g[12], &u0, &v0);
    half2_of(g[13], &u1, &v1);
    half2_of(g[14], &u2, &v2);
    int32_t w[23];
    memcpy(w, mw, sizeof w);
    const float tu = r * u0 + s * u1 + t * u2;
    float tv = r * v0 + s * v1 + t * v2;
    if (w[13] > 0) tv = 1.0f - tv;
    if (w[16] > 0) {
        uint32_t c0, c1, c2;
        memcpy(&c0, &g[20], 4);
        memcpy(&c1, &g[21], 4);
        memcpy(&c2, &g[22], 4);
        m->base = vmulv(m->base, mk(r * unorm8(c0, 0) + s * unorm8(c1, 0) + t * unorm8(c2, 0),
                                    r * unorm8(c0, 1) + s * unorm8(c1, 1) + t * unorm8(c2, 1),
                                    r * unorm8(c0, 2) + s * unorm8(c1, 2) + t * unorm8(c2, 2)));
    }
    float c[4];
    const uint32_t lv = j->tex_level;
    sample_rgba_bilinear(j->textures, j->n_textures, w[17], tu, tv, lv, c);
    m->base = vmulv(m->base, mk(c[0], c[1], c[2]));
    m->opacity *= sample_r_level(j->textures, j->n_textures, w[18], tu, tv, lv);
    m->roughness *= sample_r_level(j->textures, j->n_textures, w[20], tu, tv, lv);
    m->metalness *= sample_r_level(j->textures, j->n_textures, w[21], tu, tv, lv);
    m->ao *= sample_r_level(j->textures, j->n_textures, w[22], tu, tv, lv);
    if (w[19] >= 0) {
        const float* mm = j->inst_model + (size_t)inst * 12;
        v3 T = vnorm(xdir(mm, unpack10(g[16])));
        v3 B = vnorm(xdir(mm, unpack10(g[17])));
        if (!(w[13] > 0)) B = vmul(B, -1.0f);
        sample_rgba_bilinear(j->textures, j->n_textures, w[19], tu, tv, lv, c);
        v3 n = vadd(vadd(vmul(T, 2.0f * c[0] - 1.0f), vmul(B, 2.0f * c[1] - 1.0f)), vmul(*N, 2.0f * c[2] - 1.0f));
        n = vmul(n, 1.0f / fmaxf(sqrtf(vdot(n, n)), 0.00001f));
        const float wgt = sat(mw[12]);
        *N = vadd(vmul(*N, 1.0f - wgt), vmul(n, wgt));
    }
}

/* GetSurfaceParameters (raytracer/surface.hsh:63-140) at a closest hit;
 * returns backfaceHit (surface.hsh:99). */
static int pt_make_surface(const pt_job_t* j, v3 ro, v3 rd, int32_t tp, int32_t ino, const float* tuv,
                           pt_surf* sf) {
    pt_tri tri = pt_load_tri(j, ino, tp);
    float s = tuv[1], t = tuv[2], r = 1.0f - s - t;
    const float* mw = j->materials + (size_t)tri.material * 23;
    sf->m = pt_load_mat(mw);
    sf->P = vadd(ro, vmul(rd, tuv[0]));
    v3 N = vnorm(vadd(vadd(vmul(tri.n0, r), vmul(tri.n1, s)), vmul(tri.n2, t)));
    v3 triN = vnorm(vcross(sub(tri.v0, tri.v1), sub(tri.v0, tri.v2)));
    int flip = vdot(triN, rd) > 0.0f;
    int32_t cull;
    memcpy(&cull, &mw[15], 4);
    int backface = sf->m.twoSided > 0 || cull == 0 ? 0 : flip;
    if (flip && sf->m.twoSided > 0) triN = vmul(triN, -1.0f);
    {
        int32_t w[23];
        memcpy(w, mw, sizeof w);
        if (w[16] > 0 || (w[17] & w[18] & w[19] & w[20] & w[21] & w[22]) >= 0)
            pt_surface_textures(j, ino, tp, mw, r, s, t, &sf->m, &N);
    }
    if (vdot(N, triN) < 0.0f && sf->m.twoSided > 0) N = vmul(N, -1.0f);
    sf->V = vmul(rd, -1.0f);
    sf->N = vnorm(N);
    sf->geoN = triN;
    sf->L = sf->N;
    /* NdotV, F0 and F90 do not depend on L: set here as the light sample's
     * UpdateSurface would, so the continuation's lobe choice is defined
     * without lights */
    pt_update(sf);
    return backface;
}

/* GetLight + SampleLight (raytracer/direct.hsh:12-86): one light by streaming
 * weighted selection, a uniform point on it, sf->L towards it (UpdateSurface).
 * 0 when there are no lights. */
static int pt_sample_light(const pt_job_t* j, pt_surf* sf, uint32_t pix, uint32_t sample, uint32_t bounce,
                           uint32_t seed, v3* radiance, float* lightPdf, float* solidAngle, float* dist) {
    if (j->n_lights == 0) return 0;
    const float* sel = NULL;
    float selW = 0.0f, total = 0.0f;
    for (uint32_t li = 0; li < j->n_lights; li++) {
        const float* L = j->lights + (size_t)li * 16;
        uint32_t data;
        memcpy(&data, &L[12], 4);
        float bright = (L[8] + L[9] + L[10]) * 0.33333f;
        float w = 1.0f;
        if ((data >> 28) == 1u) {
            v3 toL = sub(ld3(L), sf->P);
            float d2 = vdot(toL, toL);
            float NdotL = fmaxf(vdot(ld3(L + 4), vmul(vnorm(toL), -1.0f)), 0.0f);
            w = bright * L[14] * NdotL / d2;
        } else {
            w = bright;
        }
        w = fminf(fmaxf(w, 0.0000001f), 1.0f);
        total += w;
        if (prng(pix, sample, bounce, 16u + li, seed) < w / total) { selW = w; sel = L; }
    }
    uint32_t data;
    memcpy(&data, &sel[12], 4);
    *lightPdf = selW / total * sel[13];
    *solidAngle = 1.0f;
    *dist = 1e12f;
    *radiance = ld3(sel + 8);
    if ((data >> 28) == 1u) {
        float r0 = prng(pix, sample, bounce, 1, seed), r1 = prng(pix, sample, bounce, 2, seed);
        int32_t linst;
        memcpy(&linst, &sel[15], 4);
        pt_tri lt = pt_load_tri(j, linst, (int32_t)(data & 0x0FFFFFFFu));
        float lu = 1.0f - sqrtf(r0), lv = r1 * sqrtf(r0), lw = 1.0f - lu - lv;
        v3 LP = vadd(vadd(vmul(lt.v0, lu), vmul(lt.v1, lv)), vmul(lt.v2, lw));
        v3 LN = vadd(vadd(vmul(lt.n0, lu), vmul(lt.n1, lv)), vmul(lt.n2, lw));
        v3 toL = sub(LP, sf->P);
        float d2 = vdot(toL, toL);
        *dist = sqrtf(d2);
        sf->L = vmul(toL, 1.0f / *dist);
        pt_update(sf);
        float NdotLl = fmaxf(vdot(LN, vmul(sf->L, -1.0f)), 0.0f);
        *solidAngle = NdotLl / (d2 * (1.0f / sel[14]));
    } else {
        sf->L = vnorm(vmul(ld3(sel + 4), -1.0f));
        pt_update(sf);
    }
    return 1;
}

static void pt_pixel(const pt_job_t* j, uint32_t pix, int32_t* stack, double* out) {
    const float* c = j->cam;
    for (uint32_t si = 0; si < j->spp; si++) {
        uint32_t sample = j->sample_offset + si;
        float jx = prng(pix, sample, 15, 0, j->seed), jy = prng(pix, sample, 15, 1, j->seed);
        float u = ((float)(pix % j->width) + jx) / (float)j->width;
        float v = ((float)(pix / j->width) + jy) / (float)j->height;
        v3 ro = mk(c[0], c[1], c[2]);
        v3 rd = vnorm(mk(c[3] + c[6] * u + c[9] * v - c[0], c[4] + c[7] * u + c[10] * v - c[1],
                         c[5] + c[8] * u + c[11] * v - c[2]));
        v3 thr = mk(1, 1, 1);
        for (uint32_t bounce = 0; bounce <= j->max_bounces; bounce++) {
            float r8[8] = { ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, 0.0f, 1e12f };
            int32_t tp, ino;
            float tuv[3];
            /* the engine's opacity check (PathTracingRenderer.cpp:186): closest
             * hits skip surfaces of opacity 0 */
            scene_closest_one(j->transparent ? &j->tsc : &j->sc, r8, 128u, stack, &tp, &ino, tuv, NULL, NULL);
            if (tp < 0) {
                /* the environment, clamped per channel (rayHit.csh:166-171) */
                if (j->env) {
                    out[0] += fminf(j->env[0] * thr.x, 10.0f);
                    out[1] += fminf(j->env[1] * thr.y, 10.0f);
                    out[2] += fminf(j->env[2] * thr.z, 10.0f);
                }
                break;
            }
            pt_surf sf;
            pt_make_surface(j, ro, rd, tp, ino, tuv, &sf);
            if (bounce == 0 && sf.m.emissive.x + sf.m.emissive.y + sf.m.emissive.z > 0.0f) {
                out[0] += sf.m.emissive.x; out[1] += sf.m.emissive.y; out[2] += sf.m.emissive.z;
            }
            v3 lrad;
            float lightPdf, solidAngle, dist;
            if (pt_sample_light(j, &sf, pix, sample, bounce, j->seed, &lrad, &lightPdf, &solidAngle, &dist)) {
                v3 refl = vmul(vadd(pt_eval_diffuse(&sf), pt_eval_specular(&sf)), sf.m.opacity);
                v3 contrib = vmul(vmulv(vmul(thr, sf.m.opacity), vmulv(refl, lrad)),
                                  solidAngle * sf.NdotL / lightPdf);
                if (sf.NdotL > 0.0f && lightPdf > 0.0f && contrib.x + contrib.y + contrib.z > 0.0f) {
                    v3 so = vadd(sf.P, vmul(sf.N, j->epsilon));
                    float s8[8] = { so.x, so.y, so.z, sf.L.x, sf.L.y, sf.L.z, 0.0f, dist - 2.0f * j->epsilon };
                    if (j->transparent) {
                        /* CheckVisibility: HitAnyTransparency (rayHit.csh:327-338) */
                        float vis = scene_any_transparency_one(&j->tsc, s8, 64u, stack);
                        if (vis > 0.0f) {
                            out[0] += contrib.x * vis; out[1] += contrib.y * vis; out[2] += contrib.z * vis;
                        }
                    } else if (!scene_any_one(&j->sc, s8, 64u, stack)) {
                        out[0] += contrib.x; out[1] += contrib.y; out[2] += contrib.z;
                    }
                }
            }
            if (bounce >= j->max_bounces) break;
            /* EvaluateIndirectLight (rayHit.csh:237-325): a partially opaque
             * surface is passed straight through with chance
             * clamp(1 - opacity, 0.1, 0.9) (:252-253, :282-291) */
            float refractChance = sf.m.opacity == 1.0f ? 0.0f : fminf(fmaxf(1.0f - sf.m.opacity, 0.1f), 0.9f);
            v3 refl, origin;
            float pdf;
            int through = 0;
            if (prng(pix, sample, bounce, 3, j->seed) >= refractChance) {
                v3 F = pt_fresnel(sf.F0, sf.F90, sf.NdotV);
                float specChance = fminf(fmaxf((F.x + F.y + F.z) * 0.33333f, 0.1f), 0.9f);
                float rnd = prng(pix, sample, bounce, 4, j->seed);
                float u0 = prng(pix, sample, bounce, 5, j->seed), u1 = prng(pix, sample, bounce, 6, j->seed);
                if (rnd < specChance) {
                    pdf = pt_sample_specular(&sf, u0, u1, &refl);
                    refl = vmul(refl, sf.m.opacity);
                    pdf *= specChance;
                } else {
                    pdf = pt_sample_diffuse(&sf, u0, u1, &refl);
                    refl = vmul(refl, (1.0f - sf.m.metalness) * sf.m.opacity);
                    pdf *= (1.0f - specChance);
                }
                pdf *= 1.0f - refractChance;
                origin = vadd(sf.P, vmul(sf.V, j->epsilon));
            } else {
                sf.L = vmul(sf.V, -1.0f);
                pdf = refractChance;
                refl = mk(1.0f - sf.m.opacity, 1.0f - sf.m.opacity, 1.0f - sf.m.opacity);
                sf.NdotL = 1.0f;
                origin = sub(sf.P, vmul(sf.N, j->epsilon));
                through = 1;
            }
            if (pdf > 0.0f && refl.x + refl.y + refl.z > 0.0f) thr = vmul(vmulv(thr, refl), sf.NdotL / pdf);
            else thr = mk(0, 0, 0);
            v3 dir = vnorm(sf.L);
            thr = vmul(thr, sf.m.ao);
            float prob = fminf(fmaxf(fmaxf(thr.x, fmaxf(thr.y, thr.z)), 0.01f), 0.99f);
            prob = bounce < 3 ? fminf(3.0f * prob, 1.0f) : prob;
            /* a pass-through is exempt from the below-surface termination (:318) */
            int alive = thr.x + thr.y + thr.z > 0.0f && prng(pix, sample, bounce, 7, j->seed) <= prob &&
                        (through || vdot(dir, sf.geoN) > 0.0f);
            if (!alive) break;
            thr = vmul(thr, 1.0f / prob);
            ro = origin;
            rd = dir;
        }
    }
}

static void* run_pt_job(void* arg) {
    pt_job_t* j = (pt_job_t*)arg;
    int32_t* stack = (int32_t*)malloc(j->stack_cap * sizeof(int32_t));
    for (uint32_t pix = j->begin; pix < j->end; pix++) {
        double o[3] = { 0, 0, 0 };
        pt_pixel(j, pix, stack, o);
        j->accum[(size_t)pix * 3 + 0] += o[0];
        j->accum[(size_t)pix * 3 + 1] += o[1];
        j->accum[(size_t)pix * 3 + 2] += o[2];
    }
    free(stack);
    return NULL;
}

void aeo_pathtrace(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, const float* inst_model,
                   uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes, const float* materials,
                   const float* lights, uint32_t n_lights, const aeo_texture* textures, uint32_t n_textures,
                   const float* cam, uint32_t width, uint32_t height,
                   uint32_t spp, uint32_t sample_offset, uint32_t max_bounces, uint32_t seed, float epsilon,
                   int threads, double* accum) {
    aeo_pathtrace_env(tlas, n_tlas, inst, inst_model, n_inst, meshes, n_meshes, materials, 0xFFFFFFFFu, lights,
                      n_lights, textures, n_textures, cam, width, height, spp, sample_offset, max_bounces, seed, epsilon,
                      NULL, threads, accum);
}

void aeo_pathtrace_env(const aeo_node* tlas, uint32_t n_tlas, const aeo_instance* inst, const float* inst_model,
                       uint32_t n_inst, const aeo_mesh* meshes, uint32_t n_meshes, const float* materials,
                       uint32_t n_materials, const float* lights, uint32_t n_lights, const aeo_texture* textures,
                       uint32_t n_textures, const float* cam, uint32_t width, uint32_t height,
                       uint32_t spp, uint32_t sample_offset, uint32_t max_bounces, uint32_t seed, float epsilon,
                       const float* env, int threads, double* accum) {
    pt_job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.env = env;
    {
        scene_t tsc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, materials, n_materials, textures, n_textures };
        proto.tsc = tsc;
    }
    for (uint32_t m = 0; m < n_meshes && !proto.transparent; m++)
        if (meshes[m].shading)
            for (uint32_t i = 0; i < meshes[m].n_tris && !proto.transparent; i++)
                proto.transparent = meshes[m].shading[(size_t)i * 24 + 23] != 1.0f;
    scene_t sc = { tlas, n_tlas, inst, n_inst, meshes, n_meshes, NULL };
    proto.sc = sc;
    proto.inst_model = inst_model;
    proto.materials = materials;
    proto.lights = lights;
    proto.n_lights = n_lights;
    proto.textures = textures;
    proto.n_textures = n_textures;
    proto.cam = cam;
    proto.width = width; proto.height = height; proto.spp = spp; proto.sample_offset = sample_offset;
    proto.max_bounces = max_bounces; proto.seed = seed; proto.epsilon = epsilon;
    proto.accum = accum;
    proto.stack_cap = scene_stack_cap(&proto.sc);
    uint32_t n = width * height;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    pt_job_t jobs[256];
    uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    int started = 0;
    for (int t = 0; t < threads; t++) {
        uint32_t b = (uint32_t)t * chunk;
        if (b >= n) break;
        jobs[t] = proto;
        jobs[t].begin = b;
        jobs[t].end = b + chunk < n ? b + chunk : n;
        pthread_create(&th[t], NULL, run_pt_job, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------------- */
/* The traversal's other consumers: RTAO, reflections, RTGI, DDGI probe     */
/* rays (statistical / tolerance oracle of the library's passes)            */
/* ---------------------------------------------------------------------- */

#define PASS_EPS 0.1f          /* EPSILON, raytracer/common.hsh:9 */
#define PASS_INF 1e12f         /* INF, raytracer/common.hsh:8 */
#define PASS_SAMPLE_SLOT 13u
#define PASS_LIGHT_SLOT 14u

enum { PASS_AO = 0, PASS_REFL = 1, PASS_GI = 2, PASS_DDGI = 3 };

typedef struct {
    pt_job_t j;               /* scene (opaque), instance transforms, materials, lights */
    scene_t tsc;              /* the same scene for the transparency variants */
    const aeo_gbuffer* gb;
    const aeo_ddgi_probes* dp;
    const aeo_pass_params* pp;
    int kind;
    float* out;
    uint32_t begin, end;
} pass_job_t;

static float4_t mat4_col(const float* m, float x, float y, float z, float w) {
    float4_t r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

/* DecodeNormal, common/normalencode.hsh:18-30 */
static v3 decode_oct(float cx, float cy) {
    float y = 1.0f - (fabsf(cx) + fabsf(cy));
    if (y < 0.0f) {
        float ox = cx, oy = cy;
        cx = (ox >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(oy));
        cy = (oy >= 0.0f ? 1.0f : -1.0f) * (1.0f - fabsf(ox));
    }
    return vnorm(mk(cx, y, cy));
}

/* SampleBlueNoise, common/bluenoise.hsh:9-32 (Heitz, Belcour, Ostromoukhov,
 * Coeurjolly, Iehl 2019), with the RGBA8 textures read as unorm floats
 * (c / 255) the way the shader's sampler returns them. */
static int blue_noise_texel(const uint8_t* t, int index, int channel) {
    float v = (float)t[(size_t)index * 4 + channel] / 255.0f * 256.0f;
    return (int)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
}

static float blue_noise(const aeo_gbuffer* g, uint32_t px, uint32_t py, int sample_index, int dim) {
    int pixel = (int)((py % 128u) * 128u + (px % 128u));
    sample_index = sample_index % 256;
    dim = dim % 4;
    int ranked = sample_index ^ blue_noise_texel(g->scrambling_ranking, pixel, 2);
    int value = blue_noise_texel(g->sobol_sequence, ranked, dim);
    value = value ^ blue_noise_texel(g->scrambling_ranking, pixel, dim % 2);
    return (0.5f + (float)value) / 256.0f;
}

static void frame_of(v3 N, v3* t, v3* b, int normalize_b) {
    v3 up = fabsf(N.z) < 0.999f ? mk(0, 0, 1) : mk(1, 0, 0);
    *t = vnorm(vcross(up, N));
    *b = normalize_b ? vnorm(vcross(N, *t)) : vcross(N, *t);
}

/* ImportanceSampleCosDir, brdf/importanceSample.hsh:82-101 */
static v3 cos_dir(v3 N, float u0, float u1) {
    float th = sqrtf(u0), phi = 6.28318530717958647692f * u1;
    v3 t, b;
    frame_of(N, &t, &b, 0);
    return vnorm(vadd(vadd(vmul(t, th * cosf(phi)), vmul(b, th * sinf(phi))), vmul(N, sqrtf(1.0f - u0))));
}

/* ImportanceSampleGGXVNDF, brdf/importanceSample.hsh:37-80 (alpha = roughness^2) */
static v3 vndf_dir(v3 N, v3 V, float alpha, float u0, float u1) {
    v3 t, b;
    frame_of(N, &t, &b, 1);
    v3 Vl = vnorm(mk(vdot(V, t) * alpha, vdot(V, b) * alpha, vdot(V, N)));
    float phi = 6.28318530717958647692f * u0;
    float z = (1.0f - u1) * (1.0f + Vl.z) + -Vl.z;
    float s = sqrtf(fminf(fmaxf(1.0f - z * z, 0.0f), 1.0f));
    v3 Hh = mk(cosf(phi) * s + Vl.x, sinf(phi) * s + Vl.y, z + Vl.z);
    v3 H = vnorm(vadd(vadd(vmul(t, Hh.x * alpha), vmul(b, Hh.y * alpha)), vmul(N, fmaxf(Hh.z, 0.0f))));
    return vnorm(sub(vmul(H, 2.0f * vdot(V, H)), V));
}

/* EvaluateHit of rtreflection.csh / rtgi.csh (diffuse + specular, visibility
 * by HitAnyTransparency) and ddgi/rayHit.csh (diffuse, HitAny; backface hits
 * give radiance 0 and a negative distance).  rgb + distance into out4. */
static void pass_eval_hit(const pass_job_t* p, v3 ro, v3 rd, uint32_t key, int32_t* stack, float* out4) {
    const aeo_pass_params* pp = p->pp;
    int opacity = (pp->flags & 1u) != 0;
    float r8[8] = { ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, 0.0f, PASS_INF };
    int32_t tp, ino;
    float tuv[3];
    scene_closest_one(opacity ? &p->tsc : &p->j.sc, r8, 128u, stack, &tp, &ino, tuv, NULL, NULL);
    v3 rad = mk(pp->environment[0], pp->environment[1], pp->environment[2]);
    float dist = tp >= 0 ? tuv[0] : PASS_INF;
    if (tp >= 0) {
        pt_surf sf;
        int backface = pt_make_surface(&p->j, ro, rd, tp, ino, tuv, &sf);
        if (p->kind == PASS_DDGI && backface) {
            rad = mk(0, 0, 0);
            dist = -dist;
        } else {
            rad = sf.m.emissive;
            v3 lrad;
            float lightPdf, solidAngle, ldist;
            if (pt_sample_light(&p->j, &sf, key, pp->frame_seed, PASS_LIGHT_SLOT, pp->seed, &lrad, &lightPdf,
                                &solidAngle, &ldist)) {
                v3 refl = p->kind == PASS_DDGI ? pt_eval_diffuse(&sf)
                                               : vadd(pt_eval_diffuse(&sf), pt_eval_specular(&sf));
                refl = vmul(refl, sf.m.opacity);
                v3 c = vmul(vmulv(refl, vmul(lrad, solidAngle)), sf.NdotL / lightPdf);
                /* CheckVisibility traces whenever NdotL > 0; the light term can
                 * be negative (a one-sided back face seen from behind gives
                 * NdotV < 0), and the shaders add it as it is */
                if (sf.NdotL > 0.0f && (c.x != 0.0f || c.y != 0.0f || c.z != 0.0f)) {
                    v3 so = vadd(sf.P, vmul(sf.N, PASS_EPS));
                    float s8[8] = { so.x, so.y, so.z, sf.L.x, sf.L.y, sf.L.z, 0.0f, ldist - 2.0f * PASS_EPS };
                    float vis;
                    if (p->kind == PASS_DDGI) vis = scene_any_one(&p->j.sc, s8, 64u, stack) ? 0.0f : 1.0f;
                    else vis = scene_any_transparency_one(&p->tsc, s8, 64u, stack);
                    rad = vadd(rad, vmul(c, vis));
                }
            }
        }
    }
    out4[0] = rad.x; out4[1] = rad.y; out4[2] = rad.z; out4[3] = dist;
}

static uint16_t half_of(float f) {   /* binary16, round to nearest even */
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7FFFFFFFu, r, rem, halfway;
    if (ax >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);
    if (ax < 0x38800000u) {
        if (ax < 0x33000000u) return (uint16_t)sign;
        uint32_t e = ax >> 23, m = (ax & 0x7FFFFFu) | 0x800000u, shift = 126u - e;
        r = m >> shift; rem = m & ((1u << shift) - 1u); halfway = 1u << (shift - 1u);
    } else {
        r = (ax - 0x38000000u) >> 13; rem = ax & 0x1FFFu; halfway = 0x1000u;
    }
    if (rem > halfway || (rem == halfway && (r & 1u))) r++;
    return (uint16_t)(sign | r);
}

static void pass_pixel(const pass_job_t* p, uint32_t pix, int32_t* stack) {
    const aeo_gbuffer* g = p->gb;
    const aeo_pass_params* pp = p->pp;
    uint32_t px = pix % g->width, py = pix / g->width;
    float depth = g->depth[pix];
    int traced = depth < 1.0f;
    float rough = 1.0f;
    if (p->kind == PASS_REFL) {
        rough = g->roughness[pix];
        traced = traced && rough <= 1.0f;
    }
    int emit = 0;
    v3 O = mk(0, 0, 0), L = mk(0, 0, 0);
    if (traced) {
        float tx, ty;
        if (g->half_res) {
            uint32_t off = g->offset ? (g->offset[pix] & 3u) : 0u;
            tx = (2.0f * (float)px + (float)(off & 1u) + 0.5f) / (2.0f * (float)g->width);
            ty = (2.0f * (float)py + (float)(off >> 1) + 0.5f) / (2.0f * (float)g->height);
        } else {
            tx = ((float)px + 0.5f) / (float)g->width;
            ty = ((float)py + 0.5f) / (float)g->height;
        }
        float4_t vs = mat4_col(g->ip_matrix, tx * 2.0f - 1.0f, ty * 2.0f - 1.0f, depth, 1.0f);
        v3 viewPos = mk(vs.x / vs.w, vs.y / vs.w, vs.z / vs.w);
        float4_t wp = mat4_col(g->iv_matrix, viewPos.x, viewPos.y, viewPos.z, 1.0f);
        float4_t vv = mat4_col(g->iv_matrix, viewPos.x, viewPos.y, viewPos.z, 0.0f);
        v3 vn = decode_oct(g->normal[(size_t)pix * 2], g->normal[(size_t)pix * 2 + 1]);
        float4_t wn = mat4_col(g->iv_matrix, vn.x, vn.y, vn.z, 0.0f);
        v3 P = mk(wp.x, wp.y, wp.z), N = vnorm(mk(wn.x, wn.y, wn.z));
        float u0, u1;
        if (g->samples) {
            u0 = g->samples[(size_t)pix * 2];
            u1 = g->samples[(size_t)pix * 2 + 1];
        } else if (g->scrambling_ranking) {
            /* int(frameSeed) % 256 for seeds below 2^31; above, the shader's
             * index is negative (a texel fetch out of range) */
            u0 = blue_noise(g, px, py, (int)(pp->frame_seed % 256u), 0);
            u1 = blue_noise(g, px, py, (int)(pp->frame_seed % 256u), 1);
        } else {
            u0 = prng(pix, pp->frame_seed, PASS_SAMPLE_SLOT, 0, pp->seed);
            u1 = prng(pix, pp->frame_seed, PASS_SAMPLE_SLOT, 1, pp->seed);
        }
        float viewLen = sqrtf(vdot(viewPos, viewPos));
        if (p->kind == PASS_AO) {
            L = vnorm(cos_dir(N, u0, u1));
            O = vadd(vadd(P, vmul(L, PASS_EPS)), vmul(N, PASS_EPS));
            emit = 1;
        } else {
            if (p->kind == PASS_REFL) {
                u1 *= (1.0f - pp->bias);
                v3 V = vnorm(mk(-vv.x, -vv.y, -vv.z));
                if (rough > 0.01f) {
                    L = vndf_dir(N, V, rough * rough, u0, u1);
                } else {
                    v3 I = vmul(V, -1.0f);
                    L = vnorm(sub(I, vmul(N, 2.0f * vdot(N, I))));
                }
            } else {
                u0 *= (1.0f - pp->bias);
                L = cos_dir(N, u0, u1);
            }
            int valid = !(isnan(L.x) && isnan(L.y) && isnan(L.z));
            if (p->kind == PASS_REFL) {
                float viewOffset = fmaxf(1.0f, viewLen) * 0.1f;
                O = vadd(vadd(P, vmul(L, PASS_EPS * 0.1f * viewOffset)), vmul(N, PASS_EPS * viewOffset * 0.1f));
                emit = valid && rough <= pp->roughness_cutoff;
            } else {
                float viewOffset = fmaxf(1.0f, viewLen);
                O = vadd(vadd(P, vmul(L, PASS_EPS * viewOffset * 0.01f)), vmul(N, PASS_EPS * 0.01f * viewOffset));
                emit = valid;
            }
        }
    }
    if (p->kind == PASS_AO) {
        float ao = 1.0f;
        if (emit) {
            float r8[8] = { O.x, O.y, O.z, L.x, L.y, L.z, 0.0f, pp->radius };
            float hit = (pp->flags & 1u) ? 1.0f - scene_any_transparency_one(&p->tsc, r8, 128u, stack)
                                         : (scene_any_one(&p->j.sc, r8, 128u, stack) ? 1.0f : 0.0f);
            ao = 1.0f - hit;
        }
        p->out[pix] = ao;
        return;
    }
    float* o4 = p->out + (size_t)pix * 4;
    o4[0] = o4[1] = o4[2] = 0.0f;
    o4[3] = 1.0f;
    if (!emit) return;
    float r4[4];
    pass_eval_hit(p, O, L, pix, stack, r4);
    float m = fmaxf(fmaxf(fmaxf(r4[0], fmaxf(r4[1], r4[2])), pp->radiance_limit), 0.01f);
    float s = pp->radiance_limit / m;
    o4[0] = r4[0] * s; o4[1] = r4[1] * s; o4[2] = r4[2] * s;
}

static void pass_probe_ray(const pass_job_t* p, uint32_t idx, int32_t* stack) {
    const aeo_ddgi_probes* d = p->dp;
    uint32_t probe = idx / d->ray_count, i = idx % d->ray_count;
    const float* pr = d->probes + (size_t)probe * 4;
    uint32_t state;
    memcpy(&state, &pr[3], 4);
    int inactive = state == 2u;
    uint32_t inactive_count = d->inactive_ray_count < d->ray_count ? d->inactive_ray_count : d->ray_count;
    if (i >= (inactive ? inactive_count : d->ray_count)) return;
    const float* v = (inactive ? d->ray_dirs_inactive : d->ray_dirs) + (size_t)i * 4;
    const float* m = d->rotation;
    v3 D = vnorm(mk(m[0] * v[0] + m[4] * v[1] + m[8] * v[2], m[1] * v[0] + m[5] * v[1] + m[9] * v[2],
                    m[2] * v[0] + m[6] * v[1] + m[10] * v[2]));
    float r4[4];
    pass_eval_hit(p, mk(pr[0], pr[1], pr[2]), D, idx, stack, r4);
    float rx = fminf(r4[0], 3200.0f), ry = fminf(r4[1], 3200.0f), rz = fminf(r4[2], 3200.0f);
    uint32_t w0 = (uint32_t)half_of(D.x) | ((uint32_t)half_of(D.y) << 16);
    uint32_t w1 = (uint32_t)half_of(rx) | ((uint32_t)half_of(ry) << 16);
    uint32_t w2 = (uint32_t)half_of(D.z) | ((uint32_t)half_of(rz) << 16);
    float* o = p->out + (size_t)idx * 4;
    memcpy(&o[0], &w0, 4);
    memcpy(&o[1], &w1, 4);
    memcpy(&o[2], &w2, 4);
    o[3] = r4[3];
}

static void* run_pass_job(void* arg) {
    pass_job_t* p = (pass_job_t*)arg;
    int32_t* stack = (int32_t*)malloc(p->j.stack_cap * sizeof(int32_t));
    for (uint32_t k = p->begin; k < p->end; k++) {
        if (p->kind == PASS_DDGI) pass_probe_ray(p, k, stack);
        else pass_pixel(p, k, stack);
    }
    free(stack);
    return NULL;
}

static void run_pass(const aeo_pass_scene* s, int kind, const aeo_gbuffer* gb, const aeo_ddgi_probes* dp,
                     const aeo_pass_params* pp, uint32_t n, int threads, float* out) {
    pass_job_t proto;
    memset(&proto, 0, sizeof(proto));
    scene_t sc = { s->tlas, s->n_tlas, s->inst, s->n_inst, s->meshes, s->n_meshes, NULL, 0, NULL, 0 };
    scene_t tsc = { s->tlas, s->n_tlas, s->inst, s->n_inst, s->meshes, s->n_meshes, s->materials, s->n_materials,
                    s->textures, s->n_textures };
    proto.j.sc = sc;
    proto.j.inst_model = s->inst_model;
    proto.j.materials = s->materials;
    proto.j.lights = s->lights;
    proto.j.n_lights = s->n_lights;
    proto.j.textures = s->textures;
    proto.j.n_textures = s->n_textures;
    proto.j.tex_level = kind == PASS_DDGI ? 4u : pp->texture_level;   /* ddgi/rayHit.csh:79 */
    proto.j.epsilon = PASS_EPS;
    proto.j.stack_cap = scene_stack_cap(&sc);
    proto.tsc = tsc;
    proto.gb = gb;
    proto.dp = dp;
    proto.pp = pp;
    proto.kind = kind;
    proto.out = out;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    pass_job_t jobs[256];
    uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    int started = 0;
    for (int t = 0; t < threads; t++) {
        uint32_t b = (uint32_t)t * chunk;
        if (b >= n) break;
        jobs[t] = proto;
        jobs[t].begin = b;
        jobs[t].end = b + chunk < n ? b + chunk : n;
        pthread_create(&th[t], NULL, run_pass_job, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

void aeo_pass_rtao(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                   float* ao) {
    run_pass(s, PASS_AO, gb, NULL, pp, gb->width * gb->height, threads, ao);
}

void aeo_pass_reflections(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                          float* rgba) {
    run_pass(s, PASS_REFL, gb, NULL, pp, gb->width * gb->height, threads, rgba);
}

void aeo_pass_rtgi(const aeo_pass_scene* s, const aeo_gbuffer* gb, const aeo_pass_params* pp, int threads,
                   float* rgba) {
    run_pass(s, PASS_GI, gb, NULL, pp, gb->width * gb->height, threads, rgba);
}

void aeo_pass_ddgi(const aeo_pass_scene* s, const aeo_ddgi_probes* dp, const aeo_pass_params* pp, int threads,
                   float* hits) {
    run_pass(s, PASS_DDGI, NULL, dp, pp, dp->n_probes * dp->ray_count, threads, hits);
}
