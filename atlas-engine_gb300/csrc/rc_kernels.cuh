// Learned radiance cache: multiresolution hash-grid encoding + spherical
// harmonics + a fused BF16 tensor-core MLP, trained online on radiance the
// path tracer produces.  The reference engine has no counterpart; the method
// follows the published neural radiance cache (Mueller et al., "Real-time
// Neural Radiance Caching for Path Tracing", 2021) and hash encoding
// (Mueller et al., "Instant Neural Graphics Primitives", 2022), written here
// from those papers.
//
// Network input (64 BF16 per query): 16 levels x 2 features of the hash grid
// (trilinear), 16 real spherical-harmonic coefficients of degree < 4 of the
// outgoing direction, the shading normal, the roughness, the vertex depth
// (bounces from the camera, which fixes how many bounces of indirect light
// the path tracer's budget leaves), zero padding.
//
// What the cache stores: the INDIRECT radiance leaving a vertex towards the
// previous one (everything the path tracer adds after the vertex's own
// next-event estimate, within the bounce budget), divided by the vertex's
// base colour and multiplied by a fixed radiance scale.  Direct light stays
// with next-event estimation at render time, so the cache's error only
// touches the smooth indirect part, and its output is modulated back by the
// base colour.
// MLP: 5 hidden layers of 64 with ReLU, no biases, linear RGB output (padded
// to 16 columns), BF16 weights, FP32 accumulation.  Inference runs on the
// tcgen05 tensor cores (rc_tc_kernels.cuh).  Training (this file) runs on
// mma.sync m16n8k16 fragments: one CTA of 4 warps handles tiles of 128
// records; each warp owns 32 rows of the activation tiles in shared memory,
// so a layer needs only warp-level synchronisation; the kernel keeps every
// layer's activations of the tile for the backward pass and reduces weight
// gradients with atomics.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "pt_kernels.cuh"
#include "trace_kernels.cuh"

namespace atlas::rt::dev {

constexpr int RC_LEVELS = 16;
constexpr int RC_IN = 64;
constexpr int RC_W = 64;
constexpr int RC_HIDDEN = 5;
constexpr int RC_OUT = 16;                 // 3 used
constexpr int RC_STRIDE = 72;              // shared row stride (bf16): conflict-free ldmatrix
constexpr int RC_TILE = 128;
constexpr int RC_THREADS = 128;
constexpr int RC_WROWS = RC_HIDDEN * RC_W + RC_OUT;         // weight rows (one per output neuron)
constexpr int RC_NPARAM = RC_WROWS * RC_W;                  // 21,504
constexpr size_t RC_WBYTES = size_t(RC_WROWS) * RC_STRIDE * 2;
constexpr size_t RC_ABYTES = size_t(RC_TILE) * RC_STRIDE * 2;

// Query / training-sample record, 4 float4: (pos, roughness), (outgoing dir,
// pixel bits), (normal, depth), (render weight or training target rgb, 1).
struct RcGrid {
    const __half2* table;      // [levels][T]
    float2* grad;              // [levels][T] (training)
    uint32_t T;                // entries per level (power of two)
    float lox, loy, loz, sx, sy, sz;     // domain: x = (pos - lo) * s in [0,1]
    float res[RC_LEVELS];
    uint32_t dense[RC_LEVELS];           // 0: hashed, else the dense stride (res + 1)
};

// Real spherical harmonics of degree < 4 (16 coefficients).
__device__ __forceinline__ void sh16(float x, float y, float z, float* o) {
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575756008f * zz - 0.31539156525252005f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (-3.0f * xx + yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * zz);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * zz);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (-xx + 3.0f * yy);
}

// Position in the grid's unit cube, clamped below 1.
__device__ __forceinline__ void rc_unit(const RcGrid& g, const float4& q0, float x[3]) {
    x[0] = fminf(fmaxf((q0.x - g.lox) * g.sx, 0.0f), 0.999999f);
    x[1] = fminf(fmaxf((q0.y - g.loy) * g.sy, 0.0f), 0.999999f);
    x[2] = fminf(fmaxf((q0.z - g.loz) * g.sz, 0.0f), 0.999999f);
}

// The eight corners of the level-l cell around x: table indices and
// trilinear weights, corner k = (dx, dy, dz) = (k & 1, (k >> 1) & 1, k >> 2).
// A corner (X, Y, Z) has index X + Y st + Z st^2 on a dense level (stride st
// = res + 1) and (X ^ Y p1 ^ Z p2) mod T on a hashed one (the spatial hash of
// the Instant-NGP paper, primes p1, p2), all arithmetic mod 2^32; the
// per-axis terms are formed once and summed or xored per corner.  Weights
// are (wx wy) wz.
__device__ __forceinline__ void rc_corners(const RcGrid& g, int l, const float x[3], uint32_t idx[8], float w[8]) {
    uint32_t c[3];
    float f[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float p = x[a] * g.res[l];
        const float fl = floorf(p);
        c[a] = uint32_t(fl);
        f[a] = p - fl;
    }
    const uint32_t st = g.dense[l];
    uint32_t ax[2] = { c[0], c[0] + 1u }, ay[2], az[2];
    if (st) {
        ay[0] = c[1] * st; ay[1] = ay[0] + st;
        az[0] = c[2] * st * st; az[1] = az[0] + st * st;
#pragma unroll
        for (int k = 0; k < 8; k++) idx[k] = ax[k & 1] + ay[(k >> 1) & 1] + az[k >> 2];
    } else {
        // spatial hash of the Instant-NGP paper: xor of coordinates times primes
        ay[0] = c[1] * 2654435761u; ay[1] = ay[0] + 2654435761u;
        az[0] = c[2] * 805459861u; az[1] = az[0] + 805459861u;
#pragma unroll
        for (int k = 0; k < 8; k++) idx[k] = (ax[k & 1] ^ ay[(k >> 1) & 1] ^ az[k >> 2]) & (g.T - 1u);
    }
    const float wx[2] = { 1.0f - f[0], f[0] }, wy[2] = { 1.0f - f[1], f[1] }, wz[2] = { 1.0f - f[2], f[2] };
    float wxy[4];
#pragma unroll
    for (int k = 0; k < 4; k++) wxy[k] = wx[k & 1] * wy[k >> 1];
#pragma unroll
    for (int k = 0; k < 8; k++) w[k] = wxy[k & 3] * wz[k >> 2];
}

// Encodes one query into the 64 BF16 network inputs (32 pairs).
__device__ __forceinline__ void rc_encode_values(const RcGrid& g, const float4& q0, const float4& q1,
                                                 const float4& q2, __nv_bfloat162 v[32]) {
    float x[3];
    rc_unit(g, q0, x);
    for (int l = 0; l < RC_LEVELS; l++) {
        uint32_t idx[8];
        float w[8];
        rc_corners(g, l, x, idx, w);
        float a0 = 0.0f, a1 = 0.0f;
        const __half2* tab = g.table + size_t(l) * g.T;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float2 e = __half22float2(tab[idx[k]]);
            a0 += w[k] * e.x;
            a1 += w[k] * e.y;
        }
        v[l] = __floats2bfloat162_rn(a0, a1);
    }
    float sh[16];
    sh16(q1.x, q1.y, q1.z, sh);
    for (int k = 0; k < 8; k++) v[16 + k] = __floats2bfloat162_rn(sh[2 * k], sh[2 * k + 1]);
    v[24] = __floats2bfloat162_rn(q2.x, q2.y);
    v[25] = __floats2bfloat162_rn(q2.z, q0.w);
    v[26] = __floats2bfloat162_rn(q2.w, 0.0f);
    for (int k = 27; k < 32; k++) v[k] = __floats2bfloat162_rn(0.0f, 0.0f);
}

// Encodes one query into a 64-wide BF16 row in shared memory.
__device__ __forceinline__ void rc_encode(const RcGrid& g, const float4& q0, const float4& q1, const float4& q2,
                                          __nv_bfloat16* row) {
    __nv_bfloat162 v[32];
    rc_encode_values(g, q0, q1, q2, v);
    uint4* dst = reinterpret_cast<uint4*>(row);
    const uint4* src = reinterpret_cast<const uint4*>(v);
#pragma unroll
    for (int k = 0; k < 8; k++) dst[k] = src[k];
}

// Gradient of the hash-grid part of the input row, scattered to the table.
__device__ __forceinline__ void rc_encode_backward(const RcGrid& g, const float4& q0, const __nv_bfloat16* drow) {
    float x[3];
    rc_unit(g, q0, x);
    for (int l = 0; l < RC_LEVELS; l++) {
        const float2 gr = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(drow)[l]);
        if (gr.x == 0.0f && gr.y == 0.0f) continue;
        uint32_t idx[8];
        float w[8];
        rc_corners(g, l, x, idx, w);
        float2* gt = g.grad + size_t(l) * g.T;
#pragma unroll
        for (int k = 0; k < 8; k++) atomicAdd(&gt[idx[k]], make_float2(w[k] * gr.x, w[k] * gr.y));
    }
}

// ---- tensor-core helpers (mma.sync.m16n8k16 BF16 -> FP32) ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void ldsm4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm4t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma16816(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Y[32 rows x 8*NB] = X[32 x 16*KS] * Wt^T for the warp's rows.  X rows at
// `x` (stride RC_STRIDE), weight rows (one per output) at `w`.
template <int NB, int KS>
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16* x, const __nv_bfloat16* w, float (&acc)[2][NB][4],
                                          uint32_t lane) {
#pragma unroll
    for (int mb = 0; mb < 2; mb++)
#pragma unroll
        for (int nb = 0; nb < NB; nb++) acc[mb][nb][0] = acc[mb][nb][1] = acc[mb][nb][2] = acc[mb][nb][3] = 0.0f;
    const uint32_t q = lane >> 3, r = lane & 7;
#pragma unroll
    for (int ks = 0; ks < KS; ks++) {
        const int k = ks * 16;
        uint32_t a[2][4];
#pragma unroll
        for (int mb = 0; mb < 2; mb++)
            ldsm4(a[mb][0], a[mb][1], a[mb][2], a[mb][3], x + (mb * 16 + (q & 1) * 8 + r) * RC_STRIDE + k + (q >> 1) * 8);
#pragma unroll
        for (int nb = 0; nb < NB; nb += 2) {
            uint32_t b0, b1, b2, b3;
            ldsm4(b0, b1, b2, b3, w + (nb * 8 + (q >> 1) * 8 + r) * RC_STRIDE + k + (q & 1) * 8);
#pragma unroll
            for (int mb = 0; mb < 2; mb++) {
                mma16816(acc[mb][nb], a[mb][0], a[mb][1], a[mb][2], a[mb][3], b0, b1);
                mma16816(acc[mb][nb + 1], a[mb][0], a[mb][1], a[mb][2], a[mb][3], b2, b3);
            }
        }
    }
}

// dX[32 x 64] = dZ[32 x 16*KS] * Wt (weights as rows = outputs; B fetched
// transposed), for the warp's rows.
template <int KS>
__device__ __forceinline__ void warp_gemm_bwd_data(const __nv_bfloat16* dz, const __nv_bfloat16* w,
                                                   float (&acc)[2][8][4], uint32_t lane) {
#pragma unroll
    for (int mb = 0; mb < 2; mb++)
#pragma unroll
        for (int nb = 0; nb < 8; nb++) acc[mb][nb][0] = acc[mb][nb][1] = acc[mb][nb][2] = acc[mb][nb][3] = 0.0f;
    const uint32_t q = lane >> 3, r = lane & 7;
#pragma unroll
    for (int ks = 0; ks < KS; ks++) {
        const int k = ks * 16;
        uint32_t a[2][4];
#pragma unroll
        for (int mb = 0; mb < 2; mb++)
            ldsm4(a[mb][0], a[mb][1], a[mb][2], a[mb][3], dz + (mb * 16 + (q & 1) * 8 + r) * RC_STRIDE + k + (q >> 1) * 8);
#pragma unroll
        for (int nb = 0; nb < 8; nb += 2) {
            uint32_t b0, b1, b2, b3;
            ldsm4t(b0, b1, b2, b3, w + (k + (q & 1) * 8 + r) * RC_STRIDE + nb * 8 + (q >> 1) * 8);
#pragma unroll
            for (int mb = 0; mb < 2; mb++) {
                mma16816(acc[mb][nb], a[mb][0], a[mb][1], a[mb][2], a[mb][3], b0, b1);
                mma16816(acc[mb][nb + 1], a[mb][0], a[mb][1], a[mb][2], a[mb][3], b2, b3);
            }
        }
    }
}

// dWt[16 rows from m0, NB blocks of 8 from n0] += dZ^T * A over the tile's
// 128 rows (both operands fetched transposed).
template <int NB>
__device__ __forceinline__ void warp_gemm_bwd_weight(const __nv_bfloat16* dz, int m0, const __nv_bfloat16* act,
                                                     int n0, float (&acc)[NB][4], uint32_t lane) {
#pragma unroll
    for (int nb = 0; nb < NB; nb++) acc[nb][0] = acc[nb][1] = acc[nb][2] = acc[nb][3] = 0.0f;
    const uint32_t q = lane >> 3, r = lane & 7;
#pragma unroll
    for (int ks = 0; ks < RC_TILE / 16; ks++) {
        const int k = ks * 16;
        uint32_t a0, a1, a2, a3;
        ldsm4t(a0, a1, a2, a3, dz + (k + (q >> 1) * 8 + r) * RC_STRIDE + m0 + (q & 1) * 8);
#pragma unroll
        for (int nb = 0; nb < NB; nb += 2) {
            uint32_t b0, b1, b2, b3;
            ldsm4t(b0, b1, b2, b3, act + (k + (q & 1) * 8 + r) * RC_STRIDE + n0 + nb * 8 + (q >> 1) * 8);
            mma16816(acc[nb], a0, a1, a2, a3, b0, b1);
            mma16816(acc[nb + 1], a0, a1, a2, a3, b2, b3);
        }
    }
}

template <int NB>
__device__ __forceinline__ void store_rows(__nv_bfloat16* y, const float (&acc)[2][NB][4], uint32_t lane, bool relu) {
    const uint32_t g = lane >> 2, c2 = (lane & 3) * 2;
#pragma unroll
    for (int mb = 0; mb < 2; mb++)
#pragma unroll
        for (int nb = 0; nb < NB; nb++) {
            float v0 = acc[mb][nb][0], v1 = acc[mb][nb][1], v2 = acc[mb][nb][2], v3 = acc[mb][nb][3];
            if (relu) {
                v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); v2 = fmaxf(v2, 0.0f); v3 = fmaxf(v3, 0.0f);
            }
            *reinterpret_cast<uint32_t*>(y + (mb * 16 + g) * RC_STRIDE + nb * 8 + c2) = pack_bf16(v0, v1);
            *reinterpret_cast<uint32_t*>(y + (mb * 16 + g + 8) * RC_STRIDE + nb * 8 + c2) = pack_bf16(v2, v3);
        }
}

constexpr int RC_INFER = 0;    // inference: accumulate throughput * max(prediction, 0) into the image
constexpr int RC_PREDICT = 1;  // inference: write predictions
constexpr int RC_TRAIN = 2;    // relative-L2 loss, gradients

struct RcMlpParams {
    RcGrid grid;
    const __nv_bfloat16* weights;    // RC_NPARAM, rows = output neurons
    float* grad_w;                   // RC_NPARAM (training)
    const float4* recs;              // 4 float4 per query / sample
    const uint32_t* n_dev;           // optional device count
    uint32_t n;                      // count, or capacity with n_dev
    uint32_t offset;                 // first record (training steps over one buffer)
    const uint32_t* offset_dev;      // inference: first record read from the device (overrides offset)
    uint32_t slice, slices;          // slices > 0: train on slice `slice` of the device count
    float4* accum;                   // RC_INFER: image
    float4* out;                     // RC_PREDICT
    float* loss;                     // RC_TRAIN: mean per-element loss (accumulated)
    uint32_t* error_word;            // tensor-memory kernels: a bounded wait that gave up
    uint32_t skip_mma;               // self-test only: issue no MMA, so every wait runs out
};

// Training (fused encode + forward + relative-L2 loss + backward with weight
// and hash-grid gradient atomics) on mma.sync BF16 fragments; inference runs
// on the tcgen05 kernel of rc_tc_kernels.cuh.
template <int MODE>
static __global__ void __launch_bounds__(RC_THREADS, 1) rc_mlp_kernel(RcMlpParams p) {
    static_assert(MODE == RC_TRAIN, "inference is rc_infer_tc_kernel");
    extern __shared__ __align__(16) unsigned char rc_smem[];
    __nv_bfloat16* wsm = reinterpret_cast<__nv_bfloat16*>(rc_smem);
    __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(rc_smem + RC_WBYTES);   // [6][128][72]
    __nv_bfloat16* dbuf = act + size_t(RC_HIDDEN + 1) * RC_TILE * RC_STRIDE;       // [2][128][72]
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    // weights into shared memory (rows of 64 -> stride 72)
    for (uint32_t i = threadIdx.x; i < uint32_t(RC_WROWS) * 8u; i += blockDim.x) {
        const uint32_t row = i >> 3, part = i & 7u;
        reinterpret_cast<uint4*>(wsm + row * RC_STRIDE)[part] =
            reinterpret_cast<const uint4*>(p.weights + size_t(row) * RC_W)[part];
    }
    __syncthreads();

    const uint32_t n = p.n_dev ? min(*p.n_dev, p.n) : p.n;
    uint32_t first = p.offset, count = n > p.offset ? n - p.offset : 0u;
    if (p.slices) {
        first = uint32_t(uint64_t(n) * p.slice / p.slices);
        count = uint32_t(uint64_t(n) * (p.slice + 1) / p.slices) - first;
    }
    const float inv_norm = count ? 1.0f / (3.0f * float(count)) : 0.0f;
    const uint32_t tiles = (count + RC_TILE - 1) / RC_TILE;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t row0 = warp * 32u;
        const uint32_t gi = tile * RC_TILE + row0 + lane;
        const bool valid = gi < count;
        float4 q0 = make_float4(0, 0, 0, 0), q1 = q0, q2 = q0, q3 = q0;
        if (valid) {
            const float4* rec = p.recs + size_t(first + gi) * 4;
            q0 = rec[0]; q1 = rec[1]; q2 = rec[2]; q3 = rec[3];
        }
        __nv_bfloat16* x0 = act + size_t(row0) * RC_STRIDE;
        if (valid) {
            rc_encode(p.grid, q0, q1, q2, x0 + lane * RC_STRIDE);
        } else {
            uint4* d = reinterpret_cast<uint4*>(x0 + lane * RC_STRIDE);
            for (int k = 0; k < 8; k++) d[k] = make_uint4(0, 0, 0, 0);
        }
        __syncwarp();
        // ---- forward ----
#pragma unroll 1
        for (int l = 0; l < RC_HIDDEN; l++) {
            const __nv_bfloat16* xin = act + size_t(l) * RC_TILE * RC_STRIDE + row0 * RC_STRIDE;
            __nv_bfloat16* yout = act + size_t(l + 1) * RC_TILE * RC_STRIDE + row0 * RC_STRIDE;
            float acc[2][8][4];
            warp_gemm<8, 4>(xin, wsm + l * RC_W * RC_STRIDE, acc, lane);
            __syncwarp();
            store_rows<8>(yout, acc, lane, true);
            __syncwarp();
        }
        float oacc[2][2][4];
        const __nv_bfloat16* xlast = act + size_t(RC_HIDDEN) * RC_TILE * RC_STRIDE + row0 * RC_STRIDE;
        warp_gemm<2, 4>(xlast, wsm + RC_HIDDEN * RC_W * RC_STRIDE, oacc, lane);
        // output element (row mb*16 + g (+8), col 2*(lane&3) + {0,1}) of n-block 0 holds RGB
        const uint32_t g = lane >> 2, cq = lane & 3u;
        // ---- relative L2 loss and its gradient (rows of the warp) ----
        __nv_bfloat16* dcur = dbuf;
        __nv_bfloat16* doth = dbuf + size_t(RC_TILE) * RC_STRIDE;
        {
            float lsum = 0.0f;
#pragma unroll
            for (int mb = 0; mb < 2; mb++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint32_t rowInWarp = mb * 16 + g + 8 * h;
                    const float t0 = __shfl_sync(0xffffffffu, q3.x, rowInWarp);
                    const float t1 = __shfl_sync(0xffffffffu, q3.y, rowInWarp);
                    const float t2 = __shfl_sync(0xffffffffu, q3.z, rowInWarp);
                    const bool rv = tile * RC_TILE + row0 + rowInWarp < count;
                    float d0 = 0.0f, d1 = 0.0f;
                    for (int e = 0; e < 2; e++) {
                        const int col = int(cq) * 2 + e;
                        const float pr = oacc[mb][0][2 * h + e];
                        const float tg = col == 0 ? t0 : (col == 1 ? t1 : t2);
                        float dd = 0.0f;
                        if (rv && col < 3) {
                            const float den = pr * pr + 0.01f;
                            const float diff = pr - tg;
                            lsum += diff * diff / den;
                            dd = 2.0f * diff / den * inv_norm;
                        }
                        if (e == 0) d0 = dd; else d1 = dd;
                    }
                    __nv_bfloat16* drow = dcur + size_t(row0 + rowInWarp) * RC_STRIDE;
                    *reinterpret_cast<uint32_t*>(drow + cq * 2) = pack_bf16(d0, d1);
                    *reinterpret_cast<uint32_t*>(drow + 8 + cq * 2) = 0u;
                }
            for (int off = 16; off > 0; off >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, off);
            if (lane == 0) atomicAdd(p.loss, lsum * inv_norm);
        }
        __syncthreads();
        // ---- output layer: dA5 = dP * W5, dW5 += dP^T * A5 ----
        {
            float acc[2][8][4];
            warp_gemm_bwd_data<1>(dcur + size_t(row0) * RC_STRIDE, wsm + RC_HIDDEN * RC_W * RC_STRIDE, acc, lane);
            store_rows<8>(doth + size_t(row0) * RC_STRIDE, acc, lane, false);
            float wacc[2][4];
            warp_gemm_bwd_weight<2>(dcur, 0, act + size_t(RC_HIDDEN) * RC_TILE * RC_STRIDE, warp * 16, wacc, lane);
            float* gw = p.grad_w + RC_HIDDEN * RC_W * RC_W;
#pragma unroll
            for (int nb = 0; nb < 2; nb++) {
                const int col = warp * 16 + nb * 8 + cq * 2;
                atomicAdd(reinterpret_cast<float2*>(gw + g * RC_W + col), make_float2(wacc[nb][0], wacc[nb][1]));
                atomicAdd(reinterpret_cast<float2*>(gw + (g + 8) * RC_W + col), make_float2(wacc[nb][2], wacc[nb][3]));
            }
        }
        __syncthreads();
        {
            __nv_bfloat16* t = dcur; dcur = doth; doth = t;
        }
        // ---- hidden layers, last to first ----
#pragma unroll 1
        for (int l = RC_HIDDEN - 1; l >= 0; l--) {
            // dZ = dY * relu'(A_{l+1}) on the warp's rows
            const __nv_bfloat16* aout = act + size_t(l + 1) * RC_TILE * RC_STRIDE;
            for (int i = lane; i < 32 * 32; i += 32) {
                const int rr = row0 + i / 32, cc = (i % 32) * 2;
                __nv_bfloat162* dz = reinterpret_cast<__nv_bfloat162*>(dcur + size_t(rr) * RC_STRIDE + cc);
                const __nv_bfloat162 av = *reinterpret_cast<const __nv_bfloat162*>(aout + size_t(rr) * RC_STRIDE + cc);
                const float2 dv = __bfloat1622float2(*dz);
                const float2 a2 = __bfloat1622float2(av);
                *dz = __floats2bfloat162_rn(a2.x > 0.0f ? dv.x : 0.0f, a2.y > 0.0f ? dv.y : 0.0f);
            }
            __syncthreads();
            {
                float acc[2][8][4];
                warp_gemm_bwd_data<4>(dcur + size_t(row0) * RC_STRIDE, wsm + l * RC_W * RC_STRIDE, acc, lane);
                store_rows<8>(doth + size_t(row0) * RC_STRIDE, acc, lane, false);
            }
            {
                float wacc[8][4];
                warp_gemm_bwd_weight<8>(dcur, warp * 16, act + size_t(l) * RC_TILE * RC_STRIDE, 0, wacc, lane);
                float* gw = p.grad_w + size_t(l) * RC_W * RC_W;
#pragma unroll
                for (int nb = 0; nb < 8; nb++) {
                    const int col = nb * 8 + cq * 2;
                    const int rA = warp * 16 + g;
                    atomicAdd(reinterpret_cast<float2*>(gw + rA * RC_W + col), make_float2(wacc[nb][0], wacc[nb][1]));
                    atomicAdd(reinterpret_cast<float2*>(gw + (rA + 8) * RC_W + col), make_float2(wacc[nb][2], wacc[nb][3]));
                }
            }
            __syncthreads();
            {
                __nv_bfloat16* t = dcur; dcur = doth; doth = t;
            }
        }
        // dcur now holds dX (input gradient): scatter the hash-grid part
        if (valid) rc_encode_backward(p.grid, q0, dcur + size_t(row0 + lane) * RC_STRIDE);
        __syncthreads();
    }
}

// Adam over [0, n) (n a multiple of 4; 16-byte aligned arrays): FP32 master,
// moments; also writes the low-precision copy (BF16 for the MLP, FP16 for the
// grid).  skip_zero: entries whose gradient is exactly zero (hash-grid
// entries no record touched) keep their parameter and moments -- the sparse
// update usual for hash encodings; it also saves most of the pass's writes.
struct RcAdamParams {
    float* master;
    float* m;
    float* v;
    float* grad;
    __nv_bfloat16* out_bf16;
    __half* out_f16;
    size_t n;
    float lr, beta1, beta2, eps;
    float step_scale;     // sqrt(1 - beta2^t) / (1 - beta1^t)
    uint32_t skip_zero;
    uint32_t zero_grad;   // leave the gradient zero behind (the next step's accumulation needs no clear)
};

__device__ __forceinline__ void adam1(const RcAdamParams& a, float gr, float& w, float& m, float& v) {
    m = a.beta1 * m + (1.0f - a.beta1) * gr;
    v = a.beta2 * v + (1.0f - a.beta2) * gr * gr;
    w = w - a.lr * a.step_scale * m / (sqrtf(v) + a.eps);
}

// One Adam step over the parameter set `a` by `blocks` blocks of the grid,
// the first of them `block`.
__device__ __forceinline__ void rc_adam_range(const RcAdamParams& a, uint32_t block, uint32_t blocks) {
    const size_t stride = size_t(blocks) * blockDim.x;
    const size_t n4 = a.n / 4;
    for (size_t i = size_t(block) * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 g = reinterpret_cast<const float4*>(a.grad)[i];
        const bool z[4] = { g.x == 0.0f, g.y == 0.0f, g.z == 0.0f, g.w == 0.0f };
        if (a.skip_zero && z[0] && z[1] && z[2] && z[3]) continue;
        float4 w = reinterpret_cast<float4*>(a.master)[i];
        float4 m = reinterpret_cast<float4*>(a.m)[i];
        float4 v = reinterpret_cast<float4*>(a.v)[i];
        const bool upd[4] = { !(a.skip_zero && z[0]), !(a.skip_zero && z[1]), !(a.skip_zero && z[2]),
                              !(a.skip_zero && z[3]) };
        if (upd[0]) adam1(a, g.x, w.x, m.x, v.x);
        if (upd[1]) adam1(a, g.y, w.y, m.y, v.y);
        if (upd[2]) adam1(a, g.z, w.z, m.z, v.z);
        if (upd[3]) adam1(a, g.w, w.w, m.w, v.w);
        reinterpret_cast<float4*>(a.master)[i] = w;
        reinterpret_cast<float4*>(a.m)[i] = m;
        reinterpret_cast<float4*>(a.v)[i] = v;
        if (a.zero_grad) reinterpret_cast<float4*>(a.grad)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (a.out_bf16) {
            __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(a.out_bf16) + 2 * i;
            o[0] = __floats2bfloat162_rn(w.x, w.y);
            o[1] = __floats2bfloat162_rn(w.z, w.w);
        }
        if (a.out_f16) {
            __half2* o = reinterpret_cast<__half2*>(a.out_f16) + 2 * i;
            o[0] = __floats2half2_rn(w.x, w.y);
            o[1] = __floats2half2_rn(w.z, w.w);
        }
    }
}

// The MLP's and the hash grid's Adam steps in one launch: the first
// `mlp_blocks` blocks update the MLP, the rest the grid.
static __global__ void rc_adam_kernel(RcAdamParams mlp, RcAdamParams grid, uint32_t mlp_blocks) {
    if (blockIdx.x < mlp_blocks) rc_adam_range(mlp, blockIdx.x, mlp_blocks);
    else rc_adam_range(grid, blockIdx.x - mlp_blocks, gridDim.x - mlp_blocks);
}

// ---- inline two-level traversal for the training-path kernel ----
// HitClosest / HitAny over the scene with a per-thread local stack: the
// structure of trace_kernel<MODE_SCENE>, with the conservative approximate
// box test (test_children_loose) and tri_test_fast.  The training
// targets are Monte Carlo estimates, so the nearest hit may break exact
// distance ties in another order than the shader's traversal.
template <bool ANY>
__device__ bool scene_trace_inline(const TraceParams& p, float ox, float oy, float oz, float dx, float dy, float dz,
                                   float tmin, float tmax, float& tOut, int32_t& triOut, int32_t& instOut,
                                   float& uOut, float& vOut) {
    constexpr int kInlineStack = 128;
    int32_t stack[kInlineStack];
    TRay wr{};
    wr.ox = ox; wr.oy = oy; wr.oz = oz; wr.dx = dx; wr.dy = dy; wr.dz = dz;
    wr.prepare();
    TRay r = wr;
    float hitDist = tmax, hu = 0.0f, hv = 0.0f;
    int32_t hitID = -1, hitInst = -1, curInst = -1;
    const float4* blasNodes = nullptr;
    const float4* blasTris = nullptr;
    uint32_t sp = 0, tlasIndex = kTlasInvalid, steps = 0;
    int32_t node = 0;
    bool occl = false;
    if (p.n_tlas == 0 || isnan(dx) || isnan(dy) || isnan(dz)) return false;
    for (;;) {
        if (++steps > p.max_steps) break;
        const bool top = sp < tlasIndex;
        if (top) {
            tlasIndex = kTlasInvalid;
            if (node < 0) {
                const uint32_t ii = uint32_t(~node);
                const float4* ip = p.instances + size_t(ii) * 4;
                const float4 c0 = __ldg(ip), c1 = __ldg(ip + 1), c2 = __ldg(ip + 2), c3 = __ldg(ip + 3);
                curInst = int32_t(ii);
                bool enter = (__float_as_uint(c3.w) & p.cull_mask) != 0u;
                MeshDesc m{};
                if (enter) {
                    m = p.meshes[__float_as_int(c3.x)];
                    enter = m.n_nodes > 0;
                }
                if (enter) {
                    r.ox = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c0);
                    r.oy = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c1);
                    r.oz = xform_row(wr.ox, wr.oy, wr.oz, 1.0f, c2);
                    r.dx = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c0);
                    r.dy = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c1);
                    r.dz = xform_row(wr.dx, wr.dy, wr.dz, 0.0f, c2);
                    r.prepare();
                    blasNodes = m.nodes;
                    blasTris = m.tris;
                    node = 0;
                    tlasIndex = sp;
                } else {
                    if (sp == 0) break;
                    node = stack[--sp];
                }
                continue;
            }
        }
        if (node < 0) {
            int32_t tp = ~node;
            bool end = false;
            do {
                const float4 a = __ldg(blasTris + size_t(tp) * 3), b = __ldg(blasTris + size_t(tp) * 3 + 1),
                             c = __ldg(blasTris + size_t(tp) * 3 + 2);
                end = a.w > 0.0f;
                float t, u, v;
                const bool hit = tri_test_fast(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, a, b, c, t, u, v);
                if (ANY) {
                    if (hit && t > tmin && t < tmax) { occl = true; end = true; }
                } else if (hit && t > tmin && t < tmax && t < hitDist) {
                    hitDist = t; hitID = tp; hu = u; hv = v; hitInst = curInst;
                }
                tp++;
            } while (!end);
            if (ANY && occl) break;
            if (sp == 0) break;
            node = stack[--sp];
        } else {
            const float4* np = (top ? p.tlas : blasNodes) + size_t(node) * 4;
            float4 n0, n1, n2, n3;
            ldg_node(np, n0, n1, n2, n3);
            bool il, ir, leftFirst;
            test_children_loose(top ? wr : r, n0, n1, n2, n3, tmin, ANY ? tmax : hitDist, il, ir, leftFirst);
            const int32_t lptr = __float_as_int(n3.x), rptr = __float_as_int(n3.y);
            int32_t next, far;
            if (ANY) {
                next = il ? lptr : rptr;
                far = rptr;
            } else {
                next = leftFirst ? lptr : rptr;
                far = leftFirst ? rptr : lptr;
            }
            if (il && ir) {
                if (sp >= kInlineStack) break;
                stack[sp++] = far;
            } else if (!il && !ir) {
                if (sp == 0) break;
                next = stack[--sp];
            }
            node = next;
        }
    }
    tOut = hitDist; triOut = hitID; instOut = hitInst; uOut = hu; vOut = hv;
    return ANY ? occl : hitID >= 0;
}

constexpr int RC_MAX_DEPTH = 3;   // vertices per training path that give records

struct RcPathParams {
    TraceParams tp;          // scene pointers for the inline traversal
    PtScene sc;
    CameraParams cam;
    uint32_t n_paths;
    uint32_t frame;
    uint32_t seed;
    uint32_t max_bounces;
    float epsilon;
    float scale;             // radiance scale of the stored targets
    float4* samples;         // 4 float4 per sample, up to RC_MAX_DEPTH per path
    uint32_t* n_samples;
};

__device__ __forceinline__ float safe_div(float a, float b) { return b > 1e-30f ? a / b : 0.0f; }

// Self-generated training paths: a random pixel, its camera ray, and the path
// tracer's estimator (next-event estimation at every vertex, continuation,
// Russian roulette) up to max_bounces bounces, with next-event estimation
// and BRDF-sampled light hits combined by the power heuristic (same
// expectation as the engine's estimator, fewer outliers in the targets).  Every vertex k < max_bounces
// (k < RC_MAX_DEPTH) with a non-black base colour gives one record: its
// indirect radiance estimate -- the next-event contributions of the later
// vertices divided by the path throughput that arrived at k -- divided by
// the base colour and scaled.
// A vertex's record, arriving throughput and base colour wait in shared
// memory (one column per thread) until the path ends, so that the kernel
// fits 128 registers and 65,536 paths run in one wave of 4 CTAs per SM.
constexpr uint32_t RC_PATH_THREADS = 128;
static __global__ void __launch_bounds__(RC_PATH_THREADS, 4) rc_paths_kernel(RcPathParams p) {
    __shared__ float4 s_rec[RC_MAX_DEPTH * 3][RC_PATH_THREADS];
    __shared__ float s_ab[RC_MAX_DEPTH * 6][RC_PATH_THREADS];    // arrive xyz, base xyz per vertex
    const uint32_t tid = threadIdx.x;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    V3 acc[RC_MAX_DEPTH] = {};
    uint32_t nv = 0;
    if (i < p.n_paths) {
        const uint32_t npix = p.cam.width * p.cam.height;
        const uint32_t key = i + (p.frame << 20);
        const uint32_t pix = min(uint32_t(rand01(key, p.seed, 0xB5297A4Du) * float(npix)), npix - 1u);
        const uint32_t sample = 0x40000000u + p.frame;       // a stream apart from the rendered samples
        const float jx = rng(pix, sample, 15, 0, p.seed ^ i), jy = rng(pix, sample, 15, 1, p.seed ^ i);
        const CameraParams& c = p.cam;
        const float u = (float(pix % c.width) + jx) / float(c.width);
        const float v = (float(pix / c.width) + jy) / float(c.height);
        V3 rd = normalize(v3(c.ox + c.rx * u + c.bx * v - c.lx, c.oy + c.ry * u + c.by * v - c.ly,
                             c.oz + c.rz * u + c.bz * v - c.lz));
        V3 ro = v3(c.lx, c.ly, c.lz);
        V3 thr = v3(1, 1, 1);
        float hitW = 0.0f;       // MIS factor of the emission the current ray may find
        const uint32_t key2 = i ^ (p.frame * 0x9E3779B9u);
        for (uint32_t b = 0; b <= p.max_bounces; b++) {
            TraceParams tp = p.tp;
            tp.cull_mask = 0x80u;   // INSTANCE_MASK_ALL
            float t, bu, bv;
            int32_t tri, inst;
            if (!scene_trace_inline<false>(tp, ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, 0.0f, 1e12f, t, tri, inst, bu, bv))
                break;
            Surf sf = make_surface(p.sc, ro, rd, t, inst, tri, bu, bv);
            // emission found by the previous vertex's continuation: part of
            // that vertex's direct light, so indirect light of the ones before
            if (b >= 2 && hitW > 0.0f && sf.mat.emissive.x + sf.mat.emissive.y + sf.mat.emissive.z > 0.0f) {
                const V3 e = thr * sf.mat.emissive * hitW;
#pragma unroll
                for (int k = 0; k < RC_MAX_DEPTH; k++)
                    if (k + 1 < int(b) && k < int(nv)) acc[k] = acc[k] + e;
            }
            if (b < p.max_bounces && b < uint32_t(RC_MAX_DEPTH)) {
                s_rec[b * 3 + 0][tid] = make_float4(sf.P.x, sf.P.y, sf.P.z, sf.mat.roughness);
                s_rec[b * 3 + 1][tid] = make_float4(sf.V.x, sf.V.y, sf.V.z, __uint_as_float(pix));
                s_rec[b * 3 + 2][tid] = make_float4(sf.N.x, sf.N.y, sf.N.z, float(b));
                s_ab[b * 6 + 0][tid] = thr.x; s_ab[b * 6 + 1][tid] = thr.y; s_ab[b * 6 + 2][tid] = thr.z;
                s_ab[b * 6 + 3][tid] = sf.mat.base.x; s_ab[b * 6 + 4][tid] = sf.mat.base.y;
                s_ab[b * 6 + 5][tid] = sf.mat.base.z;
#pragma unroll
                for (int k = 0; k < RC_MAX_DEPTH; k++)
                    if (k == int(b)) acc[k] = v3(0, 0, 0);
                nv = b + 1;
            }
            const bool cont = b < p.max_bounces;
            V3 cth, so, sd;
            float st, pl = 0.0f;
            if (b > 0 && direct_light(p.sc, sf, thr, key2, sample, b, p.seed, p.epsilon, cth, so, sd, st, &pl)) {
                if (cont) cth = cth * power_weight(pl, bsdf_pdf(sf, sf.L));
                tp.cull_mask = 0x40u;   // INSTANCE_MASK_SHADOW
                float t2, u2, v2;
                int32_t tr2, in2;
                if (!scene_trace_inline<true>(tp, so.x, so.y, so.z, sd.x, sd.y, sd.z, 0.0f, st, t2, tr2, in2, u2, v2)) {
#pragma unroll
                    for (int k = 0; k < RC_MAX_DEPTH; k++)
                        if (k < int(b) && k < int(nv)) acc[k] = acc[k] + cth;
                }
            }
            if (!cont) break;
            V3 o, d;
            bool spec = false;
            if (!continue_path(sf, thr, key2, sample, b, p.seed, p.epsilon, o, d, &spec)) break;
            hitW = b + 1 >= 2 ? mis_hit_factor(p.sc, sf, d, spec) : 0.0f;
            ro = o;
            rd = d;
        }
    }
#pragma unroll
    for (int k = 0; k < RC_MAX_DEPTH; k++) {
        const bool has = k < int(nv);
        const V3 base = has ? v3(s_ab[k * 6 + 3][tid], s_ab[k * 6 + 4][tid], s_ab[k * 6 + 5][tid]) : v3(0, 0, 0);
        const bool emit = has && base.x + base.y + base.z > 0.0f;
        const uint32_t si = warp_append(p.n_samples, emit, lane);
        if (emit) {
            const V3 arrive = v3(s_ab[k * 6 + 0][tid], s_ab[k * 6 + 1][tid], s_ab[k * 6 + 2][tid]);
            const V3 tg = v3(safe_div(acc[k].x, arrive.x * base.x), safe_div(acc[k].y, arrive.y * base.y),
                             safe_div(acc[k].z, arrive.z * base.z)) * p.scale;
            float4* o = p.samples + size_t(si) * 4;
            o[0] = s_rec[k * 3 + 0][tid];
            o[1] = s_rec[k * 3 + 1][tid];
            o[2] = s_rec[k * 3 + 2][tid];
            o[3] = make_float4(tg.x, tg.y, tg.z, 1.0f);
        }
    }
}

constexpr uint32_t RC_MAX_SPLIT = 4;

struct RcShadeParams {
    PtParams pt;             // queues, scene, accumulation, bounce budget (pt.max_bounces)
    float4* queries;         // cache queries (4 float4)
    uint32_t* n_queries;
    uint32_t query_capacity;
    uint32_t last_bounce;    // query the cache here whatever the material
    float inv_scale;         // 1 / radiance scale of the cache
    float rough_cut;         // metals at least this rough end in the cache too
    uint32_t split;          // paths per glossy metal at the first vertex (1..RC_MAX_SPLIT)
};

// Appends one item per lane that wants one (warp-aggregated), or drops it and
// flags the overflow when the queue is full.
__device__ __forceinline__ bool rc_append(uint32_t* counter, uint32_t cap, bool want, uint32_t lane, uint32_t* overflow,
                                          uint32_t& idx) {
    idx = warp_append(counter, want, lane);
    if (want && idx >= cap) {
        if (overflow) atomicOr(overflow, kErrQueueOverflow);
        return false;
    }
    return want;
}

// Rendering with the cache: emission of the first hit and next-event
// estimation at every vertex (as the path tracer).  A diffuse vertex, a metal
// with roughness >= rough_cut, or the vertex at last_bounce ends the path
// with a cache query for its indirect radiance, weighted by path throughput x
// base colour / scale.  A glossier metal continues the path; its next-event
// estimate and the emission its continuation finds are combined by the power
// heuristic (the factor travels in the continuation ray's dir.w).  At the
// first vertex a glossy metal splits into `split` independent paths (a light
// sample and a continuation each, weight 1/split), with their own random
// streams (split index in bits 24-26 of the pixel key): those pixels carry
// most of the variance of a cache-terminated frame.
static __global__ void rc_shade_kernel(RcShadeParams rp) {
    const PtParams& p = rp.pt;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t cap = queue_capacity(p);
    const uint32_t n = min(*p.n_in, cap);
    bool emitQuery = false, cont = false;
    uint32_t S = 0, key = 0;
    float4 q0{}, q1{}, q2{}, q3{};
    Surf sf{};
    V3 thr = v3(0, 0, 0);
    if (i < n) {
        const float4 h0 = p.hits_in[size_t(i) * 2];
        const int32_t triPtr = __float_as_int(h0.y);
        const float4 pay = p.pay_in[i];
        key = __float_as_uint(pay.w);
        thr = v3(pay.x, pay.y, pay.z);
        if (triPtr >= 0) {
            const float4 o4 = p.rays_in[size_t(i) * 3], d4 = p.rays_in[size_t(i) * 3 + 1];
            const float4 h1 = p.hits_in[size_t(i) * 2 + 1];
            sf = make_surface(p.sc, ld3(o4), ld3(d4), h0.x, __float_as_int(h0.z), triPtr, h1.x, h1.y);
            const bool emissive = sf.mat.emissive.x + sf.mat.emissive.y + sf.mat.emissive.z > 0.0f;
            if (p.bounce == 0 && emissive) add_radiance(p, key, sf.mat.emissive);
            if (p.bounce > 0 && emissive && d4.w > 0.0f) add_radiance(p, key, thr * sf.mat.emissive * d4.w);
            const bool query = sf.mat.metalness < 0.5f || sf.mat.roughness >= rp.rough_cut ||
                               p.bounce >= rp.last_bounce || p.bounce + 1 >= uint32_t(RC_MAX_DEPTH);
            cont = p.bounce < p.max_bounces && !query;
            // a glossy metal at the first vertex splits (light sample +
            // continuation per split); splitting the light sample of the
            // metals that end in the cache was measured and gains nothing
            S = cont && p.bounce == 0 ? rp.split : 1u;
            if (query && p.bounce < p.max_bounces) {
                const V3 w = thr * sf.mat.base * rp.inv_scale;
                if (w.x + w.y + w.z > 0.0f) {
                    emitQuery = true;
                    q0 = make_float4(sf.P.x, sf.P.y, sf.P.z, sf.mat.roughness);
                    q1 = make_float4(sf.V.x, sf.V.y, sf.V.z, __uint_as_float(key));
                    q2 = make_float4(sf.N.x, sf.N.y, sf.N.z, float(p.bounce));
                    q3 = make_float4(w.x, w.y, w.z, 1.0f);
                }
            }
        }
    }
    uint32_t qi;
    if (rc_append(rp.n_queries, rp.query_capacity, emitQuery, lane, p.overflow, qi)) {
        float4* q = rp.queries + size_t(qi) * 4;
        q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
    }
    const float invS = S > 1u ? 1.0f / float(S) : 1.0f;
#pragma unroll 1
    for (uint32_t s = 0; s < RC_MAX_SPLIT; s++) {
        const bool active = s < S;
        const uint32_t k = key | (s << 24);        // split 0 keeps the plain key
        bool emitShadow = false, emitRay = false;
        float4 shRay0{}, shRay1{}, shPay{}, outRay0{}, outRay1{}, outPay{};
        if (active) {
            Surf ss = sf;
            V3 c, so, sd;
            float st, pl = 0.0f;
            if (direct_light(p.sc, ss, thr, k, p.sample, p.bounce, p.seed, p.epsilon, c, so, sd, st, &pl)) {
                c = c * (cont ? power_weight(pl, bsdf_pdf(ss, ss.L)) * invS : invS);
                emitShadow = true;
                shRay0 = make_float4(so.x, so.y, so.z, __uint_as_float(k));
                shRay1 = make_float4(sd.x, sd.y, sd.z, st);
                shPay = make_float4(c.x, c.y, c.z, __uint_as_float(k));
            }
            if (cont) {
                V3 o, d, t2 = thr;
                bool spec = false;
                if (continue_path(ss, t2, k, p.sample, p.bounce, p.seed, p.epsilon, o, d, &spec)) {
                    emitRay = true;
                    t2 = t2 * invS;
                    outRay0 = make_float4(o.x, o.y, o.z, __uint_as_float(k));
                    outRay1 = make_float4(d.x, d.y, d.z, mis_hit_factor(p.sc, ss, d, spec));
                    outPay = make_float4(t2.x, t2.y, t2.z, __uint_as_float(k));
                }
            }
        }
        if (!__any_sync(0xffffffffu, emitShadow || emitRay)) {
            if (!__any_sync(0xffffffffu, s + 1 < S)) break;
            continue;
        }
        uint32_t si, ri;
        if (rc_append(p.n_shadow, cap, emitShadow, lane, p.overflow, si)) {
            float4* r = p.shadow_rays + size_t(si) * 3;
            r[0] = shRay0;
            r[1] = make_float4(shRay1.x, shRay1.y, shRay1.z, 0.0f);
            r[2] = make_float4(shRay1.w, __int_as_float(-1), __int_as_float(-1), 0.0f);
            p.shadow_pay[si] = shPay;
        }
        if (rc_append(p.n_out, cap, emitRay, lane, p.overflow, ri)) {
            float4* r = p.rays_out + size_t(ri) * 3;
            r[0] = outRay0;
            r[1] = outRay1;
            r[2] = make_float4(0.0f, __int_as_float(-1), __int_as_float(-1), 0.0f);
            p.pay_out[ri] = outPay;
        }
    }
}

}  // namespace atlas::rt::dev
