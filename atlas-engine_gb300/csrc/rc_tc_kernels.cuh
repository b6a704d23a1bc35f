// Radiance-cache inference on the 5th-generation tensor cores: the fused
// hash-grid encoding + 6-layer BF16 MLP of rc_kernels.cuh with every layer
// a tcgen05.mma (M = 128 queries, N = 64 or 16, K = 64 in four K = 16 steps)
// accumulating in FP32 tensor memory.
//
// Per CTA (two independent groups of 128 threads, one query row per thread;
// 3 CTAs per SM), per group:
//  * shared memory holds the weights of all six layers (shared by the
//    groups) and the group's 128 x 64 BF16 activation tile, both in the
//    no-swizzle core-matrix layout the MMA
//    descriptors describe: 8 rows x 16 bytes per core matrix, core matrices
//    128 bytes apart along K (leading byte offset) and 1024 bytes apart along
//    M / N (stride byte offset);
//  * warp 0 allocates 128 tensor-memory columns, 64 per group (lane i =
//    query row i of the group's tile);
//  * per layer thread 0 issues the four MMAs and commits them to an
//    mbarrier; every thread waits on it (bounded by the global timer), reads
//    its own row back with tcgen05.ld (the group's warp w owns lanes
//    32w..32w+31),
//    applies ReLU, rounds to BF16 and writes the row of the next layer's
//    input tile; a proxy fence and the group's named barrier hand the tile
//    back to the tensor core;
//  * after the output layer each thread has its query's RGB in registers and
//    adds (throughput x max(0, prediction)) into the image or writes the
//    prediction.
// A wait that times out sets kErrTimeout in the context's error word (the
// next ae_rt_synchronize reports AE_RT_TIMEOUT), stops the CTA's loop and
// still frees the tensor memory.
#pragma once

#include "rc_kernels.cuh"

namespace atlas::rt::dev {

constexpr uint32_t kErrTimeout = 0x4u;

constexpr uint32_t RCT_LBO = 128;                       // core matrices along K
constexpr uint32_t RCT_SBO = 1024;                      // core matrices along M / N (8 x 128 B of K = 64)
constexpr uint32_t RCT_ABYTES = RC_TILE * RC_W * 2;     // 16 KB activation tile
constexpr uint32_t RCT_WLAYER = RC_W * RC_W * 2;        // 8 KB per hidden layer
constexpr uint32_t RCT_WBYTES = RC_HIDDEN * RCT_WLAYER + RC_OUT * RC_W * 2;   // 43,008
constexpr uint32_t RCT_GROUPS = 2;                      // independent 128-row tile groups per CTA
constexpr uint32_t RCT_THREADS = RCT_GROUPS * RC_TILE;
constexpr uint32_t RCT_SMEM = RCT_WBYTES + RCT_GROUPS * RCT_ABYTES + 64;      // + mbarriers, flags, TMEM address
constexpr uint32_t RCT_TMEM_COLS = RCT_GROUPS * 64;

// Byte offset of the 16-byte chunk (row, k-block kb) in the blocked layout.
__device__ __forceinline__ uint32_t rct_off(uint32_t row, uint32_t kb) {
    return (row >> 3) * RCT_SBO + kb * RCT_LBO + (row & 7u) * 16u;
}

// tcgen05 shared-memory matrix descriptor: start address, leading and stride
// byte offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t rct_desc(uint32_t saddr) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(RCT_LBO >> 4) << 16) | (uint64_t(RCT_SBO >> 4) << 32) |
           (uint64_t(1) << 46);
}

// Instruction descriptor of kind::f16: F32 accumulator, BF16 A and B, both
// K-major, N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t rct_idesc(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the mbarrier phase with parity `parity`; false after ~200 ms of
// the global timer, or after 2^25 polls whatever the timer says.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const uint64_t start = global_ns();
    for (uint32_t it = 0; it < (1u << 25); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 63u) == 63u && global_ns() - start > 200000000ull) return false;
    }
    return false;
}

// Barrier of one 128-thread tile group (named barrier 1 + group).
__device__ __forceinline__ void group_sync(uint32_t g) {
    static_assert(RCT_GROUPS == 2, "one named barrier per group");
    if (g == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
    else asm volatile("bar.sync 2, 128;" ::: "memory");
}

// rc_encode_values with four levels' table reads in flight at once.
__device__ __forceinline__ void rc_encode_values_wide(const RcGrid& g, const float4& q0, const float4& q1,
                                                      const float4& q2, __nv_bfloat162 v[32]) {
    float x[3];
    rc_unit(g, q0, x);
#pragma unroll 4
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
#pragma unroll
    for (int k = 0; k < 8; k++) v[16 + k] = __floats2bfloat162_rn(sh[2 * k], sh[2 * k + 1]);
    v[24] = __floats2bfloat162_rn(q2.x, q2.y);
    v[25] = __floats2bfloat162_rn(q2.z, q0.w);
    v[26] = __floats2bfloat162_rn(q2.w, 0.0f);
#pragma unroll
    for (int k = 27; k < 32; k++) v[k] = __floats2bfloat162_rn(0.0f, 0.0f);
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

template <int MODE>
static __global__ void __launch_bounds__(RCT_THREADS) rc_infer_tc_kernel(RcMlpParams p) {
    extern __shared__ __align__(1024) unsigned char rct_smem[];
    unsigned char* wsm = rct_smem;
    unsigned char* tail = rct_smem + RCT_WBYTES + RCT_GROUPS * RCT_ABYTES;
    uint64_t* mbars = reinterpret_cast<uint64_t*>(tail);                       // one per group
    uint32_t* fail = reinterpret_cast<uint32_t*>(tail + 8 * RCT_GROUPS);       // one per group
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tail + 12 * RCT_GROUPS);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t g = tid / RC_TILE, row = tid % RC_TILE, gwarp = warp & 3u;
    unsigned char* act = rct_smem + RCT_WBYTES + g * RCT_ABYTES;

    // weights of every layer in the blocked layout (rows = output neurons, K = 64)
    for (uint32_t i = tid; i < uint32_t(RC_WROWS) * 8u; i += blockDim.x) {
        const uint32_t r = i >> 3, kb = i & 7u;
        const uint32_t layer = r < uint32_t(RC_HIDDEN * RC_W) ? r / RC_W : uint32_t(RC_HIDDEN);
        const uint32_t n = r - layer * RC_W;
        *reinterpret_cast<uint4*>(wsm + layer * RCT_WLAYER + rct_off(n, kb)) =
            reinterpret_cast<const uint4*>(p.weights + size_t(r) * RC_W)[kb];
    }
    if (row == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbars[g])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail[g] = 0u;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tslot)), "r"(RCT_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot + g * 64u;                     // this group's 64 columns
    const uint32_t a_addr = smem_u32(act), w_addr = smem_u32(wsm), mbar_addr = smem_u32(&mbars[g]);
    const uint32_t lane_base = tmem + ((gwarp * 32u) << 16);

    const uint32_t n = p.n_dev ? min(*p.n_dev, p.n) : p.n;
    const uint32_t first = p.offset_dev ? min(*p.offset_dev, n) : p.offset;
    const uint32_t count = n > first ? n - first : 0u;
    const uint32_t tiles = (count + RC_TILE - 1) / RC_TILE;
    uint32_t parity = 0;
    bool ok = true;
    for (uint32_t tile = blockIdx.x * RCT_GROUPS + g; tile < tiles && ok; tile += gridDim.x * RCT_GROUPS) {
        const uint32_t gi = tile * RC_TILE + row;
        const bool valid = gi < count;
        float4 q0 = make_float4(0, 0, 0, 0), q1 = q0, q2 = q0, q3 = q0;
        __nv_bfloat162 v[32];
        if (valid) {
            const float4* rec = p.recs + size_t(first + gi) * 4;
            q0 = rec[0]; q1 = rec[1]; q2 = rec[2]; q3 = rec[3];
            rc_encode_values_wide(p.grid, q0, q1, q2, v);
        } else {
#pragma unroll
            for (int k = 0; k < 32; k++) v[k] = __floats2bfloat162_rn(0.0f, 0.0f);
        }
#pragma unroll
        for (uint32_t kb = 0; kb < 8; kb++)
            *reinterpret_cast<uint4*>(act + rct_off(row, kb)) = reinterpret_cast<const uint4*>(v)[kb];
        proxy_fence();
        tc_fence_before();
        group_sync(g);
        tc_fence_after();
#pragma unroll 1
        for (int l = 0; l <= RC_HIDDEN; l++) {
            const uint32_t nn = l < RC_HIDDEN ? uint32_t(RC_W) : uint32_t(RC_OUT);
            if (row == 0 && !p.skip_mma) {
                const uint32_t idesc = rct_idesc(RC_TILE, nn);
#pragma unroll
                for (uint32_t s = 0; s < 4; s++)
                    tc_mma(tmem, rct_desc(a_addr + s * 2u * RCT_LBO),
                           rct_desc(w_addr + uint32_t(l) * RCT_WLAYER + s * 2u * RCT_LBO), idesc, s);
                tc_commit(mbar_addr);
            }
            if (!mbar_wait(mbar_addr, parity)) fail[g] = 1u;
            parity ^= 1u;
            // every thread of the group takes the same decision (a late arrival
            // seen by some threads only must not split the group's barriers)
            group_sync(g);
            ok = fail[g] == 0u;
            tc_fence_after();
            if (!ok) break;
            if (l < RC_HIDDEN) {
#pragma unroll
                for (uint32_t c = 0; c < 4; c++) {
                    float x[16];
                    tc_ld16(lane_base + c * 16u, x);
                    uint32_t pk[8];
#pragma unroll
                    for (int k = 0; k < 8; k++) pk[k] = pack_bf16(fmaxf(x[2 * k], 0.0f), fmaxf(x[2 * k + 1], 0.0f));
                    *reinterpret_cast<uint4*>(act + rct_off(row, 2 * c)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4*>(act + rct_off(row, 2 * c + 1)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
                proxy_fence();
            } else {
                float x[16];
                tc_ld16(lane_base, x);
                if (valid) {
                    if (MODE == RC_PREDICT) {
                        p.out[first + gi] = make_float4(x[0], x[1], x[2], 0.0f);
                    } else {
                        // split paths can query for the same pixel in one launch
                        float4* a = p.accum + (__float_as_uint(q1.w) & kPixelMask);
                        atomicAdd(&a->x, q3.x * fmaxf(x[0], 0.0f));
                        atomicAdd(&a->y, q3.y * fmaxf(x[1], 0.0f));
                        atomicAdd(&a->z, q3.z * fmaxf(x[2], 0.0f));
                    }
                }
            }
            tc_fence_before();
            group_sync(g);
            tc_fence_after();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (!ok && row == 0 && p.error_word) atomicOr(p.error_word, kErrTimeout);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(*tslot), "r"(RCT_TMEM_COLS)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Training on the tensor cores: encode + forward + relative-L2 loss +
// backward, every GEMM a tcgen05.mma with FP32 accumulators in tensor memory.
//
// One CTA per SM (shared and tensor memory), persistent over the tiles of its
// slice, 128 records per tile, two warp groups:
//  * the MMA group (warps 0-3, one record row per thread) issues the MMAs,
//    reads the accumulators back, applies ReLU / the loss / the ReLU
//    derivative and writes the next operand tile;
//  * the producer group (warps 4-7) encodes tile k + 1's records (the
//    hash-grid gathers) into the other of two input tiles while the MMA group
//    works on tile k, and scatters the hash-grid gradient of tile k - 1 (the
//    atomics) from a staging buffer the MMA group fills at the end of a tile.
// The groups hand buffers over through mbarriers: `full[b]` (producer ->
// MMA group: input tile b holds the next tile; the producer has scattered
// the gradient staged in buffer b two tiles before) and `grads[b]` (MMA group
// -> producer: tile k's input gradient is staged in buffer b and every MMA
// reading input tile b has completed).
//
// All operands stay in the blocked no-swizzle layout of the forward pass: a
// core matrix is 8 rows x 16 bytes (8 BF16 along the row's inner dimension),
// core matrices 128 bytes apart along that dimension and 1024 bytes apart
// along the rows.  Read K-major (rows = M or N, inner = K) the leading byte
// offset is 128 and the stride byte offset 1024; read MN-major (inner = M or
// N, rows = K) the same bytes have stride byte offset 128 and leading byte
// offset 1024, with the instruction's transpose bit for that operand.  So no
// operand is copied transposed:
//  * forward      Z_l   = A_l  W_l^T   A = A_l  (K-major), B = W_l (K-major)
//  * input grad   dA_l  = dZ_l W_l     A = dZ_l (K-major), B = W_l (MN-major)
//  * weight grad  dW_l += dZ_l^T A_l   A = dZ_l (MN-major), B = A_l (MN-major)
// The weight-gradient GEMM has M = 64 outputs (16 for the output layer); it
// runs as M = 128, whose rows past the layer's outputs read the following
// records' bytes of the dZ tile (a 2 KB margin after it keeps those reads
// inside shared memory) and are never read back.  Tensor memory holds the
// forward / input-gradient accumulator (columns 0-63) and the six weight
// gradients (64 columns each from column 64), which accumulate over every
// tile of the CTA and are added to the global FP32 gradient once, at the end.
// Every wait is bounded (kErrTimeout); a CTA that gave up still frees its
// tensor memory.
constexpr uint32_t RCTT_A0 = 44032;                                      // 2 input tiles, after the weights
constexpr uint32_t RCTT_AH = RCTT_A0 + 2 * RCT_ABYTES;                   // hidden activations A_1 .. A_5
constexpr uint32_t RCTT_DZ = RCTT_AH + RC_HIDDEN * RCT_ABYTES;           // dP / dZ tile
constexpr uint32_t RCTT_DG = RCTT_DZ + RCT_ABYTES + 2048;                // + margin; 2 x 128 grid-gradient rows (64 B)
constexpr uint32_t RCTT_Q0 = RCTT_DG + 2 * RC_TILE * 64;                 // 2 x 128 record positions (float4)
constexpr uint32_t RCTT_TAIL = RCTT_Q0 + 2 * RC_TILE * 16;               // mbarriers, flag, tensor-memory address
constexpr uint32_t RCTT_SMEM = RCTT_TAIL + 64;
constexpr uint32_t RCTT_THREADS = 2 * RC_TILE;
constexpr uint32_t RCTT_TMEM_COLS = 512;
constexpr uint32_t RCTT_DW = 64;                                         // first weight-gradient column

// MN-major reading of the blocked layout (see above).
__device__ __forceinline__ uint64_t rct_desc_mn(uint32_t saddr) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(1024u >> 4) << 16) | (uint64_t(128u >> 4) << 32) |
           (uint64_t(1) << 46);
}

// kind::f16 instruction descriptor with A (bit 15) / B (bit 16) read MN-major.
__host__ __device__ constexpr uint32_t rct_idesc_t(uint32_t m, uint32_t n, bool a_mn, bool b_mn) {
    return rct_idesc(m, n) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

static __global__ void __launch_bounds__(RCTT_THREADS, 1) rc_train_tc_kernel(RcMlpParams p) {
    extern __shared__ __align__(1024) unsigned char rctt_smem[];
    unsigned char* wsm = rctt_smem;
    unsigned char* dzt = rctt_smem + RCTT_DZ;
    unsigned char* tail = rctt_smem + RCTT_TAIL;
    uint64_t* bars = reinterpret_cast<uint64_t*>(tail);        // [0] MMA, [1..2] full, [3..4] grads
    uint32_t* fail = reinterpret_cast<uint32_t*>(tail + 40);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tail + 44);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const bool mma_group = tid < RC_TILE;
    const uint32_t row = tid & (RC_TILE - 1u);

    for (uint32_t i = tid; i < uint32_t(RC_WROWS) * 8u; i += blockDim.x) {
        const uint32_t r = i >> 3, kb = i & 7u;
        const uint32_t layer = r < uint32_t(RC_HIDDEN * RC_W) ? r / RC_W : uint32_t(RC_HIDDEN);
        const uint32_t n = r - layer * RC_W;
        *reinterpret_cast<uint4*>(wsm + layer * RCT_WLAYER + rct_off(n, kb)) =
            reinterpret_cast<const uint4*>(p.weights + size_t(r) * RC_W)[kb];
    }
    // the dZ tile and its margin start as zeros (the M = 128 reads see no stale NaNs)
    for (uint32_t i = tid; i < (RCT_ABYTES + 2048u) / 16u; i += blockDim.x)
        reinterpret_cast<uint4*>(dzt)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bars[0])) : "memory");
        for (int b = 1; b < 5; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bars[b])), "r"(RC_TILE) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *fail = 0u;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tslot)), "r"(RCTT_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    const uint32_t n = p.n_dev ? min(*p.n_dev, p.n) : p.n;
    uint32_t first = p.offset, count = n > p.offset ? n - p.offset : 0u;
    if (p.slices) {
        first = uint32_t(uint64_t(n) * p.slice / p.slices);
        count = uint32_t(uint64_t(n) * (p.slice + 1) / p.slices) - first;
    }
    const uint32_t tiles = (count + RC_TILE - 1) / RC_TILE;
    const uint32_t my_tiles = tiles > blockIdx.x ? (tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
    const uint32_t mb = smem_u32(&bars[0]);
    auto full_bar = [&](uint32_t b) { return smem_u32(&bars[1 + b]); };
    auto grads_bar = [&](uint32_t b) { return smem_u32(&bars[3 + b]); };
    auto act_addr = [&](int l, uint32_t b) {
        return smem_u32(rctt_smem) + (l == 0 ? RCTT_A0 + b * RCT_ABYTES : RCTT_AH + uint32_t(l - 1) * RCT_ABYTES);
    };
    auto act_ptr = [&](int l, uint32_t b) {
        return rctt_smem + (l == 0 ? RCTT_A0 + b * RCT_ABYTES : RCTT_AH + uint32_t(l - 1) * RCT_ABYTES);
    };
    bool ok = true;

    if (mma_group) {
        const float inv_norm = count ? 1.0f / (3.0f * float(count)) : 0.0f;
        const uint32_t lane_base = tmem + ((warp * 32u) << 16);
        const uint32_t w_addr = smem_u32(wsm), dz_addr = smem_u32(dzt);
        uint32_t parity = 0, accw = 0;
        // thread 0 issues and commits; the group waits and takes one decision
        auto wait_mma = [&]() {
            if (!mbar_wait(mb, parity)) *fail = 1u;
            parity ^= 1u;
            group_sync(0);
            ok = *fail == 0u;
            tc_fence_after();
        };
        auto put_row = [&](unsigned char* tile, const uint32_t (&pk)[32]) {
#pragma unroll
            for (uint32_t kb = 0; kb < 8; kb++)
                *reinterpret_cast<uint4*>(tile + rct_off(row, kb)) =
                    make_uint4(pk[4 * kb], pk[4 * kb + 1], pk[4 * kb + 2], pk[4 * kb + 3]);
        };
        auto handoff = [&]() {              // the group's smem writes -> the tensor core
            proxy_fence();
            tc_fence_before();
            group_sync(0);
            tc_fence_after();
        };
#pragma unroll 1
        for (uint32_t k = 0; k < my_tiles && ok; k++) {
            const uint32_t b = k & 1u;
            if (!mbar_wait(full_bar(b), (k >> 1) & 1u)) *fail = 1u;
            group_sync(0);
            ok = *fail == 0u;
            tc_fence_after();
            if (!ok) break;
            const uint32_t gi = (blockIdx.x + k * gridDim.x) * RC_TILE + row;
            const bool valid = gi < count;
            const float4 q3 = valid ? p.recs[size_t(first + gi) * 4 + 3] : make_float4(0, 0, 0, 0);
            // ---- forward: A_{l+1} = relu(A_l W_l^T); the output layer's 16 columns ----
#pragma unroll 1
            for (int l = 0; l <= RC_HIDDEN && ok; l++) {
                const uint32_t nn = l < RC_HIDDEN ? uint32_t(RC_W) : uint32_t(RC_OUT);
                if (row == 0) {
                    const uint32_t idesc = rct_idesc(RC_TILE, nn);
#pragma unroll
                    for (uint32_t s = 0; s < 4; s++)
                        tc_mma(tmem, rct_desc(act_addr(l, b) + s * 2u * RCT_LBO),
                               rct_desc(w_addr + uint32_t(l) * RCT_WLAYER + s * 2u * RCT_LBO), idesc, s);
                    tc_commit(mb);
                }
                wait_mma();
                if (!ok) break;
                if (l < RC_HIDDEN) {
                    uint32_t pk[32];
#pragma unroll
                    for (uint32_t c = 0; c < 4; c++) {
                        float x[16];
                        tc_ld16(lane_base + c * 16u, x);
#pragma unroll
                        for (int j = 0; j < 8; j++) pk[c * 8 + j] = pack_bf16(fmaxf(x[2 * j], 0.0f), fmaxf(x[2 * j + 1], 0.0f));
                    }
                    put_row(act_ptr(l + 1, b), pk);
                } else {
                    // relative L2 loss over the 3 colour outputs and its gradient dP
                    float x[16];
                    tc_ld16(lane_base, x);
                    const float tg[3] = { q3.x, q3.y, q3.z };
                    float lsum = 0.0f;
                    uint32_t pk[32];
#pragma unroll
                    for (int j = 0; j < 32; j++) pk[j] = 0u;
                    float d[3] = { 0.0f, 0.0f, 0.0f };
                    if (valid) {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const float den = x[c] * x[c] + 0.01f;
                            const float diff = x[c] - tg[c];
                            lsum += diff * diff / den;
                            d[c] = 2.0f * diff / den * inv_norm;
                        }
                    }
                    pk[0] = pack_bf16(d[0], d[1]);
                    pk[1] = pack_bf16(d[2], 0.0f);
                    put_row(dzt, pk);
                    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, off);
                    if (lane == 0) atomicAdd(p.loss, lsum * inv_norm);
                }
                handoff();
            }
            if (!ok) break;
            // ---- backward: layer l's weight gradient and the gradient of its input ----
#pragma unroll 1
            for (int l = RC_HIDDEN; l >= 0 && ok; l--) {
                if (row == 0) {
                    const uint32_t kout = l < RC_HIDDEN ? 4u : 1u;    // K = outputs of the layer, 16 per step
                    // dW_l (+)= dZ_l^T A_l: M = 128 (outputs, padded), N = 64 inputs, K = 128 records
                    const uint32_t idw = rct_idesc_t(RC_TILE, RC_W, true, true);
#pragma unroll 1
                    for (uint32_t s = 0; s < RC_TILE / 16u; s++)
                        tc_mma(tmem + RCTT_DW + uint32_t(l) * 64u, rct_desc_mn(dz_addr + s * 2u * 1024u),
                               rct_desc_mn(act_addr(l, b) + s * 2u * 1024u), idw, (accw | s) ? 1u : 0u);
                    // dA_l = dZ_l W_l: M = 128 records, N = 64 inputs, K = outputs
                    const uint32_t idx = rct_idesc_t(RC_TILE, RC_W, false, true);
#pragma unroll 1
                    for (uint32_t s = 0; s < kout; s++)
                        tc_mma(tmem, rct_desc(dz_addr + s * 2u * RCT_LBO),
                               rct_desc_mn(w_addr + uint32_t(l) * RCT_WLAYER + s * 2u * 1024u), idx, s);
                    tc_commit(mb);
                }
                wait_mma();
                if (!ok) break;
                float g[64];
#pragma unroll
                for (uint32_t c = 0; c < 4; c++) tc_ld16(lane_base + c * 16u, g + c * 16);
                if (l > 0) {
                    // dZ_{l-1} = dA_l * relu'(A_l), A_l = relu(Z_{l-1}) read back from its tile
                    const unsigned char* al = act_ptr(l, b);
                    uint32_t pk[32];
#pragma unroll
                    for (uint32_t kb = 0; kb < 8; kb++) {
                        const uint4 a4 = *reinterpret_cast<const uint4*>(al + rct_off(row, kb));
                        const uint32_t aw[4] = { a4.x, a4.y, a4.z, a4.w };
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            __nv_bfloat162 a2;
                            *reinterpret_cast<uint32_t*>(&a2) = aw[h];
                            const float2 af = __bfloat1622float2(a2);
                            const int j = int(kb) * 8 + h * 2;
                            pk[kb * 4 + h] = pack_bf16(af.x > 0.0f ? g[j] : 0.0f, af.y > 0.0f ? g[j + 1] : 0.0f);
                        }
                    }
                    put_row(dzt, pk);
                    handoff();
                } else {
                    // dA_0's hash-grid part, BF16 like the inputs, for the producer's scatter
                    uint4* dg = reinterpret_cast<uint4*>(rctt_smem + RCTT_DG + (b * RC_TILE + row) * 64u);
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        dg[j] = make_uint4(pack_bf16(g[8 * j], g[8 * j + 1]), pack_bf16(g[8 * j + 2], g[8 * j + 3]),
                                           pack_bf16(g[8 * j + 4], g[8 * j + 5]), pack_bf16(g[8 * j + 6], g[8 * j + 7]));
                }
            }
            if (!ok) break;
            accw = 1u;
            // every MMA of the tile has completed (waited): input tile b and
            // the staged gradient go back to the producer
            tc_fence_before();
            mbar_arrive(grads_bar(b));
        }
        // ---- the CTA's weight gradients into the global FP32 sums (lanes = outputs) ----
        if (ok && accw && warp < 2) {
            const uint32_t out = row;       // warps 0 and 1: lanes 0-63
#pragma unroll 1
            for (int l = 0; l <= RC_HIDDEN; l++) {
                float g[64];
#pragma unroll
                for (uint32_t c = 0; c < 4; c++)
                    tc_ld16(lane_base + RCTT_DW + uint32_t(l) * 64u + c * 16u, g + c * 16);
                const uint32_t nout = l < RC_HIDDEN ? uint32_t(RC_W) : uint32_t(RC_OUT);
                if (out < nout) {
                    float* gw = p.grad_w + size_t(l) * RC_W * RC_W + size_t(out) * RC_W;
#pragma unroll
                    for (int j = 0; j < 64; j += 2)
                        atomicAdd(reinterpret_cast<float2*>(gw + j), make_float2(g[j], g[j + 1]));
                }
            }
        }
    } else {
        // producer: encode tile k into input tile k & 1 after scattering the
        // gradient of tile k - 2, staged in the same buffer; then the last two
#pragma unroll 1
        for (uint32_t k = 0; k < my_tiles + 2 && ok; k++) {
            const uint32_t b = k & 1u;
            if (k >= 2) {
                const uint32_t kk = k - 2;
                if (!mbar_wait(grads_bar(b), (kk >> 1) & 1u)) { *fail = 1u; ok = false; break; }
                const uint32_t gi = (blockIdx.x + kk * gridDim.x) * RC_TILE + row;
                if (gi < count) {
                    const float4 q0 = reinterpret_cast<const float4*>(rctt_smem + RCTT_Q0)[b * RC_TILE + row];
                    rc_encode_backward(p.grid, q0, reinterpret_cast<const __nv_bfloat16*>(
                                                       rctt_smem + RCTT_DG + (b * RC_TILE + row) * 64u));
                }
            }
            if (k < my_tiles) {
                const uint32_t gi = (blockIdx.x + k * gridDim.x) * RC_TILE + row;
                __nv_bfloat162 v[32];
                float4 q0 = make_float4(0, 0, 0, 0);
                if (gi < count) {
                    const float4* rec = p.recs + size_t(first + gi) * 4;
                    q0 = rec[0];
                    rc_encode_values_wide(p.grid, q0, rec[1], rec[2], v);
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++) v[j] = __floats2bfloat162_rn(0.0f, 0.0f);
                }
                unsigned char* a0 = act_ptr(0, b);
#pragma unroll
                for (uint32_t kb = 0; kb < 8; kb++)
                    *reinterpret_cast<uint4*>(a0 + rct_off(row, kb)) = reinterpret_cast<const uint4*>(v)[kb];
                reinterpret_cast<float4*>(rctt_smem + RCTT_Q0)[b * RC_TILE + row] = q0;
                proxy_fence();
                mbar_arrive(full_bar(b));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*fail && tid == 0 && p.error_word) atomicOr(p.error_word, kErrTimeout);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(RCTT_TMEM_COLS)
                     : "memory");
}

}  // namespace atlas::rt::dev
