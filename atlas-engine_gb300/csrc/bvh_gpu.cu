// GPU BVH build (include/atlas_rt.h, ae_rt_mesh_build): a linear BVH over
// triangle centroids, emitted directly in the engine's GPUBVHNode /
// GPUBVHTriangle layouts (RTStructures.h:23-27, :95-103) and registered as a
// mesh of the context, so every trace entry point can use it at once.
//
// The engine builds its BVHs on the CPU with binned SAH (Volume::BVH,
// BVH.cpp:14-56, 0.13 s for 65,536 and ~0.8 s for 524,288 triangles on 8
// cores); this is the GPU alternative for meshes that change or arrive at
// run time.  Steps (Karras, "Maximizing Parallelism in the Construction of
// BVHs, Octrees, and k-d Trees", HPG 2012):
//   1. centroid bounds (one reduction, order-preserving integer min/max);
//   2. 30-bit Morton code of each centroid in those bounds, made unique by the
//      triangle index in the low 32 bits of a 64-bit key;
//   3. radix sort of the keys (CUB, from the CUDA toolkit);
//   4. one thread per inner node finds its key range and split by binary
//      search over the common-prefix lengths of neighbouring keys;
//   5. bounds bottom-up: every leaf walks towards the root, and at each node
//      the second of its two children to arrive (an atomic counter per node)
//      forms the union and continues;
//   6. emission: inner node i -> GPUBVHNode i (children's boxes and
//      pointers, ~p for the leaf at sorted position p; padding0 = 1 where a
//      coordinate lies outside the traversal's fast-division window), sorted
//      position p -> GPUBVHTriangle p (one triangle per leaf, endOfNode set).
// The root is node 0, as the traversal expects; children are not in
// pre-order (that is the host validator's test for uploaded BVHs, which
// this builder's trees skip: they are acyclic by construction).
#include "atlas_rt.h"
#include "context.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <cmath>
#include <cstring>
#include <vector>

using namespace atlas::rt::host;

namespace {

__device__ __forceinline__ uint32_t flip_float(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unflip_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// 10 bits spread to every third bit.
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box tri_box(const float* v) {
    Box b;
    for (int k = 0; k < 3; k++) {
        b.lo[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
        b.hi[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
    }
    return b;
}

// Centroid bounds: [0..2] min, [3..5] max, as flipped integers.
__global__ void centroid_bounds_kernel(const float* verts, uint32_t n, uint32_t* bounds) {
    float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Box b = tri_box(verts + size_t(i) * 9);
        for (int k = 0; k < 3; k++) {
            const float c = 0.5f * (b.lo[k] + b.hi[k]);
            lo[k] = fminf(lo[k], c);
            hi[k] = fmaxf(hi[k], c);
        }
    }
    for (int k = 0; k < 3; k++) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    }
    if ((threadIdx.x & 31u) == 0) {
        for (int k = 0; k < 3; k++) {
            atomicMin(&bounds[k], flip_float(lo[k]));
            atomicMax(&bounds[3 + k], flip_float(hi[k]));
        }
    }
}

__global__ void morton_kernel(const float* verts, uint32_t n, const uint32_t* bounds, unsigned long long* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Box b = tri_box(verts + size_t(i) * 9);
    uint32_t code = 0;
    for (int k = 0; k < 3; k++) {
        const float lo = unflip_float(bounds[k]), hi = unflip_float(bounds[3 + k]);
        const float c = 0.5f * (b.lo[k] + b.hi[k]);
        const float ext = hi - lo;
        float x = ext > 0.0f ? (c - lo) / ext : 0.5f;
        x = fminf(fmaxf(x, 0.0f), 1.0f);
        const uint32_t q = min(uint32_t(x * 1024.0f), 1023u);
        code |= spread10(q) << (2 - k);
    }
    keys[i] = (static_cast<unsigned long long>(code) << 32) | i;
}

__device__ __forceinline__ int delta(const unsigned long long* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return __clzll(static_cast<long long>(keys[i] ^ keys[j]));
}

// Inner node i of n - 1: children as engine pointers (inner index, or ~p for
// the leaf at sorted position p) and the parent links.
__global__ void karras_kernel(const unsigned long long* keys, int n, int32_t* child, int32_t* node_parent,
                              int32_t* leaf_parent) {
    const int i = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n - 1) return;
    const int d = delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    int32_t left, right;
    if (lo == gamma) {
        left = ~gamma;
        leaf_parent[gamma] = i;
    } else {
        left = gamma;
        node_parent[gamma] = i;
    }
    if (hi == gamma + 1) {
        right = ~(gamma + 1);
        leaf_parent[gamma + 1] = i;
    } else {
        right = gamma + 1;
        node_parent[gamma + 1] = i;
    }
    child[2 * i] = left;
    child[2 * i + 1] = right;
}

__device__ __forceinline__ Box load_box(const float* b) {
    Box r;
    for (int k = 0; k < 3; k++) {
        r.lo[k] = __ldcg(b + k);
        r.hi[k] = __ldcg(b + 3 + k);
    }
    return r;
}

__device__ __forceinline__ Box child_box(int32_t c, const float* node_box, const float* leaf_box) {
    return c >= 0 ? load_box(node_box + size_t(c) * 6) : load_box(leaf_box + size_t(~c) * 6);
}

// Leaf boxes in sorted order, then the inner boxes bottom-up.
__global__ void refit_kernel(const float* verts, const unsigned long long* keys, int n, const int32_t* child,
                             const int32_t* node_parent, const int32_t* leaf_parent, float* leaf_box,
                             float* node_box, uint32_t* arrivals, uint32_t* error) {
    const int p = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (p >= n) return;
    const uint32_t src = uint32_t(keys[p] & 0xffffffffull);
    const Box b = tri_box(verts + size_t(src) * 9);
    for (int k = 0; k < 3; k++) {
        leaf_box[size_t(p) * 6 + k] = b.lo[k];
        leaf_box[size_t(p) * 6 + 3 + k] = b.hi[k];
    }
    __threadfence();
    int node = leaf_parent[p];
    // a path to the root is at most 63 inner nodes long (one per bit of the
    // unique 62-bit keys, plus the root); the bound only guards the loop
    for (int hops = 0; node >= 0; hops++) {
        if (hops > 64 || node >= n - 1) {
            atomicOr(error, 1u);
            return;
        }
        if (atomicAdd(&arrivals[node], 1u) == 0u) return;   // the sibling's walk finishes this node
        __threadfence();
        const Box l = child_box(child[2 * node], node_box, leaf_box);
        const Box r = child_box(child[2 * node + 1], node_box, leaf_box);
        float* o = node_box + size_t(node) * 6;
        for (int k = 0; k < 3; k++) {
            o[k] = fminf(l.lo[k], r.lo[k]);
            o[3 + k] = fmaxf(l.hi[k], r.hi[k]);
        }
        __threadfence();
        node = node == 0 ? -1 : node_parent[node];
    }
}

__device__ __forceinline__ bool in_window(float v) {
    const float a = fabsf(v);
    return a == 0.0f || (a >= 9.094947017729282e-13f && a <= 1.099511627776e12f);
}

__global__ void emit_kernel(const float* verts, const int32_t* material, const float* opacity,
                            const unsigned long long* keys, int n, const int32_t* child, const float* node_box,
                            const float* leaf_box, ae_bvh_node* nodes, ae_bvh_triangle* tris, uint32_t* order) {
    const int i = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < n - 1) {
        ae_bvh_node nd;
        const int32_t l = child[2 * i], r = child[2 * i + 1];
        const float* lb = l >= 0 ? node_box + size_t(l) * 6 : leaf_box + size_t(~l) * 6;
        const float* rb = r >= 0 ? node_box + size_t(r) * 6 : leaf_box + size_t(~r) * 6;
        bool ok = true;
        for (int k = 0; k < 3; k++) {
            nd.leftAABB.min[k] = lb[k];
            nd.leftAABB.max[k] = lb[3 + k];
            nd.rightAABB.min[k] = rb[k];
            nd.rightAABB.max[k] = rb[3 + k];
            ok = ok && in_window(lb[k]) && in_window(lb[3 + k]) && in_window(rb[k]) && in_window(rb[3 + k]);
        }
        nd.leftPtr = l;
        nd.rightPtr = r;
        nd.padding0 = ok ? 0 : 1;
        nd.padding1 = 0;
        nodes[i] = nd;
    }
    if (i < n) {
        const uint32_t src = uint32_t(keys[i] & 0xffffffffull);
        const float* v = verts + size_t(src) * 9;
        ae_bvh_triangle t;
        t.v0[0] = v[0]; t.v0[1] = v[1]; t.v0[2] = v[2]; t.v0[3] = 1.0f;
        t.v1[0] = v[3]; t.v1[1] = v[4]; t.v1[2] = v[5];
        const int32_t m = material ? material[src] : 0;
        t.v1[3] = __int_as_float(m);
        t.v2[0] = v[6]; t.v2[1] = v[7]; t.v2[2] = v[8];
        t.v2[3] = opacity ? opacity[src] : 1.0f;
        tris[i] = t;
        if (order) order[i] = src;
    }
}

// The one-triangle mesh: one node whose two children are the triangle, as
// the engine's builder emits it (its root split duplicates the reference).
void OneTriangle(const float* v, int32_t material, float opacity, ae_bvh_node& nd, ae_bvh_triangle t[2]) {
    ae_bvh_node n{};
    for (int k = 0; k < 3; k++) {
        n.leftAABB.min[k] = std::fmin(std::fmin(v[k], v[3 + k]), v[6 + k]);
        n.leftAABB.max[k] = std::fmax(std::fmax(v[k], v[3 + k]), v[6 + k]);
    }
    n.rightAABB = n.leftAABB;
    n.leftPtr = ~0;
    n.rightPtr = ~1;
    bool ok = true;
    for (int k = 0; k < 3; k++)
        for (float c : { n.leftAABB.min[k], n.leftAABB.max[k] }) {
            const float a = std::fabs(c);
            ok = ok && (a == 0.0f || (a >= 9.094947017729282e-13f && a <= 1.099511627776e12f));
        }
    n.padding0 = ok ? 0 : 1;
    nd = n;
    for (int r = 0; r < 2; r++) {
        ae_bvh_triangle& o = t[r];
        o.v0[0] = v[0]; o.v0[1] = v[1]; o.v0[2] = v[2]; o.v0[3] = 1.0f;
        o.v1[0] = v[3]; o.v1[1] = v[4]; o.v1[2] = v[5];
        std::memcpy(&o.v1[3], &material, 4);
        o.v2[0] = v[6]; o.v2[1] = v[7]; o.v2[2] = v[8]; o.v2[3] = opacity;
    }
}

}  // namespace

// Stack entries a traversal of the linear BVH can need: along any
// root-to-leaf path the split bit of the 64-bit keys (30-bit Morton code,
// triangle index) strictly advances, so the tree is at most 64 levels deep.
static uint32_t LbvhDepthBound(uint32_t n_nodes) { return n_nodes > 64u ? 64u : n_nodes; }

extern "C" ae_rt_status ae_rt_mesh_build(ae_rt_ctx* ctx, const float* verts, uint32_t n, const int32_t* material,
                                         const float* opacity, int32_t* mesh_id, uint32_t* order_out, void* stream) {
    if (!ctx || !mesh_id) return AE_RT_INVALID_ARG;
    *mesh_id = -1;
    if (n > 0 && !verts) return Fail(ctx, AE_RT_INVALID_ARG, "null vertex buffer");
    if (n > (1u << 30)) return Fail(ctx, AE_RT_INVALID_ARG, "more than 2^30 triangles");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(ctx->upload_mutex);
    DeviceMesh m;
    if (n == 0) {
        m.depth = LbvhDepthBound(m.n_nodes);
        ctx->meshes.push_back(m);
        *mesh_id = int32_t(ctx->meshes.size() - 1);
        return AE_RT_OK;
    }
    // inputs on the device
    const bool vdev = IsDevicePointer(verts);
    const bool mdev = !material || IsDevicePointer(material);
    const bool odev = !opacity || IsDevicePointer(opacity);
    std::vector<void*> temps;
    auto cleanup = [&]() {
        for (void* p : temps) cudaFree(p);
    };
    auto dalloc = [&](void** p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) temps.push_back(*p);
        return e;
    };
#define BUILD_CUDA(call)                                \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) {                        \
            cleanup();                                  \
            return CudaFail(ctx, e_, #call);            \
        }                                               \
    } while (0)
    if (n == 1) {
        float v[9];
        int32_t mat = 0;
        float op = 1.0f;
        BUILD_CUDA(cudaMemcpy(v, verts, sizeof(v), cudaMemcpyDefault));
        if (material) BUILD_CUDA(cudaMemcpy(&mat, material, 4, cudaMemcpyDefault));
        if (opacity) BUILD_CUDA(cudaMemcpy(&op, opacity, 4, cudaMemcpyDefault));
        ae_bvh_node nd;
        ae_bvh_triangle t[2];
        OneTriangle(v, mat, op, nd, t);
        BUILD_CUDA(cudaMalloc((void**)&m.nodes, sizeof(ae_bvh_node)));
        cudaError_t e = cudaMalloc((void**)&m.tris, 2 * sizeof(ae_bvh_triangle));
        if (e == cudaSuccess) e = cudaMemcpy(m.nodes, &nd, sizeof(nd), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(m.tris, t, sizeof(t), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(m.nodes);
            cudaFree(m.tris);
            return CudaFail(ctx, e, "one-triangle mesh upload");
        }
        m.n_nodes = 1;
        m.n_tris = 2;
        m.depth = LbvhDepthBound(m.n_nodes);
        ctx->meshes.push_back(m);
        *mesh_id = int32_t(ctx->meshes.size() - 1);
        if (order_out) {
            const uint32_t o[2] = { 0, 0 };
            AE_CUDA(ctx, cudaMemcpy(order_out, o, sizeof(o), cudaMemcpyDefault));
        }
        return AE_RT_OK;
    }
    const float* d_verts = verts;
    const int32_t* d_mat = material;
    const float* d_op = opacity;
    if (!vdev) {
        void* p;
        BUILD_CUDA(dalloc(&p, size_t(n) * 36));
        BUILD_CUDA(cudaMemcpyAsync(p, verts, size_t(n) * 36, cudaMemcpyHostToDevice, s));
        d_verts = static_cast<const float*>(p);
    }
    if (!mdev) {
        void* p;
        BUILD_CUDA(dalloc(&p, size_t(n) * 4));
        BUILD_CUDA(cudaMemcpyAsync(p, material, size_t(n) * 4, cudaMemcpyHostToDevice, s));
        d_mat = static_cast<const int32_t*>(p);
    }
    if (!odev) {
        void* p;
        BUILD_CUDA(dalloc(&p, size_t(n) * 4));
        BUILD_CUDA(cudaMemcpyAsync(p, opacity, size_t(n) * 4, cudaMemcpyHostToDevice, s));
        d_op = static_cast<const float*>(p);
    }
    uint32_t* bounds;
    unsigned long long *keys, *sorted;
    int32_t *child, *node_parent, *leaf_parent;
    float *leaf_box, *node_box;
    uint32_t* arrivals;
    BUILD_CUDA(dalloc((void**)&bounds, 8 * sizeof(uint32_t)));
    BUILD_CUDA(dalloc((void**)&keys, size_t(n) * 8));
    BUILD_CUDA(dalloc((void**)&sorted, size_t(n) * 8));
    BUILD_CUDA(dalloc((void**)&child, size_t(n) * 8));
    BUILD_CUDA(dalloc((void**)&node_parent, size_t(n) * 4));
    BUILD_CUDA(dalloc((void**)&leaf_parent, size_t(n) * 4));
    BUILD_CUDA(dalloc((void**)&leaf_box, size_t(n) * 24));
    BUILD_CUDA(dalloc((void**)&node_box, size_t(n) * 24));
    BUILD_CUDA(dalloc((void**)&arrivals, size_t(n) * 4));
    const uint32_t init[8] = { 0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u };   // [6]: error
    BUILD_CUDA(cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, s));
    BUILD_CUDA(cudaMemsetAsync(arrivals, 0, size_t(n) * 4, s));
    BUILD_CUDA(cudaMemsetAsync(node_parent, 0xff, size_t(n) * 4, s));
    const uint32_t blocks = (n + 255) / 256;
    const uint32_t rblocks = blocks < uint32_t(ctx->sm_count) * 8u ? blocks : uint32_t(ctx->sm_count) * 8u;
    centroid_bounds_kernel<<<rblocks, 256, 0, s>>>(d_verts, n, bounds);
    BUILD_CUDA(cudaGetLastError());
    morton_kernel<<<blocks, 256, 0, s>>>(d_verts, n, bounds, keys);
    BUILD_CUDA(cudaGetLastError());
    size_t temp_bytes = 0;
    BUILD_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, temp_bytes, keys, sorted, int(n), 0, 62, s));
    void* temp;
    BUILD_CUDA(dalloc(&temp, temp_bytes));
    BUILD_CUDA(cub::DeviceRadixSort::SortKeys(temp, temp_bytes, keys, sorted, int(n), 0, 62, s));
    karras_kernel<<<(n - 1 + 255) / 256, 256, 0, s>>>(sorted, int(n), child, node_parent, leaf_parent);
    BUILD_CUDA(cudaGetLastError());
    refit_kernel<<<blocks, 256, 0, s>>>(d_verts, sorted, int(n), child, node_parent, leaf_parent, leaf_box, node_box,
                                        arrivals, bounds + 6);
    BUILD_CUDA(cudaGetLastError());
    cudaError_t e = cudaMalloc((void**)&m.nodes, size_t(n - 1) * sizeof(ae_bvh_node));
    if (e == cudaSuccess) e = cudaMalloc((void**)&m.tris, size_t(n) * sizeof(ae_bvh_triangle));
    if (e != cudaSuccess) {
        cudaFree(m.nodes);
        cudaFree(m.tris);
        cleanup();
        return CudaFail(ctx, e, "mesh buffers");
    }
    uint32_t* d_order = nullptr;
    const bool order_dev = order_out && IsDevicePointer(order_out);
    if (order_out) {
        if (order_dev) d_order = order_out;
        else BUILD_CUDA(dalloc((void**)&d_order, size_t(n) * 4));
    }
    emit_kernel<<<blocks, 256, 0, s>>>(d_verts, d_mat, d_op, sorted, int(n), child, node_box, leaf_box,
                                       reinterpret_cast<ae_bvh_node*>(m.nodes),
                                       reinterpret_cast<ae_bvh_triangle*>(m.tris), d_order);
    e = cudaGetLastError();
    if (e == cudaSuccess && order_out && !order_dev)
        e = cudaMemcpyAsync(order_out, d_order, size_t(n) * 4, cudaMemcpyDeviceToHost, s);
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, bounds + 6, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess || err) {
        cudaFree(m.nodes);
        cudaFree(m.tris);
        if (e != cudaSuccess) return CudaFail(ctx, e, "GPU BVH build");
        return Fail(ctx, AE_RT_BAD_BVH, "GPU BVH build produced an invalid hierarchy");
    }
#undef BUILD_CUDA
    m.n_nodes = n - 1;
    m.n_tris = n;
    m.depth = LbvhDepthBound(m.n_nodes);
        ctx->meshes.push_back(m);
    *mesh_id = int32_t(ctx->meshes.size() - 1);
    return AE_RT_OK;
}

extern "C" ae_rt_status ae_rt_mesh_get_bvh(ae_rt_ctx* ctx, int32_t mesh_id, ae_bvh_node* nodes,
                                           ae_bvh_triangle* tris, uint32_t* n_nodes, uint32_t* n_tris) {
    if (!ctx) return AE_RT_INVALID_ARG;
    if (mesh_id < 0 || size_t(mesh_id) >= ctx->meshes.size())
        return Fail(ctx, AE_RT_INVALID_ARG, "unknown mesh id " + std::to_string(mesh_id));
    const DeviceMesh& m = ctx->meshes[size_t(mesh_id)];
    if (n_nodes) *n_nodes = m.n_nodes;
    if (n_tris) *n_tris = m.n_tris;
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    if (nodes && m.n_nodes) AE_CUDA(ctx, cudaMemcpy(nodes, m.nodes, size_t(m.n_nodes) * 64, cudaMemcpyDefault));
    if (tris && m.n_tris) AE_CUDA(ctx, cudaMemcpy(tris, m.tris, size_t(m.n_tris) * 48, cudaMemcpyDefault));
    return AE_RT_OK;
}
