// Device context of the C ABI, shared by the library's translation units.
#pragma once

#include "atlas_rt.h"
#include "trace_kernels.cuh"

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

struct ae_rc;

namespace atlas::rt::host {

struct DeviceMesh {
    float4* nodes = nullptr;
    float4* tris = nullptr;
    float4* shading = nullptr;
    uint32_t n_nodes = 0;
    uint32_t n_tris = 0;
    bool transparent = false;   // a shading triangle's opacity (d2.w) is not 1: opacity texture or partial
    uint32_t depth = 0;         // inner-node levels on the longest root-to-leaf path (stack entries it can need)
};

// Grow-only device scratch buffer.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};


}  // namespace atlas::rt::host

struct ae_rt_ctx {
    int device = 0;
    int sm_count = 0;
    uint32_t blocks_per_sm = 0;         // 0: occupancy of each kernel
    int shape = 0;                      // index into kShapes
    uint32_t threads = 128;
    uint32_t max_steps_cfg = 0;
    uint32_t refill_steps = 0;
    uint32_t refill_below = 0;
    uint32_t leaf_wait = 0;
    bool count_fetches = false;
    bool near_ties = true;            // complete near-tie detection on closest-hit traces
    bool staged_rays = false;
    bool approximate = false;   // AE_RT_CFG_APPROXIMATE
    uint32_t scene_depth = 0;   // top-level depth + the deepest mesh's: stack entries a scene ray can need         // ray tiles through shared memory by bulk copy
    std::vector<atlas::rt::host::DeviceMesh> meshes;
    // two-level scene: TLAS nodes, instances (TLAS order), mesh table snapshot
    float4* d_tlas = nullptr;
    uint32_t n_tlas = 0;
    float4* d_instances = nullptr;
    uint32_t n_instances = 0;
    atlas::rt::dev::MeshDesc* d_mesh_table = nullptr;
    uint32_t n_mesh_table = 0;
    uint32_t scene_steps = 0;
    bool scene_ready = false;
    float4* d_inst_model = nullptr;     // object-to-world rows per instance (shading)
    float* d_materials = nullptr;       // GPUMaterial array
    uint32_t n_materials = 0;
    uint8_t* d_tex_pool = nullptr;      // level 0 of every texture (texture.cuh)
    void* d_tex_desc = nullptr;         // dev::TexDesc per texture
    uint32_t n_textures = 0;
    float4* d_lights = nullptr;         // GPULight array
    uint32_t n_lights = 0;
    float env[3] = { 0.0f, 0.0f, 0.0f };  // constant environment radiance of the path tracer's misses
    // path tracer queues
    atlas::rt::host::Scratch pt_rays[2], pt_pay[2], pt_hits, pt_shadow, pt_shadow_pay, pt_occ;
    atlas::rt::host::Scratch pt_gb;     // real-time G-buffer matrices
    atlas::rt::host::Scratch pt_vis[2]; // shadow visibility of the transparency traversal, per shadow queue
    // a second shadow queue: a bounce's shadow trace runs beside the next bounce's trace
    atlas::rt::host::Scratch pt_shadow2, pt_shadow_pay2, pt_occ2;
    cudaEvent_t pt_events[4] = { nullptr, nullptr, nullptr, nullptr };
    // scratch of the RTAO / reflection / GI / DDGI passes (consumers.cu)
    atlas::rt::host::Scratch pass_rays, pass_key, pass_hits, pass_rad, pass_shadow, pass_shadow_pay, pass_vis,
        pass_counts;
    uint32_t* d_pt_counts = nullptr;    // [0], [1] ray queues, [2], [3] shadow queues
    uint32_t* d_counter = nullptr;     // [1] error word; [0], [2..6] work counters (rotated per launch)
    uint32_t next_work_slot = 0;
    unsigned long long* d_fetch = nullptr;
    atlas::rt::host::Scratch rays_in, results_out, batch_table, retest_count;
    // buffers of ae_rt_cast_pass
    atlas::rt::host::Scratch cast_primary, cast_primary_hits, cast_secondary, cast_secondary_hits, cast_shadow, cast_occluded;
    uint32_t* d_cast_counts = nullptr;
    // result copies of ae_rt_cast_pass overlap the later stages on this stream
    cudaStream_t copy_stream = nullptr;
    cudaStream_t trace_stream = nullptr;  // ae_rt_cast_pass: the shadow trace beside the bounce trace
    cudaEvent_t cast_events[4] = { nullptr, nullptr, nullptr, nullptr };
    uint32_t* h_cast_counts = nullptr;  // pinned, mapped
    uint32_t* d_cast_counts_mapped = nullptr;   // its device address
    uint32_t* h_error = nullptr;        // pinned, mapped: the error word as last published
    uint32_t* d_error_mapped = nullptr;
    std::string last_error;
    std::mutex upload_mutex;
};

namespace atlas::rt::host {

inline ae_rt_status Fail(ae_rt_ctx* ctx, ae_rt_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

inline ae_rt_status CudaFail(ae_rt_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return Fail(ctx, AE_RT_OUT_OF_MEMORY, m);
    return Fail(ctx, AE_RT_CUDA_ERROR, m);
}

#define AE_CUDA(ctx, call)                                         \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return CudaFail((ctx), e_, #call);  \
    } while (0)

// True when the GPU can read `p` directly as device memory.
inline bool IsDevicePointer(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}


// Queue-driven trace over the context's two-level scene (rays, out and count
// in device memory), for the other translation units.
// Closest / any-hit trace of a scene queue for the library's own consumers
// (passes, radiance cache): the near-tie detection is skipped.
ae_rt_status TraceSceneQueue(ae_rt_ctx* ctx, bool any, const ae_packed_ray* rays, uint32_t capacity, float tmin,
                             float tmax, void* out, void* stream, const uint32_t* count_dev, uint32_t cull_mask,
                             bool per_ray_tmax);

// The transparency traversal variants over the scene (transparency.cu); with
// count_dev, `n` is the queue capacity and the count lives on the device;
// with per_ray_tmax, ray i's tmax is its third vector's x.
ae_rt_status TraceTransparency(ae_rt_ctx* ctx, bool any, const ae_packed_ray* rays, uint32_t n, float tmin,
                               float tmax, uint32_t cull_mask, void* out, void* stream,
                               const uint32_t* count_dev = nullptr, bool per_ray_tmax = false);

// The bounce loop's queues for `capacity` rays: two ray/payload queues, the
// hit buffer, two shadow queues (a bounce's shadow trace runs on
// ctx->trace_stream beside the next bounce), their counts and events.
ae_rt_status EnsureBounceQueues(ae_rt_ctx* ctx, uint32_t capacity);

}  // namespace atlas::rt::host
