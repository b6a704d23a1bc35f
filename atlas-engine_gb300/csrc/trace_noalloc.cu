// Closest-hit trace that allocates no device memory (ae_rt_trace_closest_noalloc).
//
// Who needs it: a host that manages every byte of device memory itself and
// forbids a library from calling cudaMalloc -- an engine that draws all GPU
// memory from its own pre-sized arenas at load time, a frame loop under a
// fixed memory budget, or code that must not trigger the implicit device
// synchronisation of cudaMalloc / cudaFree in the middle of a frame.  Such a
// host cannot create an ae_rt_ctx (which owns staging buffers and counters),
// so this entry point takes the BVH, rays and hit buffer as device pointers
// the caller already owns and uses no allocation at all.
//
// The only device memory of its own is the scratch the persistent traversal
// kernel needs: the work counter from which warps pull rays, and the error
// word.  It lives in the file-scope array below, 256 bytes, which every GPU
// that loads this library holds until the process exits.
#include "atlas_rt.h"
#include "trace_kernels.cuh"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kWarps = 4;
// 128 stack entries per lane, as in every other trace entry point: 32 in
// shared memory, the rest in local memory (touched only by deep rays)
constexpr int kStackEntries = 128;
constexpr int kSmemStack = 32;
constexpr int kSpillStack = kStackEntries - kSmemStack;
constexpr int kMinBlocks = 8;
constexpr uint32_t kScratchWords = 64;     // 256 bytes; this call uses words 0 (counter) and 1 (errors)
constexpr uint32_t kWordsUsed = 2;
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device.  Word 0 is zeroed by each call
// before its launch; calls that overlap on the GPU (different streams, no
// ordering between them) race on it and must not be issued.
static __device__ __align__(256) uint32_t g_trace_scratch[kScratchWords];

struct DeviceSetup {
    bool ready = false;
    uint32_t* scratch = nullptr;   // device address of g_trace_scratch on this device
    uint32_t grid = 0;             // persistent grid: SMs x resident CTAs
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

void* NoAllocKernel() {
    return reinterpret_cast<void*>(
        &atlas::rt::dev::trace_kernel<false, false, atlas::rt::dev::MODE_MESH, kWarps, kSmemStack, kSpillStack,
                                       kMinBlocks, true>);
}

// Device (or managed) memory of device `dev`.  A buffer of another GPU is
// refused: without peer access the kernel could not read it.
bool IsDeviceMemory(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Once per device, with that device current: the scratch symbol's device
// address (the host-side name of the array is only a stand-in and must never
// reach a kernel), the SM count and the kernel's occupancy.
ae_rt_status SetupDevice(int dev, DeviceSetup** out) {
    std::lock_guard<std::mutex> g(g_setup_mutex);
    DeviceSetup& s = g_setup[dev];
    if (!s.ready) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_trace_scratch) != cudaSuccess || ptr == nullptr) {
            cudaGetLastError();
            return AE_RT_CUDA_ERROR;
        }
        int sms = 0, blocks = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, NoAllocKernel(), kWarps * 32, 0) != cudaSuccess) {
            cudaGetLastError();
            return AE_RT_CUDA_ERROR;
        }
        s.scratch = static_cast<uint32_t*>(ptr);
        s.grid = uint32_t(sms) * uint32_t(blocks > 0 ? blocks : 1);
        s.ready = true;
    }
    *out = &s;
    return AE_RT_OK;
}

}  // namespace

extern "C" ae_rt_status ae_rt_trace_closest_noalloc(const ae_bvh_node* nodes, uint32_t n_nodes,
                                                    const ae_bvh_triangle* tris, uint32_t n_tris,
                                                    const ae_packed_ray* rays, uint32_t n_rays, float tmin,
                                                    float tmax, ae_hit* hits, void* stream) {
    static_assert(kWordsUsed <= kScratchWords, "scratch too small");
    if (n_rays == 0) return AE_RT_OK;
    if (n_rays > AE_RT_NOALLOC_MAX_RAYS) return AE_RT_INVALID_ARG;   // the 32-bit work counter's range
    if (!rays || !hits || (n_nodes && !nodes) || (n_tris && !tris)) return AE_RT_INVALID_ARG;
    if (n_nodes >= (1u << 31) - 1 || n_tris >= (1u << 31) - 1) return AE_RT_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return AE_RT_CUDA_ERROR;
    }
    if (dev < 0 || dev >= kMaxDevices) return AE_RT_INVALID_ARG;
    if (!IsDeviceMemory(rays, dev) || !IsDeviceMemory(hits, dev) || (n_nodes && !IsDeviceMemory(nodes, dev)) ||
        (n_tris && !IsDeviceMemory(tris, dev)))
        return AE_RT_INVALID_ARG;
    DeviceSetup* s = nullptr;
    ae_rt_status st = SetupDevice(dev, &s);
    if (st != AE_RT_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // the work counter and the error word must start at zero for every call
    if (cudaMemsetAsync(s->scratch, 0, kWordsUsed * sizeof(uint32_t), cs) != cudaSuccess) {
        cudaGetLastError();
        return AE_RT_CUDA_ERROR;
    }
    atlas::rt::dev::TraceParams p{};
    p.nodes = reinterpret_cast<const float4*>(nodes);
    p.tris = reinterpret_cast<const float4*>(tris);
    p.n_nodes = n_nodes;
    p.n_tris = n_tris;
    p.rays = reinterpret_cast<const float4*>(rays);
    p.n_rays = n_rays;
    p.n_rays_dev = nullptr;
    p.tmin = tmin;
    p.tmax = tmax;
    p.hits = reinterpret_cast<float4*>(hits);
    p.occluded = nullptr;
    p.work_counter = s->scratch;
    p.error_word = s->scratch + 1;
    p.fetch_counts = nullptr;
    p.max_steps = atlas::rt::dev::default_step_cap(n_nodes);
    uint32_t grid = s->grid;
    const uint32_t needed = (n_rays + kWarps * 32 - 1) / (kWarps * 32);
    if (needed < grid) grid = needed;
    void* args[] = { &p };
    if (cudaLaunchKernel(NoAllocKernel(), dim3(grid), dim3(kWarps * 32), args, 0, cs) != cudaSuccess) {
        cudaGetLastError();
        return AE_RT_CUDA_ERROR;
    }
    return AE_RT_OK;
}
