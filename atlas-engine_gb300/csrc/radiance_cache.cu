// Radiance cache entry points (include/atlas_rt.h, ae_rc_*): parameters and
// optimizer state in device memory, online training from self-generated
// paths, rendering with paths terminated into the cache.
#include "atlas_rt.h"
#include "context.cuh"
#include "rc_kernels.cuh"
#include "rc_tc_kernels.cuh"

#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

using namespace atlas::rt::host;
using namespace atlas::rt::dev;

struct ae_rc {
    ae_rt_ctx* ctx = nullptr;
    ae_rc_config cfg{};
    RcGrid grid{};                 // host-side description (device pointers inside)
    size_t grid_params = 0;        // levels * T * 2
    float* mlp_master = nullptr;
    float* mlp_m = nullptr;
    float* mlp_v = nullptr;
    float* mlp_grad = nullptr;
    bool grads_zero = false;       // the gradient buffers hold zeros (Adam leaves them so)
    __nv_bfloat16* mlp_bf16 = nullptr;
    float* grid_master = nullptr;
    float* grid_m = nullptr;
    float* grid_v = nullptr;
    float* grid_grad = nullptr;
    __half* grid_f16 = nullptr;
    // what ae_rc_frame's render reads: the cache as trained up to the frame
    // before, while this frame's training updates grid_f16 / mlp_bf16
    __half* grid_snap = nullptr;
    __nv_bfloat16* mlp_snap = nullptr;
    float* d_loss = nullptr;
    uint32_t* d_counts = nullptr;  // [0] training samples, [1] cache queries
    Scratch samples, queries;
    uint64_t step = 0;
    int sm_count = 0;
    float scale = 1.0f;            // radiance scale of the stored values
    uint32_t max_bounces = 3;      // bounce budget of the most recent training frame
    // work that overlaps the render: [0] first-vertex inference, [1] training paths
    cudaStream_t aux[2] = { nullptr, nullptr };
    cudaEvent_t ev[4] = { nullptr, nullptr, nullptr, nullptr };
};

namespace {

constexpr size_t kTrainSmem = RC_WBYTES + (RC_HIDDEN + 1) * RC_ABYTES + 2 * RC_ABYTES;

ae_rt_status RcFail(ae_rc* rc, ae_rt_status s, const std::string& m) { return Fail(rc ? rc->ctx : nullptr, s, m); }

#define RC_CUDA(rc, call)                                                     \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) return CudaFail((rc)->ctx, e_, #call);         \
    } while (0)

RcMlpParams MlpParams(ae_rc* rc) {
    RcMlpParams p{};
    p.grid = rc->grid;
    p.weights = rc->mlp_bf16;
    p.grad_w = rc->mlp_grad;
    p.loss = rc->d_loss;
    p.error_word = rc->ctx->d_counter + 1;
    return p;
}

uint32_t GridBlocks(ae_rc* rc, uint32_t n) {
    const uint32_t tiles = (n + RC_TILE - 1) / RC_TILE;
    uint32_t b = uint32_t(rc->sm_count);
    return tiles < b ? (tiles ? tiles : 1) : b;
}

// Gradients of the relative L2 loss over n training records (device) into
// mlp_grad / grid_grad (zeroed first); loss sum into d_loss.
ae_rt_status Backprop(ae_rc* rc, const float4* recs, uint32_t n, const uint32_t* n_dev, uint32_t slice,
                      uint32_t slices, cudaStream_t s) {
    if (!rc->grads_zero) {
        RC_CUDA(rc, cudaMemsetAsync(rc->mlp_grad, 0, RC_NPARAM * sizeof(float), s));
        RC_CUDA(rc, cudaMemsetAsync(rc->grid_grad, 0, rc->grid_params * sizeof(float), s));
    }
    rc->grads_zero = false;
    RC_CUDA(rc, cudaMemsetAsync(rc->d_loss, 0, sizeof(float), s));
    RcMlpParams p = MlpParams(rc);
    p.recs = recs;
    p.n = n;
    p.n_dev = n_dev;
    p.slice = slice;
    p.slices = slices;
    const uint32_t count = slices ? (n + slices - 1) / slices : n;
    if (rc->cfg.flags & AE_RC_TRAIN_WARP_MMA)
        rc_mlp_kernel<RC_TRAIN><<<GridBlocks(rc, count), RC_THREADS, kTrainSmem, s>>>(p);
    else
        rc_train_tc_kernel<<<GridBlocks(rc, count), RCTT_THREADS, RCTT_SMEM, s>>>(p);
    RC_CUDA(rc, cudaGetLastError());
    return AE_RT_OK;
}

ae_rt_status AdamStep(ae_rc* rc, cudaStream_t s) {
    rc->step++;
    const double b1 = rc->cfg.beta1, b2 = rc->cfg.beta2;
    const float scale = float(std::sqrt(1.0 - std::pow(b2, double(rc->step))) / (1.0 - std::pow(b1, double(rc->step))));
    RcAdamParams a{};
    a.lr = rc->cfg.learning_rate;
    a.beta1 = rc->cfg.beta1;
    a.beta2 = rc->cfg.beta2;
    a.eps = rc->cfg.epsilon;
    a.step_scale = scale;
    a.zero_grad = 1;
    RcAdamParams g = a;
    a.master = rc->mlp_master; a.m = rc->mlp_m; a.v = rc->mlp_v; a.grad = rc->mlp_grad;
    a.out_bf16 = rc->mlp_bf16; a.out_f16 = nullptr; a.n = RC_NPARAM;
    g.master = rc->grid_master; g.m = rc->grid_m; g.v = rc->grid_v; g.grad = rc->grid_grad;
    g.out_bf16 = nullptr; g.out_f16 = rc->grid_f16; g.n = rc->grid_params;
    g.skip_zero = 1;
    const uint32_t mlp_blocks = (RC_NPARAM / 4 + 255) / 256;
    rc_adam_kernel<<<mlp_blocks + uint32_t(rc->sm_count) * 8u, 256, 0, s>>>(a, g, mlp_blocks);
    RC_CUDA(rc, cudaGetLastError());
    rc->grads_zero = true;
    return AE_RT_OK;
}

void Destroy(ae_rc* rc) {
    if (!rc) return;
    cudaSetDevice(rc->ctx->device);
    for (void* p : { (void*)rc->mlp_master, (void*)rc->mlp_m, (void*)rc->mlp_v, (void*)rc->mlp_grad,
                     (void*)rc->mlp_bf16, (void*)rc->grid_master, (void*)rc->grid_m, (void*)rc->grid_v,
                     (void*)rc->grid_grad, (void*)rc->grid_f16, (void*)rc->d_loss, (void*)rc->d_counts,
                     (void*)rc->grid_snap, (void*)rc->mlp_snap })
        cudaFree(p);
    rc->samples.release();
    rc->queries.release();
    for (cudaEvent_t e : rc->ev)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : rc->aux)
        if (st) cudaStreamDestroy(st);
    delete rc;
}

ae_rt_status UploadParams(ae_rc* rc, const float* mlp, const float* grid) {
    RC_CUDA(rc, cudaMemcpy(rc->mlp_master, mlp, RC_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    RC_CUDA(rc, cudaMemcpy(rc->grid_master, grid, rc->grid_params * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<__nv_bfloat16> wb(RC_NPARAM);
    for (int i = 0; i < RC_NPARAM; i++) wb[i] = __float2bfloat16_rn(mlp[i]);
    RC_CUDA(rc, cudaMemcpy(rc->mlp_bf16, wb.data(), RC_NPARAM * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
    std::vector<__half> gh(rc->grid_params);
    for (size_t i = 0; i < rc->grid_params; i++) gh[i] = __float2half_rn(grid[i]);
    RC_CUDA(rc, cudaMemcpy(rc->grid_f16, gh.data(), rc->grid_params * sizeof(__half), cudaMemcpyHostToDevice));
    RC_CUDA(rc, cudaMemset(rc->mlp_m, 0, RC_NPARAM * sizeof(float)));
    RC_CUDA(rc, cudaMemset(rc->mlp_v, 0, RC_NPARAM * sizeof(float)));
    RC_CUDA(rc, cudaMemset(rc->grid_m, 0, rc->grid_params * sizeof(float)));
    RC_CUDA(rc, cudaMemset(rc->grid_v, 0, rc->grid_params * sizeof(float)));
    rc->step = 0;
    return AE_RT_OK;
}

bool DevPtr(const void* p) { return IsDevicePointer(p); }

ae_rt_status EnsureStreams(ae_rc* rc) {
    for (cudaStream_t& st : rc->aux)
        if (!st) RC_CUDA(rc, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (cudaEvent_t& e : rc->ev)
        if (!e) RC_CUDA(rc, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return AE_RT_OK;
}

CameraParams CamParams(const ae_camera* cam) {
    CameraParams c{};
    c.lx = cam->location[0]; c.ly = cam->location[1]; c.lz = cam->location[2];
    c.ox = cam->origin[0]; c.oy = cam->origin[1]; c.oz = cam->origin[2];
    c.rx = cam->right[0]; c.ry = cam->right[1]; c.rz = cam->right[2];
    c.bx = cam->bottom[0]; c.by = cam->bottom[1]; c.bz = cam->bottom[2];
    c.width = cam->width; c.height = cam->height;
    return c;
}

// The self-generated training records of one frame into rc->samples (count
// in d_counts[0]).  Reads the scene only, never the cache.
ae_rt_status GeneratePaths(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t n_paths, uint32_t max_bounces,
                           cudaStream_t s) {
    ae_rt_ctx* ctx = rc->ctx;
    RC_CUDA(rc, rc->samples.ensure(size_t(n_paths) * RC_MAX_DEPTH * 64));
    RC_CUDA(rc, cudaMemsetAsync(rc->d_counts, 0, sizeof(uint32_t), s));
    RcPathParams pp{};
    pp.tp.tlas = ctx->d_tlas;
    pp.tp.n_tlas = ctx->n_tlas;
    pp.tp.instances = ctx->d_instances;
    pp.tp.n_instances = ctx->n_instances;
    pp.tp.meshes = ctx->d_mesh_table;
    pp.tp.n_meshes = ctx->n_mesh_table;
    pp.tp.max_steps = ctx->scene_steps;
    pp.sc.instances = ctx->d_instances;
    pp.sc.inst_model = ctx->d_inst_model;
    pp.sc.meshes = ctx->d_mesh_table;
    pp.sc.materials = ctx->d_materials;
    pp.sc.n_materials = ctx->n_materials;
    pp.sc.lights = ctx->d_lights;
    pp.sc.n_lights = ctx->n_lights;
    pp.sc.tex.pool = ctx->d_tex_pool;
    pp.sc.tex.desc = static_cast<const atlas::rt::dev::TexDesc*>(ctx->d_tex_desc);
    pp.sc.tex.n = ctx->n_textures;
    pp.cam = CamParams(cam);
    pp.n_paths = n_paths;
    pp.frame = frame;
    pp.seed = rc->cfg.seed;
    pp.max_bounces = max_bounces;
    pp.epsilon = 0.1f;
    pp.scale = rc->scale;
    pp.samples = static_cast<float4*>(rc->samples.ptr);
    pp.n_samples = rc->d_counts;
    rc_paths_kernel<<<(n_paths + RC_PATH_THREADS - 1) / RC_PATH_THREADS, RC_PATH_THREADS, 0, s>>>(pp);
    RC_CUDA(rc, cudaGetLastError());
    return AE_RT_OK;
}

// The records in `steps` equal slices (count on the device), one Adam step each.
ae_rt_status TrainSteps(ae_rc* rc, uint32_t n_paths, uint32_t steps, float* loss_out, cudaStream_t s) {
    for (uint32_t k = 0; k < steps; k++) {
        ae_rt_status st = Backprop(rc, static_cast<const float4*>(rc->samples.ptr), n_paths * RC_MAX_DEPTH,
                                   rc->d_counts, k, steps, s);
        if (st != AE_RT_OK) return st;
        st = AdamStep(rc, s);
        if (st != AE_RT_OK) return st;
    }
    if (loss_out) {
        float l = 0.0f;
        RC_CUDA(rc, cudaMemcpyAsync(&l, rc->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        RC_CUDA(rc, cudaStreamSynchronize(s));
        *loss_out = l;
    }
    return AE_RT_OK;
}

ae_rt_status CheckTrainArgs(ae_rc* rc, const ae_camera* cam, uint32_t n_paths, uint32_t steps, uint32_t max_bounces) {
    ae_rt_ctx* ctx = rc->ctx;
    if (!cam) return AE_RT_INVALID_ARG;
    if (!ctx->scene_ready || !ctx->d_materials) return RcFail(rc, AE_RT_INVALID_ARG, "no scene / materials set");
    if (ctx->env[0] + ctx->env[1] + ctx->env[2] > 0.0f)
        return RcFail(rc, AE_RT_INVALID_ARG, "the radiance cache models no environment; set it black");
    for (const auto& m : ctx->meshes)
        if (m.transparent) return RcFail(rc, AE_RT_INVALID_ARG, "the radiance cache traces opaque scenes only");
    if (n_paths == 0 || steps == 0 || n_paths < steps) return RcFail(rc, AE_RT_INVALID_ARG, "bad training sizes");
    if (max_bounces == 0 || max_bounces > 16) return RcFail(rc, AE_RT_INVALID_ARG, "max_bounces out of range");
    return AE_RT_OK;
}

// One sample per pixel with paths ending in the cache (see ae_rc_render).
// The cache queries of the first vertex are answered on rc->aux[0] while the
// later bounces (glossy continuations, a few percent of the pixels, whose
// time is set by their longest rays) are traced on `s`: the two write
// disjoint pixels of accum (a path that ends in a query at the first vertex
// adds nothing later).  Joined before returning.
ae_rt_status RenderFrame(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t last_bounce, float* accum,
                         cudaStream_t s, bool from_snapshot = false) {
    ae_rt_ctx* ctx = rc->ctx;
    const uint32_t n = cam->width * cam->height;
    if (n > kPixelMask + 1u) return RcFail(rc, AE_RT_INVALID_ARG, "more than 2^24 pixels");
    // queues hold twice the pixels: split glossy paths add rays
    const uint32_t cap = 2u * n;
    ae_rt_status st = EnsureBounceQueues(ctx, cap);
    if (st != AE_RT_OK) return st;
    RC_CUDA(rc, rc->queries.ensure(size_t(cap) * 64));
    st = EnsureStreams(rc);
    if (st != AE_RT_OK) return st;
    void* stream = s;

    const CameraParams c = CamParams(cam);
    RcShadeParams rp{};
    PtParams& p = rp.pt;
    p.sc.instances = ctx->d_instances;
    p.sc.inst_model = ctx->d_inst_model;
    p.sc.meshes = ctx->d_mesh_table;
    p.sc.materials = ctx->d_materials;
    p.sc.n_materials = ctx->n_materials;
    p.sc.lights = ctx->d_lights;
    p.sc.n_lights = ctx->n_lights;
    p.sc.tex.pool = ctx->d_tex_pool;
    p.sc.tex.desc = static_cast<const atlas::rt::dev::TexDesc*>(ctx->d_tex_desc);
    p.sc.tex.n = ctx->n_textures;
    p.width = cam->width;
    p.height = cam->height;
    p.tile_w = cam->width;    // primary rays over the whole image
    p.tile_h = cam->height;
    p.max_bounces = rc->max_bounces;
    p.epsilon = 0.1f;
    p.seed = rc->cfg.seed + 17u;
    p.sample = frame;
    p.hits_in = static_cast<const float4*>(ctx->pt_hits.ptr);
    p.accum = reinterpret_cast<float4*>(accum);
    p.atomic_accum = 1;
    p.capacity = cap;
    p.overflow = ctx->d_counter + 1;
    rp.queries = static_cast<float4*>(rc->queries.ptr);
    rp.n_queries = rc->d_counts + 1;
    rp.query_capacity = cap;
    rp.last_bounce = last_bounce;
    rp.inv_scale = 1.0f / rc->scale;
    rp.rough_cut = rc->cfg.rough_cut > 0.0f ? rc->cfg.rough_cut : 0.35f;
    rp.split = rc->cfg.glossy_split == 0 ? 4u : (rc->cfg.glossy_split > RC_MAX_SPLIT ? RC_MAX_SPLIT : rc->cfg.glossy_split);
    const uint32_t blocks = (cap + 255) / 256;
    RC_CUDA(rc, cudaMemsetAsync(rc->d_counts + 1, 0, sizeof(uint32_t), s));
    p.rays_out = static_cast<float4*>(ctx->pt_rays[0].ptr);
    p.pay_out = static_cast<float4*>(ctx->pt_pay[0].ptr);
    p.n_out = ctx->d_pt_counts + 0;
    pt_raygen_kernel<<<blocks, 256, 0, s>>>(c, p);
    RC_CUDA(rc, cudaGetLastError());
    RcMlpParams mp = MlpParams(rc);
    if (from_snapshot) {
        mp.grid.table = reinterpret_cast<const __half2*>(rc->grid_snap);
        mp.weights = rc->mlp_snap;
    }
    mp.recs = static_cast<const float4*>(rc->queries.ptr);
    mp.n = cap;
    mp.accum = reinterpret_cast<float4*>(accum);
    cudaStream_t a0 = rc->aux[0];
    // A vertex's shadow trace and resolve run on ctx->trace_stream beside the
    // next vertex's trace and shading, with the shadow queues alternating
    // (every write into accum here is atomic).
    Scratch* shadowRays[2] = { &ctx->pt_shadow, &ctx->pt_shadow2 };
    Scratch* shadowPay[2] = { &ctx->pt_shadow_pay, &ctx->pt_shadow_pay2 };
    Scratch* shadowOcc[2] = { &ctx->pt_occ, &ctx->pt_occ2 };
    cudaStream_t side = ctx->trace_stream;
    void* sideStream = side;
    bool pending[2] = { false, false };
    const uint32_t final_bounce = last_bounce < rc->max_bounces ? last_bounce : rc->max_bounces;
    for (uint32_t b = 0; b <= final_bounce; b++) {
        const int in = int(b & 1), out = 1 - in, q = int(b & 1);
        p.bounce = b;
        p.rays_in = static_cast<const float4*>(ctx->pt_rays[in].ptr);
        p.pay_in = static_cast<const float4*>(ctx->pt_pay[in].ptr);
        p.n_in = ctx->d_pt_counts + in;
        p.rays_out = static_cast<float4*>(ctx->pt_rays[out].ptr);
        p.pay_out = static_cast<float4*>(ctx->pt_pay[out].ptr);
        p.n_out = ctx->d_pt_counts + out;
        p.shadow_rays = static_cast<float4*>(shadowRays[q]->ptr);
        p.shadow_pay = static_cast<float4*>(shadowPay[q]->ptr);
        p.n_shadow = ctx->d_pt_counts + 2 + q;
        p.shadow_occ = static_cast<const uint8_t*>(shadowOcc[q]->ptr);
        st = TraceSceneQueue(ctx, false, static_cast<const ae_packed_ray*>(ctx->pt_rays[in].ptr), cap, 0.0f, 1e12f,
                             ctx->pt_hits.ptr, stream, ctx->d_pt_counts + in, AE_RT_MASK_ALL, false);
        if (st != AE_RT_OK) return st;
        if (pending[q]) RC_CUDA(rc, cudaStreamWaitEvent(s, ctx->pt_events[2 + q], 0));
        RC_CUDA(rc, cudaMemsetAsync(ctx->d_pt_counts + out, 0, sizeof(uint32_t), s));
        RC_CUDA(rc, cudaMemsetAsync(p.n_shadow, 0, sizeof(uint32_t), s));
        rc_shade_kernel<<<blocks, 256, 0, s>>>(rp);
        RC_CUDA(rc, cudaGetLastError());
        RC_CUDA(rc, cudaEventRecord(ctx->pt_events[q], s));
        RC_CUDA(rc, cudaStreamWaitEvent(side, ctx->pt_events[q], 0));
        st = TraceSceneQueue(ctx, true, static_cast<const ae_packed_ray*>(shadowRays[q]->ptr), cap, 0.0f, 1e12f,
                             shadowOcc[q]->ptr, sideStream, p.n_shadow, AE_RT_MASK_SHADOW, true);
        if (st != AE_RT_OK) return st;
        pt_resolve_kernel<<<blocks, 256, 0, side>>>(p);
        RC_CUDA(rc, cudaGetLastError());
        RC_CUDA(rc, cudaEventRecord(ctx->pt_events[2 + q], side));
        pending[q] = true;
        if (b == 0) {
            // the first vertex's queries (all appended by this vertex's
            // shading), answered on another side stream
            RC_CUDA(rc, cudaMemcpyAsync(rc->d_counts + 2, rc->d_counts + 1, sizeof(uint32_t),
                                        cudaMemcpyDeviceToDevice, s));
            RC_CUDA(rc, cudaEventRecord(rc->ev[0], s));
            RC_CUDA(rc, cudaStreamWaitEvent(a0, rc->ev[0], 0));
            RcMlpParams m0 = mp;
            m0.n_dev = rc->d_counts + 2;
            rc_infer_tc_kernel<RC_INFER><<<GridBlocks(rc, cap) * 3, RCT_THREADS, RCT_SMEM, a0>>>(m0);
            RC_CUDA(rc, cudaGetLastError());
            RC_CUDA(rc, cudaEventRecord(rc->ev[1], a0));
        }
    }
    // the queries of the later vertices (after the first vertex's ones)
    RcMlpParams m1 = mp;
    m1.n_dev = rc->d_counts + 1;
    m1.offset_dev = rc->d_counts + 2;
    rc_infer_tc_kernel<RC_INFER><<<GridBlocks(rc, cap) * 3, RCT_THREADS, RCT_SMEM, s>>>(m1);
    RC_CUDA(rc, cudaGetLastError());
    RC_CUDA(rc, cudaStreamWaitEvent(s, rc->ev[1], 0));
    for (int q = 0; q < 2; q++)
        if (pending[q]) RC_CUDA(rc, cudaStreamWaitEvent(s, ctx->pt_events[2 + q], 0));
    return AE_RT_OK;
}

}  // namespace

extern "C" {

ae_rt_status ae_rc_create(ae_rt_ctx* ctx, const ae_rc_config* cfg, ae_rc** out) {
    if (!ctx || !cfg || !out) return AE_RT_INVALID_ARG;
    *out = nullptr;
    if (cfg->log2_table < 10 || cfg->log2_table > 24 || cfg->base_resolution < 2 ||
        cfg->max_resolution < cfg->base_resolution || cfg->max_resolution > (1u << 20))
        return Fail(ctx, AE_RT_INVALID_ARG, "radiance cache: encoding parameters out of range");
    if (!(cfg->radiance_scale >= 0.0f) || !std::isfinite(cfg->radiance_scale))
        return Fail(ctx, AE_RT_INVALID_ARG, "radiance cache: bad radiance scale");
    for (int a = 0; a < 3; a++)
        if (!(cfg->aabb_max[a] > cfg->aabb_min[a])) return Fail(ctx, AE_RT_INVALID_ARG, "radiance cache: empty domain");
    AE_CUDA(ctx, cudaSetDevice(ctx->device));
    ae_rc* rc = new (std::nothrow) ae_rc;
    if (!rc) return AE_RT_OUT_OF_MEMORY;
    rc->ctx = ctx;
    rc->cfg = *cfg;
    rc->sm_count = ctx->sm_count;
    rc->scale = cfg->radiance_scale > 0.0f ? cfg->radiance_scale : 1.0f;
    RcGrid& g = rc->grid;
    g.T = 1u << cfg->log2_table;
    g.lox = cfg->aabb_min[0]; g.loy = cfg->aabb_min[1]; g.loz = cfg->aabb_min[2];
    g.sx = 1.0f / (cfg->aabb_max[0] - cfg->aabb_min[0]);
    g.sy = 1.0f / (cfg->aabb_max[1] - cfg->aabb_min[1]);
    g.sz = 1.0f / (cfg->aabb_max[2] - cfg->aabb_min[2]);
    // geometric progression of resolutions from the base to the finest level
    const double b = std::exp((std::log(double(cfg->max_resolution)) - std::log(double(cfg->base_resolution))) /
                              double(RC_LEVELS - 1));
    for (int l = 0; l < RC_LEVELS; l++) {
        const double r = std::floor(double(cfg->base_resolution) * std::pow(b, double(l)) + 1e-6);
        g.res[l] = float(r);
        const double st = r + 1.0;
        g.dense[l] = st * st * st <= double(g.T) ? uint32_t(st) : 0u;
    }
    rc->grid_params = size_t(RC_LEVELS) * g.T * 2;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void**)&rc->mlp_master, RC_NPARAM * sizeof(float));
    alloc((void**)&rc->mlp_m, RC_NPARAM * sizeof(float));
    alloc((void**)&rc->mlp_v, RC_NPARAM * sizeof(float));
    alloc((void**)&rc->mlp_grad, RC_NPARAM * sizeof(float));
    alloc((void**)&rc->mlp_bf16, RC_NPARAM * sizeof(__nv_bfloat16));
    alloc((void**)&rc->grid_master, rc->grid_params * sizeof(float));
    alloc((void**)&rc->grid_m, rc->grid_params * sizeof(float));
    alloc((void**)&rc->grid_v, rc->grid_params * sizeof(float));
    alloc((void**)&rc->grid_grad, rc->grid_params * sizeof(float));
    alloc((void**)&rc->grid_f16, rc->grid_params * sizeof(__half));
    alloc((void**)&rc->d_loss, sizeof(float));
    alloc((void**)&rc->d_counts, 4 * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rc_mlp_kernel<RC_TRAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmem));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rc_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(RCTT_SMEM));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rc_infer_tc_kernel<RC_INFER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(RCT_SMEM));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rc_infer_tc_kernel<RC_PREDICT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(RCT_SMEM));
    if (e != cudaSuccess) {
        Destroy(rc);
        return CudaFail(ctx, e, "radiance cache allocation");
    }
    g.table = reinterpret_cast<const __half2*>(rc->grid_f16);
    g.grad = reinterpret_cast<float2*>(rc->grid_grad);
    // initial parameters: Glorot-uniform weights (output rows beyond RGB zero),
    // grid features uniform in +-1e-4
    std::mt19937 gen(cfg->seed);
    std::vector<float> w(RC_NPARAM, 0.0f);
    const float lim = std::sqrt(6.0f / float(RC_W + RC_W));
    std::uniform_real_distribution<float> uw(-lim, lim);
    for (int i = 0; i < RC_HIDDEN * RC_W * RC_W; i++) w[i] = uw(gen);
    const float limo = std::sqrt(6.0f / float(RC_W + 3));
    std::uniform_real_distribution<float> uo(-limo, limo);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < RC_W; c++) w[RC_HIDDEN * RC_W * RC_W + r * RC_W + c] = uo(gen);
    std::vector<float> gp(rc->grid_params);
    std::uniform_real_distribution<float> ug(-1e-4f, 1e-4f);
    for (auto& x : gp) x = ug(gen);
    ae_rt_status st = UploadParams(rc, w.data(), gp.data());
    if (st != AE_RT_OK) {
        Destroy(rc);
        return st;
    }
    *out = rc;
    return AE_RT_OK;
}

void ae_rc_destroy(ae_rc* rc) { Destroy(rc); }

ae_rt_status ae_rc_param_counts(const ae_rc* rc, uint32_t* n_mlp, uint64_t* n_grid) {
    if (!rc) return AE_RT_INVALID_ARG;
    if (n_mlp) *n_mlp = RC_NPARAM;
    if (n_grid) *n_grid = rc->grid_params;
    return AE_RT_OK;
}

ae_rt_status ae_rc_get_params(ae_rc* rc, float* mlp, float* grid) {
    if (!rc) return AE_RT_INVALID_ARG;
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    RC_CUDA(rc, cudaDeviceSynchronize());
    if (mlp) RC_CUDA(rc, cudaMemcpy(mlp, rc->mlp_master, RC_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    if (grid) RC_CUDA(rc, cudaMemcpy(grid, rc->grid_master, rc->grid_params * sizeof(float), cudaMemcpyDeviceToHost));
    return AE_RT_OK;
}

ae_rt_status ae_rc_set_params(ae_rc* rc, const float* mlp, const float* grid) {
    if (!rc || !mlp || !grid) return AE_RT_INVALID_ARG;
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    RC_CUDA(rc, cudaDeviceSynchronize());
    return UploadParams(rc, mlp, grid);
}

ae_rt_status ae_rc_predict(ae_rc* rc, const float* queries, uint32_t n, float* out, void* stream) {
    if (!rc) return AE_RT_INVALID_ARG;
    if (n == 0) return AE_RT_OK;
    if (!DevPtr(queries) || !DevPtr(out)) return RcFail(rc, AE_RT_INVALID_ARG, "ae_rc_predict takes device buffers");
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    RcMlpParams p = MlpParams(rc);
    p.recs = reinterpret_cast<const float4*>(queries);
    p.n = n;
    p.out = reinterpret_cast<float4*>(out);
    rc_infer_tc_kernel<RC_PREDICT><<<GridBlocks(rc, n) * 3, RCT_THREADS, RCT_SMEM, static_cast<cudaStream_t>(stream)>>>(p);
    RC_CUDA(rc, cudaGetLastError());
    return AE_RT_OK;
}

ae_rt_status ae_rc_selftest_wait_timeout(ae_rc* rc, uint32_t* timed_out) {
    if (!rc || !timed_out) return AE_RT_INVALID_ARG;
    *timed_out = 0;
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    ae_rt_status st = ae_rt_synchronize(rc->ctx, nullptr);   // start from a clean error word
    if (st != AE_RT_OK) return st;
    RC_CUDA(rc, rc->queries.ensure(size_t(RCT_THREADS) * 64));
    RC_CUDA(rc, cudaMemset(rc->queries.ptr, 0, size_t(RCT_THREADS) * 64));
    float4* out = nullptr;
    RC_CUDA(rc, cudaMalloc(&out, size_t(RCT_THREADS) * sizeof(float4)));
    RcMlpParams p = MlpParams(rc);
    p.recs = static_cast<const float4*>(rc->queries.ptr);
    p.n = RCT_THREADS;
    p.out = out;
    p.skip_mma = 1;
    rc_infer_tc_kernel<RC_PREDICT><<<1, RCT_THREADS, RCT_SMEM>>>(p);
    cudaError_t e = cudaGetLastError();
    st = e == cudaSuccess ? ae_rt_synchronize(rc->ctx, nullptr) : CudaFail(rc->ctx, e, "self-test launch");
    cudaFree(out);
    if (st == AE_RT_TIMEOUT) {
        *timed_out = 1;
        return AE_RT_OK;
    }
    return st;
}

ae_rt_status ae_rc_gradients(ae_rc* rc, const float* samples, uint32_t n, float* grad_mlp, float* grad_grid,
                             float* loss_out, void* stream) {
    if (!rc) return AE_RT_INVALID_ARG;
    if (n == 0 || !DevPtr(samples)) return RcFail(rc, AE_RT_INVALID_ARG, "ae_rc_gradients takes device samples");
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ae_rt_status st = Backprop(rc, reinterpret_cast<const float4*>(samples), n, nullptr, 0, 0, s);
    if (st != AE_RT_OK) return st;
    if (grad_mlp) RC_CUDA(rc, cudaMemcpyAsync(grad_mlp, rc->mlp_grad, RC_NPARAM * sizeof(float), cudaMemcpyDefault, s));
    if (grad_grid)
        RC_CUDA(rc, cudaMemcpyAsync(grad_grid, rc->grid_grad, rc->grid_params * sizeof(float), cudaMemcpyDefault, s));
    if (loss_out) {
        float l = 0.0f;
        RC_CUDA(rc, cudaMemcpyAsync(&l, rc->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        RC_CUDA(rc, cudaStreamSynchronize(s));
        *loss_out = l;
    }
    return AE_RT_OK;
}

ae_rt_status ae_rc_train_batch(ae_rc* rc, const float* samples, uint32_t n, float* loss_out, void* stream) {
    if (!rc) return AE_RT_INVALID_ARG;
    if (n == 0 || !DevPtr(samples)) return RcFail(rc, AE_RT_INVALID_ARG, "ae_rc_train_batch takes device samples");
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ae_rt_status st = Backprop(rc, reinterpret_cast<const float4*>(samples), n, nullptr, 0, 0, s);
    if (st != AE_RT_OK) return st;
    st = AdamStep(rc, s);
    if (st != AE_RT_OK) return st;
    if (loss_out) {
        float l = 0.0f;
        RC_CUDA(rc, cudaMemcpyAsync(&l, rc->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        RC_CUDA(rc, cudaStreamSynchronize(s));
        *loss_out = l;
    }
    return AE_RT_OK;
}

ae_rt_status ae_rc_train_frame(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t n_paths, uint32_t steps,
                               uint32_t max_bounces, float* loss_out, void* stream) {
    if (!rc) return AE_RT_INVALID_ARG;
    ae_rt_status st = CheckTrainArgs(rc, cam, n_paths, steps, max_bounces);
    if (st != AE_RT_OK) return st;
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = GeneratePaths(rc, cam, frame, n_paths, max_bounces, s);
    if (st != AE_RT_OK) return st;
    rc->max_bounces = max_bounces;
    return TrainSteps(rc, n_paths, steps, loss_out, s);
}

ae_rt_status ae_rc_render(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t last_bounce, float* accum,
                          void* stream) {
    if (!rc || !cam || !accum) return AE_RT_INVALID_ARG;
    ae_rt_ctx* ctx = rc->ctx;
    if (!ctx->scene_ready || !ctx->d_materials) return RcFail(rc, AE_RT_INVALID_ARG, "no scene / materials set");
    if (ctx->env[0] + ctx->env[1] + ctx->env[2] > 0.0f)
        return RcFail(rc, AE_RT_INVALID_ARG, "the radiance cache models no environment; set it black");
    for (const auto& m : ctx->meshes)
        if (m.transparent) return RcFail(rc, AE_RT_INVALID_ARG, "the radiance cache traces opaque scenes only");
    if (!DevPtr(accum)) return RcFail(rc, AE_RT_INVALID_ARG, "accumulation buffer must be device memory");
    RC_CUDA(rc, cudaSetDevice(ctx->device));
    return RenderFrame(rc, cam, frame, last_bounce, accum, static_cast<cudaStream_t>(stream));
}

ae_rt_status ae_rc_frame(ae_rc* rc, const ae_camera* cam, uint32_t frame, uint32_t n_paths, uint32_t steps,
                         uint32_t max_bounces, uint32_t last_bounce, float* accum, float* loss_out, void* stream) {
    if (!rc || !accum) return AE_RT_INVALID_ARG;
    ae_rt_status st = CheckTrainArgs(rc, cam, n_paths, steps, max_bounces);
    if (st != AE_RT_OK) return st;
    if (!DevPtr(accum)) return RcFail(rc, AE_RT_INVALID_ARG, "accumulation buffer must be device memory");
    RC_CUDA(rc, cudaSetDevice(rc->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = EnsureStreams(rc);
    if (st != AE_RT_OK) return st;
    // The render reads a snapshot of the cache as trained up to the previous
    // frame (the FP16 grid and BF16 weights, ~34 MB, copied on the device),
    // so that this frame's training -- its paths (scene only) and its Adam
    // steps -- runs beside the render on the side stream.
    if (!rc->grid_snap) {
        RC_CUDA(rc, cudaMalloc(&rc->grid_snap, rc->grid_params * sizeof(__half)));
        RC_CUDA(rc, cudaMalloc(&rc->mlp_snap, RC_NPARAM * sizeof(__nv_bfloat16)));
    }
    RC_CUDA(rc, cudaMemcpyAsync(rc->grid_snap, rc->grid_f16, rc->grid_params * sizeof(__half),
                                cudaMemcpyDeviceToDevice, s));
    RC_CUDA(rc, cudaMemcpyAsync(rc->mlp_snap, rc->mlp_bf16, RC_NPARAM * sizeof(__nv_bfloat16),
                                cudaMemcpyDeviceToDevice, s));
    cudaStream_t a1 = rc->aux[1];
    RC_CUDA(rc, cudaEventRecord(rc->ev[2], s));
    RC_CUDA(rc, cudaStreamWaitEvent(a1, rc->ev[2], 0));
    st = GeneratePaths(rc, cam, frame, n_paths, max_bounces, a1);
    if (st != AE_RT_OK) return st;
    st = TrainSteps(rc, n_paths, steps, nullptr, a1);
    if (st != AE_RT_OK) return st;
    RC_CUDA(rc, cudaEventRecord(rc->ev[3], a1));
    rc->max_bounces = max_bounces;
    st = RenderFrame(rc, cam, frame, last_bounce, accum, s, true);
    if (st != AE_RT_OK) return st;
    RC_CUDA(rc, cudaStreamWaitEvent(s, rc->ev[3], 0));
    if (loss_out) {
        float l = 0.0f;
        RC_CUDA(rc, cudaMemcpyAsync(&l, rc->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        RC_CUDA(rc, cudaStreamSynchronize(s));
        *loss_out = l;
    }
    return AE_RT_OK;
}

}  // extern "C"
