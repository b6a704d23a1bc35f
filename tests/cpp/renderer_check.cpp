// The engine's path from assets to a path-traced image, written the way an
// engine-side caller would write it against include/atlas_rt.h and
// include/atlas_rt.hpp, for tests/test_cpp_wrapper.py:
//
//   .aemesh + .aematerial  -> ae_mesh_asset_* / ae_material_asset_*
//   GPUMaterial table      -> ae_material_asset_to_gpu        (RayTracingWorld::UpdateMaterials)
//   triangles, BVH, packing-> ae_mesh_asset_triangles, ae_bvh_* (MeshData::BuildBVH)
//   scene                  -> ae_rt_mesh_upload, ae_rt_scene_build
//   light list             -> ae_lights_from_mesh / _instance / _normalize / _select
//   rendering              -> atlas::rt::PathTracingRenderer
//
// Checks, each against the direct C ABI call on the same inputs:
//   * 2 x 2 image subdivisions for 8 samples: the accumulation equals one
//     whole-image call of 8 samples bit for bit, the output image equals its
//     tonemap, and the sample count reads 8;
//   * a camera move restarts the count, and one full pass equals a 1-sample
//     whole-image call with the new camera;
//   * 3 x 3 subdivisions of a size that does not divide leave the remainder
//     pixels untraced, as the engine does;
//   * the real-time mode equals ae_rt_pathtrace_realtime with the frame's
//     sample streams.
// Usage: renderer_check <assets dir>; prints "ok" lines, exits non-zero on a
// mismatch or an error.
#include "atlas_rt.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace atlas::rt;

namespace {

void Ok(ae_rt_status st, const char* what) {
    if (st != AE_RT_OK)
        throw Error(st, std::string(what) + " failed: " + ae_asset_last_error());
}

void Cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
struct DeviceBuffer {
    T* ptr = nullptr;
    size_t n = 0;
    explicit DeviceBuffer(size_t count) : n(count) {
        Cuda(cudaMalloc(&ptr, n * sizeof(T)), "cudaMalloc");
        Cuda(cudaMemset(ptr, 0, n * sizeof(T)), "cudaMemset");
    }
    ~DeviceBuffer() { cudaFree(ptr); }
    std::vector<T> Host() const {
        std::vector<T> h(n);
        Cuda(cudaMemcpy(h.data(), ptr, n * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return h;
    }
};

ae_camera LookAt(const float eye[3], const float target[3], uint32_t w, uint32_t h, float fov_deg) {
    float f[3] = { target[0] - eye[0], target[1] - eye[1], target[2] - eye[2] };
    float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (float& c : f) c /= fl;
    float r[3] = { -f[2], 0.0f, f[0] };           // cross(f, up (0, 1, 0))
    float rl = std::sqrt(r[0] * r[0] + r[2] * r[2]);
    for (float& c : r) c /= rl;
    const float u[3] = { r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0] };
    const float hh = std::tan(fov_deg * 3.14159265f / 360.0f), hw = hh * float(w) / float(h);
    ae_camera c;
    std::memset(&c, 0, sizeof(c));
    for (int k = 0; k < 3; k++) {
        c.location[k] = eye[k];
        c.origin[k] = eye[k] + f[k] - r[k] * hw + u[k] * hh;
        c.right[k] = r[k] * 2.0f * hw;
        c.bottom[k] = -u[k] * 2.0f * hh;
    }
    c.width = w;
    c.height = h;
    c.jitter[0] = c.jitter[1] = 0.5f;
    return c;
}

template <class T>
bool Same(const std::vector<T>& a, const std::vector<T>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0;
}

int Run(const std::string& dir) {
    // assets
    ae_mesh_asset* mesh = nullptr;
    Ok(ae_mesh_asset_load_file((dir + "/meshes/two_part.aemesh").c_str(), &mesh), "mesh");
    ae_mesh_asset_info info;
    Ok(ae_mesh_asset_get_info(mesh, &info), "info");
    std::vector<ae_material> table(info.material_count);
    std::vector<float> emissive(size_t(info.material_count) * 3), intensity(info.material_count);
    for (uint32_t m = 0; m < info.material_count; m++) {
        ae_material_asset* mat = nullptr;
        Ok(ae_material_asset_load_file((dir + "/" + ae_mesh_asset_material_path(mesh, m)).c_str(), &mat), "material");
        Ok(ae_material_asset_to_gpu(mat, mesh, nullptr, int32_t(m), &table[m]), "to_gpu");
        Ok(ae_material_asset_get_emissive(mat, &emissive[m * 3], &intensity[m]), "emissive");
        ae_material_asset_destroy(mat);
    }
    const uint32_t n = info.triangle_count;
    std::vector<float> verts(size_t(n) * 9), normals(size_t(n) * 9), uvs(size_t(n) * 6), colors(size_t(n) * 12),
        opacity(n);
    std::vector<int32_t> material(n);
    Ok(ae_mesh_asset_triangles(mesh, table.data(), uint32_t(table.size()), verts.data(), normals.data(), uvs.data(),
                               colors.data(), material.data(), opacity.data()),
       "triangles");
    ae_bvh* bvh = nullptr;
    Ok(ae_bvh_build_triangles(verts.data(), nullptr, n, 1, &bvh), "build");
    const uint32_t nn = ae_bvh_node_count(bvh), np = ae_bvh_primitive_count(bvh);
    std::vector<ae_bvh_node> nodes(nn);
    std::vector<ae_bvh_triangle> gtris(np);
    std::vector<ae_triangle> shading(np);
    Ok(ae_bvh_get_nodes(bvh, nodes.data()), "nodes");
    Ok(ae_bvh_pack_triangles(bvh, verts.data(), material.data(), opacity.data(), gtris.data()), "pack");
    Ok(ae_bvh_pack_shading(bvh, verts.data(), normals.data(), material.data(), opacity.data(), shading.data()),
       "shading");
    Ok(ae_bvh_pack_attributes(bvh, verts.data(), normals.data(), uvs.data(), colors.data(), shading.data()),
       "attributes");

    // scene
    Context ctx(0);
    int32_t mesh_id = -1;
    ctx.Check(ae_rt_mesh_upload(ctx.get(), nodes.data(), nn, gtris.data(), shading.data(), np, &mesh_id), "upload");
    ae_bvh_instance inst;
    std::memset(&inst, 0, sizeof(inst));
    inst.inverseMatrix[0] = inst.inverseMatrix[5] = inst.inverseMatrix[10] = 1.0f;
    inst.meshOffset = mesh_id;
    inst.mask = AE_RT_MASK_ALL | AE_RT_MASK_SHADOW;
    ae_aabb box;
    for (int c = 0; c < 3; c++) {
        box.min[c] = 1e30f;
        box.max[c] = -1e30f;
    }
    for (uint32_t k = 0; k < n * 3; k++)
        for (int c = 0; c < 3; c++) {
            box.min[c] = std::fmin(box.min[c], verts[k * 3 + c]);
            box.max[c] = std::fmax(box.max[c], verts[k * 3 + c]);
        }
    uint32_t order[2], n_ordered = 0;
    ctx.Check(ae_rt_scene_build(ctx.get(), &inst, &box, 1, order, &n_ordered), "scene");
    ctx.Check(ae_rt_scene_set_materials(ctx.get(), table.data(), uint32_t(table.size())), "materials");

    // light list: the emissive triangles, placed by the instance, weighted, selected
    uint32_t nl = 0;
    Ok(ae_lights_from_mesh(shading.data(), np, emissive.data(), intensity.data(), uint32_t(table.size()), nullptr, 0,
                           &nl),
       "count lights");
    if (nl == 0) throw std::runtime_error("the fixture has no emissive triangles");
    std::vector<ae_light> mesh_lights(nl), lights(nl), selected(nl);
    Ok(ae_lights_from_mesh(shading.data(), np, emissive.data(), intensity.data(), uint32_t(table.size()),
                           mesh_lights.data(), nl, &nl),
       "lights");
    const float identity[16] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 };
    Ok(ae_lights_instance(mesh_lights.data(), nl, identity, 0, lights.data()), "instance lights");
    Ok(ae_lights_normalize(lights.data(), nl), "normalize");
    uint32_t ns = 0;
    Ok(ae_lights_select(lights.data(), nl, 128, nullptr, selected.data(), &ns), "select");
    ctx.Check(ae_rt_scene_set_lights(ctx.get(), selected.data(), ns), "set lights");

    // progressive tiles against one whole-image call
    const uint32_t W = 64, H = 40;
    const float eye[3] = { 0.0f, 2.2f, 5.5f }, target[3] = { 0.0f, 0.8f, 0.0f };
    ae_camera cam = LookAt(eye, target, W, H, 50.0f);
    DeviceBuffer<float> accum(size_t(W) * H * 4), output(size_t(W) * H * 4), ref(size_t(W) * H * 4),
        ref_out(size_t(W) * H * 4);
    PathTracerRenderTarget rt;
    rt.width = W;
    rt.height = H;
    rt.accum = accum.ptr;
    rt.output = output.ptr;
    PathTracingRenderer renderer(ctx);
    renderer.realTime = false;
    renderer.bounces = 3;
    for (int pass = 0; pass < 8 * 4; pass++) renderer.Render(rt, cam, 1.5f, 2, 2);
    ae_pt_params p;
    std::memset(&p, 0, sizeof(p));
    p.spp = 8;
    p.max_bounces = 3;
    p.seed = renderer.seed;
    p.epsilon = renderer.epsilon;
    ctx.Check(ae_rt_pathtrace(ctx.get(), &cam, &p, ref.ptr, nullptr, nullptr), "pathtrace");
    ctx.Check(ae_rt_pt_tonemap(ctx.get(), ref.ptr, W, H, 8, 1.5f, 1.0f / 2.2f, ref_out.ptr, nullptr), "tonemap");
    ctx.Synchronize();
    const std::vector<float> a = accum.Host(), r = ref.Host();
    double energy = 0.0;
    for (size_t k = 0; k < a.size(); k += 4) energy += a[k] + a[k + 1] + a[k + 2];
    if (renderer.GetSampleCount() != 8 || !Same(a, r) || !Same(output.Host(), ref_out.Host()) || !(energy > 0.0)) {
        std::fprintf(stderr, "tiles: count %d, accumulation %s, output %s, energy %g\n", renderer.GetSampleCount(),
                     Same(a, r) ? "same" : "differs", Same(output.Host(), ref_out.Host()) ? "same" : "differs",
                     energy);
        return 1;
    }
    std::printf("ok tiles: 2 x 2 subdivisions x 8 samples equal one 8-sample call (energy %.4g)\n", energy);

    // a camera move restarts the accumulation
    const float eye2[3] = { 0.6f, 2.0f, 5.5f };
    cam = LookAt(eye2, target, W, H, 50.0f);
    renderer.Render(rt, cam, 1.5f, 2, 2);
    const int32_t after_move = renderer.GetSampleCount();
    for (int pass = 0; pass < 3; pass++) renderer.Render(rt, cam, 1.5f, 2, 2);
    p.spp = 1;
    Cuda(cudaMemset(ref.ptr, 0, ref.n * sizeof(float)), "cudaMemset");
    ctx.Check(ae_rt_pathtrace(ctx.get(), &cam, &p, ref.ptr, nullptr, nullptr), "pathtrace");
    ctx.Synchronize();
    if (after_move != 0 || renderer.GetSampleCount() != 1 || !Same(accum.Host(), ref.Host())) {
        std::fprintf(stderr, "camera move: count %d then %d\n", after_move, renderer.GetSampleCount());
        return 1;
    }
    std::printf("ok camera move: the count restarted and one pass equals a 1-sample call\n");

    // subdivisions that do not divide the size: the remainder is not traced
    const uint32_t W3 = 50, H3 = 31;
    ae_camera cam3 = LookAt(eye, target, W3, H3, 50.0f);
    DeviceBuffer<float> acc3(size_t(W3) * H3 * 4);
    PathTracerRenderTarget rt3;
    rt3.width = W3;
    rt3.height = H3;
    rt3.accum = acc3.ptr;
    PathTracingRenderer r3(ctx);
    r3.realTime = false;
    r3.bounces = 3;
    for (int pass = 0; pass < 9; pass++) r3.Render(rt3, cam3, 1.0f, 3, 3);
    ctx.Synchronize();
    const std::vector<float> h3 = acc3.Host();
    bool rest_zero = true;
    size_t traced_nonzero = 0;
    for (uint32_t y = 0; y < H3; y++)
        for (uint32_t x = 0; x < W3; x++) {
            const float* px = &h3[(size_t(y) * W3 + x) * 4];
            const bool inside = x < (W3 / 3) * 3 && y < (H3 / 3) * 3;
            const bool nonzero = px[0] != 0.0f || px[1] != 0.0f || px[2] != 0.0f;
            if (!inside && nonzero) rest_zero = false;
            if (inside && nonzero) traced_nonzero++;
        }
    if (!rest_zero || r3.GetSampleCount() != 1 || traced_nonzero < 100) {
        std::fprintf(stderr, "remainder: untouched %d, count %d, traced %zu\n", int(rest_zero), r3.GetSampleCount(),
                     traced_nonzero);
        return 1;
    }
    std::printf("ok remainder: 3 x 3 subdivisions of 50 x 31 trace %zu lit pixels, none outside 48 x 30\n",
                traced_nonzero);

    // real-time mode
    DeviceBuffer<uint32_t> frame(size_t(W) * H * 3), frame_ref(size_t(W) * H * 3);
    rt.frameAccum = frame.ptr;
    renderer.realTime = true;
    renderer.maxRadiance = 16.0f;
    renderer.Render(rt, cam, 1.0f);
    ae_pt_params q;
    std::memset(&q, 0, sizeof(q));
    q.spp = uint32_t(renderer.realTimeSamplesPerFrame);
    q.max_bounces = 3;
    q.sample_offset = uint32_t(renderer.GetFrameCount()) * q.spp;
    q.seed = renderer.seed;
    q.epsilon = renderer.epsilon;
    ctx.Check(ae_rt_pathtrace_realtime(ctx.get(), &cam, &q, nullptr, frame_ref.ptr, 16.0f, nullptr), "realtime");
    ctx.Synchronize();
    if (renderer.GetFrameCount() != 1 || renderer.GetSampleCount() != 1 || !Same(frame.Host(), frame_ref.Host())) {
        std::fprintf(stderr, "real-time: frames %d, count %d\n", renderer.GetFrameCount(), renderer.GetSampleCount());
        return 1;
    }
    std::printf("ok real-time: one frame of %d samples equals ae_rt_pathtrace_realtime\n",
                renderer.realTimeSamplesPerFrame);

    ae_bvh_destroy(bvh);
    ae_mesh_asset_destroy(mesh);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <assets dir>\n", argv[0]);
        return 2;
    }
    try {
        return Run(argv[1]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
