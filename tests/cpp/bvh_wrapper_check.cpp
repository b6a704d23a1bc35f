// Drives the C++ wrapper (include/atlas_rt.hpp) for the tests in
// tests/test_cpp_wrapper.py, through binary files of plain arrays.
//
//   bvh_wrapper_check build <in> <out>
//       in:  u32 kind (0 = triangles, 1 = boxes), u32 n, then n * 9 vertex
//            floats and n * 6 box floats (kind 0) or n * 6 box floats (kind 1)
//       out: the BVH's public members as counted arrays: nodes (16 floats in
//            the GPUBVHNode layout), data (9 floats, u32 idx, u8 endOfNode),
//            refs (u32 idx, u32 nodeIdx, u8 endOfNode, 6 floats), aabbs
//            (6 floats)
//   bvh_wrapper_check trace <in> <out>
//       in:  u32 n_tris, n_tris * 9 floats, u32 n_rays, n_rays * 8 floats
//            (origin, direction, tMin, tMax)
//       out: TraceClosest (u8 hit, 3 floats t u v, i32 triPtr, u32 idx per
//            ray), TraceAny (u8), then for the first m rays GetIntersection
//            (u8, u32 closest.idx, 3 floats) and GetIntersectionAny (u8)
// Exit status 0 on success; a thrown atlas::rt::Error prints its message.
#include "atlas_rt.hpp"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <iterator>

using namespace atlas::rt;

namespace {

struct Reader {
    std::vector<char> buf;
    size_t pos = 0;
    explicit Reader(const char* path) {
        std::ifstream f(path, std::ios::binary);
        buf.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    template <class T> T get() {
        if (pos + sizeof(T) > buf.size()) throw std::runtime_error("input file too short");
        T v;
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    vec3 v3() {
        const float x = get<float>(), y = get<float>(), z = get<float>();
        return vec3(x, y, z);
    }
};

struct Writer {
    std::FILE* f;
    explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
        if (!f) throw std::runtime_error("cannot open output file");
    }
    ~Writer() { std::fclose(f); }
    template <class T> void put(T v) { std::fwrite(&v, sizeof(T), 1, f); }
    void v3(const vec3& v) { put(v.x), put(v.y), put(v.z); }
};

void WriteMembers(const BVH& b, Writer& w) {
    w.put(uint32_t(b.nodes.size()));
    for (const BVHNode& n : b.nodes) {
        w.v3(n.leftAABB.min), w.v3(n.leftAABB.max), w.v3(n.rightAABB.min), w.v3(n.rightAABB.max);
        w.put(n.leftPtr), w.put(n.rightPtr), w.put(int32_t(0)), w.put(int32_t(0));
    }
    w.put(uint32_t(b.data.size()));
    for (const BVHTriangle& t : b.data) w.v3(t.v0), w.v3(t.v1), w.v3(t.v2);
    for (const BVHTriangle& t : b.data) w.put(t.idx);
    for (const BVHTriangle& t : b.data) w.put(uint8_t(t.endOfNode));
    w.put(uint32_t(b.refs.size()));
    for (const Ref& r : b.refs) w.put(r.idx);
    for (const Ref& r : b.refs) w.put(r.nodeIdx);
    for (const Ref& r : b.refs) w.put(uint8_t(r.endOfNode));
    for (const Ref& r : b.refs) w.v3(r.aabb.min), w.v3(r.aabb.max);
    w.put(uint32_t(b.aabbs.size()));
    for (const AABB& a : b.aabbs) w.v3(a.min), w.v3(a.max);
}

int Build(const char* in, const char* out) {
    Reader r(in);
    const uint32_t kind = r.get<uint32_t>(), n = r.get<uint32_t>();
    std::vector<BVHTriangle> tris(kind == 0 ? n : 0);
    std::vector<AABB> boxes(n);
    for (uint32_t i = 0; i < tris.size(); i++) {
        tris[i].v0 = r.v3(), tris[i].v1 = r.v3(), tris[i].v2 = r.v3();
        tris[i].idx = i;
    }
    for (uint32_t i = 0; i < n; i++) {
        const vec3 mn = r.v3(), mx = r.v3();
        boxes[i] = AABB(mn, mx);
    }
    BVH b = kind == 0 ? BVH(boxes, tris) : BVH(boxes);
    Writer w(out);
    WriteMembers(b, w);
    return 0;
}

int Trace(const char* in, const char* out) {
    Reader r(in);
    const uint32_t nt = r.get<uint32_t>();
    std::vector<BVHTriangle> tris(nt);
    std::vector<AABB> boxes(nt);
    for (uint32_t i = 0; i < nt; i++) {
        tris[i].v0 = r.v3(), tris[i].v1 = r.v3(), tris[i].v2 = r.v3();
        tris[i].idx = i;
        vec3 mn, mx;
        for (int c = 0; c < 3; c++) {
            mn[c] = std::min(std::min(tris[i].v0[c], tris[i].v1[c]), tris[i].v2[c]);
            mx[c] = std::max(std::max(tris[i].v0[c], tris[i].v1[c]), tris[i].v2[c]);
        }
        boxes[i] = AABB(mn, mx);
    }
    const uint32_t nr = r.get<uint32_t>();
    std::vector<Ray> rays(nr);
    for (uint32_t i = 0; i < nr; i++) {
        const vec3 o = r.v3(), d = r.v3();
        const float tmin = r.get<float>(), tmax = r.get<float>();
        rays[i] = Ray(o, d, tmin, tmax);
    }
    BVH b(boxes, tris);
    bool refused = false;
    try {
        b.TraceClosest(rays);
    } catch (const Error& e) {
        refused = e.status == AE_RT_INVALID_ARG;
    }
    if (!refused) throw std::runtime_error("a query before Upload was not refused");
    Context ctx(0);
    b.Upload(ctx);
    const std::vector<Hit> hits = b.TraceClosest(rays);
    const std::vector<uint8_t> occ = b.TraceAny(rays);
    Writer w(out);
    for (const Hit& h : hits) w.put(uint8_t(h.hit));
    for (const Hit& h : hits) w.put(h.t), w.put(h.u), w.put(h.v);
    for (const Hit& h : hits) w.put(h.triPtr);
    for (const Hit& h : hits) w.put(h.idx);
    for (uint8_t o : occ) w.put(o);
    const uint32_t m = std::min<uint32_t>(nr, 64);
    w.put(m);
    std::vector<std::pair<int32_t, float>> stack(64);
    std::vector<uint8_t> sh(m), sa(m);
    std::vector<uint32_t> si(m);
    std::vector<vec3> sx(m);
    for (uint32_t i = 0; i < m; i++) {
        BVHTriangle closest;
        sh[i] = b.GetIntersection(stack, rays[i], closest, sx[i]) ? 1 : 0;
        si[i] = closest.idx;
        sa[i] = b.GetIntersectionAny(stack, rays[i]) ? 1 : 0;
    }
    for (uint8_t v : sh) w.put(v);
    for (uint32_t v : si) w.put(v);
    for (const vec3& v : sx) w.v3(v);
    for (uint8_t v : sa) w.put(v);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s build|trace <in> <out>\n", argv[0]);
        return 2;
    }
    try {
        const std::string mode = argv[1];
        if (mode == "build") return Build(argv[2], argv[3]);
        if (mode == "trace") return Trace(argv[2], argv[3]);
        std::fprintf(stderr, "unknown mode %s\n", argv[1]);
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
