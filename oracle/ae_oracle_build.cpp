// CPU restatement of Atlas Engine's BVH builder -- part of the ORACLE.
//
// TEST INFRASTRUCTURE ONLY.  bench.py's reference arm builds its BVH with it
// (so that arm maps no library of the product) and tests/ check it against
// the compiled reference's digests; nothing on the product path links it.
//
// What it restates (src/engine/volume/BVH.cpp, AABB.cpp):
//   Volume::BVH::BVH(aabbs, data)   :14-56   triangle BVH, root bin count 256,
//                                            minOverlap = SA(root) * 10e-6
//   Volume::BVH::BVH(aabbs)         :58-100  AABB-only BVH (top level), 64 bins,
//                                            the one-box special node
//   BVHBuilder::Build(refs, data)   :249-345 root only: object split, spatial
//                                            split when the object split's
//                                            child overlap is large, median
//                                            split when nothing improves
//   BVHBuilder::Build(refs)         :347-414 every deeper level: object split
//                                            down to 1-ref leaves, median
//                                            fallback
//   Flatten                         :416-449 pre-order, larger-SA child left
//   FindObjectSplit / PerformObjectSplit   :452-555
//   FindSpatialSplit / PerformSpatialSplit :557-758
//   SplitReference                  :760-798
//   PerformMedianSplit              :800-855
// The scalar min / max / clamp / mix are glm's GLSL definitions in the
// operand order of each call site (the signed zero that wins a tie depends
// on it), and every float expression keeps the reference's association.
// The median fallback sorts with std::sort, as the reference does, so that
// equal keys land in the same order with the same standard library.
//
// Output matches MeshData::BuildBVH's GPU layouts: 64-byte nodes
// (leftAABB, rightAABB, leftPtr, rightPtr, 0, 0) and, per BVH-order
// primitive, the original index and the end-of-leaf flag.
#include "ae_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace {

inline float gmin(float x, float y) { return (y < x) ? y : x; }   // GLSL min(x, y)
inline float gmax(float x, float y) { return (x < y) ? y : x; }   // GLSL max(x, y)
inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

struct Box {
    float lo[3] = { FLT_MAX, FLT_MAX, FLT_MAX };
    float hi[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };

    // AABB::Grow(AABB): max = max(max, o.max), min = min(min, o.min)
    void Add(const Box& o) {
        for (int k = 0; k < 3; k++) {
            hi[k] = gmax(hi[k], o.hi[k]);
            lo[k] = gmin(lo[k], o.lo[k]);
        }
    }
    // AABB::Grow(vec3): max = max(v, max), min = min(v, min)
    void AddPoint(const float* v) {
        for (int k = 0; k < 3; k++) {
            hi[k] = gmax(v[k], hi[k]);
            lo[k] = gmin(v[k], lo[k]);
        }
    }
    // AABB::Intersect: min = max(min, o.min), max = min(max, o.max)
    void Clip(const Box& o) {
        for (int k = 0; k < 3; k++) {
            lo[k] = gmax(lo[k], o.lo[k]);
            hi[k] = gmin(hi[k], o.hi[k]);
        }
    }
    float Area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Prim {
    uint32_t idx = 0;
    Box box;
};

struct Tri {
    float v[3][3];
};

struct Candidate {
    float cost = FLT_MAX;
    int axis = -1;
    uint32_t bin = 0;
    float pos = 0.0f;
    Box left, right;
};

struct Node {
    Box box;
    uint32_t depth = 0;
    uint32_t bins = 0;
    float minOverlap = 0.0f;
    float nodeCost = 0.0f;
    std::vector<Prim> leaf;       // non-empty: this is a leaf
    std::unique_ptr<Node> kid[2];

    Node(const Box& b, uint32_t d, size_t count, float overlap, uint32_t binCount)
        : box(b), depth(d), bins(binCount), minOverlap(overlap) {
        nodeCost = float(count) * box.Area();
    }

    uint32_t BinCount() const { return std::max(bins / (depth + 1), 16u); }

    uint32_t BinOf(float value, float start, float inv, uint32_t count) const {
        return uint32_t(gclamp((value - start) * inv, 0.0f, float(count) - 1.0f));
    }

    // FindObjectSplit (BVH.cpp:452-533): centroid bins, SAH sweep.
    Candidate ObjectSplit(const std::vector<Prim>& prims) const {
        Candidate best;
        const uint32_t count = BinCount();
        std::vector<Box> binBox(count), rightBox(count);
        std::vector<uint32_t> binN(count);
        for (int a = 0; a < 3; a++) {
            std::fill(binBox.begin(), binBox.end(), Box());
            std::fill(binN.begin(), binN.end(), 0u);
            std::fill(rightBox.begin(), rightBox.end(), Box());
            const float start = box.lo[a], stop = box.hi[a];
            if (fabsf(stop - start) < 1e-3f) continue;
            const float size = (stop - start) / float(count);
            const float inv = 1.0f / size;
            for (const Prim& p : prims) {
                const uint32_t b = BinOf(0.5f * (p.box.lo[a] + p.box.hi[a]), start, inv, count);
                binN[b]++;
                binBox[b].Add(p.box);
            }
            Box acc;
            for (size_t j = count - 1; j > 0; j--) {
                acc.Add(binBox[j]);
                rightBox[j - 1] = acc;
            }
            Box left;
            uint32_t nLeft = 0;
            for (size_t j = 1; j < count; j++) {
                left.Add(binBox[j - 1]);
                nLeft += binN[j - 1];
                const uint32_t nRight = uint32_t(prims.size()) - nLeft;
                if (!nLeft || !nRight) continue;
                const float cost = left.Area() * float(nLeft) + rightBox[j - 1].Area() * float(nRight);
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = a;
                    best.bin = uint32_t(j);
                    best.pos = start + float(j) * size;
                    best.left = left;
                    best.right = rightBox[j - 1];
                }
            }
        }
        return best;
    }

    // PerformObjectSplit (BVH.cpp:535-555): the same bins, split at best.bin.
    void DoObjectSplit(const std::vector<Prim>& prims, const Candidate& c, std::vector<Prim>& L,
                       std::vector<Prim>& R) const {
        const uint32_t count = BinCount();
        const float start = box.lo[c.axis], stop = box.hi[c.axis];
        const float size = (stop - start) / float(count);
        const float inv = 1.0f / size;
        for (const Prim& p : prims) {
            const uint32_t b = BinOf(0.5f * (p.box.lo[c.axis] + p.box.hi[c.axis]), start, inv, count);
            (b < c.bin ? L : R).push_back(p);
        }
    }

    // SplitReference (BVH.cpp:760-798): the triangle clipped to both sides of
    // the plane, each part intersected with the current reference box.
    static void Clip(const Tri& t, const Box& cur, float plane, int a, Box& L, Box& R) {
        L = Box();
        R = Box();
        for (int e = 0; e < 3; e++) {
            const float* p = t.v[e];
            const float* q = t.v[(e + 1) % 3];
            if ((p[a] < plane && q[a] > plane) || (p[a] > plane && q[a] < plane)) {
                const float f = gclamp((plane - p[a]) / (q[a] - p[a]), 0.0f, 1.0f);
                float x[3];
                for (int k = 0; k < 3; k++) x[k] = p[k] * (1.0f - f) + q[k] * f;   // mix(p, q, f)
                L.AddPoint(x);
                R.AddPoint(x);
            }
            if (p[a] <= plane) L.AddPoint(p);
            if (p[a] >= plane) R.AddPoint(p);
        }
        L.hi[a] = plane;
        R.lo[a] = plane;
        L.Clip(cur);
        R.Clip(cur);
    }

    // FindSpatialSplit (BVH.cpp:557-658): references clipped into every bin
    // they span, enter / exit counts per bin, SAH sweep.
    Candidate SpatialSplit(const std::vector<Prim>& prims, const std::vector<Tri>& tris) const {
        Candidate best;
        const uint32_t count = BinCount();
        std::vector<Box> binBox(count), rightBox(count);
        std::vector<uint32_t> enter(count), exit(count);
        for (int a = 0; a < 3; a++) {
            std::fill(binBox.begin(), binBox.end(), Box());
            std::fill(enter.begin(), enter.end(), 0u);
            std::fill(exit.begin(), exit.end(), 0u);
            std::fill(rightBox.begin(), rightBox.end(), Box());
            const float start = box.lo[a], stop = box.hi[a];
            if (fabsf(stop - start) < 1e-3f) continue;
            const float size = (stop - start) / float(count);
            const float inv = 1.0f / size;
            for (const Prim& p : prims) {
                const uint32_t b0 = BinOf(p.box.lo[a], start, inv, count);
                const uint32_t b1 = BinOf(p.box.hi[a], start, inv, count);
                if (b0 == b1) {
                    enter[b0]++;
                    exit[b0]++;
                    binBox[b0].Add(p.box);
                    continue;
                }
                Box cur = p.box;
                for (uint32_t j = b0; j < b1; j++) {
                    Box L, R;
                    Clip(tris[p.idx], cur, start + float(j + 1) * size, a, L, R);
                    binBox[j].Add(L);
                    cur = R;
                }
                binBox[b1].Add(cur);
                enter[b0]++;
                exit[b1]++;
            }
            Box acc;
            for (size_t j = count - 1; j > 0; j--) {
                acc.Add(binBox[j]);
                rightBox[j - 1] = acc;
            }
            Box left;
            uint32_t nRight = uint32_t(prims.size()), nLeft = 0;
            for (size_t j = 1; j < count; j++) {
                left.Add(binBox[j - 1]);
                nLeft += enter[j - 1];
                nRight -= exit[j - 1];
                if (!nLeft || !nRight) continue;
                const float cost = left.Area() * float(nLeft) + rightBox[j - 1].Area() * float(nRight);
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = a;
                    best.bin = uint32_t(j);
                    best.pos = start + float(j) * size;
                    best.left = left;
                    best.right = rightBox[j - 1];
                }
            }
        }
        return best;
    }

    // PerformSpatialSplit (BVH.cpp:660-758): references on one side go there;
    // straddling ones go left, right or to both (clipped), whichever SAH is
    // lowest given the sides so far.
    void DoSpatialSplit(const std::vector<Prim>& prims, const std::vector<Tri>& tris, Candidate& c,
                        std::vector<Prim>& L, std::vector<Prim>& R) const {
        const uint32_t count = BinCount();
        const int a = c.axis;
        const float start = box.lo[a], stop = box.hi[a];
        const float size = (stop - start) / float(count);
        const float inv = 1.0f / size;
        auto bins = [&](const Prim& p, uint32_t& b0, uint32_t& b1) {
            b0 = BinOf(p.box.lo[a], start, inv, count);
            b1 = BinOf(p.box.hi[a], start, inv, count);
        };
        for (const Prim& p : prims) {
            uint32_t b0, b1;
            bins(p, b0, b1);
            if (b1 < c.bin) {
                L.push_back(p);
                c.left.Add(p.box);
            } else if (b0 >= c.bin) {
                R.push_back(p);
                c.right.Add(p.box);
            }
        }
        for (const Prim& p : prims) {
            uint32_t b0, b1;
            bins(p, b0, b1);
            if (!(b1 >= c.bin && b0 < c.bin)) continue;
            Box pl, pr;
            Clip(tris[p.idx], p.box, c.pos, a, pl, pr);
            Box keepL = c.left, keepR = c.right, dupL = c.left, dupR = c.right;
            keepL.Add(p.box);
            keepR.Add(p.box);
            dupL.Add(pl);
            dupR.Add(pr);
            const float nl = float(L.size()), nr = float(R.size());
            const float nl1 = float(L.size() + 1), nr1 = float(R.size() + 1);
            const float sahLeft = keepL.Area() * nl1 + c.right.Area() * nr;
            const float sahRight = c.left.Area() * nl + keepR.Area() * nr1;
            const float sahDup = dupL.Area() * nl1 + dupR.Area() * nr1;
            const float m = gmin(sahDup, gmin(sahRight, sahLeft));
            if (m == sahLeft) {
                c.left = keepL;
                L.push_back(p);
            } else if (m == sahRight) {
                c.right = keepR;
                R.push_back(p);
            } else {
                c.left = dupL;
                c.right = dupR;
                Prim a1, a2;
                a1.idx = a2.idx = p.idx;
                a1.box = pl;
                a2.box = pr;
                L.push_back(a1);
                R.push_back(a2);
            }
        }
    }

    // PerformMedianSplit (BVH.cpp:800-855): the longest axis at its middle;
    // if one side stays empty, sort by extent on that axis and halve.
    Candidate MedianSplit(std::vector<Prim>& prims, std::vector<Prim>& L, std::vector<Prim>& R) const {
        Candidate c;
        const float d[3] = { box.hi[0] - box.lo[0], box.hi[1] - box.lo[1], box.hi[2] - box.lo[2] };
        int a = 0;
        a = d[1] > d[a] ? 1 : a;
        a = d[2] > d[a] ? 2 : a;
        const float cut = box.lo[a] + d[a] / 2.0f;
        for (const Prim& p : prims) {
            const float centre = (p.box.hi[a] - p.box.lo[a]) * 0.5f + p.box.lo[a];
            if (centre < cut) {
                c.left.Add(p.box);
                L.push_back(p);
            } else {
                c.right.Add(p.box);
                R.push_back(p);
            }
        }
        if (L.empty() || R.empty()) {
            c = Candidate();
            L.clear();
            R.clear();
            std::sort(prims.begin(), prims.end(), [a](const Prim& x, const Prim& y) {
                return x.box.hi[a] - x.box.lo[a] < y.box.hi[a] - y.box.lo[a];
            });
            const uint32_t half = uint32_t(prims.size() / 2);
            for (uint32_t i = 0; i < uint32_t(prims.size()); i++) {
                (i < half ? c.left : c.right).Add(prims[i].box);
                (i < half ? L : R).push_back(prims[i]);
            }
        }
        return c;
    }

    // Children at depth + 1, built by the AABB-only recursion; the top levels
    // fan out over threads (the reference hands depths <= 6 to its job system).
    void BuildChildren(std::vector<Prim>& L, std::vector<Prim>& R, const Candidate& c, bool parallel) {
        if (!L.empty()) kid[0].reset(new Node(c.left, depth + 1, L.size(), 0.0f, bins));
        if (!R.empty()) kid[1].reset(new Node(c.right, depth + 1, R.size(), 0.0f, bins));
        if (parallel && depth <= 3 && kid[0] && kid[1]) {
            std::thread t([&] { kid[0]->Build(L, parallel); });
            kid[1]->Build(R, parallel);
            t.join();
        } else {
            if (kid[0]) kid[0]->Build(L, parallel);
            if (kid[1]) kid[1]->Build(R, parallel);
        }
    }

    // BVHBuilder::Build(refs) (BVH.cpp:347-414)
    void Build(std::vector<Prim>& prims, bool parallel) {
        if (prims.size() == 1) {
            leaf = prims;
            return;
        }
        Candidate obj = ObjectSplit(prims);
        std::vector<Prim> L, R;
        Candidate c;
        if (obj.axis < 0 || obj.cost >= nodeCost) {
            c = MedianSplit(prims, L, R);
        } else {
            DoObjectSplit(prims, obj, L, R);
            c = obj;
        }
        std::vector<Prim>().swap(prims);
        BuildChildren(L, R, c, parallel);
    }

    // BVHBuilder::Build(refs, data) (BVH.cpp:249-345), for the root.
    void BuildRoot(std::vector<Prim>& prims, const std::vector<Tri>& tris, bool parallel) {
        Candidate obj = ObjectSplit(prims);
        Candidate spa;
        Box overlap = obj.left;
        overlap.Clip(obj.right);
        if (overlap.Area() >= minOverlap) spa = SpatialSplit(prims, tris);
        std::vector<Prim> L, R;
        Candidate c;
        if ((obj.axis < 0 || obj.cost >= nodeCost) && (spa.axis < 0 || spa.cost >= nodeCost)) {
            c = MedianSplit(prims, L, R);
        } else {
            if (spa.cost < obj.cost) {
                DoSpatialSplit(prims, tris, spa, L, R);
                c = spa;
            }
            if (obj.cost <= spa.cost) {
                L.clear();
                R.clear();
                DoObjectSplit(prims, obj, L, R);
                c = obj;
            }
        }
        if (L.empty() || R.empty()) {
            // the reference's last resort: the node becomes a leaf
            leaf = prims;
            return;
        }
        std::vector<Prim>().swap(prims);
        BuildChildren(L, R, c, parallel);
    }

    // Flatten (BVH.cpp:416-449): pre-order, the child of larger SA first.
    void Flatten(std::vector<aeo_node>& nodes, std::vector<Prim>& order, std::vector<uint8_t>& eon) {
        if (!leaf.empty()) {
            order.insert(order.end(), leaf.begin(), leaf.end());
            eon.resize(order.size(), 0);
            eon.back() = 1;
            return;
        }
        const size_t me = nodes.size();
        nodes.push_back(aeo_node{});
        if (kid[0]->box.Area() < kid[1]->box.Area()) std::swap(kid[0], kid[1]);
        for (int s = 0; s < 2; s++) {
            Node* k = kid[s].get();
            const int32_t ptr = !k->leaf.empty() ? ~int32_t(order.size()) : int32_t(nodes.size());
            aeo_node& nd = nodes[me];
            std::memcpy(s == 0 ? nd.lmin : nd.rmin, k->box.lo, 12);
            std::memcpy(s == 0 ? nd.lmax : nd.rmax, k->box.hi, 12);
            (s == 0 ? nd.left : nd.right) = ptr;
            k->Flatten(nodes, order, eon);
        }
    }
};

struct Result {
    std::vector<aeo_node> nodes;
    std::vector<Prim> order;
    std::vector<uint8_t> eon;
};

}  // namespace

struct aeo_bvh {
    Result r;
};

extern "C" {

aeo_bvh* aeo_build_triangles(const float* verts, uint32_t n_tris, int parallel) {
    auto* h = new aeo_bvh;
    if (n_tris == 0) return h;
    std::vector<Tri> tris(n_tris);
    std::vector<Prim> prims(n_tris);
    Box root;
    for (uint32_t i = 0; i < n_tris; i++) {
        std::memcpy(tris[i].v, verts + size_t(i) * 9, 36);
        // the triangle's box as MeshData::BuildBVH forms it (MeshData.cpp:143-146):
        // min(min(v0, v1), v2), max(max(v0, v1), v2)
        Box b;
        for (int k = 0; k < 3; k++) {
            b.lo[k] = gmin(gmin(tris[i].v[0][k], tris[i].v[1][k]), tris[i].v[2][k]);
            b.hi[k] = gmax(gmax(tris[i].v[0][k], tris[i].v[1][k]), tris[i].v[2][k]);
        }
        prims[i].idx = i;
        prims[i].box = b;
        root.Add(b);
    }
    Node top(root, 0, prims.size(), root.Area() * 10e-6f, 256);
    top.BuildRoot(prims, tris, parallel != 0);
    top.Flatten(h->r.nodes, h->r.order, h->r.eon);
    return h;
}

aeo_bvh* aeo_build_aabbs(const float* boxes, uint32_t n, int parallel) {
    auto* h = new aeo_bvh;
    if (n == 0) return h;
    std::vector<Prim> prims(n);
    Box root;
    for (uint32_t i = 0; i < n; i++) {
        prims[i].idx = i;
        std::memcpy(prims[i].box.lo, boxes + size_t(i) * 6, 12);
        std::memcpy(prims[i].box.hi, boxes + size_t(i) * 6 + 3, 12);
        root.Add(prims[i].box);
    }
    if (n == 1) {
        // BVH.cpp:80-88: the one-box tree is a node whose children are both
        // the leaf of box 0, the right one with a zero box
        aeo_node nd{};
        std::memcpy(nd.lmin, root.lo, 12);
        std::memcpy(nd.lmax, root.hi, 12);
        nd.left = ~0;
        nd.right = ~0;
        h->r.nodes.push_back(nd);
        // the root is a leaf, whose Build returns without clearing the input
        // references: Flatten appends after them, so the reference's refs
        // hold box 0 twice (the first without the end-of-leaf flag)
        h->r.order.push_back(prims[0]);
        h->r.eon.push_back(0);
    }
    Node top(root, 0, prims.size(), 0.0f, 64);
    top.Build(prims, parallel != 0);
    top.Flatten(h->r.nodes, h->r.order, h->r.eon);
    return h;
}

uint32_t aeo_bvh_node_count(const aeo_bvh* h) { return uint32_t(h->r.nodes.size()); }
uint32_t aeo_bvh_prim_count(const aeo_bvh* h) { return uint32_t(h->r.order.size()); }

void aeo_bvh_get(const aeo_bvh* h, aeo_node* nodes, uint32_t* order, uint8_t* end_of_node) {
    if (nodes && !h->r.nodes.empty()) std::memcpy(nodes, h->r.nodes.data(), h->r.nodes.size() * sizeof(aeo_node));
    for (size_t i = 0; i < h->r.order.size(); i++) {
        if (order) order[i] = h->r.order[i].idx;
        if (end_of_node) end_of_node[i] = h->r.eon[i];
    }
}

void aeo_bvh_free(aeo_bvh* h) { delete h; }

}  // extern "C"
