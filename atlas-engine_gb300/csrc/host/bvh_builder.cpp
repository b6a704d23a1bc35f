// Host BVH builder emitting Atlas Engine's flattened BVH layout.
// See bvh_builder.h for the contract.  The comments cite the reference
// function each step reproduces (src/engine/volume/BVH.cpp).
//
// Floating-point conventions reproduced from the reference's vector library
// use (GLSL-defined min/max where the second operand wins only when strictly
// smaller/larger, left-to-right sums, separate rounding of every multiply
// and add -- the library is compiled with -ffp-contract=off).
#include "bvh_builder.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <thread>

namespace atlas::rt {
namespace {

constexpr float kHuge = std::numeric_limits<float>::max();

inline float Min(float x, float y) { return (y < x) ? y : x; }
inline float Max(float x, float y) { return (x < y) ? y : x; }

inline Box Empty() { return Box{{kHuge, kHuge, kHuge}, {-kHuge, -kHuge, -kHuge}}; }

// AABB::Grow(AABB) -- AABB.cpp:104
inline void Enclose(Box& b, const Box& o) {
    for (int a = 0; a < 3; a++) {
        b.hi[a] = Max(b.hi[a], o.hi[a]);
        b.lo[a] = Min(b.lo[a], o.lo[a]);
    }
}
// AABB::Grow(vec3) -- AABB.cpp:111 (point is the first operand there)
inline void EnclosePoint(Box& b, const float* p) {
    for (int a = 0; a < 3; a++) {
        b.hi[a] = Max(p[a], b.hi[a]);
        b.lo[a] = Min(p[a], b.lo[a]);
    }
}
// AABB::Intersect -- AABB.cpp:118
inline void Clip(Box& b, const Box& o) {
    for (int a = 0; a < 3; a++) {
        b.lo[a] = Max(b.lo[a], o.lo[a]);
        b.hi[a] = Min(b.hi[a], o.hi[a]);
    }
}
// AABB::GetSurfaceArea -- AABB.cpp:125
inline float Area(const Box& b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0f * ((dx * dy + dy * dz) + dz * dx);
}

struct Ref {
    uint32_t prim = 0;
    Box box = Empty();
};

struct Split {
    float cost = kHuge;
    int axis = -1;
    uint32_t bin = 0;
    float pos = 0.0f;
    Box left = Empty();
    Box right = Empty();
};

struct TreeNode {
    Box box;
    uint32_t depth = 0;
    std::vector<Ref> leaf;                 // non-empty => leaf
    std::unique_ptr<TreeNode> kid[2];      // [0] = left side of the split, [1] = right
};

// Bin count per depth -- BVH.cpp:447
inline uint32_t BinsAt(uint32_t binBudget, uint32_t depth) {
    return std::max(binBudget / (depth + 1), 16u);
}

// Bin index of a coordinate, glm::clamp(..., 0, bins - 1) truncated -- BVH.cpp:477
inline uint32_t BinIndex(float value, float start, float inv, uint32_t bins) {
    return uint32_t(Min(Max((value - start) * inv, 0.0f), float(bins) - 1.0f));
}

// Fixed-size worker pool: tasks may enqueue more tasks; Drain() returns when
// every task has finished.  Only the build schedule depends on it.
class TaskPool {
public:
    explicit TaskPool(unsigned workers) {
        for (unsigned i = 0; i < workers; i++) threads_.emplace_back([this] { Loop(); });
    }
    ~TaskPool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : threads_) t.join();
    }
    void Push(std::function<void()> f) {
        pending_.fetch_add(1);
        {
            std::lock_guard<std::mutex> g(m_);
            q_.push_back(std::move(f));
        }
        cv_.notify_one();
    }
    void Drain() {
        while (pending_.load() != 0) {
            std::function<void()> f;
            {
                std::lock_guard<std::mutex> g(m_);
                if (!q_.empty()) { f = std::move(q_.front()); q_.pop_front(); }
            }
            if (f) { f(); pending_.fetch_sub(1); }
            else std::this_thread::yield();
        }
    }

private:
    void Loop() {
        for (;;) {
            std::function<void()> f;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [this] { return stop_ || !q_.empty(); });
                if (stop_ && q_.empty()) return;
                f = std::move(q_.front());
                q_.pop_front();
            }
            f();
            pending_.fetch_sub(1);
        }
    }
    std::vector<std::thread> threads_;
    std::deque<std::function<void()>> q_;
    std::mutex m_;
    std::condition_variable cv_;
    std::atomic<long> pending_{0};
    bool stop_ = false;
};

class Builder {
public:
    Builder(const float* verts, uint32_t binBudget, TaskPool* pool)
        : verts_(verts), binBudget_(binBudget), pool_(pool) {}

    // Root of a triangle BVH -- BVHBuilder::Build(refs, data, ...) BVH.cpp:249-341.
    // Only the root reaches this overload; it may take a spatial split.
    void BuildRoot(TreeNode* node, std::vector<Ref>& refs, float minOverlap) {
        const float nodeCost = float(refs.size()) * Area(node->box);
        // (the leaf test of BVH.cpp:253 never fires at depth 0)
        Split obj = FindObjectSplit(*node, refs);
        Split spa;
        if (node->depth <= 16) {
            Box overlap = obj.left;
            Clip(overlap, obj.right);
            if (Area(overlap) >= minOverlap) spa = FindSpatialSplit(*node, refs);
        }
        std::vector<Ref> left, right;
        left.reserve(refs.size());
        right.reserve(refs.size());
        Split chosen;
        bool objBad = obj.axis < 0 || obj.cost >= nodeCost;
        bool spaBad = spa.axis < 0 || spa.cost >= nodeCost;
        if (objBad && spaBad) {
            chosen = MedianSplit(*node, refs, left, right);
        } else {
            if (spa.cost < obj.cost) {
                DoSpatialSplit(*node, refs, spa, left, right);
                chosen = spa;
            }
            if (obj.cost <= spa.cost) {
                left.clear();
                right.clear();
                DoObjectSplit(*node, refs, obj, left, right);
                chosen = obj;
            }
        }
        // BVH.cpp:304-305: an empty side turns this node into a leaf holding
        // every reference; the non-empty side is still built but never flattened.
        if (left.empty() || right.empty()) node->leaf = refs;
        refs.clear();
        refs.shrink_to_fit();
        Spawn(node, chosen, std::move(left), std::move(right));
    }

    // BVHBuilder::Build(refs, ...) for every other node -- BVH.cpp:343-406.
    void BuildInner(TreeNode* node, std::vector<Ref>& refs) {
        if (refs.size() == 1) {
            node->leaf = refs;
            return;
        }
        const float nodeCost = float(refs.size()) * Area(node->box);
        Split obj = FindObjectSplit(*node, refs);
        std::vector<Ref> left, right;
        left.reserve(refs.size() / 2);
        right.reserve(refs.size() / 2);
        Split chosen;
        if (obj.axis < 0 || obj.cost >= nodeCost) {
            chosen = MedianSplit(*node, refs, left, right);
        } else {
            DoObjectSplit(*node, refs, obj, left, right);
            chosen = obj;
        }
        refs.clear();
        refs.shrink_to_fit();
        Spawn(node, chosen, std::move(left), std::move(right));
    }

private:
    // Children get the split's boxes; depth <= 6 sub-trees go to the pool
    // (BVH.cpp:310-339).
    void Spawn(TreeNode* node, const Split& s, std::vector<Ref>&& left, std::vector<Ref>&& right) {
        std::vector<Ref>* sides[2] = { &left, &right };
        const Box* boxes[2] = { &s.left, &s.right };
        for (int k = 0; k < 2; k++) {
            if (sides[k]->empty()) continue;
            node->kid[k] = std::make_unique<TreeNode>();
            TreeNode* kid = node->kid[k].get();
            kid->box = *boxes[k];
            kid->depth = node->depth + 1;
            if (pool_ && node->depth <= 6) {
                auto moved = std::make_shared<std::vector<Ref>>(std::move(*sides[k]));
                pool_->Push([this, kid, moved] { BuildInner(kid, *moved); });
            } else {
                BuildInner(kid, *sides[k]);
            }
        }
    }

    // BVHBuilder::FindObjectSplit -- BVH.cpp:444-528.
    Split FindObjectSplit(const TreeNode& node, const std::vector<Ref>& refs) const {
        Split best;
        const uint32_t nb = BinsAt(binBudget_, node.depth);
        std::vector<Box> binBox(nb), suffix(nb);
        std::vector<uint32_t> binCount(nb);
        for (int axis = 0; axis < 3; axis++) {
            std::fill(binBox.begin(), binBox.end(), Empty());
            std::fill(binCount.begin(), binCount.end(), 0u);
            std::fill(suffix.begin(), suffix.end(), Empty());
            const float start = node.box.lo[axis], stop = node.box.hi[axis];
            if (std::fabs(stop - start) < 1e-3f) continue;
            const float width = (stop - start) / float(nb);
            const float inv = 1.0f / width;
            for (const Ref& r : refs) {
                float c = 0.5f * (r.box.lo[axis] + r.box.hi[axis]);
                uint32_t b = BinIndex(c, start, inv, nb);
                binCount[b]++;
                Enclose(binBox[b], r.box);
            }
            Box acc = Empty();
            for (size_t j = nb - 1; j > 0; j--) {
                Enclose(acc, binBox[j]);
                suffix[j - 1] = acc;
            }
            Box lacc = Empty();
            uint32_t nLeft = 0;
            for (size_t j = 1; j < nb; j++) {
                Enclose(lacc, binBox[j - 1]);
                nLeft += binCount[j - 1];
                const uint32_t nRight = uint32_t(refs.size()) - nLeft;
                if (!nLeft || !nRight) continue;
                const float cost = Area(lacc) * float(nLeft) + Area(suffix[j - 1]) * float(nRight);
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = axis;
                    best.bin = uint32_t(j);
                    best.pos = start + float(j) * width;
                    best.left = lacc;
                    best.right = suffix[j - 1];
                }
            }
        }
        return best;
    }

    // BVHBuilder::PerformObjectSplit -- BVH.cpp:530-556.
    void DoObjectSplit(const TreeNode& node, const std::vector<Ref>& refs, const Split& s,
                       std::vector<Ref>& left, std::vector<Ref>& right) const {
        const uint32_t nb = BinsAt(binBudget_, node.depth);
        const float start = node.box.lo[s.axis], stop = node.box.hi[s.axis];
        const float width = (stop - start) / float(nb);
        const float inv = 1.0f / width;
        for (const Ref& r : refs) {
            float c = 0.5f * (r.box.lo[s.axis] + r.box.hi[s.axis]);
            if (BinIndex(c, start, inv, nb) < s.bin) left.push_back(r);
            else right.push_back(r);
        }
    }

    // BVHBuilder::SplitReference -- BVH.cpp:760-798: clip a triangle's
    // reference box at an axis-aligned plane into a left and a right part.
    void ClipReference(uint32_t prim, const Box& current, float plane, int axis, Box& l, Box& r) const {
        const float* t = verts_ + size_t(prim) * 9;
        l = Empty();
        r = Empty();
        for (int e = 0; e < 3; e++) {
            const float* a = t + 3 * e;
            const float* b = t + 3 * ((e + 1) % 3);
            const bool crosses = (a[axis] < plane && b[axis] > plane) || (a[axis] > plane && b[axis] < plane);
            if (crosses) {
                float f = Min(Max((plane - a[axis]) / (b[axis] - a[axis]), 0.0f), 1.0f);
                float p[3];
                for (int k = 0; k < 3; k++) p[k] = a[k] * (1.0f - f) + b[k] * f;
                EnclosePoint(l, p);
                EnclosePoint(r, p);
            }
            if (a[axis] <= plane) EnclosePoint(l, a);
            if (a[axis] >= plane) EnclosePoint(r, a);
        }
        l.hi[axis] = plane;
        r.lo[axis] = plane;
        Clip(l, current);
        Clip(r, current);
    }

    // BVHBuilder::FindSpatialSplit -- BVH.cpp:558-667.
    Split FindSpatialSplit(const TreeNode& node, const std::vector<Ref>& refs) const {
        Split best;
        const uint32_t nb = BinsAt(binBudget_, node.depth);
        std::vector<Box> binBox(nb), suffix(nb);
        std::vector<uint32_t> enter(nb), leave(nb);
        for (int axis = 0; axis < 3; axis++) {
            std::fill(binBox.begin(), binBox.end(), Empty());
            std::fill(enter.begin(), enter.end(), 0u);
            std::fill(leave.begin(), leave.end(), 0u);
            std::fill(suffix.begin(), suffix.end(), Empty());
            const float start = node.box.lo[axis], stop = node.box.hi[axis];
            if (std::fabs(stop - start) < 1e-3f) continue;
            const float width = (stop - start) / float(nb);
            const float inv = 1.0f / width;
            for (const Ref& r : refs) {
                const uint32_t b0 = BinIndex(r.box.lo[axis], start, inv, nb);
                const uint32_t b1 = BinIndex(r.box.hi[axis], start, inv, nb);
                if (b0 == b1) {
                    enter[b0]++;
                    leave[b0]++;
                    Enclose(binBox[b0], r.box);
                    continue;
                }
                Box rest = r.box;
                for (uint32_t j = b0; j < b1; j++) {
                    const float plane = start + float(j + 1) * width;
                    Box l, rr;
                    ClipReference(r.prim, rest, plane, axis, l, rr);
                    Enclose(binBox[j], l);
                    rest = rr;
                }
                Enclose(binBox[b1], rest);
                enter[b0]++;
                leave[b1]++;
            }
            Box acc = Empty();
            for (size_t j = nb - 1; j > 0; j--) {
                Enclose(acc, binBox[j]);
                suffix[j - 1] = acc;
            }
            Box lacc = Empty();
            uint32_t nRight = uint32_t(refs.size()), nLeft = 0;
            for (size_t j = 1; j < nb; j++) {
                Enclose(lacc, binBox[j - 1]);
                nLeft += enter[j - 1];
                nRight -= leave[j - 1];
                if (!nLeft || !nRight) continue;
                const float cost = Area(lacc) * float(nLeft) + Area(suffix[j - 1]) * float(nRight);
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = axis;
                    best.bin = uint32_t(j);
                    best.pos = start + float(j) * width;
                    best.left = lacc;
                    best.right = suffix[j - 1];
                }
            }
        }
        return best;
    }

    // BVHBuilder::PerformSpatialSplit -- BVH.cpp:669-758: references wholly on
    // one side go there; straddling ones are kept whole on the cheaper side or
    // split into two references, whichever has the lowest SAH.
    void DoSpatialSplit(const TreeNode& node, const std::vector<Ref>& refs, Split& s,
                        std::vector<Ref>& left, std::vector<Ref>& right) const {
        const uint32_t nb = BinsAt(binBudget_, node.depth);
        const float start = node.box.lo[s.axis], stop = node.box.hi[s.axis];
        const float width = (stop - start) / float(nb);
        const float inv = 1.0f / width;
        auto bins = [&](const Ref& r, uint32_t& b0, uint32_t& b1) {
            b0 = BinIndex(r.box.lo[s.axis], start, inv, nb);
            b1 = BinIndex(r.box.hi[s.axis], start, inv, nb);
        };
        for (const Ref& r : refs) {
            uint32_t b0, b1;
            bins(r, b0, b1);
            if (b1 < s.bin) {
                left.push_back(r);
                Enclose(s.left, r.box);
            } else if (b0 >= s.bin) {
                right.push_back(r);
                Enclose(s.right, r.box);
            }
        }
        for (const Ref& r : refs) {
            uint32_t b0, b1;
            bins(r, b0, b1);
            if (!(b1 >= s.bin && b0 < s.bin)) continue;
            Box l, rr;
            ClipReference(r.prim, r.box, s.pos, s.axis, l, rr);
            Box keepLeft = s.left, keepRight = s.right, dupLeft = s.left, dupRight = s.right;
            Enclose(keepLeft, r.box);
            Enclose(keepRight, r.box);
            Enclose(dupLeft, l);
            Enclose(dupRight, rr);
            const float nl = float(left.size()), nr = float(right.size());
            const float nl1 = float(left.size() + 1), nr1 = float(right.size() + 1);
            const float costKeepLeft = Area(keepLeft) * nl1 + Area(s.right) * nr;
            const float costKeepRight = Area(s.left) * nl + Area(keepRight) * nr1;
            const float costDup = Area(dupLeft) * nl1 + Area(dupRight) * nr1;
            const float m = Min(costDup, Min(costKeepRight, costKeepLeft));
            if (m == costKeepLeft) {
                s.left = keepLeft;
                left.push_back(r);
            } else if (m == costKeepRight) {
                s.right = keepRight;
                right.push_back(r);
            } else {
                s.left = dupLeft;
                s.right = dupRight;
                left.push_back(Ref{r.prim, l});
                right.push_back(Ref{r.prim, rr});
            }
        }
    }

    // BVHBuilder::PerformMedianSplit -- BVH.cpp:800-855: split at the middle
    // of the longest axis; if one side stays empty, sort by extent along that
    // axis and halve the list.
    Split MedianSplit(const TreeNode& node, std::vector<Ref>& refs,
                      std::vector<Ref>& left, std::vector<Ref>& right) const {
        Split s;
        float ext[3] = { node.box.hi[0] - node.box.lo[0], node.box.hi[1] - node.box.lo[1],
                         node.box.hi[2] - node.box.lo[2] };
        int axis = 0;
        axis = ext[1] > ext[axis] ? 1 : axis;
        axis = ext[2] > ext[axis] ? 2 : axis;
        const float cut = node.box.lo[axis] + ext[axis] / 2.0f;
        for (const Ref& r : refs) {
            float c = (r.box.hi[axis] - r.box.lo[axis]) * 0.5f + r.box.lo[axis];
            if (c < cut) {
                Enclose(s.left, r.box);
                left.push_back(r);
            } else {
                Enclose(s.right, r.box);
                right.push_back(r);
            }
        }
        if (left.empty() || right.empty()) {
            s = Split();
            left.clear();
            right.clear();
            std::sort(refs.begin(), refs.end(), [axis](const Ref& a, const Ref& b) {
                return (a.box.hi[axis] - a.box.lo[axis]) < (b.box.hi[axis] - b.box.lo[axis]);
            });
            const uint32_t half = uint32_t(refs.size() / 2);
            for (uint32_t i = 0; i < half; i++) {
                Enclose(s.left, refs[i].box);
                left.push_back(refs[i]);
            }
            for (uint32_t i = half; i < uint32_t(refs.size()); i++) {
                Enclose(s.right, refs[i].box);
                right.push_back(refs[i]);
            }
        }
        return s;
    }

    const float* verts_;
    uint32_t binBudget_;
    TaskPool* pool_;
};

// BVHBuilder::Flatten -- BVH.cpp:408-441: pre-order, larger-area child first,
// leaf pointers ~firstPrimitive, inner pointers = node index.
void Flatten(TreeNode* n, BuiltBVH& out) {
    if (!n->leaf.empty()) {
        for (const Ref& r : n->leaf) {
            out.order.push_back(r.prim);
            out.endOfNode.push_back(0);
        }
        out.endOfNode.back() = 1;
        return;
    }
    const size_t self = out.nodes.size();
    out.nodes.emplace_back();
    TreeNode* a = n->kid[0].get();
    TreeNode* b = n->kid[1].get();
    if (Area(a->box) < Area(b->box)) std::swap(a, b);
    TreeNode* sides[2] = { a, b };
    for (int k = 0; k < 2; k++) {
        TreeNode* c = sides[k];
        if (!c) continue;
        const bool isLeaf = !c->leaf.empty();
        const int32_t ptr = isLeaf ? ~int32_t(out.order.size()) : int32_t(uint32_t(out.nodes.size()));
        if (k == 0) {
            out.nodes[self].left = c->box;
            out.nodes[self].leftPtr = ptr;
        } else {
            out.nodes[self].right = c->box;
            out.nodes[self].rightPtr = ptr;
        }
        Flatten(c, out);
    }
}

unsigned PoolThreads() {
    unsigned hw = std::thread::hardware_concurrency();
    return hw > 1 ? hw - 1 : 1;
}

}  // namespace

Box TriangleBox(const float* t) {
    Box b;
    for (int a = 0; a < 3; a++) {
        b.lo[a] = Min(Min(t[a], t[3 + a]), t[6 + a]);
        b.hi[a] = Max(Max(t[a], t[3 + a]), t[6 + a]);
    }
    return b;
}

BuiltBVH BuildTriangleBVH(const TriangleInput& in, bool parallel) {
    BuiltBVH out;
    if (in.count == 0) return out;  // the reference dereferences a missing child here
    std::vector<Ref> refs(in.count);
    for (uint32_t i = 0; i < in.count; i++) {
        refs[i].prim = i;
        if (in.boxes) {
            const float* b = in.boxes + size_t(i) * 6;
            refs[i].box = Box{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}};
        } else {
            refs[i].box = TriangleBox(in.verts + size_t(i) * 9);
        }
    }
    TreeNode root;
    root.box = Empty();
    for (const Ref& r : refs) Enclose(root.box, r.box);
    const float minOverlap = Area(root.box) * 10e-6f;   // BVH.cpp:33
    {
        std::unique_ptr<TaskPool> pool;
        if (parallel) pool = std::make_unique<TaskPool>(PoolThreads());
        Builder b(in.verts, 256, pool.get());
        b.BuildRoot(&root, refs, minOverlap);
        if (pool) pool->Drain();
    }
    Flatten(&root, out);
    return out;
}

BuiltBVH BuildBoxBVH(const float* boxes, uint32_t count, bool parallel) {
    BuiltBVH out;
    if (count == 0) return out;
    std::vector<Ref> refs(count);
    TreeNode root;
    root.box = Empty();
    for (uint32_t i = 0; i < count; i++) {
        const float* b = boxes + size_t(i) * 6;
        refs[i].prim = i;
        refs[i].box = Box{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}};
        Enclose(root.box, refs[i].box);
    }
    {
        std::unique_ptr<TaskPool> pool;
        if (parallel) pool = std::make_unique<TaskPool>(PoolThreads());
        Builder b(nullptr, 64, pool.get());
        b.BuildInner(&root, refs);
        if (pool) pool->Drain();
    }
    // A single instance gets a node of its own whose both pointers name it
    // and whose right box is empty at the origin (BVH.cpp:80-88).  Its
    // reference list keeps the input reference in front of the flattened one,
    // because the one-reference build returns before clearing it
    // (BVH.cpp:60-63, :346-348, :90), so the list holds the instance twice.
    if (count == 1) {
        BuiltNode n;
        n.left = root.box;
        n.right = Box{{0, 0, 0}, {0, 0, 0}};
        n.leftPtr = ~0;
        n.rightPtr = ~0;
        out.nodes.push_back(n);
        out.order.push_back(0);
        out.endOfNode.push_back(0);
    }
    Flatten(&root, out);
    return out;
}

}  // namespace atlas::rt
