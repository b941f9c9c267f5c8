// Host binned-SAH builder; see bvh_builder.h for what it reproduces and how.
// Built with -ffp-contract=off so every float operation rounds as the
// reference's x86-64 build does.
#include "bvh_builder.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <deque>
#include <future>
#include <limits>
#include <mutex>
#include <thread>

namespace ptg {
namespace {

constexpr int kBins = 16;           // BinnedSAHBVH.h:174
constexpr int kMaxLeafPrims = 4;    // BinnedSAHBVH.cpp:62
constexpr int kParallelCutoff = 32768;

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void Merge(const Box& b) {  // AABB::Merge (AABB.cpp:10-20): std::min/std::max
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void Merge(const float* p) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float SurfaceArea() const {  // AABB.h:71-76
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
    int WidestAxis() const {  // AABB.cpp:54-71
        float best = 0.0f;
        int axis = 0;
        for (int a = 0; a < 3; a++) {
            const float w = hi[a] - lo[a];
            if (w > best) {
                best = w;
                axis = a;
            }
        }
        return axis;
    }
};

struct Prim {
    Box box;
    float c[3];
};

struct BNode {
    Box box;
    int begin, end;
    BNode* left = nullptr;
    BNode* right = nullptr;
};

// Node storage shared by all build tasks (deque keeps addresses stable).
struct Arena {
    std::mutex mu;
    std::deque<BNode> nodes;
    BNode* New(const Box& b, int begin, int end) {
        std::lock_guard<std::mutex> g(mu);
        nodes.push_back(BNode{b, begin, end});
        return &nodes.back();
    }
};

struct Builder {
    const std::vector<Prim>& prims;
    std::vector<int32_t>& ids;
    Arena& arena;
    std::atomic<int>& budget;  // threads still available for subtree tasks

    // Splits `n` (or leaves it a leaf) exactly as the reference's loop body does.
    void Split(BNode* n) {
        const int b = n->begin, e = n->end;
        if (e - b <= kMaxLeafPrims) return;
        Box cb;
        for (int i = b; i < e; i++) cb.Merge(prims[ids[i]].c);
        const int ax = cb.WidestAxis();
        std::sort(ids.begin() + b, ids.begin() + e,
                  [&](int x, int y) { return prims[x].c[ax] < prims[y].c[ax]; });
        const float len = cb.hi[ax] - cb.lo[ax];
        Box binBox[kBins];
        int binCount[kBins] = {0};
        for (int i = b; i < e; i++) {
            const Prim& p = prims[ids[i]];
            const float l = p.c[ax] - cb.lo[ax];
            const float f = std::nextafter(kBins * l / len, 0.0f);
            // zero-width centroid range: NaN bin in the reference (an undefined cast);
            // every candidate split then puts all primitives on one side -> leaf.
            int bin = std::isnan(f) ? 0 : (int)f;
            bin = std::min(std::max(bin, 0), kBins - 1);
            binBox[bin].Merge(p.box);
            binCount[bin]++;
        }
        // GetSAHCost for every candidate split k: left = bins < k, right = bins >= k.
        Box suffix[kBins + 1];
        int suffixCount[kBins + 1] = {0};
        for (int k = kBins - 1; k >= 0; k--) {
            suffix[k] = suffix[k + 1];
            suffix[k].Merge(binBox[k]);
            suffixCount[k] = suffixCount[k + 1] + binCount[k];
        }
        Box prefix;
        int prefixCount = 0;
        int bestBin = 0, bestLeft = 0;
        float minCost = std::numeric_limits<float>::max();
        Box bestL, bestR;
        for (int k = 0; k < kBins; k++) {
            if (k > 0) {
                prefix.Merge(binBox[k - 1]);
                prefixCount += binCount[k - 1];
            }
            const int nl = prefixCount, nr = suffixCount[k];
            const float sal = nl ? prefix.SurfaceArea() : 0;
            const float sar = nr ? suffix[k].SurfaceArea() : 0;
            const float cost = nl * sal + nr * sar;
            if (cost < minCost) {
                minCost = cost;
                bestBin = k;
                bestLeft = nl;
                bestL = prefix;
                bestR = suffix[k];
            }
        }
        if (bestBin == 0) return;
        // The child bounds are merges in range order (BinnedSAHBVH.cpp:163-186), where the
        // first of equal extremes wins (+0 against -0): merge the right child's bins in
        // ascending order rather than take the suffix, which merged them descending.
        bestR = Box();
        for (int k = bestBin; k < kBins; k++) bestR.Merge(binBox[k]);
        n->left = arena.New(bestL, b, b + bestLeft);
        n->right = arena.New(bestR, b + bestLeft, e);
    }

    void Build(BNode* n) {
        Split(n);
        if (!n->left) return;
        const bool bigL = n->left->end - n->left->begin > kParallelCutoff;
        const bool bigR = n->right->end - n->right->begin > kParallelCutoff;
        if (bigL && bigR && budget.fetch_sub(1) > 0) {
            auto f = std::async(std::launch::async, [this, n] { Build(n->left); });
            Build(n->right);
            f.get();
            budget.fetch_add(1);
        } else {
            if (bigL && bigR) budget.fetch_add(1);
            Build(n->right);
            Build(n->left);
        }
    }
};

}  // namespace

BvhResult BuildBinnedSah(const float* P, const int32_t* idx, int T, int threads) {
    BvhResult out;
    std::vector<Prim> prims(T);
    Box root;
    for (int t = 0; t < T; t++) {
        Prim& p = prims[t];
        const float* v[3] = {P + 3 * idx[3 * t], P + 3 * idx[3 * t + 1], P + 3 * idx[3 * t + 2]};
        for (int k = 0; k < 3; k++) p.box.Merge(v[k]);
        for (int a = 0; a < 3; a++) p.c[a] = (v[0][a] + v[1][a] + v[2][a]) / 3.0f;  // Triangle::GetCentroid
        root.Merge(p.box);
    }
    out.primIds.resize(T);
    for (int i = 0; i < T; i++) out.primIds[i] = i;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    Arena arena;
    std::atomic<int> budget(threads - 1);
    Builder bld{prims, out.primIds, arena, budget};
    BNode* r = arena.New(root, 0, T);
    bld.Build(r);

    // Number nodes in the reference's order: a node's two children get the next two
    // indices when it is split; the right subtree is then split before the left.
    out.nodes.reserve(arena.nodes.size());
    struct Item { BNode* n; int index; int depth; };
    std::vector<Item> stack;
    out.nodes.push_back({});
    stack.push_back({r, 0, 0});
    while (!stack.empty()) {
        const Item it = stack.back();
        stack.pop_back();
        BvhNodeOut& o = out.nodes[it.index];
        for (int a = 0; a < 3; a++) {
            o.lo[a] = it.n->box.lo[a];
            o.hi[a] = it.n->box.hi[a];
        }
        o.begin = it.n->begin;
        o.end = it.n->end;
        out.height = std::max(out.height, it.depth);
        if (!it.n->left) {
            o.leaf = true;
            o.child[0] = o.child[1] = (it.index == 0) ? 0 : -1;
            continue;
        }
        o.leaf = false;
        const int li = (int)out.nodes.size();
        o.child[0] = li;
        o.child[1] = li + 1;
        out.nodes.push_back({});
        out.nodes.push_back({});
        stack.push_back({it.n->left, li, it.depth + 1});
        stack.push_back({it.n->right, li + 1, it.depth + 1});
    }
    return out;
}

namespace {

struct WideCollapser {
    const BvhResult& b;
    std::vector<float>& out;  // WideNodeFloats(K) floats per wide node
    const int K;
    bool ok = true;
    // Child boxes are widened by eps on every side (eps = 2^-18 of the scene's largest
    // coordinate magnitude). The slab test's rounding (a few ulps of the plane distance)
    // then can never cut off a ray that meets a triangle inside: the traversal reports
    // every triangle the triangle test accepts, as a test of all triangles would.
    float eps = 0.0f;

    static float Area(const BvhNodeOut& n) {
        const float dx = n.hi[0] - n.lo[0], dy = n.hi[1] - n.lo[1], dz = n.hi[2] - n.lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
    // Empty child slots: code INT32_MIN and a box at +infinity on every plane, which no
    // slab test hits (the traversal tests every slot's box without reading its code).
    int NewNode() {
        const size_t nf = (size_t)WideNodeFloats(K);
        const int w = (int)(out.size() / nf);
        out.resize(out.size() + nf, 0.0f);
        float* f = &out[(size_t)w * nf];
        for (int i = 0; i < 6 * K; i++) f[i] = std::numeric_limits<float>::infinity();
        int32_t* codes = reinterpret_cast<int32_t*>(&out[(size_t)w * nf + 6 * K]);
        for (int i = 0; i < K; i++) codes[i] = INT32_MIN;
        return w;
    }
    void SetChild(int w, int i, const float* lo, const float* hi, int32_t code) {
        float* f = &out[(size_t)w * WideNodeFloats(K)];
        for (int a = 0; a < 3; a++) {
            f[K * a + i] = lo[a] - eps;
            f[K * (3 + a) + i] = hi[a] + eps;
        }
        std::memcpy(&f[6 * K + i], &code, 4);
    }
    int32_t LeafCode(int first, int count) {
        if (first >= (1 << 25)) ok = false;
        return -((first << 6) | count) - 1;
    }
    // A leaf range as a child code: one chunk, or a chain of leaf-list nodes.
    int32_t Leaf(const BvhNodeOut& n) {
        const int count = n.end - n.begin;
        if (count <= kWideLeafMax) return LeafCode(n.begin, count);
        const int w = NewNode();
        int first = n.begin, left = count;
        for (int i = 0; i < K && left > 0; i++) {
            if (i == K - 1 && left > kWideLeafMax) {
                BvhNodeOut rest = n;
                rest.begin = first;
                rest.end = n.end;
                SetChild(w, i, n.lo, n.hi, Leaf(rest));
                left = 0;
                break;
            }
            const int c = std::min(left, kWideLeafMax);
            SetChild(w, i, n.lo, n.hi, LeafCode(first, c));
            first += c;
            left -= c;
        }
        return w;
    }
    // The children of the wide node made from inner binary node bi: its two children,
    // then, while there is room, the largest-area inner child replaced by its two.
    int Pick(int bi, int* cand) const {
        const BvhNodeOut& n = b.nodes[bi];
        cand[0] = n.child[0];
        cand[1] = n.child[1];
        int nc = 2;
        while (nc < K) {
            int best = -1;
            float bestA = -1.0f;
            for (int i = 0; i < nc; i++)
                if (!b.nodes[cand[i]].leaf && Area(b.nodes[cand[i]]) > bestA) {
                    bestA = Area(b.nodes[cand[i]]);
                    best = i;
                }
            if (best < 0) break;
            const int open = cand[best];
            cand[best] = b.nodes[open].child[0];
            cand[nc++] = b.nodes[open].child[1];
        }
        return nc;
    }
    // The child code of binary node bi, its wide nodes appended in depth-first preorder.
    int32_t Code(int bi) { return b.nodes[bi].leaf ? Leaf(b.nodes[bi]) : Node(bi); }
    int32_t Node(int bi) {
        int cand[8];
        const int nc = Pick(bi, cand);
        const int w = NewNode();
        for (int i = 0; i < nc; i++) {
            const BvhNodeOut& c = b.nodes[cand[i]];
            SetChild(w, i, c.lo, c.hi, Code(cand[i]));
        }
        return w;
    }
};

// Below this many primitives the collapse runs on one thread.
constexpr int kCollapseParallelMin = 1 << 16;

// The same wide tree as one WideCollapser run from the root, built on several threads:
// the top wide nodes are laid out on one thread, the subtrees below them (tasks) are
// collapsed in parallel into their own arrays with local node numbers, and every array is
// then placed at its offset in the depth-first preorder, its node codes moved by that
// offset. Node for node and bit for bit the serial result.
bool CollapseParallel(const BvhResult& bvh, std::vector<float>* wide, int K, float eps, int threads) {
    const size_t nf = (size_t)WideNodeFloats(K);
    auto prims = [&](int bi) { return bvh.nodes[bi].end - bvh.nodes[bi].begin; };
    // top nodes: the root, then the largest inner tasks, until there are enough tasks
    std::vector<char> top(bvh.nodes.size(), 0);
    top[0] = 1;
    WideCollapser picker{bvh, *wide, K};
    const size_t target = (size_t)threads * 8;
    std::vector<int> open{0};
    for (;;) {
        // the tasks of the current top tree, largest inner one first
        std::vector<int> tasks;
        for (int t : open) {
            int cand[8];
            const int nc = picker.Pick(t, cand);
            for (int i = 0; i < nc; i++)
                if (!top[cand[i]]) tasks.push_back(cand[i]);
        }
        if (tasks.size() >= target) break;
        int best = -1;
        for (int t : tasks)
            if (!bvh.nodes[t].leaf && prims(t) >= 4096 && (best < 0 || prims(t) > prims(best))) best = t;
        if (best < 0) break;
        top[best] = 1;
        open.push_back(best);
    }
    // preorder: top nodes and tasks, as the serial collapse reaches them (a top child's
    // whole subtree before the next slot)
    struct Item {
        int bi;
        bool isTop;
    };
    std::vector<Item> order;
    struct Emitter {
        const std::vector<char>& top;
        const WideCollapser& picker;
        std::vector<Item>& order;
        void Emit(int bi) {
            order.push_back({bi, true});
            int cand[8];
            const int nc = picker.Pick(bi, cand);
            for (int i = 0; i < nc; i++) {
                if (top[cand[i]]) Emit(cand[i]);
                else order.push_back({cand[i], false});
            }
        }
    } emitter{top, picker, order};
    emitter.Emit(0);
    // the tasks, in parallel
    std::vector<int> taskOf(order.size(), -1);  // item -> task
    std::vector<int> taskNodes, taskItem;        // task -> binary node, item
    for (size_t k = 0; k < order.size(); k++)
        if (!order[k].isTop) {
            taskOf[k] = (int)taskNodes.size();
            taskNodes.push_back(order[k].bi);
            taskItem.push_back((int)k);
        }
    std::vector<std::vector<float>> local(taskNodes.size());
    std::vector<int32_t> rootCode(taskNodes.size(), 0);
    std::vector<char> okTask(taskNodes.size(), 1);
    std::atomic<size_t> next(0);
    auto work = [&]() {
        for (size_t t; (t = next.fetch_add(1)) < taskNodes.size();) {
            // about one wide node per three binary inner nodes (two per primitive at most)
            local[t].reserve(((size_t)prims(taskNodes[t]) * 2 / 3 + 16) * nf);
            WideCollapser c{bvh, local[t], K};
            c.eps = eps;
            rootCode[t] = c.Code(taskNodes[t]);
            okTask[t] = c.ok ? 1 : 0;
        }
    };
    {
        std::vector<std::thread> pool;
        for (int i = 1; i < threads; i++) pool.emplace_back(work);
        work();
        for (std::thread& th : pool) th.join();
    }
    for (char ok : okTask)
        if (!ok) return false;
    // offsets in preorder
    std::vector<int> index(order.size(), 0);
    size_t total = 0;
    for (size_t k = 0; k < order.size(); k++) {
        index[k] = (int)total;
        total += order[k].isTop ? 1 : local[taskOf[k]].size() / nf;
    }
    wide->assign(total * nf, 0.0f);
    // the top nodes, their children's codes resolved
    std::vector<int> topIndex(bvh.nodes.size(), -1), taskAt(bvh.nodes.size(), -1);
    for (size_t k = 0; k < order.size(); k++) {
        if (order[k].isTop) topIndex[order[k].bi] = index[k];
        else taskAt[order[k].bi] = (int)k;
    }
    WideCollapser writer{bvh, *wide, K};
    writer.eps = eps;
    for (size_t k = 0; k < order.size(); k++) {
        if (!order[k].isTop) continue;
        const int w = index[k];
        float* f = &(*wide)[(size_t)w * nf];
        for (int i = 0; i < 6 * K; i++) f[i] = std::numeric_limits<float>::infinity();
        int32_t* codes = reinterpret_cast<int32_t*>(f + 6 * K);
        for (int i = 0; i < K; i++) codes[i] = INT32_MIN;
        int cand[8];
        const int nc = picker.Pick(order[k].bi, cand);
        for (int i = 0; i < nc; i++) {
            const BvhNodeOut& c = bvh.nodes[cand[i]];
            int32_t code;
            if (topIndex[cand[i]] >= 0) {
                code = topIndex[cand[i]];
            } else {
                const int at = taskAt[cand[i]];
                const int32_t rc = rootCode[taskOf[at]];
                code = rc >= 0 ? rc + index[at] : rc;
            }
            writer.SetChild(w, i, c.lo, c.hi, code);
        }
    }
    // the task arrays at their offsets, node codes moved
    next = 0;
    auto place = [&]() {
        for (size_t t; (t = next.fetch_add(1)) < taskNodes.size();) {
            const int base = index[taskItem[t]];
            const std::vector<float>& src = local[t];
            float* dst = &(*wide)[(size_t)base * nf];
            std::memcpy(dst, src.data(), src.size() * sizeof(float));
            for (size_t w = 0; w < src.size() / nf; w++) {
                int32_t* codes = reinterpret_cast<int32_t*>(dst + w * nf + 6 * K);
                for (int i = 0; i < K; i++)
                    if (codes[i] >= 0) codes[i] += base;
            }
        }
    };
    {
        std::vector<std::thread> pool;
        for (int i = 1; i < threads; i++) pool.emplace_back(place);
        place();
        for (std::thread& th : pool) th.join();
    }
    return true;
}

}  // namespace

bool CollapseWide(const BvhResult& bvh, std::vector<float>* wide, int width, float* epsOut,
                  int threads) {
    wide->clear();
    if (bvh.primIds.empty()) return true;
    if (width < 2 || width > 8) return false;
    WideCollapser c{bvh, *wide, width};
    const BvhNodeOut& root = bvh.nodes[0];
    float m = 0.0f;
    for (int a = 0; a < 3; a++) m = std::max(m, std::max(std::fabs(root.lo[a]), std::fabs(root.hi[a])));
    c.eps = std::ldexp(std::max(m, 1e-30f), -18);
    if (epsOut) *epsOut = c.eps;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads > 1 && !root.leaf && (int)bvh.primIds.size() >= kCollapseParallelMin)
        return CollapseParallel(bvh, wide, width, c.eps, threads);
    wide->reserve((bvh.nodes.size() / 3 + 16) * (size_t)WideNodeFloats(width));
    if (root.leaf) {  // the root itself is a leaf: a wide root with that one leaf child
        const int w = c.NewNode();
        c.SetChild(w, 0, root.lo, root.hi, c.Leaf(root));
    } else {
        c.Node(0);
    }
    return c.ok;
}

}  // namespace ptg
