// The throughput traversal's wide BVH (CollapseWide, csrc/bvh_builder.h) checked on the
// host: builds the binned-SAH tree of a triangle soup, collapses it, and walks the wide
// tree from its root.
//
// usage: wide_bvh <soup file> <width>; the file holds int32 V, int32 T, V*3 float
// positions, T*3 int32 indices. Prints "ok nodes=<n> leaves=<n> maxleaf=<n> eps=<e>" or
// the first violation found:
// - every node is reached from the root exactly once;
// - an empty slot (code INT32_MIN) has a box at +infinity on all six planes, and only
//   trailing slots are empty;
// - an inner slot's box holds the boxes of its node's used slots;
// - a leaf slot (code -((first << 6) | count) - 1) holds 1..63 primitives, and its box
//   holds their vertices;
// - every primitive slot is in exactly one leaf;
// - the widening is 2^-18 of the root's largest coordinate;
// - the collapse on 2, 3, 8 and 16 threads gives the same array, bit for bit.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>

#include "bvh_builder.h"

static int Fail(const char* what, long a, long b) {
    std::printf("violation: %s (%ld, %ld)\n", what, a, b);
    return 1;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t V = 0, T = 0;
    if (std::fread(&V, 4, 1, f) != 1 || std::fread(&T, 4, 1, f) != 1 || V < 0 || T < 0) return 2;
    std::vector<float> pos((size_t)V * 3);
    std::vector<int32_t> idx((size_t)T * 3);
    if (std::fread(pos.data(), 4, pos.size(), f) != pos.size() ||
        std::fread(idx.data(), 4, idx.size(), f) != idx.size())
        return 2;
    std::fclose(f);
    const int K = std::atoi(argv[2]);
    const ptg::BvhResult b = ptg::BuildBinnedSah(pos.data(), idx.data(), T, 0);
    std::vector<float> wide;
    float eps = 0.0f;
    if (!ptg::CollapseWide(b, &wide, K, &eps, 1)) return Fail("collapse refused", T, K);
    // the collapse on several threads gives the same array, bit for bit
    for (int threads : {2, 3, 8, 16}) {
        std::vector<float> par;
        float e2 = 0.0f;
        if (!ptg::CollapseWide(b, &par, K, &e2, threads)) return Fail("parallel collapse refused", T, threads);
        if (par.size() != wide.size()) return Fail("parallel collapse size", (long)par.size(), (long)wide.size());
        if (e2 != eps || std::memcmp(par.data(), wide.data(), wide.size() * sizeof(float)) != 0)
            return Fail("parallel collapse differs", threads, 0);
    }
    const int nf = ptg::WideNodeFloats(K);
    const long numWide = (long)(wide.size() / nf);
    if (numWide < 1) return Fail("no wide nodes", T, 0);
    const ptg::BvhNodeOut& root = b.nodes[0];
    float m = 0.0f;
    for (int a = 0; a < 3; a++) m = std::fmax(m, std::fmax(std::fabs(root.lo[a]), std::fabs(root.hi[a])));
    if (eps != std::ldexp(std::fmax(m, 1e-30f), -18)) return Fail("widening", 0, 0);
    const float inf = std::numeric_limits<float>::infinity();
    std::vector<int> seen(numWide, 0), covered(T, 0);
    long leaves = 0, maxLeaf = 0;
    std::vector<long> stack{0};
    seen[0] = 1;
    auto box = [&](long w, int i, int a) { return wide[(size_t)w * nf + (size_t)K * a + i]; };
    auto code = [&](long w, int i) {
        int32_t c;
        std::memcpy(&c, &wide[(size_t)w * nf + 6 * K + i], 4);
        return c;
    };
    while (!stack.empty()) {
        const long w = stack.back();
        stack.pop_back();
        bool emptySeen = false;
        for (int i = 0; i < K; i++) {
            const int32_t c = code(w, i);
            if (c == INT32_MIN) {
                for (int a = 0; a < 6; a++)
                    if (box(w, i, a) != inf) return Fail("empty slot box not at +infinity", w, i);
                emptySeen = true;
                continue;
            }
            if (emptySeen) return Fail("used slot after an empty one", w, i);
            for (int a = 0; a < 3; a++)
                if (!(box(w, i, a) <= box(w, i, 3 + a))) return Fail("inverted box", w, i);
            if (c >= 0) {
                if (c >= numWide) return Fail("node code out of range", w, c);
                if (seen[c]++) return Fail("node reached twice", w, c);
                for (int j = 0; j < K; j++) {
                    if (code(c, j) == INT32_MIN) continue;
                    for (int a = 0; a < 3; a++)
                        if (box(c, j, a) < box(w, i, a) || box(c, j, 3 + a) > box(w, i, 3 + a))
                            return Fail("child box outside its slot", w, i);
                }
                stack.push_back(c);
            } else {
                const int32_t v = -(c + 1);
                const int first = v >> 6, count = v & 63;
                if (count < 1 || first + count > T) return Fail("leaf range", first, count);
                leaves++;
                if (count > maxLeaf) maxLeaf = count;
                for (int k = first; k < first + count; k++) {
                    if (covered[k]++) return Fail("primitive slot in two leaves", k, 0);
                    const int t = b.primIds[k];
                    for (int e = 0; e < 3; e++) {
                        const float* p = &pos[(size_t)idx[(size_t)t * 3 + e] * 3];
                        for (int a = 0; a < 3; a++)
                            if (p[a] < box(w, i, a) || p[a] > box(w, i, 3 + a))
                                return Fail("vertex outside its leaf box", k, a);
                    }
                }
            }
        }
    }
    for (long w = 0; w < numWide; w++)
        if (!seen[w]) return Fail("node not reached", w, 0);
    for (int k = 0; k < T; k++)
        if (covered[k] != 1) return Fail("primitive slot not in a leaf", k, covered[k]);
    std::printf("ok nodes=%ld leaves=%ld maxleaf=%ld eps=%.9g\n", numWide, leaves, maxLeaf, eps);
    return 0;
}
