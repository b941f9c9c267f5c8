// Host binned-SAH BVH builder.
//
// Produces the same tree as the reference's BinnedSAHBVH::Build
// (Core/Accel/BinnedSAHBVH.cpp:15-225): same 16-bin SAH over centroid bins of
// the widest centroid axis, the same std::sort of each node's primitive range,
// the same leaf rule (<= 4 primitives, or best split at bin 0) and the same node
// numbering (children appended in pairs, right subtree numbered before the left).
// It differs in how it gets there: one binning pass per node instead of 16 cost
// passes, and independent subtrees built on several threads, with the node
// numbers assigned in a final depth-first pass.
#pragma once
#include <cstdint>
#include <vector>

namespace ptg {

struct BvhNodeOut {
    float lo[3], hi[3];
    int32_t child[2];  // -1 -1 for leaves (children are always consecutive)
    int32_t begin, end;
    bool leaf;
};

struct BvhResult {
    std::vector<BvhNodeOut> nodes;
    std::vector<int32_t> primIds;
    int height = 0;  // longest root-to-leaf edge count
};

// Collapses the binary tree into `width`-wide nodes (width 4: 32 floats, width 8:
// 64 floats each; layout in pt_layout.h): each wide node takes a binary node's
// children and repeatedly opens the largest-area inner child until it has `width`.
// Leaves of more than 63 primitives become chains of leaf chunks. Returns false if
// a leaf starts beyond the 2^25 slots the child code can hold.
// epsOut: the widening of every child box (each side moves out by it). threads <= 0:
// hardware concurrency; the result does not depend on the thread count (node for node
// and bit for bit), nor does it on whether the collapse runs on one thread (small trees).
bool CollapseWide(const BvhResult& bvh, std::vector<float>* wide, int width = 4,
                  float* epsOut = nullptr, int threads = 0);
constexpr int kWideLeafMax = 63;
// Floats per wide node of the given width (6 bounds + 1 code per child, padded to
// whole 128-byte lines).
constexpr int WideNodeFloats(int width) { return ((7 * width + 31) / 32) * 32; }

// positions: V x 3 floats; indices: T x 3. threads <= 0: hardware concurrency.
BvhResult BuildBinnedSah(const float* positions, const int32_t* indices, int numTriangles,
                         int threads);

}  // namespace ptg
