// Device binned-SAH BVH build: the same tree as BuildBinnedSah (bvh_builder.cpp) and
// as the reference's BinnedSAHBVH::Build (Core/Accel/BinnedSAHBVH.cpp:15-225), node for
// node and primitive for primitive, built level by level on the GPU.
//
// What has to match, and how it is matched:
//  - Each node sorts its primitive range by centroid along its widest centroid axis with
//    std::sort, which is unstable: equal keys end in an order set by libstdc++'s
//    introsort, and that order is inherited by the children and ends up in the leaves.
//    The sort is reproduced exactly (SortRanges): median-of-three pivot moved to the
//    front, Hoare partition rounds run in parallel for every open subrange, heapsort
//    for a subrange whose depth budget (2 floor(log2 n)) runs out, and the final
//    insertion sort, which on the partitioned arrangement equals a stable insertion
//    sort of each block the partitioning left.
//    One partition of [f, l) around the pivot p at f: let L_k be the k-th position of
//    [f+1, l) with key >= p counting up, and R_k the k-th position of [f, l) with
//    key <= p counting down. The scans swap the pairs (L_k, R_k) for k < K, where K is
//    the first k with L_k >= R_k (a missing L_k counts as +inf), and return the cut
//    min(L_K, R_{K-1}): a swapped-in element at R_{K-1} stops the final left scan.
//    Positions and ranks come from one prefix sum of the two flags.
//  - Bin assignment, bin bounds and the 16-candidate SAH cost use the reference's float
//    expressions (no contraction: the file is built with -fmad=false).
//  - Node bounds are std::min/std::max merges in range order: among equal extremes
//    (only +0 and -0 can differ) the first in order wins. Child and root bounds are
//    reduced as (value, position) pairs, first position winning, and read back from the
//    winning primitive.
//  - Node numbering: a split node's children get the next two indices and the right
//    subtree is split before the left, so the children of the inner node of rank r in
//    right-first preorder get 2r+1 and 2r+2. Ranks come from subtree inner-node counts.
// Every loop is bounded by the range sizes; an inconsistency sets an error bit and the
// build reports failure instead of returning a tree.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "bvh_builder.h"
#include "bvh_gpu.h"

namespace ptg {
namespace {

constexpr int kBins = 16;        // BinnedSAHBVH.h:174
constexpr int kLeafMax = 4;      // BinnedSAHBVH.cpp:79
constexpr int kSmallSort = 16;   // std::sort's insertion threshold (_S_threshold)
constexpr int kThreads = 256;
constexpr int kRun = 8;          // consecutive positions per thread in the run reductions
constexpr int kScanItems = 4;    // items per thread of the prefix sum
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxLevels = 4096;  // bounds the level loop (no renderable tree comes near it)

enum ErrorBits : int {
    kErrPartition = 1,  // a partition found no stop for its left scan
    kErrCut = 2,        // a cut outside its subrange
    kErrCapacity = 4,   // a table overflowed
};

// ---- float order codes: unsigned compare = float compare, -0 and +0 alike
__device__ __forceinline__ uint32_t OrderCode(float f) {
    const uint32_t u = __float_as_uint(f == 0.0f ? 0.0f : f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float FromOrderCode(uint32_t e) {
    return __uint_as_float((e & 0x80000000u) ? (e & 0x7fffffffu) : ~e);
}

// AABB::GetSurfaceArea (AABB.h:71-76)
__device__ __forceinline__ float SurfaceArea(const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ int FloorLog2(int n) { return 31 - __clz(n); }

int Blocks(long long n, int per = kThreads) { return (int)((n + per - 1) / per); }

// ---------------------------------------------------------------- primitives
// Triangle::CalcBoundary (three AABB::Merge of the vertices) and GetCentroid.
__global__ void PrimKernel(const float* __restrict__ P, const int32_t* __restrict__ idx, int T,
                           float* __restrict__ cent, float* __restrict__ box,
                           int* __restrict__ ids) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float* v[3] = {P + 3 * (size_t)idx[3 * t], P + 3 * (size_t)idx[3 * t + 1],
                         P + 3 * (size_t)idx[3 * t + 2]};
    for (int a = 0; a < 3; a++) {
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int k = 0; k < 3; k++) {
            lo = (v[k][a] < lo) ? v[k][a] : lo;  // std::min(lo, p)
            hi = (hi < v[k][a]) ? v[k][a] : hi;  // std::max(hi, p)
        }
        box[(size_t)a * T + t] = lo;
        box[(size_t)(3 + a) * T + t] = hi;
        cent[(size_t)a * T + t] = __fdiv_rn(v[0][a] + v[1][a] + v[2][a], 3.0f);
    }
    ids[t] = t;
}

// ---------------------------------------------------------------- prefix sum (int2)
// Exclusive prefix sum of n int2 values, 1024 per block; block totals are summed
// recursively and added back.
__global__ void ScanBlocks(const int2* __restrict__ in, int2* __restrict__ out,
                           int2* __restrict__ blockSums, int n) {
    __shared__ int2 warpSums[kThreads / 32];
    const int base = (blockIdx.x * kThreads + threadIdx.x) * kScanItems;
    int2 v[kScanItems];
    int2 sum = make_int2(0, 0);
    for (int j = 0; j < kScanItems; j++) {
        v[j] = base + j < n ? in[base + j] : make_int2(0, 0);
        sum.x += v[j].x;
        sum.y += v[j].y;
    }
    // inclusive scan of the per-thread sums within the warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int2 inc = sum;
    for (int d = 1; d < 32; d <<= 1) {
        const int x = __shfl_up_sync(kFull, inc.x, d), y = __shfl_up_sync(kFull, inc.y, d);
        if (lane >= d) inc.x += x, inc.y += y;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int2 w = lane < kThreads / 32 ? warpSums[lane] : make_int2(0, 0);
        for (int d = 1; d < kThreads / 32; d <<= 1) {
            const int x = __shfl_up_sync(kFull, w.x, d), y = __shfl_up_sync(kFull, w.y, d);
            if (lane >= d) w.x += x, w.y += y;
        }
        if (lane < kThreads / 32) warpSums[lane] = w;
    }
    __syncthreads();
    int2 run = make_int2(inc.x - sum.x, inc.y - sum.y);
    if (warp > 0) run.x += warpSums[warp - 1].x, run.y += warpSums[warp - 1].y;
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) out[base + j] = run;
        run.x += v[j].x;
        run.y += v[j].y;
    }
    if (threadIdx.x == kThreads - 1 && blockSums) blockSums[blockIdx.x] = run;
}

__global__ void AddBlockOffsets(int2* __restrict__ out, const int2* __restrict__ offsets, int n) {
    const int base = (blockIdx.x * kThreads + threadIdx.x) * kScanItems;
    const int2 o = offsets[blockIdx.x];
    for (int j = 0; j < kScanItems; j++)
        if (base + j < n) out[base + j].x += o.x, out[base + j].y += o.y;
}

struct ScanScratch {
    std::vector<int2*> levels;  // block sums of each recursion level
    std::vector<int> sizes;
};

void ExclusiveScan(const int2* in, int2* out, int n, const ScanScratch& sc, int level,
                   cudaStream_t s) {
    const int per = kThreads * kScanItems;
    const int nb = (n + per - 1) / per;
    int2* sums = nb > 1 ? sc.levels[level] : nullptr;
    ScanBlocks<<<nb, kThreads, 0, s>>>(in, out, sums, n);
    if (nb > 1) {
        ExclusiveScan(sums, sums, nb, sc, level + 1, s);
        AddBlockOffsets<<<nb, kThreads, 0, s>>>(out, sums, n);
    }
}

// ---------------------------------------------------------------- run reductions
// Positions are reduced into per-target accumulators where consecutive positions
// mostly share a target (a node, or a node's bin). Each thread folds kRun
// consecutive positions, flushing with atomics when the target changes; a warp whose
// positions all share one target folds across lanes first.
__device__ __forceinline__ bool WarpUniform(int target, bool single) {
    int all = 0;
    const int key = single ? target : -3 - (int)(threadIdx.x & 31);
    __match_all_sync(kFull, key, &all);
    return all != 0 && target >= 0;
}

// Centroid bounds per active node (value only).
__global__ void CentroidBoundsKernel(int T, const int* __restrict__ nodeOf,
                                     const int* __restrict__ ids, const float* __restrict__ cent,
                                     uint32_t* __restrict__ cb /* 6 per node */) {
    const long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kRun;
    int cur = -1;
    bool single = true;
    uint32_t lo[3], hi[3];
    auto flush = [&](int node) {
        for (int a = 0; a < 3; a++) {
            atomicMin(&cb[6 * node + a], lo[a]);
            atomicMax(&cb[6 * node + 3 + a], hi[a]);
        }
    };
    for (int j = 0; j < kRun; j++) {
        const long long i = base + j;
        const int t = i < T ? nodeOf[i] : -1;
        if (t != cur) {
            if (j > 0) single = false;
            if (cur >= 0) flush(cur);
            cur = t;
            for (int a = 0; a < 3; a++) lo[a] = 0xffffffffu, hi[a] = 0u;
        }
        if (t < 0) continue;
        const int p = ids[i];
        for (int a = 0; a < 3; a++) {
            const uint32_t c = OrderCode(cent[(size_t)a * T + p]);
            lo[a] = min(lo[a], c);
            hi[a] = max(hi[a], c);
        }
    }
    if (WarpUniform(cur, single)) {
        for (int a = 0; a < 3; a++) {
            lo[a] = __reduce_min_sync(kFull, lo[a]);
            hi[a] = __reduce_max_sync(kFull, hi[a]);
        }
        if ((threadIdx.x & 31) == 0) flush(cur);
    } else if (cur >= 0) {
        flush(cur);
    }
}

// Per active node: widest centroid axis, its lower bound and extent; the node's sort
// range goes to the partition list (more than 16 primitives) or the insertion list.
struct LevelNodes {
    int* tempId;  // node record of each active node
    int* begin;
    int* end;
};
struct SegList {
    int* first;
    int* last;
    int* depth;
    float* pivot;
    int* K;
    int* cut;
    int* newL;
    int* newR;
};
struct Counters {  // device words
    int nodes;      // node records allocated
    int active;     // active nodes of the next level
    int segs;       // partition subranges of the next round
    int small;      // insertion blocks
    int heap;       // heapsort subranges
    int error;
    int pad[2];
};

__global__ void NodeAxisKernel(int nActive, LevelNodes nodes, const uint32_t* __restrict__ cb,
                               int* __restrict__ axis, float* __restrict__ cbLo,
                               float* __restrict__ len, int* __restrict__ segOfNode, SegList segs,
                               int2* __restrict__ small, Counters* cnt, int segCap, int smallCap) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nActive) return;
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = FromOrderCode(cb[6 * a + k]);
        hi[k] = FromOrderCode(cb[6 * a + 3 + k]);
    }
    int ax = 0;  // AABB::GetWidestAxis (AABB.cpp:54-71)
    float best = 0.0f;
    for (int k = 0; k < 3; k++) {
        const float w = hi[k] - lo[k];
        if (w > best) best = w, ax = k;
    }
    axis[a] = ax;
    cbLo[a] = lo[ax];
    len[a] = hi[ax] - lo[ax];
    const int b = nodes.begin[a], e = nodes.end[a], n = e - b;
    segOfNode[a] = -1;
    if (n > kSmallSort) {
        const int s = atomicAdd(&cnt->segs, 1);
        if (s >= segCap) {
            atomicOr(&cnt->error, kErrCapacity);
            return;
        }
        segs.first[s] = b;
        segs.last[s] = e;
        segs.depth[s] = 2 * FloorLog2(n);
        segOfNode[a] = s;
    } else if (n >= 2) {
        const int k = atomicAdd(&cnt->small, 1);
        if (k >= smallCap) {
            atomicOr(&cnt->error, kErrCapacity);
            return;
        }
        small[k] = make_int2(b, e);
    }
}

__global__ void KeysKernel(int T, const int* __restrict__ nodeOf, const int* __restrict__ ids,
                           const float* __restrict__ cent, const int* __restrict__ axis,
                           const int* __restrict__ segOfNode, float* __restrict__ key,
                           int* __restrict__ seg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const int a = nodeOf[i];
    if (a < 0) {
        seg[i] = -1;
        return;
    }
    key[i] = cent[(size_t)axis[a] * T + ids[i]];
    seg[i] = segOfNode[a];
}

// ---------------------------------------------------------------- std::sort rounds
__device__ __forceinline__ void SwapAt(float* key, int* ids, int x, int y) {
    const float k = key[x];
    key[x] = key[y];
    key[y] = k;
    const int d = ids[x];
    ids[x] = ids[y];
    ids[y] = d;
}

// __unguarded_partition_pivot's pivot: std::__move_median_to_first(first, first + 1,
// mid, last - 1).
__global__ void PivotKernel(int nSeg, SegList segs, float* __restrict__ key, int* __restrict__ ids) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSeg) return;
    const int f = segs.first[s], l = segs.last[s];
    const int a = f + 1, b = f + (l - f) / 2, c = l - 1;
    const float ka = key[a], kb = key[b], kc = key[c];
    int m;
    if (ka < kb) {
        if (kb < kc) m = b;
        else if (ka < kc) m = c;
        else m = a;
    } else if (ka < kc) {
        m = a;
    } else if (kb < kc) {
        m = c;
    } else {
        m = b;
    }
    SwapAt(key, ids, f, m);
    segs.pivot[s] = key[f];
    segs.K[s] = INT_MAX;
}

// flags.x: position of [f+1, l) with !(key < pivot); flags.y: position of [f, l) with
// !(pivot < key). Entry T stays zero so the prefix sum holds the totals.
__global__ void FlagsKernel(int T, const int* __restrict__ seg, SegList segs,
                            const float* __restrict__ key, int2* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > T) return;
    int2 f = make_int2(0, 0);
    const int s = i < T ? seg[i] : -1;
    if (s >= 0) {
        const float pv = segs.pivot[s], k = key[i];
        f.x = (i > segs.first[s] && !(k < pv)) ? 1 : 0;
        f.y = !(pv < k) ? 1 : 0;
    }
    flags[i] = f;
}

__global__ void RanksKernel(int T, const int* __restrict__ seg, SegList segs,
                            const int2* __restrict__ pre, int* __restrict__ lpos,
                            int* __restrict__ rpos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = i < T ? seg[i] : -1;
    unsigned cand = INT_MAX;
    if (s >= 0) {
        const int f = segs.first[s], l = segs.last[s];
        const int2 pi = pre[i], pn = pre[i + 1], pl = pre[l];
        if (pn.x != pi.x) {  // a left-scan stop: rank k counting up
            const int k = pi.x - pre[f + 1].x + 1;
            lpos[f + k - 1] = i;
            const int rightAfter = pl.y - pn.y;  // right-scan stops above i
            if (rightAfter < k) cand = (unsigned)k;
        }
        if (pn.y != pi.y) {  // a right-scan stop: rank k counting down
            const int k = pl.y - pi.y;
            rpos[f + k - 1] = i;
        }
    }
    // the first stopping rank of each subrange, one atomic per subrange per warp
    const unsigned group = __match_any_sync(kFull, s);
    const unsigned m = __reduce_min_sync(group, cand);
    if (s >= 0 && m != INT_MAX && (threadIdx.x & 31) == (unsigned)(__ffs(group) - 1))
        atomicMin(&segs.K[s], (int)m);
}

__global__ void SwapKernel(int T, const int* __restrict__ seg, SegList segs,
                           const int2* __restrict__ pre, const int* __restrict__ lpos,
                           const int* __restrict__ rpos, float* __restrict__ key,
                           int* __restrict__ ids, Counters* cnt) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= T) return;
    const int s = seg[j];
    if (s < 0) return;
    const int f = segs.first[s], l = segs.last[s];
    const int k = j - f + 1;
    const int numL = pre[l].x - pre[f + 1].x;
    const int K = min(segs.K[s], numL + 1);
    if (k < K) {
        SwapAt(key, ids, lpos[f + k - 1], rpos[f + k - 1]);
    } else if (k == K) {
        int cut;
        if (K <= numL) cut = K >= 2 ? min(lpos[f + K - 1], rpos[f + K - 2]) : lpos[f];
        else if (K >= 2) cut = rpos[f + K - 2];
        else cut = -1;
        if (cut < 0) atomicOr(&cnt->error, kErrPartition);
        if (cut <= f || cut >= l) {
            atomicOr(&cnt->error, kErrCut);
            cut = f + 1;  // keeps the bookkeeping bounded; the build reports failure
        }
        segs.cut[s] = cut;
    }
}

// Children of each partitioned subrange, as __introsort_loop continues with them:
// both halves with the decremented depth; more than 16 elements and no depth left:
// heapsort; 16 or fewer: left to the final insertion sort.
__global__ void SplitSegsKernel(int nSeg, SegList segs, SegList next, int2* __restrict__ small,
                                int2* __restrict__ heap, Counters* cnt, int segCap, int smallCap,
                                int heapCap) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSeg) return;
    const int f = segs.first[s], l = segs.last[s], cut = segs.cut[s];
    const int d = segs.depth[s] - 1;
    const int lo[2] = {f, cut}, hi[2] = {cut, l};
    int idx[2] = {-1, -1};
    for (int c = 0; c < 2; c++) {
        const int n = hi[c] - lo[c];
        if (n > kSmallSort) {
            if (d == 0) {
                const int h = atomicAdd(&cnt->heap, 1);
                if (h < heapCap) heap[h] = make_int2(lo[c], hi[c]);
                else atomicOr(&cnt->error, kErrCapacity);
            } else {
                const int x = atomicAdd(&cnt->segs, 1);
                if (x < segCap) {
                    next.first[x] = lo[c];
                    next.last[x] = hi[c];
                    next.depth[x] = d;
                    idx[c] = x;
                } else {
                    atomicOr(&cnt->error, kErrCapacity);
                }
            }
        } else if (n >= 2) {
            const int x = atomicAdd(&cnt->small, 1);
            if (x < smallCap) small[x] = make_int2(lo[c], hi[c]);
            else atomicOr(&cnt->error, kErrCapacity);
        }
    }
    segs.newL[s] = idx[0];
    segs.newR[s] = idx[1];
}

__global__ void ResegKernel(int T, int* __restrict__ seg, SegList segs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const int s = seg[i];
    if (s < 0) return;
    seg[i] = i < segs.cut[s] ? segs.newL[s] : segs.newR[s];
}

// std::__partial_sort(first, last, last): __make_heap then __sort_heap, one thread per
// subrange (reached only when a subrange exhausts its depth budget).
__device__ void AdjustHeap(float* key, int* ids, int first, int hole, int len, float vk, int vi) {
    const int top = hole;
    int second = hole;
    while (second < (len - 1) / 2) {
        second = 2 * (second + 1);
        if (key[first + second] < key[first + second - 1]) second--;
        key[first + hole] = key[first + second];
        ids[first + hole] = ids[first + second];
        hole = second;
    }
    if ((len & 1) == 0 && second == (len - 2) / 2) {
        second = 2 * (second + 1);
        key[first + hole] = key[first + second - 1];
        ids[first + hole] = ids[first + second - 1];
        hole = second - 1;
    }
    int parent = (hole - 1) / 2;  // __push_heap
    while (hole > top && key[first + parent] < vk) {
        key[first + hole] = key[first + parent];
        ids[first + hole] = ids[first + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    key[first + hole] = vk;
    ids[first + hole] = vi;
}

__global__ void HeapSortKernel(int nHeap, const int2* __restrict__ heap, float* key, int* ids) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nHeap) return;
    const int first = heap[h].x, last = heap[h].y, len = last - first;
    if (len < 2) return;
    for (int parent = (len - 2) / 2;; parent--) {  // __make_heap
        AdjustHeap(key, ids, first, parent, len, key[first + parent], ids[first + parent]);
        if (parent == 0) break;
    }
    for (int end = last; end - first > 1;) {  // __sort_heap
        --end;
        const float vk = key[end];
        const int vi = ids[end];
        key[end] = key[first];
        ids[end] = ids[first];
        AdjustHeap(key, ids, first, 0, end - first, vk, vi);
    }
}

// The final insertion sort on one block the partitioning left (stable, <= 16 elements).
__global__ void InsertionKernel(int nSmall, const int2* __restrict__ small, float* key, int* ids) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nSmall) return;
    const int first = small[b].x, last = small[b].y;
    for (int i = first + 1; i < last; i++) {
        const float vk = key[i];
        const int vi = ids[i];
        int j = i;
        while (j > first && vk < key[j - 1]) {
            key[j] = key[j - 1];
            ids[j] = ids[j - 1];
            j--;
        }
        key[j] = vk;
        ids[j] = vi;
    }
}

// ---------------------------------------------------------------- bins and SAH
// Bin of a sorted position: int(nextafter(16 l / len, 0)) (BinnedSAHBVH.cpp:115-127); a
// zero-width centroid range gives NaN, read as bin 0.
__device__ __forceinline__ int BinOf(float k, float lo, float len) {
    const float l = k - lo;
    const float f = nextafterf(__fdiv_rn(16.0f * l, len), 0.0f);
    int bin = isnan(f) ? 0 : (int)f;
    return min(max(bin, 0), kBins - 1);
}

__global__ void BinsKernel(int T, const int* __restrict__ nodeOf, const int* __restrict__ ids,
                           const float* __restrict__ key, const float* __restrict__ cbLo,
                           const float* __restrict__ len, const float* __restrict__ box,
                           uint32_t* __restrict__ bins /* per node and bin: 6 codes + count */) {
    const long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kRun;
    int cur = -1;
    bool single = true;
    uint32_t lo[3], hi[3], count = 0;
    auto flush = [&](int t) {
        uint32_t* b = bins + 7 * (size_t)t;
        for (int a = 0; a < 3; a++) {
            atomicMin(&b[a], lo[a]);
            atomicMax(&b[3 + a], hi[a]);
        }
        atomicAdd(&b[6], count);
    };
    for (int j = 0; j < kRun; j++) {
        const long long i = base + j;
        const int a = i < T ? nodeOf[i] : -1;
        const int t = a < 0 ? -1 : a * kBins + BinOf(key[i], cbLo[a], len[a]);
        if (t != cur) {
            if (j > 0) single = false;
            if (cur >= 0) flush(cur);
            cur = t;
            for (int x = 0; x < 3; x++) lo[x] = 0xffffffffu, hi[x] = 0u;
            count = 0;
        }
        if (t < 0) continue;
        const int p = ids[i];
        for (int x = 0; x < 3; x++) {
            lo[x] = min(lo[x], OrderCode(box[(size_t)x * T + p]));
            hi[x] = max(hi[x], OrderCode(box[(size_t)(3 + x) * T + p]));
        }
        count++;
    }
    if (WarpUniform(cur, single)) {
        for (int x = 0; x < 3; x++) {
            lo[x] = __reduce_min_sync(kFull, lo[x]);
            hi[x] = __reduce_max_sync(kFull, hi[x]);
        }
        count = __reduce_add_sync(kFull, count);
        if ((threadIdx.x & 31) == 0) flush(cur);
    } else if (cur >= 0) {
        flush(cur);
    }
}

struct TempNodes {  // node records in allocation order
    int* begin;
    int* end;
    int* childL;  // left child record (right = left + 1), -1 for leaves
    float* box;   // 6 per record: lo.xyz, hi.xyz
};

// GetSAHCost for the 16 candidate splits (BinnedSAHBVH.cpp:229-270) and the split.
__global__ void SahKernel(int nActive, LevelNodes nodes, const uint32_t* __restrict__ bins,
                          TempNodes tn, int* __restrict__ mid, int* __restrict__ childBase,
                          Counters* cnt, int nodeCap) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nActive) return;
    float blo[kBins][3], bhi[kBins][3];
    int bc[kBins];
    for (int k = 0; k < kBins; k++) {
        const uint32_t* b = bins + 7 * ((size_t)a * kBins + k);
        for (int x = 0; x < 3; x++) {
            blo[k][x] = FromOrderCode(b[x]);
            bhi[k][x] = FromOrderCode(b[3 + x]);
        }
        bc[k] = (int)b[6];
    }
    float slo[kBins + 1][3], shi[kBins + 1][3];
    int sc[kBins + 1];
    for (int x = 0; x < 3; x++) slo[kBins][x] = FLT_MAX, shi[kBins][x] = -FLT_MAX;
    sc[kBins] = 0;
    for (int k = kBins - 1; k >= 0; k--) {
        for (int x = 0; x < 3; x++) {
            slo[k][x] = fminf(slo[k + 1][x], blo[k][x]);
            shi[k][x] = fmaxf(shi[k + 1][x], bhi[k][x]);
        }
        sc[k] = sc[k + 1] + bc[k];
    }
    float plo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, phi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int pc = 0, bestBin = 0, bestLeft = 0;
    float minCost = FLT_MAX;
    for (int k = 0; k < kBins; k++) {
        if (k > 0) {
            for (int x = 0; x < 3; x++) {
                plo[x] = fminf(plo[x], blo[k - 1][x]);
                phi[x] = fmaxf(phi[x], bhi[k - 1][x]);
            }
            pc += bc[k - 1];
        }
        const int nl = pc, nr = sc[k];
        const float sal = nl ? SurfaceArea(plo, phi) : 0.0f;
        const float sar = nr ? SurfaceArea(slo[k], shi[k]) : 0.0f;
        const float cost = __int2float_rn(nl) * sal + __int2float_rn(nr) * sar;
        if (cost < minCost) {
            minCost = cost;
            bestBin = k;
            bestLeft = nl;
        }
    }
    const int self = nodes.tempId[a];
    if (bestBin == 0) {
        mid[a] = -1;
        tn.childL[self] = -1;
        return;
    }
    const int c = atomicAdd(&cnt->nodes, 2);
    if (c + 2 > nodeCap) {
        atomicOr(&cnt->error, kErrCapacity);
        mid[a] = -1;
        tn.childL[self] = -1;
        return;
    }
    const int b = nodes.begin[a], e = nodes.end[a];
    mid[a] = b + bestLeft;
    childBase[a] = c;
    tn.childL[self] = c;
    tn.begin[c] = b;
    tn.end[c] = b + bestLeft;
    tn.begin[c + 1] = b + bestLeft;
    tn.end[c + 1] = e;
    tn.childL[c] = tn.childL[c + 1] = -1;
}

// Bounds of new node records, merged in range order: (code << 32 | position) with the
// smallest key winning for lower bounds and (code << 32 | ~position) with the largest
// for upper bounds, so among equal values the first position wins.
// root != 0: every position belongs to record 0 (accumulator 0).
__global__ void OrderedBoundsKernel(int T, int root, const int* __restrict__ nodeOf,
                                    const int* __restrict__ mid, const int* __restrict__ childBase,
                                    int recordBase, const int* __restrict__ ids,
                                    const float* __restrict__ box,
                                    unsigned long long* __restrict__ acc /* 6 per record */) {
    const long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kRun;
    int cur = -1;
    bool single = true;
    unsigned long long lo[3], hi[3];
    auto flush = [&](int t) {
        for (int a = 0; a < 3; a++) {
            atomicMin(&acc[6 * (size_t)t + a], lo[a]);
            atomicMax(&acc[6 * (size_t)t + 3 + a], hi[a]);
        }
    };
    for (int j = 0; j < kRun; j++) {
        const long long i = base + j;
        int t = -1;
        if (i < T) {
            if (root) {
                t = 0;
            } else {
                const int a = nodeOf[i];
                if (a >= 0 && mid[a] >= 0) t = childBase[a] - recordBase + (i >= mid[a] ? 1 : 0);
            }
        }
        if (t != cur) {
            if (j > 0) single = false;
            if (cur >= 0) flush(cur);
            cur = t;
            for (int a = 0; a < 3; a++) lo[a] = ~0ull, hi[a] = 0ull;
        }
        if (t < 0) continue;
        const int p = ids[i];
        for (int a = 0; a < 3; a++) {
            const unsigned long long kl =
              ((unsigned long long)OrderCode(box[(size_t)a * T + p]) << 32) | (uint32_t)i;
            const unsigned long long kh =
              ((unsigned long long)OrderCode(box[(size_t)(3 + a) * T + p]) << 32) |
              (uint32_t)(0xffffffffu - (uint32_t)i);
            lo[a] = kl < lo[a] ? kl : lo[a];
            hi[a] = kh > hi[a] ? kh : hi[a];
        }
    }
    if (WarpUniform(cur, single)) {
        for (int a = 0; a < 3; a++)
            for (int d = 16; d >= 1; d >>= 1) {
                const unsigned long long ol = __shfl_xor_sync(kFull, lo[a], d);
                const unsigned long long oh = __shfl_xor_sync(kFull, hi[a], d);
                lo[a] = ol < lo[a] ? ol : lo[a];
                hi[a] = oh > hi[a] ? oh : hi[a];
            }
        if ((threadIdx.x & 31) == 0) flush(cur);
    } else if (cur >= 0) {
        flush(cur);
    }
}

// The winning positions' own coordinates (their sign of zero included).
__global__ void ResolveBoundsKernel(int nRecords, int recordBase, int T,
                                    const unsigned long long* __restrict__ acc,
                                    const int* __restrict__ ids, const float* __restrict__ box,
                                    float* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRecords) return;
    for (int a = 0; a < 6; a++) {
        const unsigned long long k = acc[6 * (size_t)r + a];
        float v;
        if (a < 3 ? k == ~0ull : k == 0ull) {  // empty range: AABB's initial bounds
            v = a < 3 ? FLT_MAX : -FLT_MAX;
        } else {
            const uint32_t low = (uint32_t)(k & 0xffffffffu);
            const int pos = a < 3 ? (int)low : (int)(0xffffffffu - low);
            v = box[(size_t)a * T + ids[pos]];
        }
        out[6 * (size_t)(recordBase + r) + a] = v;
    }
}

// Active nodes of the next level: children with more than four primitives.
__global__ void NextLevelKernel(int nActive, const int* __restrict__ mid,
                                const int* __restrict__ childBase, TempNodes tn,
                                LevelNodes next, int* __restrict__ childActive /* 2 per node */,
                                Counters* cnt, int activeCap) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nActive) return;
    childActive[2 * a] = childActive[2 * a + 1] = -1;
    if (mid[a] < 0) return;
    for (int c = 0; c < 2; c++) {
        const int r = childBase[a] + c;
        if (tn.end[r] - tn.begin[r] <= kLeafMax) continue;
        const int x = atomicAdd(&cnt->active, 1);
        if (x >= activeCap) {
            atomicOr(&cnt->error, kErrCapacity);
            continue;
        }
        next.tempId[x] = r;
        next.begin[x] = tn.begin[r];
        next.end[x] = tn.end[r];
        childActive[2 * a + c] = x;
    }
}

__global__ void NodeOfKernel(int T, int* __restrict__ nodeOf, const int* __restrict__ mid,
                             const int* __restrict__ childActive) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const int a = nodeOf[i];
    if (a < 0) return;
    nodeOf[i] = mid[a] < 0 ? -1 : childActive[2 * a + (i >= mid[a] ? 1 : 0)];
}

// ---------------------------------------------------------------- numbering
__global__ void InnerCountKernel(int r0, int r1, TempNodes tn, int* __restrict__ ic) {
    const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= r1) return;
    const int c = tn.childL[r];
    ic[r] = c < 0 ? 0 : 1 + ic[c] + ic[c + 1];
}

struct OutNode {  // BvhNodeOut's layout
    float lo[3], hi[3];
    int32_t child[2];
    int32_t begin, end;
    bool leaf;
};

__global__ void NumberKernel(int r0, int r1, TempNodes tn, const int* __restrict__ ic,
                             int* __restrict__ index, int* __restrict__ rank,
                             OutNode* __restrict__ out) {
    const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= r1) return;
    const int at = index[r];
    OutNode o;
    for (int a = 0; a < 3; a++) {
        o.lo[a] = tn.box[6 * (size_t)r + a];
        o.hi[a] = tn.box[6 * (size_t)r + 3 + a];
    }
    o.begin = tn.begin[r];
    o.end = tn.end[r];
    const int c = tn.childL[r];
    if (c < 0) {
        o.leaf = true;
        o.child[0] = o.child[1] = at == 0 ? 0 : -1;
    } else {
        const int k = rank[r];
        o.leaf = false;
        o.child[0] = 2 * k + 1;
        o.child[1] = 2 * k + 2;
        index[c] = 2 * k + 1;
        index[c + 1] = 2 * k + 2;
        rank[c + 1] = k + 1;               // the right subtree is numbered first
        rank[c] = k + 1 + ic[c + 1];
    }
    out[at] = o;
}

// Accumulator initialisation: groups of `stride` words, the first three lower-bound
// codes (all ones), the rest zero (upper-bound codes and counts).
__global__ void InitCodes(uint32_t* __restrict__ p, int groups, int stride) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= groups) return;
    for (int k = 0; k < stride; k++) p[(size_t)g * stride + k] = k < 3 ? 0xffffffffu : 0u;
}
__global__ void InitBounds64(unsigned long long* __restrict__ p, int groups) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= groups) return;
    for (int k = 0; k < 6; k++) p[6 * (size_t)g + k] = k < 3 ? ~0ull : 0ull;
}
__global__ void ResetCounters(Counters* c, int segs, int small, int heap, int active) {
    if (segs) c->segs = 0;
    if (small) c->small = 0;
    if (heap) c->heap = 0;
    if (active) c->active = 0;
}

// ---------------------------------------------------------------- host driver
struct Arena {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class X>
    X* Get(size_t n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(X));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<X*>(p);
    }
    ~Arena() {
        for (void* p : ptrs) cudaFree(p);
    }
};

}  // namespace

static_assert(sizeof(OutNode) == sizeof(BvhNodeOut), "node layout");
static_assert(offsetof(OutNode, leaf) == offsetof(BvhNodeOut, leaf), "node layout");
static_assert(offsetof(OutNode, begin) == offsetof(BvhNodeOut, begin), "node layout");

cudaError_t BuildBinnedSahDevice(const float* positions, int numVertices, const int32_t* indices,
                                 int T, cudaStream_t s, BvhResult* out, std::string* error,
                                 DeviceBuildStats* stats) {
    *out = BvhResult{};
    if (T <= 0) {  // the reference's empty tree: one leaf root with empty bounds
        BvhNodeOut root{};
        for (int a = 0; a < 3; a++) root.lo[a] = FLT_MAX, root.hi[a] = -FLT_MAX;
        root.child[0] = root.child[1] = 0;
        root.begin = root.end = 0;
        root.leaf = true;
        out->nodes.push_back(root);
        return cudaSuccess;
    }
    Arena ar;
    const size_t t = (size_t)T;
    const int nodeCap = 2 * T;
    const int activeCap = T / (kLeafMax + 1) + 1;
    const int segCap = T / (kSmallSort + 1) + 1;
    const int smallCap = T / 2 + 1;
    const int heapCap = segCap;
    float* dPos = ar.Get<float>(3 * (size_t)numVertices);
    int32_t* dIdx = ar.Get<int32_t>(3 * t);
    float* cent = ar.Get<float>(3 * t);
    float* box = ar.Get<float>(6 * t);
    int* ids = ar.Get<int>(t);
    float* key = ar.Get<float>(t);
    int* nodeOf = ar.Get<int>(t);
    int* seg = ar.Get<int>(t);
    int2* flags = ar.Get<int2>(t + 1);
    int2* pre = ar.Get<int2>(t + 1);
    int* lpos = ar.Get<int>(t);
    int* rpos = ar.Get<int>(t);
    TempNodes tn{ar.Get<int>(nodeCap), ar.Get<int>(nodeCap), ar.Get<int>(nodeCap),
                 ar.Get<float>(6 * (size_t)nodeCap)};
    LevelNodes lv[2];
    for (auto& l : lv) l = LevelNodes{ar.Get<int>(activeCap), ar.Get<int>(activeCap), ar.Get<int>(activeCap)};
    uint32_t* cb = ar.Get<uint32_t>(6 * (size_t)activeCap);
    int* axis = ar.Get<int>(activeCap);
    float* cbLo = ar.Get<float>(activeCap);
    float* len = ar.Get<float>(activeCap);
    int* segOfNode = ar.Get<int>(activeCap);
    uint32_t* bins = ar.Get<uint32_t>(7 * (size_t)kBins * activeCap);
    int* mid = ar.Get<int>(activeCap);
    int* childBase = ar.Get<int>(activeCap);
    int* childActive = ar.Get<int>(2 * (size_t)activeCap);
    unsigned long long* acc = ar.Get<unsigned long long>(6 * 2 * (size_t)activeCap + 6);
    SegList sl[2];
    for (auto& l : sl)
        l = SegList{ar.Get<int>(segCap), ar.Get<int>(segCap), ar.Get<int>(segCap), ar.Get<float>(segCap),
                    ar.Get<int>(segCap), ar.Get<int>(segCap), ar.Get<int>(segCap), ar.Get<int>(segCap)};
    int2* small = ar.Get<int2>(smallCap);
    int2* heap = ar.Get<int2>(heapCap);
    Counters* cnt = ar.Get<Counters>(1);
    int* ic = ar.Get<int>(nodeCap);
    int* index = ar.Get<int>(nodeCap);
    int* rank = ar.Get<int>(nodeCap);
    OutNode* outNodes = ar.Get<OutNode>(nodeCap);
    ScanScratch scan;
    for (long long n = t + 1; n > kThreads * kScanItems;) {
        n = (n + kThreads * kScanItems - 1) / (kThreads * kScanItems);
        scan.levels.push_back(ar.Get<int2>(n));
        scan.sizes.push_back((int)n);
    }
    Counters* hc = nullptr;
    if (ar.err == cudaSuccess) ar.err = cudaMallocHost(&hc, sizeof(Counters));
    if (ar.err != cudaSuccess) {
        if (error) *error = "device BVH build: allocation failed";
        if (hc) cudaFreeHost(hc);
        return ar.err;
    }
    struct HostFree {
        Counters* p;
        ~HostFree() { cudaFreeHost(p); }
    } hf{hc};
    struct Events {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Events() {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } ev;
    cudaEvent_t& e0 = ev.e0;
    cudaEvent_t& e1 = ev.e1;
    if (stats) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
    }
    int launches = 0, rounds = 0, levels = 0, heapsorts = 0;
    auto fetch = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(hc, cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e;
    };
    auto fail = [&](const char* what) {
        if (error) *error = std::string("device BVH build: ") + what;
        return cudaErrorUnknown;
    };

    cudaMemcpyAsync(dPos, positions, 3 * (size_t)numVertices * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dIdx, indices, 3 * t * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(cnt, 0, sizeof(Counters), s);
    PrimKernel<<<Blocks(T), kThreads, 0, s>>>(dPos, dIdx, T, cent, box, ids);
    // the root record: all primitives in their input order
    {
        const int one[2] = {0, T};
        const int none = -1;
        cudaMemcpyAsync(tn.begin, &one[0], sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(tn.end, &one[1], sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(tn.childL, &none, sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(acc, 0xff, 3 * sizeof(unsigned long long), s);
        cudaMemsetAsync(acc + 3, 0, 3 * sizeof(unsigned long long), s);
        OrderedBoundsKernel<<<Blocks(T, kThreads * kRun), kThreads, 0, s>>>(
          T, 1, nodeOf, mid, childBase, 0, ids, box, acc);
        ResolveBoundsKernel<<<1, 32, 0, s>>>(1, 0, T, acc, ids, box, tn.box);
        launches += 3;
    }
    const int oneNode = 1;
    cudaMemcpyAsync(&cnt->nodes, &oneNode, sizeof(int), cudaMemcpyHostToDevice, s);
    std::vector<int> levelStart = {0, 1};
    int nActive = 0;
    if (T > kLeafMax) {
        const int rootRec[3] = {0, 0, T};
        cudaMemcpyAsync(lv[0].tempId, &rootRec[0], sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(lv[0].begin, &rootRec[1], sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(lv[0].end, &rootRec[2], sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(nodeOf, 0, t * sizeof(int), s);
        nActive = 1;
    }
    int cur = 0;
    int nodesTotal = 1;
    while (nActive > 0) {
        if (++levels > kMaxLevels) return fail("tree deeper than 4096 levels");
        LevelNodes& L = lv[cur];
        LevelNodes& N = lv[cur ^ 1];
        // centroid bounds, widest axis, sort keys; node ranges become sort subranges
        InitCodes<<<Blocks(nActive), kThreads, 0, s>>>(cb, nActive, 6);
        ResetCounters<<<1, 1, 0, s>>>(cnt, 1, 1, 1, 1);
        CentroidBoundsKernel<<<Blocks(T, kThreads * kRun), kThreads, 0, s>>>(T, nodeOf, ids, cent, cb);
        NodeAxisKernel<<<Blocks(nActive), kThreads, 0, s>>>(nActive, L, cb, axis, cbLo, len, segOfNode,
                                                          sl[0], small, cnt, segCap, smallCap);
        KeysKernel<<<Blocks(T), kThreads, 0, s>>>(T, nodeOf, ids, cent, axis, segOfNode, key, seg);
        launches += 5;
        cudaError_t e = fetch();
        if (e != cudaSuccess) return e;
        int nSeg = hc->segs, sc = 0;
        // std::sort of every node range: partition rounds over all open subranges
        while (nSeg > 0 && hc->error == 0) {
            rounds++;
            SegList& S = sl[sc];
            SegList& X = sl[sc ^ 1];
            PivotKernel<<<Blocks(nSeg), kThreads, 0, s>>>(nSeg, S, key, ids);
            FlagsKernel<<<Blocks(T + 1), kThreads, 0, s>>>(T, seg, S, key, flags);
            ExclusiveScan(flags, pre, T + 1, scan, 0, s);
            RanksKernel<<<Blocks(T), kThreads, 0, s>>>(T, seg, S, pre, lpos, rpos);
            SwapKernel<<<Blocks(T), kThreads, 0, s>>>(T, seg, S, pre, lpos, rpos, key, ids, cnt);
            ResetCounters<<<1, 1, 0, s>>>(cnt, 1, 0, 0, 0);
            SplitSegsKernel<<<Blocks(nSeg), kThreads, 0, s>>>(nSeg, S, X, small, heap, cnt, segCap,
                                                             smallCap, heapCap);
            ResegKernel<<<Blocks(T), kThreads, 0, s>>>(T, seg, S);
            launches += 8 + 2 * (int)scan.levels.size() + 1;
            if ((e = fetch()) != cudaSuccess) return e;
            nSeg = hc->segs;
            sc ^= 1;
        }
        if (hc->error) break;
        heapsorts += hc->heap;
        if (hc->heap > 0) {
            HeapSortKernel<<<Blocks(hc->heap, 64), 64, 0, s>>>(hc->heap, heap, key, ids);
            launches++;
        }
        if (hc->small > 0) {
            InsertionKernel<<<Blocks(hc->small), kThreads, 0, s>>>(hc->small, small, key, ids);
            launches++;
        }
        // bins and the SAH split of every active node
        InitCodes<<<Blocks((long long)nActive * kBins), kThreads, 0, s>>>(bins, nActive * kBins, 7);
        BinsKernel<<<Blocks(T, kThreads * kRun), kThreads, 0, s>>>(T, nodeOf, ids, key, cbLo, len, box, bins);
        SahKernel<<<Blocks(nActive), kThreads, 0, s>>>(nActive, L, bins, tn, mid, childBase, cnt, nodeCap);
        launches += 3;
        if ((e = fetch()) != cudaSuccess) return e;
        if (hc->error) break;
        const int recordBase = nodesTotal, nRecords = hc->nodes - recordBase;
        nodesTotal = hc->nodes;
        if (nRecords > 0) {
            InitBounds64<<<Blocks(nRecords), kThreads, 0, s>>>(acc, nRecords);
            OrderedBoundsKernel<<<Blocks(T, kThreads * kRun), kThreads, 0, s>>>(
              T, 0, nodeOf, mid, childBase, recordBase, ids, box, acc);
            ResolveBoundsKernel<<<Blocks(nRecords), kThreads, 0, s>>>(nRecords, recordBase, T, acc, ids,
                                                                   box, tn.box);
            levelStart.push_back(nodesTotal);
            launches += 3;
        }
        ResetCounters<<<1, 1, 0, s>>>(cnt, 0, 0, 0, 1);
        NextLevelKernel<<<Blocks(nActive), kThreads, 0, s>>>(nActive, mid, childBase, tn, N, childActive,
                                                           cnt, activeCap);
        NodeOfKernel<<<Blocks(T), kThreads, 0, s>>>(T, nodeOf, mid, childActive);
        launches += 3;
        if ((e = fetch()) != cudaSuccess) return e;
        if (hc->error) break;
        nActive = hc->active;
        cur ^= 1;
    }
    if (hc->error) {
        const int bits = hc->error;
        return fail(bits & kErrCapacity ? "table capacity exceeded"
                                        : bits & kErrCut ? "partition cut outside its range"
                                                         : "partition without a stop");
    }
    // numbering: inner-node counts bottom-up, right-first preorder ranks top-down
    const int numLevels = (int)levelStart.size() - 1;
    for (int l = numLevels - 1; l >= 0; l--) {
        const int r0 = levelStart[l], r1 = levelStart[l + 1];
        InnerCountKernel<<<Blocks(r1 - r0), kThreads, 0, s>>>(r0, r1, tn, ic);
    }
    cudaMemsetAsync(index, 0, sizeof(int), s);
    cudaMemsetAsync(rank, 0, sizeof(int), s);
    for (int l = 0; l < numLevels; l++) {
        const int r0 = levelStart[l], r1 = levelStart[l + 1];
        NumberKernel<<<Blocks(r1 - r0), kThreads, 0, s>>>(r0, r1, tn, ic, index, rank, outNodes);
    }
    launches += 2 * numLevels;
    out->nodes.resize(nodesTotal);
    out->primIds.resize(t);
    cudaMemcpyAsync(out->nodes.data(), outNodes, (size_t)nodesTotal * sizeof(OutNode),
                    cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out->primIds.data(), ids, t * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (stats) cudaEventRecord(e1, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        *out = BvhResult{};
        if (error) *error = std::string("device BVH build: ") + cudaGetErrorString(e);
        return e;
    }
    out->height = numLevels - 1;
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms = ms;
        stats->levels = levels;
        stats->rounds = rounds;
        stats->heapsorts = heapsorts;
        stats->launches = launches;
    }
    return cudaSuccess;
}

}  // namespace ptg
