// Wavefront throughput path: raygen -> extend -> shade -> shadow -> accumulate.
//
// One wave is a set of work units (a job's sample block over all its pixels),
// from one image or many (batched renders and the serving loop share the same
// kernels: every path carries its job index). Each bounce runs three
// persistent-grid kernels over compacted queues:
//   extend : closest hit of every queued ray (binary BVH, 32 B nodes, both
//            children's boxes fetched as one 64 B pair, ordered short stack)
//   shade  : miss / emission / surface handling of PathTracing or
//            SimplePathTracing semantics; next-event rays go to the shadow queue,
//            continuation rays to the next ray queue (warp-aggregated appends)
//   shadow : visibility of the next-event rays, adds their radiance
// A path's radiance lives in its own slot and is added to the pixel's running
// sum in sample order after the wave, so results do not depend on batching.
// Random numbers are a counter-based stream per (seed, pixel, sample).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <utility>
#include <vector>

#include "pt_device.cuh"
#include "pt_kernels.h"

namespace ptg {

// Minimum resident blocks per SM requested from the register allocator for the
// trace (extend/shadow) and shade stages; 1 leaves the choice to the compiler.
#ifndef PT_TRACE_MIN_BLOCKS
#define PT_TRACE_MIN_BLOCKS 8
#endif
#ifndef PT_SHADE_MIN_BLOCKS
#define PT_SHADE_MIN_BLOCKS 1
#endif

enum : int { kFlagNoSignCheck = 1 };
enum : int { kShadowEnv = 0, kShadowArea = 1 };

__device__ __forceinline__ void PixelOfIndex(int q, int W, int H, int rows, int& x, int& y) {
    // bands of `rows` rows, column-major inside a band: with 8 rows a warp covers a
    // 4 x 8 pixel block
    const int band = q / (rows * W);
    const int y0 = band * rows;
    const int hb = min(rows, H - y0);
    const int r = q - band * rows * W;
    x = r / hb;
    y = y0 + r % hb;
}

// Three-input maximum and minimum (max.f32 / min.f32 with three sources, sm_100 and
// later); a NaN operand is ignored, as by fmaxf / fminf.
__device__ __forceinline__ float Max3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float Min3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Box test against [tmin, tmax]; returns the entry distance. Each plane distance is
// one fused multiply-add, plane * inv - oi with oi = o * inv. Its rounding
// (a few units in the last place of the origin's and the distance's coordinates) is
// far inside the 2^-18 widening of the child boxes, so no hit box is missed.
__device__ __forceinline__ bool SlabFast(float4 a, float4 b, V3 oi, V3 inv, float tmin, float tmax,
                                         float& tEnter) {
    const float tx0 = fmaf(a.x, inv.x, -oi.x), tx1 = fmaf(a.w, inv.x, -oi.x);
    const float ty0 = fmaf(a.y, inv.y, -oi.y), ty1 = fmaf(b.x, inv.y, -oi.y);
    const float tz0 = fmaf(a.z, inv.z, -oi.z), tz1 = fmaf(b.y, inv.z, -oi.z);
    const float tn = Max3(fminf(tx0, tx1), fminf(ty0, ty1), fmaxf(fminf(tz0, tz1), tmin));
    const float tf = Min3(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fminf(fmaxf(tz0, tz1), tmax));
    tEnter = tn;
    return tn <= tf;
}

__device__ __forceinline__ int WarpAppend(int* counter, bool pred) {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, pred);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(active) - 1;
    int base = 0;
    if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(active, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------- persistent tracer
// Warp-persistent traversal with dynamic ray fetch: each warp pulls rays from a
// queue counter and refills its idle lanes whenever a quarter of the warp has
// finished, so long rays do not hold a warp of finished lanes (the load
// imbalance of incoherent secondary rays). One node visit per loop iteration.
constexpr unsigned kFullMask = 0xffffffffu;
#ifndef PT_REFILL_LANES
#define PT_REFILL_LANES 8
#endif
constexpr int kRefillLanes = PT_REFILL_LANES;

struct LaneRay {
    V3 o, d, inv;
    float tmin, tmax, tBest;
    int best;  // slot of the closest hit; -1 none; -2 - slot when another hit tied it
    bool anyHit;
    const float4* nodes;  // the lane's 4-wide tree (rays of different jobs share a warp)
    const float4* tris;
#if PT_CHECK
    int numWide, numTris;  // bounds of nodes and tris, tested before every access
#endif
};

__device__ __forceinline__ void SortPair(float& ta, int& ca, float& tb, int& cb) {
    if (tb < ta) {
        const float t = ta;
        ta = tb;
        tb = t;
        const int c = ca;
        ca = cb;
        cb = c;
    }
}

// Entries of the traversal stack kept in shared memory per thread; deeper ones go
// to local memory. Shared entries are entry-major with one column per thread of
// the 128-thread block, so a warp's accesses always fall in 32 distinct banks.
#ifndef PT_SMEM_STACK
#define PT_SMEM_STACK 16
#endif
// 1: a warp steps every lane through inner nodes until it reaches a leaf, then
// intersects the lanes' leaves together; 0: one node or leaf per lane per step.
// Both visit the same nodes and leaves in the same order for every ray.
#ifndef PT_WHILE_WHILE
#define PT_WHILE_WHILE 1
#endif
constexpr int kTraceBlock = 128;
constexpr int kSmemStack = PT_SMEM_STACK;
constexpr int kDone = INT_MIN;  // no further item (never a child code of a visited slot)

struct TravStack {
    int2* ent;   // shared, kSmemStack x kTraceBlock {code, entry distance bits}: closest hit
    int* code;   // shared, kSmemStack x kTraceBlock codes: any-hit (no distances)
    int2 deep[kWaveStackDepth - kSmemStack > 0 ? kWaveStackDepth - kSmemStack : 1];
    int sp;
    __device__ __forceinline__ void Push(int c, float t) {
        const int2 e = make_int2(c, __float_as_int(t));  // one 8-byte store
        if (sp < kSmemStack) ent[sp * kTraceBlock + threadIdx.x] = e;
        else deep[sp - kSmemStack] = e;
        sp++;
    }
    // Any-hit rays: entries without distances (nothing is culled before the first hit,
    // which ends the ray).
    __device__ __forceinline__ void PushCode(int c) {
        if (sp < kSmemStack) code[sp * kTraceBlock + threadIdx.x] = c;
        else deep[sp - kSmemStack].x = c;
        sp++;
    }
    __device__ __forceinline__ int PopCode() {
        if (sp == 0) return kDone;
        --sp;
        return sp < kSmemStack ? code[sp * kTraceBlock + threadIdx.x] : deep[sp - kSmemStack].x;
    }
    // Next entry whose box starts no farther than tBest, or kDone.
    __device__ __forceinline__ int Pop(float tBest) {
        while (sp > 0) {
            --sp;
            const int2 e = sp < kSmemStack ? ent[sp * kTraceBlock + threadIdx.x] : deep[sp - kSmemStack];
            if (__int_as_float(e.y) <= tBest) return e.x;
        }
        return kDone;
    }
};

// Tests the triangles of leaf `cur`; returns true when an any-hit ray is done.
// Otherwise `cur` becomes the next item from the stack (or kDone).
// kAnyHit: every ray of the queue is an any-hit ray (known at compile time).
template <bool kAnyHit>
__device__ __forceinline__ bool VisitLeaf(LaneRay& r, TravStack& stk, int& cur, int& err) {
    const int v = -cur - 1;
    const int first = v >> 6, cnt = v & 63;
#if PT_CHECK
    if (first < 0 || first + cnt > r.numTris) {
        err |= kErrBounds;
        cur = kDone;
        return true;
    }
#endif
    for (int k = first; k < first + cnt; k++) {
        V3 v0, e1, e2;
        LoadTri(r.tris, k, v0, e1, e2);
        float t;
        if (TriIntersect(v0, e1, e2, r.o, r.d, t) && t >= r.tmin && t <= r.tmax) {
            if (t < r.tBest) {
                r.tBest = t;
                r.best = k;
                if (kAnyHit || r.anyHit) return true;
            } else if (t == r.tBest && r.best >= 0) {
                r.best = -2 - r.best;  // an exact tie: settled by the reference's order
            }
        }
    }
    cur = kAnyHit ? stk.PopCode() : stk.Pop(r.tBest);
    return false;
}

// Tests the children of wide node `cur`; `cur` becomes the nearest hit child and
// the other hit children are pushed farthest first (or the next stack item).
// kAnyHit: only the nearest child is picked out; the others are pushed in slot order
// (an any-hit ray ends at its first hit, and whether it hits does not depend on the
// order its boxes are visited in).
template <bool kAnyHit>
__device__ __forceinline__ void VisitInner(LaneRay& r, TravStack& stk, int& cur, int& err) {
    constexpr int K = kWide, Q = kWide / 4;
#if PT_CHECK
    if ((unsigned)cur >= (unsigned)r.numWide) {
        err |= kErrBounds;
        cur = kDone;
        return;
    }
#endif
    const float4* n = r.nodes + (kWideFloats / 4) * (size_t)cur;
    float b[6][K];
#pragma unroll
    for (int a = 0; a < 6; a++)
#pragma unroll
        for (int j = 0; j < Q; j++) {
            const float4 v = __ldg(n + a * Q + j);
            b[a][4 * j] = v.x;
            b[a][4 * j + 1] = v.y;
            b[a][4 * j + 2] = v.z;
            b[a][4 * j + 3] = v.w;
        }
    int c[K];
#pragma unroll
    for (int j = 0; j < Q; j++) {
        const int4 v = __ldg(reinterpret_cast<const int4*>(n + 6 * Q + j));
        c[4 * j] = v.x;
        c[4 * j + 1] = v.y;
        c[4 * j + 2] = v.z;
        c[4 * j + 3] = v.w;
    }
    const float inf = __int_as_float(0x7f800000);
    const V3 oi = r.o * r.inv;
    float t[K];
#pragma unroll
    for (int i = 0; i < K; i++) {
        float te;
        // an empty slot's box lies at +infinity on every plane and is never hit
        t[i] = SlabFast(make_float4(b[0][i], b[1][i], b[2][i], b[3][i]),
                        make_float4(b[4][i], b[5][i], 0.f, 0.f), oi, r.inv, 0.0f, r.tBest, te)
                 ? te
                 : inf;
    }
    if (kAnyHit && K == 4) {
        // the nearest into slot 0
        SortPair(t[0], c[0], t[1], c[1]);
        SortPair(t[2], c[2], t[3], c[3]);
        SortPair(t[0], c[0], t[2], c[2]);
        if (t[0] == inf) {
            cur = stk.PopCode();
            return;
        }
        if (stk.sp > kWaveStackDepth - (K - 1)) {  // room for K - 1 pushes
            err |= kErrStackOverflow;
            cur = kDone;
            return;
        }
#pragma unroll
        for (int i = K - 1; i >= 1; i--)
            if (t[i] != inf) stk.PushCode(c[i]);
        cur = c[0];
        return;
    }
    // sorting network, nearest first
    if (K == 4) {
        SortPair(t[0], c[0], t[1], c[1]);
        SortPair(t[2], c[2], t[3], c[3]);
        SortPair(t[0], c[0], t[2], c[2]);
        SortPair(t[1], c[1], t[3], c[3]);
        SortPair(t[1], c[1], t[2], c[2]);
    } else {
        constexpr int kNet[19][2] = {{0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6},
                                     {3, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}, {2, 4}, {3, 5},
                                     {1, 4}, {3, 6}, {1, 2}, {3, 4}, {5, 6}};
#pragma unroll
        for (int k = 0; k < 19; k++) SortPair(t[kNet[k][0] % K], c[kNet[k][0] % K], t[kNet[k][1] % K], c[kNet[k][1] % K]);
    }
    if (t[0] == inf) {
        cur = stk.Pop(r.tBest);
        return;
    }
    if (stk.sp > kWaveStackDepth - (K - 1)) {  // room for K - 1 pushes
        err |= kErrStackOverflow;
        cur = kDone;
        return;
    }
#pragma unroll
    for (int i = K - 1; i >= 1; i--)
        if (t[i] != inf) stk.Push(c[i], t[i]);
    cur = c[0];
}

// Exact distance ties. Which of two triangles at the same distance a closest-hit query
// reports depends on the order they are tested in, and the wide traversal tests them
// in another order than the reference's binary traversal. When a ray's closest
// distance was reached by more than one triangle, the reference's own traversal
// (BinnedSAHBVH::Intersect order) is run for it and its answer taken, so closest hits
// are the reference's, ties included. Out of line where it can be: ties are rare.
__device__ __forceinline__ void ResolveTieInline(const DevScene* S, V3 o, V3 d, float tmin,
                                                 float tmax, int* best, float* tBest) {
    int stack[kWaveStackDepth];
    int status = 0;
    float bd;
    const int b = TraverseReference<false>(*S, o, d, tmin, tmax, bd, stack, &status);
    if (b >= 0 && status == 0) {
        *best = b;
        *tBest = bd;
    }
}
__device__ __noinline__ void ResolveTie(const DevScene* S, V3 o, V3 d, float tmin, float tmax,
                                        int* best, float* tBest) {
    ResolveTieInline(S, o, d, tmin, tmax, best, tBest);
}

// Q provides: void Load(int i, LaneRay&) (ray, range, and the scene: nodes = nullptr
// for an empty scene) and void Finish(int i, const LaneRay&).
// Must be called by every lane of the warp, in blocks of kTraceBlock threads.
// kAnyHit: every ray Q loads is an any-hit ray.
template <bool kAnyHit, class Q>
__device__ void TraceQueue(Q& q, int n, int* fetch, int& err) {
    __shared__ int2 sEnt[!kAnyHit && kSmemStack > 0 ? kSmemStack * kTraceBlock : 1];
    __shared__ int sCode[kAnyHit && kSmemStack > 0 ? kSmemStack * kTraceBlock : 1];
    const int lane = threadIdx.x & 31;
    const unsigned lowerLanes = (1u << lane) - 1u;
    LaneRay r;
    int idx = -1;
    bool active = false;
    TravStack stk;
    stk.ent = sEnt;
    stk.code = sCode;
    stk.sp = 0;
    int cur = kDone;
    bool exhausted = false;  // warp-uniform
    for (;;) {
        const unsigned idle = __ballot_sync(kFullMask, !active);
        const int nIdle = __popc(idle);
        if (!exhausted && (nIdle >= kRefillLanes || idle == kFullMask)) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, nIdle);
            base = __shfl_sync(kFullMask, base, 0);
            exhausted = base + nIdle >= n;
            if (!active) {
                const int i = base + __popc(idle & lowerLanes);
                if (i < n) {
                    idx = i;
                    q.Load(i, r);
                    r.inv = ExactRecip(r.d);
                    r.tBest = r.tmax;
                    r.best = -1;
                    stk.sp = 0;
                    if (r.nodes) {
                        cur = 0;  // wide root
                        active = true;
                    } else {
                        q.Finish(i, r);
                    }
                }
            }
        }
        if (!__any_sync(kFullMask, active)) {
            if (exhausted) break;
            continue;
        }
#if PT_WHILE_WHILE
        const unsigned busy = __ballot_sync(kFullMask, active);
#endif
        if (active) {
            bool done = false;
#if PT_WHILE_WHILE
            while (cur >= 0) VisitInner<kAnyHit>(r, stk, cur, err);
            __syncwarp(busy);  // the lanes' leaves are intersected together
            if (cur != kDone) done = VisitLeaf<kAnyHit>(r, stk, cur, err);
#else
            if (cur >= 0) VisitInner<kAnyHit>(r, stk, cur, err);
            else if (cur != kDone) done = VisitLeaf<kAnyHit>(r, stk, cur, err);
#endif
            if (done || cur == kDone) {
                q.Finish(idx, r);
                active = false;
            }
        }
    }
}

__device__ __forceinline__ int FindUnit(const WaveUnit* __restrict__ units, int n, int key, bool byPixel) {
    int lo = 0, hi = n - 1;  // last unit whose base <= key
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int base = byPixel ? units[mid].pixelBase : units[mid].pathBase;
        if (base <= key) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

#include "raster_primary.cuh"

// raster != 0: the first bounce is rasterised (raster_primary.cuh), whose keys and tie
// marks start empty here.
__global__ void RaygenKernel(const DevJob* __restrict__ jobs, const WaveUnit* __restrict__ units,
                             WaveBuffers wb, int cur, int raster) {
    const WaveDesc wd = *wb.desc;
    const int n = wd.nPaths, nUnits = wd.nUnits;
    const RasterScratch rs = CarveRaster(wb, cur, 0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const WaveUnit u = units[FindUnit(units, nUnits, i, false)];
        const DevJob& J = jobs[u.job];
        const int W = J.st.width, H = J.st.height;
        // pixel-major path order: a pixel's samples of the unit are consecutive paths
        const int local = i - u.pathBase;
        const int q = local / u.sw, s = u.s0 + local % u.sw;
        int x, y;
        PixelOfIndex(q, W, H, wd.band, x, y);
        PathRng rng(PathKey(J.st.seed, (uint32_t)(y * W + x), (uint32_t)s));
        float r0, r1, r2, r3;
        rng.Next(r0, r1);
        rng.Next(r2, r3);
        Ray ray = GenerateRay<FastMath>(J.C, x, y, W, H, r0, r1, r2, r3);
        if (J.C.aperture == 0.0f) ray.o = LoadV3(J.C.pos);  // a pinhole: exactly the camera position
        if (raster && i >= wd.rasterFrom) {
            rs.key[i] = kNoKey;
            rs.key2[i] = kNoKey;
        }
        wb.ray[cur][2 * i] = make_float4(ray.o.x, ray.o.y, ray.o.z, __int_as_float(i));
        wb.ray[cur][2 * i + 1] = make_float4(ray.d.x, ray.d.y, ray.d.z, 1.0f);
        wb.qs0[cur][i] = make_float4(ray.T.x, ray.T.y, ray.T.z, 1.0f);
        wb.qs1[cur][i] = make_float4(0.f, 0.f, __int_as_float(0), __int_as_float(0));
        wb.qrng[cur][i] = rng.s;
        wb.pathL[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        if (wd.soleJob < 0) wb.pathJob[i] = u.job;  // read only where a wave mixes jobs (JobOf)
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        wb.counts[cur] = n;
        wb.counts[2] = wb.counts[4] = wb.counts[5] = wb.counts[6] = 0;
        wb.counts[8] = wb.counts[9] = wb.counts[10] = 0;  // raster work list (64-bit) and overflow
        wb.counts[11] = wb.counts[12] = 0;                 // raster retrace list and its fetch
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kSortBins; k += gridDim.x * blockDim.x)
        wb.sortBins[k] = 0;  // ray-sort counts start at zero in every wave
}

__device__ __forceinline__ int JobOf(const int* __restrict__ pathJob, int soleJob, int path) {
    return soleJob >= 0 ? soleJob : pathJob[path];
}

struct ExtendQueue {
    const DevJob* jobs;
    const int* pathJob;
    int soleJob;
    const float4* rays;
    float2* hit;
    __device__ void Load(int i, LaneRay& r) const {
        const float4 a = rays[2 * i], b = rays[2 * i + 1];
        const DevJob& J = jobs[JobOf(pathJob, soleJob, __float_as_int(a.w))];
        r.o = V3(a.x, a.y, a.z);
        r.d = V3(b.x, b.y, b.z);
        // SimplePathTracing intersects with distMin = kEps, PathTracing with 0
        // (SimplePathTracing.cpp:81, PathTracing.cpp:50, AccelBase.h:44-55)
        r.tmin = J.st.integrator == kSimplePathTracing ? kEps : 0.0f;
        r.tmax = kFltMax;
        r.anyHit = false;
        r.nodes = J.S.numWide > 0 ? J.S.wide : nullptr;
        r.tris = J.S.tris;
#if PT_CHECK
        r.numWide = J.S.numWide;
        r.numTris = J.S.numTris;
#endif
    }
    // a tied hit is stored as -2 - slot; the shade kernel settles it (SettleTie), which
    // keeps the reference traversal out of this kernel's registers
    __device__ void Finish(int i, const LaneRay& r) const {
        hit[i] = make_float2(r.tBest, __int_as_float(r.best));
    }
};

// The paths of the retrace list through the traversal (ExtendKernel's closest-hit query,
// the same ray): their hit queue entries are the traversal's own answers.
struct RetraceQueue {
    const DevJob* jobs;
    const int* pathJob;
    int soleJob;
    const float4* rays;
    const int* list;
    float2* hit;
    __device__ void Load(int j, LaneRay& r) const {
        const int i = list[j];
        ExtendQueue{jobs, pathJob, soleJob, rays, hit}.Load(i, r);
    }
    __device__ void Finish(int j, const LaneRay& r) const {
        hit[list[j]] = make_float2(r.tBest, __int_as_float(r.best));
    }
};
__global__ void __launch_bounds__(128, PT_TRACE_MIN_BLOCKS) RetraceKernel(const DevJob* __restrict__ jobs,
                                                                          WaveBuffers wb, int cur) {
    const RasterScratch rs = CarveRaster(wb, cur, 0);
    const int n = wb.counts[11];
    int err = 0;
    RetraceQueue q{jobs, wb.pathJob, wb.desc->soleJob, wb.ray[cur], rs.retrace, wb.hit};
    TraceQueue<false>(q, n, wb.counts + 12, err);
    if (err) atomicOr(wb.counts + 3, err);
}

// counts: [0],[1] ray queues, [2] shadow queue, [3] error bits,
//         [4] extend fetch counter, [5] shadow fetch counter, [6] shadow blocks finished,
//         [8..9] raster work list (64-bit), [10] raster overflow, [11] retrace list,
//         [12] retrace fetch counter
// rasterFirst: the first bounce, whose paths from wb.desc->rasterFrom on are rasterised
__global__ void __launch_bounds__(128, PT_TRACE_MIN_BLOCKS) ExtendKernel(const DevJob* __restrict__ jobs, WaveBuffers wb,
                                                    int cur, int rasterFirst) {
    const int n = rasterFirst ? min(wb.counts[cur], wb.desc->rasterFrom) : wb.counts[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counts[cur ^ 1] = 0;
    int err = 0;
    ExtendQueue q{jobs, wb.pathJob, wb.desc->soleJob, wb.ray[cur], wb.hit};
    TraceQueue<false>(q, n, wb.counts + 4, err);
    if (err) atomicOr(wb.counts + 3, err);
}

// kInteg: the integrator of every job in the wave, or -1 when the wave mixes them
// (then read per path). A fixed integrator halves the kernel's code.
// The staged shade kernel's sink: next-event entries and continuation rays go to the
// queues (warp-aggregated appends), terminated paths add their radiance.
struct StageSink {
    WaveBuffers& wb;
    int nxt, path;
    PathRng* rng;
    __device__ __forceinline__ void Shadow(bool shadow, float4 sh0, float4 sh1, float4 sh2, float4 sh3) {
        int sslot = WarpAppend(wb.counts + 2, shadow);
#if PT_CHECK
        if (shadow && sslot >= wb.capacity) {
            atomicOr(wb.counts + 3, kErrBounds);
            shadow = false;
        }
#endif
        if (shadow) {
            float4* e = wb.shadow + 4 * (size_t)sslot;
            e[0] = sh0;
            e[1] = sh1;
            e[2] = sh2;
            e[3] = sh3;
        }
    }
    __device__ __forceinline__ void Done(bool cont, const Ray& out, float lastPdf, float lastSin,
                                         int flags, V3 L) {
        int rslot = WarpAppend(wb.counts + nxt, cont);
#if PT_CHECK
        if (cont && rslot >= wb.capacity) {
            atomicOr(wb.counts + 3, kErrBounds);
            cont = false;
        }
#endif
        if (cont) {
            wb.ray[nxt][2 * rslot] = make_float4(out.o.x, out.o.y, out.o.z, __int_as_float(path));
            wb.ray[nxt][2 * rslot + 1] = make_float4(out.d.x, out.d.y, out.d.z, out.ior);
            wb.qs0[nxt][rslot] = make_float4(out.T.x, out.T.y, out.T.z, out.prob);
            wb.qs1[nxt][rslot] = make_float4(lastPdf, lastSin, __int_as_float(out.bounce),
                                             __int_as_float(flags));
            wb.qrng[nxt][rslot] = rng->s;
        } else {
            float4 l = wb.pathL[path];  // next-event radiance added so far
            wb.pathL[path] = make_float4(l.x + L.x, l.y + L.y, l.z + L.z, __int_as_float(flags));
        }
    }
};

// One path's shade step (SimplePathTracing.cpp:45-126, PathTracing.cpp:38-327): the
// radiance it adds at termination, its next-event entry and its continuation ray. The
// sink takes the next-event entry (Shadow, called where the entry is complete) and the
// outcome (Done). Shared by the staged shade kernel, whose sink appends to the queues,
// and the tail kernel, whose sink keeps both for the same thread.
template <int kInteg, class Sink>
__device__ __forceinline__ void ShadeOne(const DevJob& J, int path, V3 o, V3 d, float4 s0, float4 s2,
                                         float ior, float2 h, PathRng& rng, Sink& sink) {
    const DevScene& S = J.S;
    const DevSettings& st = J.st;
    V3 L;  // radiance this shade adds (terminations); next-event adds come later
    Ray in;
    in.o = o;
    in.d = d;
    in.T = V3(s0.x, s0.y, s0.z);
    in.prob = s0.w;
    in.ior = ior;
    in.bounce = __float_as_int(s2.z);
    int flags = __float_as_int(s2.w);
    const int slot = __float_as_int(h.y);
    bool cont = false;
    Ray out;
    float lastPdf = s2.x, lastSin = s2.y;
    // next-event entry
    bool shadow = false;
    float4 sh0, sh1, sh2, sh3;

    if ((kInteg >= 0 ? kInteg : st.integrator) == kSimplePathTracing) {
        // SimplePathTracing.cpp:45-126
        flags |= kFlagNoSignCheck;
        if (slot < 0) {
            L = L + in.T * EnvColor<FastMath>(S, d);
        } else {
            const int m = ResolveMaterial(S.mats, SlotMaterial(S.shade, slot), rng.Next());
            if (S.mats[m].kind == kEmission) {
                L = L + in.T * MatColor(S.mats[m]);
            } else {
                Shading si = Interpolate<FastMath>(S, slot, o, d, h.x);
                DevMaterial Mh;
                si.n = PointMaterial<FastMath>(S, m, slot, o, d, si.n, Mh);
                out = NextRay<FastMath>(Mh, in, si, rng);
                cont = true;
                if (out.bounce > st.maxBounces) {
                    out.prob *= 0.9f;
                    out.prob = SMax(0.1f, out.prob);
                    if (rng.Next() < out.prob) out.T = out.T / out.prob;
                    else cont = false;
                }
                // a path with exactly zero throughput adds nothing more
                if (out.T.x == 0.0f && out.T.y == 0.0f && out.T.z == 0.0f) cont = false;
            }
        }
    } else {
        // PathTracing.cpp:38-196; k = BSDF bounces taken so far
        const int k = in.bounce;
        if (slot < 0) {
            // one lookup for the three cases (mis = 1 multiplies exactly)
            float mis = 1.0f;
            if (k == 0) {
                flags |= kFlagNoSignCheck;
            } else {
                // alias sampler: densities in solid angle with the map's own sin theta; a
                // bounce off glass (pdf 0) had no environment sample to share the weight.
                // One body for both samplers keeps the shade step's code small.
                const bool alias = S.envAlias != nullptr;
                const float sinT = alias ? sqrtf(SMax(0.0f, 1.0f - d.z * d.z)) : lastSin;
                const bool weigh = alias ? (lastPdf > 0.0f && sinT > 0.0f)
                                         : (S.envValid && d.x != 0 && d.y != 0 && lastSin > 0);
                if (weigh) {
                    const float pdfuv = alias ? EnvPdfAlias<FastMath>(S, d) : EnvPdf<FastMath>(S, d);
                    const float pE = pdfuv / (2.0f * kPi * kPi * sinT);
                    mis = lastPdf * lastPdf / (pE * pE + lastPdf * lastPdf);
                }
            }
            L = L + mis * in.T * EnvColor<FastMath>(S, d);
        } else {
            const Shading si = Interpolate<FastMath>(S, slot, o, d, h.x);
            if (S.mats[si.mat].kind == kEmission) {
                const DevMaterial& M = S.mats[si.mat];
                if (k == 0) {
                    L = L + in.T * MatColor(M);
                    flags |= kFlagNoSignCheck;
                } else {
                    const float l2 = FastMath::SqLen(si.pos - o);
                    const float cosP = fabsf(FastMath::Dot(d, si.n));
                    const float pL = l2 / cosP * S.lightPdfArea;
                    const float mis = lastPdf * lastPdf / (pL * pL + lastPdf * lastPdf);
                    L = L + mis * in.T * MatColor(M);
                }
            } else if (k < st.maxBounces) {
                // material and BSDF normal at the shading point (texture maps applied)
                DevMaterial M;
                const V3 nb = PointMaterial<FastMath>(S, si.mat, slot, o, d, si.n, M);
                // ---- next-event estimation (PathTracing.cpp:202-327)
                const float dt = -FastMath::Dot(d, si.n);
                const V3 p = si.pos + kEps * copysignf(1.0f, dt) * si.n;
                const int nl = S.numLights;
                int index = (int)(rng.Next() * (float)(nl + 1));
                index = min(index, nl);
                if (index >= nl) {
                    if (S.envValid && M.kind != kGlass) {
                        float e0, e1;
                        rng.Next(e0, e1);
                        float pdfuv = 0.0f;
                        V3 sd;
                        const bool alias = S.envAlias != nullptr;
                        if (alias) {
                            float j0, j1;
                            rng.Next(j0, j1);
                            sd = EnvSampleAlias<FastMath>(S, e0, e1, j0, j1, pdfuv);
                        } else {
                            sd = EnvSample<FastMath>(S, e0, e1, pdfuv);
                        }
                        const float c = fabsf(FastMath::Dot(sd, si.n));
                        // sin theta of the (u, v) -> solid angle Jacobian: the map's polar
                        // angle (alias sampler), or the angle to the normal (the reference)
                        const float zc = alias ? sd.z : c;
                        const float sn = sqrtf(SMax(0.0f, 1.0f - zc * zc));
                        const float pB = 2.0f * kPi * kPi * sn * BsdfPdf<FastMath>(M, d, sd, nb);
                        const float mis = pdfuv * pdfuv / (pdfuv * pdfuv + pB * pB);
                        const V3 li = EnvColor<FastMath>(S, sd);
                        const V3 f = BxDF<FastMath>(M, d, sd, nb);
                        const V3 contrib = mis * in.T * (li * f * sn * c * 2.0f * kPi * kPi) / pdfuv;
                        if (contrib.x != 0.0f || contrib.y != 0.0f || contrib.z != 0.0f) {
                            shadow = true;
                            sh0 = make_float4(p.x, p.y, p.z, kFltMax);
                            sh1 = make_float4(sd.x, sd.y, sd.z, __int_as_float(path));
                            sh2 = make_float4(contrib.x, contrib.y, contrib.z, 0.0f);
                            sh3 = make_float4(0.f, 0.f, 0.f, 0.f);
                        }
                    }  // glass: BxDF = 0 (Glass.cpp:11-18), nothing to add
                } else {
                    float u0, u1;
                    rng.Next(u0, u1);
                    const V3 pl = SampleLightPoint<FastMath>(S, index, u0, u1);
                    const V3 dl = pl - p;
                    const float dist = FastMath::Length(dl);
                    const V3 ld = dl / dist;
                    const V3 f = BxDF<FastMath>(M, d, ld, nb);
                    // emitter material pick for the visibility test (GetMaterial with a draw)
                    const float pick = rng.Next();
                    if (f.x != 0.0f || f.y != 0.0f || f.z != 0.0f) {
                        const V3 Tfc = in.T * f * fabsf(FastMath::Dot(ld, si.n));
                        shadow = true;
                        sh0 = make_float4(p.x, p.y, p.z, dist);
                        sh1 = make_float4(ld.x, ld.y, ld.z, __int_as_float(path | (1 << 31)));
                        sh2 = make_float4(Tfc.x, Tfc.y, Tfc.z, BsdfPdf<FastMath>(M, d, ld, nb));
                        sh3 = make_float4(si.pos.x, si.pos.y, si.pos.z, pick);
                    }
                }
                // the next-event entry is handed over before the BSDF sample, so its
                // registers are free for it
                sink.Shadow(shadow, sh0, sh1, sh2, sh3);
                // ---- continuation
                Shading sb = si;
                sb.n = nb;
                out = NextRay<FastMath>(M, in, sb, rng);
                if (!(fabsf(FastMath::SqLen(out.T) - 0.0f) < kEps)) {
                    cont = true;
                    lastPdf = BsdfPdf<FastMath>(M, d, out.d, nb);
                    const float c = fabsf(FastMath::Dot(si.n, out.d));
                    lastSin = sqrtf(SMax(0.0f, 1.0f - c * c));
                    out.bounce = k + 1;
                }
            }
        }
    }
    sink.Done(cont, out, lastPdf, lastSin, flags, L);
}

// A closest hit the extend stage stored as tied (-2 - slot): the reference's answer
// for that ray (ResolveTie), with the extend query's range.
__device__ __noinline__ float2 SettleTie(const DevJob& J, V3 o, V3 d, float2 h) {
    int best = -2 - __float_as_int(h.y);
    float tb = h.x;
    // SimplePathTracing intersects with distMin = kEps, PathTracing with 0 (as ExtendQueue)
    ResolveTie(&J.S, o, d, J.st.integrator == kSimplePathTracing ? kEps : 0.0f, kFltMax, &best,
               &tb);
    return make_float2(tb, __int_as_float(best));
}

template <int kInteg>
__global__ void __launch_bounds__(128, PT_SHADE_MIN_BLOCKS) ShadeKernel(const DevJob* __restrict__ jobs, WaveBuffers wb,
                                                   int cur) {
    const int n = wb.counts[cur];
    const int nxt = cur ^ 1;
    const int sole = wb.desc->soleJob;
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counts[4] = 0;  // the next extend fetches from zero
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 ra = wb.ray[cur][2 * i], rb = wb.ray[cur][2 * i + 1];
        float2 h = wb.hit[i];
        const int path = __float_as_int(ra.w);
        const DevJob& J = jobs[JobOf(wb.pathJob, sole, path)];
        if (__float_as_int(h.y) < -1) h = SettleTie(J, V3(ra.x, ra.y, ra.z), V3(rb.x, rb.y, rb.z), h);
#if PT_CHECK
        if (__float_as_int(h.y) >= J.S.numTris || (unsigned)path >= (unsigned)wb.capacity) {
            atomicOr(wb.counts + 3, kErrBounds);
            continue;  // the appends are aggregated over the lanes that reach them
        }
#endif
        PathRng rng(wb.qrng[cur][i]);
        StageSink sink{wb, nxt, path, &rng};
        ShadeOne<kInteg>(J, path, V3(ra.x, ra.y, ra.z), V3(rb.x, rb.y, rb.z), wb.qs0[cur][i],
                         wb.qs1[cur][i], rb.w, h, rng, sink);
    }
}

// A next-event entry's visibility ray (PathTracing.cpp:202-327): environment entries
// are any-hit rays, area-light entries closest-hit rays bounded just past the light.
__device__ __forceinline__ void ShadowRay(const DevScene& S, float4 e0, float4 e1, LaneRay& r) {
    r.nodes = S.numWide > 0 ? S.wide : nullptr;
    r.tris = S.tris;
#if PT_CHECK
    r.numWide = S.numWide;
    r.numTris = S.numTris;
#endif
    r.o = V3(e0.x, e0.y, e0.z);
    r.d = V3(e1.x, e1.y, e1.z);
    r.tmin = 0.0f;
    const bool env = __float_as_int(e1.w) >= 0;
    r.anyHit = env;
    r.tmax = env ? kFltMax : e0.w + 0.05f;
}

__device__ __noinline__ void ApplyAreaLight(const DevScene& S, const float4* e, V3 o, V3 d, int best,
                                            float tBest, int path, float4* pathL);
// Adds a traced next-event entry's contribution to its path's radiance; e holds the
// entry's four float4 (read only as needed: an occluded environment entry reads one).
// kEnvOnly: the entry is an environment entry (no area light in the wave).
template <bool kEnvOnly = false>
__device__ __forceinline__ void ApplyShadow(const DevScene& S, const float4* e, const LaneRay& r,
                                            float4* pathL) {
    const float4 e1 = e[1];
    const int tag = __float_as_int(e1.w);
    const int path = tag & 0x7FFFFFFF;
    if (kEnvOnly || tag >= 0) {  // environment: adds when unoccluded
        if (r.best != -1) return;
        const float4 e2 = e[2];
        float4 l = pathL[path];
        l.x += e2.x;
        l.y += e2.y;
        l.z += e2.z;
        pathL[path] = l;
        return;
    }
    // area light: the closest hit must be an emitter at the sampled point
    if (r.best == -1) return;
    ApplyAreaLight(S, e, r.o, r.d, r.best, r.tBest, path, pathL);
}
// The area-light part of ApplyShadow, out of line: it runs once per traced entry, and
// inlined its registers crowd the traversal loop of the shadow kernel.
__device__ __noinline__ void ApplyAreaLight(const DevScene& S, const float4* e, V3 o, V3 d, int best,
                                            float tBest, int path, float4* pathL) {
    const float4 e0 = e[0], e2 = e[2], e3 = e[3];
    if (best < -1) {  // a tied closest hit: the reference's answer (range as ShadowRay's)
        best = -2 - best;
        ResolveTieInline(&S, o, d, 0.0f, e0.w + 0.05f, &best, &tBest);
    }
    const int m = ResolveMaterial(S.mats, SlotMaterial(S.shade, best), e3.w);
    if (S.mats[m].kind != kEmission) return;
    const Shading sl = Interpolate<FastMath>(S, best, o, d, tBest);
    const V3 pl = o + d * e0.w;
    if (!(fabsf(FastMath::SqLen(pl - sl.pos) - 0.0f) < kEps)) return;
    const V3 sipos(e3.x, e3.y, e3.z);
    const float l2 = FastMath::SqLen(sl.pos - sipos);
    const float cosP = fabsf(FastMath::Dot(d, sl.n));
    const float pdfArea = S.lightPdfArea;
    float mis = 0.0f;
    if (l2 > 0.0f) {
        const float pB = e2.w * cosP / l2;
        mis = pdfArea * pdfArea / (pdfArea * pdfArea + pB * pB);
    }
    const V3 li = MatColor(S.mats[sl.mat]);
    const V3 c = mis * (V3(e2.x, e2.y, e2.z) * li * cosP / (pdfArea * l2));
    float4 l = pathL[path];
    l.x += c.x;
    l.y += c.y;
    l.z += c.z;
    pathL[path] = l;
}

template <bool kEnvOnly>
struct ShadowQueue {
    const DevJob* jobs;
    const int* pathJob;
    int soleJob;
    const float4* entries;
    float4* pathL;
    __device__ void Load(int j, LaneRay& r) const {
        const float4 e0 = entries[4 * j], e1 = entries[4 * j + 1];
        ShadowRay(jobs[JobOf(pathJob, soleJob, __float_as_int(e1.w) & 0x7FFFFFFF)].S, e0, e1, r);
    }
    __device__ void Finish(int j, const LaneRay& r) const {
        const int path = __float_as_int(entries[4 * j + 1].w) & 0x7FFFFFFF;
        ApplyShadow<kEnvOnly>(jobs[JobOf(pathJob, soleJob, path)].S, entries + 4 * j, r, pathL);
    }
};

// One ray traversed by one thread (the tail kernel's form): the same node and leaf
// order as TraceQueue gives the ray.
__device__ __forceinline__ void TraceOne(LaneRay& r, TravStack& stk, int& err) {
    r.inv = ExactRecip(r.d);
    r.tBest = r.tmax;
    r.best = -1;
    stk.sp = 0;
    if (!r.nodes) return;
    int cur = 0;  // wide root
    while (cur != kDone) {
        if (cur >= 0) VisitInner<false>(r, stk, cur, err);
        else if (VisitLeaf<false>(r, stk, cur, err)) break;
    }
}

// The tail kernel's sink: the thread keeps its next-event entry and continuation;
// a terminated path adds its radiance at once (before its next-event entry is traced,
// the order the staged kernels add them in).
struct TailSink {
    float4* pathL;
    int path;
    bool shadow = false, cont = false;
    float4 sh[4];
    Ray out;
    float lastPdf = 0.0f, lastSin = 0.0f;
    int flags = 0;
    __device__ __forceinline__ void Shadow(bool s, float4 a, float4 b, float4 c, float4 d) {
        shadow = s;
        sh[0] = a;
        sh[1] = b;
        sh[2] = c;
        sh[3] = d;
    }
    __device__ __forceinline__ void Done(bool c, const Ray& o, float lp, float ls, int f, V3 L) {
        cont = c;
        out = o;
        lastPdf = lp;
        lastSin = ls;
        flags = f;
        if (!c) {
            const float4 l = pathL[path];
            pathL[path] = make_float4(l.x + L.x, l.y + L.y, l.z + L.z, __int_as_float(f));
        }
    }
};

// The last `iters` bounces of a wave in one launch: each thread takes a path from the
// queue and runs its closest hit, shade and next-event ray, bounce after bounce, until
// the path ends or the wave's iterations are used up, exactly as the staged kernels
// would (same functions, same per-path random stream, same order of radiance adds).
// Late bounces hold few rays, and one launch spares each of them a sweep of three
// latency-bound launches.
template <int kInteg>
__global__ void __launch_bounds__(128) TailKernel(const DevJob* __restrict__ jobs, WaveBuffers wb,
                                                  int cur, int iters) {
    __shared__ int2 sEnt[kSmemStack > 0 ? kSmemStack * kTraceBlock : 1];
    TravStack stk;
    stk.ent = sEnt;
    stk.code = nullptr;  // closest-hit and runtime any-hit visits only (Push / Pop)
    stk.sp = 0;
    const int n = wb.counts[cur];
    const int sole = wb.desc->soleJob;
    int err = 0;
    for (;;) {
        const int i = atomicAdd(wb.counts + 4, 1);  // reset by the shade before
        if (i >= n) break;
        const float4 ra = wb.ray[cur][2 * i], rb = wb.ray[cur][2 * i + 1];
        const int path = __float_as_int(ra.w);
        const DevJob& J = jobs[JobOf(wb.pathJob, sole, path)];
        const DevScene& S = J.S;
        V3 o(ra.x, ra.y, ra.z), d(rb.x, rb.y, rb.z);
        float ior = rb.w;
        float4 s0 = wb.qs0[cur][i], s2 = wb.qs1[cur][i];
        PathRng rng(wb.qrng[cur][i]);
        for (int it = 0; it < iters; it++) {
            LaneRay r;
            r.o = o;
            r.d = d;
            r.tmin = J.st.integrator == kSimplePathTracing ? kEps : 0.0f;  // as ExtendQueue
            r.tmax = kFltMax;
            r.anyHit = false;
            r.nodes = S.numWide > 0 ? S.wide : nullptr;
            r.tris = S.tris;
#if PT_CHECK
            r.numWide = S.numWide;
            r.numTris = S.numTris;
#endif
            TraceOne(r, stk, err);
            if (r.best < -1) {
                r.best = -2 - r.best;
                ResolveTie(&S, r.o, r.d, r.tmin, r.tmax, &r.best, &r.tBest);
            }
            TailSink sink{wb.pathL, path};
            ShadeOne<kInteg>(J, path, o, d, s0, s2, ior, make_float2(r.tBest, __int_as_float(r.best)), rng,
                             sink);
            if (sink.shadow) {
                LaneRay sr;
                ShadowRay(S, sink.sh[0], sink.sh[1], sr);
                TraceOne(sr, stk, err);
                ApplyShadow(S, sink.sh, sr, wb.pathL);
            }
            if (!sink.cont) break;
            o = sink.out.o;
            d = sink.out.d;
            ior = sink.out.ior;
            s0 = make_float4(sink.out.T.x, sink.out.T.y, sink.out.T.z, sink.out.prob);
            s2 = make_float4(sink.lastPdf, sink.lastSin, __int_as_float(sink.out.bounce),
                             __int_as_float(sink.flags));
        }
    }
    if (err) atomicOr(wb.counts + 3, err);
}

// It may run beside the next bounce's extend kernel (which touches neither the
// shadow queue nor its counters); its last block to finish clears the shadow queue
// size and fetch counter for the next shade.
// kEnvOnly: no job of the wave has area lights, so every entry is an environment
// entry, an any-hit ray (the traversal specialised for it).
template <bool kEnvOnly>
__global__ void __launch_bounds__(128, PT_TRACE_MIN_BLOCKS) ShadowKernel(const DevJob* __restrict__ jobs, WaveBuffers wb) {
    const int n = wb.counts[2];
    int err = 0;
    ShadowQueue<kEnvOnly> q{jobs, wb.pathJob, wb.desc->soleJob, wb.shadow, wb.pathL};
    TraceQueue<kEnvOnly>(q, n, wb.counts + 5, err);
    if (err) atomicOr(wb.counts + 3, err);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(wb.counts + 6, 1) == (int)gridDim.x - 1) {
            wb.counts[2] = 0;
            wb.counts[5] = 0;
            wb.counts[6] = 0;
        }
    }
}

__global__ void AccumulateKernel(const DevJob* __restrict__ jobs, const WaveUnit* __restrict__ units,
                                 WaveBuffers wb) {
    const WaveDesc wd = *wb.desc;
    const int n = wd.nPixelUnits, nUnits = wd.nUnits;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const WaveUnit u = units[FindUnit(units, nUnits, i, true)];
        const DevJob& J = jobs[u.job];
        const int W = J.st.width, H = J.st.height;
        const int q = i - u.pixelBase;
        int x, y;
        PixelOfIndex(q, W, H, wd.band, x, y);
        const size_t pixel = (size_t)y * W + x;
        float4 acc = J.accum[pixel];
        for (int s = 0; s < u.sw; s++) {
            const int p = u.pathBase + q * u.sw + s;
            const float4 l = wb.pathL[p];
            const int flags = __float_as_int(l.w);
            // PathTracing.cpp:191-195 drops a sample whose smallest channel is
            // negative or NaN; primary misses/emitters are added directly (:54,:67).
            if ((flags & kFlagNoSignCheck) || MinElem(V3(l.x, l.y, l.z)) >= 0.0f) {
                acc.x += l.x;
                acc.y += l.y;
                acc.z += l.z;
            }
        }
        J.accum[pixel] = acc;
    }
}

__global__ void FinalizeKernel(const DevJob* __restrict__ jobs, const int* __restrict__ jobList,
                               int maxPixels) {
    const DevJob& J = jobs[jobList[blockIdx.y]];
    const int n = J.st.width * J.st.height;
    const float inv = (float)J.st.spp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n && i < maxPixels;
         i += gridDim.x * blockDim.x) {
        const float4 a = J.accum[i];
        J.film[3 * i] = a.x / inv;
        J.film[3 * i + 1] = a.y / inv;
        J.film[3 * i + 2] = a.z / inv;
    }
}

struct RayBatchQueue {
    const DevScene* S;
    const float4* nodes;
    const float4* tris;
    int numWide, numTris;
    const float* rays;
    float tmin, tmax;
    int* triOut;
    float* distOut;
    __device__ void Load(int i, LaneRay& r) const {
        const float* p = rays + 6 * (size_t)i;
        r.o = V3(p[0], p[1], p[2]);
        r.d = V3(p[3], p[4], p[5]);
        r.tmin = tmin;
        r.tmax = tmax;
        r.anyHit = false;
        r.nodes = nodes;
        r.tris = tris;
#if PT_CHECK
        r.numWide = numWide;
        r.numTris = numTris;
#endif
    }
    __device__ void Finish(int i, const LaneRay& r) const {
        int best = r.best;
        float tb = r.tBest;
        if (best < -1) {
            best = -2 - best;
            ResolveTie(S, r.o, r.d, r.tmin, r.tmax, &best, &tb);
        }
        triOut[i] = best >= 0 ? TriId(tris, best) : -1;
        distOut[i] = best >= 0 ? tb : -1.0f;
    }
};

__global__ void __launch_bounds__(128) TraceKernel(DevScene S, int n, const float* __restrict__ rays,
                                                   float tmin, float tmax, int* __restrict__ triOut,
                                                   float* __restrict__ distOut, int* fetch) {
    RayBatchQueue q{&S, S.numWide > 0 ? S.wide : nullptr, S.tris, S.numWide, S.numTris, rays, tmin,
                    tmax, triOut, distOut};
    int err = 0;
    TraceQueue<false>(q, n, fetch, err);
}

// Profiling helpers: ray tallies and the reference traversal's work per ray.
__global__ void TallyKernel(const int* counts, int cur, unsigned long long* c) {
    c[3] += (unsigned long long)counts[cur];
    c[4] += (unsigned long long)counts[2];
}

__global__ void __launch_bounds__(128) RefCountKernel(const DevJob* __restrict__ jobs, WaveBuffers wb,
                                                      int cur, unsigned long long* c) {
    const int n = wb.counts[cur];
    unsigned long long nodes = 0, tris = 0;
    int stack[kWaveStackDepth];
    int status = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = wb.ray[cur][2 * i], b = wb.ray[cur][2 * i + 1];
        const DevJob& J = jobs[JobOf(wb.pathJob, wb.desc->soleJob, __float_as_int(a.w))];
        const float tmin = J.st.integrator == kSimplePathTracing ? kEps : 0.0f;
        unsigned nn = 0, nt = 0;
        float d;
        TraverseReference<true>(J.S, V3(a.x, a.y, a.z), V3(b.x, b.y, b.z), tmin, kFltMax, d, stack,
                                &status, &nn, &nt);
        nodes += nn;
        tris += nt;
    }
    for (int off = 16; off > 0; off >>= 1) {
        nodes += __shfl_down_sync(0xffffffffu, nodes, off);
        tris += __shfl_down_sync(0xffffffffu, tris, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(c + 0, nodes);
        atomicAdd(c + 1, tris);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(c + 2, (unsigned long long)n);
}

namespace {
struct StageEvents {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[6];
    void Begin(int k, cudaStream_t s) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        ev[k].push_back({a, b});
        cudaEventRecord(a, s);
    }
    void End(int k, cudaStream_t s) { cudaEventRecord(ev[k].back().second, s); }
    void Collect(double* ms) {
        for (int k = 0; k < 6; k++) {
            for (auto& p : ev[k]) {
                float t = 0.0f;
                cudaEventElapsedTime(&t, p.first, p.second);
                ms[k] += t;
                cudaEventDestroy(p.first);
                cudaEventDestroy(p.second);
            }
            ev[k].clear();
        }
    }
};
}  // namespace

namespace {
// Alignment of the buffers carved out of one allocation.
constexpr size_t kAlign = 256;
size_t Up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }
}  // namespace

// The one layout of the wave buffers: offsets from `base` (0 to measure the size).
// Returns the bytes used; fills *w when given.

// ---- ray reordering (WaveTuning::sortRays): a counting sort of the next queue by a
// coherence key, so that a warp's rays start in similar places and directions.
// Key: 64 octahedral direction cells (major), then a 12-bit Morton code of the origin's
// cell on a 16x16x16 grid over the scene bounds. The order within a bin is arbitrary;
// results do not depend on queue order (each path's state travels with its ray and
// pixel sums are formed in sample order).
__device__ __forceinline__ unsigned Spread3(unsigned v) {  // 4 bits -> every third bit
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}
__device__ __forceinline__ unsigned RayKey(const DevScene& S, float4 a, float4 b) {
    unsigned cell = 0;
    if (S.numNodes > 0) {
        const float4 n0 = __ldg(S.nodes), n1 = __ldg(S.nodes + 1);
        const float lo[3] = {n0.x, n0.y, n0.z}, hi[3] = {n0.w, n1.x, n1.y}, o[3] = {a.x, a.y, a.z};
        for (int k = 0; k < 3; k++) {
            const float ext = hi[k] - lo[k];
            const int c = ext > 0.0f ? (int)((o[k] - lo[k]) * (16.0f / ext)) : 0;
            cell |= Spread3((unsigned)min(max(c, 0), 15)) << k;
        }
    }
    const float s = fabsf(b.x) + fabsf(b.y) + fabsf(b.z);
    float px = s > 0.0f ? b.x / s : 0.0f, py = s > 0.0f ? b.y / s : 0.0f;
    if (b.z < 0.0f) {
        const float qx = (1.0f - fabsf(py)) * copysignf(1.0f, px);
        const float qy = (1.0f - fabsf(px)) * copysignf(1.0f, py);
        px = qx;
        py = qy;
    }
    const int ix = min(max((int)((px + 1.0f) * 4.0f), 0), 7);
    const int iy = min(max((int)((py + 1.0f) * 4.0f), 0), 7);
    return ((unsigned)(iy * 8 + ix) << kSortOriginBits) | cell;
}

__global__ void __launch_bounds__(128) SortKeysKernel(const DevJob* __restrict__ jobs, WaveBuffers wb,
                                                      int q) {
    const int n = wb.counts[q];
    const int soleJob = wb.desc->soleJob;
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        unsigned key = 0xffffffffu;
        if (i < n) {
            const float4 a = wb.ray[q][2 * i], b = wb.ray[q][2 * i + 1];
            key = RayKey(jobs[JobOf(wb.pathJob, soleJob, __float_as_int(a.w))].S, a, b);
            wb.sortKey[i] = key;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (i < n && lane == __ffs(peers) - 1) atomicAdd(&wb.sortBins[key], (unsigned)__popc(peers));
    }
}

// One block: exclusive scan of the counts into offsets; the counts are cleared for the
// next bounce.
__global__ void __launch_bounds__(1024) SortScanKernel(WaveBuffers wb) {
    __shared__ unsigned warpSums[32];
    constexpr int kPer = kSortBins / 1024;
    unsigned* hist = wb.sortBins;
    unsigned* off = wb.sortBins + kSortBins;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned v[kPer], sum = 0;
    for (int j = 0; j < kPer; j++) {
        v[j] = hist[t * kPer + j];
        hist[t * kPer + j] = 0;
        sum += v[j];
    }
    unsigned inc = sum;
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned x = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += x;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warpSums[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned x = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += x;
        }
        warpSums[lane] = w;
    }
    __syncthreads();
    unsigned run = inc - sum + (warp > 0 ? warpSums[warp - 1] : 0u);
    for (int j = 0; j < kPer; j++) {
        off[t * kPer + j] = run;
        run += v[j];
    }
}

__global__ void __launch_bounds__(128) SortScatterKernel(WaveBuffers wb, int src, int dst) {
    const int n = wb.counts[src];
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counts[dst] = n;
    unsigned* off = wb.sortBins + kSortBins;
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        const unsigned key = i < n ? wb.sortKey[i] : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (i < n && lane == leader) base = atomicAdd(&off[key], (unsigned)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (i >= n) continue;
        const int pos = (int)(base + __popc(peers & ((1u << lane) - 1u)));
        wb.ray[dst][2 * pos] = wb.ray[src][2 * i];
        wb.ray[dst][2 * pos + 1] = wb.ray[src][2 * i + 1];
        wb.qs0[dst][pos] = wb.qs0[src][i];
        wb.qs1[dst][pos] = wb.qs1[src][i];
        wb.qrng[dst][pos] = wb.qrng[src][i];
    }
}

static size_t LayOutWaveBuffers(uintptr_t base, int capacity, WaveBuffers* w) {
    const size_t C = (size_t)capacity;
    uintptr_t p = base;
    auto take = [&](size_t bytes) {
        const uintptr_t q = p;
        p += Up(bytes);
        return reinterpret_cast<void*>(q);
    };
    WaveBuffers v{};
    v.capacity = capacity;
    for (int k = 0; k < 2; k++) v.ray[k] = (float4*)take(C * 2 * sizeof(float4));
    for (int k = 0; k < 2; k++) v.qs0[k] = (float4*)take(C * sizeof(float4));
    for (int k = 0; k < 2; k++) v.qs1[k] = (float4*)take(C * sizeof(float4));
    for (int k = 0; k < 2; k++) v.qrng[k] = (unsigned long long*)take(C * sizeof(unsigned long long));
    v.hit = (float2*)take(C * sizeof(float2));
    v.pathL = (float4*)take(C * sizeof(float4));
    v.pathJob = (int*)take(C * sizeof(int));
    v.desc = (WaveDesc*)take(sizeof(WaveDesc));
    v.shadow = (float4*)take(C * 4 * sizeof(float4));
    v.counts = (int*)take(16 * sizeof(int));
    v.sortKey = (unsigned*)take(C * sizeof(unsigned));
    v.sortBins = (unsigned*)take(2 * (size_t)kSortBins * sizeof(unsigned));
    if (w) *w = v;
    return (size_t)(p - base);
}

size_t WaveBuffersBytes(int capacity) { return LayOutWaveBuffers(0, capacity, nullptr); }

size_t WaveBuffersBytesTwoLanes(int capacity) {
    return std::max(WaveBuffersBytes(capacity), 2 * WaveBuffersBytes(capacity / 2));
}

WaveBuffers CarveWaveBuffers(void* base, int capacity) {
    WaveBuffers w{};
    LayOutWaveBuffers(reinterpret_cast<uintptr_t>(base), capacity, &w);
    return w;
}

int DefaultStageGrid() {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int perSm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, ExtendKernel, 128, 0);
        if (perSm < 1) perSm = 1;
        grid = sms * perSm;
    }
    return grid;
}

// Grid of the shade stage: PT_SHADE_BLOCKS_PER_SM blocks per SM (0: the trace grid).
#ifndef PT_SHADE_BLOCKS_PER_SM
#define PT_SHADE_BLOCKS_PER_SM 0
#endif
static int SmCount() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    return sms;
}
static int ShadeGrid(int traceGrid) {
    return PT_SHADE_BLOCKS_PER_SM > 0 ? SmCount() * PT_SHADE_BLOCKS_PER_SM : traceGrid;
}

int StageGrid(const WaveTuning& tune) {
    return tune.blocksPerSm > 0 ? SmCount() * tune.blocksPerSm : DefaultStageGrid();
}

// The bounce iterations [it0, it0 + count) of a wave (queue parity from it0).
// A second stream and fork/join events: each bounce's shadow stage runs beside the
// next bounce's extend stage (they share no buffers), and the next shade waits for it.
struct StageOverlap {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    bool Ready() {
        if (side) return true;
        if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&join, cudaEventDisableTiming) != cudaSuccess) {
            Release();
            return false;
        }
        return true;
    }
    void Release() {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
        side = nullptr;
        fork = join = nullptr;
    }
};

// tailFrom > 0: bounces from it0 + tailFrom on run in one TailKernel launch.
// envOnly: no job of the wave has area lights (the any-hit shadow kernel).
static void LaunchBounces(const DevJob* jobs, const WaveUnit* units, const WaveBuffers& wb,
                          int integrator, int grid, int it0, int count, cudaStream_t stream,
                          WaveProfile* prof, int* nl, bool sort, StageOverlap* ov, bool envOnly,
                          int tailFrom = 0, bool raster = false) {
    StageEvents* ev = prof ? (StageEvents*)prof->events : nullptr;
    const int block = kTraceBlock;
    const int sgrid = ShadeGrid(grid);
    bool pendingShadow = false;  // a shadow stage on the side stream the next shade must wait for
    for (int it = it0; it < it0 + count; it++) {
        // sorted bounces trace queue 0 and reorder the rays shade appends to queue 1 back into it
        const int cur = sort ? 0 : (it & 1);
        if (tailFrom > 0 && it - it0 == tailFrom) {
            if (pendingShadow) {  // the tail adds radiance the pending shadow stage also adds to
                cudaStreamWaitEvent(stream, ov->join, 0);
                pendingShadow = false;
            }
            const int left = it0 + count - it;
            if (integrator == kPathTracing)
                TailKernel<kPathTracing><<<grid, block, 0, stream>>>(jobs, wb, cur, left);
            else if (integrator == kSimplePathTracing)
                TailKernel<kSimplePathTracing><<<grid, block, 0, stream>>>(jobs, wb, cur, left);
            else
                TailKernel<-1><<<grid, block, 0, stream>>>(jobs, wb, cur, left);
            *nl += 1;
            break;
        }
        if (ev) ev->Begin(1, stream);
        if (it == 0 && raster) {  // the traced units' paths, then the rasterised ones
            ExtendKernel<<<grid, block, 0, stream>>>(jobs, wb, cur, 1);
            if (ev) {  // the raster kernels have a timer of their own
                ev->End(1, stream);
                ev->Begin(5, stream);
            }
            RasterSetupKernel<<<SmCount() * 32, block, 0, stream>>>(jobs, units, wb, cur);
            RasterVisitKernel<<<SmCount() * 16, block, 0, stream>>>(jobs, units, wb, cur);
            RasterFinishKernel<<<grid, block, 0, stream>>>(wb, cur);
            // few paths, if any: a small grid (an empty launch of the full one took 0.12 ms)
            RetraceKernel<<<2 * SmCount(), block, 0, stream>>>(jobs, wb, cur);
            if (ev) {
                ev->End(5, stream);
                ev->Begin(1, stream);  // an empty interval closed below
            }
            *nl += 4;  // one more below
        } else {
            ExtendKernel<<<grid, block, 0, stream>>>(jobs, wb, cur, 0);
        }
        if (ev) {
            ev->End(1, stream);
            if (prof->countReference)
                RefCountKernel<<<grid, block, 0, stream>>>(jobs, wb, cur, prof->devCounters);
            ev->Begin(2, stream);
        }
        if (pendingShadow) {
            cudaStreamWaitEvent(stream, ov->join, 0);
            pendingShadow = false;
        }
        if (integrator == kPathTracing)
            ShadeKernel<kPathTracing><<<sgrid, block, 0, stream>>>(jobs, wb, cur);
        else if (integrator == kSimplePathTracing)
            ShadeKernel<kSimplePathTracing><<<sgrid, block, 0, stream>>>(jobs, wb, cur);
        else
            ShadeKernel<-1><<<sgrid, block, 0, stream>>>(jobs, wb, cur);
        if (ev) {
            ev->End(2, stream);
            TallyKernel<<<1, 1, 0, stream>>>(wb.counts, cur, prof->devCounters);
            ev->Begin(3, stream);
        }
        if (ov) {
            cudaEventRecord(ov->fork, stream);
            cudaStreamWaitEvent(ov->side, ov->fork, 0);
            if (envOnly) ShadowKernel<true><<<grid, block, 0, ov->side>>>(jobs, wb);
            else ShadowKernel<false><<<grid, block, 0, ov->side>>>(jobs, wb);
            cudaEventRecord(ov->join, ov->side);
            pendingShadow = true;
        } else if (envOnly) {
            ShadowKernel<true><<<grid, block, 0, stream>>>(jobs, wb);
        } else {
            ShadowKernel<false><<<grid, block, 0, stream>>>(jobs, wb);
        }
        if (ev) ev->End(3, stream);
        *nl += 3;
        if (sort) {
            SortKeysKernel<<<grid, block, 0, stream>>>(jobs, wb, 1);
            SortScanKernel<<<1, 1024, 0, stream>>>(wb);
            SortScatterKernel<<<grid, block, 0, stream>>>(wb, 1, 0);
            *nl += 3;
        }
        if (prof) {
            prof->extendLaunches++;
            prof->shadowLaunches++;
        }
    }
    if (pendingShadow) cudaStreamWaitEvent(stream, ov->join, 0);
}

// A captured sequence: for fixed-depth waves the whole wave (raygen, iters
// bounces, accumulate); for queue-polled waves a block of kPollEvery bounces.
constexpr int kPollEvery = 4;
struct WaveGraphKey {
    const void* jobs;
    const void* units;
    const void* buffers;
    int capacity, iters, integrator, grid, sort, accum, tail, raster, envOnly;
    bool operator==(const WaveGraphKey& o) const {
        return jobs == o.jobs && units == o.units && buffers == o.buffers && capacity == o.capacity &&
               iters == o.iters && integrator == o.integrator && grid == o.grid && sort == o.sort &&
               accum == o.accum && tail == o.tail && raster == o.raster && envOnly == o.envOnly;
    }
};
struct WaveGraph {
    WaveGraphKey key;
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
};
struct WaveGraphCache {
    std::vector<WaveGraph> graphs;  // few shapes per owner; least recently added dropped first
    static constexpr size_t kMax = 16;
    StageOverlap overlap[2];        // shadow-stage side streams of the two wave lanes
    // the second wave lane: its stream and each lane's "accumulated and finalised" event
    cudaStream_t waveSide = nullptr;
    cudaEvent_t waveDone[2] = {nullptr, nullptr};
    ~WaveGraphCache() {
        for (WaveGraph& g : graphs) cudaGraphExecDestroy(g.exec);
        for (StageOverlap& o : overlap) o.Release();
        for (cudaEvent_t e : waveDone)
            if (e) cudaEventDestroy(e);
        if (waveSide) cudaStreamDestroy(waveSide);
    }
};

bool WavePipeline(WaveGraphCache* cache, cudaStream_t* side, cudaEvent_t* done) {
    if (!cache) return false;
    if (!cache->waveSide) {
        if (cudaStreamCreateWithFlags(&cache->waveSide, cudaStreamNonBlocking) != cudaSuccess) {
            cache->waveSide = nullptr;
            return false;
        }
        for (cudaEvent_t& e : cache->waveDone)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    }
    *side = cache->waveSide;
    done[0] = cache->waveDone[0];
    done[1] = cache->waveDone[1];
    return done[0] && done[1];
}

__global__ void OrErrorsKernel(int* dst, const int* a, const int* b) { *dst = *a | *b; }

cudaError_t MergeWaveErrors(const WaveBuffers& into, const WaveBuffers& a, const WaveBuffers& b,
                            cudaStream_t stream) {
    OrErrorsKernel<<<1, 1, 0, stream>>>(into.counts + 3, a.counts + 3, b.counts + 3);
    return cudaGetLastError();
}

cudaError_t AccumulateWave(const DevJob* jobs, const WaveUnit* units, const WaveBuffers& wb,
                           const WaveTuning& tune, cudaStream_t stream, int* launches) {
    AccumulateKernel<<<StageGrid(tune), kTraceBlock, 0, stream>>>(jobs, units, wb);
    if (launches) (*launches)++;
    return cudaGetLastError();
}
WaveGraphCache* NewWaveGraphCache() { return new WaveGraphCache(); }
void FreeWaveGraphCache(WaveGraphCache* cache) { delete cache; }

template <class F>
static cudaError_t ReplayCaptured(WaveGraphCache* cache, const WaveGraphKey& key, cudaStream_t stream,
                                  int* nl, F&& record) {
    WaveGraph* g = nullptr;
    for (WaveGraph& c : cache->graphs)
        if (c.key == key) g = &c;
    if (!g) {
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        int kernels = 0;
        record(&kernels);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess) return e;
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return e;
        if (cache->graphs.size() >= WaveGraphCache::kMax) {
            cudaGraphExecDestroy(cache->graphs.front().exec);
            cache->graphs.erase(cache->graphs.begin());
        }
        cache->graphs.push_back(WaveGraph{key, exec, kernels});
        g = &cache->graphs.back();
    }
    *nl += g->kernels;
    return cudaGraphLaunch(g->exec, stream);
}

cudaError_t RunWave(const DevJob* jobs, const WaveUnit* units, const WaveShape& shape,
                    const WaveBuffers& wb, cudaStream_t stream, int* launches, WaveProfile* prof,
                    const WaveTuning& tune, WaveGraphCache* graphs, int lane, bool accumulate) {
    if (shape.nPaths <= 0) return cudaSuccess;
    if (shape.nPaths > wb.capacity) return cudaErrorInvalidValue;
    const int grid = StageGrid(tune);
    const int block = kTraceBlock;
    StageEvents* ev = prof ? (StageEvents*)prof->events : nullptr;
    bool useGraphs = graphs && !prof && tune.graphs && stream != 0 && stream != cudaStreamLegacy;
    if (useGraphs) {  // a caller capturing this stream records the launches themselves
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
            useGraphs = false;
    }
    // the wave's scalars (pageable source: staged before the call returns)
    WaveDesc d{};
    d.nUnits = shape.nUnits;
    d.nPaths = shape.nPaths;
    d.nPixelUnits = shape.nPixelUnits;
    d.soleJob = shape.soleJob;
    d.band = tune.band > 0 ? tune.band : 8;
    // the first bounce rasterised where the wave allows it (raster_primary.cuh)
    const bool raster = shape.raster > 0 && tune.primaryTraversal != 1 && tune.sortRays == 0 &&
                        shape.iters >= 0;
    d.rasterFrom = raster ? shape.rasterFrom : shape.nPaths;
    d.rasterUnit0 = raster ? shape.rasterUnit0 : shape.nUnits;
    d.rasterRecs = raster ? shape.raster : 0;
    if (prof && raster) prof->rasterPaths += (unsigned long long)(shape.nPaths - shape.rasterFrom);
    cudaError_t e = cudaMemcpyAsync(wb.desc, &d, sizeof(d), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    int nl = 0;
    const bool sort = tune.sortRays != 0;
    // the last bounces in one launch (fixed-depth waves; profiled renders keep every stage)
    const int tailFrom = (!prof && !sort && tune.tailBounce > 0 && shape.iters > tune.tailBounce)
                           ? tune.tailBounce : 0;
    // shadow stages beside the next extend, on the owner's side stream (not when profiling,
    // whose stage timers need one stream)
    StageOverlap* ov =
      (graphs && !prof && graphs->overlap[lane & 1].Ready()) ? &graphs->overlap[lane & 1] : nullptr;
    const bool envOnly = !shape.areaLights;
    const WaveGraphKey key{jobs, units, wb.ray[0], wb.capacity, shape.iters, shape.integrator, grid,
                           sort ? 1 : 0, accumulate ? 1 : 0, tailFrom, raster ? 1 : 0, envOnly ? 1 : 0};
    if (shape.iters >= 0) {
        auto record = [&](int* n) {
            RaygenKernel<<<grid, block, 0, stream>>>(jobs, units, wb, 0, raster ? 1 : 0);
            LaunchBounces(jobs, units, wb, shape.integrator, grid, 0, shape.iters, stream, prof, n, sort,
                          ov, envOnly, tailFrom, raster);
            if (accumulate) AccumulateKernel<<<grid, block, 0, stream>>>(jobs, units, wb);
            *n += accumulate ? 2 : 1;
        };
        if (useGraphs) {
            e = ReplayCaptured(graphs, key, stream, &nl, record);
        } else {
            if (ev) ev->Begin(0, stream);
            RaygenKernel<<<grid, block, 0, stream>>>(jobs, units, wb, 0, raster ? 1 : 0);
            if (ev) ev->End(0, stream);
            LaunchBounces(jobs, units, wb, shape.integrator, grid, 0, shape.iters, stream, prof, &nl, sort,
                          ov, envOnly, tailFrom, raster);
            if (accumulate) {
                if (ev) ev->Begin(4, stream);
                AccumulateKernel<<<grid, block, 0, stream>>>(jobs, units, wb);
                if (ev) ev->End(4, stream);
                nl++;
            }
            nl++;
        }
    } else {
        // SimplePathTracing has no depth cap: run blocks of bounces until the queue drains
        if (ev) ev->Begin(0, stream);
        RaygenKernel<<<grid, block, 0, stream>>>(jobs, units, wb, 0, 0);
        if (ev) ev->End(0, stream);
        nl++;
        for (int it = 0;; it += kPollEvery) {
            if (it > 0) {
                e = cudaMemcpyAsync(wb.hostCount, wb.counts, sizeof(int), cudaMemcpyDeviceToHost, stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess || *wb.hostCount == 0 || it >= kMaxReplayBounces) break;
            }
            if (useGraphs) {
                WaveGraphKey k = key;
                k.iters = -kPollEvery;
                e = ReplayCaptured(graphs, k, stream, &nl, [&](int* n) {
                    LaunchBounces(jobs, units, wb, shape.integrator, grid, 0, kPollEvery, stream, nullptr, n, sort,
                                  ov, envOnly);
                });
                if (e != cudaSuccess) break;
            } else {
                LaunchBounces(jobs, units, wb, shape.integrator, grid, it, kPollEvery, stream, prof, &nl, sort, ov,
                              envOnly);
            }
        }
        if (e == cudaSuccess && accumulate) {
            if (ev) ev->Begin(4, stream);
            AccumulateKernel<<<grid, block, 0, stream>>>(jobs, units, wb);
            if (ev) ev->End(4, stream);
            nl++;
        }
    }
    if (launches) *launches += nl;
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

cudaError_t FinalizeJobs(const DevJob* jobs, const int* jobList, int nJobs, int maxPixels,
                         cudaStream_t stream, int* launches, WaveProfile* prof) {
    if (nJobs <= 0) return cudaSuccess;
    StageEvents* ev = prof ? (StageEvents*)prof->events : nullptr;
    const int block = 256;
    const int gx = std::max(1, std::min(DefaultStageGrid(), (maxPixels + block - 1) / block));
    if (ev) ev->Begin(4, stream);
    FinalizeKernel<<<dim3(gx, nJobs), block, 0, stream>>>(jobs, jobList, maxPixels);
    if (ev) ev->End(4, stream);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t CollectProfile(WaveProfile* prof, cudaStream_t stream) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    StageEvents* ev = (StageEvents*)prof->events;
    if (ev) {
        ev->Collect(prof->ms);
        delete ev;
        prof->events = nullptr;
    }
    unsigned long long c[8];
    e = cudaMemcpy(c, prof->devCounters, sizeof(c), cudaMemcpyDeviceToHost);
    prof->refNodeTests = c[0];
    prof->refTriTests = c[1];
    prof->refRays = c[2];
    prof->extendRays = c[3];
    prof->shadowRays = c[4];
    return e;
}

void* NewStageEvents() { return new StageEvents(); }

// Each path's camera ray and first closest hit, in (pixel row-major, sample) order:
// index (y * W + x) * spp + s. Ties are settled in the reference's order, as the shade
// stage settles them.
__global__ void PrimaryOutKernel(const DevJob* __restrict__ jobs, WaveBuffers wb, int spp,
                                 float* __restrict__ raysOut, int* __restrict__ triOut,
                                 float* __restrict__ distOut) {
    const WaveDesc wd = *wb.desc;
    const DevJob& J = jobs[0];
    const int W = J.st.width, H = J.st.height;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < wd.nPaths; i += gridDim.x * blockDim.x) {
        const float4 a = wb.ray[0][2 * i], b = wb.ray[0][2 * i + 1];
        float2 h = wb.hit[i];
        if (__float_as_int(h.y) < -1) h = SettleTie(J, V3(a.x, a.y, a.z), V3(b.x, b.y, b.z), h);
        const int best = __float_as_int(h.y);
        int x, y;
        PixelOfIndex(i / spp, W, H, wd.band, x, y);
        const size_t o = ((size_t)y * W + x) * spp + i % spp;
        float* r = raysOut + 6 * o;
        r[0] = a.x;
        r[1] = a.y;
        r[2] = a.z;
        r[3] = b.x;
        r[4] = b.y;
        r[5] = b.z;
        triOut[o] = best >= 0 ? TriId(J.S.tris, best) : -1;
        distOut[o] = best >= 0 ? h.x : -1.0f;
    }
}

cudaError_t RunPrimaryHits(const DevJob* jobs, const WaveUnit* units, const WaveShape& shape,
                           const WaveBuffers& wb, const WaveTuning& tune, int spp, float* raysOut,
                           int* triOut, float* distOut, cudaStream_t stream, int* launches) {
    if (shape.nUnits != 1 || shape.nPaths <= 0 || shape.nPaths > wb.capacity)
        return cudaErrorInvalidValue;
    const int grid = StageGrid(tune);
    const bool raster = shape.raster > 0 && tune.primaryTraversal != 1 && tune.sortRays == 0 &&
                        shape.iters >= 0;
    WaveDesc d{};
    d.nUnits = shape.nUnits;
    d.nPaths = shape.nPaths;
    d.nPixelUnits = shape.nPixelUnits;
    d.soleJob = 0;
    d.band = tune.band > 0 ? tune.band : 8;
    d.rasterFrom = raster ? shape.rasterFrom : shape.nPaths;
    d.rasterUnit0 = raster ? shape.rasterUnit0 : shape.nUnits;
    d.rasterRecs = raster ? shape.raster : 0;
    cudaError_t e = cudaMemcpyAsync(wb.desc, &d, sizeof(d), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(wb.counts, 0, 16 * sizeof(int), stream);
    if (e != cudaSuccess) return e;
    RaygenKernel<<<grid, kTraceBlock, 0, stream>>>(jobs, units, wb, 0, raster ? 1 : 0);
    ExtendKernel<<<grid, kTraceBlock, 0, stream>>>(jobs, wb, 0, raster ? 1 : 0);
    int nl = 3;
    if (raster) {
        RasterSetupKernel<<<SmCount() * 32, kTraceBlock, 0, stream>>>(jobs, units, wb, 0);
        RasterVisitKernel<<<SmCount() * 16, kTraceBlock, 0, stream>>>(jobs, units, wb, 0);
        RasterFinishKernel<<<grid, kTraceBlock, 0, stream>>>(wb, 0);
        RetraceKernel<<<2 * SmCount(), kTraceBlock, 0, stream>>>(jobs, wb, 0);
        nl += 4;
    }
    PrimaryOutKernel<<<grid, kTraceBlock, 0, stream>>>(jobs, wb, spp, raysOut, triOut, distOut);
    if (launches) *launches += nl;
    return cudaGetLastError();
}

cudaError_t LaunchTraceClosest(const DevScene& S, int n, const float* rays, float distMin,
                               float distMax, int* triOut, float* distOut, int* fetchCounter,
                               cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(fetchCounter, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    TraceKernel<<<DefaultStageGrid(), 128, 0, stream>>>(S, n, rays, distMin, distMax, triOut, distOut,
                                                        fetchCounter);
    return cudaGetLastError();
}

}  // namespace ptg
