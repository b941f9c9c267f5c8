// Primary visibility by rasterisation (included by wavefront.cu inside namespace ptg).
//
// The first bounce of a wave unit whose job looks through a pinhole (every primary ray
// starts at the camera position) is computed by visiting, for each triangle, the
// samples whose rays can reach it, instead of tracing each ray through the BVH. The
// wave's rasterised units come after its traced ones (PrepareRasterUnits), so the extend
// kernel traces paths [0, rasterFrom) and these kernels settle [rasterFrom, nPaths):
//   setup  one thread per (unit, triangle): the three planes through the camera and the
//          triangle's edges (the cone a ray must lie in to hit it, widened by a small
//          angular margin) and the rectangle of pixels it covers (its vertices
//          projected with the camera's own mapping, one pixel of margin for the sample
//          offsets; the whole image when it reaches the camera plane); the rectangle is
//          cut into row segments of at most kRasterSeg pixels, appended to a work list;
//   visit  one warp per segment: the lanes step through the segment's (pixel, sample)
//          pairs, test each direction against the cone, and for those inside run the
//          exact triangle test of the traversal (TriIntersect) and keep the nearest hit
//          with a 64-bit atomic minimum over {distance bits, slot};
//   finish one thread per path: the nearest hit into the hit queue, an exact tie with
//          another triangle marked as the traversal marks it (a second minimum over
//          {distance bits, ~slot} holds the largest slot at the nearest distance: a tie
//          when it differs from the smallest).
// The cone test only skips pairs whose ray certainly misses, and every remaining pair
// runs the same triangle test with the same ray, so a sample's closest distance and
// triangle are the traversal's (which, with its widened boxes, also finds every hit).
// Scratch: the next queue's ray buffer holds the two keys (16 of its 32 bytes per path);
// the shadow queue holds the per-triangle records and the work list.
// Both are free until the first shade. Paths are in pixel-major order, so a pixel's
// samples are consecutive queue entries and their directions are read where raygen
// wrote them.
#pragma once

constexpr int kRasterSeg = 32;   // pixels per work item (one row segment)
constexpr int kRasterBatch = 2;  // (pixel, sample) pairs a lane loads before testing them
constexpr int kRasterRecF4 = 4;    // float4 per per-triangle record
constexpr unsigned long long kNoKey = ~0ull;
constexpr unsigned kUncertain = 0x80000000u;  // key bit: the hit may lie outside its leaf box
constexpr unsigned kNoItem = ~0u;  // an empty work-list slot

struct RasterScratch {
    unsigned long long* key;   // per path: min {distance bits, slot}, kNoKey = no hit
    unsigned long long* key2;  // per path: min {distance bits, ~slot}
    int* retrace;              // paths whose nearest hit is uncertain (RetraceKernel)
    float4* rec;               // per triangle: kRasterRecF4 float4 (cone planes with margins,
                               // pixel rect)
    uint4* items;              // {triangle slot, unit, row | segment << 16, xa | xb << 16}
    int2* overflow;           // {triangle slot, unit} whose items did not fit (visited whole)
    long long itemCap;
};

// numRecs: the wave's per-triangle records over all its rasterised units.
__device__ __forceinline__ RasterScratch CarveRaster(const WaveBuffers& wb, int cur, int numRecs) {
    const size_t C = (size_t)wb.capacity;
    RasterScratch r;
    r.key = reinterpret_cast<unsigned long long*>(wb.ray[cur ^ 1]);
    r.key2 = r.key + C;
    r.retrace = reinterpret_cast<int*>(r.key2 + C);  // the ray buffer's second half
    r.rec = wb.shadow;
    const size_t over = ((size_t)numRecs + 1) & ~(size_t)1;  // int2 entries, 16-byte multiple
    r.overflow = reinterpret_cast<int2*>(wb.shadow + kRasterRecF4 * (size_t)numRecs);
    r.items = reinterpret_cast<uint4*>(r.overflow + over);
    const long long bytes = (long long)(64 * C) - 16LL * kRasterRecF4 * numRecs - 8LL * (long long)over;
    r.itemCap = bytes > 0 ? bytes / 16 : 0;
    return r;
}

// The rasterised unit that owns record r (units [u0, n) with ascending recBase).
__device__ __forceinline__ int RasterUnitOf(const WaveUnit* __restrict__ units, int u0, int n, int r) {
    int lo = u0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (units[mid].recBase <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Pixel coordinate (continuous, origin at the image corner) of a point with camera-basis
// coordinates (X, Y, Z) (multiples of right, up, forward), Z > 0: the inverse of
// GenerateRay's sensor mapping.
__device__ __forceinline__ void ProjectPx(const DevCamera& c, float X, float Y, float Z, int W, int H,
                                          float& px, float& py) {
    const float aspect = (float)W / H;
    px = (X / (Z * c.hPerf * aspect) + 0.5f) * W;
    py = (-Y / (Z * c.hPerf) + 0.5f) * H;
    px = fminf(fmaxf(px, -1.0e9f), 1.0e9f);
    py = fminf(fmaxf(py, -1.0e9f), 1.0e9f);
}

__global__ void __launch_bounds__(128) RasterSetupKernel(const DevJob* __restrict__ jobs,
                                                         const WaveUnit* __restrict__ units,
                                                         WaveBuffers wb, int cur) {
    const WaveDesc wd = *wb.desc;
    const int R = wd.rasterRecs;
    const RasterScratch rs = CarveRaster(wb, cur, R);
    const int lane = threadIdx.x & 31;
    // whole warps step together (the item appends are warp-aggregated)
    for (int base = blockIdx.x * blockDim.x; base < R; base += gridDim.x * blockDim.x) {
        const int rec = base + threadIdx.x;
        int nItems = 0, unit = 0, k = 0;
        int x0 = 0, x1 = -1, y0 = 0, y1 = -1;
        if (rec < R) {
            unit = RasterUnitOf(units, wd.rasterUnit0, wd.nUnits, rec);
            k = rec - units[unit].recBase;
            const DevJob& J = jobs[units[unit].job];
            const DevScene& S = J.S;
            const int W = J.st.width, H = J.st.height;
            const V3 pos = LoadV3(J.C.pos), right = LoadV3(J.C.right), up = LoadV3(J.C.up),
                     fwd = LoadV3(J.C.fwd);
            const float rr = 1.0f / SqLenRn(right), uu = 1.0f / SqLenRn(up);
            V3 v0, e1, e2;
            LoadTri(S.tris, k, v0, e1, e2);
            const V3 a[3] = {v0 - pos, (v0 + e1) - pos, (v0 + e2) - pos};
            // the plane through the camera and edge k is a_k x a_k+1 = a_k x (edge k): formed
            // from the short edge vector it has no cancellation (the cross product of two
            // long, nearly parallel vectors from a distant camera would lose most digits)
            V3 n[3] = {CrossRn(a[0], e1), CrossRn(a[1], e2 - e1), CrossRn(a[2], e2 * -1.0f)};
            const V3 ce = CrossRn(e1, e2);
            const float side = DotRn(a[0], ce);  // which side of the triangle the camera is on
            float m[3];
            if (fabsf(side) > 1.0e-5f * sqrtf(__fmul_rn(SqLenRn(a[0]), SqLenRn(ce)))) {
                const float sg = side > 0.0f ? 1.0f : -1.0f;
                // The triangle test's rounding reaches outside the triangle: for a point
                // of the plane, n_e . d equals its barycentric coordinate opposite edge e
                // times |side| / t, and the test's barycentric error is at most a few ulps
                // of (|v0 - camera| + |edge|) |edge| t / |side|, so an absolute margin of
                // 2^-19 max|edge| (|v0 - camera| + max|edge|) (32 ulps of that) covers it
                // whatever the triangle's shape (a sliver's short edge has a small n_e).
                const float emax = sqrtf(fmaxf(fmaxf(SqLenRn(e1), SqLenRn(e2)), SqLenRn(e2 - e1)));
                const float mt = ldexpf(emax * (sqrtf(SqLenRn(a[0])) + emax), -19);
                for (int e = 0; e < 3; e++) {
                    n[e] = n[e] * sg;
                    m[e] = 2.0e-5f * sqrtf(SqLenRn(n[e])) + mt;  // angular margin ~2e-5 rad
                }
            } else {  // camera (nearly) in the triangle's plane, or a degenerate triangle: no cone test
                for (int e = 0; e < 3; e++) {
                    n[e] = V3(0.f, 0.f, 0.f);
                    m[e] = 1.0f;
                }
            }
            // coordinates in the camera basis: right and up are orthogonal to forward but not
            // unit length (Camera::SetViewDir crosses forward with the world up), and
            // GenerateRay scales them as they are
            float X[3], Y[3], Z[3], zmax = 0.0f;
            bool front = true, anyFront = false;
            for (int v = 0; v < 3; v++) {
                X[v] = __fmul_rn(DotRn(a[v], right), rr);
                Y[v] = __fmul_rn(DotRn(a[v], up), uu);
                Z[v] = DotRn(a[v], fwd);
                zmax = fmaxf(zmax, fabsf(Z[v]));
            }
            const float zc = 1.0e-6f * zmax + 1.0e-30f;
            for (int v = 0; v < 3; v++) {
                front = front && Z[v] > zc;
                anyFront = anyFront || Z[v] > 0.0f;
            }
            // pixel rectangle of the vertices' projections; a triangle reaching the camera
            // plane gets the whole image (primary rays only meet points in front, so one
            // wholly behind gets none)
            if (front) {
                float lx = 3.0e38f, hx = -3.0e38f, ly = 3.0e38f, hy = -3.0e38f;
                for (int v = 0; v < 3; v++) {
                    float px, py;
                    ProjectPx(J.C, X[v], Y[v], Z[v], W, H, px, py);
                    lx = fminf(lx, px);
                    hx = fmaxf(hx, px);
                    ly = fminf(ly, py);
                    hy = fmaxf(hy, py);
                }
                // a sample of pixel i sits at i + r, r in [0, 1]: pixels floor(px) - 1 .. floor(px)
                x0 = max(0, (int)floorf(lx - 0.01f) - 1);
                x1 = min(W - 1, (int)floorf(hx + 0.01f));
                y0 = max(0, (int)floorf(ly - 0.01f) - 1);
                y1 = min(H - 1, (int)floorf(hy + 0.01f));
            } else if (anyFront) {
                x0 = 0;
                x1 = W - 1;
                y0 = 0;
                y1 = H - 1;
            }
            if (x0 <= x1 && y0 <= y1) {
                nItems = (y1 - y0 + 1) * ((x1 - x0 + kRasterSeg) / kRasterSeg);
                float4* r = rs.rec + kRasterRecF4 * (size_t)rec;
                r[0] = make_float4(n[0].x, n[0].y, n[0].z, m[0]);
                r[1] = make_float4(n[1].x, n[1].y, n[1].z, m[1]);
                r[2] = make_float4(n[2].x, n[2].y, n[2].z, m[2]);
                r[3] = make_float4(__int_as_float(x0), __int_as_float(x1), __int_as_float(y0),
                                   __int_as_float(y1));
            }
        }
        // warp-aggregated reservation of the work list (a 64-bit count in counts[8..9])
        int incl = nItems;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(kFullMask, incl, 31);
        unsigned long long wbase = 0;
        if (lane == 31 && total > 0)
            wbase = atomicAdd(reinterpret_cast<unsigned long long*>(wb.counts + 8), (unsigned long long)total);
        wbase = __shfl_sync(kFullMask, wbase, 31);
        if (nItems > 0) {
            const long long first = (long long)wbase + incl - nItems;
            if (first + nItems <= rs.itemCap) {
                const int segs = (x1 - x0 + kRasterSeg) / kRasterSeg;
                long long it = first;
                for (int y = y0; y <= y1; y++)
                    for (int sgi = 0; sgi < segs; sgi++) {
                        const int xa = x0 + sgi * kRasterSeg, xb = min(x1, xa + kRasterSeg - 1);
                        rs.items[it++] = make_uint4((unsigned)k, (unsigned)unit,
                                                    (unsigned)y | ((unsigned)sgi << 16),
                                                    (unsigned)xa | ((unsigned)xb << 16));
                    }
            } else {
                // the list is full: the triangle is visited whole; the part of its
                // reservation that lies inside the list is marked empty, so every slot the
                // visit kernel reads was written
                for (long long it = first; it < rs.itemCap; it++) rs.items[it] = make_uint4(kNoItem, 0u, 0u, 0u);
                const int o = atomicAdd(wb.counts + 10, 1);
                rs.overflow[o] = make_int2(k, unit);
            }
        }
    }
}

// Whether the hit point at distance t is certainly inside the triangle's leaf box, the box
// whose entry distance the traversal tests before it tests the triangle: the point lies
// within the triangle's own bounds widened by g, the leaf box's widening (the record's
// eps) less 2^-20 (|o| + |coordinates|), which exceeds the rounding of the point, of
// v0 + e1 and of the traversal's slab distances (a few ulps each). A hit the triangle test
// accepts elsewhere (its rounding can reach far outside a triangle met at a grazing angle)
// is found by the traversal or not depending on the order it visits boxes in; such a
// path is traced instead (RetraceKernel), which gives the traversal's own answer.
// The bounds are formed once per triangle (TriangleNearBox); lo > hi when g <= 0.
struct NearBox {
    V3 lo, hi;
};
__device__ __forceinline__ NearBox TriangleNearBox(V3 v0, V3 e1, V3 e2, V3 o, float wideEps) {
    const V3 v1 = v0 + e1, v2 = v0 + e2;
    NearBox b;
    b.lo = V3(Min3(v0.x, v1.x, v2.x), Min3(v0.y, v1.y, v2.y), Min3(v0.z, v1.z, v2.z));
    b.hi = V3(Max3(v0.x, v1.x, v2.x), Max3(v0.y, v1.y, v2.y), Max3(v0.z, v1.z, v2.z));
    const float m = Max3(fabsf(o.x), fabsf(o.y), fabsf(o.z)) +
                    fmaxf(Max3(fabsf(b.lo.x), fabsf(b.lo.y), fabsf(b.lo.z)),
                          Max3(fabsf(b.hi.x), fabsf(b.hi.y), fabsf(b.hi.z)));
    const float g = wideEps - ldexpf(m, -20);
    if (g > 0.0f) {
        b.lo = b.lo - V3(g, g, g);
        b.hi = b.hi + V3(g, g, g);
    } else {
        b.lo = V3(1.f, 1.f, 1.f);
        b.hi = V3(-1.f, -1.f, -1.f);
    }
    return b;
}
__device__ __forceinline__ bool HitNearTriangle(const NearBox& b, V3 o, V3 d, float t) {
    const V3 p = o + d * t;
    return p.x >= b.lo.x && p.x <= b.hi.x && p.y >= b.lo.y && p.y <= b.hi.y && p.z >= b.lo.z &&
           p.z <= b.hi.z;
}

// Visits one row segment of triangle k: every (pixel, sample) pair of the wave's unit.
// Pixel (x, y) is pixel q = qrow + x * hb of the band order (PixelOfIndex), and its
// samples are paths pathBase + q * sw + j, whose directions are in the ray queue.
__device__ __forceinline__ void RasterSegment(const RasterScratch& rs, const float4* __restrict__ rays,
                                             const DevScene& S, int k, int rec, int y,
                                             int xa, int xb, int W, int H, int band, int pathBase,
                                             int sw, V3 o, float tmin, int lane) {
    const float4* rp = rs.rec + kRasterRecF4 * (size_t)rec;
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
    V3 v0, e1, e2;
    LoadTri(S.tris, k, v0, e1, e2);
    const NearBox nb = TriangleNearBox(v0, e1, e2, o, S.wideEps);
    const int y0 = (y / band) * band, hb = min(band, H - y0);
    const size_t qrow = (size_t)y0 * W + (y - y0);
    const int n = (xb - xa + 1) * sw;
    // (pixel, sample) of pair f = lane + 32 i, advanced without a division per pair
    const int dq = 32 / sw, dr = 32 % sw;
    int x = xa + lane / sw, j = lane % sw;
    // kRasterBatch pairs per lane at a time: their directions are loaded before any is
    // tested, so the loads' latencies overlap; the minima are fire-and-forget reductions
    for (int f0 = lane; f0 < n; f0 += 32 * kRasterBatch) {
        float4 dv[kRasterBatch];
        size_t idx[kRasterBatch];
#pragma unroll
        for (int b = 0; b < kRasterBatch; b++) {
            idx[b] = (size_t)pathBase + (qrow + (size_t)x * hb) * sw + j;
            if (f0 + 32 * b < n) dv[b] = __ldg(rays + 2 * idx[b] + 1);
            j += dr;
            x += dq;
            if (j >= sw) {
                j -= sw;
                x++;
            }
        }
#pragma unroll
        for (int b = 0; b < kRasterBatch; b++) {
            if (f0 + 32 * b >= n) break;
            const float c0 = r0.x * dv[b].x + r0.y * dv[b].y + r0.z * dv[b].z + r0.w;
            const float c1 = r1.x * dv[b].x + r1.y * dv[b].y + r1.z * dv[b].z + r1.w;
            const float c2 = r2.x * dv[b].x + r2.y * dv[b].y + r2.z * dv[b].z + r2.w;
            if (c0 >= 0.0f && c1 >= 0.0f && c2 >= 0.0f) {
                float t;
                const V3 d(dv[b].x, dv[b].y, dv[b].z);
                if (TriIntersect(v0, e1, e2, o, d, t) && t >= tmin && t < kFltMax) {
                    // a hit point not certainly inside the triangle's leaf box is marked
                    // (kUncertain); the path is traced if such a hit is its nearest
                    const unsigned w = (unsigned)k | (HitNearTriangle(nb, o, d, t) ? 0u : kUncertain);
                    // t + 0: a zero distance as +0, so that distance bits order as floats
                    const unsigned long long tb = (unsigned long long)__float_as_uint(t + 0.0f) << 32;
                    atomicMin(rs.key + idx[b], tb | w);
                    atomicMin(rs.key2 + idx[b], tb | ~w);
                }
            }
        }
    }
}

// One work item's (row segment's) unit: its job's scene, camera and image, its paths.
__device__ __forceinline__ void RasterItem(const DevJob* __restrict__ jobs, const WaveUnit& u,
                                          const RasterScratch& rs, const float4* __restrict__ rays,
                                          int band, int k, int y, int xa, int xb, int lane) {
    const DevJob& J = jobs[u.job];
    const float tmin = J.st.integrator == kSimplePathTracing ? kEps : 0.0f;
    RasterSegment(rs, rays, J.S, k, u.recBase + k, y, xa, xb, J.st.width, J.st.height, band,
                  u.pathBase, u.sw, LoadV3(J.C.pos), tmin, lane);
}

__global__ void __launch_bounds__(128) RasterVisitKernel(const DevJob* __restrict__ jobs,
                                                         const WaveUnit* __restrict__ units,
                                                         WaveBuffers wb, int cur) {
    const WaveDesc wd = *wb.desc;
    const RasterScratch rs = CarveRaster(wb, cur, wd.rasterRecs);
    const float4* rays = wb.ray[cur];
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    long long nItems = *reinterpret_cast<const long long*>(wb.counts + 8);
    if (nItems > rs.itemCap) nItems = rs.itemCap;
    // the next item is loaded while the current one is visited
    uint4 next = warp < nItems ? rs.items[warp] : make_uint4(kNoItem, 0u, 0u, 0u);
    for (long long w = warp; w < nItems; w += warps) {
        const uint4 it = next;
        if (w + warps < nItems) next = rs.items[w + warps];
        if (it.x == kNoItem) continue;
        const int k = (int)it.x, y = (int)(it.z & 0xffffu);
        const WaveUnit u = units[it.y];
#if PT_CHECK
        if (k < 0 || k >= jobs[u.job].S.numTris) continue;
#endif
        RasterItem(jobs, u, rs, rays, wd.band, k, y, (int)(it.w & 0xffffu), (int)(it.w >> 16), lane);
    }
    // triangles whose items did not fit in the list: whole, one warp each
    const int nOver = wb.counts[10];
    for (long long w = warp; w < nOver; w += warps) {
        const int2 ov = rs.overflow[w];
        const WaveUnit u = units[ov.y];
        const float4 r3 = __ldg(rs.rec + kRasterRecF4 * (size_t)(u.recBase + ov.x) + 3);
        const int x0 = __float_as_int(r3.x), x1 = __float_as_int(r3.y), y0 = __float_as_int(r3.z),
                  y1 = __float_as_int(r3.w);
        for (int y = y0; y <= y1; y++)
            for (int xa = x0; xa <= x1; xa += kRasterSeg)
                RasterItem(jobs, u, rs, rays, wd.band, ov.x, y, xa, min(x1, xa + kRasterSeg - 1), lane);
    }
}

// The nearest hit of every path into the hit queue (queue entry i = path i at the first
// bounce), as ExtendKernel would write it: {distance, slot}, {kFltMax, -1} for a miss,
// -2 - slot when another triangle tied at that distance. A path whose hits at the nearest
// distance include an uncertain one goes to the retrace list instead.
// Whole warps step together (the list appends are warp-aggregated).
__global__ void RasterFinishKernel(WaveBuffers wb, int cur) {
    const WaveDesc wd = *wb.desc;
    const RasterScratch rs = CarveRaster(wb, cur, wd.rasterRecs);
    const int n = wd.nPaths;
    if (blockIdx.x == 0 && threadIdx.x == 0) wb.counts[cur ^ 1] = 0;
    for (int b = wd.rasterFrom + blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const int i = b + threadIdx.x;
        bool retrace = false;
        if (i < n) {
            const unsigned long long key = rs.key[i];
            float2 h = make_float2(kFltMax, __int_as_float(-1));
            if (key != kNoKey) {
                const unsigned tb = (unsigned)(key >> 32);
                const unsigned w1 = (unsigned)key, w2 = ~(unsigned)rs.key2[i];  // min and max word
                const int slot = (int)(w1 & ~kUncertain);
                retrace = ((w1 | w2) & kUncertain) != 0;
                h = make_float2(__uint_as_float(tb), __int_as_float(w1 != w2 ? -2 - slot : slot));
            }
            wb.hit[i] = h;
        }
        const int at = WarpAppend(wb.counts + 11, retrace);
        if (retrace) rs.retrace[at] = i;
    }
}

