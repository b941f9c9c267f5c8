// Launch entry points of the CUDA kernels (host-callable, no torch types).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "pt_layout.h"

namespace ptg {

// Upper bound on the bounces of one replay path. SimplePathTracing has no depth
// cap (Russian roulette only), so a cap is needed to bound a GPU thread; with
// survival probability 0.9 per bounce past maxBounces it is never reached in
// practice, and hitting it sets a status bit instead of running on.
constexpr int kMaxReplayBounces = 1 << 16;
// Traversal stack depth of the throughput kernels (entries per ray).
constexpr int kWaveStackDepth = 64;

int NumTiles(const DevSettings& st);

// Reads `bytes` of `buf` (L2-resident sizes) `passes` times per launch, `reps` launches
// after one warm-up; *ms = CUDA-event time of the reps launches (probe.cu).
cudaError_t ProbeL2Read(const void* buf, size_t bytes, int passes, int reps, float* sink,
                        cudaStream_t stream, float* ms);

// Replay: one thread per tile in [tileBegin, tileEnd). stackScratch holds
// (tileEnd - tileBegin) * S.stackDepth ints. status receives error bits (OR).
cudaError_t LaunchReplay(const DevScene& S, const DevCamera& C, const DevSettings& st, float* film,
                         int* stackScratch, int* status, int tileBegin, int tileEnd,
                         cudaStream_t stream);

// AOV pass (0 UV, 1 denoising albedo, 2 denoising normal) of tiles [tileBegin, tileEnd):
// one thread per tile with the reference's per-tile stream; dspp = numSppForDenoising.
cudaError_t LaunchAov(const DevScene& S, const DevCamera& C, const DevSettings& st, int aov,
                      int dspp, float* film, int* stackScratch, int* status, int tileBegin,
                      int tileEnd, cudaStream_t stream);

// ---- wavefront (throughput) path
// A job is one image: its resident scene, camera, settings, per-pixel running
// sums and output film. Any number of jobs share a wave; every path carries its
// job index, and each job's pixels are summed in sample order, so a job's film
// does not depend on what else is in the wave.
struct DevJob {
    DevScene S;
    DevCamera C;
    DevSettings st;
    float4* accum;  // width*height running sums {rgb, 0}; zeroed before the job's first wave
    float* film;    // width*height*3 output, written by FinalizeJobs
    int32_t pad[4];
};

// One job's samples [s0, s0 + sw) over all its pixels: paths
// [pathBase, pathBase + W*H*sw) of the wave, pixel-major (pixel q of the band order owns
// paths pathBase + q*sw .. + sw - 1); pixelBase indexes the accumulate pass. recBase:
// for a unit whose first bounce is rasterised, its first per-triangle record in the
// raster scratch (the wave's raster units come last); -1 otherwise.
struct WaveUnit {
    int32_t job, s0, sw, pathBase;
    int32_t pixelBase, recBase, pad[2];
};

// Scalars of the wave being run, read by the kernels from device memory so that
// one captured launch sequence serves every wave of the same shape.
struct WaveDesc {
    int32_t nUnits, nPaths, nPixelUnits;
    int32_t soleJob;  // the wave's only job, or -1 (then read pathJob)
    int32_t band;     // rows per pixel band of the path order
    // rasterised first bounce: paths [rasterFrom, nPaths) of units [rasterUnit0, nUnits),
    // with rasterRecs per-triangle records in all
    int32_t rasterFrom, rasterUnit0, rasterRecs;
};

// Path state travels with its ray through the compacted queues (so the shade
// stage reads and writes it in queue order); only the radiance sum stays per
// path (written at termination and by next-event rays).
struct WaveBuffers {
    int capacity;                  // paths per wave
    float4* ray[2];                // per entry: {o.xyz, path}, {d.xyz, ior}
    float4* qs0[2];                // per entry: {T.xyz, prob}
    float4* qs1[2];                // per entry: {lastPdf, lastSin, bounce, flags}
    unsigned long long* qrng[2];   // per entry: random stream state
    float2* hit;                   // per entry of the current queue: {t, slot} (slot < 0: miss)
    float4* pathL;                 // per path: {L.xyz, flags}
    int* pathJob;                  // per path: job index
    struct WaveDesc* desc;         // the current wave's scalars (device)
    float4* shadow;                // 4 float4 per next-event entry
    int* counts;                   // [0],[1] ray queues; [2] shadow queue; [3] error bits; [4],[5] fetch
    int* hostCount;                // pinned host word for queue-size polls
    unsigned* sortKey;             // per entry of the next queue: coherence key (ray sorting)
    unsigned* sortBins;            // kSortBins counts, then kSortBins offsets
    size_t bytes;                  // size of the allocation carved (0: unknown)
};
// Bins of the ray-coherence key: 64 direction cells x 4096 origin cells.
constexpr int kSortOriginBits = 12;
constexpr int kSortBins = 64 << kSortOriginBits;
// Device bytes of the wave buffers for `capacity` paths, and their carving out of
// one 256-byte-aligned allocation (hostCount is left for the caller).
size_t WaveBuffersBytes(int capacity);
WaveBuffers CarveWaveBuffers(void* base, int capacity);
// Bytes for `capacity` paths that also hold two sets of capacity / 2 (two wave lanes).
size_t WaveBuffersBytesTwoLanes(int capacity);


// Optional per-stage profile (CUDA events around every stage launch; ray tallies;
// reference-order traversal work over the extended rays).
struct WaveProfile {
    double ms[6] = {0, 0, 0, 0, 0, 0};  // raygen, extend, shade, shadow, accumulate+finalize, raster
    unsigned long long extendRays = 0, shadowRays = 0, extendLaunches = 0, shadowLaunches = 0;
    unsigned long long rasterPaths = 0;  // first-bounce paths settled by the raster kernels
    unsigned long long refNodeTests = 0, refTriTests = 0, refRays = 0;
    bool countReference = false;
    unsigned long long* devCounters = nullptr;  // 8 device words, zeroed by the caller
    void* events = nullptr;                     // internal
};

// What one wave runs. iters >= 0: that many bounce iterations; iters < 0: until
// the ray queue drains (polled every 4 iterations). integrator: the one integrator
// of all the wave's jobs, or -1 when they differ; soleJob: the wave's only job, or -1.
struct WaveShape {
    int nUnits = 0, nPaths = 0, nPixelUnits = 0;
    int iters = 0, integrator = -1, soleJob = -1;
    int areaLights = 1;  // 0: no job of the wave has area lights (next-event rays are any-hit)
    // > 0: the first bounce of units [rasterUnit0, nUnits) (paths [rasterFrom, nPaths)) may
    // be rasterised (raster_primary.cuh); raster = their per-triangle records in all
    int raster = 0, rasterFrom = 0, rasterUnit0 = 0;
};
// Launch configuration (all choices give the same films). 0 = default.
struct WaveTuning {
    int blocksPerSm = 0;  // stage grid: blocks of 128 threads per SM (0: occupancy of the trace kernels)
    int band = 0;         // rows per pixel band of the path order (0: 8)
    int graphs = 1;       // replay each wave's stage sequence from a captured CUDA graph
    int sortRays = 0;     // reorder each bounce's rays by direction and origin cell before tracing
    int tailBounce = 0;   // > 0: from this bounce on, one launch finishes every path (TailKernel)
    // first bounce: 0 rasterised for units with enough rays per triangle, else traced;
    // 1 always traced through the BVH; 2 rasterised wherever the camera allows it
    int primaryTraversal = 0;
};
// Captured stage sequences, keyed by wave shape and buffers (owned by a context or server).
struct WaveGraphCache;
WaveGraphCache* NewWaveGraphCache();
void FreeWaveGraphCache(WaveGraphCache* cache);

// One wave: raygen over `units` (device), the bounce loop, and (accumulate) the
// accumulation into each job's sums. With a cache and no profile, the launches of each
// wave shape are captured once into a CUDA graph and replayed. lane (0 or 1) picks the
// cache's shadow-stage side stream for waves run on two streams at once.
cudaError_t RunWave(const DevJob* jobs, const WaveUnit* units, const WaveShape& shape,
                    const WaveBuffers& wb, cudaStream_t stream, int* launches, WaveProfile* prof,
                    const WaveTuning& tune, WaveGraphCache* graphs, int lane = 0,
                    bool accumulate = true);
// The accumulation pass of a wave run with accumulate = false.
cudaError_t AccumulateWave(const DevJob* jobs, const WaveUnit* units, const WaveBuffers& wb,
                           const WaveTuning& tune, cudaStream_t stream, int* launches);
// The cache's second wave stream and the two lanes' completion events (created on
// first use); false when they cannot be had.
bool WavePipeline(WaveGraphCache* cache, cudaStream_t* side, cudaEvent_t* done);
// into.counts[3] = a.counts[3] | b.counts[3] (error bits of two wave lanes).
cudaError_t MergeWaveErrors(const WaveBuffers& into, const WaveBuffers& a, const WaveBuffers& b,
                            cudaStream_t stream);
// film = accum / spp for the listed jobs (device list of job indices).
cudaError_t FinalizeJobs(const DevJob* jobs, const int* jobList, int nJobs, int maxPixels,
                         cudaStream_t stream, int* launches, WaveProfile* prof);
// Collects the profile's events and counters (synchronises the stream).
cudaError_t CollectProfile(WaveProfile* prof, cudaStream_t stream);

int DefaultStageGrid();
int StageGrid(const WaveTuning& tune);

// The first bounce of a one-job, one-wave render (units: its one unit; shape as RunWave
// takes it): raygen, then the closest hit of every camera ray (rasterised or traced as a
// render would), written out per (pixel row-major, sample): the ray (6 floats), the
// original triangle index (or -1) and the distance (or -1).
cudaError_t RunPrimaryHits(const DevJob* jobs, const WaveUnit* units, const WaveShape& shape,
                           const WaveBuffers& wb, const WaveTuning& tune, int spp, float* raysOut,
                           int* triOut, float* distOut, cudaStream_t stream, int* launches);

// Closest-hit traversal of the throughput path for caller rays (o.xyz, d.xyz per ray).
// fetchCounter: one device int of scratch for the persistent fetch.
cudaError_t LaunchTraceClosest(const DevScene& S, int n, const float* rays, float distMin,
                               float distMax, int* triOut, float* distOut, int* fetchCounter,
                               cudaStream_t stream);

// Fixed scratch of the no-allocation replay render (noalloc.cu): status word and
// stack area addresses on the current device; capacity of the stack area in ints.
cudaError_t NoAllocScratch(int** statusOut, int** stacksOut);
size_t NoAllocScratchInts();

}  // namespace ptg
