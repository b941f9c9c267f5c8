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

// Replay: one thread per tile in [tileBegin, tileEnd). stackScratch holds
// (tileEnd - tileBegin) * S.stackDepth ints. status receives error bits (OR).
cudaError_t LaunchReplay(const DevScene& S, const DevCamera& C, const DevSettings& st, float* film,
                         int* stackScratch, int* status, int tileBegin, int tileEnd,
                         cudaStream_t stream);

// ---- wavefront (throughput) path
struct WaveBuffers {
    int capacity;       // paths per wave
    float4* ray[2];     // 2 float4 per entry: {o.xyz, path}, {d.xyz, 0}
    float2* hit;        // {t, slot} per ray entry (slot < 0: miss)
    float4* st0;        // per path {T.xyz, prob}
    float4* st1;        // per path {L.xyz, ior}
    float4* st2;        // per path {lastPdf, lastSin, bounce, flags}
    unsigned long long* rng;  // per path
    float4* shadow;     // 4 float4 per shadow entry
    int* counts;        // [0],[1] ray queue sizes; [2] shadow queue size; [3] error bits
    float4* accum;      // per pixel running sum {rgb, 0}
    int* hostCount;     // pinned host word for queue-size polls
};
size_t WaveBytesPerPath();
size_t WaveBytesPerPixel();

// Optional per-stage profile of one wavefront render (CUDA events around every
// stage launch; ray tallies; reference-order traversal work over the extended rays).
struct WaveProfile {
    double ms[5] = {0, 0, 0, 0, 0};  // raygen, extend, shade, shadow, accumulate+finalize
    unsigned long long extendRays = 0, shadowRays = 0, extendLaunches = 0, shadowLaunches = 0;
    unsigned long long refNodeTests = 0, refTriTests = 0, refRays = 0;
    bool countReference = false;
    unsigned long long* devCounters = nullptr;  // 8 device words, zeroed by the caller
};

// Renders one image through the wavefront stages into film (device, W*H*3).
// grid: persistent grid size for the stage kernels (0 = auto). prof may be null;
// with a profile the call synchronises the stream before returning.
// wavePaths: paths per wave (<= wb.capacity; 0 = wb.capacity).
cudaError_t RenderWavefront(const DevScene& S, const DevCamera& C, const DevSettings& st,
                            const WaveBuffers& wb, float* film, cudaStream_t stream,
                            int* launches, int gridOverride, WaveProfile* prof = nullptr,
                            int wavePaths = 0);

// Closest-hit traversal of the throughput path for caller rays (o.xyz, d.xyz per ray).
cudaError_t LaunchTraceClosest(const DevScene& S, int n, const float* rays, float distMin,
                               float distMax, int* triOut, float* distOut, cudaStream_t stream);

int DefaultStageGrid();

// Fixed scratch of the no-allocation replay render (noalloc.cu): status word and
// stack area addresses on the current device; capacity of the stack area in ints.
cudaError_t NoAllocScratch(int** statusOut, int** stacksOut);
size_t NoAllocScratchInts();

}  // namespace ptg
