// The context behind the C ABI and the helpers shared by capi.cpp and server.cpp.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "petrichor_gb300.h"
#include "pt_kernels.h"
#include "scheduler.h"

namespace ptg {

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct SceneGpu {
    DevScene dev{};
    std::vector<DeviceBuffer> buffers;
    pt_scene_info info{};
    std::atomic<int> refs{0};  // serving requests that use the scene
    // alias table of the optional environment sampler, built at the first render that
    // asks for it (owned by buffers)
    const float4* envAlias = nullptr;
};

class Server;  // server.cpp

// Paths per wave: the whole image x spp when it fits, otherwise full sample blocks.
// 2^27 paths hold a 1920x1080 frame at 64 spp in one wave (about 32 GB of state).
#ifndef PT_MAX_WAVE_LOG2
#define PT_MAX_WAVE_LOG2 27
#endif
constexpr int64_t kMaxWavePaths = int64_t(1) << PT_MAX_WAVE_LOG2;
constexpr int kMaxJobsPerCall = 4096;
constexpr int kMaxUnitsPerWave = 8192;

}  // namespace ptg

struct pt_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;  // 0 = unlimited
    uint64_t used = 0;
    std::mutex mu;  // serialises device work and the scene table
    std::string lastError;
    std::map<int, std::unique_ptr<ptg::SceneGpu>> scenes;
    int nextId = 1;
    // wavefront buffers
    ptg::WaveBuffers wb{};
    std::vector<ptg::DeviceBuffer> wbBuffers;
    int wbCapacity = 0;
    // scratch for host-film renders and replay stacks
    ptg::DeviceBuffer film, stack, status;
    // wavefront job tables and per-job running sums
    ptg::DeviceBuffer jobTable, unitTable, jobList, accum;
    // launch configuration (pt_autotune / pt_set_tuning) and captured wave sequences
    ptg::WaveTuning tuning{};
    int tunedWavePaths = 0;  // 0: the automatic wave size
    double tunedProbeMs = 0.0;
    ptg::WaveGraphCache* graphs = nullptr;
    int bvhBuilder = PT_BVH_BUILDER_DEVICE;
    ptg::DeviceBuffer denoiseScratch, denoiseImages;  // pt_denoise
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    pt_stats stats{};
    uint32_t tilesDone = 0, tilesTotal = 0;
    // status word of the last no-allocation replay render (inside the fixed device
    // array), read back by pt_get_stats once ev1 has completed
    int* noallocStatus = nullptr;
    std::atomic<bool> noallocPending{false};
    std::unique_ptr<ptg::Server> server;
    // defined where ptg::Server is complete (server.cpp)
    pt_context();
    ~pt_context();
};

namespace ptg {

int Fail(pt_context* ctx, int code, const std::string& msg);
int CudaFail(pt_context* ctx, cudaError_t e, const char* what);
// Allocation counted against the context's budget (ctx->mu held).
int Alloc(pt_context* ctx, DeviceBuffer& b, size_t bytes);
void Free(pt_context* ctx, DeviceBuffer& b);
int SetDevice(pt_context* ctx);
int EnsureWaveBuffers(pt_context* ctx, int capacity);
int CheckArgs(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
              SceneGpu** out);
DevCamera ToDev(const pt_camera* c);
DevSettings ToDev(const pt_settings* s);
// The scene as one job sees it: the environment alias table attached when the
// settings ask for it (CheckArgs has built it).
DevScene JobScene(const SceneGpu& s, const pt_settings* st);

}  // namespace ptg
