// Scratch memory for the replay render that allocates nothing.
//
// Some callers cannot allocate device memory at render time: a render issued
// while another library owns the device allocator and has reserved all memory, a
// host thread that must not block on the driver's allocation lock (cudaMalloc
// and cudaFree synchronise the device), or code that was handed a fixed memory
// envelope up front. pt_render_replay_noalloc serves them: it uses the caller's
// film, the scene that is already resident, and this fixed array for the
// traversal stacks and the status word.
//
// The array is a file-scope __device__ variable of fixed size, so every GPU that
// loads this library holds it until the process exits. In host code its name is
// only a host-side stand-in: the device address is taken with
// cudaGetSymbolAddress, once per device, with that device current (the first
// call on a device does this). All calls share the one array and it keeps the
// previous call's contents: the status word is cleared on the stream before each
// launch, and calls that overlap on the GPU (different streams, no ordering)
// race on the stacks.
#include <cuda_runtime.h>

#include <mutex>

#include "pt_kernels.h"

namespace ptg {

// 16 status words followed by the traversal stacks: 4 MiB in total.
constexpr size_t kNoAllocScratchInts = size_t(1) << 20;
constexpr size_t kNoAllocStatusInts = 16;
static __device__ __align__(256) int g_noAllocScratch[kNoAllocScratchInts];

namespace {
std::mutex g_mu;
constexpr int kMaxDevices = 64;
int* g_scratchAddr[kMaxDevices] = {};
}  // namespace

size_t NoAllocScratchInts() { return kNoAllocScratchInts - kNoAllocStatusInts; }

cudaError_t NoAllocScratch(int** statusOut, int** stacksOut) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratchAddr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noAllocScratch);
        if (e != cudaSuccess) return e;
        g_scratchAddr[dev] = static_cast<int*>(p);
    }
    *statusOut = g_scratchAddr[dev];
    *stacksOut = g_scratchAddr[dev] + kNoAllocStatusInts;
    return cudaSuccess;
}

}  // namespace ptg
