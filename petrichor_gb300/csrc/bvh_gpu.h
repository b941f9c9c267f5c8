// Device binned-SAH BVH build (bvh_gpu.cu): the tree of BuildBinnedSah, built on the GPU.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "bvh_builder.h"

namespace ptg {

struct DeviceBuildStats {
    double ms = 0.0;  // device time from the first copy to the tree read back
    int levels = 0, rounds = 0, heapsorts = 0, launches = 0;
};

// positions: numVertices x 3 floats, indices: numTriangles x 3 (host memory, validated
// by the caller). Allocates its scratch (about 250 bytes per triangle) for the build
// and frees it; synchronises `stream`. On failure `out` is empty and `error` says why.
cudaError_t BuildBinnedSahDevice(const float* positions, int numVertices, const int32_t* indices,
                                 int numTriangles, cudaStream_t stream, BvhResult* out,
                                 std::string* error, DeviceBuildStats* stats);

}  // namespace ptg
