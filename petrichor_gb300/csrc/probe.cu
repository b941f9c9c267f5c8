// Memory-bandwidth probe behind pt_probe_bandwidth: the denominators of the roofline
// figures the benchmark reports (no reference counterpart; a measurement helper like
// pt_render_profile).
//
// L2 read: a buffer small enough to stay in L2 is read repeatedly with 16-byte loads
// that bypass L1 (ld.global.cg), one persistent grid of 4 blocks of 512 threads per SM,
// `passes` sweeps per launch so launch overhead is negligible; the sum of what was read
// is written once so the loads cannot be dropped.
#include <cuda_runtime.h>

#include "pt_kernels.h"

namespace ptg {

__global__ void __launch_bounds__(512) L2ReadKernel(const float4* __restrict__ buf, size_t n,
                                                    int passes, float* __restrict__ sink) {
    float acc = 0.0f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; p++) {
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(buf + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == 1.2345678e-30f) sink[0] = acc;  // never true for the probe's data
}

cudaError_t ProbeL2Read(const void* buf, size_t bytes, int passes, int reps, float* sink,
                        cudaStream_t stream, float* ms) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const size_t n = bytes / sizeof(float4);
    cudaEvent_t a = nullptr, b = nullptr;
    if ((e = cudaEventCreate(&a)) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&b)) != cudaSuccess) {
        cudaEventDestroy(a);
        return e;
    }
    L2ReadKernel<<<4 * sms, 512, 0, stream>>>((const float4*)buf, n, passes, sink);  // warm
    cudaEventRecord(a, stream);
    for (int r = 0; r < reps; r++)
        L2ReadKernel<<<4 * sms, 512, 0, stream>>>((const float4*)buf, n, passes, sink);
    cudaEventRecord(b, stream);
    e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

}  // namespace ptg
