// GPU denoiser (denoise.cu): edge-avoiding à-trous filter guided by albedo and normal.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace ptg {

// Device scratch for one width x height image.
size_t DenoiseScratchBytes(int width, int height);

// color, albedo, normal, out: device RGB float rows (albedo and normal may be null).
// Enqueued on `stream`; out may alias color.
cudaError_t Denoise(int width, int height, const float* color, const float* albedo,
                    const float* normal, int hdr, float* out, void* scratch, cudaStream_t stream,
                    int* launches);

}  // namespace ptg
