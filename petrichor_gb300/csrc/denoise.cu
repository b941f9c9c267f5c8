// GPU denoiser in place of the reference's IntelOpenImageDenoiser
// (Core/Denoiser/IntelOpenImageDenoiser.cpp:15-101), which hands the film, and
// optionally the DenoisingAlbedo and DenoisingNormal AOVs, to Intel Open Image Denoise.
// That library and its trained weights are not part of this project, so the images
// differ from the reference's; the interface and the inputs are the same.
//
// Method: the edge-avoiding à-trous wavelet filter (H. Dammertz, D. Sewtz, J. Hanika,
// H. Lensch, "Edge-Avoiding À-Trous Wavelet Transform for fast Global Illumination
// Filtering", HPG 2010), with the luminance edge-stopping function scaled by a
// per-pixel noise estimate and that estimate carried through the iterations as in
// SVGF (C. Schied et al., HPG 2017):
//  - with an albedo, the colour is divided by it where it is not black (demodulation)
//    and multiplied back at the end, so texture detail is not blurred;
//  - the noise estimate is the variance of the (log, for HDR) luminance over a 3x3
//    window, blurred 3x3 before each pass;
//  - five passes of the 5x5 B3-spline kernel at steps 1, 2, 4, 8, 16 (clamped edges),
//    each tap weighted by exp(-|l_p - l_q| / (4 sigma_p)), (n_p . n_q)^128 where both
//    normals are known, and exp(-|a_p - a_q|^2 / 0.01) with an albedo; the centre tap
//    always has weight 1.
// Without AOVs the luminance stop is the only guide and is made stricter (2 sigma).
#include <cuda_runtime.h>

#include <cmath>

#include "denoise.h"

namespace ptg {
namespace {

constexpr int kPasses = 5;
constexpr float kSigmaNormal = 128.0f;
constexpr float kInvSigmaAlbedo2 = 1.0f / (0.1f * 0.1f);

__device__ __forceinline__ float Lum(float r, float g, float b) {
    return 0.2126f * r + 0.7152f * g + 0.0722f * b;
}
__device__ __forceinline__ float EdgeLum(float r, float g, float b, int hdr) {
    const float y = fmaxf(Lum(r, g, b), 0.0f);
    return hdr ? log1pf(y) : fminf(y, 1.0f);
}
__device__ __forceinline__ int Clamp(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

struct Planes {
    int W, H, hdr;
    float4* color;   // demodulated colour .xyz, edge luminance .w (two buffers)
    float4* color2;
    float* var;      // per-pixel luminance variance (two buffers)
    float* var2;
    float* gvar;     // 3x3 blur of var
    float4* albedo;  // demodulation factor .xyz, 1 where the albedo guide applies
    float4* normal;  // unit normal .xyz, 1 where known
};

__global__ void PrepKernel(Planes P, const float* __restrict__ color, const float* __restrict__ albedo,
                           const float* __restrict__ normal) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.W || y >= P.H) return;
    const size_t p = (size_t)y * P.W + x;
    float r = color[3 * p], g = color[3 * p + 1], b = color[3 * p + 2];
    if (!isfinite(r) || !isfinite(g) || !isfinite(b)) r = g = b = 0.0f;
    float4 a = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    if (albedo) {
        const float ar = albedo[3 * p], ag = albedo[3 * p + 1], ab = albedo[3 * p + 2];
        a.w = 1.0f;  // the albedo edge stop applies
        if (isfinite(ar) && isfinite(ag) && isfinite(ab) && Lum(ar, ag, ab) > 0.01f) {
            a.x = fmaxf(ar, 1e-3f);
            a.y = fmaxf(ag, 1e-3f);
            a.z = fmaxf(ab, 1e-3f);
        }
        if (!(isfinite(ar) && isfinite(ag) && isfinite(ab))) a.w = 0.0f;
        r /= a.x;
        g /= a.y;
        b /= a.z;
    }  // the albedo edge stop compares these factors (the albedo, or 1 where it is black)
    P.albedo[p] = a;
    float4 n = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (normal) {
        const float nx = normal[3 * p], ny = normal[3 * p + 1], nz = normal[3 * p + 2];
        const float l2 = nx * nx + ny * ny + nz * nz;
        if (isfinite(l2) && l2 > 0.25f) {
            const float inv = rsqrtf(l2);
            n = make_float4(nx * inv, ny * inv, nz * inv, 1.0f);
        }
    }
    P.normal[p] = n;
    P.color[p] = make_float4(r, g, b, EdgeLum(r, g, b, P.hdr));
}

__global__ void VarianceKernel(Planes P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.W || y >= P.H) return;
    float m1 = 0.0f, m2 = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
            const float l = P.color[(size_t)Clamp(y + dy, P.H - 1) * P.W + Clamp(x + dx, P.W - 1)].w;
            m1 += l;
            m2 += l * l;
        }
    m1 *= 1.0f / 9.0f;
    m2 *= 1.0f / 9.0f;
    P.var[(size_t)y * P.W + x] = fmaxf(m2 - m1 * m1, 0.0f);
}

__global__ void BlurVarKernel(Planes P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.W || y >= P.H) return;
    float s = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++)
            s += P.var[(size_t)Clamp(y + dy, P.H - 1) * P.W + Clamp(x + dx, P.W - 1)];
    P.gvar[(size_t)y * P.W + x] = s * (1.0f / 9.0f);
}

__global__ void ATrousKernel(Planes P, int step, float sigmaLum) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.W || y >= P.H) return;
    const float h[5] = {1.0f / 16.0f, 1.0f / 4.0f, 3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
    const size_t p = (size_t)y * P.W + x;
    const float4 cp = P.color[p];
    const float4 ap = P.albedo[p], np = P.normal[p];
    const float scale = 1.0f / (sigmaLum * sqrtf(P.gvar[p]) + 1e-4f);
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, sw = 0.0f, sv = 0.0f;
    for (int ky = 0; ky < 5; ky++) {
        const int qy = Clamp(y + (ky - 2) * step, P.H - 1);
        for (int kx = 0; kx < 5; kx++) {
            const int qx = Clamp(x + (kx - 2) * step, P.W - 1);
            const size_t q = (size_t)qy * P.W + qx;
            const float4 cq = P.color[q];
            float w = 1.0f;
            if (ky != 2 || kx != 2) {
                w = __expf(-fabsf(cp.w - cq.w) * scale);
                const float4 nq = P.normal[q];
                if (np.w > 0.0f && nq.w > 0.0f) {
                    const float d = fmaxf(0.0f, np.x * nq.x + np.y * nq.y + np.z * nq.z);
                    w *= __powf(d, kSigmaNormal);
                }
                const float4 aq = P.albedo[q];
                if (ap.w > 0.0f && aq.w > 0.0f) {
                    const float dr = ap.x - aq.x, dg = ap.y - aq.y, db = ap.z - aq.z;
                    w *= __expf(-(dr * dr + dg * dg + db * db) * kInvSigmaAlbedo2);
                }
            }
            const float wh = w * h[ky] * h[kx];
            sr += wh * cq.x;
            sg += wh * cq.y;
            sb += wh * cq.z;
            sw += wh;
            sv += wh * wh * P.var[q];
        }
    }
    const float inv = 1.0f / sw;  // sw >= h2 * h2 > 0 (centre tap)
    const float r = sr * inv, g = sg * inv, b = sb * inv;
    P.color2[p] = make_float4(r, g, b, EdgeLum(r, g, b, P.hdr));
    P.var2[p] = sv * inv * inv;
}

__global__ void RemodulateKernel(Planes P, float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.W || y >= P.H) return;
    const size_t p = (size_t)y * P.W + x;
    const float4 c = P.color[p], a = P.albedo[p];
    out[3 * p] = c.x * a.x;
    out[3 * p + 1] = c.y * a.y;
    out[3 * p + 2] = c.z * a.z;
}

}  // namespace

size_t DenoiseScratchBytes(int width, int height) {
    const size_t n = (size_t)width * height;
    return n * (4 * sizeof(float4) + 3 * sizeof(float)) + 7 * 256;  // 7 planes, 256-aligned
}

cudaError_t Denoise(int width, int height, const float* color, const float* albedo,
                    const float* normal, int hdr, float* out, void* scratch, cudaStream_t stream,
                    int* launches) {
    const size_t n = (size_t)width * height;
    char* s = static_cast<char*>(scratch);
    auto carve = [&](size_t bytes) {
        char* p = s;
        s += (bytes + 255) / 256 * 256;
        return p;
    };
    Planes P;
    P.W = width;
    P.H = height;
    P.hdr = hdr ? 1 : 0;
    P.color = reinterpret_cast<float4*>(carve(n * sizeof(float4)));
    P.color2 = reinterpret_cast<float4*>(carve(n * sizeof(float4)));
    P.albedo = reinterpret_cast<float4*>(carve(n * sizeof(float4)));
    P.normal = reinterpret_cast<float4*>(carve(n * sizeof(float4)));
    P.var = reinterpret_cast<float*>(carve(n * sizeof(float)));
    P.var2 = reinterpret_cast<float*>(carve(n * sizeof(float)));
    P.gvar = reinterpret_cast<float*>(carve(n * sizeof(float)));
    const dim3 block(16, 8), grid((width + 15) / 16, (height + 7) / 8);
    const float sigmaLum = (albedo || normal) ? 4.0f : 2.0f;
    PrepKernel<<<grid, block, 0, stream>>>(P, color, albedo, normal);
    VarianceKernel<<<grid, block, 0, stream>>>(P);
    int k = 2;
    for (int pass = 0; pass < kPasses; pass++) {
        BlurVarKernel<<<grid, block, 0, stream>>>(P);
        ATrousKernel<<<grid, block, 0, stream>>>(P, 1 << pass, sigmaLum);
        float4* c = P.color;
        P.color = P.color2;
        P.color2 = c;
        float* v = P.var;
        P.var = P.var2;
        P.var2 = v;
        k += 2;
    }
    RemodulateKernel<<<grid, block, 0, stream>>>(P, out);
    k++;
    if (launches) *launches += k;
    return cudaGetLastError();
}

}  // namespace ptg
