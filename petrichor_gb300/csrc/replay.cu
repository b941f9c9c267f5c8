// Replay kernel: reproduces the reference renderer's film bit for bit.
//
// The reference draws its random numbers from one XorShift stream per 16x16
// tile, visiting the tile's pixels row-major (Core/Petrichor.cpp:79-91), so a
// pixel's samples depend on every earlier pixel of its tile. This kernel runs
// one thread per tile with that stream, the reference's BVH traversal order and
// the reference's arithmetic (ExactMath, built with -fmad=false). It is the
// parity path; the wavefront kernels are the throughput path.
#include <cuda_runtime.h>

#include "pt_device.cuh"
#include "pt_kernels.h"

namespace ptg {

__device__ __forceinline__ bool IsEmission(const DevScene& S, int m) { return S.mats[m].kind == kEmission; }

// SimplePathTracing::Render (Core/Integrator/SimplePathTracing.cpp:16-101)
__device__ void ReplaySimplePixel(const DevScene& S, const DevCamera& C, const DevSettings& st,
                                  int px, int py, float* film, RefSampler1D& s1, RefSampler2D& s2,
                                  int* stack, int* status) {
    V3 sum;
    for (int sp = 0; sp < st.spp; sp++) {
        float r0, r1, r2, r3;
        s2.Next(r0, r1);
        s2.Next(r2, r3);
        Ray ray = GenerateRay<ExactMath>(C, px, py, st.width, st.height, r0, r1, r2, r3);
        V3 contrib;
        for (int guard = 0;; guard++) {
            if (guard >= kMaxReplayBounces) {  // never reached by terminating paths; see header
                *status |= kErrBounceCap;
                break;
            }
            float dist;
            const int k = TraverseReference(S, ray.o, ray.d, kEps, kInfinity, dist, stack, status);
            if (k < 0) {
                contrib = contrib + ray.T * EnvColor<ExactMath>(S, ray.d);
                break;
            }
            const int m = ResolveMaterial(S.mats, SlotMaterial(S.shade, k), s1.Next());
            if (IsEmission(S, m)) {
                contrib = contrib + ray.T * MatColor(S.mats[m]);
                break;
            }
            Shading si = Interpolate<ExactMath>(S, k, ray.o, ray.d, dist);
            DevMaterial Mh;
            si.n = PointMaterial<ExactMath>(S, m, k, ray.o, ray.d, si.n, Mh);
            ray = NextRay<ExactMath>(Mh, ray, si, s2);
            if (ray.bounce > st.maxBounces) {
                ray.prob *= 0.9f;
                ray.prob = SMax(0.1f, ray.prob);
                if (s1.Next() < ray.prob) ray.T = ray.T / ray.prob;
                else break;
            }
        }
        sum = sum + contrib;
    }
    const V3 avg = sum / (float)st.spp;
    float* o = film + ((size_t)py * st.width + px) * 3;
    o[0] = avg.x;
    o[1] = avg.y;
    o[2] = avg.z;
}

// PathTracing::SampleLight (PathTracing.cpp:329-386): picks index, samples every
// light (one 2D draw each, as the reference does) and keeps the picked point.
__device__ V3 ReplaySampleLight(const DevScene& S, float rv, RefSampler2D& s2, bool wantEnv,
                                bool* sampleEnv) {
    const int L = S.numLights;
    int index;
    if (!wantEnv) {
        index = (int)(rv * (float)L);
        index = min(index, L - 1);
    } else {
        index = (int)(rv * (float)(L + 1));
        index = min(index, L);
        if (index >= L) {
            *sampleEnv = true;
            return V3();
        }
    }
    V3 result;
    for (int i = 0; i < L; i++) {
        float u0, u1;
        s2.Next(u0, u1);
        const V3 p = SampleLightPoint<ExactMath>(S, i, u0, u1);
        if (i == index) result = p;
    }
    return result;
}

// PathTracing::CalcLightContribution (PathTracing.cpp:202-327)
// M and nb: the shading point's material and BSDF normal (texture maps applied)
__device__ V3 ReplayLight(const DevScene& S, const Shading& si, const DevMaterial& M, V3 nb,
                          RefSampler1D& s1, RefSampler2D& s2, const Ray& ray, int* stack,
                          int* status) {
    V3 lc;
    const float dt = -Dot(ray.d, si.n);
    const V3 p = si.pos + kEps * copysignf(1.0f, dt) * si.n;
    const float pdfArea = S.lightPdfArea;
    bool sampleEnv = false;
    const V3 pl = ReplaySampleLight(S, s1.Next(), s2, true, &sampleEnv);
    if (!sampleEnv) {
        if (S.numLights == 0) return V3();
        const V3 ld = Normalized(pl - p);
        float d;
        const int k = TraverseReference(S, p, ld, 0.0f, kFltMax, d, stack, status);
        if (k >= 0) {
            if (IsEmission(S, ResolveMaterial(S.mats, SlotMaterial(S.shade, k), s1.Next()))) {
                const Shading sl = Interpolate<ExactMath>(S, k, p, ld, d);
                const float dist = SqLen(pl - sl.pos);
                if (fabsf(dist - 0.0f) < kEps) {
                    const float l2 = SqLen(sl.pos - si.pos);
                    const float cosP = fabsf(Dot(ld, sl.n));
                    float mis = 0.0f;
                    if (l2 > 0.0f) {
                        const float pL = pdfArea;
                        const float pB = BsdfPdf<ExactMath>(M, ray.d, ld, nb) * cosP / l2;
                        mis = pL * pL / (pL * pL + pB * pB);
                    }
                    const V3 li = MatColor(S.mats[sl.mat]);
                    const V3 f = BxDF<ExactMath>(M, ray.d, ld, nb);
                    const float c = fabsf(Dot(ld, si.n));
                    lc = lc + mis * ray.T * (li * f * c * cosP / (pdfArea * l2));
                }
            }
        }
    } else if (S.envValid) {
        float r0, r1;
        s2.Next(r0, r1);
        float pdfuv = 0.0f;
        const V3 sd = EnvSample<ExactMath>(S, r0, r1, pdfuv);
        const V3 eo = si.pos + kEps * copysignf(1.0f, dt) * si.n;
        float d;
        if (TraverseReference(S, eo, sd, 0.0f, kFltMax, d, stack, status) < 0) {
            const float c = fabsf(Dot(sd, si.n));
            const float sn = sqrtf(SMax(0.0f, 1.0f - c * c));
            const float pB = 2.0f * kPi * kPi * sn * BsdfPdf<ExactMath>(M, ray.d, sd, nb);
            const float mis = pdfuv * pdfuv / (pdfuv * pdfuv + pB * pB);
            const V3 li = EnvColor<ExactMath>(S, sd);
            const V3 f = BxDF<ExactMath>(M, ray.d, sd, nb);
            lc = lc + mis * ray.T * (li * f * sn * c * 2.0f * kPi * kPi) / pdfuv;
        }
    }
    return lc;
}

// PathTracing::Render (PathTracing.cpp:20-200)
__device__ void ReplayPtPixel(const DevScene& S, const DevCamera& C, const DevSettings& st, int px,
                              int py, float* film, RefSampler1D& s1, RefSampler2D& s2, int* stack,
                              int* status) {
    V3 sum;
    for (int sp = 0; sp < st.spp; sp++) {
        V3 color;
        float r0, r1, r2, r3;
        s2.Next(r0, r1);
        s2.Next(r2, r3);
        Ray ray = GenerateRay<ExactMath>(C, px, py, st.width, st.height, r0, r1, r2, r3);
        Ray prev = ray;
        Shading si;
        {
            float d;
            const int k = TraverseReference(S, ray.o, ray.d, 0.0f, kFltMax, d, stack, status);
            if (k < 0) {
                sum = sum + ray.T * EnvColor<ExactMath>(S, ray.d);
                continue;
            }
            si = Interpolate<ExactMath>(S, k, ray.o, ray.d, d);
        }
        if (IsEmission(S, si.mat)) {
            sum = sum + ray.T * MatColor(S.mats[si.mat]);
            continue;
        }
        for (int bounce = 0; bounce < st.maxBounces; bounce++) {
            DevMaterial Mh;
            const V3 nb = PointMaterial<ExactMath>(S, si.mat, si.slot, ray.o, ray.d, si.n, Mh);
            color = color + ReplayLight(S, si, Mh, nb, s1, s2, ray, stack, status);
            prev = ray;
            Shading sb = si;
            sb.n = nb;
            ray = NextRay<ExactMath>(Mh, ray, sb, s2);
            if (fabsf(SqLen(ray.T) - 0.0f) < kEps) break;
            float d;
            const int k = TraverseReference(S, ray.o, ray.d, 0.0f, kFltMax, d, stack, status);
            if (k >= 0) {
                const Shading sn = Interpolate<ExactMath>(S, k, ray.o, ray.d, d);
                if (IsEmission(S, sn.mat)) {
                    const float l2 = SqLen(sn.pos - ray.o);
                    const float cosP = fabsf(Dot(ray.d, sn.n));
                    bool unused = false;
                    ReplaySampleLight(S, s1.Next(), s2, false, &unused);
                    const float pdfArea = S.lightPdfArea;
                    const float pB = BsdfPdf<ExactMath>(Mh, prev.d, ray.d, nb);
                    const float pL = l2 / cosP * pdfArea;
                    const float mis = pB * pB / (pL * pL + pB * pB);
                    color = color + mis * ray.T * MatColor(S.mats[sn.mat]);
                    break;
                }
                si = sn;
            } else {
                if (S.envValid) {
                    const float c = fabsf(Dot(si.n, ray.d));
                    const float sn = sqrtf(SMax(0.0f, 1.0f - c * c));
                    const float pB = BsdfPdf<ExactMath>(Mh, prev.d, ray.d, nb);
                    float mis = 0.0f;
                    if (ray.d.x != 0 && ray.d.y != 0 && sn > 0) {
                        const float pE = EnvPdf<ExactMath>(S, ray.d) / (2.0f * kPi * kPi * sn);
                        mis = pB * pB / (pE * pE + pB * pB);
                    } else {
                        mis = 1.0f;
                    }
                    color = color + mis * ray.T * EnvColor<ExactMath>(S, ray.d);
                } else {
                    color = color + ray.T * EnvColor<ExactMath>(S, ray.d);
                }
                break;
            }
        }
        if (MinElem(color) >= 0.0f) sum = sum + color;
    }
    const V3 avg = sum / (float)st.spp;
    float* o = film + ((size_t)py * st.width + px) * 3;
    o[0] = avg.x;
    o[1] = avg.y;
    o[2] = avg.z;
}

// One thread per tile of TileManager (Core/TileManager.cpp:8-43), every tile seeded
// RandomSampler1D(0) / RandomSampler2D(0, 1) as the Rendered pass does.
__global__ void __launch_bounds__(64) ReplayKernel(DevScene S, DevCamera C, DevSettings st,
                                                   float* __restrict__ film,
                                                   int* __restrict__ stackScratch,
                                                   int* __restrict__ statusOut, int tileBegin,
                                                   int tileEnd) {
    const int t = tileBegin + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tileEnd) return;
    const int nx = st.width / st.tileW, ny = st.height / st.tileH;
    const int remW = st.width - nx * st.tileW, remH = st.height - ny * st.tileH;
    const int ti = t % (nx + 1), tj = t / (nx + 1);
    if (tj > ny) return;
    const int x0 = ti * st.tileW, y0 = tj * st.tileH;
    const int w = (ti != nx) ? st.tileW : remW, h = (tj != ny) ? st.tileH : remH;
    int* stack = stackScratch + (size_t)(t - tileBegin) * S.stackDepth;
    int status = 0;
    RefSampler1D s1(0);
    RefSampler2D s2(0, 1);
    for (int y = y0; y < y0 + h; y++)
        for (int x = x0; x < x0 + w; x++) {
            if (st.integrator == kSimplePathTracing)
                ReplaySimplePixel(S, C, st, x, y, film, s1, s2, stack, &status);
            else
                ReplayPtPixel(S, C, st, x, y, film, s1, s2, stack, &status);
        }
    if (status) atomicOr(statusOut, status);
}

// ---------------------------------------------------------------- AOV passes
// Core/AOV/AOVUVCoordinate.cpp:11-51: numSamplesPerPixel camera rays, hit uvs summed.
__device__ void AovUVPixel(const DevScene& S, const DevCamera& C, const DevSettings& st, int px,
                           int py, float* film, RefSampler2D& s2, int* stack, int* status) {
    V3 sum;
    for (int sp = 0; sp < st.spp; sp++) {
        float r0, r1, r2, r3;
        s2.Next(r0, r1);
        s2.Next(r2, r3);
        const Ray ray = GenerateRay<ExactMath>(C, px, py, st.width, st.height, r0, r1, r2, r3);
        float d;
        const int k = TraverseReference(S, ray.o, ray.d, kEps, kInfinity, d, stack, status);
        if (k >= 0) sum = sum + InterpolateUV(S, k, ray.o, ray.d);
    }
    const V3 avg = sum / (float)st.spp;
    float* o = film + ((size_t)py * st.width + px) * 3;
    o[0] = avg.x;
    o[1] = avg.y;
    o[2] = avg.z;
}

// AOVDenoisingAlbedo.cpp:56-133 (normal == false), AOVDenoisingNormal.cpp:54-128 (normal ==
// true): glass and zero-roughness GGX are followed up to numMaxBounces; the first other
// surface, or the environment, gives the value. Emission gives zero (the reference's
// ASSERT(false) default branch in a release build).
__device__ V3 AovPath(const DevScene& S, const DevSettings& st, Ray ray, bool normal,
                      RefSampler1D& s1, RefSampler2D& s2, int* stack, int* status) {
    for (int bounce = 0; bounce < st.maxBounces; bounce++) {
        float d;
        const int k = TraverseReference(S, ray.o, ray.d, kEps, kInfinity, d, stack, status);
        if (k < 0) return normal ? ray.T * (-ray.d) : ray.T * EnvColor<ExactMath>(S, ray.d);
        const int m = ResolveMaterial(S.mats, SlotMaterial(S.shade, k), s1.Next());
        const Shading si = Interpolate<ExactMath>(S, k, ray.o, ray.d, d);
        DevMaterial M;
        Shading sb = si;
        sb.n = PointMaterial<ExactMath>(S, m, k, ray.o, ray.d, si.n, M);
        if (M.kind == kLambert) return normal ? ray.T * si.n : ray.T * V3(M.ar, M.ag, M.ab);
        if (M.kind == kGlossy && M.alpha != 0) return normal ? ray.T * si.n : ray.T * GgxF0(M);
        if (M.kind != kGlass && M.kind != kGlossy) return V3();
        ray = NextRay<ExactMath>(M, ray, sb, s2);  // Glass::GetAlpha is always 0
    }
    return V3();
}

__device__ void AovDenoisePixel(const DevScene& S, const DevCamera& C, const DevSettings& st,
                                bool normal, int dspp, int px, int py, float* film, RefSampler1D& s1,
                                RefSampler2D& s2, int* stack, int* status) {
    V3 sum;
    for (int sp = 0; sp < dspp; sp++) {
        float r0, r1, r2, r3;
        s2.Next(r0, r1);
        s2.Next(r2, r3);
        const Ray ray = GenerateRay<ExactMath>(C, px, py, st.width, st.height, r0, r1, r2, r3);
        sum = sum + AovPath(S, st, ray, normal, s1, s2, stack, status);
    }
    const V3 avg = sum / (float)dspp;
    float* o = film + ((size_t)py * st.width + px) * 3;
    o[0] = avg.x;
    o[1] = avg.y;
    o[2] = avg.z;
}

// One thread per tile; unlike the Rendered pass, the AOV loops of Petrichor::Render
// (Core/Petrichor.cpp:104-261) advance tileIndex: tile k is seeded
// RandomSampler1D(k) / RandomSampler2D(k, k + 1).
__global__ void __launch_bounds__(64) AovKernel(DevScene S, DevCamera C, DevSettings st, int aov,
                                                int dspp, float* __restrict__ film,
                                                int* __restrict__ stackScratch,
                                                int* __restrict__ statusOut, int tileBegin,
                                                int tileEnd) {
    const int t = tileBegin + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tileEnd) return;
    const int nx = st.width / st.tileW, ny = st.height / st.tileH;
    const int remW = st.width - nx * st.tileW, remH = st.height - ny * st.tileH;
    const int ti = t % (nx + 1), tj = t / (nx + 1);
    if (tj > ny) return;
    const int x0 = ti * st.tileW, y0 = tj * st.tileH;
    const int w = (ti != nx) ? st.tileW : remW, h = (tj != ny) ? st.tileH : remH;
    int* stack = stackScratch + (size_t)(t - tileBegin) * S.stackDepth;
    int status = 0;
    RefSampler1D s1((uint32_t)t);
    RefSampler2D s2((uint32_t)t, (uint32_t)t + 1u);
    for (int y = y0; y < y0 + h; y++)
        for (int x = x0; x < x0 + w; x++) {
            if (aov == 0)
                AovUVPixel(S, C, st, x, y, film, s2, stack, &status);
            else
                AovDenoisePixel(S, C, st, aov == 2, dspp, x, y, film, s1, s2, stack, &status);
        }
    if (status) atomicOr(statusOut, status);
}

cudaError_t LaunchAov(const DevScene& S, const DevCamera& C, const DevSettings& st, int aov,
                      int dspp, float* film, int* stackScratch, int* status, int tileBegin,
                      int tileEnd, cudaStream_t stream) {
    const int n = tileEnd - tileBegin;
    if (n <= 0) return cudaSuccess;
    const int block = 64;
    AovKernel<<<(n + block - 1) / block, block, 0, stream>>>(S, C, st, aov, dspp, film, stackScratch,
                                                              status, tileBegin, tileEnd);
    return cudaGetLastError();
}

int NumTiles(const DevSettings& st) {
    return (st.width / st.tileW + 1) * (st.height / st.tileH + 1);
}

cudaError_t LaunchReplay(const DevScene& S, const DevCamera& C, const DevSettings& st, float* film,
                         int* stackScratch, int* status, int tileBegin, int tileEnd,
                         cudaStream_t stream) {
    const int n = tileEnd - tileBegin;
    if (n <= 0) return cudaSuccess;
    const int block = 64;
    ReplayKernel<<<(n + block - 1) / block, block, 0, stream>>>(S, C, st, film, stackScratch,
                                                                 status, tileBegin, tileEnd);
    return cudaGetLastError();
}

}  // namespace ptg
