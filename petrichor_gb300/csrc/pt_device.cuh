// Device-side vector math, samplers and the reference renderer's shading steps.
//
// Every function takes a math policy M:
//   ExactMath    - the transcendental calls of the reference resolve to the
//                  global double overloads (float arguments promoted, result
//                  narrowed). ExactMath evaluates them the same way, so a kernel
//                  compiled with -fmad=false reproduces the reference's floats.
//   FastMath     - single-precision library calls for the throughput path.
// Operand order inside every expression follows the reference source
// (component-wise Vector3f operators, Math/Vector3f.h), which is what makes
// bit-parity possible; the references are given per function.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pt_layout.h"

namespace ptg {

constexpr float kEps = 1.0e-3f;                    // Core/Constants.h:8
constexpr float kFltMax = 3.402823466e+38f;
constexpr float kInfinity = 0.9f * kFltMax;        // Core/Constants.h:10
constexpr float kPi = 3.14159265358979f;           // Core/Constants.h:15
constexpr float kInvPi = 1.0f / kPi;               // Core/Constants.h:16

// ---------------------------------------------------------------- V3
struct V3 {
    float x, y, z;
    __device__ V3() : x(0.f), y(0.f), z(0.f) {}
    __device__ V3(float a, float b, float c) : x(a), y(b), z(c) {}
    __device__ float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float c) { return V3(a.x * c, a.y * c, a.z * c); }
__device__ __forceinline__ V3 operator*(float c, V3 a) { return a * c; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ V3 operator/(V3 a, float c) { return V3(a.x / c, a.y / c, a.z / c); }
__device__ __forceinline__ V3 operator/(float c, V3 a) { return V3(c / a.x, c / a.y, c / a.z); }
__device__ __forceinline__ float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 Cross(V3 a, V3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float SqLen(V3 a) { return Dot(a, a); }
// Unfused forms: every product and sum rounded on its own, as g++ evaluates the
// reference's float expressions. __fmul_rn/__fadd_rn are never contracted into fused
// multiply-adds, so these give the reference's bits whatever the file's -fmad flag.
__device__ __forceinline__ float DotRn(V3 a, V3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 CrossRn(V3 a, V3 b) {
    return V3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
              __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float SqLenRn(V3 a) { return DotRn(a, a); }
// (lo + hi) * 0.5f, the product kept apart from the subtraction that follows it
__device__ __forceinline__ V3 CentreRn(V3 lo, V3 hi) {
    const V3 s = lo + hi;
    return V3(__fmul_rn(s.x, 0.5f), __fmul_rn(s.y, 0.5f), __fmul_rn(s.z, 0.5f));
}
__device__ __forceinline__ float Length(V3 a) { return sqrtf(Dot(a, a)); }  // = (float)sqrt(double)
__device__ __forceinline__ V3 Normalized(V3 a) { return a / Length(a); }
// 1 / d per component, correctly rounded whatever the file's division flags: the
// traversal's slab tests and the triangle test keep the reference's arithmetic. A
// correctly rounded reciprocal (rcp.rn.f32) is the same number as the correctly
// rounded quotient 1 / d (div.rn.f32), with fewer instructions.
__device__ __forceinline__ V3 ExactRecip(V3 d) {
    return V3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
}
// std::min / std::max argument semantics (NaN handling included)
__device__ __forceinline__ float SMin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float SMax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float MinElem(V3 a) { return SMin(a.x, SMin(a.y, a.z)); }
__device__ __forceinline__ V3 Reflected(V3 d, V3 n) { return d - 2.0f * n * Dot(d, n); }
__device__ __forceinline__ float Mod1(float x) { return x - 1.0f * floorf(x / 1.0f); }
__device__ __forceinline__ float Lerp(float a, float b, float t) { return (1.0f - t) * a + t * b; }
__device__ __forceinline__ float Pow5(float x) { const float x2 = x * x; return x * (x2 * x2); }
__device__ __forceinline__ int IClamp(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }
__device__ __forceinline__ V3 LoadV3(const float* p) { return V3(p[0], p[1], p[2]); }

// ---------------------------------------------------------------- math policies
struct ExactMath {
    static __device__ __forceinline__ float Cos(float x) { return (float)cos((double)x); }
    static __device__ __forceinline__ float Sin(float x) { return (float)sin((double)x); }
    static __device__ __forceinline__ float Acos(float x) { return (float)acos((double)x); }
    static __device__ __forceinline__ float Atan2(float y, float x) {
        return (float)atan2((double)y, (double)x);
    }
    // a * cos(x) / a * sin(x) with the float factor promoted (Lambert.cpp:67-72)
    static __device__ __forceinline__ float MulCos(float a, float x) {
        return (float)((double)a * cos((double)x));
    }
    static __device__ __forceinline__ float MulSin(float a, float x) {
        return (float)((double)a * sin((double)x));
    }
    static __device__ __forceinline__ float MulSinMul(float a, float x, float b) {
        return (float)(((double)a * sin((double)x)) * (double)b);
    }
    static __device__ __forceinline__ float SinCos(float t, float p) {
        return (float)(sin((double)t) * cos((double)p));
    }
    static __device__ __forceinline__ float SinSin(float t, float p) {
        return (float)(sin((double)t) * sin((double)p));
    }
    // Vector3f::Dot / Cross / Length: each product and sum rounded on its own
    static __device__ __forceinline__ float Dot(V3 a, V3 b) { return ::ptg::Dot(a, b); }
    static __device__ __forceinline__ V3 Cross(V3 a, V3 b) { return ::ptg::Cross(a, b); }
    static __device__ __forceinline__ float SqLen(V3 a) { return ::ptg::SqLen(a); }
    static __device__ __forceinline__ float Length(V3 a) { return ::ptg::Length(a); }
    // Vector3f::Normalized: each component divided by the length
    static __device__ __forceinline__ V3 Norm(V3 a) { return Normalized(a); }
    // -0.5f + 0.5f * sqrt(x) evaluated in double (GGX.cpp:148)
    static __device__ __forceinline__ float SmithLambda(float x) {
        return (float)((double)-0.5f + (double)0.5f * sqrt((double)x));
    }
    // -dn + sqrt(disc) evaluated in double (Vector3f.h:231-232)
    static __device__ __forceinline__ float RefractScale(float ndn, float disc) {
        return (float)((double)ndn + sqrt((double)disc));
    }
};
// Sines and cosines go through sinpif/cospif of the angle in half turns: the angles
// here are small (sampled on [0, 2 pi] or [0, pi]), the half-turn functions need no
// large-argument reduction, and the shade kernel's code stays small enough for the
// instruction cache. They agree with sinf/cosf to a few ulps.
struct FastMath {
    static __device__ __forceinline__ float Cos(float x) { return cospif(x * kInvPi); }
    static __device__ __forceinline__ float Sin(float x) { return sinpif(x * kInvPi); }
    // clamped: directions normalised with approximate division may reach |z| > 1
    static __device__ __forceinline__ float Acos(float x) { return acosf(fminf(fmaxf(x, -1.0f), 1.0f)); }
    static __device__ __forceinline__ float Atan2(float y, float x) { return atan2f(y, x); }
    static __device__ __forceinline__ float MulCos(float a, float x) { return a * Cos(x); }
    static __device__ __forceinline__ float MulSin(float a, float x) { return a * Sin(x); }
    static __device__ __forceinline__ float MulSinMul(float a, float x, float b) {
        return a * Sin(x) * b;
    }
    static __device__ __forceinline__ float SinCos(float t, float p) { return Sin(t) * Cos(p); }
    static __device__ __forceinline__ float SinSin(float t, float p) { return Sin(t) * Sin(p); }
    // dot and cross products as explicit fused multiply-adds (the same in every kernel
    // that inlines them, unlike compiler-chosen contraction)
    static __device__ __forceinline__ float Dot(V3 a, V3 b) {
        return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
    }
    static __device__ __forceinline__ V3 Cross(V3 a, V3 b) {
        return V3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
    }
    static __device__ __forceinline__ float SqLen(V3 a) { return Dot(a, a); }
    static __device__ __forceinline__ float Length(V3 a) { return sqrtf(Dot(a, a)); }
    // one division and three products instead of three divisions
    static __device__ __forceinline__ V3 Norm(V3 a) { return a * (1.0f / Length(a)); }
    static __device__ __forceinline__ float SmithLambda(float x) { return -0.5f + 0.5f * sqrtf(x); }
    static __device__ __forceinline__ float RefractScale(float ndn, float disc) {
        return ndn + sqrtf(disc);
    }
};

// ---------------------------------------------------------------- samplers
// Marsaglia xor128 (Random/XorShift.h:12-59); next() = u32 / float(UINT_MAX)
struct XorShift128 {
    uint32_t x, y, z, w;
    __device__ explicit XorShift128(uint32_t seed)
        : x(123456789u), y(362436069u), z(521288629u), w(seed) {}
    __device__ __forceinline__ float Next() {
        const uint32_t t = x ^ (x << 11);
        x = y;
        y = z;
        z = w;
        w = (w ^ (w >> 19)) ^ (t ^ (t >> 8));
        return __uint2float_rn(w) / 4294967296.0f;
    }
};
// RandomSampler1D(seed) / RandomSampler2D(seed0, seed1) (Core/Sampler/*)
struct RefSampler1D {
    XorShift128 g;
    __device__ explicit RefSampler1D(uint32_t s) : g(s) {}
    __device__ __forceinline__ float Next() { return g.Next(); }
};
struct RefSampler2D {
    XorShift128 g0, g1;
    __device__ RefSampler2D(uint32_t s0, uint32_t s1) : g0(s0), g1(s1) {}
    __device__ __forceinline__ void Next(float& a, float& b) {
        a = g0.Next();
        b = g1.Next();
    }
};

// Counter-based per-path stream for the throughput path: SplitMix64 over a
// 64-bit state keyed by (seed, pixel, sample); any draw depends only on the
// path's identity, never on scheduling or batching.
__device__ __forceinline__ uint64_t Mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t PathKey(uint32_t seed, uint32_t pixel, uint32_t sample) {
    return Mix64(Mix64(((uint64_t)seed << 32) ^ 0x5851F42D4C957F2Dull) ^
                 (((uint64_t)pixel << 32) | sample));
}
struct PathRng {
    uint64_t s;
    __device__ explicit PathRng(uint64_t state) : s(state) {}
    __device__ __forceinline__ float Next() {
        s += 0x9E3779B97F4A7C15ull;
        return (float)(uint32_t)(Mix64(s) >> 40) * (1.0f / 16777216.0f);
    }
    __device__ __forceinline__ void Next(float& a, float& b) {
        a = Next();
        b = Next();
    }
};

// ---------------------------------------------------------------- geometry
struct Ray {  // Core/Ray.h:42-48
    V3 o, d, T;
    int bounce;
    float prob, ior;
    __device__ Ray() : T(1.f, 1.f, 1.f), bounce(0), prob(1.0f), ior(1.0f) {}
};
struct Shading {  // Core/HitInfo.h:20-27 (uv and tangent formed on demand for texture maps)
    V3 n, pos;
    int mat;
    int slot;  // primitive slot of the hit
};

__device__ __forceinline__ void LoadTri(const float4* __restrict__ tris, int k, V3& v0, V3& e1, V3& e2) {
    const float4 a = __ldg(tris + 3 * k), b = __ldg(tris + 3 * k + 1), c = __ldg(tris + 3 * k + 2);
    v0 = V3(a.x, a.y, a.z);
    e1 = V3(a.w, b.x, b.y);
    e2 = V3(b.z, b.w, c.x);
}
__device__ __forceinline__ int TriId(const float4* __restrict__ tris, int k) {
    return __float_as_int(__ldg(&tris[3 * k + 2].y));
}
// Material index of the triangle in primitive slot k (before Mix resolution).
__device__ __forceinline__ int SlotMaterial(const float4* __restrict__ shade, int k) {
    return __float_as_int(__ldg(&shade[3 * k].w));
}

// Triangle::Intersect (Core/Geometry/Triangle.cpp:51-88), unfused and correctly
// rounded in every build: closest-hit IDs and distances are the reference's.
__device__ __forceinline__ bool TriIntersect(V3 v0, V3 e1, V3 e2, V3 o, V3 d, float& dist) {
    const V3 ce = CrossRn(e1, e2);
    const float invDet = __frcp_rn(DotRn(-d, ce));  // = 1 / det, correctly rounded
    const V3 vec = o - v0;
    const float w1 = __fmul_rn(DotRn(vec, CrossRn(d, e2)), invDet);
    const float w2 = __fmul_rn(DotRn(vec, CrossRn(e1, d)), invDet);
    if (w1 < 0.0f || w1 >= 1.0f) return false;
    if (w2 < 0.0f || w2 >= 1.0f) return false;
    if (__fadd_rn(w1, w2) >= 1.0f) return false;
    const float t = __fmul_rn(DotRn(vec, ce), invDet);
    if (t < 0.0f) return false;
    dist = t;
    return true;
}

// GeometryBase::GetMaterial (GeometryBase.h:59-69) with MixMaterial::GetSingleMaterial
__device__ __forceinline__ int ResolveMaterial(const DevMaterial* __restrict__ mats, int m, float r) {
    if (m >= 0 && mats[m].kind == kMix) {
        const int packed = mats[m].mat01;
        return mats[m].mix <= r ? (packed & 0xFFFF) : (packed >> 16);
    }
    return m;
}

// Triangle::Interpolate (Triangle.cpp:90-153); k = primitive slot
template <class M>
__device__ __forceinline__ Shading Interpolate(const DevScene& S, int k, V3 o, V3 d, float dist) {
    Shading si;
    si.pos = o + d * dist;
    V3 v0, e1, e2;
    LoadTri(S.tris, k, v0, e1, e2);
    const float4 s0 = __ldg(S.shade + 3 * k);
    const float4 s1 = __ldg(S.shade + 3 * k + 1);
    const V3 ce = M::Cross(e1, e2);
    if (__float_as_int(s1.w) == 0) {
        si.n = M::Norm(ce);
    } else {
        const float4 s2 = __ldg(S.shade + 3 * k + 2);
        const float invDet = 1.0f / M::Dot(-d, ce);
        const V3 vec = o - v0;
        const float w1 = M::Dot(vec, M::Cross(d, e2)) * invDet;
        const float w2 = M::Dot(vec, M::Cross(e1, d)) * invDet;
        const V3 n0(s0.x, s0.y, s0.z), n1(s1.x, s1.y, s1.z), n2(s2.x, s2.y, s2.z);
        si.n = M::Norm(w1 * (n1 - n0) + w2 * (n2 - n0) + n0);
    }
    si.mat = ResolveMaterial(S.mats, __float_as_int(s0.w), 0.0f);
    si.slot = k;
    return si;
}

// The uv of Triangle::Interpolate (Triangle.cpp:90-110) at the hit of ray (o, d) on slot k.
__device__ __forceinline__ V3 InterpolateUV(const DevScene& S, int k, V3 o, V3 d) {
    if (!S.uvs) return V3();
    V3 v0, e1, e2;
    LoadTri(S.tris, k, v0, e1, e2);
    const V3 ce = Cross(e1, e2);
    const float invDet = 1.0f / Dot(-d, ce);
    const V3 vec = o - v0;
    const float w1 = Dot(vec, Cross(d, e2)) * invDet;
    const float w2 = Dot(vec, Cross(e1, d)) * invDet;
    const float4 a = __ldg(S.uvs + 3 * k), b = __ldg(S.uvs + 3 * k + 1), c = __ldg(S.uvs + 3 * k + 2);
    const V3 uv0(a.x, a.y, a.z), uv1(b.x, b.y, b.z), uv2(c.x, c.y, c.z);
    const V3 duv1 = uv1 - uv0, duv2 = uv2 - uv0;
    return w1 * duv1 + w2 * duv2 + uv0;
}

// Triangle::SampleSurface (Triangle.cpp:155-182) for light i; pdfArea not returned
// (the per-light sum is precomputed in DevScene::lightPdfArea).
template <class M>
__device__ __forceinline__ V3 SampleLightPoint(const DevScene& S, int i, float u0, float u1) {
    const float4 a = __ldg(S.lights + 3 * i), b = __ldg(S.lights + 3 * i + 1),
                 c = __ldg(S.lights + 3 * i + 2);
    const V3 v0(a.x, a.y, a.z), e0(b.x, b.y, b.z), e1(c.x, c.y, c.z);
    const float su = sqrtf(u0);
    return v0 + (1.0f - su) * e0 + su * u1 * e1;
}

// ---------------------------------------------------------------- ONB
struct ONB {  // Math/OrthonormalBasis.cpp:10-62
    V3 u, v, w;
    template <class M>
    __device__ __forceinline__ void Build(V3 n) {
        w = M::Norm(n);
        const float sign = copysignf(1.0f, w.z);
        const float a = -1.0f / (sign + w.z);
        const float b = w.x * w.y * a;
        u = V3(1.0f + sign * w.x * w.x * a, sign * b, -sign * w.x);
        v = V3(b, sign + w.y * w.y * a, -w.y);
    }
    template <class M>
    __device__ __forceinline__ void Build(V3 ww, V3 uu) {
        w = M::Norm(ww);
        u = M::Norm(uu);
        v = M::Cross(w, u);
    }
    template <class M>
    __device__ __forceinline__ V3 WorldToLocal(V3 a) const { return V3(M::Dot(a, u), M::Dot(a, v), M::Dot(a, w)); }
    __device__ __forceinline__ V3 LocalToWorld(V3 a) const { return u * a.x + v * a.y + w * a.z; }
};

// ---------------------------------------------------------------- camera
// Camera::GenerateRay (Core/Camera.cpp:52-91); (r0,r1) sensor, (r2,r3) lens
template <class M>
__device__ __forceinline__ Ray GenerateRay(const DevCamera& c, int i, int j, int W, int H, float r0,
                                           float r1, float r2, float r3) {
    const V3 pos = LoadV3(c.pos), right = LoadV3(c.right), up = LoadV3(c.up), fwd = LoadV3(c.fwd);
    const float aspect = (float)W / H;
    const float u = (i + r0) / W - 0.5f;
    const float v = (j + r1) / H - 0.5f;
    const V3 onSensor = pos + right * u * c.hPerf * c.focusDist * aspect +
                        -up * v * c.hPerf * c.focusDist + fwd * c.focusDist;
    const float r = sqrtf(r2);
    const float theta = 2.0f * kPi * r3;
    const V3 onLens = pos + right * 0.5f * c.aperture * r * M::Cos(theta) +
                      -up * 0.5f * c.aperture * r * M::Sin(theta);
    Ray ray;
    ray.o = onLens;
    ray.d = M::Norm(onSensor - onLens);
    const float dd = M::Dot(ray.d, fwd);
    ray.T = V3(1.f, 1.f, 1.f) * dd * dd * c.focusDist * c.focusDist / M::SqLen(onSensor - onLens);
    return ray;
}

// ---------------------------------------------------------------- environment
// Texture2D::GetPixel(int,int) + bilinear GetPixel(float,float) (Texture2D.cpp:260-317)
__device__ __forceinline__ V3 EnvTexel(const DevScene& S, int i, int j) {
    const float4 t = __ldg(S.env + (size_t)S.envW * j + i);
    return V3(t.x, t.y, t.z);
}
__device__ __forceinline__ V3 EnvBilinear(const DevScene& S, float x, float y) {
    int ix0 = (int)x, ix1 = (int)(x + 1.0f), iy0 = (int)y, iy1 = (int)(y + 1.0f);
    const float wx0 = x - ix0, wy0 = y - iy0, wx1 = ix1 - x, wy1 = iy1 - y;
    ix0 = IClamp(ix0, 0, S.envW - 1);
    ix1 = IClamp(ix1, 0, S.envW - 1);
    iy0 = IClamp(iy0, 0, S.envH - 1);
    iy1 = IClamp(iy1, 0, S.envH - 1);
    const V3 c00 = EnvTexel(S, ix0, iy0), c10 = EnvTexel(S, ix1, iy0);
    const V3 c01 = EnvTexel(S, ix0, iy1), c11 = EnvTexel(S, ix1, iy1);
    const V3 cm0 = wx1 * c00 + wx0 * c10;
    const V3 cm1 = wx1 * c01 + wx0 * c11;
    return wy1 * cm0 + wy0 * cm1;
}
// The reference's importance-sampling tables are Texture2Ds that are sized but
// never marked loaded, so every texel read returns the invalid-texture colour
// (1, 0, 1) (Texture2D.cpp:263-266, Environment.cpp:56-58). A bilinear read of
// them is therefore the sum of the bilinear weights; this returns its x.
__device__ __forceinline__ float UnloadedTableBilinearX(float u, float v, int W, int H) {
    u = Mod1(u);
    v = Mod1(v);
    const float x = u * W, y = v * H;
    const int ix0 = (int)x, ix1 = (int)(x + 1.0f), iy0 = (int)y, iy1 = (int)(y + 1.0f);
    const float wx0 = x - ix0, wy0 = y - iy0, wx1 = ix1 - x, wy1 = iy1 - y;
    const float cm = wx1 * 1.0f + wx0 * 1.0f;
    return wy1 * cm + wy0 * cm;
}
// The row tables of Environment::PreCalcCumulativeDistTex (Environment.cpp:56-128)
// sum those unloaded reads: every row's luminance is 1, so the running sum is the
// exact integer j + 1 and the tables are cdf1D[j] = (j + 1) / H (one rounded
// division) and pdf1D[j] = 1 * (H / H) = 1. They are evaluated here instead of read.
__device__ __forceinline__ float EnvRowCdf(int j, int H) { return __fdiv_rn((float)(j + 1), (float)H); }
constexpr float kEnvRowPdf = 1.0f;
// Environment::GetColor (Environment.cpp:29-48)
template <class M>
__device__ __forceinline__ V3 EnvColor(const DevScene& S, V3 d) {
    const V3 base(S.envBase[0], S.envBase[1], S.envBase[2]);
    if (!S.envValid) return base;
    const float theta = M::Acos(d.z);
    const float phi = M::Atan2(d.y, d.x);
    float u = 1.0f - (phi - S.envRot) * 0.5f * kInvPi;
    float v = theta * kInvPi;
    u = Mod1(u);
    v = Mod1(v);
    u = Mod1(u);  // GetPixelByUV wraps again (Texture2D.cpp:332-334)
    v = Mod1(v);
    return base * EnvBilinear(S, u * S.envW, v * S.envH);
}
// The two bisections of Environment::ImportanceSampling (Environment.cpp:150-200), used
// for maps whose dimensions are not both powers of two.
__device__ __forceinline__ void EnvSampleSearch(const DevScene& S, float r0, float r1, float& u0, float& v0, float& pdf) {
    const int W = S.envW, H = S.envH;
    const float tw = 1.0f / W, th = 1.0f / H;
    v0 = 0.0f;
    float v1 = 1.0f;
    for (int it = 0; it < 64; it++) {
        const float v = 0.5f * (v0 + v1);
        const float y = v * H;
        const int fy = (int)y;
        const int cy = min(fy + 1, H - 1);
        const float c = Lerp(EnvRowCdf(fy, H), EnvRowCdf(cy, H), y - fy);
        const float diff = c - r0;
        if (v1 - v0 <= th) { v0 = v1 = v; break; }
        if (diff > 0) v1 = v;
        else if (diff < 0) v0 = v;
        else { v0 = v1 = v; break; }
    }
    float u1 = 1.0f;
    u0 = 0.0f;
    for (int it = 0; it < 64; it++) {
        const float u = 0.5f * (u0 + u1);
        const float c = UnloadedTableBilinearX(u, v0, W, H);
        const float diff = c - r1;
        if (u1 - u0 <= tw) { u0 = u1 = u; break; }
        if (diff >= 0) u1 = u;
        else u0 = u;
    }
    {
        const float y = v0 * H;
        const int y0 = (int)y;
        const int y1 = min(y0 + 1, H - 1);
        const float py = Lerp(kEnvRowPdf, kEnvRowPdf, y - y0);
        pdf = py * UnloadedTableBilinearX(u0, v0, W, H);
    }
}
// Environment::ImportanceSampling (Environment.cpp:130-220)
//
// When W and H are powers of two (all configured maps) both searches have a closed
// form, evaluated here bit for bit:
//   row search: every compared midpoint v is an odd multiple of 2^-k with k <= log2 H,
//     so y = v H is an integer, the lerp weight is exactly 0 and the table value is
//     cdf1D[y] = (y + 1) / H = v + 1/H exactly: the comparisons reduce to v + 1/H - r0;
//   column search: for u = 2^-k (k <= log2 W) and the row found above (a multiple of
//     1/(2H)), every bilinear weight is 0, 1/2 or 1 and the unloaded-table read is
//     exactly 1, so 1 - r1 >= 0 at every step: u shrinks to 0.5 / W whatever r1 is;
//   pdf: the same weights at (0.5 / W, v0) give exactly 1 * 1.
template <class M>
__device__ __forceinline__ V3 EnvSample(const DevScene& S, float r0, float r1, float& pdf) {
    const int W = S.envW, H = S.envH;
    const float tw = 1.0f / W, th = 1.0f / H;
    float u0, v0 = 0.0f, v1 = 1.0f;
    if (((W & (W - 1)) | (H & (H - 1))) == 0 && W <= (1 << 22) && H <= (1 << 22)) {
        for (int it = 0; it < 64; it++) {
            const float v = 0.5f * (v0 + v1);
            const float diff = (v + th) - r0;
            if (v1 - v0 <= th) { v0 = v1 = v; break; }
            if (diff > 0) v1 = v;
            else if (diff < 0) v0 = v;
            else { v0 = v1 = v; break; }
        }
        u0 = 0.5f * tw;
        pdf = 1.0f;
    } else {
        EnvSampleSearch(S, r0, r1, u0, v0, pdf);
    }
    const float theta = v0 * kPi;
    const float phi = 2.0f * kPi * (1.0f - u0) + S.envRot;
    // ONB(UnitZ, UnitX).GetDir(theta, phi): u = X, v = Y, w = Z
    const float cx = M::SinCos(theta, phi), cy = M::SinSin(theta, phi), cz = M::Cos(theta);
    return cx * V3(1.f, 0.f, 0.f) + cy * V3(0.f, 1.f, 0.f) + cz * V3(0.f, 0.f, 1.f);
}
// Environment::GetImportanceSamplingPDF (Environment.cpp:222-244)
template <class M>
__device__ __forceinline__ float EnvPdf(const DevScene& S, V3 d) {
    const float theta = M::Acos(d.z);
    const float phi = M::Atan2(d.y, d.x);
    const float u0 = 1.0f - (phi - S.envRot) * 0.5f * kInvPi;
    const float v0 = theta * kInvPi;
    const float y = v0 * S.envH;
    // d.z == -1 gives y == H, an out-of-range row in the reference (undefined
    // behaviour there); the row index is clamped to the table here.
    const int y0 = min((int)y, S.envH - 1);
    const int y1 = min(y0 + 1, S.envH - 1);
    const float py = Lerp(kEnvRowPdf, kEnvRowPdf, y - y0);
    return py * UnloadedTableBilinearX(u0, v0, S.envW, S.envH);
}

// Optional environment importance sampling from an alias table over the map's texels
// (weights: the largest luminance of the texel's bilinear footprint times sin theta at
// its centre, built at the first render that asks for it). The table column is drawn
// as a row from r0 and a column from j0 (a float holds 24 bits, too few to index the
// 2^25 cells of an 8192x4096 map at once), kept or replaced by its alias by r1, and the
// point inside the chosen cell is uniform in (u, v): r1 rescaled within its keep/alias
// branch across, j1 down. The density over (u, v) is the cell's table pdf, which the reference's MIS
// formulas take as pdfuv (PathTracing.cpp:282-327 convert it to solid angle with
// 2 pi^2 sin theta). Directions map to (u, v) exactly as EnvColor reads the map. Out of
// line: a render without it never runs this code.
template <class M>
__device__ __noinline__ V3 EnvSampleAlias(const DevScene& S, float r0, float r1, float j0, float j1,
                                          float& pdfuv) {
    const int W = S.envW, H = S.envH;
    const int row = min(max((int)(r0 * (float)H), 0), H - 1);
    const int column = min(max((int)(j0 * (float)W), 0), W - 1);
    const int i = row * W + column;
    const float4 col = __ldg(S.envAlias + i);
    const bool keep = r1 < col.x;
    const int t = keep ? i : __float_as_int(col.y);
    // the offset across the cell: r1 rescaled to [0, 1) within the branch it took, which
    // is uniform and independent of the cell chosen (j0's fraction after the column
    // would keep only log2(W) fewer bits than a float's 24)
    const float fx = fminf(fmaxf(keep ? r1 / col.x : (r1 - col.x) / (1.0f - col.x), 0.0f), 0.99999994f);
    pdfuv = t == i ? col.z : __ldg(S.envAlias + t).z;
    const int ix = t % W, iy = t / W;
    const float u0 = ((float)ix + fx) / (float)W, v0 = ((float)iy + j1) / (float)H;
    const float theta = v0 * kPi;
    const float phi = 2.0f * kPi * (1.0f - u0) + S.envRot;
    const float cx = M::SinCos(theta, phi), cy = M::SinSin(theta, phi), cz = M::Cos(theta);
    return V3(cx, cy, cz);
}
template <class M>
__device__ __noinline__ float EnvPdfAlias(const DevScene& S, V3 d) {
    const float theta = M::Acos(d.z);
    const float phi = M::Atan2(d.y, d.x);
    const float u = Mod1(1.0f - (phi - S.envRot) * 0.5f * kInvPi);
    const float v = Mod1(theta * kInvPi);
    const int ix = min((int)(u * (float)S.envW), S.envW - 1);
    const int iy = min((int)(v * (float)S.envH), S.envH - 1);
    return __ldg(S.envAlias + (size_t)iy * S.envW + ix).z;
}

// ---------------------------------------------------------------- materials
__device__ __forceinline__ V3 MatColor(const DevMaterial& m) { return V3(m.cr, m.cg, m.cb); }
// GGX::GetF0 with metalness 0 and no map (GGX.h:126-139)
// Texture2D::GetPixelByUV (Texture2D.cpp:327-335) on material texture t: wrap, then the
// bilinear fetch of Texture2D::GetPixel at (u W, v H) with edge clamping.
__device__ __forceinline__ V3 TexByUV(const DevScene& S, int t, float u, float v) {
    const int4 info = __ldg(S.texInfo + t);
    const int W = info.y, H = info.z;
    u = Mod1(u);
    v = Mod1(v);
    const float x = u * W, y = v * H;
    int ix0 = (int)x, ix1 = (int)(x + 1.0f), iy0 = (int)y, iy1 = (int)(y + 1.0f);
    const float wx0 = x - ix0, wy0 = y - iy0, wx1 = ix1 - x, wy1 = iy1 - y;
    ix0 = IClamp(ix0, 0, W - 1);
    ix1 = IClamp(ix1, 0, W - 1);
    iy0 = IClamp(iy0, 0, H - 1);
    iy1 = IClamp(iy1, 0, H - 1);
    const float4* px = S.texels + info.x;
    const float4 a = __ldg(px + (size_t)W * iy0 + ix0), b = __ldg(px + (size_t)W * iy0 + ix1);
    const float4 c = __ldg(px + (size_t)W * iy1 + ix0), d = __ldg(px + (size_t)W * iy1 + ix1);
    const V3 c00(a.x, a.y, a.z), c10(b.x, b.y, b.z), c01(c.x, c.y, c.z), c11(d.x, d.y, d.z);
    const V3 cm0 = wx1 * c00 + wx0 * c10;
    const V3 cm1 = wx1 * c01 + wx0 * c11;
    return wy1 * cm0 + wy0 * cm1;
}

// Material parameters at a shading point of a material with texture maps
// (Lambert::GetAlbedo, Lambert.cpp:117-126; GGX::GetAlpha / GetF0 / GetNormal,
// GGX.h:57-139), with uv and tangent as Triangle::Interpolate forms them
// (Triangle.cpp:90-145). Kept out of line: untextured scenes never run it, and the
// shading kernels are instruction-fetch bound, so its code stays out of their loop.
struct PointTextures {
    V3 albedo;  // Lambert: kd * texel (1 without an albedo map)
    V3 refl;    // GGX reflectance: color * texel (GgxF0 squares it)
    float alpha;
    V3 n;       // the normal the GGX functions use
};
template <class M>
__device__ __noinline__ PointTextures TexturedPoint(const DevScene& S, int mat, int k, V3 o, V3 d,
                                                     V3 n) {
    const DevMaterial m = S.mats[mat];
    PointTextures r;
    r.albedo = V3(m.ar, m.ag, m.ab);
    r.refl = MatColor(m);
    r.alpha = m.alpha;
    r.n = n;
    const bool smooth = __float_as_int(__ldg(&S.shade[3 * k + 1].w)) != 0;
    V3 v0, e1, e2;
    LoadTri(S.tris, k, v0, e1, e2);
    const V3 ce = M::Cross(e1, e2);
    const float invDet = __frcp_rn(M::Dot(-d, ce));
    const V3 vec = o - v0;
    const float w1 = M::Dot(vec, M::Cross(d, e2)) * invDet;
    const float w2 = M::Dot(vec, M::Cross(e1, d)) * invDet;
    const float4 a = __ldg(S.uvs + 3 * k), b = __ldg(S.uvs + 3 * k + 1), c = __ldg(S.uvs + 3 * k + 2);
    const V3 uv0(a.x, a.y, a.z), uv1(b.x, b.y, b.z), uv2(c.x, c.y, c.z);
    const V3 duv1 = uv1 - uv0, duv2 = uv2 - uv0;
    const V3 uv = w1 * duv1 + w2 * duv2 + uv0;
    if (m.texAlbedo >= 0) r.albedo = MatColor(m) * TexByUV(S, m.texAlbedo, uv.x, uv.y);
    if (m.texF0 >= 0) r.refl = MatColor(m) * TexByUV(S, m.texF0, uv.x, uv.y);
    if (m.texRough >= 0) {
        const V3 t = TexByUV(S, m.texRough, uv.x, uv.y);
        const float rs = m.roughStrength * (0.2126f * t.x + 0.7152f * t.y + 0.0722f * t.z);
        r.alpha = rs * rs;
    }
    if (m.texNormal < 0) return r;
    V3 tangent = duv2.y * e1 - duv1.y * e2;
    if (smooth) tangent = tangent - M::Dot(n, tangent) * n;
    if (M::SqLen(tangent) == 0.0f) tangent = V3(1.f, 0.f, 0.f);
    const V3 bw = M::Norm(n), bu = M::Norm(tangent), bv = M::Cross(bw, bu);
    const V3 nm = TexByUV(S, m.texNormal, uv.x, uv.y);
    const V3 ln = M::Norm(2.0f * nm - V3(1.f, 1.f, 1.f));
    const float s = 1.0f - m.normalStrength;
    r.n = s * ln.x * bu + ln.y * bv + s * ln.z * bw;
    return r;
}

// The material of slot k's shading point and the normal its BSDF uses: untextured
// materials are returned as stored with the shading normal.
template <class M>
__device__ __forceinline__ V3 PointMaterial(const DevScene& S, int mat, int k, V3 o, V3 d, V3 n,
                                           DevMaterial& m) {
    m = S.mats[mat];
    if (m.texMask == 0) return n;
    const PointTextures t = TexturedPoint<M>(S, mat, k, o, d, n);
    m.ar = t.albedo.x, m.ag = t.albedo.y, m.ab = t.albedo.z;
    m.cr = t.refl.x, m.cg = t.refl.y, m.cb = t.refl.z;
    m.alpha = t.alpha;
    return m.kind == kGlossy ? t.n : n;
}

__device__ __forceinline__ V3 GgxF0(const DevMaterial& m) {
    const V3 c = MatColor(m);
    return 0.16f * (c * c) * (1.0f - 0.0f) + V3(1.f, 1.f, 1.f) * 0.0f;
}
template <class M>
__device__ __forceinline__ float GgxLambda(V3 dir, V3 h, float alpha) {  // GGX.cpp:140-152
    const float a2 = alpha * alpha;
    const float c = fabsf(M::Dot(dir, h));
    const float tan2 = c > 0 ? 1.0f / (c * c) - 1.0f : kInfinity;
    return M::SmithLambda(1.0f + a2 * tan2);
}
// MaterialBase::BxDF for Lambert (Lambert.cpp:27-31, untextured albedo = 1) and GGX
// (GGX.cpp:22-57); Glass returns zero (Glass.cpp:11-18).
template <class M>
__device__ __forceinline__ V3 BxDF(const DevMaterial& m, V3 din, V3 dout, V3 n) {
    if (m.kind == kLambert) return MatColor(m) * V3(m.ar, m.ag, m.ab) * kInvPi;
    if (m.kind == kGlossy) {
        const V3 h = M::Norm(-din + dout);
        const float hn = fabsf(M::Dot(h, n));
        const float a = m.alpha, a2 = a * a, hn2 = hn * hn;
        const float k = (a2 - 1.0f) * hn2 + 1.0f;
        const float D = a2 / (kPi * k * k);
        const float li = GgxLambda<M>(dout, h, a), lo = GgxLambda<M>(-din, h, a);
        const float G = 1.0f / (1.0f + li + lo);
        const float hl = fabsf(M::Dot(h, dout));
        const V3 F = GgxF0(m) + (V3(1.f, 1.f, 1.f) - GgxF0(m)) * Pow5(1.0f - hl);
        const float ln = fabsf(M::Dot(dout, n)), vn = fabsf(M::Dot(-din, n));
        return D * G * F / (4.0f * ln * vn);
    }
    return V3(0.f, 0.f, 0.f);
}
// MaterialBase::PDF (Lambert.cpp:33-47, GGX.cpp:59-76, Glass.cpp:20-27)
template <class M>
__device__ __forceinline__ float BsdfPdf(const DevMaterial& m, V3 din, V3 dout, V3 n) {
    if (m.kind == kLambert) return m.uniform ? 0.5f * kInvPi : fabsf(M::Dot(dout, n)) * kInvPi;
    if (m.kind == kGlossy) {
        const V3 h = M::Norm(-din + dout);
        const float hn = fabsf(M::Dot(h, n));
        const float a2 = m.alpha * m.alpha, hn2 = hn * hn;
        const float tmp = 1.0f - (1.0f - a2) * hn2;
        return tmp > 0 ? kInvPi * a2 / (tmp * tmp) : kInfinity;
    }
    return 0.0f;
}
// GGX::SampleGGXVNDF (GGX.cpp:154-208)
template <class M>
__device__ __forceinline__ V3 SampleVNDF(const DevMaterial& m, V3 view, V3 n0, float u0, float u1) {
    const V3 n = n0 * copysignf(1.0f, M::Dot(view, n0));
    ONB surf;
    const V3 t = (fabsf(n.z) < 0.9999f) ? M::Cross(n, V3(0.f, 0.f, 1.f)) : V3(1.f, 0.f, 0.f);
    surf.template Build<M>(n, t);
    V3 v = surf.template WorldToLocal<M>(view);
    const float alpha = m.alpha;
    v = v * V3(alpha, alpha, 1.0f);
    v = v / M::Length(v);
    const V3 t1 = (v.z < 0.9999f) ? M::Norm(M::Cross(v, V3(0.f, 0.f, 1.f))) : V3(1.f, 0.f, 0.f);
    const V3 t2 = M::Cross(t1, v);
    const float a = 1.0f / (1.0f + v.z);
    const float r = sqrtf(u0);
    const float phi = (u1 < a) ? u1 / a * kPi : kPi + (u1 - a) / (1.0f - a) * kPi;
    const float p1 = M::MulCos(r, phi);
    const float p2 = M::MulSinMul(r, phi, (u1 < a) ? 1.0f : v.z);
    const float w = sqrtf(SMax(0.0f, 1.0f - p1 * p1 - p2 * p2));
    V3 h = p1 * t1 + p2 * t2 + w * v;
    h = V3(alpha * h.x, alpha * h.y, SMax(0.0f, h.z));
    h = surf.LocalToWorld(h);
    return h / M::Length(h);
}
// MaterialBase::CreateNextRay for Lambert (Lambert.cpp:49-98), GGX (GGX.cpp:78-138)
// and Glass (Glass.cpp:29-95). The sampler is drawn exactly where the reference
// draws (Glass draws only when it refracts).
template <class M, class S2>
__device__ __forceinline__ Ray NextRay(const DevMaterial& m, const Ray& in, const Shading& si, S2& s2) {
    Ray out;
    if (m.kind == kLambert) {
        const V3 n = si.n * copysignf(1.0f, -M::Dot(in.d, si.n));
        ONB onb;
        onb.template Build<M>(n);
        float r0, r1;
        s2.Next(r0, r1);
        // importance sampling on: sin theta = sqrt(r0), cos theta = sqrt(1 - sin^2);
        // off (Lambert.cpp:85-107): cos theta = r0, sin theta = sqrt(1 - r0^2), weight
        // f cos / pdf. One body with selects keeps the shade step's code small.
        const bool uni = m.uniform != 0;
        const float phi = 2.0f * kPi * r1;
        const float st = sqrtf(uni ? 1.0f - r0 * r0 : r0);
        const float cu = M::MulCos(st, phi);
        const float cv = M::MulSin(st, phi);
        const float cw = uni ? r0 : sqrtf(SMax(0.0f, 1.0f - st * st));  // >= 0 already with IEEE sqrt
        out.o = si.pos + kEps * n;
        out.d = cu * onb.u + cv * onb.v + cw * onb.w;
        V3 w(m.ar, m.ag, m.ab);
        if (uni) w = (BxDF<M>(m, in.d, out.d, n) * cw) / (0.5f * kInvPi);
        out.T = in.T * w;
        out.bounce = in.bounce + 1;
        return out;
    }
    if (m.kind == kGlossy) {
        const V3 n = si.n * copysignf(1.0f, -M::Dot(in.d, si.n));
        float u0, u1;
        s2.Next(u0, u1);
        const V3 h = SampleVNDF<M>(m, -in.d, si.n, u0, u1);
        const V3 od = Reflected(in.d, h);
        const float hl = fabsf(M::Dot(h, od));
        const V3 f0 = GgxF0(m);
        const V3 F = f0 + (V3(1.f, 1.f, 1.f) - f0) * Pow5(1.0f - hl);
        const float li = GgxLambda<M>(od, h, m.alpha), lo = GgxLambda<M>(-in.d, h, m.alpha);
        const float g2 = 1.0f / (1.0f + li + lo);
        const float g1 = 1.0f / (1.0f + li);
        out.o = si.pos;
        out.d = od;
        out.T = in.T * (F * g2 / g1);
        out.bounce = in.bounce + 1;
        out.o = out.o + kEps * n;
        return out;
    }
    if (m.kind == kGlass) {
        const V3 n = si.n * copysignf(1.0f, -M::Dot(in.d, si.n));
        const float eta = m.ior / in.ior;
        const float dn = M::Dot(in.d, si.n);
        const float disc = dn * dn - 1 + eta * eta;
        if (disc < 0) {  // total internal reflection
            out.o = si.pos + kEps * n;
            out.d = M::Norm(Reflected(in.d, n));
            out.T = V3(0.f, 0.f, 0.f);
            out.bounce = 0 + 1;
            out.prob = in.prob;
            out.ior = in.ior;
            return out;
        }
        const V3 rd = (1.0f / eta) * (in.d - si.n * M::RefractScale(-dn, disc));
        out.d = M::Norm(rd);
        const float nd = M::Dot(si.n, out.d);
        const float q = (1.0f - eta) / (1.0f + eta);
        const float f0 = q * q;
        const float refl = f0 + (1.0f - f0) * Pow5(1.0f - fabsf(nd));
        float r0, r1;
        s2.Next(r0, r1);
        out.T = in.T;
        out.bounce = in.bounce + 1;
        out.prob = in.prob;
        if (r0 <= refl) {  // reflection keeps the refracted direction (Glass.cpp:59-80)
            out.o = si.pos + kEps * n;
            out.ior = in.ior;
        } else {
            out.o = si.pos - kEps * n;
            out.ior = (nd < 0) ? 1.0f * eta : 1.0f / eta;
        }
        return out;
    }
    return out;  // Emission / Mix never reach CreateNextRay
}

// ---------------------------------------------------------------- reference traversal
// Per-ray error bits reported through the status word.
enum : int { kErrStackOverflow = 1, kErrBounceCap = 2, kErrBounds = 4 };

// Checked build (-DPT_CHECK=1): every node, primitive, material and queue index is
// tested against its array before the access; a bad one sets kErrBounds in the
// status word and the access is skipped. The shipped build has no checks (0).
#ifndef PT_CHECK
#define PT_CHECK 0
#endif

// BinnedSAHBVH::Intersect (Core/Accel/BinnedSAHBVH.cpp:272-374) with the slab test
// of BinnedSAHBVH.h:95-170: pop order, culling rule and child push order as the
// reference. Returns the primitive slot of the closest hit, or -1.
// kCount: also count the nodes popped and slab-tested and the triangle tests
// (the reference traversal's work per ray, used for algorithmic-byte accounting).
template <bool kCount = false>
__device__ int TraverseReference(const DevScene& S, V3 o, V3 d, float distMin, float distMax,
                                 float& bestD, int* __restrict__ stack, int* status,
                                 unsigned* nodeTests = nullptr, unsigned* triTests = nullptr) {
    if (S.numNodes == 0) return -1;
    const V3 inv = ExactRecip(d);
    const int s0 = inv.x < 0.0f, s1 = inv.y < 0.0f, s2 = inv.z < 0.0f;
    int sp = 0;
    stack[sp++] = 0;
    int best = -1;
    bestD = kInfinity;
    while (sp > 0) {
        const int ni = stack[--sp];
        if (PT_CHECK && (unsigned)ni >= (unsigned)S.numNodes) {
            *status |= kErrBounds;
            return best;
        }
        if (kCount) (*nodeTests)++;
        const float4 na = __ldg(S.nodes + 2 * ni), nb = __ldg(S.nodes + 2 * ni + 1);
        const V3 lo(na.x, na.y, na.z), hi(na.w, nb.x, nb.y);
        const V3 b0 = s0 ? hi : lo, b1 = s0 ? lo : hi;  // aabb[sign], aabb[1 - sign] for x
        float tMin = __fmul_rn(b0.x - o.x, inv.x);
        float tMax = __fmul_rn(b1.x - o.x, inv.x);
        const float tyMin = __fmul_rn((s1 ? hi : lo).y - o.y, inv.y);
        const float tyMax = __fmul_rn((s1 ? lo : hi).y - o.y, inv.y);
        if (tyMax < tMin || tMax < tyMin) continue;
        if (tMin < tyMin) tMin = tyMin;
        if (tyMax < tMax) tMax = tyMax;
        const float tzMin = __fmul_rn((s2 ? hi : lo).z - o.z, inv.z);
        const float tzMax = __fmul_rn((s2 ? lo : hi).z - o.z, inv.z);
        if (tzMax < tMin || tMax < tzMin) continue;
        if (tMin < tzMin) tMin = tzMin;
        if (tzMax < tMax) tMax = tzMax;
        float nd = kFltMax;
        const bool nearOk = (0.0f <= tMin && tMin < nd);
        if (nearOk) nd = tMin;
        const bool farOk = (0.0f <= tMax && tMax < nd);
        if (farOk) nd = tMax;
        if (!(nearOk || farOk)) continue;
        if (best >= 0) {
            const bool inside = lo.x < o.x && o.x < hi.x && lo.y < o.y && o.y < hi.y &&
                                lo.z < o.z && o.z < hi.z;  // AABB::Contains
            if (!inside && bestD < nd) continue;
        }
        const int a = __float_as_int(nb.z), cnt = __float_as_int(nb.w);
        if (PT_CHECK && (cnt >= 0 ? (a < 0 || a + cnt > S.numTris)
                                  : (a < 0 || a + 1 >= S.numNodes))) {
            *status |= kErrBounds;
            return best;
        }
        if (cnt >= 0) {
            for (int k = a; k < a + cnt; k++) {
                V3 v0, e1, e2;
                LoadTri(S.tris, k, v0, e1, e2);
                if (kCount) (*triTests)++;
                float t;
                if (TriIntersect(v0, e1, e2, o, d, t)) {
                    if (t < distMin || t > distMax) continue;
                    if (best < 0 || t < bestD) {
                        best = k;
                        bestD = t;
                    }
                }
            }
        } else {
            const float4 la = __ldg(S.nodes + 2 * a), lb = __ldg(S.nodes + 2 * a + 1);
            const float4 ra = __ldg(S.nodes + 2 * a + 2), rb = __ldg(S.nodes + 2 * a + 3);
            const float dl = SqLenRn(CentreRn(V3(la.x, la.y, la.z), V3(la.w, lb.x, lb.y)) - o);
            const float dr = SqLenRn(CentreRn(V3(ra.x, ra.y, ra.z), V3(ra.w, rb.x, rb.y)) - o);
            if (sp + 2 > S.stackDepth) {
                *status |= kErrStackOverflow;
                return best;
            }
            if (dl < dr) {
                stack[sp++] = a + 1;
                stack[sp++] = a;
            } else {
                stack[sp++] = a;
                stack[sp++] = a + 1;
            }
        }
    }
    return best;
}

}  // namespace ptg
