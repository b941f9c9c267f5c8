// CPU oracle: a restatement of the reference renderer's hot path in plain C++.
//
// TEST INFRASTRUCTURE ONLY. Tests, the smoke check and the benchmark's CPU
// baseline call this through its C ABI (oracle_*); the product never links it.
//
// Every function mirrors the reference arithmetic operation by operation (same
// operand order, float vs double promotion, no FMA contraction: build with
// -ffp-contract=off), so that its films match the reference bit for bit. Each
// block cites the reference function it restates (paths relative to the
// Petrichor project root).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <thread>
#include <vector>

namespace orc {

constexpr float kEps = 1.0e-3f;                                      // Core/Constants.h:8
constexpr float kInfinity = 0.9f * std::numeric_limits<float>::max(); // Core/Constants.h:10
constexpr float kPi = 3.14159265358979f;                             // Core/Constants.h:15
constexpr float kInvPi = 1.0f / kPi;                                 // Core/Constants.h:16

// ---------------------------------------------------------------- vector math
// Math/Vector3f.h: component-wise operators, Dot, Cross, Length, Normalized.
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator*(V3 a, float c) { return {a.x * c, a.y * c, a.z * c}; }
static inline V3 operator*(float c, V3 a) { return a * c; }  // Vector3f.h:348-351
static inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
static inline V3 operator/(V3 a, float c) { return {a.x / c, a.y / c, a.z / c}; }
static inline V3 operator/(float c, V3 a) { return {c / a.x, c / a.y, c / a.z}; }
static inline float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 Cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Length() = sqrt(Dot) evaluated in double and narrowed (Vector3f.h:169-173);
// double rounding is exact for sqrt, so sqrtf gives the same float.
static inline float Length(V3 a) { return (float)std::sqrt((double)Dot(a, a)); }
static inline V3 Normalized(V3 a) { return a / Length(a); }
static inline float SqLen(V3 a) { return Dot(a, a); }
static inline float MinElem(V3 a) { return std::min(a.x, std::min(a.y, a.z)); }
static inline V3 Reflected(V3 d, V3 n) { return d - 2.0f * n * Dot(d, n); }  // Vector3f.h:202-207
// Vector3f.h:209-234 (nullopt on total internal reflection)
static inline bool Refracted(V3 d, V3 n, float eta, V3* out) {
    const float dn = Dot(d, n);
    const float disc = dn * dn - 1 + eta * eta;
    if (disc < 0) return false;
    const float s = (float)((double)(-dn) + std::sqrt((double)disc));
    *out = (1.0f / eta) * (d - n * s);
    return true;
}
static inline float Mod1(float x) { return x - 1.0f * std::floor(x / 1.0f); }  // MathUtils.h:44-49
static inline float Lerp(float a, float b, float t) { return (1.0f - t) * a + t * b; }
static inline float Pow5(float x) { const float x2 = x * x; return x * (x2 * x2); }
static inline V3 Pow2(V3 c) { return c * c; }
static inline float Luminance(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// ---------------------------------------------------------------- RNG
// Random/XorShift.h:12-59 and Core/Sampler/RandomSampler{1D,2D}
struct XorShift128 {
    uint32_t x = 123456789u, y = 362436069u, z = 521288629u, w;
    explicit XorShift128(uint32_t seed) : w(seed) {}
    uint32_t next_u32() {
        uint32_t t = x ^ (x << 11);
        x = y;
        y = z;
        z = w;
        return w = (w ^ (w >> 19)) ^ (t ^ (t >> 8));
    }
    float next() { return next_u32() / (float)4294967295u; }
};
struct Sampler1D {
    XorShift128 g;
    explicit Sampler1D(uint32_t s) : g(s) {}
    float Next() { return g.next(); }
};
struct Sampler2D {
    XorShift128 g0, g1;
    Sampler2D(uint32_t s0, uint32_t s1) : g0(s0), g1(s1) {}
    void Next(float* a, float* b) {
        *a = g0.next();
        *b = g1.next();
    }
};

// ---------------------------------------------------------------- ONB
// Math/OrthonormalBasis.cpp:10-62
struct ONB {
    V3 u, v, w;
    void Build(V3 n) {
        w = Normalized(n);
        const float sign = std::copysign(1.0f, w.z);
        const float a = -1.0f / (sign + w.z);
        const float b = w.x * w.y * a;
        u = V3(1.0f + sign * w.x * w.x * a, sign * b, -sign * w.x);
        v = V3(b, sign + w.y * w.y * a, -w.y);
    }
    void Build(V3 ww, V3 uu) {
        w = Normalized(ww);
        u = Normalized(uu);
        v = Cross(w, u);
    }
    V3 GetDir(float theta, float phi) const {
        const float cx = (float)(std::sin((double)theta) * std::cos((double)phi));
        const float cy = (float)(std::sin((double)theta) * std::sin((double)phi));
        const float cz = (float)std::cos((double)theta);
        return cx * u + cy * v + cz * w;
    }
    V3 WorldToLocal(V3 a) const { return V3(Dot(a, u), Dot(a, v), Dot(a, w)); }
    V3 LocalToWorld(V3 a) const { return u * a.x + v * a.y + w * a.z; }
};

// ---------------------------------------------------------------- scene data
enum MatKind { kLambert = 0, kGlass = 1, kEmission = 2, kGlossy = 3, kMix = 4 };
struct Material {
    int kind;
    V3 color;  // Lambert kd / GGX reflectance strength / Glass color / Emission color
    float alpha;  // GGX: roughness^2 (GGX.cpp:16-20)
    float ior;
    float mix;
    int mat0, mat1;
    // texture maps (Scene::textures index or -1) and their strengths
    int albedoTex = -1, f0Tex = -1, roughTex = -1, normalTex = -1;
    float roughStrength = 1.0f, normalStrength = 1.0f;
    bool uniform = false;  // MaterialBase::EnableImportanceSampling(false) (read by Lambert)
};
struct Ray {  // Core/Ray.h:42-48
    V3 o, dir;
    V3 T{1, 1, 1};
    int bounce = 0;
    float prob = 1.0f;
    float ior = 1.0f;
};
struct Shading {  // Core/HitInfo.h:20-27
    V3 normal, tangent, pos, uv;
    int material;
};
struct Texture {  // Core/Texture2D.h: AoS RGB float, row-major; "valid" = loaded
    int W = 0, H = 0;
    bool valid = false;
    std::vector<V3> px;
    V3 Get(int i, int j) const {  // Texture2D.cpp:260-271
        if (!(valid && W > 0 && H > 0)) return V3(1.0f, 0.0f, 1.0f);
        return px[(size_t)W * j + i];
    }
    V3 Bilinear(float x, float y) const {  // Texture2D.cpp:287-317
        int ix0 = (int)x, ix1 = (int)(x + 1.0f), iy0 = (int)y, iy1 = (int)(y + 1.0f);
        const float wx0 = x - ix0, wy0 = y - iy0, wx1 = ix1 - x, wy1 = iy1 - y;
        ix0 = std::clamp(ix0, 0, W - 1);
        ix1 = std::clamp(ix1, 0, W - 1);
        iy0 = std::clamp(iy0, 0, H - 1);
        iy1 = std::clamp(iy1, 0, H - 1);
        const V3 c00 = Get(ix0, iy0), c10 = Get(ix1, iy0), c01 = Get(ix0, iy1),
                 c11 = Get(ix1, iy1);
        const V3 cm0 = wx1 * c00 + wx0 * c10;
        const V3 cm1 = wx1 * c01 + wx0 * c11;
        return wy1 * cm0 + wy0 * cm1;
    }
    V3 ByUV(float u, float v) const {  // Texture2D.cpp:327-335
        u = Mod1(u);
        v = Mod1(v);
        return Bilinear(u * W, v * H);
    }
};
struct Env {  // Core/Environment.{h,cpp}
    Texture tex;
    V3 base;
    float rot = 0;
    std::vector<float> pdf1D, cdf1D;
    Texture pdf2D, cdf2D;  // built like the reference: sized but never "loaded"
    bool UseIS() const { return tex.valid && tex.W > 0 && tex.H > 0; }
    void PreCalc() {  // Environment.cpp:56-128
        if (!UseIS()) return;
        const int W = tex.W, H = tex.H;
        pdf2D.W = cdf2D.W = W;
        pdf2D.H = cdf2D.H = H;
        pdf2D.px.assign((size_t)W * H, V3());
        cdf2D.px.assign((size_t)W * H, V3());
        for (int j = 0; j < H; j++)
            for (int i = 1; i < W; i++) {
                const V3 prev = cdf2D.Get(i - 1, j);
                const V3 lum = Luminance(tex.Get(i - 1, j)) * V3(1, 1, 1);
                pdf2D.px[(size_t)W * j + i] = lum;
                cdf2D.px[(size_t)W * j + i] = prev + lum;
            }
        pdf1D.clear();
        cdf1D.clear();
        float sum = 0.0f;
        for (int j = 0; j < H; j++) {
            const float l = cdf2D.Get(W - 1, j).x;
            pdf1D.push_back(l);
            sum += l;
            cdf1D.push_back(sum);
        }
        for (int j = 0; j < H; j++) {
            pdf1D[j] *= (H / sum);
            cdf1D[j] /= sum;
        }
        for (int j = 0; j < H; j++) {
            const V3 maxL = cdf2D.Get(W - 1, j);
            for (int i = 0; i < W; i++) {
                const V3 l = pdf2D.Get(i, j);
                pdf2D.px[(size_t)W * j + i] = l * (V3((float)W, (float)W, (float)W) / maxL);
                cdf2D.px[(size_t)W * j + i] = cdf2D.Get(i, j) / maxL;
            }
        }
    }
    V3 GetColor(V3 d) const {  // Environment.cpp:29-48
        if (!tex.valid) return base;
        const float theta = (float)std::acos((double)d.z);
        const float phi = (float)std::atan2((double)d.y, (double)d.x);
        float u = 1.0f - (phi - rot) * 0.5f * kInvPi;
        float v = theta * kInvPi;
        u = Mod1(u);
        v = Mod1(v);
        return base * tex.ByUV(u, v);
    }
    V3 Sample(Sampler2D& s2, float* pdf) const {  // Environment.cpp:130-220
        if (!UseIS()) return V3(1, 0, 0);
        const float tw = 1.0f / pdf2D.W, th = 1.0f / pdf2D.H;
        float r0, r1;
        s2.Next(&r0, &r1);
        float v0 = 0.0f, v1 = 1.0f;
        for (;;) {
            const float v = 0.5f * (v0 + v1);
            const float y = v * cdf2D.H;
            const int fy = (int)y;
            const int cy = std::min(fy + 1, cdf2D.H - 1);
            const float c = Lerp(cdf1D[fy], cdf1D[cy], y - fy);
            const float diff = c - r0;
            if (v1 - v0 <= th) { v0 = v1 = v; break; }
            if (diff > 0) v1 = v;
            else if (diff < 0) v0 = v;
            else { v0 = v1 = v; break; }
        }
        float u0 = 0.0f, u1 = 1.0f;
        for (;;) {
            const float u = 0.5f * (u0 + u1);
            const float c = cdf2D.ByUV(u, v0).x;
            const float diff = c - r1;
            if (u1 - u0 <= tw) { u0 = u1 = u; break; }
            if (diff >= 0) u1 = u;
            else u0 = u;
        }
        if (pdf) {
            const float y = v0 * pdf2D.H;
            const int y0 = (int)y;
            const int y1 = std::min(y0 + 1, pdf2D.H - 1);
            const float py = Lerp(pdf1D[y0], pdf1D[y1], y - y0);
            *pdf = py * pdf2D.ByUV(u0, v0).x;
        }
        const float theta = v0 * kPi;
        const float phi = 2.0f * kPi * (1.0f - u0) + rot;
        ONB onb;
        onb.Build(V3(0, 0, 1), V3(1, 0, 0));
        return onb.GetDir(theta, phi);
    }
    float Pdf(V3 d) const {  // Environment.cpp:222-244
        if (!UseIS()) return 1.0f;
        const float theta = (float)std::acos((double)d.z);
        const float phi = (float)std::atan2((double)d.y, (double)d.x);
        const float u0 = 1.0f - (phi - rot) * 0.5f * kInvPi;
        const float v0 = theta * kInvPi;
        const float y = v0 * pdf2D.H;
        // d.z == -1 gives y == H: an out-of-range read (undefined) in the reference;
        // clamped to the last row here.
        const int y0 = std::min((int)y, pdf2D.H - 1);
        const int y1 = std::min(y0 + 1, pdf2D.H - 1);
        const float py = Lerp(pdf1D[y0], pdf1D[y1], y - y0);
        return py * pdf2D.ByUV(u0, v0).x;
    }
};
struct Camera {  // Core/Camera.{h,cpp}
    V3 pos, right, up, fwd;
    float focusDist = 1.0f, sensorH = 24e-3f, hPerf = 24e-3f / 55e-3f, aperture = 25e-3f;
    void SetViewDir(V3 d) {  // Camera.cpp:38-44
        fwd = Normalized(d);
        right = Cross(fwd, V3(0, 0, 1));
        up = Cross(right, fwd);
    }
    Ray Generate(int i, int j, int W, int H, Sampler2D& s2) const {  // Camera.cpp:52-91
        float r0, r1;
        s2.Next(&r0, &r1);
        const float aspect = (float)W / H;
        const float u = (i + r0) / W - 0.5f;
        const float v = (j + r1) / H - 0.5f;
        const V3 onSensor = pos + right * u * hPerf * focusDist * aspect +
                            -up * v * hPerf * focusDist + fwd * focusDist;
        s2.Next(&r0, &r1);
        const float r = (float)std::sqrt((double)r0);
        const float theta = 2.0f * kPi * r1;
        const V3 onLens = pos + right * 0.5f * aperture * r * (float)std::cos((double)theta) +
                          -up * 0.5f * aperture * r * (float)std::sin((double)theta);
        const V3 dir = Normalized(onSensor - onLens);
        const float d = Dot(dir, fwd);
        Ray ray;
        ray.o = onLens;
        ray.dir = dir;
        ray.T = V3(1, 1, 1) * d * d * focusDist * focusDist / SqLen(onSensor - onLens);
        return ray;
    }
};

struct BVHNode {  // Core/Accel/BinnedSAHBVH.h:23-52
    V3 lo{FLT_MAX, FLT_MAX, FLT_MAX};
    V3 hi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int child[2] = {0, 0};
    int begin = 0, end = 0;
    bool leaf = false;
};

struct Scene {
    int W, H, spp, maxBounces, tileW, tileH, numThreads, integrator;
    Camera cam;
    Env env;
    std::vector<Material> mats;
    std::vector<V3> P, N, UV;
    std::vector<int> idx, triMat;
    std::vector<uint8_t> shade;
    std::vector<int> lights;
    std::vector<Texture> textures;  // material texture maps (loaded textures)
    // BVH
    std::vector<BVHNode> nodes;
    std::vector<int> primIDs;
    int maxDepth = 0;
    bool built = false;

    int NumTris() const { return (int)triMat.size(); }
    V3 Pv(int t, int k) const { return P[idx[t * 3 + k]]; }
    int GetMaterial(int t, float r) const {  // GeometryBase.h:59-69, MixMaterial.h:45-50
        const int m = triMat[t];
        if (m >= 0 && mats[m].kind == kMix) return mats[m].mix <= r ? mats[m].mat0 : mats[m].mat1;
        return m;
    }
};

// ---------------------------------------------------------------- triangle
// Core/Geometry/Triangle.cpp:51-88
static inline bool TriIntersect(const Scene& s, int t, const Ray& ray, float* dist) {
    const V3 v0 = s.Pv(t, 0);
    const V3 e1 = s.Pv(t, 1) - v0;
    const V3 e2 = s.Pv(t, 2) - v0;
    const V3 ce = Cross(e1, e2);
    const float invDet = 1.0f / Dot(-ray.dir, ce);
    const V3 vec = ray.o - v0;
    const float w1 = Dot(vec, Cross(ray.dir, e2)) * invDet;
    const float w2 = Dot(vec, Cross(e1, ray.dir)) * invDet;
    if (w1 < 0.0f || w1 >= 1.0f) return false;
    if (w2 < 0.0f || w2 >= 1.0f) return false;
    if (w1 + w2 >= 1.0f) return false;
    const float d = Dot(vec, ce) * invDet;
    if (d < 0.0f) return false;
    *dist = d;
    return true;
}
// Triangle.cpp:90-153
static Shading Interpolate(const Scene& s, int t, const Ray& ray, float dist) {
    Shading si;
    si.pos = ray.o + ray.dir * dist;
    const V3 v0 = s.Pv(t, 0);
    const V3 e1 = s.Pv(t, 1) - v0;
    const V3 e2 = s.Pv(t, 2) - v0;
    const V3 ce = Cross(e1, e2);
    const float invDet = 1.0f / Dot(-ray.dir, ce);
    const V3 vec = ray.o - v0;
    const float w1 = Dot(vec, Cross(ray.dir, e2)) * invDet;
    const float w2 = Dot(vec, Cross(e1, ray.dir)) * invDet;
    const int i0 = s.idx[t * 3], i1 = s.idx[t * 3 + 1], i2 = s.idx[t * 3 + 2];
    const V3 duv1 = s.UV[i1] - s.UV[i0];
    const V3 duv2 = s.UV[i2] - s.UV[i0];
    si.uv = w1 * duv1 + w2 * duv2 + s.UV[i0];
    si.tangent = duv2.y * e1 - duv1.y * e2;
    if (s.shade[t] == 0) {
        si.normal = Normalized(ce);
    } else {
        si.normal = w1 * (s.N[i1] - s.N[i0]) + w2 * (s.N[i2] - s.N[i0]) + s.N[i0];
        si.normal = Normalized(si.normal);
        si.tangent = si.tangent - Dot(si.normal, si.tangent) * si.normal;
    }
    if (SqLen(si.tangent) == 0.0f) si.tangent = V3(1, 0, 0);
    si.material = s.GetMaterial(t, 0.0f);
    return si;
}
// Triangle.cpp:155-182
static void SampleSurface(const Scene& s, int t, Sampler2D& s2, V3* pos, float* pdfArea) {
    const V3 v0 = s.Pv(t, 0);
    const V3 e0 = s.Pv(t, 1) - v0;
    const V3 e1 = s.Pv(t, 2) - v0;
    float u0, u1;
    s2.Next(&u0, &u1);
    const float su = (float)std::sqrt((double)u0);
    *pos = v0 + (1.0f - su) * e0 + su * u1 * e1;
    *pdfArea = 1.0f / (0.5f * Length(Cross(e0, e1)));
}

// ---------------------------------------------------------------- BVH
// Core/Accel/AABB.cpp:10-52
static inline void Merge(V3& lo, V3& hi, V3 blo, V3 bhi) {
    lo.x = std::min(lo.x, blo.x); lo.y = std::min(lo.y, blo.y); lo.z = std::min(lo.z, blo.z);
    hi.x = std::max(hi.x, bhi.x); hi.y = std::max(hi.y, bhi.y); hi.z = std::max(hi.z, bhi.z);
}
static inline float SurfaceArea(V3 lo, V3 hi) {  // AABB.h:71-76
    const V3 d = hi - lo;
    return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
}
static inline int WidestAxis(V3 lo, V3 hi) {  // AABB.cpp:54-71
    float best = 0.0f;
    int axis = 0;
    for (int a = 0; a < 3; a++) {
        const float w = hi[a] - lo[a];
        if (w > best) { best = w; axis = a; }
    }
    return axis;
}

// Core/Accel/BinnedSAHBVH.cpp:15-225 (build) and :227-270 (GetSAHCost)
static void BuildBVH(Scene& s) {
    constexpr int kBins = 16;
    const int n = s.NumTris();
    struct Prim { int bin; V3 lo, hi, c; };
    std::vector<Prim> pd(n);
    for (int t = 0; t < n; t++) {
        V3 lo{FLT_MAX, FLT_MAX, FLT_MAX}, hi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < 3; k++) Merge(lo, hi, s.Pv(t, k), s.Pv(t, k));
        pd[t] = {-1, lo, hi, (s.Pv(t, 0) + s.Pv(t, 1) + s.Pv(t, 2)) / 3.0f};
    }
    s.nodes.clear();
    s.nodes.reserve(2 * (size_t)n + 1);
    BVHNode root;
    for (int t = 0; t < n; t++) Merge(root.lo, root.hi, pd[t].lo, pd[t].hi);
    root.begin = 0;
    root.end = n;
    s.nodes.push_back(root);
    std::vector<uint32_t> stack{0};
    int depth = 1;
    s.maxDepth = 0;
    s.primIDs.resize(n);
    for (int i = 0; i < n; i++) s.primIDs[i] = i;
    while (!stack.empty()) {
        const uint32_t ni = stack.back();
        stack.pop_back();
        const int b = s.nodes[ni].begin, e = s.nodes[ni].end;
        if (e - b <= 4) { s.nodes[ni].leaf = true; depth--; continue; }
        V3 clo{FLT_MAX, FLT_MAX, FLT_MAX}, chi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int i = b; i < e; i++) Merge(clo, chi, pd[s.primIDs[i]].c, pd[s.primIDs[i]].c);
        const int ax = WidestAxis(clo, chi);
        std::sort(s.primIDs.begin() + b, s.primIDs.begin() + e,
                  [&](int a, int c) { return pd[a].c[ax] < pd[c].c[ax]; });
        const float len = chi[ax] - clo[ax];
        for (int i = b; i < e; i++) {
            Prim& p = pd[s.primIDs[i]];
            const float l = p.c[ax] - clo[ax];
            const float f = std::nextafter(kBins * l / len, 0.0f);
            // A zero-width centroid range gives NaN here; the reference converts it with
            // an undefined float->int cast. Every such node becomes a leaf either way
            // (all primitives land on one side for every candidate split).
            p.bin = std::isnan(f) ? 0 : (int)f;
        }
        int bestBin = 0, bestLeft = 0;
        float minCost = std::numeric_limits<float>::max();
        for (int k = 0; k < kBins; k++) {
            V3 llo{FLT_MAX, FLT_MAX, FLT_MAX}, lhi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
            V3 rlo = llo, rhi = lhi;
            int nl = 0, nr = 0;
            for (int i = b; i < e; i++) {
                const Prim& p = pd[s.primIDs[i]];
                if (p.bin < k) { Merge(llo, lhi, p.lo, p.hi); nl++; }
                else { Merge(rlo, rhi, p.lo, p.hi); nr++; }
            }
            const float sal = nl ? SurfaceArea(llo, lhi) : 0;
            const float sar = nr ? SurfaceArea(rlo, rhi) : 0;
            const float cost = nl * sal + nr * sar;
            if (cost < minCost) { minCost = cost; bestBin = k; bestLeft = nl; }
        }
        if (bestBin == 0) { depth--; s.nodes[ni].leaf = true; continue; }
        depth++;
        s.maxDepth = std::max(s.maxDepth, depth);
        V3 llo{FLT_MAX, FLT_MAX, FLT_MAX}, lhi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
        V3 rlo = llo, rhi = lhi;
        for (int i = b; i < e; i++) {
            const Prim& p = pd[s.primIDs[i]];
            if (p.bin < bestBin) Merge(llo, lhi, p.lo, p.hi);
            else Merge(rlo, rhi, p.lo, p.hi);
        }
        BVHNode L, R;
        L.lo = llo; L.hi = lhi; L.child[0] = L.child[1] = -1; L.begin = b; L.end = b + bestLeft;
        R.lo = rlo; R.hi = rhi; R.child[0] = R.child[1] = -1; R.begin = b + bestLeft; R.end = e;
        s.nodes.push_back(L);
        const int li = (int)s.nodes.size() - 1;
        stack.push_back(li);
        s.nodes.push_back(R);
        const int ri = (int)s.nodes.size() - 1;
        stack.push_back(ri);
        s.nodes[ni].child[0] = li;
        s.nodes[ni].child[1] = ri;
    }
    s.built = true;
}

thread_local long tl_triTests = 0;

// BinnedSAHBVH.h:95-170 (slab test with the reference's near/far choice)
static inline bool SlabHit(const BVHNode& nd, const Ray& r, V3 inv, const int* sg, float* dist) {
    const V3 b[2] = {nd.lo, nd.hi};
    float tMin = (b[sg[0]].x - r.o.x) * inv.x;
    float tMax = (b[1 - sg[0]].x - r.o.x) * inv.x;
    const float tyMin = (b[sg[1]].y - r.o.y) * inv.y;
    const float tyMax = (b[1 - sg[1]].y - r.o.y) * inv.y;
    if (tyMax < tMin || tMax < tyMin) return false;
    if (tMin < tyMin) tMin = tyMin;
    if (tyMax < tMax) tMax = tyMax;
    const float tzMin = (b[sg[2]].z - r.o.z) * inv.z;
    const float tzMax = (b[1 - sg[2]].z - r.o.z) * inv.z;
    if (tzMax < tMin || tMax < tzMin) return false;
    if (tMin < tzMin) tMin = tzMin;
    if (tzMax < tMax) tMax = tzMax;
    float d = std::numeric_limits<float>::max();
    const bool nearOk = (0.0f <= tMin && tMin < d);
    if (nearOk) d = tMin;
    const bool farOk = (0.0f <= tMax && tMax < d);
    if (farOk) d = tMax;
    if (!(nearOk || farOk)) return false;
    *dist = d;
    return true;
}
static inline bool Contains(const BVHNode& n, V3 p) {  // AABB.h:58-68
    return n.lo.x < p.x && p.x < n.hi.x && n.lo.y < p.y && p.y < n.hi.y && n.lo.z < p.z &&
           p.z < n.hi.z;
}

// BinnedSAHBVH.cpp:272-374. Returns the triangle index or -1.
static int Intersect(const Scene& s, const Ray& ray, float distMin, float distMax, float* outDist) {
    const V3 inv = 1.0f / ray.dir;
    const int sg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
    thread_local std::vector<int> st;
    st.clear();
    st.push_back(0);
    int best = -1;
    float bestD = kInfinity;
    if (s.nodes.empty()) return -1;
    while (!st.empty()) {
        const int ni = st.back();
        st.pop_back();
        const BVHNode& nd = s.nodes[ni];
        float nd_d;
        if (!SlabHit(nd, ray, inv, sg, &nd_d)) continue;
        if (best >= 0 && !Contains(nd, ray.o)) {
            if (bestD < nd_d) continue;
        }
        if (nd.leaf) {
            for (int k = nd.begin; k < nd.end; k++) {
                const int t = s.primIDs[k];
                float d;
                tl_triTests++;
                if (TriIntersect(s, t, ray, &d)) {
                    if (d < distMin || d > distMax) continue;
                    if (best < 0 || d < bestD) { best = t; bestD = d; }
                }
            }
        } else {
            const int l = nd.child[0], r = nd.child[1];
            const float dl = SqLen((s.nodes[l].lo + s.nodes[l].hi) * 0.5f - ray.o);
            const float dr = SqLen((s.nodes[r].lo + s.nodes[r].hi) * 0.5f - ray.o);
            if (dl < dr) { st.push_back(r); st.push_back(l); }
            else { st.push_back(l); st.push_back(r); }
        }
    }
    *outDist = bestD;
    return best;
}
static inline int IntersectDefault(const Scene& s, const Ray& r, float* d) {  // AccelBase.h:44-48
    return Intersect(s, r, 0.0f, std::numeric_limits<float>::max(), d);
}

// ---------------------------------------------------------------- materials
// Texture2D::GetPixelByUV (Texture2D.cpp:327-335): wrap, then bilinear at (u W, v H)
static inline V3 TexByUV(const Texture& t, float u, float v) {
    u = Mod1(u);
    v = Mod1(v);
    return t.Bilinear(u * t.W, v * t.H);
}
// Lambert::GetAlbedo (Lambert.cpp:117-126)
static inline V3 LambertAlbedo(const Scene& s, const Material& m, const Shading& si) {
    if (m.albedoTex < 0) return V3(1, 1, 1);
    return m.color * TexByUV(s.textures[m.albedoTex], si.uv.x, si.uv.y);
}
// GGX::GetF0 (GGX.h:126-139), metalness 0
static inline V3 GgxF0(const Scene& s, const Material& m, const Shading& si) {
    V3 refl = m.color;
    if (m.f0Tex >= 0) refl = refl * TexByUV(s.textures[m.f0Tex], si.uv.x, si.uv.y);
    return 0.16f * Pow2(refl) * (1.0f - 0.0f) + V3(1, 1, 1) * 0.0f;
}
// GGX::GetAlpha (GGX.h:57-73)
static inline float GgxAlpha(const Scene& s, const Material& m, const Shading& si) {
    if (m.roughTex < 0) return m.alpha;
    const float r = m.roughStrength * Luminance(TexByUV(s.textures[m.roughTex], si.uv.x, si.uv.y));
    return r * r;
}
// GGX::GetNormal (GGX.h:95-121)
static inline V3 GgxNormal(const Scene& s, const Material& m, const Shading& si) {
    if (m.normalTex < 0) return si.normal;
    ONB b;
    b.Build(si.normal, si.tangent);
    const V3 nm = TexByUV(s.textures[m.normalTex], si.uv.x, si.uv.y);
    const V3 ln = Normalized(2.0f * nm - V3(1, 1, 1));
    return (1.0f - m.normalStrength) * ln.x * b.u + ln.y * b.v + (1.0f - m.normalStrength) * ln.z * b.w;
}
static inline float GgxLambda(V3 dir, V3 h, float alpha) {  // GGX.cpp:140-152
    const float a2 = alpha * alpha;
    const float c = std::abs(Dot(dir, h));
    const float tan2 = c > 0 ? 1.0f / (c * c) - 1.0f : kInfinity;
    return (float)((double)-0.5f + (double)0.5f * std::sqrt((double)(1.0f + a2 * tan2)));
}
static V3 BxDF(const Scene& s, int m, const Ray& in, const Ray& out, const Shading& si) {
    const Material& M = s.mats[m];
    switch (M.kind) {
    case kLambert:  // Lambert.cpp:27-31
        return M.color * LambertAlbedo(s, M, si) * kInvPi;
    case kGlossy: {  // GGX.cpp:22-57
        const V3 n = GgxNormal(s, M, si);
        const V3 h = Normalized(-in.dir + out.dir);
        const float hn = std::abs(Dot(h, n));
        const float a = GgxAlpha(s, M, si), a2 = a * a, hn2 = hn * hn;
        const float k = (a2 - 1.0f) * hn2 + 1.0f;
        const float D = a2 / (kPi * k * k);
        const float li = GgxLambda(out.dir, h, a), lo = GgxLambda(-in.dir, h, a);
        const float G = 1.0f / (1.0f + li + lo);
        const float hl = std::abs(Dot(h, out.dir));
        const V3 F = GgxF0(s, M, si) + (V3(1, 1, 1) - GgxF0(s, M, si)) * Pow5(1.0f - hl);
        const float ln = std::abs(Dot(out.dir, n)), vn = std::abs(Dot(-in.dir, n));
        return D * G * F / (4.0f * ln * vn);
    }
    default:  // Glass (Glass.cpp:11-18) and anything else
        return V3(0, 0, 0);
    }
}
static float PDF(const Scene& s, int m, const Ray& in, const Ray& out, const Shading& si) {
    const Material& M = s.mats[m];
    switch (M.kind) {
    case kLambert:  // Lambert.cpp:33-47
        if (M.uniform) return 0.5f * kInvPi;
        return std::abs(Dot(out.dir, si.normal)) * kInvPi;
    case kGlossy: {  // GGX.cpp:59-76
        const V3 h = Normalized(-in.dir + out.dir);
        const float hn = std::abs(Dot(h, GgxNormal(s, M, si)));
        const float alpha = GgxAlpha(s, M, si);
        const float a2 = alpha * alpha, hn2 = hn * hn;
        const float tmp = 1.0f - (1.0f - a2) * hn2;
        return tmp > 0 ? kInvPi * a2 / (tmp * tmp) : kInfinity;
    }
    default:
        return 0.0f;
    }
}
// GGX.cpp:154-208
static V3 SampleVNDF(const Scene& s, const Material& M, V3 view, const Shading& si, Sampler2D& s2) {
    const V3 n0 = GgxNormal(s, M, si);
    const V3 n = n0 * std::copysign(1.0f, Dot(view, n0));
    ONB surf;
    const V3 t = (std::abs(n.z) < 0.9999f) ? Cross(n, V3(0, 0, 1)) : V3(1, 0, 0);
    surf.Build(n, t);
    V3 v = surf.WorldToLocal(view);
    const float alpha = GgxAlpha(s, M, si);
    v = v * V3(alpha, alpha, 1.0f);
    v = v / Length(v);
    const V3 t1 = (v.z < 0.9999f) ? Normalized(Cross(v, V3(0, 0, 1))) : V3(1, 0, 0);
    const V3 t2 = Cross(t1, v);
    float u0, u1;
    s2.Next(&u0, &u1);
    const float a = 1.0f / (1.0f + v.z);
    const float r = (float)std::sqrt((double)u0);
    const float phi = (u1 < a) ? u1 / a * kPi : kPi + (u1 - a) / (1.0f - a) * kPi;
    const float p1 = (float)((double)r * std::cos((double)phi));
    const float p2 = (float)((double)r * std::sin((double)phi) * (double)((u1 < a) ? 1.0f : v.z));
    const float w = (float)std::sqrt((double)std::max(0.0f, 1.0f - p1 * p1 - p2 * p2));
    V3 h = p1 * t1 + p2 * t2 + w * v;
    h = V3(alpha * h.x, alpha * h.y, std::max(0.0f, h.z));
    h = surf.LocalToWorld(h);
    return h / Length(h);
}
static Ray NextRay(const Scene& s, int m, const Ray& in, const Shading& si, Sampler2D& s2) {
    const Material& M = s.mats[m];
    Ray out;
    switch (M.kind) {
    case kLambert: {  // Lambert.cpp:49-98
        const V3 n = si.normal * std::copysign(1.0f, -Dot(in.dir, si.normal));
        ONB onb;
        onb.Build(n);
        float r0, r1;
        s2.Next(&r0, &r1);
        if (M.uniform) {  // Lambert.cpp:85-107
            const float ct = r0;
            const float st = (float)std::sqrt((double)(1.0f - ct * ct));
            const float phi = 2.0f * kPi * r1;
            const float cu = (float)((double)st * std::cos((double)phi));
            const float cv = (float)((double)st * std::sin((double)phi));
            out.o = si.pos + kEps * n;
            out.dir = cu * onb.u + cv * onb.v + ct * onb.w;
            out.T = in.T;
            out.bounce = in.bounce + 1;
            const V3 f = BxDF(s, m, in, out, si);
            out.T = out.T * (f * ct / PDF(s, m, in, out, si));
            return out;
        }
        const float phi = 2.0f * kPi * r1;
        const float st = (float)std::sqrt((double)r0);
        const float cu = (float)((double)st * std::cos((double)phi));
        const float cv = (float)((double)st * std::sin((double)phi));
        const float cw = (float)std::sqrt((double)(1.0f - st * st));
        out.o = si.pos + kEps * n;
        out.dir = cu * onb.u + cv * onb.v + cw * onb.w;
        out.T = in.T * LambertAlbedo(s, M, si);
        out.bounce = in.bounce + 1;
        return out;
    }
    case kGlossy: {  // GGX.cpp:78-138
        const V3 n0 = GgxNormal(s, M, si);
        const V3 n = n0 * std::copysign(1.0f, -Dot(in.dir, n0));
        const V3 h = SampleVNDF(s, M, -in.dir, si, s2);
        const V3 od = Reflected(in.dir, h);
        const float hl = std::abs(Dot(h, od));
        const V3 f0 = GgxF0(s, M, si);
        const V3 F = f0 + (V3(1, 1, 1) - f0) * Pow5(1.0f - hl);
        out.o = si.pos;
        out.dir = od;
        out.T = in.T;
        out.bounce = in.bounce + 1;
        const float alpha = GgxAlpha(s, M, si);
        const float li = GgxLambda(od, h, alpha), lo = GgxLambda(-in.dir, h, alpha);
        const float g2 = 1.0f / (1.0f + li + lo);
        const float g1 = 1.0f / (1.0f + li);
        out.T = out.T * (F * g2 / g1);
        out.o = out.o + kEps * n;
        return out;
    }
    case kGlass: {  // Glass.cpp:29-95
        const V3 n = si.normal * std::copysign(1.0f, -Dot(in.dir, si.normal));
        const float eta = M.ior / in.ior;
        V3 rd;
        if (!Refracted(in.dir, si.normal, eta, &rd)) {
            out.o = si.pos + kEps * n;
            out.dir = Normalized(Reflected(in.dir, n));
            out.T = V3(0, 0, 0);
            out.bounce = out.bounce + 1;
            out.prob = in.prob;
            out.ior = in.ior;
            return out;
        }
        out.dir = Normalized(rd);
        const float nd = Dot(si.normal, out.dir);
        const float q = (1.0f - eta) / (1.0f + eta);
        const float f0 = q * q;
        const float refl = f0 + (1.0f - f0) * Pow5(1.0f - std::abs(nd));
        float r0, r1;
        s2.Next(&r0, &r1);
        if (r0 <= refl) {
            out.o = si.pos + kEps * n;
            out.T = in.T;
            out.bounce = in.bounce + 1;
            out.prob = in.prob;
            out.ior = in.ior;
            return out;
        }
        out.o = si.pos - kEps * n;
        out.T = in.T;
        out.bounce = in.bounce + 1;
        out.prob = in.prob;
        out.ior = (nd < 0) ? out.ior * eta : out.ior / eta;
        return out;
    }
    default:  // Emission / Mix never reach here in the reference (ASSERT(false))
        return out;
    }
}

// ---------------------------------------------------------------- integrators
// Core/Integrator/SimplePathTracing.cpp:16-101
static void RenderSimple(const Scene& s, int px, int py, float* film, Sampler1D& s1, Sampler2D& s2) {
    V3 sum;
    for (int sp = 0; sp < s.spp; sp++) {
        Ray ray = s.cam.Generate(px, py, s.W, s.H, s2);
        V3 contrib;
        for (;;) {
            float d;
            const int t = Intersect(s, ray, kEps, kInfinity, &d);
            if (t < 0) {
                contrib = contrib + ray.T * s.env.GetColor(ray.dir);
                break;
            }
            const int m = s.GetMaterial(t, s1.Next());
            if (s.mats[m].kind == kEmission) {
                contrib = contrib + ray.T * s.mats[m].color;
                break;
            }
            const Shading si = Interpolate(s, t, ray, d);
            ray = NextRay(s, m, ray, si, s2);
            if (ray.bounce > s.maxBounces) {
                ray.prob *= 0.9f;
                ray.prob = std::max(0.1f, ray.prob);
                if (s1.Next() < ray.prob) ray.T = ray.T / ray.prob;
                else break;
            }
        }
        sum = sum + contrib;
    }
    const V3 avg = sum / (float)s.spp;
    float* o = film + ((size_t)py * s.W + px) * 3;
    o[0] = avg.x; o[1] = avg.y; o[2] = avg.z;
}

// ---------------------------------------------------------------- AOV passes
// Core/AOV/AOVUVCoordinate.cpp:11-51: numSamplesPerPixel camera rays; hit uv summed.
static void RenderAovUV(const Scene& s, int px, int py, float* film, Sampler2D& s2) {
    V3 sum;
    for (int sp = 0; sp < s.spp; sp++) {
        const Ray ray = s.cam.Generate(px, py, s.W, s.H, s2);
        float d;
        const int t = Intersect(s, ray, kEps, kInfinity, &d);
        if (t >= 0) sum = sum + Interpolate(s, t, ray, d).uv;
    }
    const V3 avg = sum / (float)s.spp;
    float* o = film + ((size_t)py * s.W + px) * 3;
    o[0] = avg.x; o[1] = avg.y; o[2] = avg.z;
}
// AOVDenoisingAlbedo.cpp:56-133 (normal == false) and AOVDenoisingNormal.cpp:54-128
// (normal == true): follow specular glass / zero-roughness GGX bounces up to
// numMaxBounces, then report the first diffuse-like surface (or the environment).
static V3 AovPath(const Scene& s, Ray ray, bool normal, Sampler1D& s1, Sampler2D& s2) {
    for (int bounce = 0; bounce < s.maxBounces; bounce++) {
        float d;
        const int t = Intersect(s, ray, kEps, kInfinity, &d);
        if (t < 0) return normal ? ray.T * (-ray.dir) : ray.T * s.env.GetColor(ray.dir);
        const int m = s.GetMaterial(t, s1.Next());
        const Shading si = Interpolate(s, t, ray, d);
        const Material& M = s.mats[m];
        switch (M.kind) {
        case kLambert:
            return normal ? ray.T * si.normal : ray.T * LambertAlbedo(s, M, si);
        case kGlass:  // Glass::GetAlpha is 0: always follows the refracted/reflected ray
            ray = NextRay(s, m, ray, si, s2);
            break;
        case kGlossy:
            if (GgxAlpha(s, M, si) != 0) return normal ? ray.T * si.normal : ray.T * GgxF0(s, M, si);
            ray = NextRay(s, m, ray, si, s2);
            break;
        default:  // Emission: the ASSERT(false) branch returns zero in release builds
            return V3();
        }
    }
    return V3();
}
static void RenderAovDenoise(const Scene& s, bool normal, int dspp, int px, int py, float* film,
                             Sampler1D& s1, Sampler2D& s2) {
    V3 sum;
    for (int sp = 0; sp < dspp; sp++) {
        const Ray ray = s.cam.Generate(px, py, s.W, s.H, s2);
        sum = sum + AovPath(s, ray, normal, s1, s2);
    }
    const V3 avg = sum / (float)dspp;
    float* o = film + ((size_t)py * s.W + px) * 3;
    o[0] = avg.x; o[1] = avg.y; o[2] = avg.z;
}

// PathTracing.cpp:329-386
static V3 SampleLight(const Scene& s, V3 o, float rv, Sampler2D& s2, float* pdfArea,
                      bool* sampleEnv) {
    const size_t L = s.lights.size();
    int index;
    if (sampleEnv == nullptr) {
        index = (int)(rv * L);
        index = std::min(index, (int)(L - 1));
    } else {
        index = (int)(rv * (L + 1));
        index = std::min(index, (int)L);
        if ((size_t)index >= L) { *sampleEnv = true; return V3(); }
    }
    float sumArea = 0.0f;
    V3 result;
    for (size_t i = 0; i < L; i++) {
        V3 p;
        float pa = 0.0f;
        SampleSurface(s, s.lights[i], s2, &p, &pa);
        sumArea += 1.0f / pa;
        if (i == (size_t)index) result = p;
    }
    if (pdfArea) *pdfArea = 1.0f / sumArea;
    return result;
}

// PathTracing.cpp:202-327
static V3 LightContribution(const Scene& s, const Shading& si, Sampler1D& s1, Sampler2D& s2,
                            const Ray& ray) {
    V3 lc;
    const float dt = -Dot(ray.dir, si.normal);
    const V3 p = si.pos + kEps * std::copysign(1.0f, dt) * si.normal;
    float pdfArea = 1.0f;
    bool sampleEnv = false;
    const V3 pl = SampleLight(s, p, s1.Next(), s2, &pdfArea, &sampleEnv);
    if (!sampleEnv) {
        if (s.lights.empty()) return V3();
        Ray toL;
        toL.o = p;
        toL.dir = Normalized(pl - p);
        float d;
        const int t = IntersectDefault(s, toL, &d);
        if (t >= 0 && s.mats[s.GetMaterial(t, s1.Next())].kind == kEmission) {
            const Shading sl = Interpolate(s, t, toL, d);
            const float dist = SqLen(pl - sl.pos);
            if (std::abs(dist - 0.0f) < kEps) {
                const int m = si.material;
                const float l2 = SqLen(sl.pos - si.pos);
                const float cosP = std::abs(Dot(toL.dir, sl.normal));
                float mis = 0.0f;
                if (l2 > 0.0f) {
                    const float pL = pdfArea;
                    const float pB = PDF(s, m, ray, toL, si) * cosP / l2;
                    mis = pL * pL / (pL * pL + pB * pB);
                }
                const V3 li = s.mats[sl.material].color;
                const V3 f = BxDF(s, m, ray, toL, si);
                const float c = std::abs(Dot(toL.dir, si.normal));
                lc = lc + mis * ray.T * (li * f * c * cosP / (pdfArea * l2));
            }
        }
    } else if (s.env.UseIS()) {
        float pdfuv = 0.0f;
        const V3 sd = s.env.Sample(s2, &pdfuv);
        Ray toE;
        toE.o = si.pos + kEps * std::copysign(1.0f, dt) * si.normal;
        toE.dir = sd;
        float d;
        if (IntersectDefault(s, toE, &d) < 0) {
            const float c = std::abs(Dot(toE.dir, si.normal));
            const float sn = (float)std::sqrt((double)std::max(0.0f, 1.0f - c * c));
            const int m = si.material;
            const float pB = 2.0f * kPi * kPi * sn * PDF(s, m, ray, toE, si);
            const float mis = pdfuv * pdfuv / (pdfuv * pdfuv + pB * pB);
            const V3 li = s.env.GetColor(toE.dir);
            const V3 f = BxDF(s, m, ray, toE, si);
            lc = lc + mis * ray.T * (li * f * sn * c * 2.0f * kPi * kPi) / pdfuv;
        }
    }
    return lc;
}

// PathTracing.cpp:20-200
static void RenderPT(const Scene& s, int px, int py, float* film, Sampler1D& s1, Sampler2D& s2) {
    V3 sum;
    for (int sp = 0; sp < s.spp; sp++) {
        V3 color;
        Ray ray = s.cam.Generate(px, py, s.W, s.H, s2);
        Ray prev = ray;
        Shading si;
        {
            float d;
            const int t = IntersectDefault(s, ray, &d);
            if (t < 0) {
                sum = sum + ray.T * s.env.GetColor(ray.dir);
                continue;
            }
            si = Interpolate(s, t, ray, d);
        }
        int m = si.material;
        if (s.mats[m].kind == kEmission) {
            sum = sum + ray.T * s.mats[m].color;
            continue;
        }
        for (int bounce = 0; bounce < s.maxBounces; bounce++) {
            color = color + LightContribution(s, si, s1, s2, ray);
            prev = ray;
            m = si.material;
            ray = NextRay(s, m, ray, si, s2);
            if (std::abs(SqLen(ray.T) - 0.0f) < kEps) break;
            float d;
            const int t = IntersectDefault(s, ray, &d);
            if (t >= 0) {
                const Shading sn = Interpolate(s, t, ray, d);
                if (s.mats[sn.material].kind == kEmission) {
                    float pdfArea = 0.0f;
                    const float l2 = SqLen(sn.pos - ray.o);
                    const float cosP = std::abs(Dot(ray.dir, sn.normal));
                    SampleLight(s, ray.o, s1.Next(), s2, &pdfArea, nullptr);
                    const float pB = PDF(s, m, prev, ray, si);
                    const float pL = l2 / cosP * pdfArea;
                    const float mis = pB * pB / (pL * pL + pB * pB);
                    color = color + mis * ray.T * s.mats[sn.material].color;
                    break;
                }
                si = sn;
            } else {
                if (s.env.UseIS()) {
                    const float c = std::abs(Dot(si.normal, ray.dir));
                    const float sn = (float)std::sqrt((double)std::max(0.0f, 1.0f - c * c));
                    const float pB = PDF(s, m, prev, ray, si);
                    float pE = 0.0f, mis = 0.0f;
                    if (ray.dir.x != 0 && ray.dir.y != 0 && sn > 0) {
                        pE = s.env.Pdf(ray.dir) / (2.0f * kPi * kPi * sn);
                        mis = pB * pB / (pE * pE + pB * pB);
                    } else {
                        mis = 1.0f;
                    }
                    color = color + mis * ray.T * s.env.GetColor(ray.dir);
                } else {
                    color = color + ray.T * s.env.GetColor(ray.dir);
                }
                break;
            }
        }
        if (MinElem(color) >= 0.0f) sum = sum + color;
    }
    const V3 avg = sum / (float)s.spp;
    float* o = film + ((size_t)py * s.W + px) * 3;
    o[0] = avg.x; o[1] = avg.y; o[2] = avg.z;
}

// ---------------------------------------------------------------- scene parsing
struct Blob {
    const uint8_t* p;
    size_t n, off = 0;
    void take(void* dst, size_t k) {
        if (off + k > n) throw std::runtime_error("truncated scene");
        std::memcpy(dst, p + off, k);
        off += k;
    }
    template <typename T> T get() { T v; take(&v, sizeof(T)); return v; }
};

static Scene* Parse(const void* data, size_t size) {
    Blob b{(const uint8_t*)data, size};
    char magic[8];
    b.take(magic, 8);
    if (std::memcmp(magic, "PTSCENE1", 8) != 0) throw std::runtime_error("bad magic");
    auto s = std::make_unique<Scene>();
    int st[8];
    b.take(st, sizeof(st));
    s->W = st[0]; s->H = st[1]; s->spp = st[2]; s->maxBounces = st[3];
    s->tileW = st[4]; s->tileH = st[5]; s->numThreads = st[6]; s->integrator = st[7];
    float c[12];
    b.take(c, sizeof(c));
    const uint32_t hasFocus = b.get<uint32_t>();
    s->cam.pos = V3(c[0], c[1], c[2]);
    s->cam.SetViewDir(V3(c[3], c[4], c[5]));  // Camera(pos, dir) ctor, Camera.cpp:23-27
    if (c[6] > 0.0f) s->cam.hPerf = (float)(2.0f * std::tan((double)(0.5f * c[6])));  // SetFOV
    else s->cam.hPerf = s->cam.sensorH / c[7];                                      // SetFocalLength
    if (hasFocus) s->cam.focusDist = Length(V3(c[8], c[9], c[10]) - s->cam.pos);  // FocusTo
    s->cam.aperture = c[11];
    float e[4];
    b.take(e, sizeof(e));
    const int ew = b.get<int32_t>(), eh = b.get<int32_t>();
    (void)b.get<uint32_t>();
    s->env.base = V3(e[0], e[1], e[2]);
    s->env.rot = e[3];
    if (ew > 0 && eh > 0) {
        s->env.tex.W = ew;
        s->env.tex.H = eh;
        s->env.tex.valid = true;
        s->env.tex.px.resize((size_t)ew * eh);
        b.take(s->env.tex.px.data(), (size_t)ew * eh * 12);
        s->env.PreCalc();
    }
    const uint32_t M = b.get<uint32_t>();
    std::vector<float> mf((size_t)M * 8);
    std::vector<int32_t> mi((size_t)M * 4);
    b.take(mf.data(), mf.size() * 4);
    b.take(mi.data(), mi.size() * 4);
    for (uint32_t k = 0; k < M; k++) {
        Material m;
        m.kind = mi[k * 4];
        m.color = V3(mf[k * 8], mf[k * 8 + 1], mf[k * 8 + 2]);
        m.alpha = mf[k * 8 + 3] * mf[k * 8 + 3];
        m.ior = mf[k * 8 + 4];
        m.mix = mf[k * 8 + 5];
        m.mat0 = mi[k * 4 + 1];
        m.mat1 = mi[k * 4 + 2];
        const uint32_t refs = (uint32_t)mi[k * 4 + 3];  // texture index + 1 per byte
        m.albedoTex = (int)(refs & 255) - 1;
        m.f0Tex = (int)((refs >> 8) & 255) - 1;
        m.roughTex = (int)((refs >> 16) & 255) - 1;
        m.normalTex = (int)((refs >> 24) & 255) - 1;
        m.roughStrength = mf[k * 8 + 6];
        m.normalStrength = mf[k * 8 + 7];
        s->mats.push_back(m);
    }
    const uint32_t V = b.get<uint32_t>();
    s->P.resize(V); s->N.resize(V); s->UV.resize(V);
    b.take(s->P.data(), (size_t)V * 12);
    b.take(s->N.data(), (size_t)V * 12);
    b.take(s->UV.data(), (size_t)V * 12);
    const uint32_t T = b.get<uint32_t>();
    s->idx.resize((size_t)T * 3);
    s->triMat.resize(T);
    s->shade.resize(T + ((4 - T % 4) % 4));
    b.take(s->idx.data(), (size_t)T * 12);
    b.take(s->triMat.data(), (size_t)T * 4);
    b.take(s->shade.data(), s->shade.size());
    s->shade.resize(T);
    const uint32_t L = b.get<uint32_t>();
    s->lights.resize(L);
    b.take(s->lights.data(), (size_t)L * 4);
    if (b.off < b.n) {  // optional texture-map section
        const uint32_t NT = b.get<uint32_t>();
        for (uint32_t k = 0; k < NT; k++) {
            Texture t;
            t.W = b.get<int32_t>();
            t.H = b.get<int32_t>();
            t.valid = true;
            t.px.resize((size_t)t.W * t.H);
            b.take(t.px.data(), (size_t)t.W * t.H * 12);
            s->textures.push_back(std::move(t));
        }
    }
    if (b.off < b.n) {  // optional material-flag section: bit 0 = importance sampling off
        const uint32_t NM = b.get<uint32_t>();
        if (NM != s->mats.size()) throw std::runtime_error("material flag count");
        for (uint32_t k = 0; k < NM; k++) s->mats[k].uniform = (b.get<uint32_t>() & 1u) != 0;
    }
    for (const Material& m : s->mats)
        for (int r : {m.albedoTex, m.f0Tex, m.roughTex, m.normalTex})
            if (r >= (int)s->textures.size()) throw std::runtime_error("texture index out of range");
    return s.release();
}

}  // namespace orc

using namespace orc;

extern "C" {

void* oracle_scene_parse(const void* data, size_t size) {
    try {
        return Parse(data, size);
    } catch (...) {
        return nullptr;
    }
}

void oracle_scene_free(void* s) { delete (Scene*)s; }

// Binned-SAH build; returns seconds.
double oracle_bvh_build(void* sp) {
    Scene& s = *(Scene*)sp;
    const auto t0 = std::chrono::steady_clock::now();
    BuildBVH(s);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int oracle_bvh_size(void* sp, int* numNodes, int* numIDs, int* maxDepth) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    *numNodes = (int)s.nodes.size();
    *numIDs = (int)s.primIDs.size();
    *maxDepth = s.maxDepth;
    return 0;
}

// bounds: numNodes*6 floats; ints: numNodes*5 (child0, child1, begin, end, isLeaf); ids.
int oracle_bvh_dump(void* sp, float* bounds, int32_t* ints, int32_t* ids) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    for (size_t i = 0; i < s.nodes.size(); i++) {
        const BVHNode& n = s.nodes[i];
        const float b[6] = {n.lo.x, n.lo.y, n.lo.z, n.hi.x, n.hi.y, n.hi.z};
        std::memcpy(bounds + i * 6, b, 24);
        const int32_t q[5] = {n.child[0], n.child[1], n.begin, n.end, n.leaf ? 1 : 0};
        std::memcpy(ints + i * 5, q, 20);
    }
    std::memcpy(ids, s.primIDs.data(), s.primIDs.size() * 4);
    return 0;
}

// Render tiles [tileBegin, tileEnd) (tileEnd < 0: all) into film (W*H*3 floats) with
// `threads` workers (0: hardware concurrency). Seeds as in Petrichor.cpp:72-77.
// Returns render seconds (BVH built first if needed, not included), or -1 on error.
double oracle_render(void* sp, float* film, int threads, int tileBegin, int tileEnd) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    // TileManager.cpp:8-43: (nx+1)*(ny+1) tiles, zero-size edge tiles included
    const int nx = s.W / s.tileW, ny = s.H / s.tileH;
    const int remW = s.W - nx * s.tileW, remH = s.H - ny * s.tileH;
    struct Tile { int x, y, w, h; };
    std::vector<Tile> tiles;
    for (int j = 0; j < ny + 1; j++)
        for (int i = 0; i < nx + 1; i++)
            tiles.push_back({i * s.tileW, j * s.tileH, i != nx ? s.tileW : remW,
                             j != ny ? s.tileH : remH});
    if (tileEnd < 0 || tileEnd > (int)tiles.size()) tileEnd = (int)tiles.size();
    if (tileBegin < 0) tileBegin = 0;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(tileBegin);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= tileEnd) break;
            const Tile& tl = tiles[k];
            Sampler1D s1(0);      // the Rendered pass never advances tileIndex
            Sampler2D s2(0, 1);
            for (int y = tl.y; y < tl.y + tl.h; y++)
                for (int x = tl.x; x < tl.x + tl.w; x++) {
                    if (s.integrator == 0) RenderSimple(s, x, y, film, s1, s2);
                    else RenderPT(s, x, y, film, s1, s2);
                }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; i++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// AOV pass `aov` (0 UV, 1 denoising albedo, 2 denoising normal) over all tiles; the
// AOV loops of Core/Petrichor.cpp:104-261 seed tile k with RandomSampler1D(k) and
// RandomSampler2D(k, k + 1). dspp = RenderSetting::numSppForDenoising.
double oracle_render_aov(void* sp, float* film, int threads, int aov, int dspp) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    const int nx = s.W / s.tileW, ny = s.H / s.tileH;
    const int remW = s.W - nx * s.tileW, remH = s.H - ny * s.tileH;
    const int nt = (nx + 1) * (ny + 1);
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(0);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= nt) break;
            const int i = k % (nx + 1), j = k / (nx + 1);
            const int x0 = i * s.tileW, y0 = j * s.tileH;
            const int w = i != nx ? s.tileW : remW, h = j != ny ? s.tileH : remH;
            Sampler1D s1(k);
            Sampler2D s2(k, k + 1);
            for (int y = y0; y < y0 + h; y++)
                for (int x = x0; x < x0 + w; x++) {
                    if (aov == 0) RenderAovUV(s, x, y, film, s2);
                    else RenderAovDenoise(s, aov == 2, dspp, x, y, film, s1, s2);
                }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Render an explicit list of tiles (for bounded, spatially spread CPU samples).
double oracle_render_tiles(void* sp, float* film, int threads, const int32_t* list, int n) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    const int nx = s.W / s.tileW, ny = s.H / s.tileH;
    const int remW = s.W - nx * s.tileW, remH = s.H - ny * s.tileH;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(0);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n) break;
            const int t = list[k], i = t % (nx + 1), j = t / (nx + 1);
            if (j > ny) continue;
            const int x0 = i * s.tileW, y0 = j * s.tileH;
            const int w = i != nx ? s.tileW : remW, h = j != ny ? s.tileH : remH;
            Sampler1D s1(0);
            Sampler2D s2(0, 1);
            for (int y = y0; y < y0 + h; y++)
                for (int x = x0; x < x0 + w; x++) {
                    if (s.integrator == 0) RenderSimple(s, x, y, film, s1, s2);
                    else RenderPT(s, x, y, film, s1, s2);
                }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; i++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The same integrators with decorrelated generators: per tile, three XorShift128
// streams seeded from a hash of (seed, tile, stream) and advanced 64 steps, so the
// 1D stream and the two 2D streams are independent. Used to separate the
// reference's sampling correlations from the estimator itself.
static uint32_t HashU32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
double oracle_render_decorrelated(void* sp, float* film, int threads, uint32_t seed) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    const int nx = s.W / s.tileW, ny = s.H / s.tileH;
    const int remW = s.W - nx * s.tileW, remH = s.H - ny * s.tileH;
    const int n = (nx + 1) * (ny + 1);
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(0);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int t = next.fetch_add(1);
            if (t >= n) break;
            const int i = t % (nx + 1), j = t / (nx + 1);
            const int x0 = i * s.tileW, y0 = j * s.tileH;
            const int w = i != nx ? s.tileW : remW, h = j != ny ? s.tileH : remH;
            Sampler1D s1(HashU32(HashU32(seed) ^ (uint32_t)(3 * t)));
            Sampler2D s2(HashU32(HashU32(seed) ^ (uint32_t)(3 * t + 1)),
                         HashU32(HashU32(seed) ^ (uint32_t)(3 * t + 2)));
            for (int k = 0; k < 64; k++) {
                s1.Next();
                float a, b;
                s2.Next(&a, &b);
            }
            for (int y = y0; y < y0 + h; y++)
                for (int x = x0; x < x0 + w; x++) {
                    if (s.integrator == 0) RenderSimple(s, x, y, film, s1, s2);
                    else RenderPT(s, x, y, film, s1, s2);
                }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; i++) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The listed tiles only, with the decorrelated generators of
// oracle_render_decorrelated (tile t seeded as there), so replicates over a sample
// of tiles are independent of each other and of the pixels outside the sample.
double oracle_render_tiles_decorrelated(void* sp, float* film, int threads, const int32_t* list,
                                        int n, uint32_t seed) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    const int nx = s.W / s.tileW, ny = s.H / s.tileH;
    const int remW = s.W - nx * s.tileW, remH = s.H - ny * s.tileH;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(0);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n) break;
            const int t = list[k], i = t % (nx + 1), j = t / (nx + 1);
            if (j > ny) continue;
            const int x0 = i * s.tileW, y0 = j * s.tileH;
            const int w = i != nx ? s.tileW : remW, h = j != ny ? s.tileH : remH;
            Sampler1D s1(HashU32(HashU32(seed) ^ (uint32_t)(3 * t)));
            Sampler2D s2(HashU32(HashU32(seed) ^ (uint32_t)(3 * t + 1)),
                         HashU32(HashU32(seed) ^ (uint32_t)(3 * t + 2)));
            for (int m = 0; m < 64; m++) {
                s1.Next();
                float a, b;
                s2.Next(&a, &b);
            }
            for (int y = y0; y < y0 + h; y++)
                for (int x = x0; x < x0 + w; x++) {
                    if (s.integrator == 0) RenderSimple(s, x, y, film, s1, s2);
                    else RenderPT(s, x, y, film, s1, s2);
                }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; i++) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Number of tiles of the film (TileManager.cpp:8-43).
int oracle_num_tiles(void* sp) {
    Scene& s = *(Scene*)sp;
    return (s.W / s.tileW + 1) * (s.H / s.tileH + 1);
}

// Primary rays of every pixel (row-major) from one sampler (seedA, seedB) and their
// closest hits: rays W*H*8 floats (o, dir, dist or -1, throughput.x),
// hits W*H*2 ints (triangle or -1, triangle tests).
int oracle_hits(void* sp, uint32_t seedA, uint32_t seedB, float* rays, int32_t* hits) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    Sampler2D s2(seedA, seedB);
    for (int y = 0; y < s.H; y++)
        for (int x = 0; x < s.W; x++) {
            const size_t k = (size_t)y * s.W + x;
            const Ray r = s.cam.Generate(x, y, s.W, s.H, s2);
            tl_triTests = 0;
            float d = -1.0f;
            const int t = IntersectDefault(s, r, &d);
            float* q = rays + k * 8;
            q[0] = r.o.x; q[1] = r.o.y; q[2] = r.o.z;
            q[3] = r.dir.x; q[4] = r.dir.y; q[5] = r.dir.z;
            q[6] = t >= 0 ? d : -1.0f;
            q[7] = r.T.x;
            hits[k * 2] = t;
            hits[k * 2 + 1] = (int32_t)tl_triTests;
        }
    return 0;
}

// Closest hits for caller rays (o, dir per ray: 6 floats) with [distMin, distMax].
int oracle_trace(void* sp, int n, const float* rays, float distMin, float distMax, int32_t* tri,
                 float* dist) {
    Scene& s = *(Scene*)sp;
    if (!s.built) BuildBVH(s);
    for (int i = 0; i < n; i++) {
        Ray r;
        r.o = V3(rays[i * 6], rays[i * 6 + 1], rays[i * 6 + 2]);
        r.dir = V3(rays[i * 6 + 3], rays[i * 6 + 4], rays[i * 6 + 5]);
        float d = -1.0f;
        tri[i] = Intersect(s, r, distMin, distMax, &d);
        dist[i] = tri[i] >= 0 ? d : -1.0f;
    }
    return 0;
}

// Environment importance samples from RandomSampler2D(3, 4): n*8 floats
// (dir, pdf, pdf re-evaluated, color).
int oracle_env(void* sp, int n, float* out) {
    Scene& s = *(Scene*)sp;
    Sampler2D s2(3, 4);
    for (int i = 0; i < n; i++) {
        float pdf = 0.0f;
        const V3 d = s.env.Sample(s2, &pdf);
        const V3 c = s.env.GetColor(d);
        float* q = out + (size_t)i * 8;
        q[0] = d.x; q[1] = d.y; q[2] = d.z; q[3] = pdf;
        q[4] = s.env.Pdf(d);
        q[5] = c.x; q[6] = c.y; q[7] = c.z;
    }
    return 0;
}

}  // extern "C"
