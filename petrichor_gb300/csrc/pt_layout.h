// Device-resident scene layout shared by the host uploader and the CUDA kernels.
//
// HBM layout (all arrays 16-byte aligned, read with float4 loads):
//   nodes      2 x float4 per BVH node (32 B):
//                [0] lo.x lo.y lo.z hi.x   [1] hi.y hi.z a b
//              inner: a = left child (right = left + 1), b = -1
//              leaf : a = first primitive slot, b = primitive count
//              Node order and leaf ranges are the reference binned-SAH tree's
//              (Core/Accel/BinnedSAHBVH.cpp:15-225), so slot k of a leaf is
//              m_primitiveIDs[k].
//   wide       kWide-wide nodes of the binary tree collapsed for the throughput
//              traversal, kWideFloats floats each (4-wide: 128 B, one L2 line):
//                lo.x lo.y lo.z hi.x hi.y hi.z of the children (kWide floats each, SoA),
//                then the child codes: >= 0 wide node; < 0 leaf, -(first*64+count)-1;
//                INT_MIN empty slot (whose box lies at +infinity on every plane, so the
//                slab test never hits it); padding to whole 128-byte lines
//   tris       3 x float4 per primitive slot (48 B), in leaf order:
//                [0] v0.xyz e1.x  [1] e1.yz e2.xy  [2] e2.z  triId(bits) box(bits) eps
//              box: where the slot's binary leaf node is, in float4 from `wide` (the
//              binary nodes are stored right before the wide tree, in one allocation);
//              eps: the widening of the wide tree's child boxes (a leaf's child box is
//              that node's box moved out by eps on every side)
//              e1 = v1 - v0, e2 = v2 - v0 exactly as Triangle::Intersect forms
//              them (Core/Geometry/Triangle.cpp:53-54).
//   shade      3 x float4 per primitive slot (48 B), in leaf order like tris:
//                [0] n0.xyz material(bits) [1] n1.xyz smooth(bits) [2] n2.xyz 0
//   uvs        3 x float4 per primitive slot (optional, for the UV pass): vertex uv0, uv1,
//              uv2 (xyz; the reference's uv is a Vector3f)
//   lights     3 x float4 per light: [0] v0.xyz tri(bits) [1] e0.xyz 0 [2] e1.xyz 0
//   env        float4 RGB_ texels, row-major (H x W). The importance-sampling row
//              tables are a function of H alone and are evaluated in the kernels.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define PT_HD __host__ __device__ __forceinline__
#else
#define PT_HD inline
#include <vector_types.h>
#endif

namespace ptg {

// Width of the throughput traversal's BVH nodes (4 or 8).
#ifndef PT_WIDE
#define PT_WIDE 4
#endif
constexpr int kWide = PT_WIDE;
constexpr int kWideFloats = ((7 * kWide + 31) / 32) * 32;

enum MaterialKind : int32_t {
    kLambert = 0,
    kGlass = 1,
    kEmission = 2,
    kGlossy = 3,
    kMix = 4,
};

struct __align__(16) DevMaterial {  // 80 B: whole-struct copies take 16-byte loads
    int32_t kind;
    float cr, cg, cb;  // Lambert kd / GGX reflectance strength / Glass color / Emission radiance
    float alpha;       // GGX roughness^2 (GGX.cpp:16-20)
    float ior;         // Glass
    float mix;         // Mix: mix <= r picks mat0 (MixMaterial.h:45-50)
    int32_t mat01;     // Mix: mat0 | (mat1 << 16)
    float ar, ag, ab;  // Lambert::GetAlbedo: 1 untextured; per shading point kd * texel
    int32_t texMask;   // 0: no texture maps (then the texture fields are unused)
    int32_t texAlbedo, texF0, texRough, texNormal;  // texture index or -1
    float roughStrength, normalStrength;             // GGX map strengths (normal clamped to [0, 1])
    int32_t uniform;   // Lambert: importance sampling off (uniform hemisphere, Lambert.cpp:85-107)
    int32_t pad;
};

struct DevCamera {  // derived Camera state (Core/Camera.h:121-130)
    float pos[3], right[3], up[3], fwd[3];
    float hPerf, focusDist, aperture, pad;
};

struct DevScene {
    const float4* nodes;
    const float4* wide;  // 4-wide collapse of the same tree (throughput traversal)
    const float4* tris;
    const float4* shade;
    const float4* uvs;  // nullptr: all vertex uvs are zero
    const DevMaterial* mats;
    const float4* lights;
    const float4* env;
    const float4* texels;  // material texture maps, RGB_ rows, one after another
    const int4* texInfo;   // per texture: first texel, width, height, 0
    // optional environment importance sampling (throughput path): per env texel
    // {keep threshold, alias index (bits), pdf over (u, v), 0}; nullptr: the reference's
    // sampler
    const float4* envAlias;
    int32_t numNodes, numTris, numMats, numLights;
    int32_t envW, envH, envValid, stackDepth;  // stackDepth: max traversal stack entries
    float envBase[3], envRot;
    float lightPdfArea;  // 1 / sum(1/pdfArea_i), PathTracing.cpp:363-383 (summed in light order)
    int32_t numWide;
    int32_t numTextures;
    // the widening of the wide tree's child boxes (2^-18 of the largest coordinate): a
    // leaf's child box is its binary node's box moved out by this on every side
    float wideEps;
};

// Integrators
enum Integrator : int32_t { kSimplePathTracing = 0, kPathTracing = 1 };

struct DevSettings {
    int32_t width, height, spp, maxBounces;
    int32_t tileW, tileH, integrator;
    uint32_t seed;
};

}  // namespace ptg
