// C ABI (include/petrichor_gb300.h): contexts, resident scenes, renders.
//
// Host code, built with -ffp-contract=off: the few float quantities derived
// here (camera basis, light area sum, environment row tables) are computed with
// the reference's operation order so the replay path stays bit-exact.
#include "petrichor_gb300.h"
#include "petrichor_gb300/Petrichor.hpp"  // Math::AliasMethod

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bvh_builder.h"
#include "bvh_gpu.h"
#include "denoise.h"
#include "pt_kernels.h"
#include "pt_layout.h"
#include "context.h"
#include "scheduler.h"

using namespace ptg;

namespace ptg {

int Fail(pt_context* ctx, int code, const std::string& msg) {
    if (ctx) ctx->lastError = msg;
    return code;
}

int CudaFail(pt_context* ctx, cudaError_t e, const char* what) {
    const bool sticky = e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure ||
                        e == cudaErrorIllegalInstruction || e == cudaErrorMisalignedAddress ||
                        e == cudaErrorHardwareStackError;
    return Fail(ctx, sticky ? PT_ERR_DEVICE_FAULT : PT_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

// fn(i) for i in [0, n) on the host's cores (serially for small n); fn must be safe to
// run concurrently for different i.
template <class F>
void ParallelFor(size_t n, F&& fn) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min<size_t>(hw, n / 65536 + 1);
    if (nt <= 1) {
        for (size_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::vector<std::thread> pool;
    const size_t chunk = (n + nt - 1) / nt;
    for (size_t t = 0; t < nt; t++)
        pool.emplace_back([&, t] {
            const size_t e = std::min(n, (t + 1) * chunk);
            for (size_t i = t * chunk; i < e; i++) fn(i);
        });
    for (std::thread& th : pool) th.join();
}

int Alloc(pt_context* ctx, DeviceBuffer& b, size_t bytes) {
    if (b.bytes >= bytes && b.ptr) return PT_OK;
    if (ctx->budget && ctx->used - b.bytes + bytes > ctx->budget)
        return Fail(ctx, PT_ERR_OVER_BUDGET, "allocation of " + std::to_string(bytes) +
                                                 " bytes exceeds the memory budget");
    if (b.ptr) {
        cudaFree(b.ptr);
        ctx->used -= b.bytes;
        b.ptr = nullptr;
        b.bytes = 0;
    }
    if (bytes == 0) return PT_OK;
    const cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        return Fail(ctx, PT_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.bytes = bytes;
    ctx->used += bytes;
    return PT_OK;
}

void Free(pt_context* ctx, DeviceBuffer& b) {
    if (b.ptr) {
        cudaFree(b.ptr);
        ctx->used -= b.bytes;
    }
    b.ptr = nullptr;
    b.bytes = 0;
}

template <typename T>
int Upload(pt_context* ctx, SceneGpu& s, const std::vector<T>& host, const T** devOut) {
    DeviceBuffer b;
    const size_t bytes = std::max<size_t>(host.size() * sizeof(T), 16);
    int rc = Alloc(ctx, b, bytes);
    if (rc != PT_OK) return rc;
    s.buffers.push_back(b);
    if (!host.empty()) {
        const cudaError_t e =
          cudaMemcpyAsync(b.ptr, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return CudaFail(ctx, e, "scene upload");
    }
    *devOut = (const T*)b.ptr;
    return PT_OK;
}

inline float4 F4(float a, float b, float c, float d) {
    float4 r;
    r.x = a;
    r.y = b;
    r.z = c;
    r.w = d;
    return r;
}
inline float IntBits(int32_t v) {
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

struct HV3 {
    float x, y, z;
};
inline HV3 Sub(HV3 a, HV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HV3 Cross(HV3 a, HV3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float Dot(HV3 a, HV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float Length(HV3 a) { return (float)std::sqrt((double)Dot(a, a)); }
inline HV3 Normalized(HV3 a) {
    const float l = Length(a);
    return {a.x / l, a.y / l, a.z / l};
}
inline HV3 Load(const float* p) { return {p[0], p[1], p[2]}; }

int Validate(pt_context* ctx, const pt_scene_desc* d) {
    if (!d) return Fail(ctx, PT_ERR_INVALID_ARG, "scene description is NULL");
    if (d->num_triangles && (!d->indices || !d->tri_material || !d->positions))
        return Fail(ctx, PT_ERR_INVALID_ARG, "triangles need positions, indices and materials");
    if (d->num_triangles > (1u << 30)) return Fail(ctx, PT_ERR_INVALID_ARG, "too many triangles");
    if (d->num_materials == 0 || !d->materials)
        return Fail(ctx, PT_ERR_INVALID_ARG, "at least one material is required");
    if (d->num_materials > 65535) return Fail(ctx, PT_ERR_INVALID_ARG, "too many materials");
    for (uint32_t t = 0; t < d->num_triangles * 3; t++)
        if (d->indices[t] < 0 || (uint32_t)d->indices[t] >= d->num_vertices)
            return Fail(ctx, PT_ERR_INVALID_ARG, "triangle vertex index out of range");
    for (uint32_t t = 0; t < d->num_triangles; t++)
        if (d->tri_material[t] < 0 || (uint32_t)d->tri_material[t] >= d->num_materials)
            return Fail(ctx, PT_ERR_INVALID_ARG, "triangle material index out of range");
    for (uint32_t m = 0; m < d->num_materials; m++) {
        const pt_material& M = d->materials[m];
        if (M.kind < PT_MAT_LAMBERT || M.kind > PT_MAT_MIX)
            return Fail(ctx, PT_ERR_INVALID_ARG, "unknown material kind");
        if (M.kind == PT_MAT_MIX) {
            for (int32_t r : {M.mat0, M.mat1})
                if (r < 0 || (uint32_t)r >= d->num_materials ||
                    d->materials[r].kind == PT_MAT_MIX)
                    return Fail(ctx, PT_ERR_INVALID_ARG, "mix material must reference two non-mix materials");
        }
    }
    for (uint32_t i = 0; i < d->num_lights; i++)
        if (!d->lights || d->lights[i] < 0 || (uint32_t)d->lights[i] >= d->num_triangles)
            return Fail(ctx, PT_ERR_INVALID_ARG, "light triangle index out of range");
    if ((d->env_width > 0) != (d->env_height > 0) || d->env_width < 0 || d->env_height < 0)
        return Fail(ctx, PT_ERR_INVALID_ARG, "environment size is invalid");
    if (d->env_width > 0 && !d->env_rgb) return Fail(ctx, PT_ERR_INVALID_ARG, "environment texels missing");
    for (size_t i = 0; i < (size_t)d->num_vertices * 3 && d->num_triangles; i++)
        if (!std::isfinite(d->positions[i]))
            return Fail(ctx, PT_ERR_INVALID_ARG, "vertex positions must be finite");
    if (d->num_textures && !d->textures) return Fail(ctx, PT_ERR_INVALID_ARG, "textures missing");
    int64_t texels = 0;
    for (uint32_t t = 0; t < d->num_textures; t++) {
        const pt_texture& X = d->textures[t];
        if (X.width <= 0 || X.height <= 0 || !X.rgb)
            return Fail(ctx, PT_ERR_INVALID_ARG, "texture " + std::to_string(t) + " is empty");
        texels += (int64_t)X.width * X.height;
    }
    if (texels >= (int64_t)1 << 31) return Fail(ctx, PT_ERR_INVALID_ARG, "textures too large");
    for (uint32_t m = 0; m < d->num_materials; m++) {
        const pt_material& M = d->materials[m];
        for (int32_t r : {M.tex_albedo, M.tex_f0, M.tex_roughness, M.tex_normal})
            if (r < 0 || (uint32_t)r > d->num_textures)
                return Fail(ctx, PT_ERR_INVALID_ARG, "material texture reference out of range");
    }
    return PT_OK;
}

// Texture maps a material's kind reads (Lambert: albedo; GGX: f0, roughness, normal).
bool HasTextureMaps(const pt_material& M) {
    if (M.kind == PT_MAT_LAMBERT) return M.tex_albedo > 0;
    if (M.kind == PT_MAT_GLOSSY) return M.tex_f0 > 0 || M.tex_roughness > 0 || M.tex_normal > 0;
    return false;
}

int SetDevice(pt_context* ctx) {
    const cudaError_t e = cudaSetDevice(ctx->device);
    return e == cudaSuccess ? PT_OK : CudaFail(ctx, e, "cudaSetDevice");
}

// Paths per wave: the whole image x spp when it fits in kMaxWavePaths (236 B of
// wave state per path), otherwise as many full sample blocks as fit. HBM holds
// this easily; fewer, larger waves mean fewer sparse late-bounce launches.
int WaveCapacity(const pt_context* ctx, const pt_settings* st) {
    const int64_t px = (int64_t)st->width * st->height;
    int64_t cap = std::min<int64_t>(px * st->spp, kMaxWavePaths);
    cap = std::max<int64_t>(cap, std::min<int64_t>(px, kMaxWavePaths));
    const int64_t limit = st->wave_paths > 0 ? st->wave_paths : ctx->tunedWavePaths;
    if (limit > 0) cap = std::min<int64_t>(cap, std::max<int64_t>(limit, px));
    return (int)std::max<int64_t>(cap, 1);
}


WaveGraphCache* Graphs(pt_context* ctx) {
    if (!ctx->graphs) ctx->graphs = NewWaveGraphCache();
    return ctx->graphs;
}

int EnsureWaveBuffers(pt_context* ctx, int capacity) {
    if (ctx->wbCapacity >= capacity) return PT_OK;
    for (auto& b : ctx->wbBuffers) Free(ctx, b);
    ctx->wbBuffers.assign(1, DeviceBuffer{});
    ctx->wbCapacity = 0;
    const size_t bytes = WaveBuffersBytesTwoLanes(capacity);
    const int rc = Alloc(ctx, ctx->wbBuffers[0], bytes);
    if (rc != PT_OK) return rc;
    int* hostCount = ctx->wb.hostCount;
    ctx->wb = CarveWaveBuffers(ctx->wbBuffers[0].ptr, capacity);
    ctx->wb.hostCount = hostCount;
    ctx->wb.bytes = bytes;
    cudaMemsetAsync(ctx->wb.counts, 0, 16 * sizeof(int), ctx->stream);
    if (!ctx->wb.hostCount) {
        const cudaError_t e = cudaMallocHost(&ctx->wb.hostCount, sizeof(int) * 4);
        if (e != cudaSuccess) return CudaFail(ctx, e, "cudaMallocHost");
    }
    ctx->wbCapacity = capacity;
    return PT_OK;
}

int EnsureTables(pt_context* ctx, int nJobs, size_t accumPixels) {
    int rc;
    if ((rc = Alloc(ctx, ctx->jobTable, sizeof(DevJob) * (size_t)std::max(nJobs, 1))) != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->unitTable, 2 * sizeof(WaveUnit) * kMaxUnitsPerWave)) != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->jobList, sizeof(int) * (size_t)std::max(nJobs, 1))) != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->accum, sizeof(float4) * std::max<size_t>(accumPixels, 1))) != PT_OK) return rc;
    return PT_OK;
}

WaveTables Tables(pt_context* ctx) {
    WaveTables t;
    t.jobs = (DevJob*)ctx->jobTable.ptr;
    t.units = (WaveUnit*)ctx->unitTable.ptr;
    t.units2 = t.units + kMaxUnitsPerWave;
    t.jobList = (int*)ctx->jobList.ptr;
    t.maxUnits = kMaxUnitsPerWave;
    return t;
}

// Alias table of the optional environment sampler (PT_ENV_SAMPLING_ALIAS). Cell (ix, iy)
// of the map is the region EnvColor fills by blending texels ix..ix+1 and iy..iy+1
// (clamped at the last row and column). Its weight is the largest Rec. 709 luminance of
// those four texels times sin theta at the cell centre (the area of the cell on the
// sphere), so the table follows the radiance the cell can return. A map without
// positive luminance falls back to sin theta alone. Stored per cell as {keep threshold,
// alias index (bits), density over (u, v) = weight / mean weight, 0}. Built on the host
// with Math::AliasMethod (Vose's construction) from the texels already on the device;
// ctx->mu held.
int EnsureEnvAlias(pt_context* ctx, SceneGpu& s) {
    if (s.envAlias || !s.dev.envValid) return PT_OK;
    const int W = s.dev.envW, H = s.dev.envH;
    const size_t N = (size_t)W * H;
    std::vector<float4> tex(N);
    cudaError_t e = cudaMemcpyAsync(tex.data(), s.dev.env, N * sizeof(float4), cudaMemcpyDeviceToHost,
                                    ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "environment read-back");
    auto lum = [&](int x, int y) {
        const float4 t = tex[(size_t)y * W + x];
        const double l = 0.2126 * t.x + 0.7152 * t.y + 0.0722 * t.z;
        return std::isfinite(l) && l > 0.0 ? l : 0.0;
    };
    std::vector<double> w(N);
    double total = 0.0;
    for (int pass = 0; pass < 2 && !(total > 0.0); pass++) {
        total = 0.0;
        for (int iy = 0; iy < H; iy++) {
            const double sinT = std::sin(M_PI * (iy + 0.5) / H);
            const int iy1 = std::min(iy + 1, H - 1);
            for (int ix = 0; ix < W; ix++) {
                const int ix1 = std::min(ix + 1, W - 1);
                const double l = pass == 0 ? std::max(std::max(lum(ix, iy), lum(ix1, iy)),
                                                      std::max(lum(ix, iy1), lum(ix1, iy1)))
                                           : 1.0;
                w[(size_t)iy * W + ix] = l * sinT;
                total += l * sinT;
            }
        }
    }
    Petrichor::Math::AliasMethod am;
    am.Construct(w);
    if (!am.IsValid()) return Fail(ctx, PT_ERR_INVALID_ARG, "environment map has no sampling weight");
    std::vector<float> thr = am.GetThresholds();
    std::vector<int32_t> alias = am.GetAliases();
    // a column of zero weight never keeps itself (leftovers of rounding keep threshold 1),
    // so every drawn cell has a positive density
    const size_t heaviest = (size_t)(std::max_element(w.begin(), w.end()) - w.begin());
    for (size_t i = 0; i < N; i++)
        if (!(w[i] > 0.0) && alias[i] == (int32_t)i) {
            thr[i] = 0.0f;
            alias[i] = (int32_t)heaviest;
        }
    std::vector<float4> table(N);
    for (size_t i = 0; i < N; i++)
        table[i] = F4(thr[i], IntBits(alias[i]), (float)(w[i] / total * (double)N), 0.0f);
    const int rc = Upload(ctx, s, table, &s.envAlias);
    if (rc != PT_OK) return rc;
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "environment alias upload");
    s.info.device_bytes += s.buffers.back().bytes;
    return PT_OK;
}

int CheckArgs(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
              SceneGpu** out) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    if (!cam || !st) return Fail(ctx, PT_ERR_INVALID_ARG, "camera and settings are required");
    if (st->width <= 0 || st->height <= 0 || st->spp <= 0 || st->max_bounces < 0)
        return Fail(ctx, PT_ERR_INVALID_ARG, "width, height and spp must be positive");
    if ((int64_t)st->width * st->height > (1ll << 28))
        return Fail(ctx, PT_ERR_INVALID_ARG, "image too large");
    if (st->tile_width <= 0 || st->tile_height <= 0)
        return Fail(ctx, PT_ERR_INVALID_ARG, "tile size must be positive");
    if (st->integrator != PT_INTEGRATOR_SIMPLE && st->integrator != PT_INTEGRATOR_PT)
        return Fail(ctx, PT_ERR_INVALID_ARG, "unknown integrator");
    if (st->mode != PT_MODE_REPLAY && st->mode != PT_MODE_WAVEFRONT)
        return Fail(ctx, PT_ERR_INVALID_ARG, "unknown mode");
    if (st->wave_paths < 0) return Fail(ctx, PT_ERR_INVALID_ARG, "wave_paths must be >= 0");
    if (st->env_sampling != PT_ENV_SAMPLING_REFERENCE && st->env_sampling != PT_ENV_SAMPLING_ALIAS)
        return Fail(ctx, PT_ERR_INVALID_ARG, "unknown env_sampling");
    if (st->env_sampling == PT_ENV_SAMPLING_ALIAS && st->mode != PT_MODE_WAVEFRONT)
        return Fail(ctx, PT_ERR_INVALID_ARG, "the alias environment sampler is a wavefront-mode option");
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return Fail(ctx, PT_ERR_NOT_FOUND, "unknown scene id");
    if (st->env_sampling == PT_ENV_SAMPLING_ALIAS) {
        const int rc = EnsureEnvAlias(ctx, *it->second);
        if (rc != PT_OK) return rc;
    }
    *out = it->second.get();
    return PT_OK;
}

DevScene JobScene(const SceneGpu& s, const pt_settings* st) {
    DevScene S = s.dev;
    S.envAlias = st->env_sampling == PT_ENV_SAMPLING_ALIAS ? s.envAlias : nullptr;
    return S;
}

DevCamera ToDev(const pt_camera* c) {
    DevCamera d{};
    for (int a = 0; a < 3; a++) {
        d.pos[a] = c->pos[a];
        d.right[a] = c->right[a];
        d.up[a] = c->up[a];
        d.fwd[a] = c->forward[a];
    }
    d.hPerf = c->h_perf;
    d.focusDist = c->focus_dist;
    d.aperture = c->aperture;
    return d;
}

DevSettings ToDev(const pt_settings* s) {
    DevSettings d{};
    d.width = s->width;
    d.height = s->height;
    d.spp = s->spp;
    d.maxBounces = s->max_bounces;
    d.tileW = s->tile_width;
    d.tileH = s->tile_height;
    d.integrator = s->integrator;
    d.seed = s->seed;
    return d;
}

// Enqueue one render into a device film on `stream`.
int RenderOnStream(pt_context* ctx, SceneGpu& sg, const pt_camera* cam, const pt_settings* st,
                   float* dFilm, cudaStream_t stream) {
    const DevCamera C = ToDev(cam);
    const DevSettings S = ToDev(st);
    cudaError_t e;
    int launches = 0;
    e = cudaEventRecord(ctx->ev0, stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "cudaEventRecord");
    if (st->mode == PT_MODE_REPLAY) {
        const int tiles = NumTiles(S);
        int rc = Alloc(ctx, ctx->stack, (size_t)tiles * sg.dev.stackDepth * sizeof(int));
        if (rc != PT_OK) return rc;
        rc = Alloc(ctx, ctx->status, 16);
        if (rc != PT_OK) return rc;
        cudaMemsetAsync(ctx->status.ptr, 0, sizeof(int), stream);
        ctx->tilesTotal = tiles;
        ctx->tilesDone = 0;
        // chunks of tiles so progress can be reported between launches
        const int chunk = std::max(1, std::min(tiles, 8192));
        for (int t0 = 0; t0 < tiles; t0 += chunk) {
            const int t1 = std::min(tiles, t0 + chunk);
            e = LaunchReplay(sg.dev, C, S, dFilm, (int*)ctx->stack.ptr, (int*)ctx->status.ptr, t0, t1,
                             stream);
            launches++;
            if (e != cudaSuccess) return CudaFail(ctx, e, "replay launch");
        }
    } else {
        const int cap = WaveCapacity(ctx, st);
        int rc = EnsureWaveBuffers(ctx, cap);
        if (rc != PT_OK) return rc;
        if ((rc = EnsureTables(ctx, 1, (size_t)st->width * st->height)) != PT_OK) return rc;
        DevJob job{};
        job.S = JobScene(sg, st);
        job.C = C;
        job.st = S;
        job.accum = (float4*)ctx->accum.ptr;
        job.film = dFilm;
        e = RenderJobs({job}, Tables(ctx), ctx->wb, cap, stream, &launches, nullptr, ctx->tuning,
                       Graphs(ctx));
        if (e != cudaSuccess) return CudaFail(ctx, e, "wavefront render");
    }
    e = cudaEventRecord(ctx->ev1, stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "cudaEventRecord");
    ctx->stats.kernel_launches += launches;
    ctx->stats.renders++;
    return PT_OK;
}

int FinishStats(pt_context* ctx, cudaStream_t stream) {
    ctx->noallocPending = false;
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "render");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.last_render_ms = ms;
    int status = 0;
    if (ctx->status.ptr) cudaMemcpy(&status, ctx->status.ptr, sizeof(int), cudaMemcpyDeviceToHost);
    int wstatus = 0;
    if (ctx->wb.counts) cudaMemcpy(&wstatus, ctx->wb.counts + 3, sizeof(int), cudaMemcpyDeviceToHost);
    ctx->stats.last_device_status = status | (wstatus << 8);
    ctx->tilesDone = ctx->tilesTotal;
    return PT_OK;
}

}  // namespace ptg

extern "C" {

int pt_abi_version(void) { return PT_ABI_VERSION; }

const char* pt_status_string(int s) {
    switch (s) {
    case PT_OK: return "ok";
    case PT_ERR_INVALID_ARG: return "invalid argument";
    case PT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PT_ERR_OVER_BUDGET: return "over the memory budget";
    case PT_ERR_TIMEOUT: return "timed out";
    case PT_ERR_CUDA: return "CUDA error";
    case PT_ERR_NOT_FOUND: return "not found";
    case PT_ERR_UNSUPPORTED: return "unsupported";
    case PT_ERR_BUSY: return "busy";
    case PT_ERR_CANCELLED: return "cancelled";
    case PT_ERR_NO_DEVICE: return "no CUDA device";
    case PT_ERR_DEVICE_FAULT: return "device fault (context unusable)";
    default: return "unknown status";
    }
}

int pt_context_create(int device, uint64_t budget, pt_context** out) {
    if (!out) return PT_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return PT_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return PT_ERR_INVALID_ARG;
    auto ctx = std::make_unique<pt_context>();
    ctx->device = device;
    ctx->budget = budget;
    if (SetDevice(ctx.get()) != PT_OK) return PT_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
        return PT_ERR_CUDA;
    ctx->stats.memory_budget = budget;
    *out = ctx.release();
    return PT_OK;
}

int pt_context_destroy(pt_context* ctx) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    pt_serve_stop(ctx);  // the server thread takes ctx->mu itself
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (auto& kv : ctx->scenes)
            for (auto& b : kv.second->buffers) Free(ctx, b);
        ctx->scenes.clear();
        for (auto& b : ctx->wbBuffers) Free(ctx, b);
        if (ctx->wb.hostCount) cudaFreeHost(ctx->wb.hostCount);
        Free(ctx, ctx->film);
        Free(ctx, ctx->stack);
        Free(ctx, ctx->status);
        Free(ctx, ctx->jobTable);
        Free(ctx, ctx->unitTable);
        Free(ctx, ctx->jobList);
        Free(ctx, ctx->accum);
        Free(ctx, ctx->denoiseScratch);
        Free(ctx, ctx->denoiseImages);
        FreeWaveGraphCache(ctx->graphs);
        ctx->graphs = nullptr;
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return PT_OK;
}

const char* pt_last_error(const pt_context* ctx) { return ctx ? ctx->lastError.c_str() : ""; }

int pt_camera_init(const float pos[3], const float dir[3], float fov, float focalLength,
                   const float* focusTarget, float aperture, pt_camera* out) {
    if (!pos || !dir || !out) return PT_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    const HV3 p = Load(pos);
    // Camera::SetViewDir (Camera.cpp:38-44), world up = +Z
    const HV3 f = Normalized(Load(dir));
    const HV3 r = Cross(f, HV3{0.0f, 0.0f, 1.0f});
    const HV3 u = Cross(r, f);
    const HV3* src[4] = {&p, &r, &u, &f};
    float* dst[4] = {out->pos, out->right, out->up, out->forward};
    for (int k = 0; k < 4; k++) {
        dst[k][0] = src[k]->x;
        dst[k][1] = src[k]->y;
        dst[k][2] = src[k]->z;
    }
    const float sensor = 24e-3f;
    if (fov > 0.0f) out->h_perf = (float)(2.0f * std::tan((double)(0.5f * fov)));  // SetFOV
    else if (focalLength > 0.0f) out->h_perf = sensor / focalLength;             // SetFocalLength
    else return PT_ERR_INVALID_ARG;
    out->focus_dist = focusTarget ? Length(Sub(Load(focusTarget), p)) : 1.0f;  // FocusTo
    out->aperture = aperture;
    return PT_OK;
}

int pt_scene_upload(pt_context* ctx, const pt_scene_desc* d, pt_scene_id* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    int rc = Validate(ctx, d);
    if (rc != PT_OK) return rc;
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    auto sg = std::make_unique<SceneGpu>();
    const int T = (int)d->num_triangles;
    const auto t0 = std::chrono::steady_clock::now();
    BvhResult bvh;
    if (ctx->bvhBuilder == PT_BVH_BUILDER_DEVICE) {
        std::string why;
        const cudaError_t be = BuildBinnedSahDevice(d->positions, (int)d->num_vertices, d->indices, T,
                                                    ctx->stream, &bvh, &why, nullptr);
        if (be != cudaSuccess)
            return Fail(ctx, be == cudaErrorMemoryAllocation ? PT_ERR_OUT_OF_MEMORY : PT_ERR_CUDA, why);
    } else {
        bvh = BuildBinnedSah(d->positions, d->indices, T, 0);
    }
    const double buildSec =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // nodes
    std::vector<float4> nodes(bvh.nodes.size() * 2);
    for (size_t i = 0; i < bvh.nodes.size(); i++) {
        const BvhNodeOut& n = bvh.nodes[i];
        const int32_t a = n.leaf ? n.begin : n.child[0];
        const int32_t b = n.leaf ? (n.end - n.begin) : -1;
        nodes[2 * i] = F4(n.lo[0], n.lo[1], n.lo[2], n.hi[0]);
        nodes[2 * i + 1] = F4(n.hi[1], n.hi[2], IntBits(a), IntBits(b));
    }
    // wide collapse for the throughput traversal
    std::vector<float> wideF;
    float wideEps = 0.0f;
    if (!CollapseWide(bvh, &wideF, kWide, &wideEps))
        return Fail(ctx, PT_ERR_UNSUPPORTED, "too many triangles for the wide BVH leaf encoding");
    std::vector<float4> wide(wideF.size() / 4);
    std::memcpy(wide.data(), wideF.data(), wideF.size() * sizeof(float));
    // the binary leaf node of every primitive slot, as an offset in float4 from the wide
    // tree (stored after the binary nodes): its widened box bounds where the throughput
    // traversal counts a hit (a hit before the ray enters that box is not one)
    std::vector<int32_t> boxOf((size_t)T, 0);
    for (size_t i = 0; i < bvh.nodes.size(); i++)
        if (bvh.nodes[i].leaf)
            for (int k = bvh.nodes[i].begin; k < bvh.nodes[i].end; k++)
                boxOf[(size_t)k] = (int32_t)(2 * i) - (int32_t)nodes.size();
    // triangles in leaf order
    std::vector<float4> tris((size_t)T * 3);
    ParallelFor((size_t)T, [&](size_t kk) {
        const int k = (int)kk;
        const int t = bvh.primIds[k];
        const HV3 v0 = Load(d->positions + 3 * d->indices[3 * t]);
        const HV3 e1 = Sub(Load(d->positions + 3 * d->indices[3 * t + 1]), v0);
        const HV3 e2 = Sub(Load(d->positions + 3 * d->indices[3 * t + 2]), v0);
        tris[3 * (size_t)k] = F4(v0.x, v0.y, v0.z, e1.x);
        tris[3 * (size_t)k + 1] = F4(e1.y, e1.z, e2.x, e2.y);
        tris[3 * (size_t)k + 2] = F4(e2.z, IntBits(t), IntBits(boxOf[(size_t)k]), wideEps);
    });
    // shading records, also in leaf order: a hit's slot addresses both records
    // without a dependent read of the triangle id
    std::vector<float4> shade((size_t)T * 3);
    ParallelFor((size_t)T, [&](size_t kk) {
        const int k = (int)kk;
        const int t = bvh.primIds[k];
        HV3 n[3] = {{0, 0, 1}, {0, 0, 1}, {0, 0, 1}};
        if (d->normals)
            for (int v = 0; v < 3; v++) n[v] = Load(d->normals + 3 * d->indices[3 * t + v]);
        const int smooth = d->tri_shading ? (d->tri_shading[t] ? 1 : 0) : 0;
        shade[3 * (size_t)k] = F4(n[0].x, n[0].y, n[0].z, IntBits(d->tri_material[t]));
        shade[3 * (size_t)k + 1] = F4(n[1].x, n[1].y, n[1].z, IntBits(smooth));
        shade[3 * (size_t)k + 2] = F4(n[2].x, n[2].y, n[2].z, 0.0f);
    });
    // vertex uvs in leaf order, for the UV pass and texture maps (omitted when the
    // scene has neither)
    bool anyTex = false;
    for (uint32_t m = 0; m < d->num_materials; m++) anyTex = anyTex || HasTextureMaps(d->materials[m]);
    std::vector<float4> uvs;
    bool anyUV = false;
    if (d->uvs)
        for (size_t i = 0; i < (size_t)d->num_vertices * 3 && !anyUV; i++) anyUV = d->uvs[i] != 0.0f;
    if (anyUV || anyTex) {
        uvs.assign((size_t)std::max(T, 1) * 3, F4(0.0f, 0.0f, 0.0f, 0.0f));
        if (d->uvs)
            ParallelFor((size_t)T, [&](size_t k) {
                const int t = bvh.primIds[k];
                for (int v = 0; v < 3; v++) {
                    const float* u = d->uvs + 3 * (size_t)d->indices[3 * t + v];
                    uvs[3 * k + v] = F4(u[0], u[1], u[2], 0.0f);
                }
            });
    }
    // material texture maps: texels as {r, g, b, 0}, one texture after another
    std::vector<float4> texels(1, F4(0.0f, 0.0f, 0.0f, 0.0f));
    std::vector<int4> texInfo(std::max<uint32_t>(d->num_textures, 1), int4{0, 0, 0, 0});
    if (anyTex) {
        size_t total = 0;
        for (uint32_t t = 0; t < d->num_textures; t++) {
            const pt_texture& X = d->textures[t];
            texInfo[t] = int4{(int)total, X.width, X.height, 0};
            total += (size_t)X.width * X.height;
        }
        texels.assign(std::max<size_t>(total, 1), F4(0.0f, 0.0f, 0.0f, 0.0f));
        for (uint32_t t = 0; t < d->num_textures; t++) {
            const pt_texture& X = d->textures[t];
            float4* dst = texels.data() + texInfo[t].x;
            ParallelFor((size_t)X.width * X.height, [&](size_t i) {
                dst[i] = F4(X.rgb[3 * i], X.rgb[3 * i + 1], X.rgb[3 * i + 2], 0.0f);
            });
        }
    }
    // materials
    std::vector<DevMaterial> mats(d->num_materials);
    for (uint32_t m = 0; m < d->num_materials; m++) {
        const pt_material& M = d->materials[m];
        DevMaterial& o = mats[m];
        o.kind = M.kind;
        o.cr = M.color[0];
        o.cg = M.color[1];
        o.cb = M.color[2];
        o.alpha = M.roughness * M.roughness;  // GGX::GGX (GGX.cpp:16-20)
        o.ior = M.ior;
        o.mix = M.mix;
        o.mat01 = M.kind == PT_MAT_MIX ? (M.mat0 | (M.mat1 << 16)) : 0;
        o.ar = o.ag = o.ab = 1.0f;  // Lambert::GetAlbedo without a texture
        const bool lam = M.kind == PT_MAT_LAMBERT, ggx = M.kind == PT_MAT_GLOSSY;
        o.texAlbedo = lam ? M.tex_albedo - 1 : -1;
        o.texF0 = ggx ? M.tex_f0 - 1 : -1;
        o.texRough = ggx ? M.tex_roughness - 1 : -1;
        o.texNormal = ggx ? M.tex_normal - 1 : -1;
        o.texMask = HasTextureMaps(M) ? 1 : 0;
        o.uniform = M.uniform_sampling != 0 ? 1 : 0;
        o.roughStrength = M.roughness_strength;
        o.normalStrength = std::min(1.0f, std::max(0.0f, M.normal_strength));  // GGX::SetNormalMap
    }
    // lights and 1 / sum(1 / pdfArea_i) (PathTracing.cpp:363-383, Triangle.cpp:155-182)
    std::vector<float4> lights((size_t)std::max<uint32_t>(d->num_lights, 1) * 3);
    float sumArea = 0.0f;
    for (uint32_t i = 0; i < d->num_lights; i++) {
        const int t = d->lights[i];
        const HV3 v0 = Load(d->positions + 3 * d->indices[3 * t]);
        const HV3 e0 = Sub(Load(d->positions + 3 * d->indices[3 * t + 1]), v0);
        const HV3 e1 = Sub(Load(d->positions + 3 * d->indices[3 * t + 2]), v0);
        lights[3 * i] = F4(v0.x, v0.y, v0.z, IntBits(t));
        lights[3 * i + 1] = F4(e0.x, e0.y, e0.z, 0.0f);
        lights[3 * i + 2] = F4(e1.x, e1.y, e1.z, 0.0f);
        const float pdfAreaEach = 1.0f / (0.5f * Length(Cross(e0, e1)));
        sumArea += 1.0f / pdfAreaEach;
    }
    // environment texels (the importance-sampling row tables of
    // Environment::PreCalcCumulativeDistTex depend on H alone; the kernels evaluate them)
    const int W = d->env_width, H = d->env_height;
    std::vector<float4> env((size_t)std::max(W * H, 1));
    if (W > 0)
        ParallelFor((size_t)W * H, [&](size_t i) {
            env[i] = F4(d->env_rgb[3 * i], d->env_rgb[3 * i + 1], d->env_rgb[3 * i + 2], 0.0f);
        });
    SceneGpu& s = *sg;
    DevScene& D = s.dev;
    // binary nodes and wide tree in one allocation, the wide tree right after the nodes
    std::vector<float4> tree;
    tree.reserve(nodes.size() + wide.size());
    tree.insert(tree.end(), nodes.begin(), nodes.end());
    tree.insert(tree.end(), wide.begin(), wide.end());
    if ((rc = Upload(ctx, s, tree, &D.nodes)) != PT_OK ||
        (rc = Upload(ctx, s, tris, &D.tris)) != PT_OK ||
        (rc = Upload(ctx, s, shade, &D.shade)) != PT_OK ||
        (rc = Upload(ctx, s, mats, &D.mats)) != PT_OK ||
        (rc = Upload(ctx, s, lights, &D.lights)) != PT_OK ||
        (rc = Upload(ctx, s, env, &D.env)) != PT_OK ||
        (anyTex && (rc = Upload(ctx, s, texels, &D.texels)) != PT_OK) ||
        (anyTex && (rc = Upload(ctx, s, texInfo, &D.texInfo)) != PT_OK) ||
        ((anyUV || anyTex) && (rc = Upload(ctx, s, uvs, &D.uvs)) != PT_OK)) {
        for (auto& b : s.buffers) Free(ctx, b);
        return rc;
    }
    D.wide = D.nodes + nodes.size();
    D.numNodes = T > 0 ? (int)bvh.nodes.size() : 0;
    D.numWide = (int)(wide.size() / (kWideFloats / 4));
    D.numTris = T;
    D.numMats = (int)d->num_materials;
    D.numLights = (int)d->num_lights;
    D.numTextures = anyTex ? (int)d->num_textures : 0;
    D.envW = W;
    D.envH = H;
    D.envValid = W > 0 ? 1 : 0;
    D.stackDepth = bvh.height + 2;
    D.wideEps = wideEps;
    for (int a = 0; a < 3; a++) D.envBase[a] = d->env_base_color[a];
    D.envRot = d->env_z_rotation;
    D.lightPdfArea = 1.0f / sumArea;
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        for (auto& b : s.buffers) Free(ctx, b);
        return CudaFail(ctx, e, "scene upload");
    }
    if (bvh.height + 1 >= kWaveStackDepth) {
        for (auto& b : s.buffers) Free(ctx, b);
        return Fail(ctx, PT_ERR_UNSUPPORTED, "BVH height " + std::to_string(bvh.height) +
                                                 " exceeds the traversal stack");
    }
    s.info.num_triangles = T;
    s.info.num_nodes = (uint32_t)bvh.nodes.size();
    s.info.tree_height = bvh.height;
    s.info.num_lights = d->num_lights;
    s.info.build_seconds = buildSec;
    s.info.bvh_builder = ctx->bvhBuilder;
    for (auto& b : s.buffers) s.info.device_bytes += b.bytes;
    const int id = ctx->nextId++;
    ctx->scenes[id] = std::move(sg);
    *out = id;
    return PT_OK;
}

int pt_scene_release(pt_context* ctx, pt_scene_id id) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return Fail(ctx, PT_ERR_NOT_FOUND, "unknown scene id");
    if (it->second->refs > 0)
        return Fail(ctx, PT_ERR_BUSY, "scene is used by queued or running served requests");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& b : it->second->buffers) Free(ctx, b);
    ctx->scenes.erase(it);
    return PT_OK;
}

int pt_scene_info_get(pt_context* ctx, pt_scene_id id, pt_scene_info* info) {
    if (!ctx || !info) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return Fail(ctx, PT_ERR_NOT_FOUND, "unknown scene id");
    *info = it->second->info;
    return PT_OK;
}

int pt_render(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
              float* film) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!film) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    const size_t bytes = (size_t)st->width * st->height * 3 * sizeof(float);
    if ((rc = Alloc(ctx, ctx->film, bytes)) != PT_OK) return rc;
    if ((rc = RenderOnStream(ctx, *sg, cam, st, (float*)ctx->film.ptr, ctx->stream)) != PT_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(film, ctx->film.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "film download");
    return FinishStats(ctx, ctx->stream);
}

int pt_render_device(pt_context* ctx, pt_scene_id scene, const pt_camera* cam,
                     const pt_settings* st, float* dFilm, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!dFilm) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    return RenderOnStream(ctx, *sg, cam, st, dFilm, s);
}

// One AOV pass into a device film on `stream` (replay semantics, tile chunks).
int AovOnStream(pt_context* ctx, SceneGpu& sg, const pt_camera* cam, const pt_settings* st, int aov,
                float* dFilm, cudaStream_t stream) {
    if (aov < PT_AOV_UV || aov > PT_AOV_DENOISING_NORMAL) return Fail(ctx, PT_ERR_INVALID_ARG, "bad AOV");
    if (st->denoising_spp < 0) return Fail(ctx, PT_ERR_INVALID_ARG, "denoising_spp < 0");
    const int dspp = st->denoising_spp > 0 ? st->denoising_spp : 128;  // RenderSetting.h default
    const DevCamera C = ToDev(cam);
    const DevSettings S = ToDev(st);
    const int tiles = NumTiles(S);
    int rc = Alloc(ctx, ctx->stack, (size_t)tiles * sg.dev.stackDepth * sizeof(int));
    if (rc != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->status, 16)) != PT_OK) return rc;
    cudaError_t e = cudaEventRecord(ctx->ev0, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.ptr, 0, sizeof(int), stream);
    const int chunk = std::max(1, std::min(tiles, 8192));
    int launches = 0;
    for (int t0 = 0; t0 < tiles && e == cudaSuccess; t0 += chunk) {
        e = LaunchAov(sg.dev, C, S, aov, dspp, dFilm, (int*)ctx->stack.ptr, (int*)ctx->status.ptr, t0,
                      std::min(tiles, t0 + chunk), stream);
        launches++;
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "AOV render");
    ctx->stats.kernel_launches += launches;
    return PT_OK;
}

int pt_render_aov(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
                  int32_t aov, float* film) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!film) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    const size_t bytes = (size_t)st->width * st->height * 3 * sizeof(float);
    if ((rc = Alloc(ctx, ctx->film, bytes)) != PT_OK) return rc;
    if ((rc = AovOnStream(ctx, *sg, cam, st, aov, (float*)ctx->film.ptr, ctx->stream)) != PT_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(film, ctx->film.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return CudaFail(ctx, e, "film download");
    return FinishStats(ctx, ctx->stream);
}

int pt_render_aov_device(pt_context* ctx, pt_scene_id scene, const pt_camera* cam,
                         const pt_settings* st, int32_t aov, float* dFilm, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!dFilm) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    return AovOnStream(ctx, *sg, cam, st, aov, dFilm, stream ? (cudaStream_t)stream : ctx->stream);
}

int pt_set_tuning(pt_context* ctx, const pt_tuning* t) {
    if (!ctx || !t) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    if (t->wave_paths < 0 || t->blocks_per_sm < 0 || t->blocks_per_sm > 64 || t->band_rows < 0 ||
        t->band_rows > 4096 || (t->use_graphs != 0 && t->use_graphs != 1) ||
        (t->sort_rays != 0 && t->sort_rays != 1) || t->tail_bounce < 0 || t->tail_bounce > 64 ||
        t->primary_traversal < 0 || t->primary_traversal > 2)
        return Fail(ctx, PT_ERR_INVALID_ARG, "bad tuning");
    ctx->tunedWavePaths = t->wave_paths;
    ctx->tuning.blocksPerSm = t->blocks_per_sm;
    ctx->tuning.band = t->band_rows;
    ctx->tuning.graphs = t->use_graphs;
    ctx->tuning.sortRays = t->sort_rays;
    ctx->tuning.tailBounce = t->tail_bounce;
    ctx->tuning.primaryTraversal = t->primary_traversal;
    return PT_OK;
}

int pt_get_tuning(pt_context* ctx, pt_tuning* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    out->wave_paths = ctx->tunedWavePaths;
    out->blocks_per_sm = ctx->tuning.blocksPerSm;
    out->band_rows = ctx->tuning.band;
    out->use_graphs = ctx->tuning.graphs;
    out->sort_rays = ctx->tuning.sortRays;
    out->tail_bounce = ctx->tuning.tailBounce;
    out->primary_traversal = ctx->tuning.primaryTraversal;
    out->probe_ms = ctx->tunedProbeMs;
    return PT_OK;
}

// Coordinate descent over the launch configuration: each knob in turn takes the
// value with the shortest probe render (best of two timed runs after one warm-up,
// which also captures the graphs), the others held at their current best.
int pt_autotune(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
                int32_t probeSpp, pt_tuning* out) {
    if (!ctx || probeSpp < 0) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    pt_settings ps = *st;
    ps.mode = PT_MODE_WAVEFRONT;
    ps.spp = probeSpp > 0 ? probeSpp : std::min(st->spp, 4);
    ps.wave_paths = 0;
    const size_t bytes = (size_t)ps.width * ps.height * 3 * sizeof(float);
    if ((rc = Alloc(ctx, ctx->film, bytes)) != PT_OK) return rc;
    auto probe = [&](const WaveTuning& t, double* ms) {
        ctx->tuning = t;
        *ms = 1e300;
        for (int r = 0; r < 3; r++) {
            int k = RenderOnStream(ctx, *sg, cam, &ps, (float*)ctx->film.ptr, ctx->stream);
            if (k == PT_OK) k = FinishStats(ctx, ctx->stream);
            if (k != PT_OK) return k;
            if (r > 0) *ms = std::min(*ms, ctx->stats.last_render_ms);
        }
        return PT_OK;
    };
    WaveTuning best = ctx->tuning;
    double bestMs = 0.0;
    if ((rc = probe(best, &bestMs)) != PT_OK) return rc;
    const int grids[] = {0, 4, 12, 16, 24};
    const int bands[] = {8, 4, 16, 32};
    const int graphs[] = {1, 0};
    const int sorts[] = {0, 1};
    const int tails[] = {0, 8};
    for (int knob = 0; knob < 5; knob++) {
        const int* vals = knob == 0 ? grids : knob == 1 ? bands : knob == 2 ? graphs : knob == 3 ? sorts : tails;
        const int nv = knob == 0 ? 5 : knob == 1 ? 4 : 2;
        for (int i = 0; i < nv; i++) {
            WaveTuning t = best;
            int& field = knob == 0 ? t.blocksPerSm
                         : knob == 1 ? t.band
                         : knob == 2 ? t.graphs
                         : knob == 3 ? t.sortRays
                                     : t.tailBounce;
            if (field == vals[i]) continue;
            field = vals[i];
            double ms = 0.0;
            if ((rc = probe(t, &ms)) != PT_OK) {
                ctx->tuning = best;
                return rc;
            }
            if (ms < bestMs) {
                bestMs = ms;
                best = t;
            }
        }
    }
    ctx->tuning = best;
    ctx->tunedProbeMs = bestMs;
    if (out) {
        out->wave_paths = ctx->tunedWavePaths;
        out->blocks_per_sm = best.blocksPerSm;
        out->band_rows = best.band;
        out->use_graphs = best.graphs;
        out->sort_rays = best.sortRays;
        out->tail_bounce = best.tailBounce;
        out->primary_traversal = best.primaryTraversal;
        out->probe_ms = bestMs;
    }
    return PT_OK;
}

int pt_render_profile(pt_context* ctx, pt_scene_id scene, const pt_camera* cam,
                      const pt_settings* st, float* dFilm, int32_t countReference, pt_profile* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!dFilm) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if (st->mode != PT_MODE_WAVEFRONT)
        return Fail(ctx, PT_ERR_UNSUPPORTED, "profiling covers the wavefront mode");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    const int cap = WaveCapacity(ctx, st);
    if ((rc = EnsureWaveBuffers(ctx, cap)) != PT_OK) return rc;
    if ((rc = EnsureTables(ctx, 1, (size_t)st->width * st->height)) != PT_OK) return rc;
    DeviceBuffer counters;
    if ((rc = Alloc(ctx, counters, 8 * sizeof(unsigned long long))) != PT_OK) return rc;
    cudaMemsetAsync(counters.ptr, 0, 8 * sizeof(unsigned long long), ctx->stream);
    WaveProfile prof;
    prof.countReference = countReference != 0;
    prof.devCounters = (unsigned long long*)counters.ptr;
    int launches = 0;
    DevJob job{};
    job.S = JobScene(*sg, st);
    job.C = ToDev(cam);
    job.st = ToDev(st);
    job.accum = (float4*)ctx->accum.ptr;
    job.film = dFilm;
    cudaError_t e =
      RenderJobs({job}, Tables(ctx), ctx->wb, cap, ctx->stream, &launches, &prof, ctx->tuning, nullptr);
    if (e == cudaSuccess) e = CollectProfile(&prof, ctx->stream);
    Free(ctx, counters);
    if (e != cudaSuccess) return CudaFail(ctx, e, "profiled render");
    ctx->stats.kernel_launches += launches;
    std::memset(out, 0, sizeof(*out));
    out->raygen_ms = prof.ms[0];
    out->extend_ms = prof.ms[1];
    out->shade_ms = prof.ms[2];
    out->shadow_ms = prof.ms[3];
    out->accumulate_ms = prof.ms[4];
    out->extend_rays = prof.extendRays;
    out->shadow_rays = prof.shadowRays;
    out->extend_launches = prof.extendLaunches;
    out->shadow_launches = prof.shadowLaunches;
    out->ref_node_tests = prof.refNodeTests;
    out->ref_tri_tests = prof.refTriTests;
    out->ref_rays = prof.refRays;
    out->raster_ms = prof.ms[5];
    out->raster_paths = prof.rasterPaths;
    return PT_OK;
}

int pt_batch_render(pt_context* ctx, int32_t n, const pt_job* jobs, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    if (n <= 0 || n > kMaxJobsPerCall || !jobs)
        return Fail(ctx, PT_ERR_INVALID_ARG, "batch size must be 1.." + std::to_string(kMaxJobsPerCall));
    std::vector<DevJob> dj(n);
    size_t pixels = 0;
    int64_t paths = 0;
    int maxPx = 0;
    for (int i = 0; i < n; i++) {
        SceneGpu* sg = nullptr;
        int rc = CheckArgs(ctx, jobs[i].scene, &jobs[i].camera, &jobs[i].settings, &sg);
        if (rc != PT_OK) return rc;
        if (jobs[i].settings.mode != PT_MODE_WAVEFRONT)
            return Fail(ctx, PT_ERR_INVALID_ARG, "batched renders use the wavefront mode");
        if (!jobs[i].film_device) return Fail(ctx, PT_ERR_INVALID_ARG, "job film is NULL");
        dj[i].S = JobScene(*sg, &jobs[i].settings);
        dj[i].C = ToDev(&jobs[i].camera);
        dj[i].st = ToDev(&jobs[i].settings);
        dj[i].film = jobs[i].film_device;
        const int P = jobs[i].settings.width * jobs[i].settings.height;
        pixels += P;
        paths += (int64_t)P * jobs[i].settings.spp;
        maxPx = std::max(maxPx, P);
    }
    int rc = SetDevice(ctx);
    if (rc != PT_OK) return rc;
    const int cap = (int)std::max<int64_t>(std::min<int64_t>(paths, kMaxWavePaths), maxPx);
    if ((rc = EnsureWaveBuffers(ctx, cap)) != PT_OK) return rc;
    if ((rc = EnsureTables(ctx, n, pixels)) != PT_OK) return rc;
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        dj[i].accum = (float4*)ctx->accum.ptr + off;
        off += (size_t)dj[i].st.width * dj[i].st.height;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    int launches = 0;
    cudaError_t e = cudaEventRecord(ctx->ev0, s);
    if (e == cudaSuccess)
        e = RenderJobs(dj, Tables(ctx), ctx->wb, cap, s, &launches, nullptr, ctx->tuning, Graphs(ctx));
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, s);
    if (e != cudaSuccess) return CudaFail(ctx, e, "batched render");
    ctx->stats.kernel_launches += launches;
    ctx->stats.renders += n;
    return PT_OK;
}

int pt_render_replay_noalloc(pt_context* ctx, pt_scene_id scene, const pt_camera* cam,
                             const pt_settings* st, float* dFilm, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!dFilm) return Fail(ctx, PT_ERR_INVALID_ARG, "film is NULL");
    if (st->mode != PT_MODE_REPLAY)
        return Fail(ctx, PT_ERR_INVALID_ARG, "the no-allocation render runs the replay mode only");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    const DevSettings S = ToDev(st);
    const int tiles = NumTiles(S);
    const size_t need = (size_t)tiles * sg->dev.stackDepth;
    if (need > NoAllocScratchInts())
        return Fail(ctx, PT_ERR_INVALID_ARG,
                    "render needs " + std::to_string(need) + " stack ints of scratch; the fixed "
                    "no-allocation array holds " + std::to_string(NoAllocScratchInts()));
    int *status = nullptr, *stacks = nullptr;
    cudaError_t e = NoAllocScratch(&status, &stacks);
    if (e != cudaSuccess) return CudaFail(ctx, e, "no-allocation scratch lookup");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    ctx->noallocPending = false;
    e = cudaEventRecord(ctx->ev0, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), s);  // status starts at zero
    if (e != cudaSuccess) return CudaFail(ctx, e, "status clear");
    ctx->tilesTotal = (uint32_t)tiles;
    ctx->tilesDone = 0;
    e = LaunchReplay(sg->dev, ToDev(cam), S, dFilm, stacks, status, 0, tiles, s);
    if (e != cudaSuccess) return CudaFail(ctx, e, "replay launch");
    // pt_get_stats waits for this event, then reads the status word and the time
    e = cudaEventRecord(ctx->ev1, s);
    if (e != cudaSuccess) return CudaFail(ctx, e, "cudaEventRecord");
    ctx->noallocStatus = status;
    ctx->noallocPending = true;
    ctx->stats.kernel_launches++;
    ctx->stats.renders++;
    return PT_OK;
}

int pt_trace_closest(pt_context* ctx, pt_scene_id scene, int32_t n, const float* rays,
                     float distMin, float distMax, int32_t* tri, float* dist, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return Fail(ctx, PT_ERR_NOT_FOUND, "unknown scene id");
    if (n < 0 || (n > 0 && (!rays || !tri || !dist)))
        return Fail(ctx, PT_ERR_INVALID_ARG, "bad ray buffers");
    int rc = SetDevice(ctx);
    if (rc != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->status, 16)) != PT_OK) return rc;
    const cudaError_t e = LaunchTraceClosest(it->second->dev, n, rays, distMin, distMax, tri, dist,
                                             (int*)ctx->status.ptr + 1,
                                             stream ? (cudaStream_t)stream : ctx->stream);
    ctx->stats.kernel_launches++;
    return e == cudaSuccess ? PT_OK : CudaFail(ctx, e, "trace");
}

int pt_primary_hits(pt_context* ctx, pt_scene_id scene, const pt_camera* cam, const pt_settings* st,
                    float* rays, int32_t* tri, float* dist, void* stream) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    SceneGpu* sg = nullptr;
    int rc = CheckArgs(ctx, scene, cam, st, &sg);
    if (rc != PT_OK) return rc;
    if (!rays || !tri || !dist) return Fail(ctx, PT_ERR_INVALID_ARG, "output buffer is NULL");
    if (st->mode != PT_MODE_WAVEFRONT)
        return Fail(ctx, PT_ERR_UNSUPPORTED, "primary hits are those of the wavefront mode");
    const int cap = WaveCapacity(ctx, st);
    if ((int64_t)st->width * st->height * st->spp > cap)
        return Fail(ctx, PT_ERR_INVALID_ARG, "the camera rays do not fit in one wave");
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    if ((rc = EnsureWaveBuffers(ctx, cap)) != PT_OK) return rc;
    if ((rc = EnsureTables(ctx, 1, (size_t)st->width * st->height)) != PT_OK) return rc;
    std::vector<DevJob> jobs(1);
    jobs[0].S = JobScene(*sg, st);
    jobs[0].C = ToDev(cam);
    jobs[0].st = ToDev(st);
    jobs[0].accum = (float4*)ctx->accum.ptr;
    std::vector<WaveUnit> units(1);
    units[0] = WaveUnit{0, 0, st->spp, 0, 0, -1, {0, 0}};
    const WaveShape shape = ShapeOf(jobs, units, ctx->tuning.primaryTraversal);
    const WaveTables T = Tables(ctx);
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    int launches = 0;
    cudaError_t e = cudaMemcpyAsync(T.jobs, jobs.data(), sizeof(DevJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(T.units, units.data(), sizeof(WaveUnit), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = RunPrimaryHits(T.jobs, T.units, shape, ctx->wb, ctx->tuning, st->spp, rays, tri, dist, s,
                           &launches);
    ctx->stats.kernel_launches += launches;
    return e == cudaSuccess ? PT_OK : CudaFail(ctx, e, "primary hits");
}

int pt_bvh_build(const float* positions, uint32_t numVertices, const int32_t* indices,
                 uint32_t numTriangles, int32_t threads, uint32_t* numNodes, uint32_t* height,
                 float* bounds, int32_t* nodeInts, int32_t* primIds) {
    if (!numNodes || (numTriangles && (!positions || !indices))) return PT_ERR_INVALID_ARG;
    for (uint32_t t = 0; t < numTriangles * 3; t++)
        if (indices[t] < 0 || (uint32_t)indices[t] >= numVertices) return PT_ERR_INVALID_ARG;
    const BvhResult r = BuildBinnedSah(positions, indices, (int)numTriangles, threads);
    *numNodes = (uint32_t)r.nodes.size();
    if (height) *height = (uint32_t)r.height;
    if (bounds && nodeInts) {
        for (size_t i = 0; i < r.nodes.size(); i++) {
            const BvhNodeOut& n = r.nodes[i];
            for (int a = 0; a < 3; a++) {
                bounds[6 * i + a] = n.lo[a];
                bounds[6 * i + 3 + a] = n.hi[a];
            }
            nodeInts[5 * i] = n.child[0];
            nodeInts[5 * i + 1] = n.child[1];
            nodeInts[5 * i + 2] = n.begin;
            nodeInts[5 * i + 3] = n.end;
            nodeInts[5 * i + 4] = n.leaf ? 1 : 0;
        }
    }
    if (primIds) std::memcpy(primIds, r.primIds.data(), r.primIds.size() * sizeof(int32_t));
    return PT_OK;
}

int pt_bvh_build_device(pt_context* ctx, const float* positions, uint32_t numVertices,
                        const int32_t* indices, uint32_t numTriangles, uint32_t* numNodes,
                        uint32_t* height, float* bounds, int32_t* nodeInts, int32_t* primIds,
                        pt_bvh_build_stats* stats) {
    if (!ctx || !numNodes || (numTriangles && (!positions || !indices))) return PT_ERR_INVALID_ARG;
    if (numTriangles > (1u << 30)) return Fail(ctx, PT_ERR_INVALID_ARG, "too many triangles");
    for (uint32_t t = 0; t < numTriangles * 3; t++)
        if (indices[t] < 0 || (uint32_t)indices[t] >= numVertices)
            return Fail(ctx, PT_ERR_INVALID_ARG, "triangle vertex index out of range");
    for (size_t i = 0; i < (size_t)numVertices * 3; i++)
        if (!std::isfinite(positions[i])) return Fail(ctx, PT_ERR_INVALID_ARG, "vertex positions must be finite");
    std::lock_guard<std::mutex> g(ctx->mu);
    int rc = SetDevice(ctx);
    if (rc != PT_OK) return rc;
    BvhResult r;
    std::string why;
    DeviceBuildStats st;
    const cudaError_t e = BuildBinnedSahDevice(positions, (int)numVertices, indices, (int)numTriangles,
                                               ctx->stream, &r, &why, &st);
    if (e != cudaSuccess)
        return Fail(ctx, e == cudaErrorMemoryAllocation ? PT_ERR_OUT_OF_MEMORY : PT_ERR_CUDA, why);
    *numNodes = (uint32_t)r.nodes.size();
    if (height) *height = (uint32_t)r.height;
    if (stats) {
        stats->device_ms = st.ms;
        stats->levels = st.levels;
        stats->rounds = st.rounds;
        stats->heapsorts = st.heapsorts;
        stats->launches = st.launches;
    }
    if (bounds && nodeInts) {
        for (size_t i = 0; i < r.nodes.size(); i++) {
            const BvhNodeOut& n = r.nodes[i];
            for (int a = 0; a < 3; a++) {
                bounds[6 * i + a] = n.lo[a];
                bounds[6 * i + 3 + a] = n.hi[a];
            }
            nodeInts[5 * i] = n.child[0];
            nodeInts[5 * i + 1] = n.child[1];
            nodeInts[5 * i + 2] = n.begin;
            nodeInts[5 * i + 3] = n.end;
            nodeInts[5 * i + 4] = n.leaf ? 1 : 0;
        }
    }
    if (primIds && !r.primIds.empty()) std::memcpy(primIds, r.primIds.data(), r.primIds.size() * sizeof(int32_t));
    return PT_OK;
}

namespace {
int DenoiseArgs(pt_context* ctx, int32_t width, int32_t height, const float* color, const float* out) {
    if (!ctx || !color || !out) return PT_ERR_INVALID_ARG;
    if (width <= 0 || height <= 0 || (int64_t)width * height > (int64_t)1 << 28)
        return Fail(ctx, PT_ERR_INVALID_ARG, "image size is invalid");
    return PT_OK;
}
}  // namespace

int pt_denoise_device(pt_context* ctx, int32_t width, int32_t height, const float* color,
                      const float* albedo, const float* normal, int32_t hdr, float* out,
                      void* stream) {
    int rc = DenoiseArgs(ctx, width, height, color, out);
    if (rc != PT_OK) return rc;
    std::lock_guard<std::mutex> g(ctx->mu);
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    if ((rc = Alloc(ctx, ctx->denoiseScratch, DenoiseScratchBytes(width, height))) != PT_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    int launches = 0;
    const cudaError_t e = Denoise(width, height, color, albedo, normal, hdr, out,
                                  ctx->denoiseScratch.ptr, s, &launches);
    ctx->stats.kernel_launches += launches;
    return e == cudaSuccess ? PT_OK : CudaFail(ctx, e, "denoise");
}

int pt_denoise(pt_context* ctx, int32_t width, int32_t height, const float* color,
               const float* albedo, const float* normal, int32_t hdr, float* out) {
    int rc = DenoiseArgs(ctx, width, height, color, out);
    if (rc != PT_OK) return rc;
    std::lock_guard<std::mutex> g(ctx->mu);
    if ((rc = SetDevice(ctx)) != PT_OK) return rc;
    const size_t img = (size_t)width * height * 3 * sizeof(float);
    if ((rc = Alloc(ctx, ctx->denoiseScratch, DenoiseScratchBytes(width, height))) != PT_OK ||
        (rc = Alloc(ctx, ctx->denoiseImages, 4 * img)) != PT_OK)
        return rc;
    float* d = static_cast<float*>(ctx->denoiseImages.ptr);
    float *dc = d, *da = d + img / 4, *dn = d + img / 2, *dout = d + 3 * img / 4;
    cudaStream_t s = ctx->stream;
    cudaMemcpyAsync(dc, color, img, cudaMemcpyHostToDevice, s);
    if (albedo) cudaMemcpyAsync(da, albedo, img, cudaMemcpyHostToDevice, s);
    if (normal) cudaMemcpyAsync(dn, normal, img, cudaMemcpyHostToDevice, s);
    int launches = 0;
    cudaError_t e = Denoise(width, height, dc, albedo ? da : nullptr, normal ? dn : nullptr, hdr, dout,
                            ctx->denoiseScratch.ptr, s, &launches);
    ctx->stats.kernel_launches += launches;
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, img, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? PT_OK : CudaFail(ctx, e, "denoise");
}

int pt_set_bvh_builder(pt_context* ctx, int32_t builder) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    if (builder != PT_BVH_BUILDER_HOST && builder != PT_BVH_BUILDER_DEVICE)
        return Fail(ctx, PT_ERR_INVALID_ARG, "unknown BVH builder");
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->bvhBuilder = builder;
    return PT_OK;
}

int pt_probe_bandwidth(pt_context* ctx, uint64_t bytes, int32_t passes, int32_t reps, double* gbs) {
    if (!ctx || !gbs || passes < 0 || reps < 0) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    if (bytes == 0) bytes = uint64_t(32) << 20;
    if (passes == 0) passes = 16;
    if (reps == 0) reps = 10;
    bytes &= ~uint64_t(15);
    if (bytes == 0) return Fail(ctx, PT_ERR_INVALID_ARG, "probe buffer under 16 bytes");
    int rc = SetDevice(ctx);
    if (rc != PT_OK) return rc;
    DeviceBuffer buf, sink;
    if ((rc = Alloc(ctx, buf, bytes)) != PT_OK) return rc;
    if ((rc = Alloc(ctx, sink, 16)) != PT_OK) {
        Free(ctx, buf);
        return rc;
    }
    cudaError_t e = cudaMemsetAsync(buf.ptr, 0, bytes, ctx->stream);
    float ms = 0.0f;
    if (e == cudaSuccess)
        e = ProbeL2Read(buf.ptr, bytes, passes, reps, (float*)sink.ptr, ctx->stream, &ms);
    ctx->stats.kernel_launches += reps + 1;
    Free(ctx, buf);
    Free(ctx, sink);
    if (e != cudaSuccess) return CudaFail(ctx, e, "bandwidth probe");
    *gbs = (double)bytes * passes * reps / (ms / 1e3) / 1e9;
    return PT_OK;
}

int pt_get_stats(pt_context* ctx, pt_stats* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(ctx->mu);
    if (ctx->noallocPending) {
        // the last render was a no-allocation one: wait for it, then read its status
        // word from the fixed array (a 4-byte copy into host memory; nothing allocated)
        int rc = SetDevice(ctx);
        if (rc != PT_OK) return rc;
        cudaError_t e = cudaEventSynchronize(ctx->ev1);
        int status = 0;
        if (e == cudaSuccess)
            e = cudaMemcpy(&status, ctx->noallocStatus, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return CudaFail(ctx, e, "no-allocation render status");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->stats.last_render_ms = ms;
        ctx->stats.last_device_status = status;
        ctx->tilesDone = ctx->tilesTotal;
        ctx->noallocPending = false;
    }
    ctx->stats.device_bytes_in_use = ctx->used;
    *out = ctx->stats;
    return PT_OK;
}

int pt_get_progress(pt_context* ctx, uint32_t* done, uint32_t* total) {
    if (!ctx || !done || !total) return PT_ERR_INVALID_ARG;
    // a no-allocation render is one launch: all of its tiles are done once it has run
    if (ctx->noallocPending && cudaEventQuery(ctx->ev1) == cudaSuccess) {
        *done = *total = ctx->tilesTotal;
        return PT_OK;
    }
    *done = ctx->tilesDone;
    *total = ctx->tilesTotal;
    return PT_OK;
}

}  // extern "C"
