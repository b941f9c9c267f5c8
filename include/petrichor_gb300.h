/*
 * petrichor_gb300.h - C ABI of the GB300 path-tracing core.
 *
 * Plain pointers, sizes and status codes; no C++ or torch types. Every call
 * returns PT_OK (0) or a negative PT_ERR_* code; pt_last_error() gives the
 * message of the last failing call on a context. A context is safe to use from
 * several host threads (calls are serialised per context).
 *
 * Reference interfaces replaced (paths relative to the Petrichor project):
 *   pt_render            Petrichor::Core::Petrichor::Render(const Scene&)
 *                        (LibPetrichor/Core/Petrichor.h:30-31, Petrichor.cpp:35-264)
 *   pt_scene_upload      what Render reads from Scene: GetGeometries/GetLights/
 *                        GetEnvironment/GetMaterial (LibPetrichor/Core/Scene.h:95-173)
 *                        plus BinnedSAHBVH::Build (Core/Accel/BinnedSAHBVH.cpp:15-225)
 *   pt_camera_init       Camera(pos, dir), SetFOV, SetFocalLength, FocusTo,
 *                        SetApeture (LibPetrichor/Core/Camera.h:19-83)
 *   pt_settings          RenderSetting (LibPetrichor/Core/RenderSetting.h:10-21)
 *   pt_trace_closest     AccelBase::Intersect(ray, scene, distMin, distMax)
 *                        (LibPetrichor/Core/Accel/AccelBase.h:36-55)
 *   pt_get_progress      Petrichor::GetNumRenderedTiles / GetNumTiles
 *                        (LibPetrichor/Core/Petrichor.h:41-51)
 *   pt_batch_render      repeated Petrichor::Render calls, one per scene and image
 *                        (LibPetrichor/Core/Petrichor.cpp:35-102): many images in shared waves
 *   pt_serve_*           no reference counterpart: a resident render service (scenes
 *                        stay in HBM; requests are batched continuously)
 *   pt_render_profile    SCOPE_LOGGER timers around the render passes
 *                        (LibPetrichor/Core/Logger.h:63-94, used at Petrichor.cpp:37,58)
 *   pt_bvh_build         BinnedSAHBVH::Build alone, on the host, returning the tree
 *                        (LibPetrichor/Core/Accel/BinnedSAHBVH.cpp:15-225)
 *   pt_bvh_build_device  the same build on the GPU (the same tree, node for node)
 *   pt_set_bvh_builder   which of the two pt_scene_upload runs
 *   pt_denoise           IntelOpenImageDenoiser::Denoise
 *                        (LibPetrichor/Core/Denoiser/IntelOpenImageDenoiser.cpp:15-101)
 */
#ifndef PETRICHOR_GB300_H_
#define PETRICHOR_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_ABI_VERSION 5

/* status codes */
#define PT_OK 0
#define PT_ERR_INVALID_ARG (-1)
#define PT_ERR_OUT_OF_MEMORY (-2)
#define PT_ERR_OVER_BUDGET (-3)
#define PT_ERR_TIMEOUT (-4)
#define PT_ERR_CUDA (-5)
#define PT_ERR_NOT_FOUND (-6)
#define PT_ERR_UNSUPPORTED (-7)
#define PT_ERR_BUSY (-8)
#define PT_ERR_CANCELLED (-9)
#define PT_ERR_NO_DEVICE (-10)
#define PT_ERR_DEVICE_FAULT (-11)

/* material kinds: MaterialTypes order (LibPetrichor/Core/Material/MaterialBase.h:15-22) */
#define PT_MAT_LAMBERT 0
#define PT_MAT_GLASS 1
#define PT_MAT_EMISSION 2
#define PT_MAT_GLOSSY 3 /* GGX */
#define PT_MAT_MIX 4

/* shading types (LibPetrichor/Core/Geometry/Triangle.h:15-19) */
#define PT_SHADING_FLAT 0
#define PT_SHADING_SMOOTH 1

/* integrators */
#define PT_INTEGRATOR_SIMPLE 0 /* SimplePathTracing: what Petrichor::Render runs */
#define PT_INTEGRATOR_PT 1     /* PathTracing: MIS next-event estimation */

/* render modes */
#define PT_MODE_REPLAY 0    /* reproduces the reference's per-tile random stream: same film bits */
#define PT_MODE_WAVEFRONT 1 /* throughput path: per-(pixel, sample) stream, same estimator */

/* environment light sampling in the PathTracing integrator's next-event step */
#define PT_ENV_SAMPLING_REFERENCE 0 /* the reference's tables (Environment.cpp:56-244) */
#define PT_ENV_SAMPLING_ALIAS 1     /* opt-in, wavefront mode: alias table over the map's
                                       texels (Math::AliasMethod); a different, unbiased
                                       estimator, so the film differs from the reference's */

typedef struct pt_context pt_context;
typedef int32_t pt_scene_id;

/* One material (Lambert(kd) / GGX(f0, roughness) / Glass(color, ior) /
 * Emission(color) / MixMaterial(mat0, mat1, mix)), with the texture maps of
 * Lambert::SetTexAlbedo and GGX::SetF0Texture / SetRoughnessMap / SetNormalMap
 * (LibPetrichor/Core/Material/Lambert.h, GGX.h). Texture references are
 * 1 + an index into pt_scene_desc.textures; 0 = none, so a zeroed struct has no maps. */
typedef struct pt_material {
  int32_t kind;
  float color[3];  /* Lambert kd, GGX reflectance ("f0" argument), Glass color, Emission radiance */
  float roughness; /* GGX */
  float ior;       /* Glass */
  float mix;       /* Mix */
  int32_t mat0;    /* Mix: index of the material picked when mix <= r */
  int32_t mat1;    /* Mix: the other one */
  int32_t tex_albedo;          /* Lambert: albedo = kd * texel */
  int32_t tex_f0;              /* GGX: reflectance = color * texel */
  int32_t tex_roughness;       /* GGX: alpha = (roughness_strength * luminance(texel))^2 */
  int32_t tex_normal;          /* GGX: tangent-space normal map */
  float roughness_strength;    /* GGX::SetRoughnessMap strength */
  float normal_strength;       /* GGX::SetNormalMap strength, clamped to [0, 1] */
  int32_t uniform_sampling;    /* Lambert: 1 = MaterialBase::EnableImportanceSampling(false),
                                  uniform hemisphere sampling; 0 = the default (cosine) */
} pt_material;

/* An RGB texture (Texture2D): height rows of width texels, sampled bilinearly
 * with wrap-around (Texture2D::GetPixelByUV). */
typedef struct pt_texture {
  int32_t width, height;
  const float* rgb; /* height * width * 3 */
} pt_texture;

/* Scene geometry, materials, lights and environment (host memory; copied). */
typedef struct pt_scene_desc {
  uint32_t num_vertices;
  const float* positions; /* num_vertices * 3 */
  const float* normals;   /* num_vertices * 3 (smooth shading) */
  const float* uvs;       /* num_vertices * 3, may be NULL */
  uint32_t num_triangles;
  const int32_t* indices;      /* num_triangles * 3 */
  const int32_t* tri_material; /* num_triangles */
  const uint8_t* tri_shading;  /* num_triangles, PT_SHADING_*; NULL = flat */
  uint32_t num_materials;
  const pt_material* materials;
  uint32_t num_lights;
  const int32_t* lights; /* triangle indices registered with Scene::AppendLight */
  float env_base_color[3];
  float env_z_rotation;
  int32_t env_width, env_height; /* 0 = no texture (base colour only) */
  const float* env_rgb;          /* env_height rows of env_width RGB texels */
  uint32_t num_textures;         /* material texture maps (pt_material.tex_*) */
  const pt_texture* textures;
} pt_scene_desc;

/* Derived camera state (the private members of Petrichor's Camera). Fill it with
 * pt_camera_init to get the reference's exact arithmetic. */
typedef struct pt_camera {
  float pos[3], right[3], up[3], forward[3];
  float h_perf;     /* sensor height / focal length */
  float focus_dist; /* FocusTo distance */
  float aperture;   /* lens diameter */
  float reserved;
} pt_camera;

typedef struct pt_settings {
  int32_t width, height;  /* RenderSetting::outputWidth/outputHeight */
  int32_t spp;            /* numSamplesPerPixel */
  int32_t max_bounces;    /* numMaxBounces */
  int32_t tile_width, tile_height;
  int32_t integrator;     /* PT_INTEGRATOR_* */
  int32_t mode;           /* PT_MODE_* */
  uint32_t seed;          /* wavefront stream seed */
  int32_t wave_paths;     /* wavefront: paths per wave (0 = automatic); the film does
                             not depend on it */
  int32_t denoising_spp;  /* numSppForDenoising: samples of the denoising AOV passes
                             (0 = the reference's default, 128) */
  int32_t env_sampling;   /* PT_ENV_SAMPLING_* (0, the reference's, when unset) */
} pt_settings;

typedef struct pt_scene_info {
  uint32_t num_triangles, num_nodes, tree_height, num_lights;
  uint64_t device_bytes;
  double build_seconds;  /* binned-SAH build, wall time */
  int32_t bvh_builder;   /* PT_BVH_BUILDER_* that built the tree */
  int32_t reserved;
} pt_scene_info;

typedef struct pt_stats {
  double last_render_ms;      /* device time of the last render (CUDA events) */
  uint64_t kernel_launches;   /* kernels launched by this context so far */
  uint64_t device_bytes_in_use;
  uint64_t memory_budget;
  uint64_t renders;
  int32_t last_device_status; /* error bits reported by kernels (0 = none) */
  int32_t reserved;
} pt_stats;

int pt_abi_version(void);
const char* pt_status_string(int status);

/* Context on one CUDA device. memory_budget_bytes = 0: no limit. */
int pt_context_create(int device, uint64_t memory_budget_bytes, pt_context** out);
int pt_context_destroy(pt_context* ctx);
const char* pt_last_error(const pt_context* ctx);

/* Camera(pos, dir); SetFOV(fov) if fov > 0 else SetFocalLength(focal_length);
 * FocusTo(*focus_target) if not NULL; SetApeture(aperture). */
int pt_camera_init(const float pos[3], const float view_dir[3], float fov, float focal_length,
                   const float* focus_target, float aperture, pt_camera* out);

/* Copies the scene to the device and builds its binned-SAH BVH (kept resident). */
int pt_scene_upload(pt_context* ctx, const pt_scene_desc* desc, pt_scene_id* out);
int pt_scene_release(pt_context* ctx, pt_scene_id scene);
int pt_scene_info_get(pt_context* ctx, pt_scene_id scene, pt_scene_info* info);

/* Renders into a host film of width*height*3 floats (row-major RGB, the layout
 * of Texture2D::GetRawDataPtr). Blocks until the film is written. */
int pt_render(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
              const pt_settings* settings, float* film_rgb);

/* AOV passes of Petrichor::Render (Core/Petrichor.cpp:104-261; Core/AOV/AOVUVCoordinate.cpp,
 * AOVDenoisingAlbedo.cpp, AOVDenoisingNormal.cpp). */
#define PT_AOV_UV 0               /* AOVUVCoordinate: mean hit uv over settings.spp samples */
#define PT_AOV_DENOISING_ALBEDO 1 /* AOVDenoisingAlbedo: settings.denoising_spp samples */
#define PT_AOV_DENOISING_NORMAL 2 /* AOVDenoisingNormal: settings.denoising_spp samples */
/* Renders one AOV pass into a host film of width*height*3 floats, bit-identical to
 * the reference's pass: the reference's per-tile random streams (tile k seeded k),
 * traversal order and arithmetic. settings.mode is ignored. Synchronous. */
int pt_render_aov(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                  const pt_settings* settings, int32_t aov, float* film_rgb);
/* Same, into a device film, enqueued on `stream` (NULL = the context's stream). */
int pt_render_aov_device(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                         const pt_settings* settings, int32_t aov, float* film_rgb_device,
                         void* stream);

/* Same, into a device film, enqueued on `stream` (cudaStream_t; NULL = the
 * context's stream). Returns once the work is enqueued. */
int pt_render_device(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                     const pt_settings* settings, float* film_rgb_device, void* stream);

/* One image of a batch: a resident scene, its camera and settings (mode must be
 * PT_MODE_WAVEFRONT) and a device film of width*height*3 floats. */
typedef struct pt_job {
  pt_scene_id scene;
  pt_camera camera;
  pt_settings settings;
  float* film_device;
} pt_job;

/* Renders n images (any sizes, scenes, spp and integrators) in shared persistent
 * waves. Each film equals what pt_render_device produces for that job alone (per
 * pixel sums in sample order, random stream keyed by (seed, pixel, sample)).
 * Enqueued on `stream` (NULL = the context's stream); it waits on the stream only
 * when a SimplePathTracing job needs its queue polled. */
int pt_batch_render(pt_context* ctx, int32_t n, const pt_job* jobs, void* stream);

/* ---- serving loop: continuous batching of render requests over resident scenes.
 * A server thread packs the pending samples of every admitted request into shared
 * waves; requests that arrive while others run are admitted as slots and memory
 * free up and join the next wave. A request's film is the same as its
 * pt_render_device film (same seed), alone or in any mix. */
#define PT_REQ_QUEUED 0
#define PT_REQ_RUNNING 1
#define PT_REQ_DONE 2
#define PT_REQ_CANCELLED 3
#define PT_REQ_FAILED 4

typedef struct pt_serve_config {
  int32_t wave_paths;     /* paths per wave (0: 64M); the server holds two waves' state */
  int32_t max_active;     /* requests admitted at once (0: 256) */
  uint64_t state_budget;  /* device bytes for per-request state: sums + film staging (0: 4 GiB) */
} pt_serve_config;

typedef struct pt_request_status {
  int32_t state;        /* PT_REQ_* */
  int32_t status;       /* PT_OK or the error of a failed request */
  double submit_s;      /* seconds since pt_serve_start */
  double admit_s;       /* admitted to a slot (-1 while queued) */
  double done_s;        /* film written (-1 until then) */
  uint32_t samples_done, samples_total;
} pt_request_status;

int pt_serve_start(pt_context* ctx, const pt_serve_config* config);
/* Queues a render (settings.mode must be PT_MODE_WAVEFRONT). The film is written
 * to job->film_device, or, when film_host is not NULL, copied to film_host
 * (width*height*3 floats; pinned memory recommended) once finished. Requests
 * whose state can never fit the state budget fail with PT_ERR_OVER_BUDGET. */
int pt_serve_submit(pt_context* ctx, const pt_job* job, float* film_host, uint64_t* request_id);
int pt_serve_poll(pt_context* ctx, uint64_t request_id, pt_request_status* out);
/* Waits until the request is done, cancelled or failed (PT_ERR_TIMEOUT after timeout_s). */
int pt_serve_wait(pt_context* ctx, uint64_t request_id, double timeout_s, pt_request_status* out);
int pt_serve_cancel(pt_context* ctx, uint64_t request_id);
/* A deadline `seconds` after the request's submission (0 clears it): a request not
 * done by then takes no further samples and, once its waves in flight retire, ends
 * PT_REQ_FAILED with status PT_ERR_TIMEOUT. Checked between waves (at least every
 * 20 ms while the server idles). PT_ERR_BUSY if the request already finished. */
int pt_serve_set_deadline(pt_context* ctx, uint64_t request_id, double seconds);
/* Forgets a finished request (its status can no longer be polled). */
int pt_serve_release(pt_context* ctx, uint64_t request_id);
/* Stops the server after the wave in flight; queued and running requests are cancelled. */
int pt_serve_stop(pt_context* ctx);

/* Closest hits for n device rays (o.xyz, dir.xyz) within [dist_min, dist_max]:
 * original triangle index (or -1) and distance (or -1). Enqueued on `stream`. */
int pt_trace_closest(pt_context* ctx, pt_scene_id scene, int32_t n, const float* rays_device,
                     float dist_min, float dist_max, int32_t* tri_device, float* dist_device,
                     void* stream);

/* The first bounce of a wavefront render, for checking it: every camera ray of the
 * render (width * height * spp of them, which must fit in one wave) and its closest
 * hit, computed as a render computes them (rasterised or traced through the BVH, as
 * pt_tuning.primary_traversal and the scene allow; exact ties settled in the
 * reference's traversal order). Written per (pixel, sample), index
 * (y * width + x) * spp + s, to device buffers: rays_device 6 floats (o.xyz, dir.xyz),
 * tri_device the original triangle index (or -1), dist_device the distance (or -1).
 * Wavefront mode only. Enqueued on `stream`.
 * No counterpart in the reference: its closest hits are what pt_trace_closest
 * returns for the same rays (AccelBase::Intersect). */
int pt_primary_hits(pt_context* ctx, pt_scene_id scene, const pt_camera* cam,
                    const pt_settings* settings, float* rays_device, int32_t* tri_device,
                    float* dist_device, void* stream);

/* Host-only binned-SAH build of the triangles (no device needed). Call with
 * NULL outputs to get *num_nodes; then with bounds (num_nodes*6 floats: lo.xyz,
 * hi.xyz), node_ints (num_nodes*5: child0, child1, begin, end, is_leaf) and
 * prim_ids (num_triangles) to fill them. threads <= 0: all host threads. */
int pt_bvh_build(const float* positions, uint32_t num_vertices, const int32_t* indices,
                 uint32_t num_triangles, int32_t threads, uint32_t* num_nodes,
                 uint32_t* tree_height, float* bounds, int32_t* node_ints, int32_t* prim_ids);

/* The same build on the context's GPU: the reference's tree node for node, including
 * the order std::sort leaves equal keys in. Outputs as pt_bvh_build, sized for
 * max(1, 2 * num_triangles) nodes; *num_nodes receives the count; stats may be NULL.
 * Synchronous; temporary device memory of about 250 bytes per triangle. */
typedef struct pt_bvh_build_stats {
  double device_ms;   /* device time, uploads to tree read back */
  int32_t levels;     /* tree levels built */
  int32_t rounds;     /* parallel partition rounds of the per-node sorts */
  int32_t heapsorts;  /* sort subranges that ran out of depth budget (heapsorted) */
  int32_t launches;   /* kernels launched */
} pt_bvh_build_stats;
int pt_bvh_build_device(pt_context* ctx, const float* positions, uint32_t num_vertices,
                        const int32_t* indices, uint32_t num_triangles, uint32_t* num_nodes,
                        uint32_t* tree_height, float* bounds, int32_t* node_ints,
                        int32_t* prim_ids, pt_bvh_build_stats* stats);

/* Builder pt_scene_upload uses: both give the same tree; the device builder is the
 * default. */
/* Denoiser in place of IntelOpenImageDenoiser::Denoise(color[, albedo, normal], isHDR):
 * Intel Open Image Denoise is not part of this library, so the images are not the
 * reference's. An edge-avoiding à-trous wavelet filter on the GPU (Dammertz et al.
 * 2010) with a per-pixel noise estimate, guided by the DenoisingAlbedo and
 * DenoisingNormal AOVs when given. Images are width x height RGB float rows; albedo
 * and normal may be NULL; hdr != 0 for unbounded radiance. out may equal color.
 * pt_denoise: host buffers, synchronous. pt_denoise_device: device buffers, enqueued
 * on `stream` (NULL: the context's stream). */
int pt_denoise(pt_context* ctx, int32_t width, int32_t height, const float* color,
               const float* albedo, const float* normal, int32_t hdr, float* out);
int pt_denoise_device(pt_context* ctx, int32_t width, int32_t height, const float* color,
                      const float* albedo, const float* normal, int32_t hdr, float* out,
                      void* stream);

#define PT_BVH_BUILDER_HOST 0
#define PT_BVH_BUILDER_DEVICE 1
int pt_set_bvh_builder(pt_context* ctx, int32_t builder);

/* Per-stage device times (CUDA events around every stage launch) and work tallies
 * of one wavefront render. With count_reference != 0 every extended ray is also
 * walked in the reference's traversal order to count its node and triangle
 * tests (the algorithmic work per ray). Synchronous. extend_rays counts every
 * path's closest-hit query, including the first-bounce ones that the raster
 * kernels settle (raster_paths of them, in raster_ms; extend_ms is the traversal
 * kernel alone). */
typedef struct pt_profile {
  double raygen_ms, extend_ms, shade_ms, shadow_ms, accumulate_ms;
  uint64_t extend_rays, shadow_rays, extend_launches, shadow_launches;
  uint64_t ref_node_tests, ref_tri_tests, ref_rays;
  double raster_ms;
  uint64_t raster_paths;
} pt_profile;
int pt_render_profile(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                      const pt_settings* settings, float* film_rgb_device, int32_t count_reference,
                      pt_profile* out);

/* Launch configuration of the wavefront path: what the batch autotuner picks. Every
 * configuration gives the same films; only speed differs. Zero fields keep the
 * defaults. No reference counterpart (the reference's only knobs are tile size and
 * thread count, RenderSetting.h:10-21). */
typedef struct pt_tuning {
  int32_t wave_paths;    /* paths per wave (0: the whole job, up to 2^27) */
  int32_t blocks_per_sm; /* stage kernel grid, blocks of 128 threads per SM (0: occupancy) */
  int32_t band_rows;     /* rows per pixel band of the path order (0: 8) */
  int32_t use_graphs;    /* 1: replay each wave's stage sequence from a captured CUDA graph */
  int32_t sort_rays;     /* 1: reorder each bounce's rays by direction and origin cell */
  int32_t tail_bounce;   /* > 0: from this bounce on, one launch finishes every path (0: off) */
  int32_t primary_traversal; /* first-bounce rays of a pinhole PathTracing job: 0 rasterised
                                when the unit has at least 16 rays per triangle, else traced;
                                1 always traced through the BVH; 2 rasterised whenever the
                                unit has at least 2 rays per triangle */
  int32_t reserved;
  double probe_ms;       /* pt_autotune: probe render time of the chosen configuration */
} pt_tuning;
/* Times candidate grids, pixel bands and graph replay on probe renders of one job
 * (its scene, camera and settings in wavefront mode, spp reduced to probe_spp; 0:
 * min(spp, 4)), then keeps the fastest for the context's later wavefront renders,
 * batches and servers. Synchronous; writes the choice to *out when not NULL. */
int pt_autotune(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                const pt_settings* settings, int32_t probe_spp, pt_tuning* out);
int pt_set_tuning(pt_context* ctx, const pt_tuning* tuning);
int pt_get_tuning(pt_context* ctx, pt_tuning* out);

/* Replay render that allocates no device memory: for callers that cannot call
 * cudaMalloc while rendering (another allocator owns the device memory, or the
 * thread must not take the driver's allocation lock). Inputs are the resident
 * scene, camera and settings (mode must be PT_MODE_REPLAY); the output is the
 * caller's device film. Scratch (traversal stacks, status word) is a fixed 4 MiB
 * __device__ array held by every GPU that loads the library: renders needing more
 * than (tiles * (BVH height + 2)) = 1048560 stack ints are rejected with
 * PT_ERR_INVALID_ARG. The first call on a device looks up the array's address;
 * make it before any stream capture. All calls share the array, so calls that
 * overlap on the GPU race. Enqueued on `stream` (NULL = the context's stream).
 * pt_get_stats after this call waits for the render and reports its status word
 * in last_device_status (0 = clean; kernel error bits otherwise) and its device
 * time in last_render_ms; pt_get_progress reports all of its tiles once it has run.
 * No counterpart in the reference. */
int pt_render_replay_noalloc(pt_context* ctx, pt_scene_id scene, const pt_camera* camera,
                             const pt_settings* settings, float* film_rgb_device, void* stream);

/* Measured L2 read bandwidth of this device, the roofline denominator of kernels
 * served from L2: a `bytes` buffer (0: 32 MiB; it must fit in L2) read `passes`
 * times per launch (0: 16) over `reps` launches (0: 10) with loads that bypass L1,
 * timed with CUDA events. *gbs = bytes read / time. Allocates and frees its buffer.
 * Synchronous. No reference counterpart (a measurement helper, like
 * pt_render_profile). */
int pt_probe_bandwidth(pt_context* ctx, uint64_t bytes, int32_t passes, int32_t reps, double* gbs);

int pt_get_stats(pt_context* ctx, pt_stats* out);
/* Tiles finished / total of the last replay render (reference tile grid). */
int pt_get_progress(pt_context* ctx, uint32_t* rendered_tiles, uint32_t* num_tiles);

#ifdef __cplusplus
}
#endif
#endif /* PETRICHOR_GB300_H_ */
