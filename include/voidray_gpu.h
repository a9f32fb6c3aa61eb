/*
 * voidray_gpu.h — C ABI of the GB300 (sm_103a) path-tracing backend.
 *
 * The library replaces voidray's CPU integrator: the progressive sample loop
 * `iterative_render` (voidray_renderer/src/render/iterative.rs:11-55), the
 * recursive estimator `trace_ray` (voidray_renderer/src/core/tracer.rs:9-56)
 * and the intersection query `SceneAcceleration::hit`
 * (voidray_renderer/src/core/scene.rs:182-185), plus the colour-management
 * arithmetic of post_process.glsl / tonemapping.glsl
 * (voidray_renderer/src/shaders/post_process.glsl:23-49,
 *  voidray_renderer/src/shaders/tonemapping.glsl:2-40).
 *
 * Conventions
 *  - Every entry point returns a vr_status; VR_OK is 0.  On failure the
 *    thread-local message is available from vr_last_error().  Nothing aborts
 *    the process (the reference panics / unwraps instead,
 *    voidray_renderer/src/render/renderer.rs:104,204).
 *  - Plain pointers and sizes only.  "host" arguments are CPU memory owned by
 *    the caller; "_device" variants take CUDA device pointers and an optional
 *    CUDA stream passed as void* (NULL = the library's per-handle stream).
 *  - A vr_scene owns its device memory (BVH, triangles, shading data,
 *    environment, importance-sampling tables).  Calls on different scenes
 *    may come from different threads; calls on one scene must be serialised
 *    by the caller, as the reference serialises them on its render thread
 *    (voidray_renderer/src/render/renderer.rs:47).
 *  - There is no CPU fallback: without a usable CUDA device every compute
 *    entry point returns VR_ERR_NO_DEVICE.
 */
#ifndef VOIDRAY_GPU_H
#define VOIDRAY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VR_ABI_VERSION 4

typedef enum vr_status {
    VR_OK = 0,
    VR_ERR_INVALID = 1,     /* bad argument / descriptor                          */
    VR_ERR_UNSUPPORTED = 2, /* feature the GPU path does not cover               */
    VR_ERR_CUDA = 3,        /* CUDA runtime error                                */
    VR_ERR_OOM = 4,         /* device allocation failed                          */
    VR_ERR_STACK = 5,       /* traversal stack overflow detected by a kernel     */
    VR_ERR_TIMEOUT = 6,     /* a bounded device wait or budget ran out           */
    VR_ERR_NO_DEVICE = 7,   /* no CUDA device                                    */
    VR_ERR_CANCELLED = 8    /* job cancelled                                     */
} vr_status;

/* ---------------------------------------------------------------- scene -- */

/* Material kinds: the closed set of voidray_common materials.
 * voidray_common/src/simple.rs:15-58 (Materials::*), :60-81 (LambertianBSDF),
 * voidray_common/src/microfacet.rs:9-101 (MicrofacetBSDF). */
typedef enum vr_material_kind {
    VR_MAT_LAMBERTIAN = 0,      /* Materials::lambertian(albedo)                */
    VR_MAT_METAL = 1,           /* Materials::metal(albedo, fuzz)               */
    VR_MAT_DIELECTRIC = 2,      /* Materials::dielectric(ir)                    */
    VR_MAT_EMISSION = 3,        /* Materials::{emissive,colored_emissive}; color
                                   already multiplied by strength               */
    VR_MAT_LAMBERTIAN_BSDF = 4, /* Materials::lambertian_bsdf(albedo)           */
    VR_MAT_MICROFACET = 5,      /* MicrofacetBSDF {color,index,roughness,
                                   metallic,emittance,transparent}              */
    VR_MAT_MIX = 6              /* MixMaterial {first, second, factor} of the
                                   legacy crate (voidray/src/common/materials.rs:
                                   188-203): one uniform draw u per hit; u >=
                                   factor shades with `mix_first`, else with
                                   `mix_second`.  Children may be mixes, at most
                                   VR_MAX_MIX_DEPTH levels deep (no cycles).    */
} vr_material_kind;

#define VR_MAX_MIX_DEPTH 8

typedef struct vr_material {
    int32_t kind;       /* vr_material_kind                                     */
    float color[3];     /* albedo / emitted radiance / microfacet colour        */
    float fuzz;         /* metal                                                */
    float ir;           /* dielectric ior; microfacet index                     */
    float roughness;    /* microfacet Beckmann m                                */
    float metallic;     /* microfacet                                           */
    float emittance;    /* microfacet (stored, unused by its scatter, as in the
                           reference)                                           */
    int32_t transparent;/* microfacet                                           */
    int32_t albedo_texture;  /* Lambertian: ColorType::Texture (simple.rs:83-133),
                                index into vr_scene_desc.textures, -1 = color */
    int32_t normal_texture;  /* Lambertian: normal map (its raw RGB replaces the
                                shading normal of the scatter, simple.rs:109-113),
                                -1 = none                                        */
    int32_t mix_first;       /* VR_MAT_MIX: material indices of the two children */
    int32_t mix_second;
    float mix_factor;        /* VR_MAT_MIX: probability of `mix_second`          */
} vr_material;

/* One triangle mesh: Mesh::from_buffers (voidray_renderer/src/core/mesh.rs:76-116).
 * normals == NULL means zero vertex normals, like Vertex::position
 * (mesh.rs:25-33, used by Surfaces::quad).  uvs == NULL means zero uvs. */
typedef struct vr_mesh_desc {
    const float* positions;   /* 3 * num_vertices                              */
    const float* normals;     /* 3 * num_vertices or NULL                      */
    const float* uvs;         /* 2 * num_vertices or NULL                      */
    const uint32_t* indices;  /* 3 * num_triangles                             */
    uint32_t num_vertices;
    uint32_t num_triangles;
    uint32_t material;        /* index into vr_scene_desc.materials            */
    uint32_t pad_;
} vr_mesh_desc;

typedef enum vr_env_kind {
    VR_ENV_NONE = 0,    /* scene.environment == None -> black (tracer.rs:31)   */
    VR_ENV_UNIFORM = 1, /* Environments::uniform (environments.rs:29-33)       */
    VR_ENV_HDRI = 2     /* Environments::hdri lat-long RGB f32 (environments.rs:35-90) */
} vr_env_kind;

typedef struct vr_environment_desc {
    int32_t kind;         /* vr_env_kind                                        */
    float color[3];       /* uniform colour                                     */
    const float* image;   /* HDRI: width*height*3 f32, row 0 first (image crate order) */
    uint32_t width;
    uint32_t height;
    int32_t importance_sample; /* build the 2D CDF used by VR_EST_NEE          */
    int32_t pad_;
} vr_environment_desc;

/* Camera (voidray_renderer/src/core/camera.rs:7-22).  direction and up as the
 * reference stores them after Camera::look_at (unit, orthogonal). */
typedef struct vr_camera_desc {
    float eye[3];
    float direction[3];
    float up[3];
    float fov;            /* radians, on the longer image axis                  */
    int32_t has_dof;
    float aperture;
    float focal_point[3];
} vr_camera_desc;

/* ImageTexture (voidray_renderer/src/core/texture.rs:28-98): RGB f32, row 0
 * first; sample(u, v) wraps u, v into [0, 1) as the reference does and reads
 * the texel nearest to (u W, (1 - v) H) or blends the four around it, with
 * the reference's linear-index modulo at the edges. */
typedef enum vr_texture_sampling {
    VR_TEX_NEAREST = 0,
    VR_TEX_BILINEAR = 1
} vr_texture_sampling;

typedef struct vr_texture_desc {
    const float* image;       /* width * height * 3 f32                           */
    uint32_t width;
    uint32_t height;
    int32_t sampling;         /* vr_texture_sampling                              */
    int32_t pad_;
} vr_texture_desc;

/* Analytic surfaces (voidray_common/src/surfaces.rs:31-114): Surfaces::sphere
 * (quadratic, normal (p - c) / r, uv 0) and Surfaces::ground_plane (y =
 * height, normal +y, uv (x, z)).  Tested against every ray beside the
 * triangle BVH; their prim id in hits is num_triangles + index. */
typedef enum vr_analytic_kind {
    VR_ANALYTIC_SPHERE = 1,
    VR_ANALYTIC_GROUND_PLANE = 2
} vr_analytic_kind;

typedef struct vr_analytic_desc {
    int32_t kind;             /* vr_analytic_kind                               */
    float center[3];          /* sphere                                         */
    float radius;             /* sphere                                         */
    float height;             /* ground plane                                   */
    uint32_t material;        /* index into vr_scene_desc.materials             */
    uint32_t pad_;
} vr_analytic_desc;

typedef struct vr_scene_desc {
    const vr_mesh_desc* meshes;
    uint32_t num_meshes;
    uint32_t num_materials;
    const vr_material* materials;
    vr_environment_desc environment;
    vr_camera_desc camera;
    uint32_t bvh_max_leaf;  /* 0 = default (4)                                  */
    uint32_t bvh_bins;      /* 0 = default (16)                                 */
    const vr_analytic_desc* analytics;  /* may be NULL when num_analytics == 0  */
    uint32_t num_analytics;             /* at most VR_MAX_ANALYTICS             */
    uint32_t num_textures;
    const vr_texture_desc* textures;    /* may be NULL when num_textures == 0   */
} vr_scene_desc;
#define VR_MAX_ANALYTICS 64

typedef struct vr_scene vr_scene;

/* Builds the scene: binned-SAH BVH2 on the host, flattened to 64-byte nodes and
 * 48-byte triangles (16-byte aligned), uploaded to the current CUDA device.
 * Replaces Scene::build_acceleration (voidray_renderer/src/core/scene.rs:163-178). */
vr_status vr_scene_create(const vr_scene_desc* desc, vr_scene** out);
vr_status vr_scene_destroy(vr_scene* scene);

typedef struct vr_scene_info {
    uint64_t num_triangles;
    uint64_t num_nodes;
    uint64_t device_bytes;   /* all device memory held by the scene           */
    uint32_t max_depth;
    uint32_t max_leaf;
    double sah_cost;
    double build_ms;
} vr_scene_info;
vr_status vr_scene_info_get(const vr_scene* scene, vr_scene_info* info);

/* Host-only structural check, usable without a GPU: lowers the descriptor,
 * builds and flattens the BVH and verifies its invariants (every triangle in
 * exactly one leaf, every child box encloses its subtree, depth within the
 * traversal stack).  Fills info (device_bytes = bytes the scene would hold). */
vr_status vr_scene_validate(const vr_scene_desc* desc, vr_scene_info* info);

/* Replace the camera of a built scene (the GUI edits Scene.camera between renders). */
vr_status vr_scene_set_camera(vr_scene* scene, const vr_camera_desc* camera);

/* ------------------------------------------------------------ settings -- */

/* RenderMode (voidray_renderer/src/core/settings.rs:8-12): Normal = 0, Full = 1. */
typedef enum vr_render_mode { VR_MODE_NORMAL = 0, VR_MODE_FULL = 1 } vr_render_mode;

/* Estimator.  VR_EST_REFERENCE reproduces trace_ray_internal exactly
 * (tracer.rs:19-56: per-level firefly clamp, miss -> environment).
 * VR_EST_NEE is the production estimator (no reference counterpart):
 * forward throughput, environment importance sampling with shadow rays and
 * MIS at Lambertian vertices, per-contribution clamp. */
typedef enum vr_estimator { VR_EST_REFERENCE = 0, VR_EST_NEE = 1 } vr_estimator;

/* RenderSettings (settings.rs:15-34) plus the GPU-only knobs. */
typedef struct vr_render_settings {
    uint32_t total_samples;   /* divides the accumulated sum (iterative.rs:45)  */
    float update_frequency;   /* render-thread chunking (renderer.rs:78); unused by vr_render */
    int32_t render_mode;      /* vr_render_mode                                 */
    float firefly_clamp;      /* Color::clamp(max) per level (tracer.rs:50)     */
    uint32_t max_bounces;
    int32_t estimator;        /* vr_estimator                                   */
    uint32_t rr_depth;        /* Russian roulette from this depth; 0 = off      */
    uint32_t wavefront_paths; /* paths per wavefront; 0 = autotuned default     */
} vr_render_settings;

/* Tonemap (settings.rs:36-55): None=0, ACES=1, Reinhard=2, Filmic=3, Uncharted2=4. */
typedef struct vr_color_management {
    int32_t tonemap;
    float gamma;
    float exposure;
    int32_t transparent;
} vr_color_management;

/* ------------------------------------------------------------- render -- */

/* iterative_render (voidray_renderer/src/render/iterative.rs:11-55):
 * for every pixel, sums `samples` jittered paths, scales by
 * 1/settings.total_samples and adds the result to rgba (RGBA f32, row-major,
 * width*height*4); alpha gains 1.0 per call as Color::a() returns 1
 * (voidray_renderer/src/util/color.rs:54-56).  Sample s of pixel p draws from
 * the PCG32 stream (seed, first_sample + s, p), so successive calls with
 * advancing first_sample continue one progressive render.
 * The row of pixel index i is i / width (the reference's i / height,
 * iterative.rs:26, is only correct for square images). */
vr_status vr_render(vr_scene* scene, const vr_render_settings* settings,
                    uint32_t samples, float* rgba, uint32_t width,
                    uint32_t height, uint64_t seed, uint32_t first_sample);
/* Same, rgba is device memory; runs on `stream` (NULL = scene stream). */
vr_status vr_render_device(vr_scene* scene, const vr_render_settings* settings,
                           uint32_t samples, float* rgba_device, uint32_t width,
                           uint32_t height, uint64_t seed, uint32_t first_sample,
                           void* stream);

/* vr_render_device plus first-hit feature buffers (AOVs) for the denoiser;
 * no counterpart in the reference.  rgba_device receives exactly what
 * vr_render_device writes for the same arguments.  albedo_device and
 * normal_device (RGBA f32, width*height*4, device memory) receive, summed
 * over the same samples and scaled by 1/settings.total_samples like the
 * radiance: the first hit's surface colour clamped to 1 (1 for dielectrics;
 * the environment colour clamped to 1 for rays that miss) and the first
 * hit's shading normal facing the camera ray (0 for misses); alpha gains 1.0
 * per call. */
vr_status vr_render_aov_device(vr_scene* scene, const vr_render_settings* settings,
                               uint32_t samples, float* rgba_device, float* albedo_device,
                               float* normal_device, uint32_t width, uint32_t height,
                               uint64_t seed, uint32_t first_sample, void* stream);

/* Same render as vr_render_device, for callers that cannot allocate device
 * memory while they render.  No counterpart in the reference.  Such callers
 * are, for example, a host application (a game engine, a compositor, a
 * framework with its own caching allocator) that has already reserved the
 * GPU's memory for its own pool, so a cudaMalloc from the library would fail
 * or evict its data; and a real-time frame loop that cannot afford the
 * device-wide synchronisation that cudaFree implies, nor an allocation that
 * fails in the middle of a frame.  vr_render_device grows a per-scene scratch
 * with cudaMalloc when an image or wavefront needs more; this entry point
 * calls no cudaMalloc, cudaFree or allocating library routine.  Its wavefront
 * scratch (ray queues, path state, per-pixel sums) lives in one device array
 * of VR_NOALLOC_SCRATCH_BYTES (64 MiB) inside the library, which every GPU
 * that loads the library holds until the process exits.  The image must fit
 * in it: 16 bytes per pixel plus room for at least 1024 paths (about 4
 * Mpixels, e.g. 2000x2000); larger images are rejected with
 * VR_ERR_UNSUPPORTED before anything is launched, and the wavefront is sized
 * to what remains.  The first call on each device looks up the array's
 * device address with that device current (a one-time set-up); make that
 * first call before any stream capture.  All calls share the one array and
 * it keeps the last call's contents (the pixel sums are cleared by every
 * call), so calls that overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller.  The scene must have been
 * created beforehand with vr_scene_create, which allocates its own memory. */
#define VR_NOALLOC_SCRATCH_BYTES (64u << 20)
vr_status vr_render_device_noalloc(vr_scene* scene, const vr_render_settings* settings,
                                   uint32_t samples, float* rgba_device, uint32_t width,
                                   uint32_t height, uint64_t seed, uint32_t first_sample,
                                   void* stream);

/* ------------------------------------------------------------- batch -- */

/* Multi-scene rendering (no reference counterpart): many render jobs -- each
 * a scene with its own settings, image, seed and sample range -- share one
 * wavefront launch per stage.  Every job owns a segment of the path state and
 * of each ray queue with its own counters; paths of all jobs are traced by
 * the same persistent kernels.  A job's image is bit-identical to rendering
 * it alone with vr_render_device (same sample streams, same per-pixel
 * summation order). */
typedef struct vr_render_job {
    vr_scene* scene;
    vr_render_settings settings;
    uint32_t samples;
    uint32_t width;
    uint32_t height;
    uint32_t first_sample;
    uint64_t seed;
    float* rgba_device;       /* RGBA f32 accumulation buffer, += like vr_render */
    float* albedo_device;     /* optional first-hit AOV buffers, += like          */
    float* normal_device;     /* vr_render_aov_device (both set or both NULL)     */
} vr_render_job;

typedef struct vr_batch vr_batch;
/* max_wave_paths: paths per wavefront over all jobs (0 = 2^26; at most 2^28).  A batch keeps
 * scratch for its largest wave (about 180 bytes per path with NEE) until destroyed. */
vr_status vr_batch_create(uint64_t max_wave_paths, vr_batch** out);
vr_status vr_batch_destroy(vr_batch* batch);
/* Enqueues all jobs on `stream` (NULL = legacy default stream); scenes must
 * live on the batch's device.  Returns before the GPU finishes. */
vr_status vr_batch_render(vr_batch* batch, const vr_render_job* jobs, uint32_t count, void* stream);
/* Waits for `stream` and reports kernel-side errors. */
vr_status vr_batch_synchronize(vr_batch* batch, void* stream);
/* Launch shapes of the shade and raygen stages (process-wide; the autotuner
 * in voidray_gb300/autotune.py sets them).  Results do not depend on them. */
typedef struct vr_tuning {
    uint32_t shade_block;          /* 64, 128 or 256 threads (default 256)   */
    uint32_t shade_blocks_per_sm;  /* resident blocks per SM, 1-32 (8)       */
    uint32_t raygen_block;         /* 64, 128 or 256 threads (256)           */
    uint32_t generation;           /* out: bumped by every set                */
} vr_tuning;
vr_status vr_tuning_get(vr_tuning* tuning);
vr_status vr_tuning_set(const vr_tuning* tuning);

/* With graphs enabled, every wavefront's stage sequence (raygen, each depth's
 * extend / shade / shadow, accumulate) is captured once as a CUDA graph and
 * replayed on later calls with the same job-set shape (job count, paths,
 * depth); the per-call data (sample offsets, seeds, scenes) is read from the
 * device job table, so results are identical to direct launches.  A shape
 * is captured the second time it shows up (shapes that never repeat run
 * directly).  Needs a non-NULL stream; off by default.  No counterpart in the
 * reference. */
vr_status vr_batch_set_graphs(vr_batch* batch, int32_t enable);
vr_status vr_batch_graph_stats(vr_batch* batch, uint64_t* captures, uint64_t* replays);

/* --------------------------------------------------------- serving stats --
 * Per-pass error statistics of many progressive jobs in one launch (no
 * reference counterpart; used by the serving loop).  Each job keeps two
 * half-buffers of RGBA f32 sample sums A and B (n_a, n_b samples) and, when
 * it is denoised, the denoiser outputs DA, DB of the half means.  With
 * a = A/n_a, b = B/n_b, m = (A + B)/(n_a + n_b), d = m^2 + 1e-2 and the sums
 * over RGB, the kernel writes for every 16 x 16 pixel tile t of job j, at
 * out[tile_offset + k * tiles + t] (tiles = ceil(h/16) * ceil(w/16)):
 *   k = 0: SUM over the tile of (a-b)^2 n_a n_b / n^2 / d   (the plain estimate)
 *   k = 1..5 (denoised jobs only): MEANS over the tile's pixels and channels
 *          of (a-b)^2/d, (DA-b)^2/d, (DB-a)^2/d, (DA-DB)^2/d, (DA-DB)(a-b)/d.
 * Sums are in fp64 in a fixed order (deterministic). */
typedef struct vr_stats_job {
    const float* sum_a;
    const float* sum_b;
    const float* den_a;       /* NULL: plain statistic only                     */
    const float* den_b;
    uint32_t n_a, n_b;
    uint32_t width, height;
    uint64_t tile_offset;
} vr_stats_job;
#define VR_STATS_TILE 16
#define VR_STATS_MAX_JOBS 128  /* per call */
vr_status vr_serve_stats_device(const vr_stats_job* jobs, uint32_t count, double* out_device, void* stream);

/* A served job's final image, on the device (no reference counterpart).
 * vr_serve_sum_device: out[k] = a[k] + b[k] for `pairs` (1-3) pairs of RGBA
 * f32 buffers of `pixels` pixels (the full sums of the job's radiance,
 * albedo and normal halves, the denoiser's input with scale 1/samples).
 * vr_serve_blend_device: rgb (3 f32 per pixel) = the plain mean
 * (sum_a + sum_b) / samples, or with `denoised` (RGBA, the denoised full
 * mean) and `alpha_tiles` (one weight per VR_STATS_TILE x VR_STATS_TILE tile,
 * row-major over the tiles) alpha D + (1 - alpha) mean per pixel.  All
 * buffers are device memory; RGBA buffers 16-byte aligned. */
vr_status vr_serve_sum_device(const float* const* a, const float* const* b, float* const* out, uint32_t pairs,
                              uint64_t pixels, void* stream);
vr_status vr_serve_blend_device(const float* sum_a, const float* sum_b, uint32_t samples, const float* denoised,
                                const float* alpha_tiles, uint32_t width, uint32_t height, float* rgb,
                                void* stream);

typedef struct vr_render_stats {
    uint64_t paths;          /* camera paths traced                            */
    uint64_t extend_rays;    /* closest-hit rays                               */
    uint64_t shadow_rays;    /* any-hit rays                                   */
    uint64_t wavefronts;
    double ms;               /* wall time of the last render call             */
    uint32_t error_flags;    /* device status word (VR_ERR_STACK etc.)        */
    uint32_t pad_;
} vr_render_stats;
vr_status vr_render_stats_get(const vr_scene* scene, vr_render_stats* stats);
/* Totals over every vr_batch_render call of the batch (synchronises the device). */
vr_status vr_batch_stats_get(vr_batch* batch, vr_render_stats* stats);

/* Instrumentation (no reference counterpart).  VR_INSTR_STAGE_TIMES brackets
 * every wavefront stage launch with CUDA events on the render stream;
 * VR_INSTR_WORK runs the extend and shadow stages in a counting variant that
 * adds their traversal work (inner-node visits, triangle tests).  Counting
 * changes kernel timing, so it belongs in a separate run.  Setting the flags
 * resets the accumulators; vr_scene_instrument_get synchronises the scene. */
#define VR_INSTR_STAGE_TIMES 1u
#define VR_INSTR_WORK 2u
enum { VR_STAGE_RAYGEN = 0, VR_STAGE_EXTEND = 1, VR_STAGE_SHADE = 2, VR_STAGE_SHADOW = 3,
       VR_STAGE_ACCUMULATE = 4, VR_NUM_STAGES = 5 };
typedef struct vr_instrument {
    double stage_ms[8];
    uint64_t stage_launches[8];
    uint64_t extend_node_visits;
    uint64_t extend_tri_tests;
    uint64_t shadow_node_visits;
    uint64_t shadow_tri_tests;
    uint64_t retired_paths;  /* VR_INSTR_WORK: paths that ended (queue conservation:
                                equals the camera paths traced) */
    uint64_t metal_fallbacks;/* VR_INSTR_WORK: Metal::scatter's rejection loop (a
                                direction above the surface, simple.rs:140-161)
                                ran out of its 64 tries and the path was absorbed */
} vr_instrument;
vr_status vr_scene_instrument(vr_scene* scene, uint32_t flags);
vr_status vr_scene_instrument_get(vr_scene* scene, vr_instrument* out);

/* post_process.glsl:23-49: out = pow(tonemap(rgb * scale * 2^exposure), 1/gamma), a = 1. */
vr_status vr_tonemap(const float* rgba_in, float* rgba_out, uint32_t width,
                     uint32_t height, const vr_color_management* cm, float scale);
vr_status vr_tonemap_device(const float* rgba_in_device, float* rgba_out_device,
                            uint32_t width, uint32_t height,
                            const vr_color_management* cm, float scale, void* stream);

/* The legacy viewport's post-processing (voidray/src/shaders/
 * viewport_fragment.glsl:27-67 with tonemapping.glsl:1-69): its own tonemap
 * numbering, exposure as a linear factor, gamma 1 for Filmic, and with
 * `transparent` the output alpha is the scaled input alpha (else 1). */
typedef enum vr_legacy_tonemap {
    VR_LEGACY_TONEMAP_NONE = 0,
    VR_LEGACY_TONEMAP_SIMPLE_ACES = 1,
    VR_LEGACY_TONEMAP_SIMPLE_REINHARD = 2,
    VR_LEGACY_TONEMAP_LUMA_REINHARD = 3,
    VR_LEGACY_TONEMAP_LUMA_WHITEPRESERVING_REINHARD = 4,
    VR_LEGACY_TONEMAP_ROM_BIN_DA_HOUSE = 5,
    VR_LEGACY_TONEMAP_FILMIC = 6,
    VR_LEGACY_TONEMAP_UNCHARTED_2 = 7
} vr_legacy_tonemap;
vr_status vr_tonemap_legacy(const float* rgba_in, float* rgba_out, uint32_t width, uint32_t height,
                            int32_t tonemap, float gamma, float exposure, int32_t transparent, float scale);
vr_status vr_tonemap_legacy_device(const float* rgba_in_device, float* rgba_out_device, uint32_t width,
                                   uint32_t height, int32_t tonemap, float gamma, float exposure,
                                   int32_t transparent, float scale, void* stream);

/* relative MSE over RGB: mean((x-r)^2/(r^2+eps)), eps = 1e-2; each image is
 * RGBA f32 scaled by its own factor first. */
vr_status vr_relmse_device(const float* rgba_device, float scale,
                           const float* ref_rgba_device, float ref_scale,
                           uint32_t width, uint32_t height, double* out, void* stream);

/* ---------------------------------------------------------- intersect -- */

/* A ray: origin, tmin, direction, tmax (32 bytes).  The triangle test rejects
 * |det| < tmin, as Triangle::hit does with its t_min argument
 * (voidray_renderer/src/core/mesh.rs:156). */
typedef struct vr_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} vr_ray;

/* Closest (or any) hit: triangle id in mesh-concatenation order, t and the
 * barycentrics (u weights vertex 1, v weights vertex 2, as mesh.rs:176-178).
 * prim == VR_MISS for no hit. */
#define VR_MISS 0xFFFFFFFFu
typedef struct vr_hit {
    uint32_t prim;
    float t;
    float u;
    float v;
} vr_hit;

/* SceneAcceleration::hit over a batch of rays (host memory). any_hit != 0
 * returns any intersection in (tmin, tmax) instead of the closest. */
vr_status vr_intersect(vr_scene* scene, const vr_ray* rays, uint64_t count,
                       vr_hit* hits, int32_t any_hit);
vr_status vr_intersect_device(vr_scene* scene, const vr_ray* rays_device,
                              uint64_t count, vr_hit* hits_device,
                              int32_t any_hit, void* stream);

/* Environment::sample (voidray_renderer/src/core/traits.rs:66-69) of the
 * scene's environment for `count` directions (3 f32 each, host memory; need
 * not be normalised): RGB f32 into rgb (3 per direction).  The same lookup
 * the integrator applies to escaping rays (HDRI: bilinear with the
 * reference's linear-index wrap and pole saturation). */
vr_status vr_environment_sample(vr_scene* scene, const float* directions, uint64_t count, float* rgb);

/* Traversal work counters for the same rays and kernels (inner-node visits,
 * triangle tests), used to state the algorithmic bytes of a launch. */
vr_status vr_intersect_count_device(vr_scene* scene, const vr_ray* rays_device,
                                    uint64_t count, int32_t any_hit,
                                    uint64_t* node_visits, uint64_t* tri_tests,
                                    void* stream);

/* --------------------------------------------------------------- misc -- */

const char* vr_last_error(void);
int32_t vr_abi_version(void);
/* 1 if a CUDA device is usable, 0 otherwise (never fails). */
int32_t vr_device_available(void);
/* Device synchronisation of the scene stream. */
vr_status vr_scene_synchronize(vr_scene* scene);

#ifdef __cplusplus
}
#endif

#endif /* VOIDRAY_GPU_H */
