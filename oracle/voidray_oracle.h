/*
 * voidray_oracle.h — CPU oracle for the voidray path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a C++ restatement of the reference's CPU
 * integrator (LevKruglyak/voidray, Rust), used as the checker for the GPU
 * library and as the timed CPU baseline.  The product never links or calls
 * it.  Parity is unpinned: the reference ships no golden vectors or
 * known-answer tests for this path and cannot be built here (Rust), so the
 * restatement is anchored on analytic known-answer tests instead.
 *
 * Reference files restated (paths within the reference project):
 *   voidray_renderer/src/render/iterative.rs:11-55   iterative_render
 *   voidray_renderer/src/core/tracer.rs:9-56         trace_ray(_internal)
 *   voidray_renderer/src/core/camera.rs:26-82        Camera / cast_ray
 *   voidray_renderer/src/core/scene.rs:163-185       build_acceleration / hit
 *   voidray_renderer/src/core/bvh.rs:48-181          median BVH, traversal
 *   voidray_renderer/src/core/mesh.rs:76-218         Mesh, Triangle::hit
 *   voidray_renderer/src/util/{aabb,ray,math,color}.rs
 *   voidray_common/src/simple.rs:60-232              materials
 *   voidray_common/src/microfacet.rs:120-313         MicrofacetBSDF
 *   voidray_common/src/environments.rs:19-90         environments
 *   voidray_renderer/src/shaders/{post_process,tonemapping}.glsl
 *
 * Random numbers: the reference draws from the OS-seeded thread_rng
 * (iterative.rs:29); no stream can be reproduced.  The oracle draws from a
 * PCG32 stream per (seed, sample, pixel) with samplers of the same
 * distributions (rand_distr 0.4.3 UnitSphere/UnitDisc/UnitCircle, rand 0.8.5
 * gen_range / gen::<f32> / gen_bool), so the GPU library can be checked path
 * by path on identical streams.
 */
#ifndef VOIDRAY_ORACLE_H
#define VOIDRAY_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh {
    const float* positions;  /* 3*nv */
    const float* normals;    /* 3*nv or NULL (zero, Vertex::position) */
    const float* uvs;        /* 2*nv or NULL */
    const uint32_t* indices; /* 3*nt */
    uint32_t num_vertices;
    uint32_t num_triangles;
    uint32_t surface;        /* index in the scene's surface list */
    uint32_t pad_;
} orc_mesh;

/* Surfaces::sphere / Surfaces::ground_plane (voidray_common/src/surfaces.rs) */
typedef struct orc_analytic {
    int32_t kind;            /* 1 sphere, 2 ground plane */
    float center[3];
    float radius;
    float height;
    uint32_t surface;        /* index in the scene's surface list */
    uint32_t pad_;
} orc_analytic;

typedef struct orc_object { uint32_t surface; uint32_t material; } orc_object;

typedef struct orc_material {
    int32_t kind; float color[3]; float fuzz; float ir; float roughness;
    float metallic; float emittance; int32_t transparent;
    int32_t albedo_texture; int32_t normal_texture;  /* -1: none */
    int32_t mix_first; int32_t mix_second; float mix_factor;  /* kind 6: MixMaterial */
} orc_material;

/* ImageTexture (voidray_renderer/src/core/texture.rs) */
typedef struct orc_texture {
    const float* image; uint32_t width; uint32_t height; int32_t sampling; int32_t pad_;
} orc_texture;

typedef struct orc_env {
    int32_t kind; float color[3]; const float* image; uint32_t width; uint32_t height;
    int32_t importance_sample; int32_t pad_;
} orc_env;

typedef struct orc_camera {
    float eye[3]; float direction[3]; float up[3]; float fov;
    int32_t has_dof; float aperture; float focal_point[3];
} orc_camera;

typedef struct orc_scene_desc {
    const orc_mesh* meshes; uint32_t num_meshes;
    uint32_t num_materials; const orc_material* materials;
    const orc_object* objects; uint32_t num_objects; uint32_t pad_;
    orc_env env;
    orc_camera camera;
    const orc_analytic* analytics; uint32_t num_analytics; uint32_t num_textures;
    const orc_texture* textures;
} orc_scene_desc;

typedef struct orc_settings {
    uint32_t total_samples; int32_t render_mode; float firefly_clamp;
    uint32_t max_bounces; int32_t estimator; uint32_t rr_depth;
} orc_settings;

typedef struct orc_ray { float org[3]; float tmin; float dir[3]; float tmax; } orc_ray;
typedef struct orc_hit { uint32_t prim; float t; float u; float v; } orc_hit;

typedef struct orc_scene orc_scene;

orc_scene* orc_scene_create(const orc_scene_desc* desc);
void orc_scene_destroy(orc_scene* s);
const char* orc_last_error(void);

/* mode 0: the reference's two-level median BVH traversal (closest hit);
 * second_t (optional) receives the second-nearest accepted t seen.
 * mode 1: brute force over every triangle (closest), second_t likewise.
 * mode 2: any hit in (tmin, tmax): closest from mode 0 if its t < tmax. */
void orc_intersect(const orc_scene* s, const orc_ray* rays, uint64_t n,
                   orc_hit* hits, float* second_t, int32_t mode, int32_t threads);

/* Triangle::hit of one triangle (global id) with the ray's tmin as epsilon;
 * returns 1 on a hit with t > tmin (tmax ignored, as the reference does). */
int32_t orc_triangle_hit(const orc_scene* s, uint32_t prim, const orc_ray* ray,
                         float* t, float* u, float* v);
/* Moller-Trumbore in double precision, no epsilon; returns 0 if parallel. */
int32_t orc_reintersect_f64(const orc_scene* s, uint32_t prim, const orc_ray* ray,
                            double* t, double* u, double* v);

/* iterative_render over pixels [pixel_begin, pixel_end) (end 0 = all).
 * rays_out (optional) receives extend and shadow ray counts. */
void orc_render(const orc_scene* s, const orc_settings* st, uint32_t samples,
                float* rgba, uint32_t width, uint32_t height, uint64_t seed,
                uint32_t first_sample, uint32_t pixel_begin, uint32_t pixel_end,
                int32_t threads, uint64_t* rays_out);

/* One path's radiance (debug / unit tests). */
void orc_trace_path(const orc_scene* s, const orc_settings* st, uint32_t width,
                    uint32_t height, uint32_t pixel, uint32_t sample, uint64_t seed,
                    float* rgb_out);

/* post_process.glsl + tonemapping.glsl restated. */
void orc_tonemap(const float* rgba_in, float* rgba_out, uint64_t num_pixels,
                 int32_t tonemap, float gamma, float exposure, float scale);
/* The legacy viewport's post-processing (voidray/src/shaders/viewport_fragment.glsl). */
void orc_tonemap_legacy(const float* rgba_in, float* rgba_out, uint64_t num_pixels, int32_t tonemap,
                        float gamma, float exposure, int32_t transparent, float scale);

/* Environment lookup (HDRIEnvironment::sample / UniformEnvironment::sample). */
void orc_env_eval(const orc_scene* s, const float* dir, float* rgb_out);
/* Importance-sampling tables (extension): sample with four uniforms and pdf. */
int32_t orc_env_sample(const orc_scene* s, const float* u4, float* dir_out,
                       float* pdf_out);
float orc_env_pdf(const orc_scene* s, const float* dir);
/* Copies of the tables for comparison with the library's: sizes H+1,
 * H*(W+1), H*W. Returns 0 if the scene has none. */
int32_t orc_env_tables(const orc_scene* s, float* marginal, float* conditional,
                       float* cell_prob);

/* PCG32 stream check: n outputs of stream (seed, sample, pixel). */
void orc_pcg32(uint64_t seed, uint32_t sample, uint32_t pixel, uint32_t n, uint32_t* out);
/* Samplers on that stream: kind 0 unit sphere, 1 unit disc, 2 unit circle,
 * 3 uniform [0,1); writes n vectors of 3 floats. */
void orc_sampler(uint64_t seed, uint32_t sample, uint32_t pixel, int32_t kind,
                 uint32_t n, float* out);

/* AABB::hit (util/aabb.rs:86-148). */
int32_t orc_aabb_hit(const float* bmin, const float* bmax, const orc_ray* ray,
                     float t_min, float t_max);

uint64_t orc_num_triangles(const orc_scene* s);
int32_t orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
