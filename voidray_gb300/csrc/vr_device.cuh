// vr_device.cuh — device-side data layout and per-path arithmetic of the
// GB300 wavefront integrator.
//
// Every translation unit is compiled with -fmad=false so that each f32
// operation rounds separately, the way the reference's Rust code (no FMA
// contraction) and cgmath 0.18 compute them: dot = (x*x' + y*y') + z*z',
// normalize = v * (1/|v|).  Where speed matters and exactness does not (the
// BVH slab tests) the code calls fmaf explicitly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vr {

constexpr float PI_F = 3.14159265358979323846f;
constexpr float INF_F = __builtin_huge_valf();
constexpr float SCENE_TMIN = 0.00001f;  // SceneAcceleration::hit (scene.rs:183)
constexpr int REJECT_TRIES = 64;        // bound on the reference's rejection loops
constexpr int STACK_SIZE = 96;          // traversal stack entries (the builder keeps 3 x wide depth + 1 below it)
constexpr uint32_t MISS = 0xFFFFFFFFu;

// device status word bits
enum : uint32_t { ERRF_STACK = 1u, ERRF_QUEUE = 2u, ERRF_TIMEOUT = 4u };

enum MatKind : int32_t { M_LAMB = 0, M_METAL = 1, M_DIEL = 2, M_EMIT = 3, M_LBSDF = 4, M_MICRO = 5, M_MIX = 6 };
constexpr int MAX_MIX_DEPTH = 8;  // VR_MAX_MIX_DEPTH

struct Material {  // same layout as vr_material
    int32_t kind;
    float color[3];
    float fuzz, ir, roughness, metallic, emittance;
    int32_t transparent;
    int32_t albedo_tex, normal_tex;  // -1: none
    int32_t mix_first, mix_second;   // M_MIX children
    float mix_factor;
};

// BVH: 4-wide nodes of 8 x float4 (128 bytes; layout in vr_traverse.cuh),
// node 0 the root; leaves are ranges of at most 16 triangles.
// Triangle = 3 x float4 (48 bytes) in leaf order: (v0, prim id bits),
// (v1 - v0, 0), (v2 - v0, 0); the edges are the f32 differences the
// reference computes in Triangle::hit (mesh.rs:150-151).
// Shading record per prim (global id) = 4 x float4:
//   (n0, material id bits), (n1, 0), (n2, 0), (face normal, 0)
struct SceneView {
    const float4* nodes;
    const float4* tris;
    const float4* shade;
    const float2* uvs;  // 3 per prim
    const Material* materials;
    int32_t num_materials;
    // analytic surfaces: 2 float4 each, (center | radius) or (0, height, 0, 0),
    // then (kind bits, material bits, 0, 0); prim id = num_tris + index
    const float4* analytic;
    uint32_t num_analytic;
    uint32_t num_tris;
    // image textures: per texture (texel offset, width, height, sampling) as
    // int bits; texels RGB f32
    const int4* tex_info;
    const float* texels;
    uint32_t num_textures;
    // environment
    int32_t env_kind;
    float env_color[3];
    const float* env_img;
    uint32_t env_w, env_h;
    const float* env_marg;   // H+1
    const float* env_cond;   // H*(W+1)
    const float* env_cell;   // H*W
    int32_t env_is;
    float env_density_scale; // W*H/(2 pi^2) as f32
    const uint32_t* env_gmarg;  // guide of the marginal search, env_gm + 1 entries
    const uint32_t* env_gcond;  // guides of the conditional rows, H * (env_gc + 1)
    uint32_t env_gm, env_gc;    // powers of two
    // camera acceleration (camera.rs:38-53)
    float c_origin[3], c_dir[3], c_right[3], c_up[3];
    float c_d;
    int32_t c_dof;
    float c_aperture, c_focal;
};

// ------------------------------------------------------------ vec3 ------
struct V3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ V3 vmul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float mag2(V3 a) { return dot(a, a); }
__host__ __device__ __forceinline__ V3 normalize(V3 a) { return a * (1.0f / sqrtf(mag2(a))); }
__host__ __device__ __forceinline__ V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }
__host__ __device__ __forceinline__ V3 xyz(float4 a) { return v3(a.x, a.y, a.z); }
__host__ __device__ __forceinline__ V3 clampc(V3 c, float m) { return v3(fminf(c.x, m), fminf(c.y, m), fminf(c.z, m)); }
__host__ __device__ __forceinline__ float max3(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__host__ __device__ __forceinline__ bool near_zero(V3 v) {  // math.rs:6-9
    const float e = 1.0e-8f;
    return fabsf(v.x) < e && fabsf(v.y) < e && fabsf(v.z) < e;
}
__host__ __device__ __forceinline__ V3 reflect(V3 v, V3 n) { return v - (2.0f * dot(v, n)) * n; }  // math.rs:12-14
__host__ __device__ __forceinline__ V3 refract(V3 uv, V3 n, float eta) {                         // math.rs:16-21
    float cos_theta = fminf(dot(n, -uv), 1.0f);
    V3 out_perp = eta * (uv + cos_theta * n);
    V3 out_parallel = -(sqrtf(fabsf(1.0f - mag2(out_perp)))) * n;
    return out_perp + out_parallel;
}
__host__ __device__ __forceinline__ float powi2(float x) { return x * x; }
__host__ __device__ __forceinline__ float powi3(float x) { return x * (x * x); }
__host__ __device__ __forceinline__ float powi5(float x) { float s = x * x; s = s * s; return x * s; }
__host__ __device__ __forceinline__ V3 lerp3(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }

// ------------------------------------------------------------ rng -------
// PCG32 with one stream per (sample, pixel): inc = (sample<<32 | pixel)<<1 | 1.
__host__ __device__ __forceinline__ uint64_t pcg_inc(uint32_t sample, uint32_t pixel) {
    uint64_t stream = ((uint64_t)sample << 32) | (uint64_t)pixel;
    return (stream << 1) | 1ull;
}
__host__ __device__ __forceinline__ uint32_t pcg_next(uint64_t& state, uint64_t inc) {
    uint64_t old = state;
    state = old * 6364136223846793005ULL + inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
__host__ __device__ __forceinline__ uint64_t pcg_init(uint64_t seed, uint64_t inc) {
    uint64_t st = 0;
    pcg_next(st, inc);
    st += seed;
    pcg_next(st, inc);
    return st;
}
struct Rng {
    uint64_t state, inc;
    __device__ __forceinline__ uint32_t next() { return pcg_next(state, inc); }
    __device__ __forceinline__ float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    __device__ __forceinline__ float range(float lo, float hi) {
        float scale = hi - lo;
        return uniform() * scale + lo;
    }
};
// rand_distr 0.4.3 UnitSphere (Marsaglia), UnitDisc, UnitCircle with a bound.
__device__ __forceinline__ V3 unit_sphere(Rng& r) {
    for (int i = 0; i < REJECT_TRIES; ++i) {
        float x1 = r.range(-1.0f, 1.0f), x2 = r.range(-1.0f, 1.0f);
        float sum = x1 * x1 + x2 * x2;
        if (sum >= 1.0f) continue;
        float factor = 2.0f * sqrtf(1.0f - sum);
        return v3(x1 * factor, x2 * factor, 1.0f - 2.0f * sum);
    }
    return v3(0.0f, 0.0f, 1.0f);
}
__device__ __forceinline__ void unit_disc(Rng& r, float* x, float* y) {
    for (int i = 0; i < REJECT_TRIES; ++i) {
        float x1 = r.range(-1.0f, 1.0f), x2 = r.range(-1.0f, 1.0f);
        if (x1 * x1 + x2 * x2 <= 1.0f) { *x = x1; *y = x2; return; }
    }
    *x = 0.0f; *y = 0.0f;
}
__device__ __forceinline__ void unit_circle(Rng& r, float* x, float* y) {
    for (int i = 0; i < REJECT_TRIES; ++i) {
        float x1 = r.range(-1.0f, 1.0f), x2 = r.range(-1.0f, 1.0f);
        float x1sq = x1 * x1, x2sq = x2 * x2;
        float sum = x1sq + x2sq;
        if (sum >= 1.0f) continue;
        float diff = x1sq - x2sq;
        *x = diff / sum; *y = 2.0f * x1 * x2 / sum; return;
    }
    *x = 1.0f; *y = 0.0f;
}

// ------------------------------------------------------ analytic surfaces --
constexpr uint32_t A_SPHERE = 1, A_PLANE = 2;

// Sphere::hit (surfaces.rs:45-80) and GroundPlane::hit (surfaces.rs:86-105),
// in the reference's operation order: true and t when the surface is hit in
// the reference's (tmin, tmax) window.
__device__ __forceinline__ bool analytic_hit(float4 a0, uint32_t kind, V3 o, V3 d, float tmin, float tmax, float& t) {
    if (kind == A_SPHERE) {
        const V3 oc = o - v3(a0.x, a0.y, a0.z);
        const float a = mag2(d);
        const float half_b = dot(oc, d);
        const float c = mag2(oc) - a0.w * a0.w;
        const float disc = half_b * half_b - a * c;
        if (disc < 0.0f) return false;
        const float sq = sqrtf(disc);
        float root = (-half_b - sq) / a;
        if (root < tmin || tmax < root) {
            root = (-half_b + sq) / a;
            if (root < tmin || tmax < root) return false;
        }
        t = root;
        return true;
    }
    const float tt = (a0.y - o.y) / d.y;
    if (tt <= tmin || tt >= tmax) return false;
    t = tt;
    return true;
}

// Nearest analytic hit in front of t_best (prim = num_tris + index).
__device__ __forceinline__ void analytic_closest(const float4* ana, uint32_t nana, uint32_t ntris, V3 o, V3 d,
                                                 float tmin, float tmax, float& t_best, uint32_t& prim) {
    for (uint32_t i = 0; i < nana; ++i) {
        const float4 a0 = __ldg(ana + 2 * i), a1 = __ldg(ana + 2 * i + 1);
        float t;
        if (analytic_hit(a0, __float_as_uint(a1.x), o, d, tmin, tmax, t) && t < t_best) {
            t_best = t;
            prim = ntris + i;
        }
    }
}

__device__ __forceinline__ bool analytic_any(const float4* ana, uint32_t nana, V3 o, V3 d, float tmin, float tmax) {
    for (uint32_t i = 0; i < nana; ++i) {
        const float4 a0 = __ldg(ana + 2 * i), a1 = __ldg(ana + 2 * i + 1);
        float t;
        if (analytic_hit(a0, __float_as_uint(a1.x), o, d, tmin, tmax, t)) return true;
    }
    return false;
}

}  // namespace vr
