// vr_kernels.cu — sm_103a kernels of the wavefront integrator.
//
//   k_intersect      closest / any hit over a ray batch (SceneAcceleration::hit,
//                    voidray_renderer/src/core/scene.rs:182-185)
//   k_raygen         iterative_render's per-sample camera ray (render/iterative.rs:25-42,
//                    core/camera.rs:69-82)
//   k_extend         closest hit of every live path (the reference's recursion step,
//                    core/tracer.rs:29)
//   k_shade          miss -> environment, hit -> material scatter (tracer.rs:30-50,
//                    voidray_common/src/simple.rs, microfacet.rs), NEE shadow-ray
//                    generation, Russian roulette, warp-aggregated queue compaction
//   k_shadow         any-hit visibility of the NEE shadow rays
//   k_accumulate     per-pixel sum in sample order (iterative.rs:37-43)
//   k_finalize       rgba += sum / total_samples, alpha += 1 (iterative.rs:45-51)
//   k_tonemap        post_process.glsl:23-49 + tonemapping.glsl:2-40; the legacy
//                    viewport's curves (voidray/src/shaders/viewport_fragment.glsl:27-67)
//   k_relmse         relative MSE reduction
//
// No tensor cores: traversal and shading are FP32 SIMT, bound by memory
// latency and bandwidth; BVH nodes and triangles are read as 128-bit
// read-only loads (ld.global.nc.v4.f32).
#include <cuda_runtime.h>

#include "vr_device.cuh"
#include "vr_kernels.h"
#include "vr_traverse.cuh"

namespace vr {

// ----------------------------------------------------------------------------
// Traversal
// ----------------------------------------------------------------------------
// vr_ray batch -> vr_hit batch
struct BatchIo {
    const float4* rays;
    float4* hits;
    const float4* nodes;
    const float4* tris;
    const float4* ana;  // analytic surfaces, tested after the BVH
    uint32_t nana, ntris;
    bool any;
    const uint32_t* perm;  // trace order (k_ray_scatter), or null: the caller's order
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd, const float4*& n, const float4*& t) const {
        if (perm) i = __ldg(perm + i);
        ro = __ldg(rays + 2 * (size_t)i);
        rd = __ldg(rays + 2 * (size_t)i + 1);
        n = nodes;
        t = tris;
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        if (perm) i = __ldg(perm + i);
        HitOut o = h;
        if (overflow) o.prim = MISS;
        if (nana && !overflow && !(any && o.prim != MISS)) {
            const float4 ro = __ldg(rays + 2 * (size_t)i), rd = __ldg(rays + 2 * (size_t)i + 1);
            float tb = o.prim == MISS ? INF_F : o.t;
            uint32_t pb = o.prim;
            analytic_closest(ana, nana, ntris, xyz(ro), xyz(rd), ro.w, rd.w, tb, pb);
            if (pb != o.prim) {
                o.prim = pb;
                o.t = tb;
                o.u = o.v = 0.0f;
            }
        }
        hits[i] = pack_hit(o);
    }
};

// Trace order of a batch query: rays grouped by direction octant and by a
// cell of their origin (3 bits per axis, Morton order) in the scene's bounds,
// so that a warp's rays start near each other heading into one octant.  A
// counting sort over the 4096 keys: per-block histograms, one scan, a scatter
// with warp-aggregated cursors.
constexpr uint32_t RAY_BINS = RAY_SORT_BINS;
__device__ __forceinline__ uint32_t ray_key(float4 ro, float4 rd, float3 lo, float3 sc) {
    auto cell = [](float v, float l, float s) { return (uint32_t)fminf(fmaxf((v - l) * s, 0.0f), 7.0f); };
    const uint32_t cx = cell(ro.x, lo.x, sc.x), cy = cell(ro.y, lo.y, sc.y), cz = cell(ro.z, lo.z, sc.z);
    uint32_t m = 0;
    for (int b = 0; b < 3; ++b)
        m |= (((cx >> b) & 1u) << (3 * b)) | (((cy >> b) & 1u) << (3 * b + 1)) | (((cz >> b) & 1u) << (3 * b + 2));
    const uint32_t oct = (rd.x < 0.0f ? 1u : 0u) | (rd.y < 0.0f ? 2u : 0u) | (rd.z < 0.0f ? 4u : 0u);
    return (oct << 9) | m;
}
__global__ void k_ray_hist(const float4* __restrict__ rays, uint32_t n, float3 lo, float3 sc, uint32_t* keys,
                           uint32_t* hist) {
    __shared__ uint32_t h[RAY_BINS];
    for (uint32_t t = threadIdx.x; t < RAY_BINS; t += blockDim.x) h[t] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t k = ray_key(__ldg(rays + 2 * (size_t)i), __ldg(rays + 2 * (size_t)i + 1), lo, sc);
        keys[i] = k;
        atomicAdd(&h[k], 1u);
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < RAY_BINS; t += blockDim.x)
        if (h[t]) atomicAdd(&hist[t], h[t]);
}
// exclusive prefix of the 4096 counts, in place (one block of 1024 threads)
__global__ void __launch_bounds__(1024) k_ray_scan(uint32_t* hist) {
    __shared__ uint32_t wsum[32];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; ++k) {
        v[k] = hist[4 * t + k];
        s += v[k];
    }
    uint32_t x = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    uint32_t base = x - s + (warp ? wsum[warp - 1] : 0u);
    for (int k = 0; k < 4; ++k) {
        hist[4 * t + k] = base;
        base += v[k];
    }
}
__global__ void k_ray_scatter(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* cursor, uint32_t* perm) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {  // warp-uniform trip count
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < n;
        const uint32_t k = valid ? keys[i] : 0xffffffffu;
        const uint32_t grp = __match_any_sync(0xffffffffu, k);
        const uint32_t leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&cursor[k], (uint32_t)__popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) perm[base + __popc(grp & ((1u << lane) - 1u))] = i;
    }
}

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128, VR_ISECT_MINB) k_intersect(BatchIo io, uint32_t n, uint32_t* counter,
                                                                  uint32_t* status, unsigned long long* work) {
    persistent_trace<ANY, COUNT, BatchIo, true>(n, counter, io, status, work);
}

// ----------------------------------------------------------------------------
// Environment (voidray_common/src/environments.rs:19-90) and its importance
// sampling (extension)
// ----------------------------------------------------------------------------
__device__ __forceinline__ size_t sat_usize(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 1.8446744e19f) return ~(size_t)0;
    return (size_t)x;
}
__device__ __forceinline__ V3 env_px(const float* img, size_t i) {
    return v3(__ldg(img + 3 * i), __ldg(img + 3 * i + 1), __ldg(img + 3 * i + 2));
}
// i % len for i <= 2 len: the linear index of a bilinear neighbour of a texel
// (x0 < W, y0 < H) wraps at most twice, so two conditional subtractions give
// the reference's modulo without a 64-bit division.
__device__ __forceinline__ size_t wrap_index(size_t i, size_t len) {
    if (i >= len) i -= len;
    if (i >= len) i -= len;
    return i;
}
__device__ V3 env_eval(const SceneView& s, V3 dir) {
    if (s.env_kind == 1) return load3(s.env_color);
    if (s.env_kind != 2) return v3(0.0f, 0.0f, 0.0f);
    V3 d = normalize(dir);
    float sx = acosf(-d.y);
    float sy = atan2f(-d.z, d.x) + PI_F;
    float u = sx / PI_F;
    float vv = sy / (2.0f * PI_F);
    float x = vv * (float)s.env_w;
    float y = (float)(s.env_h - 1) - (u * (float)s.env_h);
    size_t W = s.env_w, H = s.env_h, len = W * H;
    size_t x0 = min(sat_usize(x), W - 1);
    size_t y0 = min(sat_usize(y), H - 1);
    float ax = x - (float)x0;
    float ay = y - (float)y0;
    const float* img = s.env_img;
    const size_t i0 = y0 * W + x0;  // < len
    return lerp3(lerp3(env_px(img, i0), env_px(img, wrap_index(i0 + 1, len)), ax),
                 lerp3(env_px(img, wrap_index(i0 + W, len)), env_px(img, wrap_index(i0 + W + 1, len)), ax), ay);
}
// Largest i < n with cdf[i] <= u (cdf[0] = 0 <= u): a binary search of the
// non-decreasing CDF, started from the guide table's bracket.  u in [0, 1)
// and m a power of two make k / m <= u < (k + 1) / m exact, and the result
// for u lies between the results for k / m and (k + 1) / m, which the guide
// holds; so the search returns exactly what a search of all of [0, n) does.
__device__ __forceinline__ uint32_t cdf_find(const float* cdf, uint32_t n, const uint32_t* guide, uint32_t m,
                                             float u) {
    uint32_t k = (uint32_t)(u * (float)m);
    if (k >= m) k = m - 1;
    uint32_t lo = __ldg(guide + k), hi = min(__ldg(guide + k + 1) + 1u, n);
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) <= u) lo = mid; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ V3 dir_from_angles(float st, float ct, float phi) {
    return v3(-st * cosf(phi), -ct, st * sinf(phi));
}
__device__ __forceinline__ float cell_density(const SceneView& s, uint32_t j, uint32_t i, float st) {
    return __ldg(s.env_cell + (size_t)j * s.env_w + i) * s.env_density_scale / st;
}
__device__ bool env_sample(const SceneView& s, float u1, float u2, float u3, float u4, V3* dir, float* pdf) {
    uint32_t j = cdf_find(s.env_marg, s.env_h, s.env_gmarg, s.env_gm, u1);
    uint32_t i = cdf_find(s.env_cond + (size_t)j * (s.env_w + 1), s.env_w, s.env_gcond + (size_t)j * (s.env_gc + 1),
                          s.env_gc, u2);
    float theta = ((float)j + u3) * (PI_F / (float)s.env_h);
    float phi = ((float)i + u4) * (2.0f * PI_F / (float)s.env_w);
    float st = sinf(theta), ct = cosf(theta);
    if (!(st > 0.0f)) return false;
    *dir = dir_from_angles(st, ct, phi);
    *pdf = cell_density(s, j, i, st);
    return *pdf > 0.0f;
}
__device__ float env_pdf(const SceneView& s, V3 d) {
    float theta = acosf(-d.y);
    float phi = atan2f(-d.z, d.x) + PI_F;
    float fj = theta * ((float)s.env_h / PI_F);
    float fi = phi * ((float)s.env_w / (2.0f * PI_F));
    uint32_t j = (uint32_t)fminf(fmaxf(fj, 0.0f), (float)(s.env_h - 1));
    uint32_t i = (uint32_t)fminf(fmaxf(fi, 0.0f), (float)(s.env_w - 1));
    float st = sinf(theta);
    if (!(st > 0.0f)) return 0.0f;
    return cell_density(s, j, i, st);
}

// ----------------------------------------------------------------------------
// Materials (voidray_common/src/simple.rs, microfacet.rs; core/traits.rs:19-41)
// ----------------------------------------------------------------------------
struct SurfHit {
    V3 point, normal;
    V3 snormal;  // normal the Lambertian scatter uses (the normal map's raw RGB when there is one)
    float t;
    bool front;
};

__device__ __forceinline__ bool is_normal_f(float x) {  // f32::is_normal: exponent neither 0 nor 255
    const uint32_t e = (__float_as_uint(x) >> 23) & 0xffu;
    return e != 0u && e != 0xffu;
}
__device__ __forceinline__ V3 local_to_world_mul(V3 n, V3 h) {  // math.rs:50-60 (rows ns, nss, n)
    V3 ns = is_normal_f(n.x) ? normalize(v3(n.y, -n.x, 0.0f)) : normalize(v3(0.0f, -n.z, n.y));
    V3 nss = cross(n, ns);
    return v3(dot(ns, h), dot(nss, h), dot(n, h));
}
// ImageTexture::sample (texture.rs:82-98): u, v wrapped into [0, 1) the
// reference's way, then nearest_sample (:52-57) or bilinear_sample (:59-78),
// both with the linear-index modulo at the edges.
__device__ V3 tex_sample(const SceneView& s, int32_t tix, float u, float v) {
    const int4 ti = __ldg(s.tex_info + tix);
    const size_t W = (uint32_t)ti.y, H = (uint32_t)ti.z, len = W * H;
    const float* img = s.texels + ti.x;
    if (u < 0.0f) u -= truncf(u) - 1.0f;
    if (v < 0.0f) v -= truncf(v) - 1.0f;
    const float x = fmodf(u, 1.0f) * (float)W;
    const float y = (1.0f - fmodf(v, 1.0f)) * (float)H;
    const size_t x0 = min(sat_usize(x), W - 1), y0 = min(sat_usize(y), H - 1);
    const size_t i0 = y0 * W + x0;  // < len
    if (ti.w == 0) return env_px(img, i0);
    const float ax = x - (float)x0, ay = y - (float)y0;
    return lerp3(lerp3(env_px(img, i0), env_px(img, wrap_index(i0 + 1, len)), ax),
                 lerp3(env_px(img, wrap_index(i0 + W, len)), env_px(img, wrap_index(i0 + W + 1, len)), ax), ay);
}

// MixMaterial::scatter (legacy voidray/src/common/materials.rs:195-203): one
// uniform draw per level picks the child that shades this hit; the scene
// builder guarantees every chain ends within MAX_MIX_DEPTH levels.
__device__ __forceinline__ void resolve_mix(const SceneView& s, Material& m, Rng& rng) {
#pragma unroll 1
    for (int d = 0; m.kind == M_MIX && d < MAX_MIX_DEPTH; ++d) {
        const float u = rng.uniform();
        m = s.materials[u >= m.mix_factor ? m.mix_first : m.mix_second];
    }
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float signum_f(float x) {
    if (isnan(x)) return x;
    return signbit(x) ? -1.0f : 1.0f;
}

__device__ V3 micro_bsdf(const Material& m, V3 n, V3 wo, V3 wi) {
    V3 color = load3(m.color);
    float n_dot_wi = dot(n, wi), n_dot_wo = dot(n, wo);
    bool wi_out = !signbit(n_dot_wi), wo_out = !signbit(n_dot_wo);
    if (!m.transparent && (!wi_out || !wo_out)) return v3(0.0f, 0.0f, 0.0f);
    float m2 = m.roughness * m.roughness;
    if (wi_out == wo_out) {
        V3 h = normalize(wi + wo);
        float wo_dot_h = dot(wo, h), n_dot_h = dot(n, h), nh2 = powi2(n_dot_h);
        float dd = expf((nh2 - 1.0f) / (m2 * nh2)) / (m2 * PI_F * nh2 * nh2);
        V3 f;
        if (!wi_out && sqrtf(1.0f - wo_dot_h * wo_dot_h) * m.ir > 1.0f) {
            f = v3(1.0f, 1.0f, 1.0f);
        } else {
            float f0s = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
            V3 f0 = lerp3(v3(f0s, f0s, f0s), color, m.metallic);
            f = f0 + (v3(1.0f, 1.0f, 1.0f) - f0) * powi5(1.0f - wo_dot_h);
        }
        float g = fminf(n_dot_wi * n_dot_h, n_dot_wo * n_dot_h);
        g = (2.0f * g) / wo_dot_h;
        g = fminf(g, 1.0f);
        V3 spec = dd * f * g / (4.0f * n_dot_wo * n_dot_wi);
        if (m.transparent) return spec;
        V3 diffuse = vmul(v3(1.0f, 1.0f, 1.0f) - f, color) / PI_F;
        return spec + diffuse;
    }
    float eta_t = wo_out ? m.ir : 1.0f / m.ir;
    V3 h = normalize(wi * eta_t + wo);
    float wi_dot_h = dot(wi, h), wo_dot_h = dot(wo, h), n_dot_h = dot(n, h), nh2 = powi2(n_dot_h);
    float dd = expf((nh2 - 1.0f) / (m2 * nh2)) / (m2 * PI_F * nh2 * nh2);
    float f0s = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
    V3 f0 = lerp3(v3(f0s, f0s, f0s), color, m.metallic);
    V3 f = f0 + (v3(1.0f, 1.0f, 1.0f) - f0) * powi5(1.0f - fabsf(wi_dot_h));
    float g = fminf(fabsf(n_dot_wi * n_dot_h), fabsf(n_dot_wo * n_dot_h));
    g = (2.0f * g) / fabsf(wo_dot_h);
    g = fminf(g, 1.0f);
    float lead = fabsf(wi_dot_h * wo_dot_h / (n_dot_wi * n_dot_wo));
    V3 btdf = lead * (dd * (v3(1.0f, 1.0f, 1.0f) - f) * g / powi2(eta_t * wi_dot_h + wo_dot_h));
    return vmul(btdf, color);
}

__device__ bool micro_sample(const Material& m, V3 n, V3 wo, Rng& rng, V3* wi_out, float* p_out) {
    V3 color = load3(m.color);
    float m2 = m.roughness * m.roughness;
    float f0 = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
    float mean = (color.x + color.y + color.z) / 3.0f;
    float f = (1.0f - m.metallic) * f0 + m.metallic * mean;
    f = lerpf(f, 1.0f, 0.2f);
    float eta_t = dot(wo, n) > 0.0f ? m.ir : 1.0f / m.ir;
    V3 wi;
    if (rng.uniform() < f) {
        float theta = atanf(sqrtf(m2 * -logf(rng.uniform())));
        float st = sinf(theta), ct = cosf(theta);
        float x, y;
        unit_circle(rng, &x, &y);
        V3 h = local_to_world_mul(n, v3(x * st, y * st, ct));
        wi = -reflect(wo, h);
    } else if (!m.transparent) {
        float x, y;
        unit_disc(rng, &x, &y);
        float z = sqrtf(1.0f - x * x - y * y);
        wi = local_to_world_mul(n, v3(x, y, z));
    } else {
        float theta = atanf(sqrtf(m2 * -logf(rng.uniform())));
        float st = sinf(theta), ct = cosf(theta);
        float x, y;
        unit_circle(rng, &x, &y);
        V3 h = local_to_world_mul(n, v3(x * st, y * st, ct));
        float cos_to = dot(h, wo);
        V3 wo_perp = wo - h * cos_to;
        V3 wi_perp = -wo_perp / eta_t;
        float sin2_ti = mag2(wi_perp);
        if (sin2_ti > 1.0f) return false;
        float cos_ti = sqrtf(1.0f - sin2_ti);
        wi = -signum_f(cos_to) * cos_ti * h + wi_perp;
    }
    auto beckmann_pdf = [&](V3 h) {
        float ct = fabsf(dot(h, n));
        float st = sqrtf(1.0f - ct * ct);
        return (1.0f / (PI_F * m2 * powi3(ct))) * expf(-powi2(st / ct) / m2);
    };
    float p = 0.0f;
    {
        V3 h = normalize(wi + wo);
        float p_h = beckmann_pdf(h);
        p += f * p_h / (4.0f * fabsf(dot(h, wo)));
    }
    if (!m.transparent) {
        p += (1.0f - f) * fmaxf(dot(wi, n), 0.0f) / PI_F;
    } else if (!signbit(dot(wo, n)) != !signbit(dot(wi, n))) {
        V3 h = normalize(wi * eta_t + wo);
        float p_h = beckmann_pdf(h);
        float h_dot_wo = dot(h, wo), h_dot_wi = dot(h, wi);
        float jac = fabsf(h_dot_wo) / powi2(eta_t * h_dot_wi + h_dot_wo);
        p += (1.0f - f) * p_h * jac;
    }
    if (p == 0.0f) return false;
    *wi_out = wi;
    *p_out = p;
    return true;
}

// Material::scatter; returns true when a continuation ray is produced.
__device__ bool scatter(const Material& m, V3 ro, V3 rd, const SurfHit& hit, Rng& rng, V3* att, V3* out_dir) {
    switch (m.kind) {
    case M_LAMB: {
        V3 dir = hit.snormal + unit_sphere(rng);
        if (near_zero(dir)) dir = hit.snormal;
        *out_dir = normalize(dir);
        *att = load3(m.color);
        return true;
    }
    case M_METAL: {
        V3 reflected = normalize(reflect(rd, hit.normal));
        for (int i = 0; i < REJECT_TRIES; ++i) {
            V3 d = normalize(reflected + m.fuzz * unit_sphere(rng));
            if (dot(d, hit.normal) > 0.0f) {
                *out_dir = d;
                *att = load3(m.color);
                return true;
            }
        }
        *att = v3(0.0f, 0.0f, 0.0f);
        return false;
    }
    case M_DIEL: {
        float rr = hit.front ? 1.0f / m.ir : m.ir;
        V3 ud = normalize(rd);
        float cos_t = fminf(dot(hit.normal, -ud), 1.0f);
        float sin_t = sqrtf(1.0f - cos_t * cos_t);
        bool cannot = (rr * sin_t) > 1.0f;
        V3 dir;
        if (cannot) {
            dir = reflect(ud, hit.normal);
        } else {
            float r0 = (1.0f - rr) / (1.0f + rr);
            r0 = r0 * r0;
            float refl = r0 + (1.0f - r0) * powi5(1.0f - cos_t);
            if (refl > rng.range(0.0f, 1.0f)) dir = reflect(ud, hit.normal);
            else dir = refract(ud, hit.normal, rr);
        }
        *out_dir = normalize(dir);
        *att = v3(1.0f, 1.0f, 1.0f);
        return true;
    }
    case M_EMIT:
        *att = load3(m.color);
        return false;
    case M_LBSDF: {
        V3 wi = normalize(unit_sphere(rng));
        V3 f = load3(m.color) / PI_F;
        *out_dir = normalize(wi);
        *att = f * fabsf(dot(wi, hit.normal)) * (1.0f / 1.0f);
        return true;
    }
    case M_MICRO: {
        V3 wo = normalize(rd);
        V3 wi;
        float pdf;
        if (micro_sample(m, hit.normal, wo, rng, &wi, &pdf)) {
            V3 f = micro_bsdf(m, hit.normal, wo, wi);
            *out_dir = normalize(wi);
            *att = f * fabsf(dot(wi, hit.normal)) * (1.0f / pdf);
            return true;
        }
        *att = v3(0.0f, 0.0f, 0.0f);
        return false;
    }
    }
    *att = v3(0.0f, 0.0f, 0.0f);
    return false;
}

// ----------------------------------------------------------------------------
// Wavefront stages
// ----------------------------------------------------------------------------
// ----------------------------------------------------------------------------
// Jobs.  A wavefront holds the paths of one or more render jobs (scenes with
// their own settings, image and sample range).  Job r owns the slots
// [base, base + paths) of every per-path array and of each ray queue half;
// its queue sizes live in its own counters, counts[r * JOB_COUNTERS + ...].
// Path slot p of job r is its global sample-major path g = g0 + (p - base):
// pixel = g % num_pixels, sample = first_sample + g / num_pixels.
// ----------------------------------------------------------------------------
// Tiled pixel order: rows of 8x8 tiles, row-major inside a tile (the last
// tile row and column may be narrower); a bijection of [0, W*H).
constexpr uint32_t PIX_TILE = 8;
__device__ __forceinline__ uint32_t tiled_index(uint32_t x, uint32_t y, uint32_t W, uint32_t H) {
    const uint32_t R = y / PIX_TILE, th = min(PIX_TILE, H - R * PIX_TILE);
    const uint32_t b = x / PIX_TILE, bw = min(PIX_TILE, W - b * PIX_TILE);
    return R * PIX_TILE * W + b * PIX_TILE * th + (y - R * PIX_TILE) * bw + (x - b * PIX_TILE);
}
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t P, uint32_t W, uint32_t H) {
    const uint32_t R = P / (PIX_TILE * W), rem = P - R * PIX_TILE * W;
    const uint32_t th = min(PIX_TILE, H - R * PIX_TILE);
    const uint32_t b = rem / (PIX_TILE * th), rem2 = rem - b * PIX_TILE * th;
    const uint32_t bw = min(PIX_TILE, W - b * PIX_TILE);
    const uint32_t yy = rem2 / bw;
    return (R * PIX_TILE + yy) * W + b * PIX_TILE + (rem2 - yy * bw);
}

// (pixel, sample) of the path in slot p (see Job::head for the slot order).
__device__ __forceinline__ void path_coords(const Job& j, uint32_t p, uint32_t& pixel, uint32_t& sample) {
    const uint32_t o = p - j.base;
    if (o >= j.head && o - j.head < j.rows * j.num_pixels) {
        const uint32_t om = o - j.head;
        const uint32_t P = om / j.rows;
        pixel = tiled_pixel(P, j.width, j.height);
        sample = j.first_sample + j.row0 + (om - P * j.rows);
        return;
    }
    const uint64_t g = j.g0 + o;
    pixel = (uint32_t)(g % j.num_pixels);
    sample = j.first_sample + (uint32_t)(g / j.num_pixels);
}

// Block-wide exclusive prefix over the jobs of one per-job counter into
// shared memory: pre[r] = sum of counter over jobs < r, pre[njobs] = total.
__device__ __forceinline__ void job_prefix(const uint32_t* counts, uint32_t which, uint32_t njobs, uint32_t* pre) {
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        uint32_t carry = 0;
        for (uint32_t r0 = 0; r0 < njobs; r0 += 32) {
            const uint32_t r = r0 + lane;
            const uint32_t v = (r < njobs) ? counts[r * JOB_COUNTERS + which] : 0u;
            uint32_t x = v;
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
                if (lane >= (uint32_t)off) x += y;
            }
            if (r < njobs) pre[r] = carry + x - v;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) pre[njobs] = carry;
    }
    __syncthreads();
}

// Largest r with pre[r] <= i.
__device__ __forceinline__ uint32_t find_job(const uint32_t* pre, uint32_t njobs, uint32_t i) {
    uint32_t lo = 0, hi = njobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pre[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// A wave of at most STAGED_JOBS jobs has its job table copied to shared
// memory by every block of a kernel that reads it per ray or path (the copy
// is uniform across the block); larger waves read the table in global memory.
constexpr uint32_t STAGED_JOBS = 8;
__device__ __forceinline__ const Job* stage_jobs(const Wave& w, Job* sj) {
    if (w.njobs > STAGED_JOBS) return w.jobs;
    const uint32_t words = w.njobs * (uint32_t)(sizeof(Job) / 4);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(w.jobs);
    uint32_t* dst = reinterpret_cast<uint32_t*>(sj);
    for (uint32_t t = threadIdx.x; t < words; t += blockDim.x) dst[t] = src[t];
    __syncthreads();
    return sj;
}

// Clears the wave's counters and fetch cursors; depth-0 queue size = paths.
__global__ void k_wave_begin(Wave w, PathState ps) {
    const uint32_t n = w.njobs * JOB_COUNTERS;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = i / JOB_COUNTERS, c = i % JOB_COUNTERS;
        ps.counts[i] = (c == 0) ? w.jobs[r].paths : 0u;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * MAX_DEPTH_SLOTS; i += gridDim.x * blockDim.x)
        ps.cursors[i] = 0u;
}

// ONE: a single-job wave, whose job is read from the kernel parameters.
template <bool ONE>
__global__ void k_raygen(Wave w, PathState ps) {
    __shared__ uint32_t pre[MAX_JOBS + 1];
    __shared__ Job sj[ONE ? 1 : STAGED_JOBS];
    const Job* jobs = w.jobs;
    if (!ONE) {
        if (threadIdx.x == 0)
            for (uint32_t r = 0; r <= w.njobs; ++r) pre[r] = (r < w.njobs) ? w.jobs[r].base : w.total_paths;
        __syncthreads();
        jobs = stage_jobs(w, sj);
    }
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < w.total_paths; p += stride) {
        const uint32_t r = ONE ? 0u : find_job(pre, w.njobs, p);
        const Job& j = ONE ? w.first : jobs[r];
        const SceneView& s = j.view;
        uint32_t pixel, sample;
        path_coords(j, p, pixel, sample);
        // iterative.rs:25-40 (row = pixel / width)
        const uint32_t W = j.width, H = j.height;
        const uint32_t x = pixel % W, y = pixel / W;
        const float dmax = (float)max(W, H);
        const float fx = ((float)(2 * x + 1) - (float)W) / dmax;
        const float fy = ((float)(2 * (H - y) - 1) - (float)H) / dmax;
        Rng rng;
        rng.inc = pcg_inc(sample, pixel);
        rng.state = pcg_init(j.seed, rng.inc);
        const float lo = -1.0f / dmax, hi = 1.0f / dmax;
        const float jx = rng.range(lo, hi);
        const float jy = rng.range(lo, hi);
        const float cx = fx + jx, cy = fy + jy;
        // cast_ray (camera.rs:69-82)
        V3 origin = load3(s.c_origin);
        V3 nd = s.c_d * load3(s.c_dir) + cx * load3(s.c_right) + cy * load3(s.c_up);
        if (s.c_dof) {
            V3 focal_point = origin + normalize(nd) * s.c_focal;
            float dx, dy;
            unit_disc(rng, &dx, &dy);
            origin = origin + (dx * load3(s.c_right) + dy * load3(s.c_up)) * s.c_aperture;
            nd = focal_point - origin;
        }
        V3 dir = normalize(normalize(nd));
        ps.q_org[p] = make_float4(origin.x, origin.y, origin.z, SCENE_TMIN);
        ps.q_dir[p] = make_float4(dir.x, dir.y, dir.z, INF_F);
        ps.q_path[p] = p;
        ps.rng[p] = rng.state;
        ps.thr[p] = make_float4(1.0f, 1.0f, 1.0f, -1.0f);
        ps.rad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Closest hit of every job's live queue of depth k (persistent, dynamic fetch).
// Concatenated index i -> job r, entry l = i - pre[r] of r's queue segment.
template <bool ONE>
struct ExtendIo {
    const float4* org;  // queue half of depth k
    const float4* dir;
    float4* hits;
    const Job* jobs;
    const uint32_t* pre;
    uint32_t njobs;
    const float4* nodes1;  // ONE: the single job's BVH
    const float4* tris1;
    __device__ __forceinline__ uint32_t slot(uint32_t i, uint32_t& r) const {
        if (ONE) {  // a single job's segment starts at slot 0
            r = 0;
            return i;
        }
        r = find_job(pre, njobs, i);
        return jobs[r].base + (i - pre[r]);
    }
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd, const float4*& n, const float4*& t) const {
        uint32_t r;
        const uint32_t q = slot(i, r);
        ro = org[q];
        rd = dir[q];
        n = ONE ? nodes1 : jobs[r].view.nodes;
        t = ONE ? tris1 : jobs[r].view.tris;
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        uint32_t r;
        const uint32_t q = slot(i, r);
        HitOut o = h;
        if (overflow) o.prim = MISS;
        hits[q] = pack_hit(o);  // analytic surfaces are tested by k_shade
    }
};

template <bool COUNT, bool ONE>
__global__ void __launch_bounds__(128, VR_TRACE_MINB) k_extend(Wave w, PathState ps, uint32_t k, uint32_t* status,
                                                               unsigned long long* work) {
    __shared__ uint32_t pre[MAX_JOBS + 1];
    uint32_t n;
    if (ONE) {
        n = ps.counts[k];
    } else {
        job_prefix(ps.counts, k, w.njobs, pre);
        n = pre[w.njobs];
    }
    __shared__ Job sj[ONE ? 1 : STAGED_JOBS];
    const uint32_t half = (k & 1) ? ps.cap : 0;
    if (!ONE && w.njobs <= STAGED_JOBS) {  // a separate inlined copy that reads the jobs from shared memory
        stage_jobs(w, sj);
        ExtendIo<ONE> io{ps.q_org + half, ps.q_dir + half, ps.hits, sj, pre, w.njobs, w.first.view.nodes,
                         w.first.view.tris};
        persistent_trace<false, COUNT>(n, &ps.cursors[k], io, status, work);
    } else {
        ExtendIo<ONE> io{ps.q_org + half, ps.q_dir + half, ps.hits, w.jobs, pre, w.njobs, w.first.view.nodes,
                         w.first.view.tris};
        persistent_trace<false, COUNT>(n, &ps.cursors[k], io, status, work);
    }
}

// Reference estimator: the path's radiance is the recursion of
// trace_ray_internal unwound from its leaf: L = leaf; L = min(att_d * L, clamp)
// for d = k-1 .. 0 (tracer.rs:44-50).
__device__ __forceinline__ void unwind(const PathState& ps, uint32_t p, uint32_t k, V3 leaf, float fc) {
    V3 L = leaf;
    for (int d = (int)k - 1; d >= 0; --d) {
        const float* a = ps.att + (size_t)d * 3 * ps.cap;
        V3 att = v3(a[p], a[ps.cap + p], a[2 * ps.cap + p]);
        L = clampc(vmul(att, L), fc);
    }
    ps.rad[p] = make_float4(L.x, L.y, L.z, 0.0f);
}

__device__ __forceinline__ void rad_add(const PathState& ps, uint32_t p, V3 c) {
    float4 r = ps.rad[p];
    ps.rad[p] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, r.w);
}

// Direction octant (sign bits of x, y, z).
__device__ __forceinline__ uint32_t octant(V3 d) {
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}
constexpr uint32_t BIN_JOBS = 8;  // jobs per shade block that are appended in (job, octant) runs

// Appends the active lanes with `want` to job r's queue segment: one atomic
// per group of lanes of the same job; returns this lane's slot in the segment.
__device__ __forceinline__ uint32_t queue_append(bool want, uint32_t r, uint32_t* counter_of_job, uint32_t lane) {
    const uint32_t active = __activemask();
    const uint32_t wm = __ballot_sync(active, want);
    uint32_t slot = 0;
    if (want) {
        const uint32_t grp = __match_any_sync(wm, r);
        const uint32_t leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(counter_of_job, __popc(grp));
        base = __shfl_sync(grp, base, leader);
        slot = base + __popc(grp & ((1u << lane) - 1u));
    }
    return slot;
}

// One live path at depth k: the hit's material (or the environment on a miss),
// next event estimation, the scatter and Russian roulette; returns the
// continuation and shadow rays to append.  `j` is the path's job, read from
// the kernel parameters, shared memory or the job table (the caller picks, so
// that each inlined copy loads from one known address space).
__device__ __forceinline__ void shade_path(const Job& j, const PathState& ps, uint32_t k, uint32_t in_half,
                                           uint32_t local, unsigned long long* retired, bool& cont,
                                           bool& want_shadow, V3& new_o, V3& new_d, V3& sh_dir, V3& sh_c,
                                           uint32_t& p) {
        const SceneView& s = j.view;
        const RenderParams& rp = j.rp;
        const float fc = rp.firefly_clamp;
        const bool nee_mode = rp.estimator == 1;
        const bool last = (k + 1 >= rp.max_bounces);
        const uint32_t q = in_half + j.base + local;
        p = ps.q_path[q];
        const float4 ro4 = ps.q_org[q], rd4 = ps.q_dir[q];
        const V3 ro = xyz(ro4), rd = xyz(rd4);
        float4 hh = ps.hits[q - in_half];
        uint32_t prim = __float_as_uint(hh.x);
        if (s.num_analytic) {  // SceneAcceleration::hit keeps the nearest surface, analytic ones included
            float tb = prim == MISS ? INF_F : hh.y;
            uint32_t pb = prim;
            analytic_closest(s.analytic, s.num_analytic, s.num_tris, ro, rd, ro4.w, rd4.w, tb, pb);
            if (pb != prim) {
                prim = pb;
                hh = make_float4(__uint_as_float(pb), tb, 0.0f, 0.0f);
            }
        }
        uint32_t pixel, sample;
        path_coords(j, p, pixel, sample);
        Rng rng;
        rng.inc = pcg_inc(sample, pixel);
        rng.state = ps.rng[p];
        const float4 thr4 = ps.thr[p];
        V3 T = xyz(thr4);
        float prev_pdf = thr4.w;
        if (prim == MISS) {
            const V3 le = env_eval(s, rd);
            if (k == 0 && j.aov_psum) {  // first-hit AOVs of a miss: environment (clamped), no normal
                ps.aov[p] = make_float4(fminf(le.x, 1.0f), fminf(le.y, 1.0f), fminf(le.z, 1.0f), 0.0f);
                ps.aov[ps.cap + p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            if (nee_mode) {
                float wgt = 1.0f;
                if (prev_pdf >= 0.0f && s.env_is) {
                    float pl = env_pdf(s, rd);
                    float a = prev_pdf * prev_pdf, b = pl * pl;
                    wgt = a / (a + b);
                }
                rad_add(ps, p, clampc(vmul(T, le) * wgt, fc));
            } else {
                unwind(ps, p, k, le, fc);
            }
        } else {
            const float t = hh.y;
            const V3 point = ro + rd * t;
            Material m;
            V3 normal;
            float uvx = 0.0f, uvy = 0.0f;  // HitRecord::uv
            if (prim < s.num_tris) {
                // shading record and normal (mesh.rs:176-188, ray.rs:34-49)
                const float4* sh = s.shade + 4 * (size_t)prim;
                const float4 s0 = __ldg(sh), s1 = __ldg(sh + 1), s2 = __ldg(sh + 2), s3 = __ldg(sh + 3);
                m = s.materials[__float_as_uint(s0.w)];
                const float u = hh.z, v = hh.w;
                const float wb = 1.0f - u - v;
                normal = u * xyz(s1) + v * xyz(s2) + wb * xyz(s0);
                const V3 fnm = xyz(s3);
                const float ang = acosf(dot(normal, fnm) / (sqrtf(mag2(normal)) * sqrtf(mag2(fnm))));
                if (ang > 30.0f * PI_F / 180.0f) normal = fnm;
                if (s.uvs && s.num_textures) {  // u v1.uv + v v2.uv + (1 - u - v) v0.uv (mesh.rs:177)
                    const float2 t0 = __ldg(s.uvs + 3 * (size_t)prim), t1 = __ldg(s.uvs + 3 * (size_t)prim + 1),
                                 t2 = __ldg(s.uvs + 3 * (size_t)prim + 2);
                    uvx = u * t1.x + v * t2.x + wb * t0.x;
                    uvy = u * t1.y + v * t2.y + wb * t0.y;
                }
            } else {
                // analytic surface: sphere normal (p - c) / r, uv 0; ground plane +y, uv (x, z)
                // (surfaces.rs:74-75, 98-102)
                const float4 a0 = __ldg(s.analytic + 2 * (size_t)(prim - s.num_tris));
                const float4 a1 = __ldg(s.analytic + 2 * (size_t)(prim - s.num_tris) + 1);
                m = s.materials[__float_as_uint(a1.y)];
                const bool sphere = __float_as_uint(a1.x) == A_SPHERE;
                normal = sphere ? (point - v3(a0.x, a0.y, a0.z)) / a0.w : v3(0.0f, 1.0f, 0.0f);
                if (!sphere) {
                    uvx = point.x;
                    uvy = point.z;
                }
            }
            resolve_mix(s, m, rng);
            SurfHit hit;
            hit.point = point;
            hit.t = t;
            hit.front = dot(rd, normal) < 0.0f;
            hit.normal = hit.front ? normal : -normal;
            hit.snormal = hit.normal;
            if (m.albedo_tex >= 0) {  // ColorType::Texture: the albedo is the texture at the hit's uv
                const V3 c = tex_sample(s, m.albedo_tex, uvx, uvy);
                m.color[0] = c.x;
                m.color[1] = c.y;
                m.color[2] = c.z;
            }
            if (m.normal_tex >= 0) hit.snormal = tex_sample(s, m.normal_tex, uvx, uvy);
            if (k == 0 && j.aov_psum) {  // first-hit AOVs: surface colour (1 for glass), shading normal
                const V3 al = (m.kind == M_DIEL) ? v3(1.0f, 1.0f, 1.0f)
                                                 : v3(fminf(m.color[0], 1.0f), fminf(m.color[1], 1.0f),
                                                      fminf(m.color[2], 1.0f));
                ps.aov[p] = make_float4(al.x, al.y, al.z, 0.0f);
                ps.aov[ps.cap + p] = make_float4(hit.normal.x, hit.normal.y, hit.normal.z, 0.0f);
            }
            if (rp.render_mode != 1) {
                const V3 nn = normalize(hit.normal);
                const V3 c = (0.5f * nn) + v3(1.0f, 1.0f, 1.0f) * 0.5f;
                if (nee_mode) rad_add(ps, p, clampc(vmul(T, c), fc));
                else unwind(ps, p, k, clampc(c, fc), fc);
            } else {
                // next event estimation at Lambertian vertices whose scatter is
                // cosine-distributed around the shading normal (not with a normal map)
                const bool lamb = (m.kind == M_LAMB) && m.normal_tex < 0 &&
                                  !(hit.normal.x == 0.0f && hit.normal.y == 0.0f && hit.normal.z == 0.0f);
                if (nee_mode && lamb && s.env_is) {
                    const float u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform(), u4 = rng.uniform();
                    V3 dl;
                    float pl;
                    if (env_sample(s, u1, u2, u3, u4, &dl, &pl)) {
                        const float cosl = dot(hit.normal, dl);
                        if (cosl > 0.0f) {
                            const float pb = cosl / PI_F;
                            const float a = pl * pl, b = pb * pb;
                            const float wgt = a / (a + b);
                            const float fscale = cosl / PI_F * wgt / pl;
                            sh_c = vmul(vmul(T, load3(m.color)), env_eval(s, dl)) * fscale;
                            sh_dir = dl;
                            want_shadow = true;
                        }
                    }
                }
                V3 att, nd;
                if (!scatter(m, ro, rd, hit, rng, &att, &nd)) {
                    // instrumented runs count the metal paths absorbed by the bounded rejection loop
                    if (retired && m.kind == M_METAL) atomicAdd(retired + 1, 1ull);
                    if (nee_mode) rad_add(ps, p, clampc(vmul(T, att), fc));
                    else unwind(ps, p, k, clampc(att, fc), fc);
                } else {
                    V3 tn = vmul(T, att);
                    if (nee_mode) prev_pdf = lamb ? dot(hit.normal, nd) / PI_F : -1.0f;
                    bool alive = true;
                    if (rp.rr_depth != 0 && k >= rp.rr_depth) {
                        const float qq = fminf(max3(tn), 0.95f);
                        const float ur = rng.uniform();
                        if (!(ur < qq)) {
                            alive = false;
                        } else {
                            att = att / qq;
                            tn = tn / qq;
                        }
                    }
                    if (!nee_mode) {
                        if (!alive || last) {
                            // continuation not traced: it contributes BLACK
                            const V3 lk = clampc(vmul(att, v3(0.0f, 0.0f, 0.0f)), fc);
                            unwind(ps, p, k, lk, fc);
                        } else {
                            float* a = ps.att + (size_t)k * 3 * ps.cap;
                            a[p] = att.x;
                            a[ps.cap + p] = att.y;
                            a[2 * ps.cap + p] = att.z;
                        }
                    }
                    if (alive && !last) {
                        cont = true;
                        new_o = hit.point;
                        new_d = nd;
                        ps.thr[p] = make_float4(tn.x, tn.y, tn.z, prev_pdf);
                    }
                }
                if (want_shadow) new_o = hit.point;
            }
        }
        ps.rng[p] = rng.state;
}

template <bool ONE>
__global__ void __launch_bounds__(256, 4) k_shade(Wave w, PathState ps, uint32_t k, unsigned long long* retired) {
    __shared__ uint32_t pre[MAX_JOBS + 1];
    uint32_t n;
    if (ONE) {
        if (threadIdx.x == 0) pre[0] = 0;
        __syncthreads();
        n = ps.counts[k];
    } else {
        job_prefix(ps.counts, k, w.njobs, pre);
        n = pre[w.njobs];
    }
    const uint32_t in_half = (k & 1) ? ps.cap : 0;
    const uint32_t out_half = (k & 1) ? 0 : ps.cap;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    // the jobs this block's entries belong to (a contiguous range: job
    // segments are concatenated); they are copied to shared memory, so that
    // every thread reads its job there instead of from the job table in
    // global memory
    __shared__ uint32_t s_rlo, s_nj;
    __shared__ Job s_jobs[ONE ? 1 : BIN_JOBS];
    const bool all_staged = !ONE && w.njobs <= BIN_JOBS;
    if (all_staged) {
        const uint32_t words = w.njobs * (uint32_t)(sizeof(Job) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(w.jobs);
        uint32_t* dst = reinterpret_cast<uint32_t*>(s_jobs);
        for (uint32_t t = threadIdx.x; t < words; t += blockDim.x) dst[t] = src[t];
        __syncthreads();
    }
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        if (threadIdx.x == 0) {
            const uint32_t last = min(i0 + blockDim.x, n) - 1u;
            const uint32_t rlo = ONE ? 0u : find_job(pre, w.njobs, i0);
            s_rlo = rlo;
            s_nj = (ONE ? 0u : find_job(pre, w.njobs, last)) - rlo + 1u;
        }
        __syncthreads();
        bool cont = false, want_shadow = false;
        V3 new_o, new_d, sh_dir, sh_c;
        uint32_t p = 0, r = 0;
        if (ONE) {
            if (i < n)
                shade_path(w.first, ps, k, in_half, i, retired, cont, want_shadow, new_o, new_d, sh_dir, sh_c, p);
        } else {
            // a wave of at most BIN_JOBS jobs was copied to shared memory
            // once; otherwise the block's jobs pass through shared memory
            // BIN_JOBS at a time (one round unless the block spans more jobs)
            if (i < n) r = find_job(pre, w.njobs, i);
            const uint32_t rend = s_rlo + s_nj;
            for (uint32_t c0 = all_staged ? 0u : s_rlo; c0 < rend; c0 += BIN_JOBS) {
                const uint32_t cn = all_staged ? w.njobs : min(BIN_JOBS, rend - c0);
                if (!all_staged) {
                    if (c0 != s_rlo) __syncthreads();  // the previous round's paths have read their jobs
                    const uint32_t words = cn * (uint32_t)(sizeof(Job) / 4);
                    const uint32_t* src = reinterpret_cast<const uint32_t*>(w.jobs + c0);
                    uint32_t* dst = reinterpret_cast<uint32_t*>(s_jobs);
                    for (uint32_t t = threadIdx.x; t < words; t += blockDim.x) dst[t] = src[t];
                    __syncthreads();
                }
                if (i < n && r >= c0 && r < c0 + cn)
                    shade_path(s_jobs[r - c0], ps, k, in_half, i - pre[r], retired, cont, want_shadow, new_o, new_d,
                               sh_dir, sh_c, p);
                if (all_staged) break;
            }
        }
        // queue conservation (instrumented runs): every path that does not
        // continue is retired here, exactly once
        if (retired) {
            const uint32_t gone = __ballot_sync(0xffffffffu, i < n && !cont);
            if (lane == 0 && gone) atomicAdd(retired, (unsigned long long)__popc(gone));
        }
        // Compaction into the job's next queue segment and shadow segment.  The
        // block appends its rays in runs of equal (job, direction octant): the
        // block covers a few neighbouring pixels (pixel-major slots), so a
        // warp of the next traversal gets rays from one small region heading
        // into one octant, which visit the same nodes in the same order.
        // Blocks spanning more than BIN_JOBS jobs append per warp instead.
        const uint32_t base_r = (ONE || i >= n) ? 0u : w.jobs[r].base;
        __shared__ uint32_t s_cnt[2][BIN_JOBS * 8];
        __shared__ uint32_t s_base[2][BIN_JOBS];
        for (uint32_t t = threadIdx.x; t < 2 * BIN_JOBS * 8; t += blockDim.x) (&s_cnt[0][0])[t] = 0u;
        __syncthreads();
        uint32_t cs = 0, ss = 0;
        if (s_nj <= BIN_JOBS) {
            const uint32_t jl = r - s_rlo;
            const uint32_t ke = jl * 8 + (cont ? octant(new_d) : 0u);
            const uint32_t ks = jl * 8 + (want_shadow ? octant(sh_dir) : 0u);
            if (cont) cs = atomicAdd(&s_cnt[0][ke], 1u);
            if (want_shadow) ss = atomicAdd(&s_cnt[1][ks], 1u);
            __syncthreads();
            const uint32_t nj = s_nj;
            if (threadIdx.x < 2 * nj) {  // one thread per (queue, job): bin offsets and one global atomic
                const uint32_t qsel = threadIdx.x / nj, jj = threadIdx.x - qsel * nj;
                uint32_t* c = &s_cnt[qsel][jj * 8];
                uint32_t tot = 0;
                for (int b = 0; b < 8; ++b) {
                    const uint32_t v = c[b];
                    c[b] = tot;
                    tot += v;
                }
                const uint32_t ctr = (s_rlo + jj) * JOB_COUNTERS + (qsel ? MAX_DEPTH_SLOTS + k : k + 1);
                s_base[qsel][jj] = tot ? atomicAdd(&ps.counts[ctr], tot) : 0u;
            }
            __syncthreads();
            if (cont) cs += s_base[0][jl] + s_cnt[0][ke];
            if (want_shadow) ss += s_base[1][jl] + s_cnt[1][ks];
        } else {
            cs = queue_append(cont, r, &ps.counts[r * JOB_COUNTERS + k + 1], lane);
            ss = queue_append(want_shadow, r, &ps.counts[r * JOB_COUNTERS + MAX_DEPTH_SLOTS + k], lane);
        }
        __syncthreads();  // s_cnt is cleared again by the next iteration
        if (cont) {
            const uint32_t q = out_half + base_r + cs;
            ps.q_org[q] = make_float4(new_o.x, new_o.y, new_o.z, SCENE_TMIN);
            ps.q_dir[q] = make_float4(new_d.x, new_d.y, new_d.z, INF_F);
            ps.q_path[q] = p;
        }
        if (want_shadow) {
            const uint32_t q = base_r + ss;
            ps.s_org[q] = make_float4(new_o.x, new_o.y, new_o.z, SCENE_TMIN);
            ps.s_dir[q] = make_float4(sh_dir.x, sh_dir.y, sh_dir.z, INF_F);
            ps.s_path[q] = p;
            ps.s_contrib[q] = make_float4(sh_c.x, sh_c.y, sh_c.z, 0.0f);
        }
    }
}

// NEE visibility: adds the (clamped) contribution when nothing is hit
// (persistent any-hit traversal).  A stack overflow counts as occluded.
template <bool ONE>
struct ShadowIo {
    PathState ps;
    const Job* jobs;
    const uint32_t* pre;
    uint32_t njobs;
    const float4* nodes1;  // ONE: the single job's BVH, clamp and analytic surfaces
    const float4* tris1;
    float fc1;
    const float4* ana1;
    uint32_t nana1;
    __device__ __forceinline__ uint32_t slot(uint32_t i, uint32_t& r) const {
        if (ONE) {
            r = 0;
            return i;
        }
        r = find_job(pre, njobs, i);
        return jobs[r].base + (i - pre[r]);
    }
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd, const float4*& n, const float4*& t) const {
        uint32_t r;
        const uint32_t q = slot(i, r);
        ro = ps.s_org[q];
        rd = ps.s_dir[q];
        n = ONE ? nodes1 : jobs[r].view.nodes;
        t = ONE ? tris1 : jobs[r].view.tris;
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        uint32_t r;
        const uint32_t q = slot(i, r);
        if (overflow || h.prim != MISS) return;
        const uint32_t nana = ONE ? nana1 : jobs[r].view.num_analytic;
        if (nana) {  // an analytic surface in the way also occludes
            const float4 ro = ps.s_org[q], rd = ps.s_dir[q];
            if (analytic_any(ONE ? ana1 : jobs[r].view.analytic, nana, xyz(ro), xyz(rd), ro.w, rd.w)) return;
        }
        rad_add(ps, ps.s_path[q], clampc(xyz(ps.s_contrib[q]), ONE ? fc1 : jobs[r].rp.firefly_clamp));
    }
};

template <bool COUNT, bool ONE>
__global__ void __launch_bounds__(128, VR_SHADOW_MINB) k_shadow(Wave w, PathState ps, uint32_t k, uint32_t* status,
                                                               unsigned long long* work) {
    __shared__ uint32_t pre[MAX_JOBS + 1];
    uint32_t n;
    if (ONE) {
        n = ps.counts[MAX_DEPTH_SLOTS + k];
    } else {
        job_prefix(ps.counts, MAX_DEPTH_SLOTS + k, w.njobs, pre);
        n = pre[w.njobs];
    }
    __shared__ Job sj[ONE ? 1 : STAGED_JOBS];
    const bool staged = !ONE && w.njobs <= STAGED_JOBS;
    if (staged) stage_jobs(w, sj);
    auto run = [&](const Job* jobs) {
        ShadowIo<ONE> io{ps,
                         jobs,
                         pre,
                         w.njobs,
                         w.first.view.nodes,
                         w.first.view.tris,
                         w.first.rp.firefly_clamp,
                         w.first.view.analytic,
                         w.first.view.num_analytic};
        persistent_trace<true, COUNT>(n, &ps.cursors[MAX_DEPTH_SLOTS + k], io, status, work);
    };
    if (staged) run(sj);  // a separate inlined copy that reads the jobs from shared memory
    else run(w.jobs);
}

// Per-pixel running sum, in sample order, of each job's paths of this wave
// (blockIdx.y = job).
template <bool ONE>
__global__ void k_accumulate(Wave w, PathState ps) {
    const Job& j = ONE ? w.first : w.jobs[blockIdx.y];
    const uint32_t NP = j.num_pixels;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t mid = j.rows * NP;
    for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < NP; px += stride) {
        // global indices g = s*NP + px inside [g0, g0 + paths), s in [s_begin, s_end)
        const uint64_t g0 = j.g0, g1 = j.g0 + j.paths;
        const uint64_t s_begin = (g0 > px) ? (g0 - px + NP - 1) / NP : 0;
        const uint64_t s_end = (g1 > px) ? (g1 - px + NP - 1) / NP : 0;
        if (s_begin >= s_end) continue;
        const uint32_t tp = j.rows ? tiled_index(px % j.width, px / j.width, j.width, j.height) : 0u;
        // slot of sample row s of this pixel (Job::head)
        auto slot = [&](uint64_t s) -> uint32_t {
            const uint32_t o = (uint32_t)(s * NP + px - g0);
            return j.base + ((o >= j.head && o - j.head < mid) ? j.head + tp * j.rows + (uint32_t)(s - j.row0) : o);
        };
        float4 acc = j.psum[px];
        for (uint64_t s = s_begin; s < s_end; ++s) {
            const float4 rr = ps.rad[slot(s)];
            acc.x = acc.x + rr.x;
            acc.y = acc.y + rr.y;
            acc.z = acc.z + rr.z;
        }
        j.psum[px] = acc;
        if (j.aov_psum) {
            float4 aa = j.aov_psum[px], an = j.aov_psum[NP + px];
            for (uint64_t s = s_begin; s < s_end; ++s) {
                const uint32_t q = slot(s);
                const float4 a = ps.aov[q], nn = ps.aov[ps.cap + q];
                aa.x += a.x;
                aa.y += a.y;
                aa.z += a.z;
                an.x += nn.x;
                an.y += nn.y;
                an.z += nn.z;
            }
            j.aov_psum[px] = aa;
            j.aov_psum[NP + px] = an;
        }
    }
}

// Adds this wave's queue sizes to the running totals
// (totals[0] camera paths, [1] extend rays, [2] shadow rays).
__global__ void k_wave_stats(Wave w, PathState ps, uint32_t bounces, unsigned long long* totals) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long ext = 0, shd = 0;
    for (uint32_t r = 0; r < w.njobs; ++r) {
        const uint32_t* c = ps.counts + r * JOB_COUNTERS;
        for (uint32_t k = 0; k < bounces; ++k) ext += c[k];
        for (uint32_t k = 0; k < bounces; ++k) shd += c[MAX_DEPTH_SLOTS + k];
    }
    totals[0] += w.total_paths;
    totals[1] += ext;
    totals[2] += shd;
}

// iterative_render with samples = 0 (iterative.rs:37-50): the colour stays
// BLACK, so rgb gains +0.0 and alpha gains Color::a() = 1, like any call
__global__ void k_empty_pass(float4* __restrict__ rgba, uint32_t np) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < np; px += stride) {
        float4 o = rgba[px];
        o.x = o.x + 0.0f;
        o.y = o.y + 0.0f;
        o.z = o.z + 0.0f;
        o.w = o.w + 1.0f;
        rgba[px] = o;
    }
}

__global__ void k_finalize(const float4* __restrict__ psum, float4* __restrict__ rgba, uint32_t np, float inv_total) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < np; px += stride) {
        const float4 c = psum[px];
        float4 o = rgba[px];
        o.x = o.x + c.x * inv_total;
        o.y = o.y + c.y * inv_total;
        o.z = o.z + c.z * inv_total;
        o.w = o.w + 1.0f;
        rgba[px] = o;
    }
}

// ----------------------------------------------------------------------------
// Colour management (post_process.glsl:23-49, tonemapping.glsl:2-40)
// ----------------------------------------------------------------------------
__device__ __forceinline__ V3 glsl_mat3_mul(const float* m, V3 c) {
    return v3(m[0], m[1], m[2]) * c.x + v3(m[3], m[4], m[5]) * c.y + v3(m[6], m[7], m[8]) * c.z;
}
__device__ __forceinline__ float filmic1(float x) {
    x = fmaxf(0.0f, x - 0.004f);
    return (x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f);
}
__device__ __forceinline__ float unch1(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}
// Codes 0-4 are Tonemap::as_i32 of voidray_renderer; 5-7 are the curves only
// the legacy viewport has (voidray/src/shaders/tonemapping.glsl:17-45).
// `transparent` keeps the scaled input alpha (legacy viewport_fragment.glsl:62-66).
__global__ void k_tonemap(const float4* __restrict__ in, float4* __restrict__ out, uint32_t np, int32_t tonemap,
                          float inv_gamma, float ex, float scale, int32_t transparent) {
    const float A[9] = {0.59719f, 0.076f, 0.0284f, 0.35458f, 0.90834f, 0.13383f, 0.04823f, 0.01566f, 0.83777f};
    const float B[9] = {1.60475f, -0.10208f, -0.00327f, -0.53108f, 1.10813f, -0.07276f, -0.07367f, -0.00605f, 1.07602f};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
        const float4 p = in[i];
        V3 c = v3(p.x * scale, p.y * scale, p.z * scale) * ex;
        if (tonemap == 1) {
            c = glsl_mat3_mul(A, c);
            V3 num = v3(c.x * (c.x + 0.0245786f) - 0.000090537f, c.y * (c.y + 0.0245786f) - 0.000090537f,
                        c.z * (c.z + 0.0245786f) - 0.000090537f);
            V3 den = v3(c.x * (0.983729f * c.x + 0.432951f) + 0.238081f, c.y * (0.983729f * c.y + 0.432951f) + 0.238081f,
                        c.z * (0.983729f * c.z + 0.432951f) + 0.238081f);
            c = v3(num.x / den.x, num.y / den.y, num.z / den.z);
            c = glsl_mat3_mul(B, c);
        } else if (tonemap == 2) {
            const float white = 2.0f;
            const float luma = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
            const float tml = luma * (1.0f + luma / (white * white)) / (1.0f + luma);
            c = c * (tml / luma);
        } else if (tonemap == 3) {
            c = v3(filmic1(c.x), filmic1(c.y), filmic1(c.z));
        } else if (tonemap == 4) {
            c = c * 2.0f;
            V3 r = v3(unch1(c.x), unch1(c.y), unch1(c.z));
            c = r / unch1(11.2f);
        } else if (tonemap == 5) {  // legacy tonemap_simple_reinhard: color *= e / (1 + color / e), e = 1.5
            const float e = 1.5f;
            c = v3(c.x * (e / (1.0f + c.x / e)), c.y * (e / (1.0f + c.y / e)), c.z * (e / (1.0f + c.z / e)));
        } else if (tonemap == 6) {  // legacy tonemap_luma_reinhard
            const float luma = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
            const float tml = luma / (1.0f + luma);
            c = c * (tml / luma);
        } else if (tonemap == 7) {  // legacy tonemap_rombindahouse: exp(-1 / (2.72 color + 0.15))
            c = v3(expf(-1.0f / (2.72f * c.x + 0.15f)), expf(-1.0f / (2.72f * c.y + 0.15f)),
                   expf(-1.0f / (2.72f * c.z + 0.15f)));
        }
        out[i] = make_float4(powf(c.x, inv_gamma), powf(c.y, inv_gamma), powf(c.z, inv_gamma),
                             transparent ? p.w * scale : 1.0f);
    }
}

__global__ void k_relmse(const float4* __restrict__ a, float sa, const float4* __restrict__ r, float sr, uint32_t np,
                         double* __restrict__ out) {
    __shared__ double red[32];
    double acc = 0.0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
        const float4 x = a[i], y = r[i];
        const double xs[3] = {(double)x.x * sa, (double)x.y * sa, (double)x.z * sa};
        const double ys[3] = {(double)y.x * sr, (double)y.y * sr, (double)y.z * sr};
        for (int c = 0; c < 3; ++c) {
            const double dd = xs[c] - ys[c];
            acc += dd * dd / (ys[c] * ys[c] + 1e-2);
        }
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (threadIdx.x == 0) atomicAdd(out, acc);
    }
}

// ----------------------------------------------------------------------------
// Launchers
// ----------------------------------------------------------------------------
static int g_num_sms = 0;
static int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}
static Tuning g_tuning;

Tuning get_tuning() { return g_tuning; }

bool set_tuning(const Tuning& t) {
    auto ok_block = [](uint32_t b) { return b == 64 || b == 128 || b == 256; };
    if (!ok_block(t.shade_block) || !ok_block(t.raygen_block) || t.shade_blocks_per_sm < 1 ||
        t.shade_blocks_per_sm > 32)
        return false;
    const uint32_t gen = g_tuning.generation + 1;
    g_tuning = t;
    g_tuning.generation = gen;
    return true;
}

static unsigned grid_for(uint64_t n, int block, int per_sm) {
    uint64_t want = (n + block - 1) / block;
    uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (want > cap) want = cap;
    if (want == 0) want = 1;
    return (unsigned)want;
}

// Resident blocks of a persistent kernel: SMs x blocks per SM at its occupancy.
template <class K>
static unsigned persistent_grid(K kernel, int block) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm <= 0)
        per_sm = 4;
    return (unsigned)(num_sms() * per_sm);
}

cudaError_t launch_ray_sort(const float4* rays, uint32_t n, const float* lo, const float* hi, uint32_t* keys,
                            uint32_t* hist, uint32_t* perm, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(hist, 0, RAY_BINS * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    float3 l = make_float3(lo[0], lo[1], lo[2]), sc;
    auto scale = [](float a, float b) { return b > a ? 8.0f / (b - a) : 0.0f; };
    sc = make_float3(scale(lo[0], hi[0]), scale(lo[1], hi[1]), scale(lo[2], hi[2]));
    const unsigned grid = grid_for(n, 256, 4);
    k_ray_hist<<<grid, 256, 0, st>>>(rays, n, l, sc, keys, hist);
    k_ray_scan<<<1, 1024, 0, st>>>(hist);
    k_ray_scatter<<<grid, 256, 0, st>>>(keys, n, hist, perm);
    return cudaGetLastError();
}

template <bool ANY, bool COUNT>
static cudaError_t intersect_impl(const SceneView& s, const float4* rays, uint64_t n, float4* hits,
                                  uint32_t* counter, uint32_t* status, unsigned long long* work, cudaStream_t st,
                                  const uint32_t* perm = nullptr) {
    static unsigned grid = 0;
    if (!grid) grid = persistent_grid(k_intersect<ANY, COUNT>, 128);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_intersect<ANY, COUNT><<<grid, 128, 0, st>>>(BatchIo{rays, hits, s.nodes, s.tris, s.analytic, s.num_analytic,
                                                           s.num_tris, ANY, perm},
                                                   (uint32_t)n, counter, status,
                                                   work);
    return cudaGetLastError();
}

cudaError_t launch_intersect(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                             uint32_t* counter, uint32_t* status, cudaStream_t st, const uint32_t* perm) {
    if (n == 0) return cudaSuccess;
    return any ? intersect_impl<true, false>(s, rays, n, hits, counter, status, nullptr, st, perm)
               : intersect_impl<false, false>(s, rays, n, hits, counter, status, nullptr, st, perm);
}

cudaError_t launch_intersect_count(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                                   uint32_t* counter, unsigned long long* work, uint32_t* status, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    return any ? intersect_impl<true, true>(s, rays, n, hits, counter, status, work, st)
               : intersect_impl<false, true>(s, rays, n, hits, counter, status, work, st);
}

cudaError_t launch_raygen(const Wave& w, const PathState& ps, cudaStream_t st) {
    k_wave_begin<<<grid_for((uint64_t)w.njobs * JOB_COUNTERS, 256, 1), 256, 0, st>>>(w, ps);
    const int rb = (int)g_tuning.raygen_block;
    if (w.njobs == 1 && !w.from_table) k_raygen<true><<<grid_for(w.total_paths, rb, 2048 / rb), rb, 0, st>>>(w, ps);
    else k_raygen<false><<<grid_for(w.total_paths, rb, 2048 / rb), rb, 0, st>>>(w, ps);
    return cudaGetLastError();
}

template <bool COUNT, bool ONE>
static void extend_impl(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                        cudaStream_t st) {
    static unsigned g = 0;
    if (!g) g = persistent_grid(k_extend<COUNT, ONE>, 128);
    k_extend<COUNT, ONE><<<g, 128, 0, st>>>(w, ps, k, status, work);
}

cudaError_t launch_extend(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                          cudaStream_t st) {
    const bool one = w.njobs == 1 && !w.from_table;
    if (work) one ? extend_impl<true, true>(w, ps, k, status, work, st) : extend_impl<true, false>(w, ps, k, status, work, st);
    else one ? extend_impl<false, true>(w, ps, k, status, nullptr, st) : extend_impl<false, false>(w, ps, k, status, nullptr, st);
    return cudaGetLastError();
}

cudaError_t launch_shade(const Wave& w, const PathState& ps, uint32_t k, unsigned long long* retired,
                         cudaStream_t st) {
    const int sb = (int)g_tuning.shade_block, per_sm = (int)g_tuning.shade_blocks_per_sm;
    if (w.njobs == 1 && !w.from_table)
        k_shade<true><<<grid_for(w.total_paths, sb, per_sm), sb, 0, st>>>(w, ps, k, retired);
    else
        k_shade<false><<<grid_for(w.total_paths, sb, per_sm), sb, 0, st>>>(w, ps, k, retired);
    return cudaGetLastError();
}

template <bool COUNT, bool ONE>
static void shadow_impl(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                        cudaStream_t st) {
    static unsigned g = 0;
    if (!g) g = persistent_grid(k_shadow<COUNT, ONE>, 128);
    k_shadow<COUNT, ONE><<<g, 128, 0, st>>>(w, ps, k, status, work);
}

cudaError_t launch_shadow(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                          cudaStream_t st) {
    const bool one = w.njobs == 1 && !w.from_table;
    if (work) one ? shadow_impl<true, true>(w, ps, k, status, work, st) : shadow_impl<true, false>(w, ps, k, status, work, st);
    else one ? shadow_impl<false, true>(w, ps, k, status, nullptr, st) : shadow_impl<false, false>(w, ps, k, status, nullptr, st);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const Wave& w, const PathState& ps, uint32_t max_pixels, unsigned long long* totals,
                              cudaStream_t st) {
    dim3 grid(grid_for(max_pixels, 256, 8), w.njobs);
    if (w.njobs == 1 && !w.from_table) k_accumulate<true><<<grid, 256, 0, st>>>(w, ps);
    else k_accumulate<false><<<grid, 256, 0, st>>>(w, ps);
    if (totals) k_wave_stats<<<1, 32, 0, st>>>(w, ps, w.max_bounces, totals);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const float4* psum, float4* rgba, uint32_t np, float inv_total, cudaStream_t st) {
    k_finalize<<<grid_for(np, 256, 8), 256, 0, st>>>(psum, rgba, np, inv_total);
    return cudaGetLastError();
}

cudaError_t launch_tonemap(const float4* in, float4* out, uint32_t np, int32_t tonemap, float inv_gamma, float ex,
                           float scale, int32_t transparent, cudaStream_t st) {
    if (np == 0) return cudaSuccess;
    k_tonemap<<<grid_for(np, 256, 8), 256, 0, st>>>(in, out, np, tonemap, inv_gamma, ex, scale, transparent);
    return cudaGetLastError();
}

// Environment::sample (core/traits.rs:66-69) for a batch of directions
__global__ void k_env_sample(SceneView s, const float* __restrict__ dirs, uint64_t n, float* __restrict__ rgb) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const V3 c = env_eval(s, v3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

cudaError_t launch_empty_pass(float4* rgba, uint32_t np, cudaStream_t st) {
    if (np == 0) return cudaSuccess;
    k_empty_pass<<<grid_for(np, 256, 8), 256, 0, st>>>(rgba, np);
    return cudaGetLastError();
}

cudaError_t launch_env_sample(const SceneView& s, const float* dirs, uint64_t n, float* rgb, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_env_sample<<<grid_for((uint32_t)(n < (1u << 30) ? n : (1u << 30)), 256, 4), 256, 0, st>>>(s, dirs, n, rgb);
    return cudaGetLastError();
}

cudaError_t launch_relmse(const float4* a, float sa, const float4* r, float sr, uint32_t np, double* out,
                          cudaStream_t st) {
    k_relmse<<<grid_for(np, 256, 4), 256, 0, st>>>(a, sa, r, sr, np, out);
    return cudaGetLastError();
}

}  // namespace vr
