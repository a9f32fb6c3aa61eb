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
//   k_tonemap        post_process.glsl:23-49 + tonemapping.glsl:2-40
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
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd) const {
        ro = __ldg(rays + 2 * (size_t)i);
        rd = __ldg(rays + 2 * (size_t)i + 1);
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        HitOut o = h;
        if (overflow) o.prim = MISS;
        hits[i] = pack_hit(o);
    }
};

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128, VR_TRACE_MINB) k_intersect(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                   BatchIo io, uint32_t n, uint32_t* counter, uint32_t* status,
                                                   unsigned long long* work) {
    persistent_trace<ANY, COUNT>(nodes, tris, n, counter, io, status, work);
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
    return lerp3(lerp3(env_px(img, (y0 * W + x0) % len), env_px(img, (y0 * W + x0 + 1) % len), ax),
                 lerp3(env_px(img, ((y0 + 1) * W + x0) % len), env_px(img, ((y0 + 1) * W + x0 + 1) % len), ax), ay);
}
__device__ __forceinline__ uint32_t cdf_find(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, hi = n;
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
    uint32_t j = cdf_find(s.env_marg, s.env_h, u1);
    uint32_t i = cdf_find(s.env_cond + (size_t)j * (s.env_w + 1), s.env_w, u2);
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
        V3 dir = hit.normal + unit_sphere(rng);
        if (near_zero(dir)) dir = hit.normal;
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
// Path index p of a wavefront maps to global sample-major index g = g0 + p,
// pixel = g % NP, sample = first_sample + g / NP.
__device__ __forceinline__ void path_coords(const WaveParams& w, uint32_t p, uint32_t& pixel, uint32_t& sample) {
    uint64_t g = w.g0 + p;
    pixel = (uint32_t)(g % w.num_pixels);
    sample = w.first_sample + (uint32_t)(g / w.num_pixels);
}

__global__ void k_raygen(SceneView s, WaveParams w, PathState ps) {
    const uint32_t stride = gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x < MAX_DEPTH_SLOTS * 4) ps.counts[threadIdx.x] = 0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < w.paths; p += stride) {
        uint32_t pixel, sample;
        path_coords(w, p, pixel, sample);
        // iterative.rs:25-40 (row = pixel / width)
        const uint32_t W = w.width, H = w.height;
        const uint32_t x = pixel % W, y = pixel / W;
        const float dmax = (float)max(W, H);
        const float fx = ((float)(2 * x + 1) - (float)W) / dmax;
        const float fy = ((float)(2 * (H - y) - 1) - (float)H) / dmax;
        Rng rng;
        rng.inc = pcg_inc(sample, pixel);
        rng.state = pcg_init(w.seed, rng.inc);
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

// Closest hit of the live queue of depth k.
// Closest hit of the live queue of depth k (persistent, dynamic fetch).
struct ExtendIo {
    const float4* org;
    const float4* dir;
    float4* hits;
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd) const {
        ro = org[i];
        rd = dir[i];
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        HitOut o = h;
        if (overflow) o.prim = MISS;
        hits[i] = pack_hit(o);
    }
};

template <bool COUNT>
__global__ void __launch_bounds__(128, VR_TRACE_MINB) k_extend(SceneView s, PathState ps, uint32_t k, uint32_t* status,
                                                unsigned long long* work) {
    const uint32_t n = (k == 0) ? ps.first_count : ps.counts[k];
    const uint32_t base = (k & 1) ? ps.cap : 0;
    ExtendIo io{ps.q_org + base, ps.q_dir + base, ps.hits};
    persistent_trace<false, COUNT>(s.nodes, s.tris, n, &ps.counts[2 * MAX_DEPTH_SLOTS + k], io, status, work);
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

__global__ void __launch_bounds__(256) k_shade(SceneView s, WaveParams w, RenderParams rp, PathState ps, uint32_t k) {
    const uint32_t n = (k == 0) ? ps.first_count : ps.counts[k];
    const uint32_t in_base = (k & 1) ? ps.cap : 0;
    const uint32_t out_base = (k & 1) ? 0 : ps.cap;
    const uint32_t stride = gridDim.x * blockDim.x;
    const float fc = rp.firefly_clamp;
    const bool nee_mode = rp.estimator == 1;
    const bool last = (k + 1 >= rp.max_bounces);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        bool cont = false, want_shadow = false;
        V3 new_o, new_d, sh_dir, sh_c;
        uint32_t p = 0;
        if (i < n) {
            p = ps.q_path[in_base + i];
            const float4 ro4 = ps.q_org[in_base + i], rd4 = ps.q_dir[in_base + i];
            const V3 ro = xyz(ro4), rd = xyz(rd4);
            const float4 hh = ps.hits[i];
            const uint32_t prim = __float_as_uint(hh.x);
            uint32_t pixel, sample;
            path_coords(w, p, pixel, sample);
            Rng rng;
            rng.inc = pcg_inc(sample, pixel);
            rng.state = ps.rng[p];
            const float4 thr4 = ps.thr[p];
            V3 T = xyz(thr4);
            float prev_pdf = thr4.w;
            if (prim == MISS) {
                const V3 le = env_eval(s, rd);
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
                // shading record and normal (mesh.rs:176-188, ray.rs:34-49)
                const float4* sh = s.shade + 4 * (size_t)prim;
                const float4 s0 = __ldg(sh), s1 = __ldg(sh + 1), s2 = __ldg(sh + 2), s3 = __ldg(sh + 3);
                const Material m = s.materials[__float_as_uint(s0.w)];
                const float u = hh.z, v = hh.w, t = hh.y;
                const float wb = 1.0f - u - v;
                V3 normal = u * xyz(s1) + v * xyz(s2) + wb * xyz(s0);
                const V3 fnm = xyz(s3);
                const float ang = acosf(dot(normal, fnm) / (sqrtf(mag2(normal)) * sqrtf(mag2(fnm))));
                if (ang > 30.0f * PI_F / 180.0f) normal = fnm;
                SurfHit hit;
                hit.point = ro + rd * t;
                hit.t = t;
                hit.front = dot(rd, normal) < 0.0f;
                hit.normal = hit.front ? normal : -normal;
                if (rp.render_mode != 1) {
                    const V3 nn = normalize(hit.normal);
                    const V3 c = (0.5f * nn) + v3(1.0f, 1.0f, 1.0f) * 0.5f;
                    if (nee_mode) rad_add(ps, p, clampc(vmul(T, c), fc));
                    else unwind(ps, p, k, clampc(c, fc), fc);
                } else {
                    const bool lamb = (m.kind == M_LAMB) &&
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
                        if (nee_mode) rad_add(ps, p, clampc(vmul(T, att), fc));
                        else unwind(ps, p, k, clampc(att, fc), fc);
                    } else {
                        V3 tn = vmul(T, att);
                        if (nee_mode) prev_pdf = lamb ? dot(hit.normal, nd) / PI_F : -1.0f;
                        bool alive = true;
                        if (rp.rr_depth != 0 && k >= rp.rr_depth) {
                            const float q = fminf(max3(tn), 0.95f);
                            const float ur = rng.uniform();
                            if (!(ur < q)) {
                                alive = false;
                            } else {
                                att = att / q;
                                tn = tn / q;
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
        // warp-aggregated compaction into the next queue and the shadow queue
        const uint32_t active = __activemask();
        const uint32_t cm = __ballot_sync(active, cont);
        if (cm) {
            const uint32_t leader = __ffs(cm) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&ps.counts[k + 1], __popc(cm));
            base = __shfl_sync(active, base, leader);
            if (cont) {
                const uint32_t slot = base + __popc(cm & ((1u << lane) - 1u));
                ps.q_org[out_base + slot] = make_float4(new_o.x, new_o.y, new_o.z, SCENE_TMIN);
                ps.q_dir[out_base + slot] = make_float4(new_d.x, new_d.y, new_d.z, INF_F);
                ps.q_path[out_base + slot] = p;
            }
        }
        const uint32_t sm = __ballot_sync(active, want_shadow);
        if (sm) {
            const uint32_t leader = __ffs(sm) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&ps.counts[MAX_DEPTH_SLOTS + k], __popc(sm));
            base = __shfl_sync(active, base, leader);
            if (want_shadow) {
                const uint32_t slot = base + __popc(sm & ((1u << lane) - 1u));
                ps.s_org[slot] = make_float4(new_o.x, new_o.y, new_o.z, SCENE_TMIN);
                ps.s_dir[slot] = make_float4(sh_dir.x, sh_dir.y, sh_dir.z, INF_F);
                ps.s_path[slot] = p;
                ps.s_contrib[slot] = make_float4(sh_c.x, sh_c.y, sh_c.z, 0.0f);
            }
        }
    }
}

// NEE visibility: adds the (clamped) contribution when nothing is hit
// (persistent any-hit traversal).  A stack overflow counts as occluded.
struct ShadowIo {
    const float4* org;
    const float4* dir;
    const uint32_t* path;
    const float4* contrib;
    PathState ps;
    float fc;
    __device__ __forceinline__ void load(uint32_t i, float4& ro, float4& rd) const {
        ro = org[i];
        rd = dir[i];
    }
    __device__ __forceinline__ void store(uint32_t i, const HitOut& h, bool overflow) const {
        if (!overflow && h.prim == MISS) rad_add(ps, path[i], clampc(xyz(contrib[i]), fc));
    }
};

template <bool COUNT>
__global__ void __launch_bounds__(128, VR_TRACE_MINB) k_shadow(SceneView s, RenderParams rp, PathState ps, uint32_t k,
                                                uint32_t* status, unsigned long long* work) {
    const uint32_t n = ps.counts[MAX_DEPTH_SLOTS + k];
    ShadowIo io{ps.s_org, ps.s_dir, ps.s_path, ps.s_contrib, ps, rp.firefly_clamp};
    persistent_trace<true, COUNT>(s.nodes, s.tris, n, &ps.counts[3 * MAX_DEPTH_SLOTS + k], io, status, work);
}

// Per-pixel running sum in sample order over this wavefront's paths.
__global__ void k_accumulate(WaveParams w, PathState ps, float4* __restrict__ psum) {
    const uint32_t NP = w.num_pixels;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < NP; px += stride) {
        // global indices g = s*NP + px inside [g0, g0 + paths)
        uint64_t g0 = w.g0, g1 = w.g0 + w.paths;
        uint64_t s_begin = (g0 > px) ? (g0 - px + NP - 1) / NP : 0;
        if (s_begin * NP + px >= g1) continue;
        float4 acc = psum[px];
        for (uint64_t g = s_begin * NP + px; g < g1; g += NP) {
            const float4 r = ps.rad[g - g0];
            acc.x = acc.x + r.x;
            acc.y = acc.y + r.y;
            acc.z = acc.z + r.z;
        }
        psum[px] = acc;
    }
}

// Adds this wavefront's queue sizes to the running totals
// (totals[0] camera paths, [1] extend rays, [2] shadow rays).
__global__ void k_wave_stats(PathState ps, uint32_t paths, uint32_t bounces, unsigned long long* totals) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long ext = bounces > 0 ? paths : 0, shd = 0;
    for (uint32_t k = 1; k < bounces; ++k) ext += ps.counts[k];
    for (uint32_t k = 0; k < bounces; ++k) shd += ps.counts[MAX_DEPTH_SLOTS + k];
    totals[0] += paths;
    totals[1] += ext;
    totals[2] += shd;
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
__global__ void k_tonemap(const float4* __restrict__ in, float4* __restrict__ out, uint32_t np, int32_t tonemap,
                          float inv_gamma, float ex, float scale) {
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
        }
        out[i] = make_float4(powf(c.x, inv_gamma), powf(c.y, inv_gamma), powf(c.z, inv_gamma), 1.0f);
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

template <bool ANY, bool COUNT>
static cudaError_t intersect_impl(const SceneView& s, const float4* rays, uint64_t n, float4* hits,
                                  uint32_t* counter, uint32_t* status, unsigned long long* work, cudaStream_t st) {
    static unsigned grid = 0;
    if (!grid) grid = persistent_grid(k_intersect<ANY, COUNT>, 128);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_intersect<ANY, COUNT><<<grid, 128, 0, st>>>(s.nodes, s.tris, BatchIo{rays, hits}, (uint32_t)n, counter, status,
                                                   work);
    return cudaGetLastError();
}

cudaError_t launch_intersect(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                             uint32_t* counter, uint32_t* status, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    return any ? intersect_impl<true, false>(s, rays, n, hits, counter, status, nullptr, st)
               : intersect_impl<false, false>(s, rays, n, hits, counter, status, nullptr, st);
}

cudaError_t launch_intersect_count(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                                   uint32_t* counter, unsigned long long* work, uint32_t* status, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    return any ? intersect_impl<true, true>(s, rays, n, hits, counter, status, work, st)
               : intersect_impl<false, true>(s, rays, n, hits, counter, status, work, st);
}

cudaError_t launch_raygen(const SceneView& s, const WaveParams& w, const PathState& ps, cudaStream_t st) {
    k_raygen<<<grid_for(w.paths, 256, 8), 256, 0, st>>>(s, w, ps);
    return cudaGetLastError();
}

cudaError_t launch_extend(const SceneView& s, const WaveParams& w, const PathState& ps, uint32_t k, uint32_t* status,
                          unsigned long long* work, cudaStream_t st) {
    static unsigned g0 = 0, g1 = 0;
    PathState p = ps;
    p.first_count = w.paths;
    if (work) {
        if (!g1) g1 = persistent_grid(k_extend<true>, 128);
        k_extend<true><<<g1, 128, 0, st>>>(s, p, k, status, work);
    } else {
        if (!g0) g0 = persistent_grid(k_extend<false>, 128);
        k_extend<false><<<g0, 128, 0, st>>>(s, p, k, status, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_shade(const SceneView& s, const WaveParams& w, const RenderParams& rp, const PathState& ps,
                         uint32_t k, cudaStream_t st) {
    PathState p = ps;
    p.first_count = w.paths;
    k_shade<<<grid_for(w.paths, 256, 8), 256, 0, st>>>(s, w, rp, p, k);
    return cudaGetLastError();
}

cudaError_t launch_shadow(const SceneView& s, const WaveParams& w, const RenderParams& rp, const PathState& ps,
                          uint32_t k, uint32_t* status, unsigned long long* work, cudaStream_t st) {
    static unsigned g0 = 0, g1 = 0;
    if (work) {
        if (!g1) g1 = persistent_grid(k_shadow<true>, 128);
        k_shadow<true><<<g1, 128, 0, st>>>(s, rp, ps, k, status, work);
    } else {
        if (!g0) g0 = persistent_grid(k_shadow<false>, 128);
        k_shadow<false><<<g0, 128, 0, st>>>(s, rp, ps, k, status, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const WaveParams& w, const PathState& ps, const RenderParams& rp, float4* psum,
                              unsigned long long* totals, cudaStream_t st) {
    k_accumulate<<<grid_for(w.num_pixels, 256, 8), 256, 0, st>>>(w, ps, psum);
    if (totals) k_wave_stats<<<1, 32, 0, st>>>(ps, w.paths, rp.max_bounces, totals);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const float4* psum, float4* rgba, uint32_t np, float inv_total, cudaStream_t st) {
    k_finalize<<<grid_for(np, 256, 8), 256, 0, st>>>(psum, rgba, np, inv_total);
    return cudaGetLastError();
}

cudaError_t launch_tonemap(const float4* in, float4* out, uint32_t np, int32_t tonemap, float inv_gamma, float ex,
                           float scale, cudaStream_t st) {
    if (np == 0) return cudaSuccess;
    k_tonemap<<<grid_for(np, 256, 8), 256, 0, st>>>(in, out, np, tonemap, inv_gamma, ex, scale);
    return cudaGetLastError();
}

cudaError_t launch_relmse(const float4* a, float sa, const float4* r, float sr, uint32_t np, double* out,
                          cudaStream_t st) {
    k_relmse<<<grid_for(np, 256, 4), 256, 0, st>>>(a, sa, r, sr, np, out);
    return cudaGetLastError();
}

}  // namespace vr
