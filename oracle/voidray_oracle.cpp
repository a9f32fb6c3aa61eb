// voidray_oracle.cpp — CPU oracle (test infrastructure only; see voidray_oracle.h).
//
// A restatement of the reference's CPU integrator in C++17.  Floating-point
// expressions keep the reference's operation order (cgmath 0.18 semantics:
// dot = (x*x' + y*y') + z*z', cross as (y*z'-z*y', ...), normalize = v * (1/|v|))
// and must be compiled without contraction (-ffp-contract=off) so that every
// operation rounds as the Rust f32 code does.  Bugs and quirks of the
// reference are kept on purpose; each is marked QUIRK with its source line.
// Parity is unpinned: no golden vectors exist for this path upstream.
#include "voidray_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;
const float PI_F = 3.14159265358979323846f;     // std::f32::consts::PI
const float INF_F = std::numeric_limits<float>::infinity();

// ------------------------------------------------------------------ vec3 --
struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float mag2(V3 a) { return dot(a, a); }
inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(mag2(a))); }
inline V3 vmin(V3 a, V3 b) { return v3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }
// Color::clamp (util/color.rs:30-36): componentwise f32::min.
inline V3 clampc(V3 c, float m) { return v3(std::fmin(c.x, m), std::fmin(c.y, m), std::fmin(c.z, m)); }
// math.rs:6-9
inline bool near_zero(V3 v) {
    const float e = 1.0e-8f;
    return std::fabs(v.x) < e && std::fabs(v.y) < e && std::fabs(v.z) < e;
}
// math.rs:12-14
inline V3 reflect(V3 v, V3 n) { return v - (2.0f * dot(v, n)) * n; }
// math.rs:16-21
inline V3 refract(V3 uv, V3 n, float etai_over_etat) {
    float cos_theta = std::fmin(dot(n, -uv), 1.0f);
    V3 out_perp = etai_over_etat * (uv + cos_theta * n);
    V3 out_parallel = -(std::sqrt(std::fabs(1.0f - mag2(out_perp)))) * n;
    return out_perp + out_parallel;
}
inline float powi2(float x) { return x * x; }
inline float powi3(float x) { return x * (x * x); }
inline float powi5(float x) { float s = x * x; s = s * s; return x * s; }

// ------------------------------------------------------------------ rng ---
// PCG32 (O'Neill 2014, pcg32_srandom_r / pcg32_random_r), one stream per path.
struct Pcg32 {
    uint64_t state, inc;
    Pcg32(uint64_t seed, uint32_t sample, uint32_t pixel) {
        uint64_t stream = ((uint64_t)sample << 32) | (uint64_t)pixel;
        state = 0;
        inc = (stream << 1) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    // rand 0.8 Standard f32: 24 high bits scaled into [0,1).
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    // gen_range(low..high): low + u*(high-low).
    float range(float low, float high) {
        float scale = high - low;
        return uniform() * scale + low;
    }
};
const int REJECT_TRIES = 64;
// rand_distr 0.4.3 UnitSphere (Marsaglia 1972).
V3 unit_sphere(Pcg32& r) {
    for (int i = 0; i < REJECT_TRIES; ++i) {
        float x1 = r.range(-1.0f, 1.0f), x2 = r.range(-1.0f, 1.0f);
        float sum = x1 * x1 + x2 * x2;
        if (sum >= 1.0f) continue;
        float factor = 2.0f * std::sqrt(1.0f - sum);
        return v3(x1 * factor, x2 * factor, 1.0f - 2.0f * sum);
    }
    return v3(0.0f, 0.0f, 1.0f);
}
// rand_distr 0.4.3 UnitDisc (rejection from the square).
void unit_disc(Pcg32& r, float* x, float* y) {
    for (int i = 0; i < REJECT_TRIES; ++i) {
        float x1 = r.range(-1.0f, 1.0f), x2 = r.range(-1.0f, 1.0f);
        if (x1 * x1 + x2 * x2 <= 1.0f) { *x = x1; *y = x2; return; }
    }
    *x = 0.0f; *y = 0.0f;
}
// rand_distr 0.4.3 UnitCircle (von Neumann / Marsaglia).
void unit_circle(Pcg32& r, float* x, float* y) {
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

// ----------------------------------------------------------------- aabb ---
struct Aabb {
    V3 min, max;
};
inline Aabb aabb_default() { return Aabb{v3(INF_F, INF_F, INF_F), v3(-INF_F, -INF_F, -INF_F)}; }
inline bool aabb_is_default(const Aabb& b) {
    return b.min.x == INF_F && b.min.y == INF_F && b.min.z == INF_F &&
           b.max.x == -INF_F && b.max.y == -INF_F && b.max.z == -INF_F;
}
inline Aabb surround(const Aabb& a, const Aabb& b) { return Aabb{vmin(a.min, b.min), vmax(a.max, b.max)}; }
inline Aabb from_point(V3 p) { return Aabb{p, p}; }
inline V3 centroid(const Aabb& b) { return (b.min + b.max) / 2.0f; }
// aabb.rs:62-83
Aabb epsilon_expand(Aabb b, float eps) {
    V3 d = b.max - b.min;
    V3 c = centroid(b);
    if (d.x < eps) { b.min.x = c.x - eps; b.max.x = c.x + eps; }
    if (d.y < eps) { b.min.y = c.y - eps; b.max.y = c.y + eps; }
    if (d.z < eps) { b.min.z = c.z - eps; b.max.z = c.z + eps; }
    return b;
}
struct Ray {
    V3 o, d;
};
// aabb.rs:86-148.  QUIRK (aabb.rs:88-90): the default (empty) box always hits.
bool aabb_hit(const Aabb& b, const Ray& r, float t_min, float t_max) {
    if (aabb_is_default(b)) return true;
    for (int a = 0; a < 3; ++a) {
        float inv_d = 1.0f / comp(r.d, a);
        float t0 = (comp(b.min, a) - comp(r.o, a)) * inv_d;
        float t1 = (comp(b.max, a) - comp(r.o, a)) * inv_d;
        if (inv_d < 0.0f) std::swap(t0, t1);
        if (t0 > t_min) t_min = t0;
        if (t1 < t_max) t_max = t1;
        if (t_max <= t_min) return false;
    }
    return true;
}

// f32::total_cmp ordering key (used by the BVH sort, bvh.rs:82-106).
inline int32_t total_key(float f) {
    int32_t k;
    std::memcpy(&k, &f, 4);
    k ^= (int32_t)(((uint32_t)(k >> 31)) >> 1);
    return k;
}

// ------------------------------------------------------------------ bvh ---
// BvhNode (bvh.rs:41-45) as an index tree.
struct Node {
    int kind;  // 0 none, 1 object, 2 split
    uint32_t handle;
    Aabb bounds;
    int left, right;
};
struct Bvh {
    std::vector<Node> nodes;
    int root = -1;
};

// BvhNode::from_list (bvh.rs:48-130): median split on the axis of largest
// centroid spread, stable sort by centroid (total_cmp), left = first len/2.
template <class BoundsFn>
int bvh_build(Bvh& bvh, std::vector<uint32_t>& objects, const BoundsFn& bounds_ref) {
    Node n{};
    if (objects.empty()) {
        n.kind = 0;
        bvh.nodes.push_back(n);
        return (int)bvh.nodes.size() - 1;
    }
    if (objects.size() == 1) {
        n.kind = 1;
        n.handle = objects[0];
        bvh.nodes.push_back(n);
        return (int)bvh.nodes.size() - 1;
    }
    Aabb bounds = bounds_ref(objects[0]);
    Aabb cents = from_point(centroid(bounds_ref(objects[0])));
    for (size_t i = 1; i < objects.size(); ++i) {
        bounds = surround(bounds, bounds_ref(objects[i]));
        cents = surround(cents, from_point(centroid(bounds_ref(objects[i]))));
    }
    V3 spread = cents.max - cents.min;
    int axis;
    if (spread.x > spread.y && spread.x > spread.z) axis = 0;
    else if (spread.y > spread.x && spread.y > spread.z) axis = 1;
    else axis = 2;
    std::vector<std::pair<int32_t, uint32_t>> keyed(objects.size());
    for (size_t i = 0; i < objects.size(); ++i)
        keyed[i] = {total_key(comp(centroid(bounds_ref(objects[i])), axis)), objects[i]};
    std::stable_sort(keyed.begin(), keyed.end(),
                     [](const std::pair<int32_t, uint32_t>& a, const std::pair<int32_t, uint32_t>& b) {
                         return a.first < b.first;
                     });
    size_t half = objects.size() / 2;
    std::vector<uint32_t> left, right;
    left.reserve(half);
    right.reserve(objects.size() - half);
    for (size_t i = 0; i < keyed.size(); ++i) (i < half ? left : right).push_back(keyed[i].second);
    int li = bvh_build(bvh, left, bounds_ref);
    int ri = bvh_build(bvh, right, bounds_ref);
    n.kind = 2;
    n.bounds = bounds;
    n.left = li;
    n.right = ri;
    bvh.nodes.push_back(n);
    return (int)bvh.nodes.size() - 1;
}

// ----------------------------------------------------------------- scene --
struct Hit {
    V3 point, normal;
    V3 snormal;     // normal of the Lambertian scatter: the normal map's RGB when there is one
    float t;
    float uvx, uvy;
    bool front_face;
    uint32_t prim;  // global triangle id (the reference drops it, mesh.rs:124)
    float bu, bv;   // barycentrics
};
// HitRecord::new (ray.rs:34-49)
inline void make_hit(Hit& h, V3 point, V3 outward, float t, float ux, float uy, const Ray& r) {
    h.front_face = dot(r.d, outward) < 0.0f;
    h.normal = h.front_face ? outward : -outward;
    h.snormal = h.normal;
    h.point = point;
    h.t = t;
    h.uvx = ux;
    h.uvy = uy;
}

struct Mesh {
    std::vector<V3> pos, nrm;
    std::vector<float> uv;  // 2 per vertex
    std::vector<uint32_t> idx;
    std::vector<V3> face_n;
    Aabb bounds;
    Bvh bvh;
    bool has_bvh = false;
    uint32_t first_prim = 0;
};

struct EnvTables {
    uint32_t W = 0, H = 0;
    std::vector<float> marginal, conditional, cell;
};

struct Analytic {
    int kind;  // 1 sphere, 2 ground plane
    V3 center;
    float radius, height;
    int surface;
};

struct Texture {
    uint32_t w = 0, h = 0;
    int sampling = 0;  // 0 nearest, 1 bilinear
    std::vector<float> img;
};

struct Scene {
    std::vector<Mesh> meshes;
    std::vector<Analytic> analytics;
    std::vector<Texture> textures;
    std::vector<int> mesh_surface;      // surface index of each mesh
    std::vector<int> surf_mesh;         // per surface: mesh index or -1
    std::vector<int> surf_analytic;     // per surface: analytic index or -1
    std::vector<orc_material> materials;
    std::vector<int> surface_material;  // material of surface s (QUIRK, scene.rs:377)
    Bvh top;
    orc_env env{};
    std::vector<float> env_img;
    EnvTables tables;
    bool has_tables = false;
    // CameraAcceleration (camera.rs:38-53)
    V3 c_origin, c_dir, c_right, c_up;
    float c_d = 1.0f;
    bool c_dof = false;
    float c_aperture = 0.0f, c_focal = 0.0f;
    uint64_t num_prims = 0;
};

// Triangle::hit (mesh.rs:144-188).  QUIRK: the determinant test uses t_min
// as an absolute epsilon (mesh.rs:156) and t_max is ignored (mesh.rs:144).
bool triangle_hit(const Mesh& m, uint32_t tri, const Ray& r, float tmin, Hit& out) {
    const uint32_t* ix = &m.idx[3 * tri];
    V3 p0 = m.pos[ix[0]], p1 = m.pos[ix[1]], p2 = m.pos[ix[2]];
    V3 e1 = p1 - p0;
    V3 e2 = p2 - p0;
    V3 h = cross(r.d, e2);
    float a = dot(e1, h);
    if (a > -tmin && a < tmin) return false;
    float f = 1.0f / a;
    V3 s = r.o - p0;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    V3 q = cross(s, e1);
    float v = f * dot(r.d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = f * dot(e2, q);
    float w = 1.0f - u - v;
    V3 normal = u * m.nrm[ix[1]] + v * m.nrm[ix[2]] + w * m.nrm[ix[0]];
    float uvx = u * m.uv[2 * ix[1]] + v * m.uv[2 * ix[2]] + w * m.uv[2 * ix[0]];
    float uvy = u * m.uv[2 * ix[1] + 1] + v * m.uv[2 * ix[2] + 1] + w * m.uv[2 * ix[0] + 1];
    // cgmath InnerSpace::angle = acos(a.b / (|a| |b|)).  QUIRK: a zero
    // normal gives NaN, the comparison is false and the zero normal stays.
    V3 fnm = m.face_n[tri];
    float ang = std::acos(dot(normal, fnm) / (std::sqrt(mag2(normal)) * std::sqrt(mag2(fnm))));
    if (ang > 30.0f * PI_F / 180.0f) normal = fnm;
    if (t > tmin) {
        make_hit(out, r.o + r.d * t, normal, t, uvx, uvy, r);
        out.prim = m.first_prim + tri;
        out.bu = u;
        out.bv = v;
        return true;
    }
    return false;
}

struct HitPair {
    bool ok = false;
    Hit best;
    float second = INF_F;
};
inline void note_second(HitPair& hp, float t) {
    if (t < hp.second) hp.second = t;
}
// merge_optionals (bvh.rs:165-181): strictly smaller left wins, ties go right.
HitPair merge(const HitPair& l, const HitPair& r) {
    HitPair out;
    if (l.ok && r.ok) {
        const HitPair& w = (l.best.t < r.best.t) ? l : r;
        const HitPair& o = (l.best.t < r.best.t) ? r : l;
        out = w;
        note_second(out, o.best.t);
        note_second(out, o.second);
    } else if (l.ok) {
        out = l;
        note_second(out, r.second);
    } else if (r.ok) {
        out = r;
        note_second(out, l.second);
    } else {
        out.second = std::fmin(l.second, r.second);
    }
    return out;
}

HitPair mesh_bvh_hit(const Mesh& m, int ni, const Ray& r, float tmin, float tmax) {
    const Node& n = m.bvh.nodes[ni];
    HitPair hp;
    if (n.kind == 1) {
        hp.ok = triangle_hit(m, n.handle, r, tmin, hp.best);
        return hp;
    }
    if (n.kind == 2 && aabb_hit(n.bounds, r, tmin, tmax)) {
        return merge(mesh_bvh_hit(m, n.left, r, tmin, tmax), mesh_bvh_hit(m, n.right, r, tmin, tmax));
    }
    return hp;
}
// Mesh::hit (mesh.rs:122-140)
HitPair mesh_hit(const Mesh& m, const Ray& r, float tmin, float tmax) {
    if (m.has_bvh) return mesh_bvh_hit(m, m.bvh.root, r, tmin, tmax);
    HitPair hp;
    float closest = tmax;
    uint32_t nt = (uint32_t)m.face_n.size();
    for (uint32_t i = 0; i < nt; ++i) {
        Hit h;
        if (triangle_hit(m, i, r, tmin, h)) {
            if (closest > h.t) {
                if (hp.ok) note_second(hp, hp.best.t);
                closest = h.t;
                hp.best = h;
                hp.ok = true;
            } else {
                note_second(hp, h.t);
            }
        }
    }
    return hp;
}
// Sphere::hit (surfaces.rs:45-80) and GroundPlane::hit (surfaces.rs:86-105).
// The hit's prim id is num_prims + analytic index.
HitPair analytic_hit(const Scene& s, int ai, const Ray& r, float tmin, float tmax) {
    const Analytic& a = s.analytics[ai];
    HitPair hp;
    Hit h;
    h.prim = (uint32_t)(s.num_prims + ai);
    h.bu = h.bv = 0.0f;
    if (a.kind == 1) {
        V3 oc = r.o - a.center;
        float aa = mag2(r.d);
        float half_b = dot(oc, r.d);
        float c = mag2(oc) - a.radius * a.radius;
        float disc = half_b * half_b - aa * c;
        if (disc < 0.0f) return hp;
        float sq = std::sqrt(disc);
        float root = (-half_b - sq) / aa;
        if (root < tmin || tmax < root) {
            root = (-half_b + sq) / aa;
            if (root < tmin || tmax < root) return hp;
        }
        V3 point = r.o + r.d * root;
        V3 normal = (point - a.center) / a.radius;
        make_hit(h, point, normal, root, 0.0f, 0.0f, r);
    } else {
        float t = (a.height - r.o.y) / r.d.y;
        if (t <= tmin || t >= tmax) return hp;
        V3 point = r.o + r.d * t;
        make_hit(h, point, v3(0.0f, 1.0f, 0.0f), t, point.x, point.z, r);
    }
    hp.ok = true;
    hp.best = h;
    return hp;
}
HitPair surface_hit(const Scene& s, int si, const Ray& r, float tmin, float tmax) {
    if (s.surf_mesh[si] >= 0) return mesh_hit(s.meshes[s.surf_mesh[si]], r, tmin, tmax);
    return analytic_hit(s, s.surf_analytic[si], r, tmin, tmax);
}
HitPair top_hit(const Scene& s, int ni, const Ray& r, float tmin, float tmax) {
    const Node& n = s.top.nodes[ni];
    HitPair hp;
    if (n.kind == 1) return surface_hit(s, (int)n.handle, r, tmin, tmax);
    if (n.kind == 2 && aabb_hit(n.bounds, r, tmin, tmax))
        return merge(top_hit(s, n.left, r, tmin, tmax), top_hit(s, n.right, r, tmin, tmax));
    return hp;
}
// SceneAcceleration::hit (scene.rs:182-185): t_min = 1e-5, t_max = INF.
const float SCENE_TMIN = 0.00001f;
inline HitPair scene_hit(const Scene& s, const Ray& r, float tmin = SCENE_TMIN, float tmax = INF_F) {
    if (s.top.root < 0) return HitPair{};
    return top_hit(s, s.top.root, r, tmin, tmax);
}
int mesh_of_prim(const Scene& s, uint32_t prim) {
    // meshes are few; linear search is fine for the oracle
    for (size_t i = 0; i < s.meshes.size(); ++i) {
        const Mesh& m = s.meshes[i];
        if (prim >= m.first_prim && prim < m.first_prim + m.face_n.size()) return (int)i;
    }
    return -1;
}
int surface_of_prim(const Scene& s, uint32_t prim) {
    if (prim >= s.num_prims) {
        const uint64_t a = prim - s.num_prims;
        return a < s.analytics.size() ? s.analytics[a].surface : -1;
    }
    const int m = mesh_of_prim(s, prim);
    return m < 0 ? -1 : s.mesh_surface[m];
}

// ----------------------------------------------------------- environment --
inline V3 env_px(const Scene& s, size_t i) {
    const float* p = &s.env_img[3 * i];
    return v3(p[0], p[1], p[2]);
}
inline size_t sat_usize(float x) {  // Rust `as usize`: NaN and negatives -> 0
    if (!(x > 0.0f)) return 0;
    if (x >= 18446744073709551615.0f) return SIZE_MAX;
    return (size_t)x;
}
inline V3 lerp3(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }  // math.rs:24-29
// HDRIEnvironment::bilinear_sample (environments.rs:57-77).  QUIRK: wrap by
// modulo of the linear index (x0+1 runs into the next row).
V3 hdri_bilinear(const Scene& s, float x, float y) {
    size_t W = s.env.width, H = s.env.height, len = W * H;
    size_t x0 = std::min(sat_usize(x), W - 1);
    size_t y0 = std::min(sat_usize(y), H - 1);
    float ax = x - (float)x0;
    float ay = y - (float)y0;
    return lerp3(lerp3(env_px(s, (y0 * W + x0) % len), env_px(s, (y0 * W + x0 + 1) % len), ax),
                 lerp3(env_px(s, ((y0 + 1) * W + x0) % len), env_px(s, ((y0 + 1) * W + x0 + 1) % len), ax),
                 ay);
}
// Environment::sample; the direction is normalised again (environments.rs:81).
V3 env_eval(const Scene& s, V3 dir) {
    if (s.env.kind == 1) return load3(s.env.color);
    if (s.env.kind != 2) return v3(0.0f, 0.0f, 0.0f);
    V3 d = normalize(dir);
    // to_spherical_coords (math.rs:32-37)
    float sx = std::acos(-d.y);
    float sy = std::atan2(-d.z, d.x) + PI_F;
    float u = sx / PI_F;
    float v = sy / (2.0f * PI_F);
    float x = v * (float)s.env.width;
    float y = (float)(s.env.height - 1) - (u * (float)s.env.height);
    return hdri_bilinear(s, x, y);
}

// Importance-sampling tables (extension, no reference counterpart).
// Cell (j, i) covers theta in [j, j+1)*pi/H and phi in [i, i+1)*2pi/W; its
// weight is (luminance of the environment at the cell centre + a floor of
// 1e-3 of the mean) * sin(theta_centre).
inline V3 dir_from_angles(float sin_t, float cos_t, float phi) {
    return v3(-sin_t * std::cos(phi), -cos_t, sin_t * std::sin(phi));
}
void build_env_tables(Scene& s) {
    const uint32_t W = s.env.width, H = s.env.height;
    EnvTables& T = s.tables;
    T.W = W;
    T.H = H;
    std::vector<double> lum((size_t)W * H);
    double lsum = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        float theta = ((float)j + 0.5f) * (PI_F / (float)H);
        float st = std::sin(theta), ct = std::cos(theta);
        for (uint32_t i = 0; i < W; ++i) {
            float phi = ((float)i + 0.5f) * (2.0f * PI_F / (float)W);
            V3 c = env_eval(s, dir_from_angles(st, ct, phi));
            float l = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
            if (!(l > 0.0f) || !std::isfinite(l)) l = 0.0f;
            lum[(size_t)j * W + i] = (double)l;
            lsum += (double)l;
        }
    }
    double floor_l = 1e-3 * (lsum / ((double)W * H));
    if (!(floor_l > 0.0)) floor_l = 1.0;
    std::vector<double> w((size_t)W * H), rows(H);
    double total = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        float theta = ((float)j + 0.5f) * (PI_F / (float)H);
        double st = (double)std::sin(theta);
        double rs = 0.0;
        for (uint32_t i = 0; i < W; ++i) {
            double x = (lum[(size_t)j * W + i] + floor_l) * st;
            w[(size_t)j * W + i] = x;
            rs += x;
        }
        rows[j] = rs;
        total += rs;
    }
    T.marginal.assign(H + 1, 0.0f);
    T.conditional.assign((size_t)H * (W + 1), 0.0f);
    T.cell.assign((size_t)W * H, 0.0f);
    double acc = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        T.marginal[j] = (float)(acc / total);
        acc += rows[j];
        double ra = 0.0;
        float* cr = &T.conditional[(size_t)j * (W + 1)];
        for (uint32_t i = 0; i < W; ++i) {
            cr[i] = (float)(ra / rows[j]);
            ra += w[(size_t)j * W + i];
            T.cell[(size_t)j * W + i] = (float)(w[(size_t)j * W + i] / total);
        }
        cr[W] = 1.0f;
    }
    T.marginal[H] = 1.0f;
}
// largest k in [0, n) with cdf[k] <= u (cdf[0] == 0, cdf[n] == 1)
inline uint32_t cdf_find(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, hi = n;  // invariant: cdf[lo] <= u, answer in [lo, hi)
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid; else hi = mid;
    }
    return lo;
}
const double INV_CELL_AREA_NUM = 1.0 / (2.0 * 3.14159265358979323846 * 3.14159265358979323846);
inline float cell_density(const EnvTables& T, uint32_t j, uint32_t i, float sin_t) {
    // p_cell / (dtheta * dphi * sin_t) with dtheta*dphi = 2 pi^2 / (H W)
    float scale = (float)((double)T.W * (double)T.H * INV_CELL_AREA_NUM);
    return T.cell[(size_t)j * T.W + i] * scale / sin_t;
}
bool env_sample(const Scene& s, float u1, float u2, float u3, float u4, V3* dir, float* pdf) {
    const EnvTables& T = s.tables;
    uint32_t j = cdf_find(T.marginal.data(), T.H, u1);
    uint32_t i = cdf_find(&T.conditional[(size_t)j * (T.W + 1)], T.W, u2);
    float theta = ((float)j + u3) * (PI_F / (float)T.H);
    float phi = ((float)i + u4) * (2.0f * PI_F / (float)T.W);
    float st = std::sin(theta), ct = std::cos(theta);
    if (!(st > 0.0f)) return false;
    *dir = dir_from_angles(st, ct, phi);
    *pdf = cell_density(T, j, i, st);
    return *pdf > 0.0f;
}
float env_pdf(const Scene& s, V3 d) {
    const EnvTables& T = s.tables;
    float theta = std::acos(-d.y);
    float phi = std::atan2(-d.z, d.x) + PI_F;
    float fj = theta * ((float)T.H / PI_F);
    float fi = phi * ((float)T.W / (2.0f * PI_F));
    uint32_t j = (uint32_t)std::min(std::max(fj, 0.0f), (float)(T.H - 1));
    uint32_t i = (uint32_t)std::min(std::max(fi, 0.0f), (float)(T.W - 1));
    float st = std::sin(theta);
    if (!(st > 0.0f)) return 0.0f;
    return cell_density(T, j, i, st);
}

// ------------------------------------------------------------- materials --
enum { M_LAMB = 0, M_METAL = 1, M_DIEL = 2, M_EMIT = 3, M_LBSDF = 4, M_MICRO = 5, M_MIX = 6 };

// local_to_world (math.rs:50-60).  QUIRK: cgmath's Matrix3::new is column
// major, so the matrix built there has rows ns, nss, n and M*h = (ns.h, nss.h, n.h).
inline V3 local_to_world_mul(V3 n, V3 h) {
    V3 ns = std::isnormal(n.x) ? normalize(v3(n.y, -n.x, 0.0f)) : normalize(v3(0.0f, -n.z, n.y));
    V3 nss = cross(n, ns);
    return v3(dot(ns, h), dot(nss, h), dot(n, h));
}
inline float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline V3 lerpv(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }

// MicrofacetBSDF::bsdf (microfacet.rs:120-208)
V3 micro_bsdf(const orc_material& m, V3 n, V3 wo, V3 wi) {
    V3 color = load3(m.color);
    float n_dot_wi = dot(n, wi), n_dot_wo = dot(n, wo);
    bool wi_out = !std::signbit(n_dot_wi), wo_out = !std::signbit(n_dot_wo);
    if (!m.transparent && (!wi_out || !wo_out)) return v3(0, 0, 0);
    float m2 = m.roughness * m.roughness;
    if (wi_out == wo_out) {
        V3 h = normalize(wi + wo);
        float wo_dot_h = dot(wo, h), n_dot_h = dot(n, h), nh2 = powi2(n_dot_h);
        float d = std::exp((nh2 - 1.0f) / (m2 * nh2)) / (m2 * PI_F * nh2 * nh2);
        V3 f;
        if (!wi_out && std::sqrt(1.0f - wo_dot_h * wo_dot_h) * m.ir > 1.0f) {
            f = v3(1, 1, 1);
        } else {
            float f0s = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
            V3 f0 = lerpv(v3(f0s, f0s, f0s), color, m.metallic);
            f = f0 + (v3(1, 1, 1) - f0) * powi5(1.0f - wo_dot_h);
        }
        float g = std::fmin(n_dot_wi * n_dot_h, n_dot_wo * n_dot_h);
        g = (2.0f * g) / wo_dot_h;
        g = std::fmin(g, 1.0f);
        V3 spec = d * f * g / (4.0f * n_dot_wo * n_dot_wi);
        if (m.transparent) return spec;
        V3 diffuse = mul(v3(1, 1, 1) - f, color) / PI_F;
        return spec + diffuse;
    }
    float eta_t = wo_out ? m.ir : 1.0f / m.ir;
    V3 h = normalize(wi * eta_t + wo);
    float wi_dot_h = dot(wi, h), wo_dot_h = dot(wo, h), n_dot_h = dot(n, h), nh2 = powi2(n_dot_h);
    float d = std::exp((nh2 - 1.0f) / (m2 * nh2)) / (m2 * PI_F * nh2 * nh2);
    float f0s = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
    V3 f0 = lerpv(v3(f0s, f0s, f0s), color, m.metallic);
    V3 f = f0 + (v3(1, 1, 1) - f0) * powi5(1.0f - std::fabs(wi_dot_h));
    float g = std::fmin(std::fabs(n_dot_wi * n_dot_h), std::fabs(n_dot_wo * n_dot_h));
    g = (2.0f * g) / std::fabs(wo_dot_h);
    g = std::fmin(g, 1.0f);
    float lead = std::fabs(wi_dot_h * wo_dot_h / (n_dot_wi * n_dot_wo));
    V3 btdf = lead * (d * (v3(1, 1, 1) - f) * g / powi2(eta_t * wi_dot_h + wo_dot_h));
    return mul(btdf, color);
}
inline float signum(float x) {
    if (std::isnan(x)) return x;
    return std::signbit(x) ? -1.0f : 1.0f;
}
// MicrofacetBSDF::sample (microfacet.rs:222-313)
bool micro_sample(const orc_material& m, V3 n, V3 wo, Pcg32& rng, V3* wi_out, float* p_out) {
    V3 color = load3(m.color);
    float m2 = m.roughness * m.roughness;
    float f0 = powi2((m.ir - 1.0f) / (m.ir + 1.0f));
    float mean = (color.x + color.y + color.z) / 3.0f;
    float f = (1.0f - m.metallic) * f0 + m.metallic * mean;
    f = lerpf(f, 1.0f, 0.2f);
    float eta_t = dot(wo, n) > 0.0f ? m.ir : 1.0f / m.ir;
    auto beckmann = [&](Pcg32& r) {
        float theta = std::atan(std::sqrt(m2 * -std::log(r.uniform())));
        float st = std::sin(theta), ct = std::cos(theta);
        float x, y;
        unit_circle(r, &x, &y);
        return local_to_world_mul(n, v3(x * st, y * st, ct));
    };
    auto beckmann_pdf = [&](V3 h) {
        float ct = std::fabs(dot(h, n));
        float st = std::sqrt(1.0f - ct * ct);
        return (1.0f / (PI_F * m2 * powi3(ct))) * std::exp(-powi2(st / ct) / m2);
    };
    V3 wi;
    if (rng.uniform() < f) {
        V3 h = beckmann(rng);
        wi = -reflect(wo, h);
    } else if (!m.transparent) {
        float x, y;
        unit_disc(rng, &x, &y);
        float z = std::sqrt(1.0f - x * x - y * y);
        wi = local_to_world_mul(n, v3(x, y, z));
    } else {
        V3 h = beckmann(rng);
        float cos_to = dot(h, wo);
        V3 wo_perp = wo - h * cos_to;
        V3 wi_perp = -wo_perp / eta_t;
        float sin2_ti = mag2(wi_perp);
        if (sin2_ti > 1.0f) return false;
        float cos_ti = std::sqrt(1.0f - sin2_ti);
        wi = -signum(cos_to) * cos_ti * h + wi_perp;
    }
    float p = 0.0f;
    {
        V3 h = normalize(wi + wo);
        float p_h = beckmann_pdf(h);
        p += f * p_h / (4.0f * std::fabs(dot(h, wo)));
    }
    if (!m.transparent) {
        p += (1.0f - f) * std::fmax(dot(wi, n), 0.0f) / PI_F;
    } else if (!std::signbit(dot(wo, n)) != !std::signbit(dot(wi, n))) {
        V3 h = normalize(wi * eta_t + wo);
        float p_h = beckmann_pdf(h);
        float h_dot_wo = dot(h, wo), h_dot_wi = dot(h, wi);
        float jac = std::fabs(h_dot_wo) / powi2(eta_t * h_dot_wi + h_dot_wo);
        p += (1.0f - f) * p_h * jac;
    }
    if (p == 0.0f) return false;
    *wi_out = wi;
    *p_out = p;
    return true;
}

// Material::scatter for the closed set (simple.rs, traits.rs:19-41).
// Returns true if a continuation ray was produced.
// ImageTexture::sample (texture.rs:82-98) with nearest_sample / bilinear_sample (:52-78)
V3 tex_sample(const Scene& s, int tix, float u, float v) {
    const Texture& t = s.textures[tix];
    const size_t W = t.w, H = t.h, len = W * H;
    auto px = [&](size_t i) { return v3(t.img[3 * i], t.img[3 * i + 1], t.img[3 * i + 2]); };
    if (u < 0.0f) u -= std::trunc(u) - 1.0f;
    if (v < 0.0f) v -= std::trunc(v) - 1.0f;
    const float x = std::fmod(u, 1.0f) * (float)W;
    const float y = (1.0f - std::fmod(v, 1.0f)) * (float)H;
    const size_t x0 = std::min(sat_usize(x), W - 1), y0 = std::min(sat_usize(y), H - 1);
    if (t.sampling == 0) return px((y0 * W + x0) % len);
    const float ax = x - (float)x0, ay = y - (float)y0;
    return lerp3(lerp3(px((y0 * W + x0) % len), px((y0 * W + x0 + 1) % len), ax),
                 lerp3(px(((y0 + 1) * W + x0) % len), px(((y0 + 1) * W + x0 + 1) % len), ax), ay);
}
// Lambertian textures (simple.rs:102-133): the albedo and the scatter normal from the hit's uv
// MixMaterial::scatter (legacy voidray/src/common/materials.rs:195-203):
// `gen_range(0.0..1.0) >= factor` picks the first child, else the second;
// one draw per level of mixing, before the child's own draws.
void resolve_mix(const Scene& s, orc_material& m, Pcg32& rng) {
    for (int d = 0; m.kind == M_MIX && d < 8; ++d) {
        float u = rng.uniform();
        m = s.materials[u >= m.mix_factor ? m.mix_first : m.mix_second];
    }
}

void apply_textures(const Scene& s, orc_material& m, Hit& hit) {
    if (m.albedo_texture >= 0) {
        V3 c = tex_sample(s, m.albedo_texture, hit.uvx, hit.uvy);
        m.color[0] = c.x;
        m.color[1] = c.y;
        m.color[2] = c.z;
    }
    if (m.normal_texture >= 0) hit.snormal = tex_sample(s, m.normal_texture, hit.uvx, hit.uvy);
}

bool scatter(const orc_material& m, const Ray& ray, const Hit& hit, Pcg32& rng, V3* att, Ray* out) {
    switch (m.kind) {
    case M_LAMB: {  // simple.rs:102-133
        V3 normal = hit.snormal;
        V3 dir = normal + unit_sphere(rng);
        if (near_zero(dir)) dir = normal;
        *out = Ray{hit.point, normalize(dir)};
        *att = load3(m.color);
        return true;
    }
    case M_METAL: {  // simple.rs:140-161; the rejection loop is bounded
        V3 reflected = normalize(reflect(ray.d, hit.normal));
        for (int i = 0; i < REJECT_TRIES; ++i) {
            V3 d = normalize(reflected + m.fuzz * unit_sphere(rng));
            if (dot(d, hit.normal) > 0.0f) {
                *out = Ray{hit.point, d};
                *att = load3(m.color);
                return true;
            }
        }
        *att = v3(0, 0, 0);
        return false;
    }
    case M_DIEL: {  // simple.rs:200-232
        float rr = hit.front_face ? 1.0f / m.ir : m.ir;
        V3 ud = normalize(ray.d);
        float cos_t = std::fmin(dot(hit.normal, -ud), 1.0f);
        float sin_t = std::sqrt(1.0f - cos_t * cos_t);
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
        *out = Ray{hit.point, normalize(dir)};
        *att = v3(1, 1, 1);
        return true;
    }
    case M_EMIT:  // simple.rs:175-185
        *att = load3(m.color);
        return false;
    case M_LBSDF: {  // simple.rs:64-81 + traits.rs:23-40 (pdf 1.0, as the reference)
        V3 wi = normalize(unit_sphere(rng));
        V3 f = load3(m.color) / PI_F;
        *out = Ray{ray.o + ray.d * hit.t, normalize(wi)};
        *att = f * std::fabs(dot(wi, hit.normal)) * (1.0f / 1.0f);
        return true;
    }
    case M_MICRO: {  // traits.rs:23-40 with microfacet.rs
        V3 wo = normalize(ray.d);
        V3 wi;
        float pdf;
        if (micro_sample(m, hit.normal, wo, rng, &wi, &pdf)) {
            V3 f = micro_bsdf(m, hit.normal, wo, wi);
            *out = Ray{ray.o + ray.d * hit.t, normalize(wi)};
            *att = f * std::fabs(dot(wi, hit.normal)) * (1.0f / pdf);
            return true;
        }
        *att = v3(0, 0, 0);
        return false;
    }
    }
    *att = v3(0, 0, 0);
    return false;
}

// --------------------------------------------------------------- camera ---
// cast_ray (camera.rs:69-82).  QUIRK: the direction is normalised twice
// (camera.rs:81 and Ray::new).
Ray cast_ray(const Scene& s, float x, float y, Pcg32& rng) {
    V3 origin = s.c_origin;
    V3 nd = s.c_d * s.c_dir + x * s.c_right + y * s.c_up;
    if (s.c_dof) {
        V3 focal_point = origin + normalize(nd) * s.c_focal;
        float dx, dy;
        unit_disc(rng, &dx, &dy);
        origin = origin + (dx * s.c_right + dy * s.c_up) * s.c_aperture;
        nd = focal_point - origin;
    }
    return Ray{origin, normalize(normalize(nd))};
}

struct Counters {
    uint64_t extend = 0, shadow = 0;
};

inline float max3(V3 a) { return std::fmax(a.x, std::fmax(a.y, a.z)); }

// Russian roulette (extension): after a scatter at depth >= rr_depth the
// continuation survives with q = min(max(T*att), 0.95) and att is divided by q.
inline bool russian_roulette(const orc_settings& st, uint32_t depth, V3& att, V3& tn, Pcg32& rng) {
    if (st.rr_depth == 0 || depth < st.rr_depth) return true;
    float q = std::fmin(max3(tn), 0.95f);
    float u = rng.uniform();
    if (!(u < q)) return false;
    att = att / q;
    tn = tn / q;
    return true;
}

// trace_ray_internal (tracer.rs:19-56), recursive as in the reference.
V3 trace_ref(const Scene& s, const orc_settings& st, const Ray& ray, uint32_t depth, V3 thr, Pcg32& rng,
             Counters& c) {
    V3 color = v3(0, 0, 0);
    if (depth < st.max_bounces) {
        c.extend++;
        HitPair hp = scene_hit(s, ray);
        if (!hp.ok) return env_eval(s, ray.d);
        Hit hit = hp.best;
        orc_material m = s.materials[s.surface_material[surface_of_prim(s, hit.prim)]];
        resolve_mix(s, m, rng);
        apply_textures(s, m, hit);
        V3 att;
        Ray sc;
        bool has;
        if (st.render_mode == 1) {
            has = scatter(m, ray, hit, rng, &att, &sc);
        } else {  // RenderMode::Normal (tracer.rs:40)
            V3 nn = normalize(hit.normal);
            att = (0.5f * nn) + v3(1, 1, 1) * 0.5f;
            has = false;
        }
        V3 delta;
        if (has) {
            V3 tn = mul(thr, att);
            V3 next = v3(0, 0, 0);
            if (russian_roulette(st, depth, att, tn, rng)) next = trace_ref(s, st, sc, depth + 1, tn, rng, c);
            delta = mul(att, next);
        } else {
            delta = att;
        }
        color = color + clampc(delta, st.firefly_clamp);
    }
    return color;
}

// Production estimator (extension): forward throughput, environment next
// event estimation with MIS at Lambertian vertices, RR, clamp per contribution.
V3 trace_nee(const Scene& s, const orc_settings& st, Ray ray, Pcg32& rng, Counters& c) {
    V3 T = v3(1, 1, 1), L = v3(0, 0, 0);
    bool specular = true;
    float prev_pdf = 0.0f;
    const bool env_is = s.has_tables;
    for (uint32_t depth = 0; depth < st.max_bounces; ++depth) {
        c.extend++;
        HitPair hp = scene_hit(s, ray);
        if (!hp.ok) {
            V3 le = env_eval(s, ray.d);
            float w = 1.0f;
            if (!specular && env_is) {
                float pl = env_pdf(s, ray.d);
                float a = prev_pdf * prev_pdf, b = pl * pl;
                w = a / (a + b);
            }
            L = L + clampc(mul(T, le) * w, st.firefly_clamp);
            break;
        }
        Hit hit = hp.best;
        orc_material m = s.materials[s.surface_material[surface_of_prim(s, hit.prim)]];
        resolve_mix(s, m, rng);
        apply_textures(s, m, hit);
        if (st.render_mode != 1) {
            V3 nn = normalize(hit.normal);
            L = L + clampc(mul(T, (0.5f * nn) + v3(1, 1, 1) * 0.5f), st.firefly_clamp);
            break;
        }
        const bool lamb = (m.kind == M_LAMB) && m.normal_texture < 0 &&
                          !(hit.normal.x == 0.0f && hit.normal.y == 0.0f && hit.normal.z == 0.0f);
        if (lamb && env_is) {
            float u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform(), u4 = rng.uniform();
            V3 dl;
            float pl;
            if (env_sample(s, u1, u2, u3, u4, &dl, &pl)) {
                float cosl = dot(hit.normal, dl);
                if (cosl > 0.0f) {
                    float pb = cosl / PI_F;
                    float a = pl * pl, b = pb * pb;
                    float w = a / (a + b);
                    float fscale = cosl / PI_F * w / pl;
                    V3 contrib = mul(mul(T, load3(m.color)), env_eval(s, dl)) * fscale;
                    c.shadow++;
                    HitPair sh = scene_hit(s, Ray{hit.point, dl});
                    if (!sh.ok) L = L + clampc(contrib, st.firefly_clamp);
                }
            }
        }
        V3 att;
        Ray sc;
        if (!scatter(m, ray, hit, rng, &att, &sc)) {
            L = L + clampc(mul(T, att), st.firefly_clamp);
            break;
        }
        T = mul(T, att);
        if (lamb) {
            prev_pdf = dot(hit.normal, sc.d) / PI_F;
            specular = false;
        } else {
            specular = true;
        }
        V3 a2 = att;
        if (!russian_roulette(st, depth, a2, T, rng)) break;
        ray = sc;
    }
    return L;
}

V3 trace_path(const Scene& s, const orc_settings& st, uint32_t W, uint32_t H, uint32_t pixel, uint32_t sample,
              uint64_t seed, Counters& c) {
    // iterative.rs:25-33 (row = index / width, see header)
    uint32_t x = pixel % W, y = pixel / W;
    float d = (float)std::max(W, H);
    float fx = ((float)(2 * x + 1) - (float)W) / d;
    float fy = ((float)(2 * (H - y) - 1) - (float)H) / d;
    Pcg32 rng(seed, sample, pixel);
    float lo = -1.0f / d, hi = 1.0f / d;
    float dx = rng.range(lo, hi);
    float dy = rng.range(lo, hi);
    Ray r = cast_ray(s, fx + dx, fy + dy, rng);
    if (st.estimator == 1) return trace_nee(s, st, r, rng, c);
    return trace_ref(s, st, r, 0, v3(1, 1, 1), rng, c);
}

// ------------------------------------------------------------- tonemap ---
// tonemapping.glsl:2-40.  GLSL mat3(...) is column major: M*c = c.x*col0 + ...
V3 glsl_mat3_mul(const float* m, V3 c) {
    V3 c0 = load3(m), c1 = load3(m + 3), c2 = load3(m + 6);
    return c0 * c.x + c1 * c.y + c2 * c.z;
}
V3 tm_aces(V3 c) {
    static const float A[9] = {0.59719f, 0.076f, 0.0284f, 0.35458f, 0.90834f, 0.13383f, 0.04823f, 0.01566f, 0.83777f};
    static const float B[9] = {1.60475f, -0.10208f, -0.00327f, -0.53108f, 1.10813f, -0.07276f, -0.07367f, -0.00605f, 1.07602f};
    c = glsl_mat3_mul(A, c);
    V3 num = v3(c.x * (c.x + 0.0245786f) - 0.000090537f, c.y * (c.y + 0.0245786f) - 0.000090537f,
                c.z * (c.z + 0.0245786f) - 0.000090537f);
    V3 den = v3(c.x * (0.983729f * c.x + 0.432951f) + 0.238081f, c.y * (0.983729f * c.y + 0.432951f) + 0.238081f,
                c.z * (0.983729f * c.z + 0.432951f) + 0.238081f);
    c = v3(num.x / den.x, num.y / den.y, num.z / den.z);
    return glsl_mat3_mul(B, c);
}
V3 tm_reinhard(V3 c) {
    float white = 2.0f;
    float luma = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
    float tml = luma * (1.0f + luma / (white * white)) / (1.0f + luma);
    return c * (tml / luma);
}
inline float filmic1(float x) {
    x = std::fmax(0.0f, x - 0.004f);
    return (x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f);
}
inline float unch1(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}
V3 tm_uncharted2(V3 c) {
    const float W = 11.2f;
    c = c * 2.0f;
    V3 r = v3(unch1(c.x), unch1(c.y), unch1(c.z));
    float white = unch1(W);
    return r / white;
}

}  // namespace

struct orc_scene {
    Scene s;
};

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

orc_scene* orc_scene_create(const orc_scene_desc* d) {
    if (!d) { g_err = "null descriptor"; return nullptr; }
    std::unique_ptr<orc_scene> h(new orc_scene());
    Scene& s = h->s;
    s.materials.assign(d->materials, d->materials + d->num_materials);
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        const orc_texture& td = d->textures[i];
        if (!td.image || !td.width || !td.height) { g_err = "empty texture"; return nullptr; }
        Texture t;
        t.w = td.width;
        t.h = td.height;
        t.sampling = td.sampling;
        t.img.assign(td.image, td.image + 3 * (size_t)td.width * td.height);
        s.textures.push_back(std::move(t));
    }
    for (const orc_material& m : s.materials) {
        if (m.albedo_texture >= (int)d->num_textures || m.normal_texture >= (int)d->num_textures) {
            g_err = "texture index out of range";
            return nullptr;
        }
        if (m.kind == M_MIX && (m.mix_first < 0 || m.mix_first >= (int)d->num_materials || m.mix_second < 0 ||
                                m.mix_second >= (int)d->num_materials)) {
            g_err = "mix child out of range";
            return nullptr;
        }
    }
    uint64_t prim = 0;
    for (uint32_t mi = 0; mi < d->num_meshes; ++mi) {
        const orc_mesh& md = d->meshes[mi];
        Mesh m;
        m.first_prim = (uint32_t)prim;
        m.pos.resize(md.num_vertices);
        m.nrm.resize(md.num_vertices, v3(0, 0, 0));
        m.uv.assign(2 * (size_t)md.num_vertices, 0.0f);
        for (uint32_t v = 0; v < md.num_vertices; ++v) {
            m.pos[v] = load3(md.positions + 3 * v);
            if (md.normals) m.nrm[v] = load3(md.normals + 3 * v);
            if (md.uvs) { m.uv[2 * v] = md.uvs[2 * v]; m.uv[2 * v + 1] = md.uvs[2 * v + 1]; }
        }
        m.idx.assign(md.indices, md.indices + 3 * (size_t)md.num_triangles);
        for (uint32_t i : m.idx)
            if (i >= md.num_vertices) { g_err = "index out of range"; return nullptr; }
        // Mesh::from_buffers (mesh.rs:76-116): face normal (p2-p1)x(p0-p1)
        m.face_n.resize(md.num_triangles);
        for (uint32_t t = 0; t < md.num_triangles; ++t) {
            V3 e1 = m.pos[m.idx[3 * t]] - m.pos[m.idx[3 * t + 1]];
            V3 e2 = m.pos[m.idx[3 * t + 2]] - m.pos[m.idx[3 * t + 1]];
            m.face_n[t] = normalize(cross(e2, e1));
        }
        Aabb b = aabb_default();
        for (const V3& p : m.pos) b = surround(b, Aabb{p, p});
        m.bounds = b;
        prim += md.num_triangles;
        s.meshes.push_back(std::move(m));
    }
    s.num_prims = prim;
    // per-mesh median BVH when more than SMALL_MESH = 4 triangles (mesh.rs:43, 112-114)
    for (Mesh& m : s.meshes) {
        if (m.idx.size() > 4 * 3) {
            std::vector<uint32_t> objs(m.face_n.size());
            for (uint32_t i = 0; i < objs.size(); ++i) objs[i] = i;
            const Mesh* mp = &m;
            auto bounds_ref = [mp](uint32_t t) {
                const uint32_t* ix = &mp->idx[3 * t];
                Aabb b = surround(from_point(mp->pos[ix[0]]), surround(from_point(mp->pos[ix[1]]), from_point(mp->pos[ix[2]])));
                return epsilon_expand(b, 0.001f);
            };
            m.bvh.root = bvh_build(m.bvh, objs, bounds_ref);
            m.has_bvh = true;
        }
    }
    // the surface list: meshes and analytic surfaces at their surface indices
    const size_t nsurf = d->num_meshes + (size_t)d->num_analytics;
    s.surf_mesh.assign(nsurf, -1);
    s.surf_analytic.assign(nsurf, -1);
    for (uint32_t mi = 0; mi < d->num_meshes; ++mi) {
        const uint32_t si = d->meshes[mi].surface;
        if (si >= nsurf || s.surf_mesh[si] >= 0) { g_err = "bad mesh surface index"; return nullptr; }
        s.surf_mesh[si] = (int)mi;
        s.mesh_surface.push_back((int)si);
    }
    for (uint32_t ai = 0; ai < d->num_analytics; ++ai) {
        const orc_analytic& ad = d->analytics[ai];
        if (ad.surface >= nsurf || s.surf_mesh[ad.surface] >= 0 || s.surf_analytic[ad.surface] >= 0) {
            g_err = "bad analytic surface index";
            return nullptr;
        }
        s.surf_analytic[ad.surface] = (int)ai;
        s.analytics.push_back(Analytic{ad.kind, load3(ad.center), ad.radius, ad.height, (int)ad.surface});
    }
    // QUIRK (scene.rs:283-285, 377-378): the top-level BVH is over surface
    // indices and the hit surface index is used as the object index.
    s.surface_material.assign(nsurf, -1);
    for (size_t si = 0; si < nsurf; ++si) {
        if (si >= d->num_objects) { g_err = "surface without an object at the same index"; return nullptr; }
        uint32_t mat = d->objects[si].material;
        if (mat >= d->num_materials) { g_err = "material index out of range"; return nullptr; }
        s.surface_material[si] = (int)mat;
    }
    {
        std::vector<uint32_t> objs(nsurf);
        for (uint32_t i = 0; i < objs.size(); ++i) objs[i] = i;
        const Scene* sp = &s;
        // Bounded::bounds: mesh box, sphere center +- r, ground plane infinite in x, z (surfaces.rs:37-43, 107-114)
        auto bounds_ref = [sp](uint32_t i) {
            if (sp->surf_mesh[i] >= 0) return sp->meshes[sp->surf_mesh[i]].bounds;
            const Analytic& a = sp->analytics[sp->surf_analytic[i]];
            if (a.kind == 1) {
                V3 rr = v3(a.radius, a.radius, a.radius);
                return Aabb{a.center - rr, a.center + rr};
            }
            return Aabb{v3(-INF_F, a.height - 0.0001f, -INF_F), v3(INF_F, a.height + 0.0001f, INF_F)};
        };
        s.top.root = objs.empty() ? -1 : bvh_build(s.top, objs, bounds_ref);
    }
    s.env = d->env;
    if (s.env.kind == 2) {
        if (!d->env.image || d->env.width == 0 || d->env.height == 0) { g_err = "bad hdri"; return nullptr; }
        s.env_img.assign(d->env.image, d->env.image + 3 * (size_t)d->env.width * d->env.height);
        s.env.image = nullptr;
        if (d->env.importance_sample) {
            build_env_tables(s);
            s.has_tables = true;
        }
    }
    // Camera::build_acceleration (camera.rs:38-53)
    const orc_camera& c = d->camera;
    s.c_origin = load3(c.eye);
    s.c_dir = load3(c.direction);
    s.c_up = load3(c.up);
    s.c_d = 1.0f / std::tan(c.fov / 2.0f);
    s.c_right = normalize(cross(s.c_dir, s.c_up));
    s.c_dof = c.has_dof != 0;
    if (s.c_dof) {
        s.c_aperture = c.aperture;
        s.c_focal = dot(load3(c.focal_point) - s.c_origin, s.c_dir);
    }
    return h.release();
}

void orc_scene_destroy(orc_scene* s) { delete s; }

int32_t orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void set_threads(int32_t t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

static HitPair brute(const Scene& s, const Ray& r, float tmin) {
    HitPair hp;
    for (size_t a = 0; a < s.analytics.size(); ++a) {
        HitPair ha = analytic_hit(s, (int)a, r, tmin, INF_F);
        if (ha.ok && (!hp.ok || ha.best.t < hp.best.t)) hp = ha;
    }
    for (const Mesh& m : s.meshes) {
        uint32_t nt = (uint32_t)m.face_n.size();
        for (uint32_t i = 0; i < nt; ++i) {
            Hit h;
            if (triangle_hit(m, i, r, tmin, h)) {
                if (!hp.ok || h.t < hp.best.t) {
                    if (hp.ok) note_second(hp, hp.best.t);
                    hp.best = h;
                    hp.ok = true;
                } else {
                    note_second(hp, h.t);
                }
            }
        }
    }
    return hp;
}

void orc_intersect(const orc_scene* sh, const orc_ray* rays, uint64_t n, orc_hit* hits, float* second_t,
                   int32_t mode, int32_t threads) {
    const Scene& s = sh->s;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const orc_ray& q = rays[i];
        Ray r{load3(q.org), load3(q.dir)};
        HitPair hp = (mode == 1) ? brute(s, r, q.tmin) : scene_hit(s, r, q.tmin, INF_F);
        orc_hit& o = hits[i];
        bool ok = hp.ok;
        if (mode == 2 && ok && !(hp.best.t < q.tmax)) ok = false;
        if (mode != 2 && ok && !(hp.best.t < q.tmax)) ok = false;
        if (ok) {
            o.prim = hp.best.prim;
            o.t = hp.best.t;
            o.u = hp.best.bu;
            o.v = hp.best.bv;
        } else {
            o.prim = 0xFFFFFFFFu;
            o.t = INF_F;
            o.u = 0.0f;
            o.v = 0.0f;
        }
        if (second_t) second_t[i] = hp.second;
    }
}

int32_t orc_triangle_hit(const orc_scene* sh, uint32_t prim, const orc_ray* q, float* t, float* u, float* v) {
    const Scene& s = sh->s;
    int si = mesh_of_prim(s, prim);
    if (si < 0) return 0;
    const Mesh& m = s.meshes[si];
    Hit h;
    Ray r{load3(q->org), load3(q->dir)};
    if (!triangle_hit(m, prim - m.first_prim, r, q->tmin, h)) return 0;
    *t = h.t;
    *u = h.bu;
    *v = h.bv;
    return 1;
}

int32_t orc_reintersect_f64(const orc_scene* sh, uint32_t prim, const orc_ray* q, double* t, double* u, double* v) {
    const Scene& s = sh->s;
    int si = mesh_of_prim(s, prim);
    if (si < 0) return 0;
    const Mesh& m = s.meshes[si];
    const uint32_t* ix = &m.idx[3 * (prim - m.first_prim)];
    double p[3][3];
    for (int k = 0; k < 3; ++k) {
        V3 pp = m.pos[ix[k]];
        p[k][0] = pp.x; p[k][1] = pp.y; p[k][2] = pp.z;
    }
    double o[3] = {q->org[0], q->org[1], q->org[2]}, d[3] = {q->dir[0], q->dir[1], q->dir[2]};
    double e1[3], e2[3], s3[3], h[3], qq[3];
    for (int k = 0; k < 3; ++k) { e1[k] = p[1][k] - p[0][k]; e2[k] = p[2][k] - p[0][k]; s3[k] = o[k] - p[0][k]; }
    auto crs = [](const double* a, const double* b, double* c) {
        c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto dt = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    crs(d, e2, h);
    double a = dt(e1, h);
    if (a == 0.0) return 0;
    double f = 1.0 / a;
    *u = f * dt(s3, h);
    crs(s3, e1, qq);
    *v = f * dt(d, qq);
    *t = f * dt(e2, qq);
    return 1;
}

void orc_render(const orc_scene* sh, const orc_settings* st, uint32_t samples, float* rgba, uint32_t W, uint32_t H,
                uint64_t seed, uint32_t first_sample, uint32_t pb, uint32_t pe, int32_t threads, uint64_t* rays_out) {
    const Scene& s = sh->s;
    set_threads(threads);
    uint32_t np = W * H;
    if (pe == 0 || pe > np) pe = np;
    uint64_t ext = 0, shd = 0;
    const float inv_total = 1.0f / (float)st->total_samples;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : ext, shd)
    for (int64_t p = (int64_t)pb; p < (int64_t)pe; ++p) {
        Counters c;
        V3 color = v3(0, 0, 0);
        for (uint32_t k = 0; k < samples; ++k)
            color = color + trace_path(s, *st, W, H, (uint32_t)p, first_sample + k, seed, c);
        color = color * inv_total;  // iterative.rs:45
        float* px = rgba + 4 * (size_t)p;
        px[0] += color.x;
        px[1] += color.y;
        px[2] += color.z;
        px[3] += 1.0f;  // Color::a() == 1 (color.rs:54-56)
        ext += c.extend;
        shd += c.shadow;
    }
    if (rays_out) {
        rays_out[0] = ext;
        rays_out[1] = shd;
    }
}

void orc_trace_path(const orc_scene* sh, const orc_settings* st, uint32_t W, uint32_t H, uint32_t pixel,
                    uint32_t sample, uint64_t seed, float* rgb) {
    Counters c;
    V3 r = trace_path(sh->s, *st, W, H, pixel, sample, seed, c);
    rgb[0] = r.x;
    rgb[1] = r.y;
    rgb[2] = r.z;
}

void orc_tonemap(const float* in, float* out, uint64_t n, int32_t tonemap, float gamma, float exposure, float scale) {
    float ex = std::pow(2.0f, exposure);
    for (uint64_t i = 0; i < n; ++i) {
        const float* p = in + 4 * i;
        V3 c = v3(p[0] * scale, p[1] * scale, p[2] * scale) * ex;
        switch (tonemap) {
        case 1: c = tm_aces(c); break;
        case 2: c = tm_reinhard(c); break;
        case 3: c = v3(filmic1(c.x), filmic1(c.y), filmic1(c.z)); break;
        case 4: c = tm_uncharted2(c); break;
        default: break;
        }
        float g = 1.0f / gamma;
        float* o = out + 4 * i;
        o[0] = std::pow(c.x, g);
        o[1] = std::pow(c.y, g);
        o[2] = std::pow(c.z, g);
        o[3] = 1.0f;
    }
}

// Legacy viewport (voidray/src/shaders/viewport_fragment.glsl:27-67,
// tonemapping.glsl:17-45): its numbering, linear exposure, Filmic without
// gamma, alpha kept when transparent.
void orc_tonemap_legacy(const float* in, float* out, uint64_t n, int32_t tonemap, float gamma, float exposure,
                        int32_t transparent, float scale) {
    if (tonemap == 6) gamma = 1.0f;
    for (uint64_t i = 0; i < n; ++i) {
        const float* p = in + 4 * i;
        V3 c = v3(p[0] * scale, p[1] * scale, p[2] * scale) * exposure;
        switch (tonemap) {
        case 1: c = tm_aces(c); break;
        case 2: {
            const float e = 1.5f;
            c = v3(c.x * (e / (1.0f + c.x / e)), c.y * (e / (1.0f + c.y / e)), c.z * (e / (1.0f + c.z / e)));
            break;
        }
        case 3: {
            float luma = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
            float tml = luma / (1.0f + luma);
            c = c * (tml / luma);
            break;
        }
        case 4: c = tm_reinhard(c); break;
        case 5:
            c = v3(std::exp(-1.0f / (2.72f * c.x + 0.15f)), std::exp(-1.0f / (2.72f * c.y + 0.15f)),
                   std::exp(-1.0f / (2.72f * c.z + 0.15f)));
            break;
        case 6: c = v3(filmic1(c.x), filmic1(c.y), filmic1(c.z)); break;
        case 7: c = tm_uncharted2(c); break;
        default: break;
        }
        float g = 1.0f / gamma;
        float* o = out + 4 * i;
        o[0] = std::pow(c.x, g);
        o[1] = std::pow(c.y, g);
        o[2] = std::pow(c.z, g);
        o[3] = transparent ? p[3] * scale : 1.0f;
    }
}

void orc_env_eval(const orc_scene* sh, const float* dir, float* rgb) {
    V3 c = env_eval(sh->s, load3(dir));
    rgb[0] = c.x;
    rgb[1] = c.y;
    rgb[2] = c.z;
}

int32_t orc_env_sample(const orc_scene* sh, const float* u4, float* dir, float* pdf) {
    if (!sh->s.has_tables) return 0;
    V3 d;
    if (!env_sample(sh->s, u4[0], u4[1], u4[2], u4[3], &d, pdf)) return 0;
    dir[0] = d.x;
    dir[1] = d.y;
    dir[2] = d.z;
    return 1;
}

float orc_env_pdf(const orc_scene* sh, const float* dir) {
    if (!sh->s.has_tables) return 0.0f;
    return env_pdf(sh->s, load3(dir));
}

int32_t orc_env_tables(const orc_scene* sh, float* marginal, float* conditional, float* cell) {
    if (!sh->s.has_tables) return 0;
    const EnvTables& T = sh->s.tables;
    std::copy(T.marginal.begin(), T.marginal.end(), marginal);
    std::copy(T.conditional.begin(), T.conditional.end(), conditional);
    std::copy(T.cell.begin(), T.cell.end(), cell);
    return 1;
}

void orc_pcg32(uint64_t seed, uint32_t sample, uint32_t pixel, uint32_t n, uint32_t* out) {
    Pcg32 r(seed, sample, pixel);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next();
}

void orc_sampler(uint64_t seed, uint32_t sample, uint32_t pixel, int32_t kind, uint32_t n, float* out) {
    Pcg32 r(seed, sample, pixel);
    for (uint32_t i = 0; i < n; ++i) {
        float* o = out + 3 * i;
        if (kind == 0) {
            V3 v = unit_sphere(r);
            o[0] = v.x; o[1] = v.y; o[2] = v.z;
        } else if (kind == 1) {
            unit_disc(r, &o[0], &o[1]);
            o[2] = 0.0f;
        } else if (kind == 2) {
            unit_circle(r, &o[0], &o[1]);
            o[2] = 0.0f;
        } else {
            o[0] = r.uniform(); o[1] = 0.0f; o[2] = 0.0f;
        }
    }
}

int32_t orc_aabb_hit(const float* bmin, const float* bmax, const orc_ray* q, float t_min, float t_max) {
    Aabb b{load3(bmin), load3(bmax)};
    return aabb_hit(b, Ray{load3(q->org), load3(q->dir)}, t_min, t_max) ? 1 : 0;
}

uint64_t orc_num_triangles(const orc_scene* s) { return s->s.num_prims; }

}  // extern "C"
