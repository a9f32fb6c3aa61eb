// vr_build.cpp — host-side scene lowering: binned-SAH BVH2 builder,
// flattening to the 16-byte-aligned node / triangle arrays the traversal
// kernels read with 128-bit loads, shading records, camera and environment
// importance-sampling tables.
//
// Replaces Scene::build_acceleration (voidray_renderer/src/core/scene.rs:163-178)
// and the per-mesh BvhNode::from_list (core/bvh.rs:48-130, a median split).
// The two-level surface/mesh structure of the reference is flattened into one
// BVH over all triangles, each carrying its mesh's material; closest-hit
// results do not depend on the tree (only exact ties in t may resolve
// differently).  Compiled with -ffp-contract=off: face normals and edge
// vectors round exactly as the reference computes them.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <future>
#include <system_error>
#include <thread>

#include "vr_host.h"

namespace vr {
namespace {

struct PrimRef {
    float lo[3], hi[3], c[3];
    uint32_t id;
};
struct BNode {
    float lo[3], hi[3];
    int32_t left = -1, right = -1;  // children (inner) ; -1 for leaves
    uint32_t first = 0, count = 0;  // leaf range in the prim order
};
struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float* l, const float* h) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], l[a]); hi[a] = std::max(hi[a], h[a]); }
    }
    void growp(const float* p) { grow(p, p); }
    double area() const {
        double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        if (!(dx >= 0) || !(dy >= 0) || !(dz >= 0)) return 0.0;
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

constexpr int DEPTH_LIMIT = 62;  // keeps the BVH2 traversal stack (64 entries) in bounds
constexpr int WIDE_STACK = 96;   // entries of the 4-wide traversal's stack
constexpr double C_TRAV = 1.0, C_ISECT = 1.0;

// Threads the BVH build may use: VR_BUILD_THREADS when set (>= 1), else the
// host's hardware threads.  The tree does not depend on it.
unsigned build_threads() {
    static const unsigned n = [] {
        if (const char* v = std::getenv("VR_BUILD_THREADS")) {
            const long k = std::strtol(v, nullptr, 10);
            if (k >= 1) return (unsigned)std::min(k, 1024L);
        }
        const unsigned hw = std::thread::hardware_concurrency();
        return hw ? hw : 1u;
    }();
    return n;
}

// Runs body(chunk, begin, end) over [b, e) cut into `chunks` pieces, the
// pieces after the first on their own threads.
template <class F>
void for_chunks(uint32_t b, uint32_t e, int chunks, F&& body) {
    std::vector<std::future<void>> tasks;
    const uint64_t n = e - b;
    auto edge = [&](int c) { return b + (uint32_t)(n * (uint64_t)c / (uint64_t)chunks); };
    for (int c = 1; c < chunks; ++c) {
        try {
            tasks.push_back(std::async(std::launch::async, [&body, c, lo = edge(c), hi = edge(c + 1)] {
                body(c, lo, hi);
            }));
        } catch (const std::system_error&) {
            body(c, edge(c), edge(c + 1));
        }
    }
    body(0, edge(0), edge(1));
    for (auto& t : tasks) t.get();
}

// Pieces for a pass over n records: one below 2^16, else up to one per
// hardware thread.  Every parallel pass here either writes disjoint slots or
// reduces by min / max / integer sums, exact in any order, so no result
// depends on the number of pieces.
int chunks_for(uint64_t n) {
    if (n < (1u << 16)) return 1;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(build_threads(), n >> 15));
}

struct Builder {
    std::vector<PrimRef>& refs;
    uint32_t max_leaf;
    int nbins;
    std::vector<BNode> nodes;
    uint32_t max_depth = 0;
    Builder(std::vector<PrimRef>& r, uint32_t ml, int nb) : refs(r), max_leaf(ml), nbins(nb) {}

    static int ceil_log2(uint64_t n) {
        int k = 0;
        while ((1ull << k) < n) ++k;
        return k;
    }

    // Bin of a centroid coordinate; total for every float (an extent that
    // overflowed to infinity makes the product NaN, which lands in bin 0).
    int bin_of(float c, float lo, float scale) const {
        const float f = (c - lo) * scale;
        if (!(f > 0.0f)) return 0;
        if (f >= (float)nbins) return nbins - 1;
        return (int)f;
    }

    int make_leaf(uint32_t b, uint32_t e, const Box& bx) {
        BNode n;
        std::memcpy(n.lo, bx.lo, sizeof n.lo);
        std::memcpy(n.hi, bx.hi, sizeof n.hi);
        n.first = b;
        n.count = e - b;
        nodes.push_back(n);
        return (int)nodes.size() - 1;
    }

    // Builds [b, e) and returns its node index.
    int build(uint32_t b, uint32_t e, int depth) {
        max_depth = std::max<uint32_t>(max_depth, (uint32_t)depth);
        Box bx;
        uint32_t mid = 0;
        if (!split(b, e, depth, bx, mid)) return make_leaf(b, e, bx);
        BNode node;
        std::memcpy(node.lo, bx.lo, sizeof node.lo);
        std::memcpy(node.hi, bx.hi, sizeof node.hi);
        nodes.push_back(node);
        const int self = (int)nodes.size() - 1;
        const int l = build(b, mid, depth + 1);
        const int r = build(mid, e, depth + 1);
        nodes[self].left = l;
        nodes[self].right = r;
        return self;
    }

    void bounds(uint32_t b, uint32_t e, Box& bx, Box& cb) const {
        const int chunks = chunks_for(e - b);
        std::vector<Box> pb(chunks), pc(chunks);
        for_chunks(b, e, chunks, [&](int c, uint32_t lo, uint32_t hi) {
            for (uint32_t i = lo; i < hi; ++i) { pb[c].grow(refs[i].lo, refs[i].hi); pc[c].growp(refs[i].c); }
        });
        for (int c = 0; c < chunks; ++c) {
            bx.grow(pb[c].lo, pb[c].hi);
            cb.grow(pc[c].lo, pc[c].hi);
        }
    }

    // Centroid bins of [b, e) on the three axes (axes with scale 0 skipped):
    // bins / counts [3][nbins].
    void bin_centroids(uint32_t b, uint32_t e, const Box& cb, const float scale[3], Box* bins,
                       uint32_t* counts) const {
        const int chunks = chunks_for(e - b);
        const size_t per = 3 * (size_t)nbins;
        std::vector<Box> pb(chunks * per);
        std::vector<uint32_t> pn(chunks * per, 0);
        for_chunks(b, e, chunks, [&](int c, uint32_t lo, uint32_t hi) {
            Box* bb = &pb[c * per];
            uint32_t* bn = &pn[c * per];
            bool on[3];
            for (int a = 0; a < 3; ++a) on[a] = scale[a] > 0.0f;
            for (uint32_t i = lo; i < hi; ++i) {  // one pass over the records, all three axes
                const PrimRef& r = refs[i];
                for (int a = 0; a < 3; ++a) {
                    if (!on[a]) continue;
                    const int k = a * nbins + bin_of(r.c[a], cb.lo[a], scale[a]);
                    bb[k].grow(r.lo, r.hi);
                    bn[k]++;
                }
            }
        });
        for (int c = 0; c < chunks; ++c)
            for (size_t k = 0; k < per; ++k) {
                bins[k].grow(pb[c * per + k].lo, pb[c * per + k].hi);
                counts[k] += pn[c * per + k];
            }
    }

    // Bounds of [b, e) into bx; false when [b, e) becomes a leaf, else the
    // range is partitioned at `mid` by the binned SAH (object median when the
    // centroids are degenerate or the depth guard applies).
    bool split(uint32_t b, uint32_t e, int depth, Box& bx, uint32_t& mid) {
        Box cb;
        bounds(b, e, bx, cb);
        const uint32_t n = e - b;
        if (n == 1) return false;
        const bool force_median = depth + ceil_log2((n + max_leaf - 1) / max_leaf) + 1 >= DEPTH_LIMIT;
        if (force_median && n <= max_leaf) return false;
        int best_axis = -1, best_bin = -1;
        double best_cost = INFINITY;
        const double parent_area = bx.area();
        if (!force_median) {
            float scale[3];
            for (int a = 0; a < 3; ++a) {
                const float ext = cb.hi[a] - cb.lo[a];
                scale[a] = ext > 0.0f ? (float)nbins / ext : 0.0f;
            }
            std::vector<Box> bins3(3 * (size_t)nbins);
            std::vector<uint32_t> counts3(3 * (size_t)nbins, 0);
            bin_centroids(b, e, cb, scale, bins3.data(), counts3.data());
            std::vector<double> right_area(nbins), right_cnt(nbins);
            for (int a = 0; a < 3; ++a) {
                if (!(scale[a] > 0.0f)) continue;
                const Box* bb = &bins3[(size_t)a * nbins];
                const uint32_t* bc = &counts3[(size_t)a * nbins];
                Box acc;
                uint32_t cnt = 0;
                for (int k = nbins - 1; k > 0; --k) {
                    acc.grow(bb[k].lo, bb[k].hi);
                    cnt += bc[k];
                    right_area[k] = acc.area();
                    right_cnt[k] = cnt;
                }
                acc = Box();
                cnt = 0;
                for (int k = 0; k < nbins - 1; ++k) {
                    acc.grow(bb[k].lo, bb[k].hi);
                    cnt += bc[k];
                    if (cnt == 0 || cnt == n) continue;
                    double cost = C_TRAV + C_ISECT * (acc.area() * cnt + right_area[k + 1] * right_cnt[k + 1]) /
                                               std::max(parent_area, 1e-300);
                    if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = k; }
                }
            }
            const double leaf_cost = C_ISECT * n;
            if (n <= max_leaf && (best_axis < 0 || leaf_cost <= best_cost)) return false;
        }
        if (best_axis >= 0) {
            const int a = best_axis;
            const float ext = cb.hi[a] - cb.lo[a];
            const float scale = (float)nbins / ext;
            auto it = std::partition(refs.begin() + b, refs.begin() + e, [&](const PrimRef& r) {
                return bin_of(r.c[a], cb.lo[a], scale) <= best_bin;
            });
            mid = (uint32_t)(it - refs.begin());
        } else {
            // degenerate centroids or depth guard: object median on the widest axis
            int a = 0;
            float w = -1.0f;
            for (int k = 0; k < 3; ++k)
                if (cb.hi[k] - cb.lo[k] > w) { w = cb.hi[k] - cb.lo[k]; a = k; }
            mid = b + n / 2;
            std::nth_element(refs.begin() + b, refs.begin() + mid, refs.begin() + e,
                             [a](const PrimRef& x, const PrimRef& y) { return x.c[a] < y.c[a]; });
        }
        if (mid == b || mid == e) mid = b + n / 2;
        return true;
    }
};

// A subtree in preorder (root first), child indices relative to its array.
struct SubTree {
    std::vector<BNode> nodes;
    uint32_t max_depth = 0;
};

constexpr uint32_t PAR_MIN_PRIMS = 1u << 15;

// Builds [b, e) into `out`.  While the tree is shallower than `spawn_depth`
// and the range holds at least PAR_MIN_PRIMS primitives, the left subtree is
// built on another thread; the halves touch disjoint ranges of `refs`, and the
// result is spliced as [node, left subtree, right subtree], which is exactly
// the array the serial depth-first build produces.
void build_subtree(std::vector<PrimRef>& refs, uint32_t max_leaf, int nbins, uint32_t b, uint32_t e, int depth,
                   int spawn_depth, SubTree& out) {
    Builder B(refs, max_leaf, nbins);
    if (depth >= spawn_depth || e - b < PAR_MIN_PRIMS) {
        B.nodes.reserve((e - b) / 2 + 16);
        B.build(b, e, depth);
        out.nodes = std::move(B.nodes);
        out.max_depth = B.max_depth;
        return;
    }
    Box bx;
    uint32_t mid = 0;
    if (!B.split(b, e, depth, bx, mid)) {
        B.make_leaf(b, e, bx);
        out.nodes = std::move(B.nodes);
        out.max_depth = (uint32_t)depth;
        return;
    }
    SubTree left, right;
    auto build_left = [&] { build_subtree(refs, max_leaf, nbins, b, mid, depth + 1, spawn_depth, left); };
    std::future<void> task;
    try {
        task = std::async(std::launch::async, build_left);
    } catch (const std::system_error&) {
        build_left();  // no thread to be had: build it here
    }
    build_subtree(refs, max_leaf, nbins, mid, e, depth + 1, spawn_depth, right);
    if (task.valid()) task.get();  // rethrows what the other thread threw
    out.nodes.reserve(1 + left.nodes.size() + right.nodes.size());
    BNode self;
    std::memcpy(self.lo, bx.lo, sizeof self.lo);
    std::memcpy(self.hi, bx.hi, sizeof self.hi);
    self.left = 1;
    self.right = 1 + (int32_t)left.nodes.size();
    out.nodes.push_back(self);
    for (const SubTree* t : {&left, &right}) {
        const int32_t off = (int32_t)out.nodes.size();
        for (BNode n : t->nodes) {
            if (n.left >= 0) {
                n.left += off;
                n.right += off;
            }
            out.nodes.push_back(n);
        }
    }
    out.max_depth = std::max<uint32_t>((uint32_t)depth, std::max(left.max_depth, right.max_depth));
}

// Levels of the tree whose subtrees get their own thread: about four
// subtrees per hardware thread.
int spawn_depth_for_host() {
    const unsigned hw = build_threads();
    int d = 2;
    while ((1u << (d - 2)) < hw && d < 8) ++d;
    return hw == 1 ? 0 : d;
}

inline V3 dir_from_angles(float sin_t, float cos_t, float phi) {
    return v3(-sin_t * std::cos(phi), -cos_t, sin_t * std::sin(phi));
}

inline size_t sat_usize(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 18446744073709551615.0f) return SIZE_MAX;
    return (size_t)x;
}

void build_env_tables(HostScene& hs) {
    const SceneView& v = hs.view;
    const uint32_t W = v.env_w, H = v.env_h;
    EnvTables& T = hs.tables;
    T.W = W;
    T.H = H;
    // Rows are evaluated on several threads; every floating-point sum below
    // runs in the serial order (cells row-major, rows top to bottom), so the
    // tables do not depend on the thread count.
    const int chunks = (uint64_t)W * H >= (1u << 16) ? (int)std::min<unsigned>(build_threads(), H) : 1;
    std::vector<double> lum((size_t)W * H);
    for_chunks(0, H, chunks, [&](int, uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; ++j) {
            float theta = ((float)j + 0.5f) * (PI_F / (float)H);
            float st = std::sin(theta), ct = std::cos(theta);
            for (uint32_t i = 0; i < W; ++i) {
                float phi = ((float)i + 0.5f) * (2.0f * PI_F / (float)W);
                V3 c = env_eval_host(v, hs.env_img.data(), dir_from_angles(st, ct, phi));
                float l = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
                if (!(l > 0.0f) || !std::isfinite(l)) l = 0.0f;
                lum[(size_t)j * W + i] = (double)l;
            }
        }
    });
    double lsum = 0.0;
    for (double l : lum) lsum += l;
    double floor_l = 1e-3 * (lsum / ((double)W * H));
    if (!(floor_l > 0.0)) floor_l = 1.0;
    std::vector<double> w((size_t)W * H), rows(H);
    for_chunks(0, H, chunks, [&](int, uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; ++j) {
            float theta = ((float)j + 0.5f) * (PI_F / (float)H);
            double st = (double)std::sin(theta);
            double rs = 0.0;
            for (uint32_t i = 0; i < W; ++i) {
                double x = (lum[(size_t)j * W + i] + floor_l) * st;
                w[(size_t)j * W + i] = x;
                rs += x;
            }
            rows[j] = rs;
        }
    });
    double total = 0.0;
    for (uint32_t j = 0; j < H; ++j) total += rows[j];
    T.marginal.assign(H + 1, 0.0f);
    T.conditional.assign((size_t)H * (W + 1), 0.0f);
    T.cell.assign((size_t)W * H, 0.0f);
    double acc = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        T.marginal[j] = (float)(acc / total);
        acc += rows[j];
    }
    for_chunks(0, H, chunks, [&](int, uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; ++j) {
            double ra = 0.0;
            float* cr = &T.conditional[(size_t)j * (W + 1)];
            for (uint32_t i = 0; i < W; ++i) {
                cr[i] = (float)(ra / rows[j]);
                ra += w[(size_t)j * W + i];
                T.cell[(size_t)j * W + i] = (float)(w[(size_t)j * W + i] / total);
            }
            cr[W] = 1.0f;
        }
    });
    T.marginal[H] = 1.0f;
    // Guide tables: guide[k] = the index the device's search returns for
    // u = k / M (the largest i < n with cdf[i] <= u; the CDFs are
    // non-decreasing, so that index is non-decreasing in u).  For u in
    // [k/M, (k+1)/M) the search then only needs [guide[k], guide[k+1]].
    auto pow2_at_least = [](uint32_t x, uint32_t lo, uint32_t hi) {
        uint32_t m = lo;
        while (m < x && m < hi) m <<= 1;
        return m;
    };
    auto guide = [](const float* cdf, uint32_t n, uint32_t m, uint32_t* g) {
        for (uint32_t k = 0; k <= m; ++k) {
            const float u = (float)k / (float)m;  // exact: m is a power of two
            const uint32_t c = (uint32_t)(std::upper_bound(cdf, cdf + n, u) - cdf);
            g[k] = c > 0 ? c - 1 : 0;
        }
    };
    T.gm = pow2_at_least(H, 16, 4096);
    T.gc = pow2_at_least(W / 4, 16, 1024);
    T.guide_marginal.assign(T.gm + 1, 0);
    guide(T.marginal.data(), H, T.gm, T.guide_marginal.data());
    T.guide_conditional.assign((size_t)H * (T.gc + 1), 0);
    for_chunks(0, H, chunks, [&](int, uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; ++j)
            guide(&T.conditional[(size_t)j * (W + 1)], W, T.gc, &T.guide_conditional[(size_t)j * (T.gc + 1)]);
    });
}

}  // namespace

V3 env_eval_host(const SceneView& v, const float* img, V3 dir) {
    if (v.env_kind == VR_ENV_UNIFORM) return load3(v.env_color);
    if (v.env_kind != VR_ENV_HDRI) return v3(0.0f, 0.0f, 0.0f);
    V3 d = normalize(dir);
    float sx = std::acos(-d.y);
    float sy = std::atan2(-d.z, d.x) + PI_F;
    float u = sx / PI_F;
    float vv = sy / (2.0f * PI_F);
    float x = vv * (float)v.env_w;
    float y = (float)(v.env_h - 1) - (u * (float)v.env_h);
    size_t W = v.env_w, H = v.env_h, len = W * H;
    size_t x0 = std::min(sat_usize(x), W - 1);
    size_t y0 = std::min(sat_usize(y), H - 1);
    float ax = x - (float)x0;
    float ay = y - (float)y0;
    auto px = [&](size_t i) { return load3(img + 3 * (i % len)); };
    return lerp3(lerp3(px(y0 * W + x0), px(y0 * W + x0 + 1), ax),
                 lerp3(px((y0 + 1) * W + x0), px((y0 + 1) * W + x0 + 1), ax), ay);
}

void set_camera(SceneView& v, const vr_camera_desc& c) {
    V3 dir = load3(c.direction), up = load3(c.up), eye = load3(c.eye);
    V3 right = normalize(cross(dir, up));
    for (int a = 0; a < 3; ++a) {
        v.c_origin[a] = (&eye.x)[a];
        v.c_dir[a] = (&dir.x)[a];
        v.c_up[a] = (&up.x)[a];
        v.c_right[a] = (&right.x)[a];
    }
    v.c_d = 1.0f / std::tan(c.fov / 2.0f);
    v.c_dof = c.has_dof ? 1 : 0;
    v.c_aperture = c.has_dof ? c.aperture : 0.0f;
    v.c_focal = c.has_dof ? dot(load3(c.focal_point) - eye, dir) : 0.0f;
}

namespace {
// 4-wide nodes collapsed from the flattened BVH2: a wide node holds the
// children of a BVH2 node, and repeatedly the children of its inner child
// with the largest surface area in place of that child, until it has four
// (or only leaves are left).  Layout (8 x float4): for children 0/1 and
// 2/3 the BVH2 pair layout (x lo/hi, y lo/hi per child, then both z
// ranges), then the four child codes (>= 0 wide node, < 0 leaf code as in
// the BVH2, 0x7fffffff an empty slot), then zeros.  Wide nodes are in
// depth-first preorder.
void collapse_wide(HostScene& hs) {
    hs.wide.clear();
    hs.wide_depth = 0;
    const size_t nb2 = hs.nodes.size() / 4;
    if (nb2 == 0) return;
    auto code = [&](size_t p, int s) {
        int32_t c;
        const float f = s ? hs.nodes[4 * p + 3].y : hs.nodes[4 * p + 3].x;
        std::memcpy(&c, &f, 4);
        return c;
    };
    auto box = [&](size_t p, int s, float* lo, float* hi) {
        const float4 a = hs.nodes[4 * p + s], z = hs.nodes[4 * p + 2];
        lo[0] = a.x; hi[0] = a.y; lo[1] = a.z; hi[1] = a.w;
        lo[2] = s ? z.z : z.x; hi[2] = s ? z.w : z.y;
    };
    auto area = [&](size_t p, int s) {
        float lo[3], hi[3];
        box(p, s, lo, hi);
        const double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    };
    struct Entry {
        uint32_t p;
        int s;
    };
    std::vector<std::array<Entry, 4>> sets;
    std::vector<uint8_t> counts;
    std::vector<int32_t> wide_of(nb2, -1);
    std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 1u}};  // (BVH2 node, depth)
    while (!stack.empty()) {
        const auto [f, depth] = stack.back();
        stack.pop_back();
        hs.wide_depth = std::max(hs.wide_depth, depth);
        wide_of[f] = (int32_t)sets.size();
        std::array<Entry, 4> e{};
        int n = 2;
        e[0] = {f, 0};
        e[1] = {f, 1};
        while (n < 4) {
            int best = -1;
            double ba = -1.0;
            for (int k = 0; k < n; ++k)
                if (code(e[k].p, e[k].s) >= 0 && area(e[k].p, e[k].s) > ba) {
                    ba = area(e[k].p, e[k].s);
                    best = k;
                }
            if (best < 0) break;
            const uint32_t g = (uint32_t)code(e[best].p, e[best].s);
            for (int k = n; k > best + 1; --k) e[k] = e[k - 1];
            e[best] = {g, 0};
            e[best + 1] = {g, 1};
            ++n;
        }
        sets.push_back(e);
        counts.push_back((uint8_t)n);
        for (int k = n - 1; k >= 0; --k)
            if (code(e[k].p, e[k].s) >= 0) stack.push_back({(uint32_t)code(e[k].p, e[k].s), depth + 1});
    }
    hs.wide.assign(sets.size() * 8, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (size_t w = 0; w < sets.size(); ++w) {
        float lo[4][3] = {}, hi[4][3] = {};
        int32_t c[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
        for (int k = 0; k < counts[w]; ++k) {
            const Entry& en = sets[w][k];
            box(en.p, en.s, lo[k], hi[k]);
            const int32_t cc = code(en.p, en.s);
            c[k] = cc >= 0 ? wide_of[cc] : cc;
        }
        float4* o = &hs.wide[8 * w];
        for (int pr = 0; pr < 2; ++pr) {
            const int a = 2 * pr, b = 2 * pr + 1;
            o[3 * pr + 0] = make_float4(lo[a][0], hi[a][0], lo[a][1], hi[a][1]);
            o[3 * pr + 1] = make_float4(lo[b][0], hi[b][0], lo[b][1], hi[b][1]);
            o[3 * pr + 2] = make_float4(lo[a][2], hi[a][2], lo[b][2], hi[b][2]);
        }
        float fc[4];
        std::memcpy(fc, c, sizeof fc);
        o[6] = make_float4(fc[0], fc[1], fc[2], fc[3]);
    }
}

vr_status build_host_scene_impl(const vr_scene_desc* d, HostScene& hs, std::string& err);
vr_status validate_host_scene_impl(const HostScene& hs, std::string& err);

// Nothing thrown below (a host allocation failing, a worker thread's
// exception passed on by its future) crosses the C ABI: it becomes a status.
template <class F>
vr_status guarded(std::string& err, F&& body) {
    try {
        return body();
    } catch (const std::bad_alloc&) {
        err = "host allocation failed while lowering the scene";
        return VR_ERR_OOM;
    } catch (const std::exception& e) {
        err = std::string("scene lowering failed: ") + e.what();
        return VR_ERR_INVALID;
    }
}
}  // namespace

vr_status build_host_scene(const vr_scene_desc* d, HostScene& hs, std::string& err) {
    return guarded(err, [&] { return build_host_scene_impl(d, hs, err); });
}

vr_status validate_host_scene(const HostScene& hs, std::string& err) {
    return guarded(err, [&] { return validate_host_scene_impl(hs, err); });
}

namespace {
vr_status build_host_scene_impl(const vr_scene_desc* d, HostScene& hs, std::string& err) {
    auto t0 = std::chrono::steady_clock::now();
    if (!d) { err = "null scene descriptor"; return VR_ERR_INVALID; }
    if (d->num_meshes && !d->meshes) { err = "meshes is NULL"; return VR_ERR_INVALID; }
    if (d->num_materials && !d->materials) { err = "materials is NULL"; return VR_ERR_INVALID; }
    hs.materials.resize(d->num_materials);
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        static_assert(sizeof(Material) == sizeof(vr_material), "material layout");
        std::memcpy(&hs.materials[i], &d->materials[i], sizeof(Material));
        if (hs.materials[i].kind < 0 || hs.materials[i].kind > M_MIX) {
            err = "material " + std::to_string(i) + ": unsupported kind";
            return VR_ERR_UNSUPPORTED;
        }
        const Material& mt = hs.materials[i];
        for (int32_t tix : {mt.albedo_tex, mt.normal_tex})
            if (tix < -1 || tix >= (int32_t)d->num_textures) {
                err = "material " + std::to_string(i) + ": texture index out of range";
                return VR_ERR_INVALID;
            }
        if ((mt.albedo_tex >= 0 || mt.normal_tex >= 0) && mt.kind != M_LAMB) {
            err = "material " + std::to_string(i) + ": only Lambertian materials take textures";
            return VR_ERR_UNSUPPORTED;
        }
        if (mt.kind == M_MIX && (mt.mix_first < 0 || mt.mix_first >= (int32_t)d->num_materials ||
                                 mt.mix_second < 0 || mt.mix_second >= (int32_t)d->num_materials)) {
            err = "material " + std::to_string(i) + ": mix child index out of range";
            return VR_ERR_INVALID;
        }
    }
    // MixMaterial chains end in a plain material within MAX_MIX_DEPTH levels (this also
    // rules out cycles), so the kernels resolve a mix with a bounded loop
    {
        std::vector<int> depth(hs.materials.size(), -1);  // levels of mixing below material i
        for (size_t pass = 0; pass <= MAX_MIX_DEPTH + 1; ++pass)
            for (size_t i = 0; i < hs.materials.size(); ++i) {
                const Material& mt = hs.materials[i];
                if (mt.kind != M_MIX) { depth[i] = 0; continue; }
                const int a = depth[mt.mix_first], b = depth[mt.mix_second];
                if (a >= 0 && b >= 0) depth[i] = 1 + std::max(a, b);
            }
        for (size_t i = 0; i < hs.materials.size(); ++i)
            if (depth[i] < 0 || depth[i] > MAX_MIX_DEPTH) {
                err = "material " + std::to_string(i) + ": mix chain deeper than VR_MAX_MIX_DEPTH or cyclic";
                return VR_ERR_INVALID;
            }
    }
    // image textures (texture.rs:28-98)
    if (d->num_textures && !d->textures) { err = "textures is NULL"; return VR_ERR_INVALID; }
    hs.tex_info.clear();
    hs.texels.clear();
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        const vr_texture_desc& t = d->textures[i];
        if (!t.image || !t.width || !t.height) {
            err = "texture " + std::to_string(i) + ": empty image";
            return VR_ERR_INVALID;
        }
        if (t.sampling != VR_TEX_NEAREST && t.sampling != VR_TEX_BILINEAR) {
            err = "texture " + std::to_string(i) + ": unknown sampling";
            return VR_ERR_INVALID;
        }
        const size_t n = 3 * (size_t)t.width * t.height;
        if (hs.texels.size() + n >= (size_t)INT32_MAX) { err = "textures too large"; return VR_ERR_INVALID; }
        hs.tex_info.push_back(make_int4((int)hs.texels.size(), (int)t.width, (int)t.height, t.sampling));
        hs.texels.insert(hs.texels.end(), t.image, t.image + n);
    }
    uint64_t np = 0;
    bool any_uv = false;
    for (uint32_t m = 0; m < d->num_meshes; ++m) {
        const vr_mesh_desc& md = d->meshes[m];
        if (md.num_triangles && (!md.positions || !md.indices)) {
            err = "mesh " + std::to_string(m) + ": positions/indices NULL";
            return VR_ERR_INVALID;
        }
        if (md.material >= d->num_materials) {
            err = "mesh " + std::to_string(m) + ": material index out of range";
            return VR_ERR_INVALID;
        }
        np += md.num_triangles;
        any_uv = any_uv || md.uvs;
    }
    if (np >= (1ull << 27)) { err = "too many triangles (the leaf encoding holds 2^27)"; return VR_ERR_INVALID; }
    hs.num_prims = np;
    std::vector<PrimRef> refs(np);
    std::vector<float4> v0e(np * 3);  // v0, e1, e2 by prim id
    hs.shade.resize(np * 4);
    if (any_uv) hs.uvs.resize(np * 3);
    Box scene_box;
    // prim ids run over the meshes in order; pieces of the id range are
    // lowered on separate threads, each stopping at its first bad triangle,
    // and the error of the lowest id is the one reported
    std::vector<uint64_t> first_prim(d->num_meshes + 1, 0);
    for (uint32_t m = 0; m < d->num_meshes; ++m) first_prim[m + 1] = first_prim[m] + d->meshes[m].num_triangles;
    const int lchunks = chunks_for(np);
    std::vector<Box> chunk_box(lchunks);
    std::vector<std::string> chunk_err(lchunks);
    for_chunks(0, (uint32_t)np, lchunks, [&](int c, uint32_t lo, uint32_t hi) {
        uint32_t m = (uint32_t)(std::upper_bound(first_prim.begin(), first_prim.end(), (uint64_t)lo) -
                                first_prim.begin()) - 1;
        for (uint64_t p = lo; p < hi; ++p) {
            while (p >= first_prim[m + 1]) ++m;
            const vr_mesh_desc& md = d->meshes[m];
            const uint64_t t = p - first_prim[m];
            uint32_t ix[3] = {md.indices[3 * t], md.indices[3 * t + 1], md.indices[3 * t + 2]};
            for (int k = 0; k < 3; ++k)
                if (ix[k] >= md.num_vertices) {
                    chunk_err[c] = "mesh " + std::to_string(m) + ": index out of range";
                    return;
                }
            V3 P[3], N[3];
            for (int k = 0; k < 3; ++k) {
                P[k] = load3(md.positions + 3 * (size_t)ix[k]);
                if (!std::isfinite(P[k].x) || !std::isfinite(P[k].y) || !std::isfinite(P[k].z)) {
                    chunk_err[c] = "mesh " + std::to_string(m) + ": vertex " + std::to_string(ix[k]) +
                                   " has a non-finite position";
                    return;
                }
                N[k] = md.normals ? load3(md.normals + 3 * (size_t)ix[k]) : v3(0.0f, 0.0f, 0.0f);
                if (any_uv) {
                    hs.uvs[3 * p + k] = md.uvs ? make_float2(md.uvs[2 * (size_t)ix[k]], md.uvs[2 * (size_t)ix[k] + 1])
                                               : make_float2(0.0f, 0.0f);
                }
            }
            // Triangle::hit edges (mesh.rs:150-151)
            V3 e1 = P[1] - P[0], e2 = P[2] - P[0];
            // face normal, Mesh::from_buffers (mesh.rs:80-84)
            V3 fe1 = P[0] - P[1], fe2 = P[2] - P[1];
            V3 fn = normalize(cross(fe2, fe1));
            uint32_t pid = (uint32_t)p;
            float pbits;
            std::memcpy(&pbits, &pid, 4);
            float mbits;
            std::memcpy(&mbits, &md.material, 4);
            v0e[3 * p + 0] = make_float4(P[0].x, P[0].y, P[0].z, pbits);
            v0e[3 * p + 1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
            v0e[3 * p + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
            hs.shade[4 * p + 0] = make_float4(N[0].x, N[0].y, N[0].z, mbits);
            hs.shade[4 * p + 1] = make_float4(N[1].x, N[1].y, N[1].z, 0.0f);
            hs.shade[4 * p + 2] = make_float4(N[2].x, N[2].y, N[2].z, 0.0f);
            hs.shade[4 * p + 3] = make_float4(fn.x, fn.y, fn.z, 0.0f);
            PrimRef& r = refs[p];
            for (int a = 0; a < 3; ++a) {
                float x0 = (&P[0].x)[a], x1 = (&P[1].x)[a], x2 = (&P[2].x)[a];
                r.lo[a] = std::min(x0, std::min(x1, x2));
                r.hi[a] = std::max(x0, std::max(x1, x2));
                r.c[a] = 0.5f * (r.lo[a] + r.hi[a]);
            }
            r.id = pid;
            chunk_box[c].grow(r.lo, r.hi);
        }
    });
    for (int c = 0; c < lchunks; ++c) {
        if (!chunk_err[c].empty()) {
            err = chunk_err[c];
            return VR_ERR_INVALID;
        }
        scene_box.grow(chunk_box[c].lo, chunk_box[c].hi);
    }
    // BVH
    uint32_t max_leaf = d->bvh_max_leaf ? d->bvh_max_leaf : 4;
    int nbins = d->bvh_bins ? (int)d->bvh_bins : 16;
    if (max_leaf > 16) max_leaf = 16;
    if (nbins < 2) nbins = 2;
    if (nbins > 64) nbins = 64;
    hs.max_leaf = max_leaf;
    hs.nodes.clear();
    hs.tris.clear();
    if (np > 0) {
        SubTree T;
        build_subtree(refs, max_leaf, nbins, 0, (uint32_t)np, 0, spawn_depth_for_host(), T);
        std::vector<BNode>& nodes = T.nodes;
        const int root = 0;
        hs.max_depth = T.max_depth + 1;
        // conservative padding keeps the f32 slab test from culling a box whose
        // triangle is hit right on its boundary
        float smax = 0.0f;
        for (int a = 0; a < 3; ++a) smax = std::max(smax, std::max(std::fabs(scene_box.lo[a]), std::fabs(scene_box.hi[a])));
        const float pad = std::max(smax, 1e-20f) * 1e-6f;
        // triangle order = prim order after partitioning
        hs.tris.resize(np * 3);
        for_chunks(0, (uint32_t)np, chunks_for(np), [&](int, uint32_t lo, uint32_t hi) {
            for (uint64_t i = lo; i < hi; ++i)
                for (int k = 0; k < 3; ++k) hs.tris[3 * i + k] = v0e[3 * (size_t)refs[i].id + k];
        });
        // flatten inner nodes depth first
        std::vector<int> order;  // builder node -> flat index
        std::vector<int> flat_of(nodes.size(), -1);
        std::vector<int> stack;
        auto is_leaf = [&](int n) { return nodes[n].left < 0; };
        int root_inner = root;
        if (is_leaf(root)) {
            // single leaf: an inner root whose both children are that leaf
            BNode rn = nodes[root];
            rn.left = root;
            rn.right = root;
            nodes.push_back(rn);
            root_inner = (int)nodes.size() - 1;
            flat_of.push_back(-1);
        }
        stack.push_back(root_inner);
        while (!stack.empty()) {
            int n = stack.back();
            stack.pop_back();
            flat_of[n] = (int)order.size();
            order.push_back(n);
            const BNode& bn = nodes[n];
            if (!is_leaf(bn.right) && bn.right != n) stack.push_back(bn.right);
            if (!is_leaf(bn.left) && bn.left != n) stack.push_back(bn.left);
        }
        hs.nodes.resize(order.size() * 4);
        for_chunks(0, (uint32_t)order.size(), chunks_for(order.size()), [&](int, uint32_t flo, uint32_t fhi) {
          for (size_t f = flo; f < fhi; ++f) {
            const BNode& bn = nodes[order[f]];
            const BNode& c0 = nodes[bn.left];
            const BNode& c1 = nodes[bn.right];
            auto lo = [&](const BNode& c, int a) { return c.lo[a] - pad; };
            auto hi = [&](const BNode& c, int a) { return c.hi[a] + pad; };
            hs.nodes[4 * f + 0] = make_float4(lo(c0, 0), hi(c0, 0), lo(c0, 1), hi(c0, 1));
            hs.nodes[4 * f + 1] = make_float4(lo(c1, 0), hi(c1, 0), lo(c1, 1), hi(c1, 1));
            hs.nodes[4 * f + 2] = make_float4(lo(c0, 2), hi(c0, 2), lo(c1, 2), hi(c1, 2));
            // leaf child: ~(first << 4 | count - 1), negative; inner child: its flat index
            auto leaf_code = [](const BNode& c) { return (int32_t)~((c.first << 4) | (c.count - 1)); };
            int32_t r0 = is_leaf(bn.left) ? leaf_code(c0) : flat_of[bn.left];
            int32_t r1 = is_leaf(bn.right) ? leaf_code(c1) : flat_of[bn.right];
            int32_t n0 = is_leaf(bn.left) ? (int32_t)c0.count : 0;
            int32_t n1 = is_leaf(bn.right) ? (int32_t)c1.count : 0;
            float fr0, fr1, fn0, fn1;
            std::memcpy(&fr0, &r0, 4);
            std::memcpy(&fr1, &r1, 4);
            std::memcpy(&fn0, &n0, 4);
            std::memcpy(&fn1, &n1, 4);
            hs.nodes[4 * f + 3] = make_float4(fr0, fr1, fn0, fn1);
          }
        });
        // SAH cost of the tree, summed in flat order
        double sah = 0.0;
        const double root_area = Box(scene_box).area();
        for (size_t f = 0; f < order.size(); ++f) {
            const BNode& bn = nodes[order[f]];
            const BNode& c0 = nodes[bn.left];
            const BNode& c1 = nodes[bn.right];
            Box nb;
            nb.grow(bn.lo, bn.hi);
            sah += C_TRAV * nb.area() / std::max(root_area, 1e-300);
            for (const BNode* c : {&c0, &c1}) {
                if (c->left < 0) {
                    Box cb2;
                    cb2.grow(c->lo, c->hi);
                    sah += C_ISECT * c->count * cb2.area() / std::max(root_area, 1e-300);
                }
            }
        }
        hs.sah_cost = sah;
        collapse_wide(hs);
    }
    // environment
    SceneView& v = hs.view;
    v.env_kind = d->environment.kind;
    for (int a = 0; a < 3; ++a) v.env_color[a] = d->environment.color[a];
    if (v.env_kind == VR_ENV_HDRI) {
        const vr_environment_desc& e = d->environment;
        if (!e.image || e.width == 0 || e.height == 0) { err = "HDRI environment without an image"; return VR_ERR_INVALID; }
        v.env_w = e.width;
        v.env_h = e.height;
        hs.env_img.assign(e.image, e.image + 3 * (size_t)e.width * e.height);
        if (e.importance_sample) {
            build_env_tables(hs);
            hs.has_tables = true;
            // W*H / (2 pi^2): the cell solid-angle factor, same rounding as the oracle
            v.env_density_scale = (float)((double)e.width * (double)e.height *
                                          (1.0 / (2.0 * 3.14159265358979323846 * 3.14159265358979323846)));
        }
    } else if (v.env_kind != VR_ENV_NONE && v.env_kind != VR_ENV_UNIFORM) {
        err = "unsupported environment kind";
        return VR_ERR_UNSUPPORTED;
    }
    v.env_is = hs.has_tables ? 1 : 0;
    v.num_materials = (int32_t)d->num_materials;
    // analytic surfaces (surfaces.rs:31-114)
    if (d->num_analytics && !d->analytics) { err = "analytics is NULL"; return VR_ERR_INVALID; }
    if (d->num_analytics > VR_MAX_ANALYTICS) { err = "too many analytic surfaces"; return VR_ERR_UNSUPPORTED; }
    hs.analytic.clear();
    for (uint32_t i = 0; i < d->num_analytics; ++i) {
        const vr_analytic_desc& a = d->analytics[i];
        if (a.material >= d->num_materials) {
            err = "analytic surface " + std::to_string(i) + ": material index out of range";
            return VR_ERR_INVALID;
        }
        float kb, mb;
        std::memcpy(&kb, &a.kind, 4);
        std::memcpy(&mb, &a.material, 4);
        if (a.kind == VR_ANALYTIC_SPHERE)
            hs.analytic.push_back(make_float4(a.center[0], a.center[1], a.center[2], a.radius));
        else if (a.kind == VR_ANALYTIC_GROUND_PLANE)
            hs.analytic.push_back(make_float4(0.0f, a.height, 0.0f, 0.0f));
        else {
            err = "analytic surface " + std::to_string(i) + ": unsupported kind";
            return VR_ERR_UNSUPPORTED;
        }
        hs.analytic.push_back(make_float4(kb, mb, 0.0f, 0.0f));
    }
    v.num_analytic = d->num_analytics;
    v.num_tris = (uint32_t)np;
    v.num_textures = d->num_textures;
    set_camera(v, d->camera);
    hs.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return VR_OK;
}

vr_status validate_host_scene_impl(const HostScene& hs, std::string& err) {
    const uint64_t np = hs.num_prims;
    if (np == 0) return hs.nodes.empty() ? VR_OK : (err = "nodes without triangles", VR_ERR_INVALID);
    const uint64_t nn = hs.nodes.size() / 4;
    std::vector<uint32_t> seen(np, 0);
    std::vector<uint8_t> visited(nn, 0);
    struct Item {
        int32_t node;
        float lo[3], hi[3];
        uint32_t depth;
    };
    std::vector<Item> stack;
    Item root{0, {-INFINITY, -INFINITY, -INFINITY}, {INFINITY, INFINITY, INFINITY}, 1};
    stack.push_back(root);
    auto as_int = [](float f) {
        int32_t i;
        std::memcpy(&i, &f, 4);
        return i;
    };
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        if (it.node < 0 || (uint64_t)it.node >= nn) { err = "child index out of range"; return VR_ERR_INVALID; }
        if (visited[it.node]++) { err = "node reached twice"; return VR_ERR_INVALID; }
        if (it.depth >= (uint32_t)(DEPTH_LIMIT + 2)) { err = "tree deeper than the traversal stack"; return VR_ERR_INVALID; }
        const float4* n = &hs.nodes[4 * (size_t)it.node];
        float clo[2][3] = {{n[0].x, n[0].z, n[2].x}, {n[1].x, n[1].z, n[2].z}};
        float chi[2][3] = {{n[0].y, n[0].w, n[2].y}, {n[1].y, n[1].w, n[2].w}};
        int32_t ref[2] = {as_int(n[3].x), as_int(n[3].y)};
        int32_t cnt[2] = {as_int(n[3].z), as_int(n[3].w)};
        const bool dup_root = (it.node == 0 && ref[0] == ref[1] && cnt[0] == cnt[1] && cnt[0] > 0);
        for (int c = 0; c < 2; ++c) {
            for (int a = 0; a < 3; ++a) {
                if (!(clo[c][a] <= chi[c][a])) { err = "inverted child box"; return VR_ERR_INVALID; }
                if (clo[c][a] < it.lo[a] || chi[c][a] > it.hi[a]) {
                    // a child box lies inside its parent's (padded) box
                    const float slack = 4e-6f * std::max(1.0f, std::max(std::fabs(it.lo[a]), std::fabs(it.hi[a])));
                    if (clo[c][a] < it.lo[a] - slack || chi[c][a] > it.hi[a] + slack) {
                        err = "child box outside its parent";
                        return VR_ERR_INVALID;
                    }
                }
            }
            if (cnt[c] > 0) {
                if (dup_root && c == 1) continue;
                // leaf code ~(first << 4 | count - 1)
                if (ref[c] >= 0) { err = "leaf child without a leaf code"; return VR_ERR_INVALID; }
                const uint32_t code = ~(uint32_t)ref[c];
                const uint32_t first = code >> 4, count = (code & 15u) + 1u;
                if ((int32_t)count != cnt[c]) { err = "leaf code and count disagree"; return VR_ERR_INVALID; }
                if ((uint64_t)first + count > np) { err = "leaf range out of bounds"; return VR_ERR_INVALID; }
                for (int32_t k = 0; k < cnt[c]; ++k) {
                    const float4* t = &hs.tris[3 * ((size_t)first + k)];
                    uint32_t pid;
                    std::memcpy(&pid, &t[0].w, 4);
                    if (pid >= np) { err = "prim id out of range"; return VR_ERR_INVALID; }
                    seen[pid]++;
                    const float vx[3][3] = {{t[0].x, t[0].y, t[0].z},
                                            {t[0].x + t[1].x, t[0].y + t[1].y, t[0].z + t[1].z},
                                            {t[0].x + t[2].x, t[0].y + t[2].y, t[0].z + t[2].z}};
                    for (int q = 0; q < 3; ++q)
                        for (int a = 0; a < 3; ++a) {
                            const float slack = 4e-6f * std::max(1.0f, std::fabs(vx[q][a]));
                            if (vx[q][a] < clo[c][a] - slack || vx[q][a] > chi[c][a] + slack) {
                                err = "triangle outside its leaf box";
                                return VR_ERR_INVALID;
                            }
                        }
                }
            } else {
                Item ch{ref[c], {clo[c][0], clo[c][1], clo[c][2]}, {chi[c][0], chi[c][1], chi[c][2]}, it.depth + 1};
                stack.push_back(ch);
            }
        }
    }
    for (uint64_t i = 0; i < nn; ++i)
        if (!visited[i]) { err = "unreachable node"; return VR_ERR_INVALID; }
    for (uint64_t p = 0; p < np; ++p)
        if (seen[p] != 1) { err = "triangle " + std::to_string(p) + " appears " + std::to_string(seen[p]) + " times"; return VR_ERR_INVALID; }
    // the 4-wide nodes: a tree over every triangle once (the single-leaf
    // scene's duplicated leaf aside), child codes in range, every leaf's
    // triangles inside its box, stack use within the wide traversal's stack
    const uint64_t nw = hs.wide.size() / 8;
    if (hs.wide.size() % 8 || (nn > 0 && nw == 0)) { err = "wide node array size"; return VR_ERR_INVALID; }
    if (nw) {
        if (3ull * hs.wide_depth + 1 > (uint64_t)WIDE_STACK) { err = "wide tree deeper than the traversal stack"; return VR_ERR_INVALID; }
        std::vector<uint8_t> wvis(nw, 0);
        std::vector<uint32_t> wseen(np, 0);
        std::vector<uint32_t> wst{0};
        while (!wst.empty()) {
            const uint32_t w = wst.back();
            wst.pop_back();
            if (wvis[w]) { err = "wide node reached twice"; return VR_ERR_INVALID; }
            wvis[w] = 1;
            const float4* o = &hs.wide[8 * (size_t)w];
            int32_t cd[4];
            std::memcpy(cd, &o[6], sizeof cd);
            for (int c = 0; c < 4; ++c) {
                if (cd[c] == 0x7fffffff) continue;
                const float4 xy = o[3 * (c >> 1) + (c & 1)], z = o[3 * (c >> 1) + 2];
                const float lo[3] = {xy.x, xy.z, (c & 1) ? z.z : z.x}, hi[3] = {xy.y, xy.w, (c & 1) ? z.w : z.y};
                if (cd[c] >= 0) {
                    if ((uint64_t)cd[c] >= nw) { err = "wide child index out of range"; return VR_ERR_INVALID; }
                    wst.push_back((uint32_t)cd[c]);
                    continue;
                }
                const uint32_t code = ~(uint32_t)cd[c];
                const uint32_t first = code >> 4, count = (code & 15u) + 1u;
                if ((uint64_t)first + count > np) { err = "wide leaf range out of bounds"; return VR_ERR_INVALID; }
                for (uint32_t k = 0; k < count; ++k) {
                    const float4* t = &hs.tris[3 * ((size_t)first + k)];
                    uint32_t pid;
                    std::memcpy(&pid, &t[0].w, 4);
                    if (pid >= np) { err = "prim id out of range"; return VR_ERR_INVALID; }
                    wseen[pid]++;
                    const float vx[3][3] = {{t[0].x, t[0].y, t[0].z},
                                            {t[0].x + t[1].x, t[0].y + t[1].y, t[0].z + t[1].z},
                                            {t[0].x + t[2].x, t[0].y + t[2].y, t[0].z + t[2].z}};
                    for (int q = 0; q < 3; ++q)
                        for (int a = 0; a < 3; ++a) {
                            const float slack = 4e-6f * std::max(1.0f, std::fabs(vx[q][a]));
                            if (vx[q][a] < lo[a] - slack || vx[q][a] > hi[a] + slack) {
                                err = "triangle outside its wide leaf box";
                                return VR_ERR_INVALID;
                            }
                        }
                }
            }
        }
        for (uint64_t i = 0; i < nw; ++i)
            if (!wvis[i]) { err = "unreachable wide node"; return VR_ERR_INVALID; }
        for (uint64_t p = 0; p < np; ++p)
            if (wseen[p] != 1 && !(np <= 16 && wseen[p] == 2)) {
                err = "triangle " + std::to_string(p) + " appears " + std::to_string(wseen[p]) + " times in the wide tree";
                return VR_ERR_INVALID;
            }
    }
    return VR_OK;
}
}  // namespace

}  // namespace vr
