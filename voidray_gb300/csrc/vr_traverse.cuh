// vr_traverse.cuh — 4-wide BVH traversal of the sm_103a kernels (closest and any hit).
//
// Node layout (128 bytes; seven 128-bit loads):
//   f[0] = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)   f[3] = the same for c2
//   f[1] = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)   f[4] = the same for c3
//   f[2] = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)   f[5] = the same for c2, c3
//   f[6] = (code0, code1, code2, code3); code >= 0: wide node index,
//          code < 0: leaf ~(first << 4 | count - 1) over the leaf-ordered
//          triangle array (3 x float4 per triangle: v0 | prim id, e1, e2),
//          SENTINEL: an empty slot;  f[7] unused.
// The nodes are the binned-SAH BVH2 collapsed to four children per node
// (vr_build.cpp), which halves the dependent node fetches of a ray.
//
// Traversal is the persistent "while-while" scheme of Aila & Laine (2009):
// resident warps pull rays from a queue; each lane walks inner nodes nearest
// child first and postpones the first leaf it reaches, so that leaves are
// intersected when every lane of the warp holds one (the triangle tests then
// run with the whole warp active).  When enough lanes have finished, the warp
// stores their results and refills them from the queue.  Of a node's hit
// children the nearest is visited next and the others are pushed with their
// entry distances, farthest first; popped entries beyond the current closest
// hit are skipped.  Any-hit traversal pushes node indices alone and keeps no
// order among a node's hit children (shadow rays), or only visits the nearest
// first (queries of the batch intersection API).
#pragma once
#include "vr_device.cuh"

namespace vr {

struct HitOut {
    uint32_t prim;
    float t, u, v;
};

#ifndef VR_TRACE_MINB
#define VR_TRACE_MINB 9  // minimum resident blocks per SM requested from ptxas (55 registers, no spills)
#endif
#ifndef VR_SHADOW_MINB
#define VR_SHADOW_MINB VR_TRACE_MINB  // the same for the any-hit shadow kernel
#endif
#ifndef VR_ISECT_MINB
#define VR_ISECT_MINB VR_TRACE_MINB  // the same for the batch intersection kernel
#endif
#ifndef VR_DYN_FETCH
#define VR_DYN_FETCH 16  // refill a warp's lanes once at least this many have finished
#endif
constexpr int SENTINEL = 0x7fffffff;  // "no node": the walk is finished
#ifndef VR_DYN_FETCH_ANY
#define VR_DYN_FETCH_ANY VR_DYN_FETCH  // the same for any-hit (shadow) traversal
#endif
constexpr int DYN_FETCH = VR_DYN_FETCH;
constexpr int DYN_FETCH_ANY = VR_DYN_FETCH_ANY;

// Triangle::hit (mesh.rs:144-188) on the precomputed (v0, e1, e2): the same
// operations in the same order, each rounded separately (-fmad=false), so
// t/u/v are the values the reference computes.  The determinant test uses
// tmin as an absolute epsilon like the reference; a hit is accepted for
// tmin < t < best.  Returns true on the first accepted hit when ANY.
template <bool ANY>
__device__ __forceinline__ bool leaf_test(const float4* __restrict__ tris, int first, int count, V3 o, V3 d,
                                          float tmin, float& best, HitOut& h, uint32_t& ntest, bool counting) {
    for (int k = 0; k < count; ++k) {
        const float4* tp = tris + 3 * (first + k);
        const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (counting) ntest++;
        const V3 v0 = xyz(a), e1 = xyz(b), e2 = xyz(c);
        const V3 hh = cross(d, e2);
        const float det = dot(e1, hh);
        if (det > -tmin && det < tmin) continue;
        const float f = 1.0f / det;
        const V3 s = o - v0;
        const float u = f * dot(s, hh);
        if (u < 0.0f || u > 1.0f) continue;
        const V3 q = cross(s, e1);
        const float v = f * dot(d, q);
        if (v < 0.0f || u + v > 1.0f) continue;
        const float t = f * dot(e2, q);
        if (t > tmin && t < best) {
            best = t;
            h.prim = __float_as_uint(a.w);
            h.t = t;
            h.u = u;
            h.v = v;
            if (ANY) return true;
        }
    }
    return false;
}

__device__ __forceinline__ float4 pack_hit(const HitOut& h) {
    return make_float4(__uint_as_float(h.prim), h.t, h.u, h.v);
}

// Warp-reduced work counters (inner-node visits, triangle tests).
__device__ __forceinline__ void add_work(unsigned long long* work, uint32_t nv, uint32_t nt) {
    unsigned long long a = nv, b = nt;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(work, a);
        atomicAdd(work + 1, b);
    }
}

// Io supplies load(i, ro, rd, nodes, tris) -- the ray and the BVH of its
// scene, so that rays of different scenes can share a launch -- and
// store(i, hit, overflow).  `counter` is the queue's fetch cursor (zero
// before the launch).  Every lane of the block's warps must call this
// (warp-uniform control flow at the votes).
template <bool ANY, bool COUNT, class Io, bool NEAREST_ANY = false>
__device__ __forceinline__ void persistent_trace(uint32_t n, uint32_t* counter, const Io& io, uint32_t* status,
                                                 unsigned long long* work) {
    const uint32_t lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const float4* nodes = nullptr;  // BVH of the current ray's scene
    const float4* tris = nullptr;
    // closest hit: (node, entry distance) pairs, one 64-bit access each;
    // any hit: node indices alone (every pushed child lies within the ray's
    // fixed [tmin, tmax], so no entry is ever culled)
    int2 stack[ANY ? 1 : STACK_SIZE];
    int stack_node[ANY ? STACK_SIZE : 1];
    V3 o = v3(0.0f, 0.0f, 0.0f), d = v3(0.0f, 0.0f, 1.0f);
    float ix = 0.0f, iy = 0.0f, iz = 0.0f, ox = 0.0f, oy = 0.0f, oz = 0.0f, tmin = 0.0f, best = 0.0f;
    int node = SENTINEL, leaf = 0, sp = 0;
    HitOut h{MISS, INF_F, 0.0f, 0.0f};
    uint32_t ray = 0, nv = 0, nt = 0;
    bool has = false, alive = true, overflow = false;

    auto pop = [&]() -> int {
        if (ANY) return sp > 0 ? stack_node[--sp] : SENTINEL;
        while (sp > 0) {
            const int2 e = stack[--sp];
            if (__int_as_float(e.y) <= best) return e.x;
        }
        return SENTINEL;
    };
    auto push = [&](int k, float t) { stack[sp++] = make_int2(k, __float_as_int(t)); };

    while (true) {
        // finished lanes store their result
        if (has && node == SENTINEL && leaf >= 0) {
            if (overflow) atomicOr(status, ERRF_STACK);
            io.store(ray, h, overflow);
            has = false;
        }
        // and take new rays, one atomic per warp
        const bool need = alive && !has;
        const unsigned needm = __ballot_sync(FULL, need);
        if (needm) {
            const int leader = __ffs(needm) - 1;
            uint32_t base = 0;
            if (lane == (uint32_t)leader) base = atomicAdd(counter, (uint32_t)__popc(needm));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                ray = base + __popc(needm & ((1u << lane) - 1u));
                if (ray < n) {
                    float4 ro, rd;
                    io.load(ray, ro, rd, nodes, tris);
                    o = xyz(ro);
                    d = xyz(rd);
                    const float eps = 1e-18f;
                    ix = 1.0f / (fabsf(rd.x) > eps ? rd.x : copysignf(eps, rd.x));
                    iy = 1.0f / (fabsf(rd.y) > eps ? rd.y : copysignf(eps, rd.y));
                    iz = 1.0f / (fabsf(rd.z) > eps ? rd.z : copysignf(eps, rd.z));
                    ox = ro.x * ix;
                    oy = ro.y * iy;
                    oz = ro.z * iz;
                    tmin = ro.w;
                    best = rd.w;
                    node = nodes ? 0 : SENTINEL;  // a scene without triangles: the ray misses
                    leaf = 0;
                    sp = 0;
                    overflow = false;
                    h = HitOut{MISS, INF_F, 0.0f, 0.0f};
                    has = true;
                } else {
                    alive = false;
                }
            }
        }
        if (!__any_sync(FULL, has)) break;

        do {
            // inner nodes until every lane in the loop holds a postponed leaf
            while (node >= 0 && node != SENTINEL) {
                // 4-wide node: slab tests of the four children, the hit ones
                // visited nearest first (the others pushed farthest first)
                const float4* np = nodes + 8 * node;
                if (COUNT) nv++;
                float t0, t1, t2, t3;
                const int4 cd = __ldg(reinterpret_cast<const int4*>(np) + 6);
                {
                    const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
                    const float a0 = fmaf(n0.x, ix, -ox), b0 = fmaf(n0.y, ix, -ox);
                    const float c0 = fmaf(n0.z, iy, -oy), d0 = fmaf(n0.w, iy, -oy);
                    const float e0 = fmaf(n2.x, iz, -oz), f0 = fmaf(n2.y, iz, -oz);
                    const float a1 = fmaf(n1.x, ix, -ox), b1 = fmaf(n1.y, ix, -ox);
                    const float c1 = fmaf(n1.z, iy, -oy), d1 = fmaf(n1.w, iy, -oy);
                    const float e1 = fmaf(n2.z, iz, -oz), f1 = fmaf(n2.w, iz, -oz);
                    const float tn0 = fmaxf(fmaxf(fminf(a0, b0), fminf(c0, d0)), fmaxf(fminf(e0, f0), tmin));
                    const float tf0 = fminf(fminf(fmaxf(a0, b0), fmaxf(c0, d0)), fminf(fmaxf(e0, f0), best));
                    const float tn1 = fmaxf(fmaxf(fminf(a1, b1), fminf(c1, d1)), fmaxf(fminf(e1, f1), tmin));
                    const float tf1 = fminf(fminf(fmaxf(a1, b1), fmaxf(c1, d1)), fminf(fmaxf(e1, f1), best));
                    t0 = (tn0 <= tf0 && cd.x != SENTINEL) ? tn0 : INF_F;
                    t1 = (tn1 <= tf1 && cd.y != SENTINEL) ? tn1 : INF_F;
                }
                {
                    const float4 n0 = __ldg(np + 3), n1 = __ldg(np + 4), n2 = __ldg(np + 5);
                    const float a0 = fmaf(n0.x, ix, -ox), b0 = fmaf(n0.y, ix, -ox);
                    const float c0 = fmaf(n0.z, iy, -oy), d0 = fmaf(n0.w, iy, -oy);
                    const float e0 = fmaf(n2.x, iz, -oz), f0 = fmaf(n2.y, iz, -oz);
                    const float a1 = fmaf(n1.x, ix, -ox), b1 = fmaf(n1.y, ix, -ox);
                    const float c1 = fmaf(n1.z, iy, -oy), d1 = fmaf(n1.w, iy, -oy);
                    const float e1 = fmaf(n2.z, iz, -oz), f1 = fmaf(n2.w, iz, -oz);
                    const float tn0 = fmaxf(fmaxf(fminf(a0, b0), fminf(c0, d0)), fmaxf(fminf(e0, f0), tmin));
                    const float tf0 = fminf(fminf(fmaxf(a0, b0), fmaxf(c0, d0)), fminf(fmaxf(e0, f0), best));
                    const float tn1 = fmaxf(fmaxf(fminf(a1, b1), fminf(c1, d1)), fmaxf(fminf(e1, f1), tmin));
                    const float tf1 = fminf(fminf(fmaxf(a1, b1), fmaxf(c1, d1)), fminf(fmaxf(e1, f1), best));
                    t2 = (tn0 <= tf0 && cd.z != SENTINEL) ? tn0 : INF_F;
                    t3 = (tn1 <= tf1 && cd.w != SENTINEL) ? tn1 : INF_F;
                }
                int k0 = cd.x, k1 = cd.y, k2 = cd.z, k3 = cd.w;
                const int nh = (t0 < INF_F) + (t1 < INF_F) + (t2 < INF_F) + (t3 < INF_F);
                if (ANY) {
                    // any hit: visit one hit child and push the others, in
                    // no particular order (NEAREST_ANY: the nearest first,
                    // by an argmin rather than a sort)
                    if (nh == 0) {
                        node = pop();
                    } else if (sp + nh - 1 > STACK_SIZE) {
                        overflow = true;
                        node = SENTINEL;
                        leaf = 0;
                        break;
                    } else {
                        if (NEAREST_ANY) {
                            auto lower_first = [](float& ta, int& ka, float& tb, int& kb) {
                                if (tb < ta) {
                                    const float tt = ta;
                                    const int kk = ka;
                                    ta = tb;
                                    ka = kb;
                                    tb = tt;
                                    kb = kk;
                                }
                            };
                            lower_first(t0, k0, t1, k1);
                            lower_first(t2, k2, t3, k3);
                            lower_first(t0, k0, t2, k2);
                        }
                        node = SENTINEL;
                        if (t3 < INF_F) node = k3;
                        if (t2 < INF_F) {
                            if (node != SENTINEL) stack_node[sp++] = node;
                            node = k2;
                        }
                        if (t1 < INF_F) {
                            if (node != SENTINEL) stack_node[sp++] = node;
                            node = k1;
                        }
                        if (t0 < INF_F) {
                            if (node != SENTINEL) stack_node[sp++] = node;
                            node = k0;
                        }
                    }
                    if (node < 0 && leaf >= 0) {
                        leaf = node;
                        node = pop();
                    }
                    if (!__any_sync(__activemask(), leaf >= 0)) break;
                    continue;
                }
                // sort by entry distance (misses, at infinity, end up last)
                auto cswap = [](float& ta, int& ka, float& tb, int& kb) {
                    const bool sw = tb < ta;
                    const float tt = sw ? tb : ta;
                    const int kk = sw ? kb : ka;
                    tb = sw ? ta : tb;
                    kb = sw ? ka : kb;
                    ta = tt;
                    ka = kk;
                };
                cswap(t0, k0, t1, k1);
                cswap(t2, k2, t3, k3);
                cswap(t0, k0, t2, k2);
                cswap(t1, k1, t3, k3);
                cswap(t1, k1, t2, k2);
                if (nh == 0) {
                    node = pop();
                } else {
                    if (sp + nh - 1 > STACK_SIZE) {
                        overflow = true;
                        node = SENTINEL;
                        leaf = 0;
                        break;
                    }
                    if (nh > 3) push(k3, t3);
                    if (nh > 2) push(k2, t2);
                    if (nh > 1) push(k1, t1);
                    node = k0;
                }
                // postpone the first leaf reached
                if (node < 0 && leaf >= 0) {
                    leaf = node;
                    node = pop();
                }
                if (!__any_sync(__activemask(), leaf >= 0)) break;
            }
            // intersect the postponed leaf (and any leaf that follows it)
            while (leaf < 0) {
                const uint32_t code = ~(uint32_t)leaf;
                const bool found = leaf_test<ANY>(tris, (int)(code >> 4), (int)(code & 15u) + 1, o, d, tmin, best, h,
                                                  nt, COUNT);
                if (ANY && found) {
                    node = SENTINEL;
                    leaf = 0;
                    break;
                }
                leaf = node;
                if (node < 0) node = pop();
            }
        } while (__popc(__ballot_sync(FULL, node == SENTINEL)) < (ANY ? DYN_FETCH_ANY : DYN_FETCH));
    }
    if (COUNT) add_work(work, nv, nt);
}

}  // namespace vr
