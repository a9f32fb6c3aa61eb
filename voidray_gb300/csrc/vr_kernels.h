// vr_kernels.h — launch interface between the C-ABI layer and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "vr_device.cuh"

namespace vr {

constexpr uint32_t MAX_DEPTH_SLOTS = 32;  // max_bounces must stay below this

// One wavefront: global sample-major path indices [g0, g0 + paths).
struct WaveParams {
    uint64_t g0;
    uint64_t seed;
    uint32_t paths;
    uint32_t num_pixels;
    uint32_t width, height;
    uint32_t first_sample;
    uint32_t pad_;
};

struct RenderParams {
    float firefly_clamp;
    uint32_t max_bounces;
    int32_t render_mode;
    int32_t estimator;
    uint32_t rr_depth;
};

// Device scratch of the wavefront integrator (structure of arrays, `cap`
// paths).  Ray queues are double buffered (2*cap entries).
struct PathState {
    uint32_t cap;
    uint32_t first_count;
    float4* q_org;      // (origin, tmin)    2*cap
    float4* q_dir;      // (direction, tmax) 2*cap
    uint32_t* q_path;   // path index        2*cap
    float4* hits;       // (prim bits, t, u, v) cap
    uint64_t* rng;      // PCG32 state       cap
    float4* thr;        // (throughput, previous bsdf pdf or -1) cap
    float4* rad;        // path radiance     cap
    float* att;         // reference estimator: attenuation per depth, [depth][rgb][cap]
    float4* s_org;      // shadow queue      cap
    float4* s_dir;
    float4* s_contrib;
    uint32_t* s_path;
    uint32_t* counts;   // 4*MAX_DEPTH_SLOTS words: [k] live paths at depth k, [M + k] shadow rays,
                        // [2M + k] extend fetch cursor, [3M + k] shadow fetch cursor
};

// Batch closest/any hit; `counter` is a device word the persistent kernel
// uses as its ray-fetch cursor (reset by the launcher).
cudaError_t launch_intersect(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                             uint32_t* counter, uint32_t* status, cudaStream_t st);
cudaError_t launch_intersect_count(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                                   uint32_t* counter, unsigned long long* work, uint32_t* status, cudaStream_t st);
// Wavefront stages, in launch order: raygen, then per depth k extend, shade
// and (NEE) shadow, then accumulate.  `work` (optional) receives traversal
// work counters (node visits, triangle tests) of that launch.
cudaError_t launch_raygen(const SceneView& s, const WaveParams& w, const PathState& ps, cudaStream_t st);
cudaError_t launch_extend(const SceneView& s, const WaveParams& w, const PathState& ps, uint32_t k, uint32_t* status,
                          unsigned long long* work, cudaStream_t st);
cudaError_t launch_shade(const SceneView& s, const WaveParams& w, const RenderParams& rp, const PathState& ps,
                         uint32_t k, cudaStream_t st);
cudaError_t launch_shadow(const SceneView& s, const WaveParams& w, const RenderParams& rp, const PathState& ps,
                          uint32_t k, uint32_t* status, unsigned long long* work, cudaStream_t st);
cudaError_t launch_accumulate(const WaveParams& w, const PathState& ps, const RenderParams& rp, float4* psum,
                              unsigned long long* totals, cudaStream_t st);
cudaError_t launch_finalize(const float4* psum, float4* rgba, uint32_t np, float inv_total, cudaStream_t st);
cudaError_t launch_tonemap(const float4* in, float4* out, uint32_t np, int32_t tonemap, float inv_gamma, float ex,
                           float scale, cudaStream_t st);
cudaError_t launch_relmse(const float4* a, float sa, const float4* r, float sr, uint32_t np, double* out,
                          cudaStream_t st);

}  // namespace vr
