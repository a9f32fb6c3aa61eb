// vr_kernels.h — launch interface between the C-ABI layer and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "vr_device.cuh"

namespace vr {

constexpr uint32_t MAX_DEPTH_SLOTS = 32;  // max_bounces must stay below this

struct RenderParams {
    float firefly_clamp;
    uint32_t max_bounces;
    int32_t render_mode;
    int32_t estimator;
    uint32_t rr_depth;
};

// One render job's part of a wavefront (device memory, one per job per wave).
struct Job {
    SceneView view;
    RenderParams rp;
    uint64_t seed;
    uint64_t g0;            // first global sample-major path of this wave
    uint32_t paths;         // paths of the job in this wave
    uint32_t base;          // first slot of the job's segment in every per-path array
    uint32_t num_pixels, width, height, first_sample;
    // Slot order of the job's paths in this wave.  Its global paths
    // [g0, g0 + paths) are `head` paths that finish a partly rendered sample
    // row, then `rows` full sample rows (row0 = the first of them), then the
    // start of the next row.  Head and tail keep the global order; the full
    // rows are stored pixel-major in tiled pixel order (slot head + P * rows + s
    // holds row row0 + s of tiled pixel P), so that a warp's rays and the
    // warps fetched after it start from the same few pixels.
    uint32_t head, rows, row0, pad_;
    float4* psum;           // per-pixel running sums (float4 per pixel)
    float4* aov_psum;       // optional: first-hit albedo sums [0, np), normal sums [np, 2 np)
};

constexpr uint32_t MAX_JOBS = 256;                       // jobs per wavefront
static_assert(sizeof(Job) % 4 == 0, "jobs are copied to shared memory as 32-bit words");
constexpr uint32_t JOB_COUNTERS = 2 * MAX_DEPTH_SLOTS;   // [k] queue size, [M + k] shadow queue size

// A wavefront: jobs[0..njobs) in device memory, their segments packed from slot 0.
struct Wave {
    const Job* jobs;
    uint32_t njobs;
    uint32_t total_paths;
    uint32_t max_bounces;   // over the jobs
    uint32_t any_nee;       // some job uses the NEE estimator
    uint32_t from_table;    // read every job from `jobs` even when njobs == 1 (graph replays)
    Job first;              // copy of jobs[0]: single-job waves read it from kernel parameters
};

// Device scratch of the wavefront integrator (structure of arrays, `cap`
// paths).  Ray queues are double buffered (2*cap entries).
struct PathState {
    uint32_t cap;
    uint32_t pad_;
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
    uint32_t* counts;   // MAX_JOBS * JOB_COUNTERS per-job queue sizes
    uint32_t* cursors;  // 2 * MAX_DEPTH_SLOTS fetch cursors: [k] extend, [M + k] shadow
    float4* aov;        // 2*cap, when some job wants AOVs: first-hit albedo [0, cap), normal [cap, 2 cap)
};

// Launch shapes chosen at run time (the autotuner's knobs): block size and
// resident blocks per SM of the shade / raygen stages.  `generation` changes
// on every set so cached CUDA graphs can tell a new shape.
struct Tuning {
    uint32_t shade_block = 256;
    uint32_t shade_blocks_per_sm = 8;
    uint32_t raygen_block = 256;
    uint32_t generation = 0;
};
Tuning get_tuning();
bool set_tuning(const Tuning& t);  // false: out of range (unchanged)

// Batch closest/any hit; `counter` is a device word the persistent kernel
// uses as its ray-fetch cursor (reset by the launcher).
// `perm` (optional): the order to trace the rays in (launch_ray_sort);
// hits are written back at the rays' own indices.
cudaError_t launch_intersect(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                             uint32_t* counter, uint32_t* status, cudaStream_t st, const uint32_t* perm = nullptr);
// Trace order of n rays: grouped by direction octant, then by origin cell
// (Morton order of 8 x 8 x 8 cells of the box lo..hi).  keys and perm hold n
// words each, hist 4096.
constexpr uint32_t RAY_SORT_BINS = 4096;
cudaError_t launch_ray_sort(const float4* rays, uint32_t n, const float* lo, const float* hi, uint32_t* keys,
                            uint32_t* hist, uint32_t* perm, cudaStream_t st);
cudaError_t launch_intersect_count(const SceneView& s, const float4* rays, uint64_t n, float4* hits, bool any,
                                   uint32_t* counter, unsigned long long* work, uint32_t* status, cudaStream_t st);
// Wavefront stages, in launch order: raygen (clears the wave's counters),
// then per depth k extend, shade and (NEE) shadow, then accumulate.  `work`
// (optional) receives traversal work counters (node visits, triangle tests).
cudaError_t launch_raygen(const Wave& w, const PathState& ps, cudaStream_t st);
cudaError_t launch_extend(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                          cudaStream_t st);
// `retired` (optional) counts the paths that end at this depth; retired[1]
// the Metal scatters whose bounded rejection loop ran out
cudaError_t launch_shade(const Wave& w, const PathState& ps, uint32_t k, unsigned long long* retired,
                         cudaStream_t st);
cudaError_t launch_shadow(const Wave& w, const PathState& ps, uint32_t k, uint32_t* status, unsigned long long* work,
                          cudaStream_t st);
cudaError_t launch_accumulate(const Wave& w, const PathState& ps, uint32_t max_pixels, unsigned long long* totals,
                              cudaStream_t st);
cudaError_t launch_finalize(const float4* psum, float4* rgba, uint32_t np, float inv_total, cudaStream_t st);
cudaError_t launch_tonemap(const float4* in, float4* out, uint32_t np, int32_t tonemap, float inv_gamma, float ex,
                           float scale, int32_t transparent, cudaStream_t st);
// rgba += (0, 0, 0, 1): a render call with zero samples
cudaError_t launch_empty_pass(float4* rgba, uint32_t np, cudaStream_t st);
cudaError_t launch_env_sample(const SceneView& s, const float* dirs, uint64_t n, float* rgb, cudaStream_t st);
cudaError_t launch_relmse(const float4* a, float sa, const float4* r, float sr, uint32_t np, double* out,
                          cudaStream_t st);

}  // namespace vr
