// vr_capi.cu — implementation of the C ABI declared in include/voidray_gpu.h.
//
// Ownership: a vr_scene owns its device memory and one non-blocking CUDA
// stream; a vr_batch owns the scratch of multi-scene renders.  Render scratch
// (path state, ray queues, per-job counters and pixel sums) is allocated
// lazily and grown when a larger wavefront is requested.  Errors are returned
// as vr_status with a thread-local message; kernel-side faults that can be
// detected (traversal stack overflow) are recorded in a device status word
// and reported by the next synchronising call.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/voidray_gpu.h"
#include "vr_host.h"
#include "vr_kernels.h"

namespace {
thread_local std::string g_err;

vr_status fail(vr_status s, const std::string& m) {
    g_err = m;
    return s;
}

#define VR_CK(expr)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (expr);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            vr_status s_ = (e_ == cudaErrorMemoryAllocation) ? VR_ERR_OOM : VR_ERR_CUDA;              \
            return fail(s_, std::string(#expr) + ": " + cudaGetErrorString(e_));                       \
        }                                                                                             \
    } while (0)

bool device_ok() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n > 0;
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

vr_status ensure_buf(DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes) return VR_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    VR_CK(cudaMalloc(&b.p, bytes));
    b.bytes = bytes;
    return VR_OK;
}

// Wavefront scratch: per-slot path state and queues for `cap` slots, per-job
// counters, fetch cursors and a device table of Job entries.
struct Engine {
    vr::PathState ps{};
    uint32_t cap = 0, bounces = 0;
    bool aov = false;
    std::vector<void*> allocs;
    uint64_t bytes = 0;
    vr::Job* table = nullptr;  // device Job entries (waves x jobs of one chunk)
    size_t table_cap = 0;

    void release() {
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
        ps = vr::PathState{};
        cap = bounces = 0;
        aov = false;
        bytes = 0;
        table = nullptr;
        table_cap = 0;
    }
    template <class T>
    vr_status alloc(T** out, size_t count) {
        void* p = nullptr;
        const size_t b = std::max<size_t>(count * sizeof(T), 16);
        VR_CK(cudaMalloc(&p, b));
        allocs.push_back(p);
        bytes += b;
        *out = static_cast<T*>(p);
        return VR_OK;
    }
    // (re)allocates for `c` slots and reference-estimator attenuation of depth `b`
    vr_status ensure(uint32_t c, uint32_t b, cudaStream_t sync_stream, bool want_aov = false) {
        if (cap >= c && bounces >= b && table && (aov || !want_aov)) return VR_OK;
        if (sync_stream) VR_CK(cudaStreamSynchronize(sync_stream));
        c = std::max(c, cap);
        b = std::max(b, bounces);
        want_aov = want_aov || aov;
        release();
        vr_status st;
#define EA(field, n)                                  \
    if ((st = alloc(&ps.field, (n))) != VR_OK) {      \
        release();                                    \
        return st;                                    \
    }
        EA(q_org, 2 * (size_t)c);
        EA(q_dir, 2 * (size_t)c);
        EA(q_path, 2 * (size_t)c);
        EA(hits, (size_t)c);
        EA(rng, (size_t)c);
        EA(thr, (size_t)c);
        EA(rad, (size_t)c);
        EA(att, (size_t)std::max<uint32_t>(b, 1) * 3 * c);
        EA(s_org, (size_t)c);
        EA(s_dir, (size_t)c);
        EA(s_contrib, (size_t)c);
        EA(s_path, (size_t)c);
        EA(counts, (size_t)vr::MAX_JOBS * vr::JOB_COUNTERS);
        EA(cursors, 2 * (size_t)vr::MAX_DEPTH_SLOTS);
        if (want_aov) EA(aov, 2 * (size_t)c);
#undef EA
        table_cap = 4096;
        if ((st = alloc(&table, table_cap)) != VR_OK) {
            release();
            return st;
        }
        ps.cap = c;
        cap = c;
        bounces = b;
        aov = want_aov;
        return VR_OK;
    }
};

// Stage-event instrumentation of one scene.
struct Instr {
    uint32_t flags = 0;
    std::vector<cudaEvent_t> events;  // pool, reused across calls
    std::vector<int> event_stage;     // stage of the launch that ends at events[i] (i >= 1)
    size_t used = 0;
    double stage_ms[8] = {0};
    uint64_t stage_launches[8] = {0};
    unsigned long long* work = nullptr;  // device: extend visits, tests, shadow visits, tests, retired paths,
                                         // metal fallbacks

    vr_status mark(int stage, cudaStream_t cs) {
        if (!(flags & VR_INSTR_STAGE_TIMES)) return VR_OK;
        if (used == events.size()) {
            cudaEvent_t e;
            VR_CK(cudaEventCreate(&e));
            events.push_back(e);
            event_stage.push_back(-1);
        }
        event_stage[used] = stage;
        VR_CK(cudaEventRecord(events[used], cs));
        used++;
        return VR_OK;
    }
    // folds recorded events into the per-stage totals (after a synchronisation)
    vr_status collect() {
        for (size_t i = 1; i < used; ++i) {
            const int st = event_stage[i];
            if (st < 0) continue;
            float ms = 0.0f;
            VR_CK(cudaEventElapsedTime(&ms, events[i - 1], events[i]));
            stage_ms[st] += ms;
            stage_launches[st] += 1;
        }
        used = 0;
        return VR_OK;
    }
};

// Instantiated CUDA graphs of whole waves (wave begin, raygen, every depth's
// extend / shade / shadow, accumulate), keyed by everything the launches bake
// in.  The per-pass data (the Job entries: sample offsets, seeds, scenes) is
// read from the device table, which is uploaded before each replay, so one
// graph serves every pass of an unchanged job set.
struct GraphKey {
    const void* table;
    const void* ps_tag;
    const void* status;
    const void* totals;
    uint32_t njobs, total, max_bounces, any_nee, max_pixels, cap, tuning_generation, pad_;
};

struct GraphCache {
    struct Entry {
        GraphKey key;
        cudaGraphExec_t exec;
        uint64_t used;
    };
    std::vector<Entry> entries;
    std::vector<GraphKey> seen;  // shapes launched once without a graph (capture on the second sight)
    uint64_t tick = 0, captures = 0, replays = 0;
    bool broken = false;  // capture failed once: launch directly from then on

    void clear() {
        for (Entry& e : entries) cudaGraphExecDestroy(e.exec);
        entries.clear();
        seen.clear();
    }
    // true the first time a shape shows up (it then runs without a graph:
    // shapes that never repeat, like adaptive passes, cost no capture)
    bool first_sight(const GraphKey& k) {
        for (const GraphKey& s : seen)
            if (std::memcmp(&s, &k, sizeof k) == 0) return false;
        if (seen.size() >= 1024) seen.erase(seen.begin());
        seen.push_back(k);
        return true;
    }
    cudaGraphExec_t find(const GraphKey& k) {
        for (Entry& e : entries)
            if (std::memcmp(&e.key, &k, sizeof k) == 0) {
                e.used = ++tick;
                return e.exec;
            }
        return nullptr;
    }
    void insert(const GraphKey& k, cudaGraphExec_t x) {
        if (entries.size() >= 256) {
            size_t lru = 0;
            for (size_t i = 1; i < entries.size(); ++i)
                if (entries[i].used < entries[lru].used) lru = i;
            cudaGraphExecDestroy(entries[lru].exec);
            entries.erase(entries.begin() + lru);
        }
        entries.push_back({k, x, ++tick});
    }
};

}  // namespace

namespace vr {
vr_status set_error(vr_status s, const std::string& message) { return fail(s, message); }
bool device_usable() { return device_ok(); }
}  // namespace vr

struct vr_scene {
    int device = 0;
    cudaStream_t stream = nullptr;
    vr::SceneView view{};
    std::vector<void*> allocs;
    uint64_t scene_bytes = 0;
    vr_scene_info info{};
    vr_render_stats stats{};
    uint32_t* status = nullptr;            // device status word
    uint32_t* fetch = nullptr;             // ray-fetch cursor of the batch intersection kernel
    unsigned long long* totals = nullptr;  // device: paths, extend, shadow, counters x2
    Engine eng;                            // render scratch
    float4* psum = nullptr;
    uint32_t psum_cap = 0;
    DevBuf aov_psum;                       // first-hit AOV sums (2 float4 per pixel)
    DevBuf stage_a, stage_b;               // host-call staging
    DevBuf sortbuf;                        // batch queries: sort keys, trace order, histogram
    float blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};  // bounds of the triangles (the root node's children)
    Instr instr;
};

struct vr_batch {
    int device = 0;
    uint64_t max_wave_paths = 0;
    bool use_graphs = false;
    GraphCache graphs;
    Engine eng;
    DevBuf psum;       // pixel sums of all jobs of a call
    uint32_t* status = nullptr;
    unsigned long long* totals = nullptr;
    vr_render_stats stats{};
};

namespace {

template <class T>
vr_status upload(vr_scene* s, const std::vector<T>& v, const T** out) {
    *out = nullptr;
    if (v.empty()) return VR_OK;
    void* p = nullptr;
    size_t bytes = v.size() * sizeof(T);
    VR_CK(cudaMalloc(&p, bytes));
    s->allocs.push_back(p);
    s->scene_bytes += bytes;
    VR_CK(cudaMemcpy(p, v.data(), bytes, cudaMemcpyHostToDevice));
    *out = static_cast<const T*>(p);
    return VR_OK;
}

cudaStream_t pick(vr_scene* s, void* stream) { return stream ? static_cast<cudaStream_t>(stream) : s->stream; }

vr_status check_flags(uint32_t* status_dev, vr_render_stats& stats) {
    uint32_t flags = 0;
    VR_CK(cudaMemcpy(&flags, status_dev, 4, cudaMemcpyDeviceToHost));
    stats.error_flags |= flags;
    if (flags) {
        VR_CK(cudaMemset(status_dev, 0, 4));
        if (flags & vr::ERRF_STACK) return fail(VR_ERR_STACK, "traversal stack overflow in a kernel");
        return fail(VR_ERR_CUDA, "kernel reported error flags " + std::to_string(flags));
    }
    return VR_OK;
}
vr_status check_status(vr_scene* s) { return check_flags(s->status, s->stats); }

vr_status validate_settings(const vr_render_settings* st) {
    if (!st) return fail(VR_ERR_INVALID, "null settings");
    if (st->total_samples == 0) return fail(VR_ERR_INVALID, "total_samples must be > 0");
    if (st->max_bounces >= vr::MAX_DEPTH_SLOTS)
        return fail(VR_ERR_UNSUPPORTED, "max_bounces must be below " + std::to_string(vr::MAX_DEPTH_SLOTS));
    if (st->render_mode != VR_MODE_NORMAL && st->render_mode != VR_MODE_FULL)
        return fail(VR_ERR_INVALID, "render_mode");
    if (st->estimator != VR_EST_REFERENCE && st->estimator != VR_EST_NEE) return fail(VR_ERR_INVALID, "estimator");
    return VR_OK;
}

vr_status validate_render(const vr_scene* scene, const vr_render_settings* st, uint32_t w, uint32_t h) {
    if (!scene || !st) return fail(VR_ERR_INVALID, "null scene or settings");
    if (w == 0 || h == 0) return fail(VR_ERR_INVALID, "empty image");
    if ((uint64_t)w * h >= (1ull << 31)) return fail(VR_ERR_INVALID, "image too large");
    return validate_settings(st);
}

// One render job on the host side of the wave planner.
struct HostJob {
    vr::Job tmpl;      // view, rp, seed, num_pixels, width, height, first_sample, psum
    uint64_t total;    // paths = samples * pixels
    uint64_t done = 0;
    float4* rgba;
    float inv_total;
    float4* albedo = nullptr;  // optional AOV outputs (accumulated like rgba)
    float4* normal = nullptr;
};

// Single-job waves of at least this many paths launch their stages directly
// even when graphs are on.
constexpr uint32_t SINGLE_JOB_GRAPH_LIMIT = 1u << 22;

// Plans waves of at most `cap` slots over the jobs (each wave takes, in job
// order, as many of every unfinished job's next paths as fit), uploads the
// Job entries of up to `table_cap` entries at a time, and launches the stage
// sequence of every wave.  A job whose last paths ran in a wave is finalised
// right after it.  `instr` (optional) brackets every launch with events.
// With `graphs` (and a capturable stream) every wave runs as a replay of a
// cached CUDA graph of its stage sequence.
vr_status run_waves(std::vector<HostJob>& jobs, const vr::PathState& ps, uint32_t cap, vr::Job* table,
                    size_t table_cap, uint32_t* status, unsigned long long* totals, Instr* instr, cudaStream_t cs,
                    uint64_t* waves_out, GraphCache* graphs = nullptr) {
    vr_status r;
    unsigned long long* wk = (instr && (instr->flags & VR_INSTR_WORK)) ? instr->work : nullptr;
    if (instr && (instr->flags & VR_INSTR_STAGE_TIMES) && instr->used > 0) {
        VR_CK(cudaStreamSynchronize(cs));
        if ((r = instr->collect()) != VR_OK) return r;
    }
    if (instr && (r = instr->mark(-1, cs)) != VR_OK) return r;
    uint64_t waves = 0;
    std::vector<vr::Job> chunk;
    struct WaveHost {
        size_t first, njobs;
        uint32_t total, max_bounces, max_pixels;
        bool any_nee;
        std::vector<size_t> finishing;
    };
    std::vector<WaveHost> plan;
    auto pending = [&]() {
        for (const HostJob& j : jobs)
            if (j.done < j.total) return true;
        return false;
    };
    std::vector<size_t> entry_job;  // job index of every chunk entry
    while (pending()) {
        // plan a chunk of waves whose entries fit the device table
        chunk.clear();
        entry_job.clear();
        plan.clear();
        while (pending()) {
            WaveHost wh{chunk.size(), 0, 0, 0, 0, false, {}};
            uint32_t left = cap;
            // A job with at least a full wave of paths left gets the wave to
            // itself (whole sample rows): single-job waves run the single-job
            // kernel variants, about 5% faster than the multi-job ones.  The
            // jobs' tails and the small jobs share the remaining waves.
            size_t solo = jobs.size();
            for (size_t i = 0; i < jobs.size(); ++i)
                if (jobs[i].total - jobs[i].done >= cap) {
                    solo = i;
                    break;
                }
            for (size_t i = (solo < jobs.size() ? solo : 0); i < jobs.size() && left > 0 && wh.njobs < vr::MAX_JOBS;
                 ++i) {
                HostJob& j = jobs[i];
                if (j.done >= j.total) continue;
                if (solo < jobs.size() && i != solo) break;
                uint32_t take = (uint32_t)std::min<uint64_t>(left, j.total - j.done);
                // a job that does not finish in this wave takes whole sample rows
                // when it can (pixel-major slot order), leaving the rest of the
                // wave to the jobs after it
                if (take < j.total - j.done && take >= j.tmpl.num_pixels)
                    take -= (take + (uint32_t)(j.done % j.tmpl.num_pixels)) % j.tmpl.num_pixels;
                vr::Job e = j.tmpl;
                e.g0 = j.done;
                e.paths = take;
                e.base = cap - left;
                {  // slot order (vr::Job::head): partial row, full rows pixel-major, partial row
                    const uint64_t np = e.num_pixels;
                    const uint64_t head = std::min<uint64_t>((np - e.g0 % np) % np, take);
                    e.head = (uint32_t)head;
                    e.rows = (uint32_t)((take - head) / np);
                    e.row0 = (uint32_t)((e.g0 + head) / np);
                    e.pad_ = 0;
                }
                chunk.push_back(e);
                entry_job.push_back(i);
                wh.njobs++;
                wh.total += take;
                wh.max_bounces = std::max(wh.max_bounces, e.rp.max_bounces);
                wh.max_pixels = std::max(wh.max_pixels, e.num_pixels);
                wh.any_nee = wh.any_nee || e.rp.estimator == VR_EST_NEE;
                left -= take;
                j.done += take;
                if (j.done == j.total) wh.finishing.push_back(i);
            }
            if (chunk.size() > table_cap) {  // does not fit this chunk: undo and run what is planned
                for (size_t k = wh.first; k < chunk.size(); ++k) jobs[entry_job[k]].done -= chunk[k].paths;
                chunk.resize(wh.first);
                entry_job.resize(wh.first);
                break;
            }
            plan.push_back(std::move(wh));
        }
        if (plan.empty()) return fail(VR_ERR_INVALID, "wave table too small for one wave");
        // pageable host -> device: the host vector may be reused once the call returns
        VR_CK(cudaMemcpyAsync(table, chunk.data(), chunk.size() * sizeof(vr::Job), cudaMemcpyHostToDevice, cs));
        const bool graphs_on = graphs && !graphs->broken && cs && !instr;
        for (const WaveHost& wh : plan) {
            // A replayed graph reads its jobs from the device table, i.e. runs
            // the multi-job kernel variants, which cost about 5% over the
            // single-job ones (job fields from shared memory instead of kernel
            // parameters); a large single-job wave gains nothing from a graph
            // (its launches are microseconds against a wave of milliseconds),
            // so it launches directly.
            const bool use_graphs = graphs_on && (wh.njobs > 1 || wh.total < SINGLE_JOB_GRAPH_LIMIT);
            const vr::Wave wv{table + wh.first, (uint32_t)wh.njobs, wh.total,         wh.max_bounces,
                              wh.any_nee ? 1u : 0u, use_graphs ? 1u : 0u, chunk[wh.first]};
            auto stages = [&]() -> vr_status {
                VR_CK(vr::launch_raygen(wv, ps, cs));
                if (instr && (r = instr->mark(VR_STAGE_RAYGEN, cs)) != VR_OK) return r;
                for (uint32_t k = 0; k < wv.max_bounces; ++k) {
                    VR_CK(vr::launch_extend(wv, ps, k, status, wk, cs));
                    if (instr && (r = instr->mark(VR_STAGE_EXTEND, cs)) != VR_OK) return r;
                    VR_CK(vr::launch_shade(wv, ps, k, wk ? wk + 4 : nullptr, cs));
                    if (instr && (r = instr->mark(VR_STAGE_SHADE, cs)) != VR_OK) return r;
                    if (wv.any_nee) {
                        VR_CK(vr::launch_shadow(wv, ps, k, status, wk ? wk + 2 : nullptr, cs));
                        if (instr && (r = instr->mark(VR_STAGE_SHADOW, cs)) != VR_OK) return r;
                    }
                }
                VR_CK(vr::launch_accumulate(wv, ps, wh.max_pixels, totals, cs));
                if (instr && (r = instr->mark(VR_STAGE_ACCUMULATE, cs)) != VR_OK) return r;
                return VR_OK;
            };
            if (use_graphs) {
                GraphKey key;
                std::memset(&key, 0, sizeof key);
                key.table = wv.jobs;
                key.ps_tag = ps.q_org;
                key.status = status;
                key.totals = totals;
                key.njobs = wv.njobs;
                key.total = wv.total_paths;
                key.max_bounces = wv.max_bounces;
                key.any_nee = wv.any_nee;
                key.max_pixels = wh.max_pixels;
                key.cap = ps.cap;
                key.tuning_generation = vr::get_tuning().generation;
                cudaGraphExec_t ex = graphs->find(key);
                const bool capture = !ex && !graphs->first_sight(key);
                if (capture) {
                    VR_CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                    const vr_status sr = stages();
                    cudaGraph_t g = nullptr;
                    const cudaError_t ee = cudaStreamEndCapture(cs, &g);
                    cudaError_t ie = cudaErrorUnknown;
                    if (sr == VR_OK && ee == cudaSuccess && g) ie = cudaGraphInstantiate(&ex, g, 0);
                    if (g) cudaGraphDestroy(g);
                    if (ie != cudaSuccess) {
                        // capture not possible here: run the stages directly from now on
                        cudaGetLastError();
                        graphs->broken = true;
                        ex = nullptr;
                    } else {
                        graphs->insert(key, ex);
                        graphs->captures++;
                    }
                } else if (ex) {
                    graphs->replays++;
                }
                if (ex) {
                    VR_CK(cudaGraphLaunch(ex, cs));
                } else if ((r = stages()) != VR_OK) {  // from_table stays set: same results
                    return r;
                }
            } else if ((r = stages()) != VR_OK) {
                return r;
            }
            for (size_t i : wh.finishing) {
                const HostJob& j = jobs[i];
                VR_CK(vr::launch_finalize(j.tmpl.psum, j.rgba, j.tmpl.num_pixels, j.inv_total, cs));
                if (j.tmpl.aov_psum) {
                    VR_CK(vr::launch_finalize(j.tmpl.aov_psum, j.albedo, j.tmpl.num_pixels, j.inv_total, cs));
                    VR_CK(vr::launch_finalize(j.tmpl.aov_psum + j.tmpl.num_pixels, j.normal, j.tmpl.num_pixels,
                                              j.inv_total, cs));
                }
            }
            ++waves;
        }
    }
    if (waves_out) *waves_out += waves;
    return VR_OK;
}

HostJob make_job(const vr::SceneView& view, const vr_render_settings* st, uint32_t samples, float* rgba, uint32_t w,
                 uint32_t h, uint64_t seed, uint32_t first_sample, float4* psum) {
    HostJob j{};
    j.tmpl.view = view;
    j.tmpl.rp = vr::RenderParams{st->firefly_clamp, st->max_bounces, st->render_mode, st->estimator, st->rr_depth};
    j.tmpl.seed = seed;
    j.tmpl.num_pixels = w * h;
    j.tmpl.width = w;
    j.tmpl.height = h;
    j.tmpl.first_sample = first_sample;
    j.tmpl.psum = psum;
    j.total = (uint64_t)samples * w * h;
    j.rgba = reinterpret_cast<float4*>(rgba);
    j.inv_total = 1.0f / (float)st->total_samples;
    return j;
}

}  // namespace

extern "C" {

const char* vr_last_error(void) { return g_err.c_str(); }
int32_t vr_abi_version(void) { return VR_ABI_VERSION; }
int32_t vr_device_available(void) { return device_ok() ? 1 : 0; }

vr_status vr_scene_create(const vr_scene_desc* desc, vr_scene** out) {
    if (!out) return fail(VR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    vr::HostScene hs;
    std::string err;
    vr_status st = vr::build_host_scene(desc, hs, err);
    if (st != VR_OK) return fail(st, err);
    vr_scene* s = new vr_scene();
    auto cleanup = [&](vr_status r) {
        vr_scene_destroy(s);
        return r;
    };
    cudaGetDevice(&s->device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(fail(VR_ERR_CUDA, "stream creation failed"));
    s->view = hs.view;
    if (!hs.wide.empty()) {  // triangle bounds: the union of the root's child boxes
        for (int a = 0; a < 3; ++a) {
            s->blo[a] = INFINITY;
            s->bhi[a] = -INFINITY;
        }
        int32_t cd[4];
        std::memcpy(cd, &hs.wide[6], sizeof cd);
        for (int c = 0; c < 4; ++c) {
            if (cd[c] == 0x7fffffff) continue;
            const float4 xy = hs.wide[3 * (c >> 1) + (c & 1)], z = hs.wide[3 * (c >> 1) + 2];
            const float lo[3] = {xy.x, xy.z, (c & 1) ? z.z : z.x}, hi[3] = {xy.y, xy.w, (c & 1) ? z.w : z.y};
            for (int a = 0; a < 3; ++a) {
                s->blo[a] = std::min(s->blo[a], lo[a]);
                s->bhi[a] = std::max(s->bhi[a], hi[a]);
            }
        }
    }
    if ((st = upload(s, hs.wide, &s->view.nodes)) != VR_OK) return cleanup(st);  // the 4-wide tree
    if ((st = upload(s, hs.tris, &s->view.tris)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.shade, &s->view.shade)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.uvs, &s->view.uvs)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.materials, &s->view.materials)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.analytic, &s->view.analytic)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.tex_info, &s->view.tex_info)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.texels, &s->view.texels)) != VR_OK) return cleanup(st);
    if ((st = upload(s, hs.env_img, &s->view.env_img)) != VR_OK) return cleanup(st);
    if (hs.has_tables) {
        if ((st = upload(s, hs.tables.marginal, &s->view.env_marg)) != VR_OK) return cleanup(st);
        if ((st = upload(s, hs.tables.conditional, &s->view.env_cond)) != VR_OK) return cleanup(st);
        if ((st = upload(s, hs.tables.cell, &s->view.env_cell)) != VR_OK) return cleanup(st);
        if ((st = upload(s, hs.tables.guide_marginal, &s->view.env_gmarg)) != VR_OK) return cleanup(st);
        if ((st = upload(s, hs.tables.guide_conditional, &s->view.env_gcond)) != VR_OK) return cleanup(st);
        s->view.env_gm = hs.tables.gm;
        s->view.env_gc = hs.tables.gc;
    }
    void* p = nullptr;
    if (cudaMalloc(&p, 64) != cudaSuccess) return cleanup(fail(VR_ERR_OOM, "status alloc"));
    s->allocs.push_back(p);
    s->status = static_cast<uint32_t*>(p);
    if (cudaMalloc(&p, 64) != cudaSuccess) return cleanup(fail(VR_ERR_OOM, "fetch alloc"));
    s->allocs.push_back(p);
    s->fetch = static_cast<uint32_t*>(p);
    if (cudaMalloc(&p, 8 * sizeof(unsigned long long)) != cudaSuccess) return cleanup(fail(VR_ERR_OOM, "totals alloc"));
    s->allocs.push_back(p);
    s->totals = static_cast<unsigned long long*>(p);
    if (cudaMemset(s->status, 0, 64) != cudaSuccess || cudaMemset(s->totals, 0, 64) != cudaSuccess)
        return cleanup(fail(VR_ERR_CUDA, "memset"));
    s->info.num_triangles = hs.num_prims;
    s->info.num_nodes = hs.wide.size() / 8;
    s->info.device_bytes = s->scene_bytes;
    s->info.max_depth = hs.max_depth;
    s->info.max_leaf = hs.max_leaf;
    s->info.sah_cost = hs.sah_cost;
    s->info.build_ms = hs.build_ms;
    *out = s;
    return VR_OK;
}

vr_status vr_scene_validate(const vr_scene_desc* desc, vr_scene_info* info) {
    vr::HostScene hs;
    std::string err;
    vr_status st = vr::build_host_scene(desc, hs, err);
    if (st != VR_OK) return fail(st, err);
    st = vr::validate_host_scene(hs, err);
    if (st != VR_OK) return fail(st, err);
    if (info) {
        *info = vr_scene_info{};
        info->num_triangles = hs.num_prims;
        info->num_nodes = hs.wide.size() / 8;
        // every array vr_scene_create uploads (textures and materials included)
        info->device_bytes = hs.wide.size() * sizeof(float4) + hs.tris.size() * sizeof(float4) +
                             hs.shade.size() * sizeof(float4) + hs.uvs.size() * sizeof(float2) +
                             hs.materials.size() * sizeof(hs.materials[0]) + hs.analytic.size() * sizeof(float4) +
                             hs.tex_info.size() * sizeof(int4) + hs.texels.size() * sizeof(float) +
                             hs.env_img.size() * sizeof(float) +
                             (hs.has_tables ? (hs.tables.marginal.size() + hs.tables.conditional.size() +
                                               hs.tables.cell.size()) * sizeof(float)
                                            : 0);
        info->max_depth = hs.max_depth;
        info->max_leaf = hs.max_leaf;
        info->sah_cost = hs.sah_cost;
        info->build_ms = hs.build_ms;
    }
    return VR_OK;
}

vr_status vr_scene_instrument(vr_scene* s, uint32_t flags) {
    if (!s) return fail(VR_ERR_INVALID, "null scene");
    VR_CK(cudaStreamSynchronize(s->stream));
    if (!s->instr.work) VR_CK(cudaMalloc(&s->instr.work, 6 * sizeof(unsigned long long)));
    VR_CK(cudaMemset(s->instr.work, 0, 6 * sizeof(unsigned long long)));
    s->instr.flags = flags;
    s->instr.used = 0;
    for (int i = 0; i < 8; ++i) {
        s->instr.stage_ms[i] = 0.0;
        s->instr.stage_launches[i] = 0;
    }
    return VR_OK;
}

vr_status vr_scene_instrument_get(vr_scene* s, vr_instrument* out) {
    if (!s || !out) return fail(VR_ERR_INVALID, "null argument");
    VR_CK(cudaDeviceSynchronize());
    vr_status r = s->instr.collect();
    if (r != VR_OK) return r;
    *out = vr_instrument{};
    for (int i = 0; i < 8; ++i) {
        out->stage_ms[i] = s->instr.stage_ms[i];
        out->stage_launches[i] = s->instr.stage_launches[i];
    }
    if (s->instr.work) {
        unsigned long long w[6];
        VR_CK(cudaMemcpy(w, s->instr.work, sizeof w, cudaMemcpyDeviceToHost));
        out->extend_node_visits = w[0];
        out->extend_tri_tests = w[1];
        out->shadow_node_visits = w[2];
        out->shadow_tri_tests = w[3];
        out->retired_paths = w[4];
        out->metal_fallbacks = w[5];
    }
    return VR_OK;
}

vr_status vr_scene_destroy(vr_scene* s) {
    if (!s) return VR_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (cudaEvent_t e : s->instr.events) cudaEventDestroy(e);
    if (s->instr.work) cudaFree(s->instr.work);
    s->eng.release();
    if (s->psum) cudaFree(s->psum);
    if (s->aov_psum.p) cudaFree(s->aov_psum.p);
    if (s->stage_a.p) cudaFree(s->stage_a.p);
    if (s->stage_b.p) cudaFree(s->stage_b.p);
    if (s->sortbuf.p) cudaFree(s->sortbuf.p);
    for (void* p : s->allocs) cudaFree(p);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return VR_OK;
}

vr_status vr_scene_info_get(const vr_scene* s, vr_scene_info* info) {
    if (!s || !info) return fail(VR_ERR_INVALID, "null argument");
    *info = s->info;
    info->device_bytes = s->scene_bytes;
    return VR_OK;
}

vr_status vr_scene_set_camera(vr_scene* s, const vr_camera_desc* cam) {
    if (!s || !cam) return fail(VR_ERR_INVALID, "null argument");
    vr::set_camera(s->view, *cam);
    return VR_OK;
}

vr_status vr_scene_synchronize(vr_scene* s) {
    if (!s) return fail(VR_ERR_INVALID, "null scene");
    VR_CK(cudaStreamSynchronize(s->stream));
    return check_status(s);
}

vr_status vr_render_device(vr_scene* s, const vr_render_settings* st, uint32_t samples, float* rgba, uint32_t w,
                           uint32_t h, uint64_t seed, uint32_t first_sample, void* stream) {
    vr_status r = validate_render(s, st, w, h);
    if (r != VR_OK) return r;
    if (!rgba) return fail(VR_ERR_INVALID, "rgba is NULL");
    if ((uint64_t)first_sample + samples >= (1ull << 31)) return fail(VR_ERR_INVALID, "sample index out of range");
    cudaStream_t cs = pick(s, stream);
    const uint32_t np = w * h;
    if (samples == 0) {
        VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(rgba), np, cs));
        return VR_OK;
    }
    const uint64_t total = (uint64_t)samples * np;
    // default wavefront: 2^28 paths (at most: a render of fewer paths holds
    // only those; about 48 GB of path state with the NEE estimator).  Fewer,
    // larger waves spend less time in their deep-bounce tails, whose
    // launches keep few rays alive: on the 2M-triangle 1080p frame 2^26
    // paths gave 952 M samples/s, 2^27 1017 M, 2^28 1053 M
    uint64_t cap = st->wavefront_paths ? st->wavefront_paths : (1ull << 28);
    if (cap > (1ull << 28)) cap = 1ull << 28;
    if (cap > total) cap = total;
    if (cap > np) cap -= cap % np;  // whole sample rows per wavefront: every slot in pixel-major order
    const uint32_t att_depth = st->estimator == VR_EST_REFERENCE ? st->max_bounces : 0;
    if ((r = s->eng.ensure((uint32_t)cap, att_depth, s->stream)) != VR_OK) return r;
    if (s->psum_cap < np) {
        VR_CK(cudaStreamSynchronize(s->stream));
        if (s->psum) cudaFree(s->psum);
        s->psum = nullptr;
        s->psum_cap = 0;
        VR_CK(cudaMalloc(&s->psum, (size_t)np * sizeof(float4)));
        s->psum_cap = np;
    }
    VR_CK(cudaMemsetAsync(s->psum, 0, (size_t)np * sizeof(float4), cs));
    std::vector<HostJob> jobs{make_job(s->view, st, samples, rgba, w, h, seed, first_sample, s->psum)};
    auto t0 = std::chrono::steady_clock::now();
    if ((r = run_waves(jobs, s->eng.ps, (uint32_t)cap, s->eng.table, s->eng.table_cap, s->status, s->totals, &s->instr,
                       cs, &s->stats.wavefronts)) != VR_OK)
        return r;
    s->stats.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return VR_OK;
}

vr_status vr_render_aov_device(vr_scene* s, const vr_render_settings* st, uint32_t samples, float* rgba,
                               float* albedo, float* normal, uint32_t w, uint32_t h, uint64_t seed,
                               uint32_t first_sample, void* stream) {
    vr_status r = validate_render(s, st, w, h);
    if (r != VR_OK) return r;
    if (!rgba || !albedo || !normal) return fail(VR_ERR_INVALID, "rgba, albedo and normal must be set");
    if ((uint64_t)first_sample + samples >= (1ull << 31)) return fail(VR_ERR_INVALID, "sample index out of range");
    cudaStream_t cs = pick(s, stream);
    const uint32_t np = w * h;
    if (samples == 0) {
        for (float* buf : {rgba, albedo, normal}) VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(buf), np, cs));
        return VR_OK;
    }
    const uint64_t total = (uint64_t)samples * np;
    uint64_t cap = st->wavefront_paths ? st->wavefront_paths : (1ull << 28);
    if (cap > (1ull << 28)) cap = 1ull << 28;
    if (cap > total) cap = total;
    if (cap > np) cap -= cap % np;  // whole sample rows per wavefront
    const uint32_t att_depth = st->estimator == VR_EST_REFERENCE ? st->max_bounces : 0;
    if ((r = s->eng.ensure((uint32_t)cap, att_depth, s->stream, true)) != VR_OK) return r;
    if (s->psum_cap < np) {
        VR_CK(cudaStreamSynchronize(s->stream));
        if (s->psum) cudaFree(s->psum);
        s->psum = nullptr;
        s->psum_cap = 0;
        VR_CK(cudaMalloc(&s->psum, (size_t)np * sizeof(float4)));
        s->psum_cap = np;
    }
    if (s->aov_psum.bytes < 2 * (size_t)np * sizeof(float4)) {
        VR_CK(cudaStreamSynchronize(s->stream));
        if ((r = ensure_buf(s->aov_psum, 2 * (size_t)np * sizeof(float4))) != VR_OK) return r;
    }
    VR_CK(cudaMemsetAsync(s->psum, 0, (size_t)np * sizeof(float4), cs));
    VR_CK(cudaMemsetAsync(s->aov_psum.p, 0, 2 * (size_t)np * sizeof(float4), cs));
    HostJob j = make_job(s->view, st, samples, rgba, w, h, seed, first_sample, s->psum);
    j.tmpl.aov_psum = static_cast<float4*>(s->aov_psum.p);
    j.albedo = reinterpret_cast<float4*>(albedo);
    j.normal = reinterpret_cast<float4*>(normal);
    std::vector<HostJob> jobs{j};
    return run_waves(jobs, s->eng.ps, (uint32_t)cap, s->eng.table, s->eng.table_cap, s->status, s->totals, &s->instr, cs,
                     &s->stats.wavefronts);
}

vr_status vr_render(vr_scene* s, const vr_render_settings* st, uint32_t samples, float* rgba, uint32_t w, uint32_t h,
                    uint64_t seed, uint32_t first_sample) {
    vr_status r = validate_render(s, st, w, h);
    if (r != VR_OK) return r;
    if (!rgba) return fail(VR_ERR_INVALID, "rgba is NULL");
    const size_t bytes = (size_t)w * h * 4 * sizeof(float);
    if ((r = ensure_buf(s->stage_a, bytes)) != VR_OK) return r;
    auto t0 = std::chrono::steady_clock::now();
    VR_CK(cudaMemcpyAsync(s->stage_a.p, rgba, bytes, cudaMemcpyHostToDevice, s->stream));
    if ((r = vr_render_device(s, st, samples, static_cast<float*>(s->stage_a.p), w, h, seed, first_sample, nullptr)) !=
        VR_OK)
        return r;
    VR_CK(cudaMemcpyAsync(rgba, s->stage_a.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    VR_CK(cudaStreamSynchronize(s->stream));
    s->stats.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return check_status(s);
}

vr_status vr_render_stats_get(const vr_scene* cs, vr_render_stats* out) {
    if (!cs || !out) return fail(VR_ERR_INVALID, "null argument");
    vr_scene* s = const_cast<vr_scene*>(cs);
    VR_CK(cudaStreamSynchronize(s->stream));
    unsigned long long t[3] = {0, 0, 0};
    VR_CK(cudaMemcpy(t, s->totals, sizeof t, cudaMemcpyDeviceToHost));
    uint32_t flags = 0;
    VR_CK(cudaMemcpy(&flags, s->status, 4, cudaMemcpyDeviceToHost));
    *out = s->stats;
    out->paths = t[0];
    out->extend_rays = t[1];
    out->shadow_rays = t[2];
    out->error_flags |= flags;
    return VR_OK;
}

// ------------------------------------------------------------------ batch --

vr_status vr_batch_create(uint64_t max_wave_paths, vr_batch** out) {
    if (!out) return fail(VR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    vr_batch* b = new vr_batch();
    cudaGetDevice(&b->device);
    b->max_wave_paths = max_wave_paths ? std::min<uint64_t>(max_wave_paths, 1ull << 28) : (1ull << 26);
    void* p = nullptr;
    if (cudaMalloc(&p, 64) != cudaSuccess) {
        delete b;
        return fail(VR_ERR_OOM, "status alloc");
    }
    b->status = static_cast<uint32_t*>(p);
    if (cudaMalloc(&p, 64) != cudaSuccess) {
        cudaFree(b->status);
        delete b;
        return fail(VR_ERR_OOM, "totals alloc");
    }
    b->totals = static_cast<unsigned long long*>(p);
    cudaMemset(b->status, 0, 64);
    cudaMemset(b->totals, 0, 64);
    *out = b;
    return VR_OK;
}

vr_status vr_batch_destroy(vr_batch* b) {
    if (!b) return VR_OK;
    cudaDeviceSynchronize();
    b->graphs.clear();
    b->eng.release();
    if (b->psum.p) cudaFree(b->psum.p);
    if (b->status) cudaFree(b->status);
    if (b->totals) cudaFree(b->totals);
    delete b;
    return VR_OK;
}

vr_status vr_batch_render(vr_batch* b, const vr_render_job* jobs, uint32_t count, void* stream) {
    if (!b) return fail(VR_ERR_INVALID, "null batch");
    if (count && !jobs) return fail(VR_ERR_INVALID, "null jobs");
    vr_status r;
    uint64_t total = 0, pixels = 0;
    uint32_t att_depth = 0;
    bool want_aov = false;
    for (uint32_t i = 0; i < count; ++i) {
        const vr_render_job& j = jobs[i];
        if ((r = validate_render(j.scene, &j.settings, j.width, j.height)) != VR_OK)
            return fail(r, "job " + std::to_string(i) + ": " + g_err);
        if (!j.rgba_device) return fail(VR_ERR_INVALID, "job " + std::to_string(i) + ": rgba is NULL");
        if (!j.albedo_device != !j.normal_device)
            return fail(VR_ERR_INVALID, "job " + std::to_string(i) + ": set both AOV buffers or neither");
        const bool aov = j.albedo_device && j.samples;
        want_aov = want_aov || aov;
        if ((uint64_t)j.first_sample + j.samples >= (1ull << 31))
            return fail(VR_ERR_INVALID, "job " + std::to_string(i) + ": sample index out of range");
        if (j.scene->device != b->device) return fail(VR_ERR_INVALID, "job " + std::to_string(i) + ": other device");
        total += (uint64_t)j.samples * j.width * j.height;
        pixels += (uint64_t)j.width * j.height * (aov ? 3 : 1);
        if (j.settings.estimator == VR_EST_REFERENCE) att_depth = std::max(att_depth, j.settings.max_bounces);
    }
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // zero-sample jobs still add (0, 0, 0, 1) to their images, like iterative_render
    for (uint32_t i = 0; i < count; ++i) {
        const vr_render_job& j = jobs[i];
        if (j.samples) continue;
        const uint32_t np = j.width * j.height;
        VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(j.rgba_device), np, cs));
        if (j.albedo_device) {
            VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(j.albedo_device), np, cs));
            VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(j.normal_device), np, cs));
        }
    }
    if (total == 0) return VR_OK;
    uint64_t cap = std::min<uint64_t>(b->max_wave_paths, total);
    if (count == 1 && cap > (uint64_t)jobs[0].width * jobs[0].height)  // one job: whole sample rows per wave
        cap -= cap % ((uint64_t)jobs[0].width * jobs[0].height);
    const void* before = b->eng.ps.q_org;
    if ((r = b->eng.ensure((uint32_t)cap, att_depth, cs, want_aov)) != VR_OK) return r;
    if (b->eng.ps.q_org != before) b->graphs.clear();  // graphs bake in the old scratch pointers
    if (b->psum.bytes < pixels * sizeof(float4)) {
        VR_CK(cudaStreamSynchronize(cs));
        if ((r = ensure_buf(b->psum, pixels * sizeof(float4))) != VR_OK) return r;
    }
    VR_CK(cudaMemsetAsync(b->psum.p, 0, pixels * sizeof(float4), cs));
    std::vector<HostJob> hj;
    hj.reserve(count);
    float4* ps = static_cast<float4*>(b->psum.p);
    for (uint32_t i = 0; i < count; ++i) {
        const vr_render_job& j = jobs[i];
        if (j.samples == 0) continue;
        hj.push_back(make_job(j.scene->view, &j.settings, j.samples, j.rgba_device, j.width, j.height, j.seed,
                              j.first_sample, ps));
        ps += (size_t)j.width * j.height;
        if (j.albedo_device) {
            hj.back().tmpl.aov_psum = ps;
            hj.back().albedo = reinterpret_cast<float4*>(j.albedo_device);
            hj.back().normal = reinterpret_cast<float4*>(j.normal_device);
            ps += 2 * (size_t)j.width * j.height;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    if ((r = run_waves(hj, b->eng.ps, (uint32_t)cap, b->eng.table, b->eng.table_cap, b->status, b->totals, nullptr, cs,
                       &b->stats.wavefronts, b->use_graphs ? &b->graphs : nullptr)) != VR_OK)
        return r;
    b->stats.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return VR_OK;
}

vr_status vr_tuning_get(vr_tuning* out) {
    if (!out) return fail(VR_ERR_INVALID, "null argument");
    const vr::Tuning t = vr::get_tuning();
    out->shade_block = t.shade_block;
    out->shade_blocks_per_sm = t.shade_blocks_per_sm;
    out->raygen_block = t.raygen_block;
    out->generation = t.generation;
    return VR_OK;
}

vr_status vr_tuning_set(const vr_tuning* in) {
    if (!in) return fail(VR_ERR_INVALID, "null argument");
    vr::Tuning t;
    t.shade_block = in->shade_block;
    t.shade_blocks_per_sm = in->shade_blocks_per_sm;
    t.raygen_block = in->raygen_block;
    if (!vr::set_tuning(t))
        return fail(VR_ERR_INVALID, "blocks must be 64, 128 or 256 threads, 1-32 shade blocks per SM");
    return VR_OK;
}

vr_status vr_batch_set_graphs(vr_batch* b, int32_t enable) {
    if (!b) return fail(VR_ERR_INVALID, "null batch");
    b->use_graphs = enable != 0;
    return VR_OK;
}

vr_status vr_batch_graph_stats(vr_batch* b, uint64_t* captures, uint64_t* replays) {
    if (!b || !captures || !replays) return fail(VR_ERR_INVALID, "null argument");
    *captures = b->graphs.captures;
    *replays = b->graphs.replays;
    return VR_OK;
}

vr_status vr_batch_synchronize(vr_batch* b, void* stream) {
    if (!b) return fail(VR_ERR_INVALID, "null batch");
    VR_CK(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return check_flags(b->status, b->stats);
}

vr_status vr_batch_stats_get(vr_batch* b, vr_render_stats* out) {
    if (!b || !out) return fail(VR_ERR_INVALID, "null argument");
    VR_CK(cudaDeviceSynchronize());
    unsigned long long t[3] = {0, 0, 0};
    VR_CK(cudaMemcpy(t, b->totals, sizeof t, cudaMemcpyDeviceToHost));
    *out = b->stats;
    out->paths = t[0];
    out->extend_rays = t[1];
    out->shadow_rays = t[2];
    return VR_OK;
}

// -------------------------------------------------------------- intersect --

vr_status vr_intersect_device(vr_scene* s, const vr_ray* rays, uint64_t n, vr_hit* hits, int32_t any_hit,
                              void* stream) {
    if (!s) return fail(VR_ERR_INVALID, "null scene");
    if (n && (!rays || !hits)) return fail(VR_ERR_INVALID, "null rays/hits");
    if (n == 0) return VR_OK;
    cudaStream_t cs = pick(s, stream);
    if (s->info.num_triangles == 0 && s->view.num_analytic == 0) {
        // empty scene: every ray misses
        VR_CK(cudaMemsetAsync(hits, 0xFF, n * sizeof(vr_hit), cs));
        return VR_OK;
    }
    const uint64_t chunk = 1ull << 30;  // the persistent kernel indexes rays with 32 bits
    // closest-hit batches of at least SORT_MIN rays are traced in sorted order
    // (octant, origin cell): same results, more coherent warps (1M-triangle
    // soup, 16.8M rays: 1033 -> 1072 M rays/s); any-hit rays stop early and
    // do not repay the sort (2266 -> 2232 M rays/s with it)
    constexpr uint64_t SORT_MIN = 1u << 16;
    const bool sort = n >= SORT_MIN && s->view.nodes && !any_hit;
    vr_status r;
    if (sort && (r = ensure_buf(s->sortbuf, (2 * std::min(chunk, n) + vr::RAY_SORT_BINS) * sizeof(uint32_t))) != VR_OK)
        return r;
    for (uint64_t b = 0; b < n; b += chunk) {
        const uint64_t m = std::min(chunk, n - b);
        const float4* rb = reinterpret_cast<const float4*>(rays + b);
        uint32_t* perm = nullptr;
        if (sort && m >= SORT_MIN) {
            uint32_t* keys = static_cast<uint32_t*>(s->sortbuf.p);
            perm = keys + m;
            VR_CK(vr::launch_ray_sort(rb, (uint32_t)m, s->blo, s->bhi, keys, perm + m, perm, cs));
        }
        VR_CK(vr::launch_intersect(s->view, rb, m, reinterpret_cast<float4*>(hits + b), any_hit != 0, s->fetch,
                                   s->status, cs, perm));
    }
    return VR_OK;
}

vr_status vr_intersect(vr_scene* s, const vr_ray* rays, uint64_t n, vr_hit* hits, int32_t any_hit) {
    if (!s) return fail(VR_ERR_INVALID, "null scene");
    if (n == 0) return VR_OK;
    if (!rays || !hits) return fail(VR_ERR_INVALID, "null rays/hits");
    vr_status r;
    if ((r = ensure_buf(s->stage_a, n * sizeof(vr_ray))) != VR_OK) return r;
    if ((r = ensure_buf(s->stage_b, n * sizeof(vr_hit))) != VR_OK) return r;
    VR_CK(cudaMemcpyAsync(s->stage_a.p, rays, n * sizeof(vr_ray), cudaMemcpyHostToDevice, s->stream));
    if ((r = vr_intersect_device(s, static_cast<const vr_ray*>(s->stage_a.p), n, static_cast<vr_hit*>(s->stage_b.p),
                                 any_hit, nullptr)) != VR_OK)
        return r;
    VR_CK(cudaMemcpyAsync(hits, s->stage_b.p, n * sizeof(vr_hit), cudaMemcpyDeviceToHost, s->stream));
    VR_CK(cudaStreamSynchronize(s->stream));
    return check_status(s);
}

vr_status vr_environment_sample(vr_scene* s, const float* dirs, uint64_t n, float* rgb) {
    if (!s) return fail(VR_ERR_INVALID, "null scene");
    if (n == 0) return VR_OK;
    if (!dirs || !rgb) return fail(VR_ERR_INVALID, "null directions/rgb");
    vr_status r;
    const size_t bytes = n * 3 * sizeof(float);
    if ((r = ensure_buf(s->stage_a, bytes)) != VR_OK) return r;
    if ((r = ensure_buf(s->stage_b, bytes)) != VR_OK) return r;
    VR_CK(cudaMemcpyAsync(s->stage_a.p, dirs, bytes, cudaMemcpyHostToDevice, s->stream));
    VR_CK(vr::launch_env_sample(s->view, static_cast<const float*>(s->stage_a.p), n, static_cast<float*>(s->stage_b.p),
                                s->stream));
    VR_CK(cudaMemcpyAsync(rgb, s->stage_b.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    VR_CK(cudaStreamSynchronize(s->stream));
    return check_status(s);
}

vr_status vr_intersect_count_device(vr_scene* s, const vr_ray* rays, uint64_t n, int32_t any_hit,
                                    uint64_t* node_visits, uint64_t* tri_tests, void* stream) {
    if (!s || !node_visits || !tri_tests) return fail(VR_ERR_INVALID, "null argument");
    *node_visits = 0;
    *tri_tests = 0;
    if (n == 0 || s->info.num_triangles == 0) return VR_OK;
    if (!rays) return fail(VR_ERR_INVALID, "null rays");
    if (n >= (1ull << 31)) return fail(VR_ERR_INVALID, "too many rays for one counting launch");
    cudaStream_t cs = pick(s, stream);
    vr_status r;
    if ((r = ensure_buf(s->stage_b, n * sizeof(vr_hit))) != VR_OK) return r;
    unsigned long long* c = s->totals + 4;
    VR_CK(cudaMemsetAsync(c, 0, 2 * sizeof(unsigned long long), cs));
    VR_CK(vr::launch_intersect_count(s->view, reinterpret_cast<const float4*>(rays), n,
                                     static_cast<float4*>(s->stage_b.p), any_hit != 0, s->fetch, c, s->status, cs));
    unsigned long long hc[2];
    VR_CK(cudaMemcpyAsync(hc, c, sizeof hc, cudaMemcpyDeviceToHost, cs));
    VR_CK(cudaStreamSynchronize(cs));
    *node_visits = hc[0];
    *tri_tests = hc[1];
    return check_status(s);
}

// ---------------------------------------------------------------- colour --

vr_status vr_tonemap_device(const float* in, float* out, uint32_t w, uint32_t h, const vr_color_management* cm,
                            float scale, void* stream) {
    if (!in || !out || !cm) return fail(VR_ERR_INVALID, "null argument");
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    if (cm->tonemap < 0 || cm->tonemap > 4) return fail(VR_ERR_INVALID, "tonemap");
    const float ex = std::pow(2.0f, cm->exposure);
    const float inv_gamma = 1.0f / cm->gamma;
    VR_CK(vr::launch_tonemap(reinterpret_cast<const float4*>(in), reinterpret_cast<float4*>(out), w * h, cm->tonemap,
                             inv_gamma, ex, scale, 0, static_cast<cudaStream_t>(stream)));
    return VR_OK;
}

vr_status vr_tonemap_legacy_device(const float* in, float* out, uint32_t w, uint32_t h, int32_t tonemap, float gamma,
                                   float exposure, int32_t transparent, float scale, void* stream) {
    if (!in || !out) return fail(VR_ERR_INVALID, "null argument");
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    // legacy numbering (viewport_fragment.glsl:10-17) -> kernel curve codes
    static const int32_t code[8] = {0, 1, 5, 6, 2, 7, 3, 4};
    if (tonemap < 0 || tonemap > 7) return fail(VR_ERR_INVALID, "legacy tonemap");
    if (tonemap == VR_LEGACY_TONEMAP_FILMIC) gamma = 1.0f;  // "Filmic doesn't have gamma"
    VR_CK(vr::launch_tonemap(reinterpret_cast<const float4*>(in), reinterpret_cast<float4*>(out), w * h,
                             code[tonemap], 1.0f / gamma, exposure, scale, transparent ? 1 : 0,
                             static_cast<cudaStream_t>(stream)));
    return VR_OK;
}

vr_status vr_tonemap(const float* in, float* out, uint32_t w, uint32_t h, const vr_color_management* cm, float scale) {
    if (!in || !out || !cm) return fail(VR_ERR_INVALID, "null argument");
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    const size_t bytes = (size_t)w * h * 16;
    if (bytes == 0) return VR_OK;
    void *din = nullptr, *dout = nullptr;
    VR_CK(cudaMalloc(&din, bytes));
    if (cudaMalloc(&dout, bytes) != cudaSuccess) {
        cudaFree(din);
        return fail(VR_ERR_OOM, "tonemap buffer");
    }
    vr_status r = VR_OK;
    if (cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice) != cudaSuccess) r = fail(VR_ERR_CUDA, "copy in");
    if (r == VR_OK) r = vr_tonemap_device(static_cast<float*>(din), static_cast<float*>(dout), w, h, cm, scale, nullptr);
    if (r == VR_OK && cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) r = fail(VR_ERR_CUDA, "copy out");
    cudaFree(din);
    cudaFree(dout);
    return r;
}

vr_status vr_tonemap_legacy(const float* in, float* out, uint32_t w, uint32_t h, int32_t tonemap, float gamma,
                            float exposure, int32_t transparent, float scale) {
    if (!in || !out) return fail(VR_ERR_INVALID, "null argument");
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    if (tonemap < 0 || tonemap > 7) return fail(VR_ERR_INVALID, "legacy tonemap");
    const size_t bytes = (size_t)w * h * 16;
    if (bytes == 0) return VR_OK;
    void *din = nullptr, *dout = nullptr;
    VR_CK(cudaMalloc(&din, bytes));
    if (cudaMalloc(&dout, bytes) != cudaSuccess) {
        cudaFree(din);
        return fail(VR_ERR_OOM, "tonemap buffer");
    }
    vr_status r = VR_OK;
    if (cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice) != cudaSuccess) r = fail(VR_ERR_CUDA, "copy in");
    if (r == VR_OK)
        r = vr_tonemap_legacy_device(static_cast<float*>(din), static_cast<float*>(dout), w, h, tonemap, gamma,
                                     exposure, transparent, scale, nullptr);
    if (r == VR_OK && cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) r = fail(VR_ERR_CUDA, "copy out");
    cudaFree(din);
    cudaFree(dout);
    return r;
}

vr_status vr_relmse_device(const float* a, float sa, const float* ref, float sr, uint32_t w, uint32_t h, double* out,
                           void* stream) {
    if (!a || !ref || !out) return fail(VR_ERR_INVALID, "null argument");
    if (!device_ok()) return fail(VR_ERR_NO_DEVICE, "no CUDA device");
    double* d = nullptr;
    VR_CK(cudaMalloc(&d, sizeof(double)));
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    vr_status r = VR_OK;
    if (cudaMemsetAsync(d, 0, sizeof(double), cs) != cudaSuccess) r = fail(VR_ERR_CUDA, "memset");
    if (r == VR_OK && vr::launch_relmse(reinterpret_cast<const float4*>(a), sa, reinterpret_cast<const float4*>(ref),
                                        sr, w * h, d, cs) != cudaSuccess)
        r = fail(VR_ERR_CUDA, "relmse launch");
    double sum = 0.0;
    if (r == VR_OK && cudaMemcpyAsync(&sum, d, sizeof(double), cudaMemcpyDeviceToHost, cs) != cudaSuccess)
        r = fail(VR_ERR_CUDA, "copy");
    if (r == VR_OK && cudaStreamSynchronize(cs) != cudaSuccess) r = fail(VR_ERR_CUDA, "sync");
    cudaFree(d);
    if (r == VR_OK) *out = sum / (3.0 * (double)w * (double)h);
    return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Render without device allocation (no counterpart in the reference).
//
// Callers that cannot call cudaMalloc while they render -- a host application
// that has reserved the GPU's memory for its own pool, a real-time frame loop
// that cannot take cudaFree's device-wide synchronisation or an allocation
// failure mid-frame -- use vr_render_device_noalloc.  Its wavefront scratch
// (ray queues, path state, per-pixel sums) lives in this file-scope device
// array of VR_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library
// holds until the process exits.  The scene itself is still built, and its
// memory allocated, by vr_scene_create beforehand.
// ---------------------------------------------------------------------------
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[VR_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// The array's host-side name is only a stand-in; kernels need its device
// address, looked up once per device with that device current.
vr_status noalloc_scratch(void** out) {
    int dev = 0;
    VR_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(VR_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(VR_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return VR_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

vr_status render_device_noalloc(vr_scene* s, const vr_render_settings* st, uint32_t samples, float* rgba,
                                uint32_t w, uint32_t h, uint64_t seed, uint32_t first_sample, void* stream) {
    vr_status r = validate_render(s, st, w, h);
    if (r != VR_OK) return r;
    if (!rgba) return fail(VR_ERR_INVALID, "rgba is NULL");
    if ((uint64_t)first_sample + samples >= (1ull << 31)) return fail(VR_ERR_INVALID, "sample index out of range");
    const uint32_t np = w * h;
    if (samples == 0) {
        VR_CK(vr::launch_empty_pass(reinterpret_cast<float4*>(rgba), np, pick(s, stream)));
        return VR_OK;
    }
    const uint64_t total = (uint64_t)samples * np;
    const bool need_att = st->estimator == VR_EST_REFERENCE;
    // fixed layout: pixel sums, counters, wave table, then the per-path arrays
    const size_t table_entries = 2048;
    const size_t psum_bytes = align256((size_t)np * sizeof(float4));
    const size_t counts_bytes = align256((size_t)vr::MAX_JOBS * vr::JOB_COUNTERS * sizeof(uint32_t)) +
                                align256(2 * (size_t)vr::MAX_DEPTH_SLOTS * sizeof(uint32_t));
    const size_t table_bytes = align256(table_entries * sizeof(vr::Job));
    const size_t per_path = 10 * sizeof(float4) + sizeof(uint64_t) + 3 * sizeof(uint32_t) +
                            (need_att ? (size_t)st->max_bounces * 3 * sizeof(float) : 0);
    const size_t fixed = psum_bytes + counts_bytes + table_bytes + 16 * 256;  // 16 arrays rounded up to 256 bytes
    const uint64_t min_paths = 1024;
    if (fixed + min_paths * per_path > (size_t)VR_NOALLOC_SCRATCH_BYTES)
        return fail(VR_ERR_UNSUPPORTED, "image of " + std::to_string(np) + " pixels does not fit the " +
                                            std::to_string(VR_NOALLOC_SCRATCH_BYTES >> 20) +
                                            " MiB no-alloc scratch (16 bytes per pixel plus at least 1024 paths)");
    uint64_t cap = ((size_t)VR_NOALLOC_SCRATCH_BYTES - fixed) / per_path;
    if (st->wavefront_paths && st->wavefront_paths < cap) cap = st->wavefront_paths;
    if (cap > total) cap = total;
    void* base = nullptr;
    if ((r = noalloc_scratch(&base)) != VR_OK) return r;
    unsigned char* p = static_cast<unsigned char*>(base);
    auto carve = [&](size_t bytes) {
        void* q = p;
        p += align256(bytes);
        return q;
    };
    float4* psum = static_cast<float4*>(carve((size_t)np * sizeof(float4)));
    vr::PathState ps{};
    ps.counts = static_cast<uint32_t*>(carve((size_t)vr::MAX_JOBS * vr::JOB_COUNTERS * sizeof(uint32_t)));
    ps.cursors = static_cast<uint32_t*>(carve(2 * (size_t)vr::MAX_DEPTH_SLOTS * sizeof(uint32_t)));
    vr::Job* table = static_cast<vr::Job*>(carve(table_entries * sizeof(vr::Job)));
    ps.q_org = static_cast<float4*>(carve(2 * cap * sizeof(float4)));
    ps.q_dir = static_cast<float4*>(carve(2 * cap * sizeof(float4)));
    ps.hits = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.thr = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.rad = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.s_org = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.s_dir = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.s_contrib = static_cast<float4*>(carve(cap * sizeof(float4)));
    ps.rng = static_cast<uint64_t*>(carve(cap * sizeof(uint64_t)));
    ps.q_path = static_cast<uint32_t*>(carve(2 * cap * sizeof(uint32_t)));
    ps.s_path = static_cast<uint32_t*>(carve(cap * sizeof(uint32_t)));
    ps.att = need_att ? static_cast<float*>(carve((size_t)st->max_bounces * 3 * cap * sizeof(float))) : nullptr;
    if ((size_t)(p - static_cast<unsigned char*>(base)) > (size_t)VR_NOALLOC_SCRATCH_BYTES)
        return fail(VR_ERR_INVALID, "no-alloc scratch layout overflow");
    ps.cap = (uint32_t)cap;
    cudaStream_t cs = pick(s, stream);
    // the array keeps the previous call's contents: the pixel sums must start
    // at zero (queue counters are cleared at the start of every wavefront)
    VR_CK(cudaMemsetAsync(psum, 0, (size_t)np * sizeof(float4), cs));
    std::vector<HostJob> jobs{make_job(s->view, st, samples, rgba, w, h, seed, first_sample, psum)};
    return run_waves(jobs, ps, (uint32_t)cap, table, table_entries, s->status, s->totals, nullptr, cs, nullptr);
}

}  // namespace

extern "C" {

// The planner's host vectors and the error strings may throw; nothing crosses
// the C ABI as an exception.
vr_status vr_render_device_noalloc(vr_scene* s, const vr_render_settings* st, uint32_t samples, float* rgba,
                                   uint32_t w, uint32_t h, uint64_t seed, uint32_t first_sample, void* stream) {
    try {
        return render_device_noalloc(s, st, samples, rgba, w, h, seed, first_sample, stream);
    } catch (const std::bad_alloc&) {
        return fail(VR_ERR_OOM, "host allocation failed in vr_render_device_noalloc");
    } catch (const std::exception& e) {
        return fail(VR_ERR_INVALID, std::string("vr_render_device_noalloc: ") + e.what());
    }
}

}  // extern "C"
