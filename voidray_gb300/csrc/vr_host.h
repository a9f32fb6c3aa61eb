// vr_host.h — host-side scene lowering shared by the C-ABI implementation.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/voidray_gpu.h"
#include "vr_device.cuh"

namespace vr {

// Sets the thread-local message vr_last_error() returns; returns s.
vr_status set_error(vr_status s, const std::string& message);
// True when a CUDA device is usable (clears the error a failed probe leaves).
bool device_usable();

// Environment importance-sampling tables (no reference counterpart).
struct EnvTables {
    uint32_t W = 0, H = 0;
    std::vector<float> marginal;     // H+1
    std::vector<float> conditional;  // H*(W+1)
    std::vector<float> cell;         // H*W, probability of each cell
    // guide tables of the inverse-CDF search: for u in [k/M, (k+1)/M) the
    // searched index lies in [guide[k], guide[k+1]] (M a power of two)
    uint32_t gm = 0, gc = 0;                // M of the marginal / of every conditional row
    std::vector<uint32_t> guide_marginal;   // gm + 1
    std::vector<uint32_t> guide_conditional;  // H * (gc + 1)
};

// Everything vr_scene_create uploads, laid out as the kernels read it.
struct HostScene {
    std::vector<float4> nodes;  // 4 per BVH2 node (the SAH build; collapsed into `wide`, not uploaded)
    std::vector<float4> wide;   // 8 per 4-wide node: the tree the kernels traverse
    uint32_t wide_depth = 0;
    std::vector<float4> tris;   // 3 per triangle, leaf order
    std::vector<float4> shade;  // 4 per prim, global id order
    std::vector<float2> uvs;    // 3 per prim, empty if no mesh has uvs
    std::vector<Material> materials;
    std::vector<float4> analytic;  // 2 per analytic surface
    std::vector<int4> tex_info;    // per texture: texel offset, width, height, sampling
    std::vector<float> texels;
    std::vector<float> env_img;
    EnvTables tables;
    bool has_tables = false;
    SceneView view{};           // host copy; device pointers filled on upload
    uint64_t num_prims = 0;
    uint32_t max_depth = 0, max_leaf = 0;
    double sah_cost = 0.0;
    double build_ms = 0.0;
};

// Lowers the descriptor and builds the binned-SAH BVH.  Returns VR_OK or an
// error with a message in `err`.
vr_status build_host_scene(const vr_scene_desc* desc, HostScene& out, std::string& err);

// Structural invariants of the flattened BVH (host only).
vr_status validate_host_scene(const HostScene& hs, std::string& err);

// CameraAcceleration (camera.rs:38-53) into the view.
void set_camera(SceneView& view, const vr_camera_desc& cam);

// Reference environment lookup on the host (used to build the tables).
V3 env_eval_host(const SceneView& view, const float* img, V3 dir);

}  // namespace vr
