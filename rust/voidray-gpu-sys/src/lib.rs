//! Raw bindings of libvoidray_gb300, the GB300 (sm_103a) wavefront path
//! tracer that replaces voidray_renderer's CPU integrator.  Every item here is
//! a field-for-field, argument-for-argument restatement of the C headers in
//! the repository's `include/` directory (`voidray_gpu.h`, `voidray_denoise.h`,
//! `voidray_assets.h`); `tests/test_rust_sys.py` checks that they agree.
//!
//! The reference call sites these entry points replace:
//! - `Scene::build_acceleration` (voidray_renderer/src/core/scene.rs:163-178)
//!   -> `vr_scene_create`;
//! - `iterative_render(target, &accel, &settings, samples)`
//!   (voidray_renderer/src/render/iterative.rs:11-16, called from
//!   render/renderer.rs:67,87) -> `vr_render`;
//! - `SceneAcceleration::hit` (core/scene.rs:182-185) -> `vr_intersect`;
//! - `Environment::sample` (core/traits.rs:66-69) -> `vr_environment_sample`;
//! - `PostProcessingPass::render` / post_process.glsl
//!   (render/post_process.rs:43-86) -> `vr_tonemap`.
//! Everything else (batches, the denoiser, the asset decoders) has no
//! reference counterpart.
//!
//! Every function returns a `vr_status` (0 = `VR_OK`); `vr_last_error` gives
//! the message of the calling thread's last failure.  Nothing panics or
//! aborts across this boundary.
#![allow(non_camel_case_types)]
#![no_std]

use core::ffi::{c_char, c_void};

/// `vr_status` and the other C enums travel as `int32_t`.
pub type vr_status = i32;
pub type vr_material_kind = i32;
pub type vr_env_kind = i32;
pub type vr_texture_sampling = i32;
pub type vr_analytic_kind = i32;
pub type vr_render_mode = i32;
pub type vr_estimator = i32;
pub type vr_legacy_tonemap = i32;
pub type vr_image_format = i32;

pub const VR_ABI_VERSION: i32 = 4;

pub const VR_OK: vr_status = 0;
pub const VR_ERR_INVALID: vr_status = 1;
pub const VR_ERR_UNSUPPORTED: vr_status = 2;
pub const VR_ERR_CUDA: vr_status = 3;
pub const VR_ERR_OOM: vr_status = 4;
pub const VR_ERR_STACK: vr_status = 5;
pub const VR_ERR_TIMEOUT: vr_status = 6;
pub const VR_ERR_NO_DEVICE: vr_status = 7;
pub const VR_ERR_CANCELLED: vr_status = 8;

/// Materials::* of voidray_common/src/simple.rs:15-58 and MicrofacetBSDF
/// (voidray_common/src/microfacet.rs:9-101); kind 6 is the legacy crate's
/// MixMaterial (voidray/src/common/materials.rs:188-203).
pub const VR_MAT_LAMBERTIAN: vr_material_kind = 0;
pub const VR_MAT_METAL: vr_material_kind = 1;
pub const VR_MAT_DIELECTRIC: vr_material_kind = 2;
pub const VR_MAT_EMISSION: vr_material_kind = 3;
pub const VR_MAT_LAMBERTIAN_BSDF: vr_material_kind = 4;
pub const VR_MAT_MICROFACET: vr_material_kind = 5;
pub const VR_MAT_MIX: vr_material_kind = 6;
pub const VR_MAX_MIX_DEPTH: u32 = 8;

/// Environments::{uniform, hdri} (voidray_common/src/environments.rs:9-17).
pub const VR_ENV_NONE: vr_env_kind = 0;
pub const VR_ENV_UNIFORM: vr_env_kind = 1;
pub const VR_ENV_HDRI: vr_env_kind = 2;

/// ImageTexture sampling (voidray_renderer/src/core/texture.rs:82-98).
pub const VR_TEX_NEAREST: vr_texture_sampling = 0;
pub const VR_TEX_BILINEAR: vr_texture_sampling = 1;

/// Surfaces::{sphere, ground_plane} (voidray_common/src/surfaces.rs:31-113).
pub const VR_ANALYTIC_SPHERE: vr_analytic_kind = 1;
pub const VR_ANALYTIC_GROUND_PLANE: vr_analytic_kind = 2;
pub const VR_MAX_ANALYTICS: u32 = 64;

/// RenderMode (voidray_renderer/src/core/settings.rs:3-7); the estimator has
/// no reference counterpart (the reference's recursion is VR_EST_REFERENCE).
pub const VR_MODE_NORMAL: vr_render_mode = 0;
pub const VR_MODE_FULL: vr_render_mode = 1;
pub const VR_EST_REFERENCE: vr_estimator = 0;
pub const VR_EST_NEE: vr_estimator = 1;

/// The legacy crate's viewport tonemaps (voidray/src/shaders/viewport_fragment.glsl:27-67).
pub const VR_LEGACY_TONEMAP_NONE: vr_legacy_tonemap = 0;
pub const VR_LEGACY_TONEMAP_SIMPLE_ACES: vr_legacy_tonemap = 1;
pub const VR_LEGACY_TONEMAP_SIMPLE_REINHARD: vr_legacy_tonemap = 2;
pub const VR_LEGACY_TONEMAP_LUMA_REINHARD: vr_legacy_tonemap = 3;
pub const VR_LEGACY_TONEMAP_LUMA_WHITEPRESERVING_REINHARD: vr_legacy_tonemap = 4;
pub const VR_LEGACY_TONEMAP_ROM_BIN_DA_HOUSE: vr_legacy_tonemap = 5;
pub const VR_LEGACY_TONEMAP_FILMIC: vr_legacy_tonemap = 6;
pub const VR_LEGACY_TONEMAP_UNCHARTED_2: vr_legacy_tonemap = 7;

pub const VR_MISS: u32 = 0xFFFF_FFFF;
pub const VR_NOALLOC_SCRATCH_BYTES: u64 = 64 << 20;
pub const VR_STATS_TILE: u32 = 16;
pub const VR_STATS_MAX_JOBS: u32 = 128;
pub const VR_INSTR_STAGE_TIMES: u32 = 1;
pub const VR_INSTR_WORK: u32 = 2;
pub const VR_STAGE_RAYGEN: u32 = 0;
pub const VR_STAGE_EXTEND: u32 = 1;
pub const VR_STAGE_SHADE: u32 = 2;
pub const VR_STAGE_SHADOW: u32 = 3;
pub const VR_STAGE_ACCUMULATE: u32 = 4;
pub const VR_NUM_STAGES: u32 = 5;
pub const VR_DN_LOSS_L1_LOG: i32 = 0;
pub const VR_DN_LOSS_RELMSE: i32 = 1;
pub const VR_DN_BACKEND_MMA_SYNC: i32 = 0;
pub const VR_DN_BACKEND_TCGEN05: i32 = 1;
pub const VR_IMAGE_UNKNOWN: vr_image_format = 0;
pub const VR_IMAGE_JPEG: vr_image_format = 1;

/// Opaque handles: a built scene (device BVH, shading records, environment),
/// a batch (shared wavefront scratch), a denoiser (weights and workspaces).
#[repr(C)]
pub struct vr_scene {
    _p: [u8; 0],
}
#[repr(C)]
pub struct vr_batch {
    _p: [u8; 0],
}
#[repr(C)]
pub struct vr_denoiser {
    _p: [u8; 0],
}

// ------------------------------------------------------------ scene lowering
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_material {
    pub kind: i32,
    pub color: [f32; 3],
    pub fuzz: f32,
    pub ir: f32,
    pub roughness: f32,
    pub metallic: f32,
    pub emittance: f32,
    pub transparent: i32,
    pub albedo_texture: i32,
    pub normal_texture: i32,
    pub mix_first: i32,
    pub mix_second: i32,
    pub mix_factor: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_mesh_desc {
    pub positions: *const f32,
    pub normals: *const f32,
    pub uvs: *const f32,
    pub indices: *const u32,
    pub num_vertices: u32,
    pub num_triangles: u32,
    pub material: u32,
    pub pad_: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_environment_desc {
    pub kind: i32,
    pub color: [f32; 3],
    pub image: *const f32,
    pub width: u32,
    pub height: u32,
    pub importance_sample: i32,
    pub pad_: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_camera_desc {
    pub eye: [f32; 3],
    pub direction: [f32; 3],
    pub up: [f32; 3],
    pub fov: f32,
    pub has_dof: i32,
    pub aperture: f32,
    pub focal_point: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_texture_desc {
    pub image: *const f32,
    pub width: u32,
    pub height: u32,
    pub sampling: i32,
    pub pad_: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_analytic_desc {
    pub kind: i32,
    pub center: [f32; 3],
    pub radius: f32,
    pub height: f32,
    pub material: u32,
    pub pad_: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_scene_desc {
    pub meshes: *const vr_mesh_desc,
    pub num_meshes: u32,
    pub num_materials: u32,
    pub materials: *const vr_material,
    pub environment: vr_environment_desc,
    pub camera: vr_camera_desc,
    pub bvh_max_leaf: u32,
    pub bvh_bins: u32,
    pub analytics: *const vr_analytic_desc,
    pub num_analytics: u32,
    pub num_textures: u32,
    pub textures: *const vr_texture_desc,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_scene_info {
    pub num_triangles: u64,
    pub num_nodes: u64,
    pub device_bytes: u64,
    pub max_depth: u32,
    pub max_leaf: u32,
    pub sah_cost: f64,
    pub build_ms: f64,
}

// ------------------------------------------------------------------- render
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_render_settings {
    pub total_samples: u32,
    pub update_frequency: f32,
    pub render_mode: i32,
    pub firefly_clamp: f32,
    pub max_bounces: u32,
    pub estimator: i32,
    pub rr_depth: u32,
    pub wavefront_paths: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_color_management {
    pub tonemap: i32,
    pub gamma: f32,
    pub exposure: f32,
    pub transparent: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_render_job {
    pub scene: *mut vr_scene,
    pub settings: vr_render_settings,
    pub samples: u32,
    pub width: u32,
    pub height: u32,
    pub first_sample: u32,
    pub seed: u64,
    pub rgba_device: *mut f32,
    pub albedo_device: *mut f32,
    pub normal_device: *mut f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_tuning {
    pub shade_block: u32,
    pub shade_blocks_per_sm: u32,
    pub raygen_block: u32,
    pub generation: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_stats_job {
    pub sum_a: *const f32,
    pub sum_b: *const f32,
    pub den_a: *const f32,
    pub den_b: *const f32,
    pub n_a: u32,
    pub n_b: u32,
    pub width: u32,
    pub height: u32,
    pub tile_offset: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_render_stats {
    pub paths: u64,
    pub extend_rays: u64,
    pub shadow_rays: u64,
    pub wavefronts: u64,
    pub ms: f64,
    pub error_flags: u32,
    pub pad_: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_instrument {
    pub stage_ms: [f64; 8],
    pub stage_launches: [u64; 8],
    pub extend_node_visits: u64,
    pub extend_tri_tests: u64,
    pub shadow_node_visits: u64,
    pub shadow_tri_tests: u64,
    pub retired_paths: u64,
    pub metal_fallbacks: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_ray {
    pub org: [f32; 3],
    pub tmin: f32,
    pub dir: [f32; 3],
    pub tmax: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_hit {
    pub prim: u32,
    pub t: f32,
    pub u: f32,
    pub v: f32,
}

// ---------------------------------------------------- denoiser and assets
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_denoiser_info {
    pub param_count: u64,
    pub steps: u64,
    pub workspace_bytes: u64,
    pub flops_per_pixel: f64,
    pub num_layers: u32,
    pub input_channels: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_denoiser_layer {
    pub c1: u32,
    pub c2: u32,
    pub up1: u32,
    pub cout: u32,
    pub relu: u32,
    pub level: u32,
    pub w_offset: u64,
    pub b_offset: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_image_info {
    pub width: u32,
    pub height: u32,
    pub components: u32,
    pub format: u32,
    pub progressive: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct vr_obj_mesh {
    pub positions: *mut f32,
    pub uvs: *mut f32,
    pub normals: *mut f32,
    pub indices: *mut u32,
    pub num_vertices: u32,
    pub num_triangles: u32,
}

#[link(name = "voidray_gb300")]
extern "C" {
    // Scene::build_acceleration (core/scene.rs:163-178) and its inputs
    pub fn vr_scene_create(desc: *const vr_scene_desc, out: *mut *mut vr_scene) -> vr_status;
    pub fn vr_scene_destroy(scene: *mut vr_scene) -> vr_status;
    pub fn vr_scene_info_get(scene: *const vr_scene, info: *mut vr_scene_info) -> vr_status;
    pub fn vr_scene_validate(desc: *const vr_scene_desc, info: *mut vr_scene_info) -> vr_status;
    pub fn vr_scene_set_camera(scene: *mut vr_scene, camera: *const vr_camera_desc) -> vr_status;
    pub fn vr_scene_synchronize(scene: *mut vr_scene) -> vr_status;
    // iterative_render (render/iterative.rs:11-55): rgba += sum of samples / total_samples
    pub fn vr_render(
        scene: *mut vr_scene,
        settings: *const vr_render_settings,
        samples: u32,
        rgba: *mut f32,
        width: u32,
        height: u32,
        seed: u64,
        first_sample: u32,
    ) -> vr_status;
    pub fn vr_render_device(
        scene: *mut vr_scene,
        settings: *const vr_render_settings,
        samples: u32,
        rgba_device: *mut f32,
        width: u32,
        height: u32,
        seed: u64,
        first_sample: u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_render_aov_device(
        scene: *mut vr_scene,
        settings: *const vr_render_settings,
        samples: u32,
        rgba_device: *mut f32,
        albedo_device: *mut f32,
        normal_device: *mut f32,
        width: u32,
        height: u32,
        seed: u64,
        first_sample: u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_render_device_noalloc(
        scene: *mut vr_scene,
        settings: *const vr_render_settings,
        samples: u32,
        rgba_device: *mut f32,
        width: u32,
        height: u32,
        seed: u64,
        first_sample: u32,
        stream: *mut c_void,
    ) -> vr_status;
    // Many jobs per wavefront, launch shapes, serving statistics (no reference counterpart)
    pub fn vr_batch_create(max_wave_paths: u64, out: *mut *mut vr_batch) -> vr_status;
    pub fn vr_batch_destroy(batch: *mut vr_batch) -> vr_status;
    pub fn vr_batch_render(
        batch: *mut vr_batch,
        jobs: *const vr_render_job,
        count: u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_batch_synchronize(batch: *mut vr_batch, stream: *mut c_void) -> vr_status;
    pub fn vr_batch_set_graphs(batch: *mut vr_batch, enable: i32) -> vr_status;
    pub fn vr_batch_graph_stats(
        batch: *mut vr_batch,
        captures: *mut u64,
        replays: *mut u64,
    ) -> vr_status;
    pub fn vr_batch_stats_get(batch: *mut vr_batch, stats: *mut vr_render_stats) -> vr_status;
    pub fn vr_tuning_get(tuning: *mut vr_tuning) -> vr_status;
    pub fn vr_tuning_set(tuning: *const vr_tuning) -> vr_status;
    pub fn vr_serve_stats_device(
        jobs: *const vr_stats_job,
        count: u32,
        out_device: *mut f64,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_serve_sum_device(
        a: *const *const f32,
        b: *const *const f32,
        out: *const *mut f32,
        pairs: u32,
        pixels: u64,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_serve_blend_device(
        sum_a: *const f32,
        sum_b: *const f32,
        samples: u32,
        denoised: *const f32,
        alpha_tiles: *const f32,
        width: u32,
        height: u32,
        rgb: *mut f32,
        stream: *mut c_void,
    ) -> vr_status;
    // Statistics and instrumentation
    pub fn vr_render_stats_get(scene: *const vr_scene, stats: *mut vr_render_stats) -> vr_status;
    pub fn vr_scene_instrument(scene: *mut vr_scene, flags: u32) -> vr_status;
    pub fn vr_scene_instrument_get(scene: *mut vr_scene, out: *mut vr_instrument) -> vr_status;
    pub fn vr_relmse_device(
        rgba_device: *const f32,
        scale: f32,
        ref_rgba_device: *const f32,
        ref_scale: f32,
        width: u32,
        height: u32,
        out: *mut f64,
        stream: *mut c_void,
    ) -> vr_status;
    // post_process.glsl / tonemapping.glsl (render/post_process.rs:43-86) and the legacy viewport shader
    pub fn vr_tonemap(
        rgba_in: *const f32,
        rgba_out: *mut f32,
        width: u32,
        height: u32,
        cm: *const vr_color_management,
        scale: f32,
    ) -> vr_status;
    pub fn vr_tonemap_device(
        rgba_in_device: *const f32,
        rgba_out_device: *mut f32,
        width: u32,
        height: u32,
        cm: *const vr_color_management,
        scale: f32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_tonemap_legacy(
        rgba_in: *const f32,
        rgba_out: *mut f32,
        width: u32,
        height: u32,
        tonemap: i32,
        gamma: f32,
        exposure: f32,
        transparent: i32,
        scale: f32,
    ) -> vr_status;
    pub fn vr_tonemap_legacy_device(
        rgba_in_device: *const f32,
        rgba_out_device: *mut f32,
        width: u32,
        height: u32,
        tonemap: i32,
        gamma: f32,
        exposure: f32,
        transparent: i32,
        scale: f32,
        stream: *mut c_void,
    ) -> vr_status;
    // SceneAcceleration::hit (core/scene.rs:182-185) and Environment::sample (core/traits.rs:66-69) over batches
    pub fn vr_intersect(
        scene: *mut vr_scene,
        rays: *const vr_ray,
        count: u64,
        hits: *mut vr_hit,
        any_hit: i32,
    ) -> vr_status;
    pub fn vr_intersect_device(
        scene: *mut vr_scene,
        rays_device: *const vr_ray,
        count: u64,
        hits_device: *mut vr_hit,
        any_hit: i32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_intersect_count_device(
        scene: *mut vr_scene,
        rays_device: *const vr_ray,
        count: u64,
        any_hit: i32,
        node_visits: *mut u64,
        tri_tests: *mut u64,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_environment_sample(
        scene: *mut vr_scene,
        directions: *const f32,
        count: u64,
        rgb: *mut f32,
    ) -> vr_status;
    // Errors and the library
    pub fn vr_last_error() -> *const c_char;
    pub fn vr_abi_version() -> i32;
    pub fn vr_device_available() -> i32;
    // The learned denoiser (voidray_denoise.h; no reference counterpart)
    pub fn vr_denoiser_create(seed: u64, out: *mut *mut vr_denoiser) -> vr_status;
    pub fn vr_denoiser_destroy(net: *mut vr_denoiser) -> vr_status;
    pub fn vr_denoiser_info_get(net: *const vr_denoiser, info: *mut vr_denoiser_info) -> vr_status;
    pub fn vr_denoiser_layer_get(index: u32, layer: *mut vr_denoiser_layer) -> vr_status;
    pub fn vr_denoiser_set_loss(net: *mut vr_denoiser, kind: i32) -> vr_status;
    pub fn vr_denoiser_set_backend(net: *mut vr_denoiser, backend: i32) -> vr_status;
    pub fn vr_denoiser_status(net: *mut vr_denoiser, flags: *mut u32) -> vr_status;
    pub fn vr_denoiser_get_params(net: *mut vr_denoiser, host: *mut f32, count: u64) -> vr_status;
    pub fn vr_denoiser_set_params(net: *mut vr_denoiser, host: *const f32, count: u64) -> vr_status;
    pub fn vr_denoise_device(
        net: *mut vr_denoiser,
        rgba: *const f32,
        albedo: *const f32,
        normal: *const f32,
        scale: f32,
        out_rgba: *mut f32,
        width: u32,
        height: u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_denoise_batch_device(
        net: *mut vr_denoiser,
        rgba: *const f32,
        albedo: *const f32,
        normal: *const f32,
        scales: *const f32,
        out_rgba: *mut f32,
        batch: u32,
        width: u32,
        height: u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_denoiser_gradients_device(
        net: *mut vr_denoiser,
        rgba: *const f32,
        albedo: *const f32,
        normal: *const f32,
        target: *const f32,
        scale_in: f32,
        scale_target: f32,
        batch: u32,
        width: u32,
        height: u32,
        loss_host: *mut f32,
        grads_host: *mut f32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_denoiser_train_step_device(
        net: *mut vr_denoiser,
        rgba: *const f32,
        albedo: *const f32,
        normal: *const f32,
        target: *const f32,
        scale_in: f32,
        scale_target: f32,
        batch: u32,
        width: u32,
        height: u32,
        lr: f32,
        loss_host: *mut f32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_dn_conv3x3_device(
        src1: *const u16,
        c1: u32,
        up1: i32,
        src2: *const u16,
        c2: u32,
        weight: *const u16,
        bias: *const f32,
        mask: *const u16,
        out_bf16: *mut u16,
        out_f32: *mut f32,
        cout: u32,
        n: u32,
        h: u32,
        w: u32,
        relu: i32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_dn_conv3x3_tc_device(
        src1: *const u16,
        c1: u32,
        src2: *const u16,
        c2: u32,
        weight: *const u16,
        bias: *const f32,
        mask: *const u16,
        out_bf16: *mut u16,
        out_f32: *mut f32,
        cout: u32,
        n: u32,
        h: u32,
        w: u32,
        relu: i32,
        status_device: *mut u32,
        stream: *mut c_void,
    ) -> vr_status;
    pub fn vr_dn_conv3x3_wgrad_device(
        dz: *const u16,
        src1: *const u16,
        c1: u32,
        up1: i32,
        src2: *const u16,
        c2: u32,
        dw: *mut f32,
        cout: u32,
        n: u32,
        h: u32,
        w: u32,
        stream: *mut c_void,
    ) -> vr_status;
    // Host decoders (voidray_assets.h) for hosts without the image / obj-rs crates (core/texture.rs:36-50, core/mesh.rs:46-74)
    pub fn vr_image_info_get(data: *const u8, size: usize, info: *mut vr_image_info) -> vr_status;
    pub fn vr_image_decode_rgb8(
        data: *const u8,
        size: usize,
        rgb: *mut u8,
        capacity: usize,
    ) -> vr_status;
    pub fn vr_png_unfilter(
        data: *const u8,
        size: usize,
        rows: u32,
        stride: u32,
        bpp: u32,
        out: *mut u8,
    ) -> vr_status;
    pub fn vr_tiff_lzw_decode(
        src: *const u8,
        size: usize,
        out: *mut u8,
        capacity: usize,
        length: *mut usize,
    ) -> vr_status;
    pub fn vr_obj_parse(text: *const c_char, size: usize, mesh: *mut vr_obj_mesh) -> vr_status;
    pub fn vr_obj_free(mesh: *mut vr_obj_mesh) -> vr_status;
}
