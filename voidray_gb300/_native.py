"""ctypes binding of ``include/voidray_gpu.h`` and ``include/voidray_denoise.h`` (libvoidray_gb300.so).

The library is the only compute path: if it is missing, importing anything
that renders raises immediately; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libvoidray_gb300.so"

VR_OK = 0
STATUS_NAMES = {
    0: "VR_OK", 1: "VR_ERR_INVALID", 2: "VR_ERR_UNSUPPORTED", 3: "VR_ERR_CUDA", 4: "VR_ERR_OOM",
    5: "VR_ERR_STACK", 6: "VR_ERR_TIMEOUT", 7: "VR_ERR_NO_DEVICE", 8: "VR_ERR_CANCELLED",
}
VR_MISS = 0xFFFFFFFF


class VoidrayError(RuntimeError):
    """A non-OK vr_status with the library's message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class vr_material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("color", C.c_float * 3), ("fuzz", C.c_float), ("ir", C.c_float),
                ("roughness", C.c_float), ("metallic", C.c_float), ("emittance", C.c_float),
                ("transparent", C.c_int32), ("albedo_texture", C.c_int32), ("normal_texture", C.c_int32),
                ("mix_first", C.c_int32), ("mix_second", C.c_int32), ("mix_factor", C.c_float)]


class vr_texture_desc(C.Structure):
    _fields_ = [("image", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("sampling", C.c_int32),
                ("pad_", C.c_int32)]


class vr_mesh_desc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p), ("indices", C.c_void_p),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32), ("material", C.c_uint32),
                ("pad_", C.c_uint32)]


class vr_environment_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("color", C.c_float * 3), ("image", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("importance_sample", C.c_int32), ("pad_", C.c_int32)]


class vr_camera_desc(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("direction", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float),
                ("has_dof", C.c_int32), ("aperture", C.c_float), ("focal_point", C.c_float * 3)]


class vr_analytic_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("center", C.c_float * 3), ("radius", C.c_float), ("height", C.c_float),
                ("material", C.c_uint32), ("pad_", C.c_uint32)]


class vr_scene_desc(C.Structure):
    _fields_ = [("meshes", C.c_void_p), ("num_meshes", C.c_uint32), ("num_materials", C.c_uint32),
                ("materials", C.c_void_p), ("environment", vr_environment_desc), ("camera", vr_camera_desc),
                ("bvh_max_leaf", C.c_uint32), ("bvh_bins", C.c_uint32), ("analytics", C.c_void_p),
                ("num_analytics", C.c_uint32), ("num_textures", C.c_uint32), ("textures", C.c_void_p)]


class vr_scene_info(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("num_nodes", C.c_uint64), ("device_bytes", C.c_uint64),
                ("max_depth", C.c_uint32), ("max_leaf", C.c_uint32), ("sah_cost", C.c_double),
                ("build_ms", C.c_double)]


class vr_render_settings(C.Structure):
    _fields_ = [("total_samples", C.c_uint32), ("update_frequency", C.c_float), ("render_mode", C.c_int32),
                ("firefly_clamp", C.c_float), ("max_bounces", C.c_uint32), ("estimator", C.c_int32),
                ("rr_depth", C.c_uint32), ("wavefront_paths", C.c_uint32)]


class vr_render_job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("settings", vr_render_settings), ("samples", C.c_uint32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("first_sample", C.c_uint32), ("seed", C.c_uint64),
                ("rgba_device", C.c_void_p), ("albedo_device", C.c_void_p), ("normal_device", C.c_void_p)]


class vr_color_management(C.Structure):
    _fields_ = [("tonemap", C.c_int32), ("gamma", C.c_float), ("exposure", C.c_float), ("transparent", C.c_int32)]


class vr_render_stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("wavefronts", C.c_uint64), ("ms", C.c_double), ("error_flags", C.c_uint32), ("pad_", C.c_uint32)]


class vr_denoiser_info(C.Structure):
    _fields_ = [("param_count", C.c_uint64), ("steps", C.c_uint64), ("workspace_bytes", C.c_uint64),
                ("flops_per_pixel", C.c_double), ("num_layers", C.c_uint32), ("input_channels", C.c_uint32)]


class vr_denoiser_layer(C.Structure):
    _fields_ = [("c1", C.c_uint32), ("c2", C.c_uint32), ("up1", C.c_uint32), ("cout", C.c_uint32),
                ("relu", C.c_uint32), ("level", C.c_uint32), ("w_offset", C.c_uint64), ("b_offset", C.c_uint64)]


class vr_stats_job(C.Structure):
    _fields_ = [("sum_a", C.c_void_p), ("sum_b", C.c_void_p), ("den_a", C.c_void_p), ("den_b", C.c_void_p),
                ("n_a", C.c_uint32), ("n_b", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("tile_offset", C.c_uint64)]


class vr_image_info(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("components", C.c_uint32), ("format", C.c_uint32),
                ("progressive", C.c_uint32), ("reserved", C.c_uint32)]


class vr_obj_mesh(C.Structure):
    _fields_ = [("positions", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_uint32)),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32)]


STATS_TILE = 16
STATS_MAX_JOBS = 128


class vr_tuning(C.Structure):
    _fields_ = [("shade_block", C.c_uint32), ("shade_blocks_per_sm", C.c_uint32), ("raygen_block", C.c_uint32),
                ("generation", C.c_uint32)]


class vr_instrument(C.Structure):
    _fields_ = [("stage_ms", C.c_double * 8), ("stage_launches", C.c_uint64 * 8),
                ("extend_node_visits", C.c_uint64), ("extend_tri_tests", C.c_uint64),
                ("shadow_node_visits", C.c_uint64), ("shadow_tri_tests", C.c_uint64), ("retired_paths", C.c_uint64),
                ("metal_fallbacks", C.c_uint64)]


STAGES = ["raygen", "extend", "shade", "shadow", "accumulate"]
INSTR_STAGE_TIMES = 1
INSTR_WORK = 2

# every function declared in include/*.h: (name, restype, argtypes)
P = C.c_void_p
_SIGS = [
    ("vr_scene_create", C.c_int, [P, P]),
    ("vr_scene_destroy", C.c_int, [P]),
    ("vr_scene_info_get", C.c_int, [P, P]),
    ("vr_scene_validate", C.c_int, [P, P]),
    ("vr_scene_set_camera", C.c_int, [P, P]),
    ("vr_render", C.c_int, [P, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32]),
    ("vr_render_device", C.c_int, [P, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, P]),
    ("vr_render_aov_device", C.c_int,
     [P, P, C.c_uint32, P, P, P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, P]),
    ("vr_render_stats_get", C.c_int, [P, P]),
    ("vr_tonemap", C.c_int, [P, P, C.c_uint32, C.c_uint32, P, C.c_float]),
    ("vr_tonemap_device", C.c_int, [P, P, C.c_uint32, C.c_uint32, P, C.c_float, P]),
    ("vr_tonemap_legacy", C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_int32, C.c_float, C.c_float, C.c_int32,
                                    C.c_float]),
    ("vr_tonemap_legacy_device", C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_int32, C.c_float, C.c_float,
                                           C.c_int32, C.c_float, P]),
    ("vr_relmse_device", C.c_int, [P, C.c_float, P, C.c_float, C.c_uint32, C.c_uint32, P, P]),
    ("vr_intersect", C.c_int, [P, P, C.c_uint64, P, C.c_int32]),
    ("vr_intersect_device", C.c_int, [P, P, C.c_uint64, P, C.c_int32, P]),
    ("vr_intersect_count_device", C.c_int, [P, P, C.c_uint64, C.c_int32, P, P, P]),
    ("vr_environment_sample", C.c_int, [P, P, C.c_uint64, P]),
    ("vr_last_error", C.c_char_p, []),
    ("vr_abi_version", C.c_int32, []),
    ("vr_device_available", C.c_int32, []),
    ("vr_scene_synchronize", C.c_int, [P]),
    ("vr_render_device_noalloc", C.c_int, [P, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, P]),
    ("vr_batch_create", C.c_int, [C.c_uint64, P]),
    ("vr_batch_destroy", C.c_int, [P]),
    ("vr_batch_render", C.c_int, [P, P, C.c_uint32, P]),
    ("vr_batch_synchronize", C.c_int, [P, P]),
    ("vr_tuning_get", C.c_int, [P]),
    ("vr_tuning_set", C.c_int, [P]),
    ("vr_batch_set_graphs", C.c_int, [P, C.c_int32]),
    ("vr_batch_graph_stats", C.c_int, [P, P, P]),
    ("vr_serve_stats_device", C.c_int, [P, C.c_uint32, P, P]),
    ("vr_serve_sum_device", C.c_int, [P, P, P, C.c_uint32, C.c_uint64, P]),
    ("vr_serve_blend_device", C.c_int, [P, P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, P, P]),
    ("vr_batch_stats_get", C.c_int, [P, P]),
    ("vr_scene_instrument", C.c_int, [P, C.c_uint32]),
    ("vr_scene_instrument_get", C.c_int, [P, P]),
    # include/voidray_denoise.h
    ("vr_denoiser_create", C.c_int, [C.c_uint64, P]),
    ("vr_denoiser_destroy", C.c_int, [P]),
    ("vr_denoiser_info_get", C.c_int, [P, P]),
    ("vr_denoiser_layer_get", C.c_int, [C.c_uint32, P]),
    ("vr_denoiser_set_loss", C.c_int, [P, C.c_int32]),
    ("vr_denoiser_set_backend", C.c_int, [P, C.c_int32]),
    ("vr_denoiser_status", C.c_int, [P, P]),
    ("vr_dn_conv3x3_tc_device", C.c_int,
     [P, C.c_uint32, P, C.c_uint32, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, P, P]),
    ("vr_denoiser_get_params", C.c_int, [P, P, C.c_uint64]),
    ("vr_denoiser_set_params", C.c_int, [P, P, C.c_uint64]),
    ("vr_denoise_device", C.c_int, [P, P, P, P, C.c_float, P, C.c_uint32, C.c_uint32, P]),
    ("vr_denoise_batch_device", C.c_int, [P, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P]),
    ("vr_denoiser_gradients_device", C.c_int,
     [P, P, P, P, P, C.c_float, C.c_float, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P]),
    ("vr_denoiser_train_step_device", C.c_int,
     [P, P, P, P, P, C.c_float, C.c_float, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, P, P]),
    ("vr_dn_conv3x3_device", C.c_int,
     [P, C.c_uint32, C.c_int32, P, C.c_uint32, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
      C.c_int32, P]),
    ("vr_dn_conv3x3_wgrad_device", C.c_int,
     [P, P, C.c_uint32, C.c_int32, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P]),
    # include/voidray_assets.h
    ("vr_image_info_get", C.c_int, [P, C.c_size_t, P]),
    ("vr_image_decode_rgb8", C.c_int, [P, C.c_size_t, P, C.c_size_t]),
    ("vr_png_unfilter", C.c_int, [P, C.c_size_t, C.c_uint32, C.c_uint32, C.c_uint32, P]),
    ("vr_tiff_lzw_decode", C.c_int, [P, C.c_size_t, P, C.c_size_t, P]),
    ("vr_obj_parse", C.c_int, [P, C.c_size_t, P]),
    ("vr_obj_free", C.c_int, [P]),
]
EXPORTED = [name for name, _, _ in _SIGS]

_lib = None


def lib() -> C.CDLL:
    """Loads the native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("VOIDRAY_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise VoidrayError(7, f"native library {path} is missing; build it with "
                                  "`python -m voidray_gb300.build`")
        dll = C.CDLL(str(path))
        for name, res, args in _SIGS:
            fn = getattr(dll, name)
            fn.restype = res
            fn.argtypes = args
        _lib = dll
    return _lib


def check(status: int) -> None:
    if status != VR_OK:
        msg = lib().vr_last_error()
        raise VoidrayError(status, msg.decode("utf-8", "replace") if msg else "")


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
