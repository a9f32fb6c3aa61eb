"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker / baseline, never by the product.
Parity unpinned: the reference ships no golden vectors for this path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    src = [HERE / "voidray_oracle.cpp", HERE / "voidray_oracle.h", HERE / "Makefile"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in src):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", str(HERE)], check=True)
    return LIB


class orc_mesh(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p), ("indices", C.c_void_p),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32), ("surface", C.c_uint32),
                ("pad_", C.c_uint32)]


class orc_analytic(C.Structure):
    _fields_ = [("kind", C.c_int32), ("center", C.c_float * 3), ("radius", C.c_float), ("height", C.c_float),
                ("surface", C.c_uint32), ("pad_", C.c_uint32)]


class orc_object(C.Structure):
    _fields_ = [("surface", C.c_uint32), ("material", C.c_uint32)]


class orc_material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("color", C.c_float * 3), ("fuzz", C.c_float), ("ir", C.c_float),
                ("roughness", C.c_float), ("metallic", C.c_float), ("emittance", C.c_float),
                ("transparent", C.c_int32), ("albedo_texture", C.c_int32), ("normal_texture", C.c_int32),
                ("mix_first", C.c_int32), ("mix_second", C.c_int32), ("mix_factor", C.c_float)]


class orc_texture(C.Structure):
    _fields_ = [("image", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("sampling", C.c_int32),
                ("pad_", C.c_int32)]


class orc_env(C.Structure):
    _fields_ = [("kind", C.c_int32), ("color", C.c_float * 3), ("image", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("importance_sample", C.c_int32), ("pad_", C.c_int32)]


class orc_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("direction", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float),
                ("has_dof", C.c_int32), ("aperture", C.c_float), ("focal_point", C.c_float * 3)]


class orc_scene_desc(C.Structure):
    _fields_ = [("meshes", C.c_void_p), ("num_meshes", C.c_uint32), ("num_materials", C.c_uint32),
                ("materials", C.c_void_p), ("objects", C.c_void_p), ("num_objects", C.c_uint32),
                ("pad_", C.c_uint32), ("env", orc_env), ("camera", orc_camera), ("analytics", C.c_void_p),
                ("num_analytics", C.c_uint32), ("num_textures", C.c_uint32), ("textures", C.c_void_p)]


class orc_settings(C.Structure):
    _fields_ = [("total_samples", C.c_uint32), ("render_mode", C.c_int32), ("firefly_clamp", C.c_float),
                ("max_bounces", C.c_uint32), ("estimator", C.c_int32), ("rr_depth", C.c_uint32)]


P = C.c_void_p
_SIGS = {
    "orc_scene_create": (P, [P]),
    "orc_scene_destroy": (None, [P]),
    "orc_last_error": (C.c_char_p, []),
    "orc_intersect": (None, [P, P, C.c_uint64, P, P, C.c_int32, C.c_int32]),
    "orc_triangle_hit": (C.c_int32, [P, C.c_uint32, P, P, P, P]),
    "orc_reintersect_f64": (C.c_int32, [P, C.c_uint32, P, P, P, P]),
    "orc_render": (None, [P, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32,
                          C.c_uint32, C.c_int32, P]),
    "orc_trace_path": (None, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, P]),
    "orc_tonemap": (None, [P, P, C.c_uint64, C.c_int32, C.c_float, C.c_float, C.c_float]),
    "orc_tonemap_legacy": (None, [P, P, C.c_uint64, C.c_int32, C.c_float, C.c_float, C.c_int32, C.c_float]),
    "orc_env_eval": (None, [P, P, P]),
    "orc_env_sample": (C.c_int32, [P, P, P, P]),
    "orc_env_pdf": (C.c_float, [P, P]),
    "orc_env_tables": (C.c_int32, [P, P, P, P]),
    "orc_pcg32": (None, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, P]),
    "orc_sampler": (None, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, C.c_uint32, P]),
    "orc_aabb_hit": (C.c_int32, [P, P, P, C.c_float, C.c_float]),
    "orc_num_triangles": (C.c_uint64, [P]),
    "orc_max_threads": (C.c_int32, []),
}
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        d = C.CDLL(str(LIB))
        for k, (r, a) in _SIGS.items():
            fn = getattr(d, k)
            fn.restype = r
            fn.argtypes = a
        _lib = d
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleScene:
    """The oracle's restatement of a voidray_gb300.scene.Scene (same inputs)."""

    def __init__(self, scene):
        keep = []
        mesh_surfs = [(s, x) for s, x in enumerate(scene.surfaces) if isinstance(x, int)]
        ana_surfs = [(s, x) for s, x in enumerate(scene.surfaces) if not isinstance(x, int)]
        n = len(mesh_surfs)
        meshes = (orc_mesh * max(1, n))()
        for k, (s, mi) in enumerate(mesh_surfs):
            m = scene.meshes[mi]
            keep.append(m)
            meshes[k] = orc_mesh(_p(m.positions), _p(m.normals), _p(m.uvs), _p(m.indices), len(m.positions),
                                 len(m.indices), s, 0)
        anas = (orc_analytic * max(1, len(ana_surfs)))()
        for k, (s, a) in enumerate(ana_surfs):
            anas[k].kind, anas[k].radius, anas[k].height, anas[k].surface = a.kind, a.radius, a.height, s
            for j in range(3):
                anas[k].center[j] = float(a.center[j])
        flat = scene.flat_materials()
        mats = (orc_material * max(1, len(flat)))()
        for i, (m, first, second) in enumerate(flat):
            c = mats[i]
            c.mix_first, c.mix_second, c.mix_factor = first, second, m.factor
            c.kind = m.kind
            for k in range(3):
                c.color[k] = float(m.color[k])
            c.fuzz, c.ir, c.roughness, c.metallic = m.fuzz, m.ir, m.roughness, m.metallic
            c.emittance, c.transparent = m.emittance, int(m.transparent)
            c.albedo_texture, c.normal_texture = m.albedo_texture, m.normal_texture
        texs = (orc_texture * max(1, len(scene.textures)))()
        for i, t in enumerate(scene.textures):
            keep.append(t.image)
            texs[i] = orc_texture(_p(t.image), t.image.shape[1], t.image.shape[0], int(t.sample_type), 0)
        keep += [anas, texs]
        objs = (orc_object * max(1, len(scene.objects)))(*[orc_object(o.surface, o.material) for o in scene.objects])
        d = orc_scene_desc()
        d.meshes, d.num_meshes = C.addressof(meshes), n
        d.analytics, d.num_analytics = C.addressof(anas), len(ana_surfs)
        d.textures, d.num_textures = C.addressof(texs), len(scene.textures)
        d.materials, d.num_materials = C.addressof(mats), len(flat)
        d.objects, d.num_objects = C.addressof(objs), len(scene.objects)
        env = scene.environment
        if env is not None:
            d.env.kind = env.kind
            for k in range(3):
                d.env.color[k] = float(env.color[k])
            if env.image is not None:
                d.env.image = _p(env.image)
                d.env.height, d.env.width = env.image.shape[0], env.image.shape[1]
                d.env.importance_sample = int(env.importance_sample)
        cam = scene.camera
        c = d.camera
        for k in range(3):
            c.eye[k], c.direction[k], c.up[k] = float(cam.eye[k]), float(cam.direction[k]), float(cam.up[k])
        c.fov = float(cam.fov)
        if cam.dof is not None:
            c.has_dof = 1
            c.aperture = float(cam.dof[0])
            for k in range(3):
                c.focal_point[k] = float(cam.dof[1][k])
        h = lib().orc_scene_create(C.byref(d))
        if not h:
            raise RuntimeError("oracle scene: " + lib().orc_last_error().decode())
        self._h = C.c_void_p(h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_scene_destroy(self._h)
            self._h = None

    def intersect(self, rays: np.ndarray, mode: int = 0, threads: int = 0, second: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((len(rays), 4), np.float32)
        sec = np.empty(len(rays), np.float32) if second else None
        lib().orc_intersect(self._h, _p(rays), len(rays), _p(hits), _p(sec), mode, threads)
        return (hits, sec) if second else hits

    def triangle_hit(self, prim: int, ray):
        ray = np.ascontiguousarray(ray, np.float32).reshape(8)
        t, u, v = C.c_float(), C.c_float(), C.c_float()
        ok = lib().orc_triangle_hit(self._h, prim, _p(ray), C.byref(t), C.byref(u), C.byref(v))
        return (t.value, u.value, v.value) if ok else None

    def reintersect_f64(self, prim: int, ray):
        ray = np.ascontiguousarray(ray, np.float32).reshape(8)
        t, u, v = C.c_double(), C.c_double(), C.c_double()
        ok = lib().orc_reintersect_f64(self._h, prim, _p(ray), C.byref(t), C.byref(u), C.byref(v))
        return (t.value, u.value, v.value) if ok else None

    def render(self, settings, samples: int, width: int, height: int, seed: int = 0, first_sample: int = 0,
               rgba: np.ndarray | None = None, pixel_range=(0, 0), threads: int = 0):
        st = orc_settings(int(settings.total_samples), int(settings.render_mode), float(settings.firefly_clamp),
                          int(settings.max_bounces), int(settings.estimator), int(settings.rr_depth))
        if rgba is None:
            rgba = np.zeros((height, width, 4), np.float32)
        rays = np.zeros(2, np.uint64)
        lib().orc_render(self._h, C.byref(st), samples, _p(rgba), width, height, seed, first_sample,
                         pixel_range[0], pixel_range[1], threads, _p(rays))
        return rgba, rays

    def trace_path(self, settings, width, height, pixel, sample, seed=0):
        st = orc_settings(int(settings.total_samples), int(settings.render_mode), float(settings.firefly_clamp),
                          int(settings.max_bounces), int(settings.estimator), int(settings.rr_depth))
        out = np.zeros(3, np.float32)
        lib().orc_trace_path(self._h, C.byref(st), width, height, pixel, sample, seed, _p(out))
        return out

    def env_eval(self, d):
        d = np.ascontiguousarray(d, np.float32).reshape(3)
        out = np.zeros(3, np.float32)
        lib().orc_env_eval(self._h, _p(d), _p(out))
        return out

    def env_tables(self, width, height):
        m = np.zeros(height + 1, np.float32)
        c = np.zeros(height * (width + 1), np.float32)
        cell = np.zeros(height * width, np.float32)
        ok = lib().orc_env_tables(self._h, _p(m), _p(c), _p(cell))
        return (m, c, cell) if ok else None


def tonemap(rgba: np.ndarray, tonemap: int, gamma: float, exposure: float, scale: float) -> np.ndarray:
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.empty_like(rgba)
    lib().orc_tonemap(_p(rgba), _p(out), rgba.size // 4, tonemap, gamma, exposure, scale)
    return out


def tonemap_legacy(rgba: np.ndarray, tonemap: int, gamma: float, exposure: float, transparent: bool,
                   scale: float) -> np.ndarray:
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.empty_like(rgba)
    lib().orc_tonemap_legacy(_p(rgba), _p(out), rgba.size // 4, tonemap, gamma, exposure, int(transparent), scale)
    return out


def pcg32(seed: int, sample: int, pixel: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_pcg32(seed, sample, pixel, n, _p(out))
    return out


def sampler(seed: int, sample: int, pixel: int, kind: int, n: int) -> np.ndarray:
    out = np.zeros((n, 3), np.float32)
    lib().orc_sampler(seed, sample, pixel, kind, n, _p(out))
    return out


def aabb_hit(bmin, bmax, ray, t_min, t_max) -> bool:
    bmin = np.ascontiguousarray(bmin, np.float32)
    bmax = np.ascontiguousarray(bmax, np.float32)
    ray = np.ascontiguousarray(ray, np.float32).reshape(8)
    return bool(lib().orc_aabb_hit(_p(bmin), _p(bmax), _p(ray), t_min, t_max))


def max_threads() -> int:
    return int(lib().orc_max_threads())
