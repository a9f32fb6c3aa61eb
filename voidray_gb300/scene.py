"""Host-side mirror of voidray_renderer's scene, camera, material and settings API.

Names, argument meaning and defaults follow the reference so that code written
against ``voidray_renderer`` / ``voidray_common`` reads the same here:

  Scene.add_material / add_mesh / add_object / add_analytic_surface
        voidray_renderer/src/core/scene.rs:112-161
  Scene.build_acceleration -> SceneAcceleration   scene.rs:163-178
  SceneAcceleration.hit                            scene.rs:182-185
  Camera.look_at                                   core/camera.rs:26-36
  Mesh.from_buffers / Vertex.position              core/mesh.rs:25-33, 76-116
  Materials.*                                      voidray_common/src/simple.rs:15-58
  MicrofacetBSDF.*                                 voidray_common/src/microfacet.rs:29-101
  Environments.uniform / hdri                      voidray_common/src/environments.rs:9-17
  Surfaces.quad                                    voidray_common/src/surfaces.rs:18-28
  RenderSettings / ColorManagementSettings / Tonemap / RenderMode
                                                   core/settings.rs:3-74
  iterative_render                                 render/iterative.rs:11-55

Where the reference panics (an index out of range, an unsupported trait
object) this mirror raises VoidrayError.  Every render and intersection runs in
the native library on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from ._native import VoidrayError, check, lib, ptr

f32 = np.float32
PI = f32(math.pi)  # std::f32::consts::PI


# ----------------------------------------------------------------- f32 math --
def _v(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).reshape(3)


def _dot(a, b) -> np.float32:
    # cgmath: (x*x' + y*y') + z*z', each operation rounded to f32
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def _normalize(a) -> np.ndarray:
    r = f32(f32(1.0) / f32(np.sqrt(_dot(a, a))))
    return (a * r).astype(np.float32)


def degrees_to_radians(deg: float) -> np.float32:
    """math.rs:40-43 (degrees * PI / 180 in f32)."""
    return f32(f32(f32(deg) * PI) / f32(180.0))


def hex_color(x: int) -> np.ndarray:
    """color.rs:20-25."""
    return np.array([((x >> 16) & 0xFF) / 255.0, ((x >> 8) & 0xFF) / 255.0, (x & 0xFF) / 255.0], dtype=np.float32)


# --------------------------------------------------------------- settings ---
class RenderMode(enum.IntEnum):
    """settings.rs:8-12 (reference order Normal, Full)."""
    Normal = 0
    Full = 1


class Tonemap(enum.IntEnum):
    """settings.rs:36-55 (Tonemap::as_i32)."""
    NONE = 0
    ACES = 1
    Reinhard = 2
    Filmic = 3
    Uncharted2 = 4


class Estimator(enum.IntEnum):
    """REFERENCE reproduces trace_ray_internal; NEE is the production estimator."""
    REFERENCE = 0
    NEE = 1


@dataclass
class RenderSettings:
    """settings.rs:15-34, defaults included, plus the GPU-only knobs."""
    total_samples: int = 100
    update_frequency: float = 0.1
    render_mode: RenderMode = RenderMode.Full
    firefly_clamp: float = 3.0
    max_bounces: int = 10
    estimator: Estimator = Estimator.REFERENCE
    rr_depth: int = 0
    wavefront_paths: int = 0

    def to_c(self) -> N.vr_render_settings:
        return N.vr_render_settings(int(self.total_samples), float(self.update_frequency), int(self.render_mode),
                                    float(self.firefly_clamp), int(self.max_bounces), int(self.estimator),
                                    int(self.rr_depth), int(self.wavefront_paths))


@dataclass
class ColorManagementSettings:
    """settings.rs:57-74."""
    tonemap: Tonemap = Tonemap.NONE
    gamma: float = 2.2
    exposure: float = 0.0
    transparent: bool = True

    def to_c(self) -> N.vr_color_management:
        return N.vr_color_management(int(self.tonemap), float(self.gamma), float(self.exposure), int(self.transparent))


@dataclass
class Settings:
    render: RenderSettings = field(default_factory=RenderSettings)
    color_management: ColorManagementSettings = field(default_factory=ColorManagementSettings)


# -------------------------------------------------------------- materials ---
@dataclass
class Material:
    kind: int
    color: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    fuzz: float = 0.0
    ir: float = 1.0
    roughness: float = 1.0
    metallic: float = 0.0
    emittance: float = 0.0
    transparent: bool = False
    albedo_texture: int = -1   # TextureHandle of ColorType::Texture, -1: use `color`
    normal_texture: int = -1   # TextureHandle of the normal map, -1: none
    first: Optional["Material"] = None   # MixMaterial children and factor
    second: Optional["Material"] = None
    factor: float = 0.0

    def to_c(self, first: int = -1, second: int = -1) -> N.vr_material:
        m = N.vr_material()
        m.mix_first, m.mix_second, m.mix_factor = int(first), int(second), float(self.factor)
        m.kind = self.kind
        for i in range(3):
            m.color[i] = float(self.color[i])
        m.fuzz, m.ir, m.roughness = float(self.fuzz), float(self.ir), float(self.roughness)
        m.metallic, m.emittance, m.transparent = float(self.metallic), float(self.emittance), int(self.transparent)
        m.albedo_texture, m.normal_texture = int(self.albedo_texture), int(self.normal_texture)
        return m


class SampleType(enum.IntEnum):
    """texture.rs:23-26."""
    Nearest = 0
    Bilinear = 1


@dataclass
class ImageTexture:
    """ImageTexture (texture.rs:28-98) from a decoded RGB f32 image (H x W x 3,
    row 0 first); file decoding is not on the GPU path."""
    image: np.ndarray
    sample_type: SampleType = SampleType.Bilinear

    def __post_init__(self):
        self.image = np.ascontiguousarray(self.image, dtype=np.float32)
        if self.image.ndim != 3 or self.image.shape[2] != 3 or self.image.size == 0:
            raise VoidrayError(1, "texture image must be H x W x 3")

    @staticmethod
    def from_file(path: str, sample_type: SampleType = SampleType.Bilinear) -> "ImageTexture":
        """ImageTexture::new (texture.rs:36-50): `image::open(path).to_rgb32f()`."""
        from .assets import load_image_rgb32f

        return ImageTexture(load_image_rgb32f(path), sample_type)


LAMBERTIAN, METAL, DIELECTRIC, EMISSION, LAMBERTIAN_BSDF, MICROFACET, MIX = range(7)
MAX_MIX_DEPTH = 8  # VR_MAX_MIX_DEPTH


class Materials:
    """voidray_common/src/simple.rs:15-58."""

    @staticmethod
    def lambertian(albedo) -> Material:
        return Material(LAMBERTIAN, _v(albedo))

    @staticmethod
    def lambertian_bsdf(albedo) -> Material:
        return Material(LAMBERTIAN_BSDF, _v(albedo))

    @staticmethod
    def metal(albedo, fuzz: float) -> Material:
        return Material(METAL, _v(albedo), fuzz=float(f32(fuzz)))

    @staticmethod
    def dielectric(ir: float) -> Material:
        return Material(DIELECTRIC, np.ones(3, np.float32), ir=float(f32(ir)))

    @staticmethod
    def emissive(strength: float) -> Material:
        return Materials.colored_emissive(np.ones(3, np.float32), strength)

    @staticmethod
    def colored_emissive(color, strength: float) -> Material:
        # Emission::new: color * strength in f32 (simple.rs:168-172)
        return Material(EMISSION, (_v(color) * f32(strength)).astype(np.float32))

    @staticmethod
    def lambertian_texture(albedo: int, normal: int) -> Material:
        """simple.rs:36-41: albedo texture and normal map (TextureHandles)."""
        return Material(LAMBERTIAN, np.zeros(3, np.float32), albedo_texture=int(albedo), normal_texture=int(normal))

    @staticmethod
    def lambertian_texture_no_normal(albedo: int) -> Material:
        """simple.rs:29-34."""
        return Material(LAMBERTIAN, np.zeros(3, np.float32), albedo_texture=int(albedo))

    @staticmethod
    def mix(first: Material, second: Material, factor: float) -> Material:
        """MixMaterial::new(first, second, factor) of the legacy crate
        (voidray/src/common/materials.rs:188-203): each hit draws u in [0, 1)
        and shades with `first` when u >= factor, else with `second`."""
        if not isinstance(first, Material) or not isinstance(second, Material):
            raise VoidrayError(1, "MixMaterial children must be materials")
        return Material(MIX, np.zeros(3, np.float32), first=first, second=second, factor=float(f32(factor)))


class MicrofacetBSDF:
    """voidray_common/src/microfacet.rs:29-101."""

    @staticmethod
    def make(color, index, roughness, metallic, emittance, transparent) -> Material:
        return Material(MICROFACET, _v(color), ir=float(f32(index)), roughness=float(f32(roughness)),
                        metallic=float(f32(metallic)), emittance=float(f32(emittance)), transparent=bool(transparent))

    @staticmethod
    def diffuse(color):
        return MicrofacetBSDF.make(color, 1.5, 1.0, 0.0, 0.0, False)

    @staticmethod
    def specular(color, roughness):
        return MicrofacetBSDF.make(color, 1.5, roughness, 0.0, 0.0, False)

    @staticmethod
    def clear(index, roughness):
        return MicrofacetBSDF.make(hex_color(0xFFFFFF), index, roughness, 0.0, 0.0, True)

    @staticmethod
    def transparent(color, index, roughness):
        return MicrofacetBSDF.make(color, index, roughness, 0.0, 0.0, True)

    @staticmethod
    def metallic(color, roughness):
        return MicrofacetBSDF.make(color, 1.5, roughness, 1.0, 0.0, False)

    @staticmethod
    def light(color, emittance):
        return MicrofacetBSDF.make(color, 1.0, 1.0, 0.0, emittance, False)


# ------------------------------------------------------------------ meshes ---
@dataclass
class Vertex:
    position: np.ndarray
    uv: np.ndarray
    normal: np.ndarray

    @staticmethod
    def position_only(p) -> "Vertex":
        """Vertex::position (mesh.rs:25-33): zero uv, zero normal."""
        return Vertex(_v(p), np.zeros(2, np.float32), np.zeros(3, np.float32))


class Mesh:
    """Indexed triangle mesh (mesh.rs:35-41); arrays are f32 / u32."""

    def __init__(self, positions, indices, normals=None, uvs=None):
        self.positions = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        self.normals = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        self.uvs = None if uvs is None else np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 2)
        if self.indices.size and int(self.indices.max()) >= len(self.positions):
            raise VoidrayError(1, "mesh index out of range")

    @staticmethod
    def from_buffers(vertices: Sequence[Vertex], indices) -> "Mesh":
        pos = np.stack([v.position for v in vertices]).astype(np.float32)
        nrm = np.stack([v.normal for v in vertices]).astype(np.float32)
        uv = np.stack([v.uv for v in vertices]).astype(np.float32)
        return Mesh(pos, indices, None if not nrm.any() else nrm, None if not uv.any() else uv)

    @staticmethod
    def from_file(path: str) -> "Mesh":
        """Mesh::from_file (mesh.rs:46-74): the OBJ's vertices numbered as obj-rs
        numbers (position, texture, normal) triples, then Mesh::from_buffers."""
        from .assets import load_obj

        pos, uv, nrm, idx = load_obj(path)
        return Mesh(pos, idx, None if not nrm.any() else nrm, None if not uv.any() else uv)

    @property
    def num_triangles(self) -> int:
        return len(self.indices)


class Surfaces:
    """voidray_common/src/surfaces.rs:7-29."""

    @staticmethod
    def quad(q1, q2, q3, q4) -> Mesh:
        # zero vertex normals, as Vertex::position (surfaces.rs:18-28)
        return Mesh(np.stack([_v(q1), _v(q2), _v(q3), _v(q4)]), [0, 1, 2, 2, 0, 3])

    @staticmethod
    def sphere(center, radius) -> "AnalyticSurface":
        """Sphere (surfaces.rs:31-80)."""
        return AnalyticSurface(1, _v(center), float(f32(radius)), 0.0)

    @staticmethod
    def ground_plane(height) -> "AnalyticSurface":
        """GroundPlane y = height (surfaces.rs:82-114)."""
        return AnalyticSurface(2, np.zeros(3, np.float32), 0.0, float(f32(height)))


@dataclass
class AnalyticSurface:
    """An analytic surface of the closed set the GPU path covers: kind 1
    sphere (center, radius), kind 2 ground plane (height)."""
    kind: int
    center: np.ndarray
    radius: float
    height: float


# ------------------------------------------------------------- environment --
@dataclass
class Environment:
    kind: int
    color: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    image: Optional[np.ndarray] = None  # H x W x 3 f32, row 0 first
    importance_sample: bool = True


class Environments:
    """voidray_common/src/environments.rs:9-17."""

    @staticmethod
    def uniform(background) -> Environment:
        return Environment(1, _v(background))

    @staticmethod
    def hdri_image(image: np.ndarray, importance_sample: bool = True) -> Environment:
        """Environments::hdri with the decoded RGB f32 image (no file decoding here)."""
        img = np.ascontiguousarray(image, dtype=np.float32)
        if img.ndim != 3 or img.shape[2] != 3:
            raise VoidrayError(1, "HDRI image must be H x W x 3")
        return Environment(2, np.zeros(3, np.float32), img, importance_sample)

    @staticmethod
    def hdri(path: str, importance_sample: bool = True) -> Environment:
        """Environments::hdri (environments.rs:14-16, 42-55): decodes the file
        (EXR, PNG, JPEG or TIFF) to RGB f32."""
        from .assets import load_image_rgb32f

        return Environments.hdri_image(load_image_rgb32f(path), importance_sample)


# ------------------------------------------------------------------ camera ---
@dataclass
class Camera:
    """camera.rs:7-36; `fov` in radians on the longer image axis."""
    eye: np.ndarray
    direction: np.ndarray
    up: np.ndarray
    fov: float
    dof: Optional[tuple] = None  # (aperture, focal_point)

    @staticmethod
    def look_at(eye, center, up, fov) -> "Camera":
        eye, center, up = _v(eye), _v(center), _v(up)
        direction = _normalize((center - eye).astype(np.float32))
        d = _dot(up, direction)
        up2 = _normalize((up - (d * direction).astype(np.float32)).astype(np.float32))
        return Camera(eye, direction, up2, float(f32(fov)))

    def to_c(self) -> N.vr_camera_desc:
        c = N.vr_camera_desc()
        for i in range(3):
            c.eye[i], c.direction[i], c.up[i] = float(self.eye[i]), float(self.direction[i]), float(self.up[i])
        c.fov = float(self.fov)
        if self.dof is not None:
            c.has_dof = 1
            c.aperture = float(self.dof[0])
            for i in range(3):
                c.focal_point[i] = float(self.dof[1][i])
        return c


# ------------------------------------------------------------------- scene ---
@dataclass
class Object:
    surface: int
    material: int


class Scene:
    """scene.rs:36-161.  Handles are plain ints."""

    def __init__(self):
        self.camera = Camera.look_at((1.0, 0.0, 10.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), float(PI / f32(6.0)))
        self.materials: list[Material] = []
        self.meshes: list[Mesh] = []
        self.surfaces: list[int] = []  # surface -> mesh index
        self.objects: list[Object] = []
        self.textures: list[ImageTexture] = []
        self.environment: Optional[Environment] = None

    @staticmethod
    def empty() -> "Scene":
        return Scene()

    def add_material(self, material: Material) -> int:
        self.materials.append(material)
        return len(self.materials) - 1

    def flat_materials(self) -> list:
        """The material table the library receives: the scene's materials at
        their handles, then the children of MixMaterials (one entry per
        distinct child object), as (material, first, second) index triples."""
        out = [[m, -1, -1] for m in self.materials]
        index = {id(m): i for i, m in enumerate(self.materials)}

        def place(m: Material, depth: int) -> int:
            if depth > MAX_MIX_DEPTH:
                raise VoidrayError(1, f"MixMaterial nested deeper than {MAX_MIX_DEPTH} levels")
            k = index.get(id(m))
            if k is None:
                k = index[id(m)] = len(out)
                out.append([m, -1, -1])
                expand(k, depth)
            return k

        def expand(k: int, depth: int) -> None:
            m = out[k][0]
            if m.kind == MIX:
                out[k][1] = place(m.first, depth + 1)
                out[k][2] = place(m.second, depth + 1)

        for k in range(len(self.materials)):
            expand(k, 0)
        return [tuple(e) for e in out]

    def add_texture(self, texture: ImageTexture) -> int:
        """scene.rs: textures are addressed by TextureHandle."""
        self.textures.append(texture)
        return len(self.textures) - 1

    def add_mesh(self, mesh: Mesh) -> int:
        self.meshes.append(mesh)
        self.surfaces.append(len(self.meshes) - 1)
        return len(self.surfaces) - 1

    def add_analytic_surface(self, surface: "AnalyticSurface") -> int:
        """scene.rs:110-116: analytic surfaces share the surface list with meshes."""
        if not isinstance(surface, AnalyticSurface):
            raise VoidrayError(2, "only Surfaces.sphere / Surfaces.ground_plane are supported by the GPU path")
        self.surfaces.append(surface)
        return len(self.surfaces) - 1

    def add_mesh_from_file(self, path: str) -> int:
        """scene.rs:137-144 with Mesh::from_file (OBJ, obj-rs TexturedVertex rules)."""
        return self.add_mesh(Mesh.from_file(path))

    def add_image_texture(self, path: str, sample_type: "SampleType" = None) -> int:
        """scene.rs:154-160: decodes the file (PNG, EXR, JPEG or TIFF) to RGB f32."""
        return self.add_texture(ImageTexture.from_file(path, SampleType.Bilinear if sample_type is None
                                                       else sample_type))

    def add_object(self, material: int, surface: int) -> int:
        self.objects.append(Object(surface, material))
        return len(self.objects) - 1

    def surface_materials(self) -> list[int]:
        """Material of each surface.  The reference's top-level BVH is built over
        surface indices and the hit surface index is then used as an object
        index (scene.rs:283-285, 377-378), so surface s renders with
        objects[s].material."""
        if len(self.objects) < len(self.surfaces):
            raise VoidrayError(1, "surface without an object at the same index (the reference panics here)")
        out = []
        for s in range(len(self.surfaces)):
            m = self.objects[s].material
            if m >= len(self.materials):
                raise VoidrayError(1, "material index out of range")
            out.append(m)
        return out

    def num_triangles(self) -> int:
        return sum(m.num_triangles for m in self.meshes)

    # lowering to the C descriptor -------------------------------------------
    def to_c(self, bvh_max_leaf: int = 0, bvh_bins: int = 0):
        """Returns (vr_scene_desc, keepalive) for the native library."""
        mats = self.surface_materials()
        keep = []
        mesh_surfs = [(s, x) for s, x in enumerate(self.surfaces) if isinstance(x, int)]
        ana_surfs = [(s, x) for s, x in enumerate(self.surfaces) if not isinstance(x, int)]
        meshes = (N.vr_mesh_desc * max(1, len(mesh_surfs)))()
        anas = (N.vr_analytic_desc * max(1, len(ana_surfs)))()
        for k, (s, a) in enumerate(ana_surfs):
            anas[k].kind, anas[k].radius, anas[k].height, anas[k].material = a.kind, a.radius, a.height, mats[s]
            for j in range(3):
                anas[k].center[j] = float(a.center[j])
        for k, (s, mi) in enumerate(mesh_surfs):
            m = self.meshes[mi]
            keep.append(m)
            d = meshes[k]
            d.positions = ptr(m.positions)
            d.normals = ptr(m.normals)
            d.uvs = ptr(m.uvs)
            d.indices = ptr(m.indices)
            d.num_vertices = len(m.positions)
            d.num_triangles = len(m.indices)
            d.material = mats[s]
        flat = self.flat_materials()
        cm = (N.vr_material * max(1, len(flat)))(*[m.to_c(a, b) for m, a, b in flat])
        desc = N.vr_scene_desc()
        desc.meshes = C.addressof(meshes)
        desc.num_meshes = len(mesh_surfs)
        desc.analytics = C.addressof(anas)
        desc.num_analytics = len(ana_surfs)
        texs = (N.vr_texture_desc * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            keep.append(t.image)
            texs[i] = N.vr_texture_desc(ptr(t.image), t.image.shape[1], t.image.shape[0], int(t.sample_type), 0)
        desc.textures = C.addressof(texs)
        desc.num_textures = len(self.textures)
        keep.append(texs)
        desc.materials = C.addressof(cm)
        desc.num_materials = len(flat)
        env = self.environment
        if env is not None:
            desc.environment.kind = env.kind
            for i in range(3):
                desc.environment.color[i] = float(env.color[i])
            if env.image is not None:
                keep.append(env.image)
                desc.environment.image = ptr(env.image)
                desc.environment.height, desc.environment.width = env.image.shape[0], env.image.shape[1]
                desc.environment.importance_sample = int(env.importance_sample)
        desc.camera = self.camera.to_c()
        desc.bvh_max_leaf = bvh_max_leaf
        desc.bvh_bins = bvh_bins
        keep += [meshes, cm, anas]
        return desc, keep

    def validate(self, **kw) -> N.vr_scene_info:
        """Host-only BVH build and structural check (no GPU needed)."""
        desc, keep = self.to_c(**kw)
        info = N.vr_scene_info()
        check(lib().vr_scene_validate(C.byref(desc), C.byref(info)))
        return info

    def build_acceleration(self, **kw) -> "SceneAcceleration":
        return SceneAcceleration(self, **kw)


class SceneAcceleration:
    """GPU-resident scene (vr_scene handle)."""

    def __init__(self, scene: Scene, **kw):
        desc, keep = scene.to_c(**kw)
        h = C.c_void_p()
        check(lib().vr_scene_create(C.byref(desc), C.byref(h)))
        self._h = h
        self._keep_lists(scene)

    def _keep_lists(self, scene: Scene) -> None:
        """Scene::build_acceleration (scene.rs:163-178) keeps copies of the
        scene's lists; the *_ref accessors read them."""
        self.camera = scene.camera
        self.environment = scene.environment
        self._objects = list(scene.objects)
        self._surfaces = list(scene.surfaces)
        self._textures = list(scene.textures)
        self._meshes = list(scene.meshes)
        self._materials = list(scene.materials)

    # scene.rs:207-225; handles are plain ints
    def surface_ref(self, surface: int):
        """The mesh of a mesh surface, or the AnalyticSurface."""
        s = self._surfaces[surface]
        return self._meshes[s] if isinstance(s, int) else s

    def material_ref(self, material: int) -> "Material":
        return self._materials[material]

    def texture_ref(self, texture: int) -> "ImageTexture":
        return self._textures[texture]

    def mesh_ref(self, mesh: int) -> "Mesh":
        return self._meshes[mesh]

    def object_ref(self, obj: int) -> "Object":
        return self._objects[obj]

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise VoidrayError(1, "scene destroyed")
        return self._h

    def info(self) -> N.vr_scene_info:
        info = N.vr_scene_info()
        check(lib().vr_scene_info_get(self.handle, C.byref(info)))
        return info

    def set_camera(self, camera: Camera) -> None:
        c = camera.to_c()
        check(lib().vr_scene_set_camera(self.handle, C.byref(c)))
        self.camera = camera

    def hit(self, rays: np.ndarray, any_hit: bool = False) -> np.ndarray:
        """Batch SceneAcceleration::hit.  rays: (n, 8) f32 (org, tmin, dir, tmax).
        Returns (n, 4) records viewed as f32 with column 0 holding the u32 prim id."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.empty((len(rays), 4), dtype=np.float32)
        check(lib().vr_intersect(self.handle, ptr(rays), len(rays), ptr(hits), int(any_hit)))
        return hits

    def environment_sample(self, directions: np.ndarray) -> np.ndarray:
        """Environment::sample (traits.rs:66-69) for (n, 3) directions -> (n, 3) RGB."""
        d = np.ascontiguousarray(directions, dtype=np.float32).reshape(-1, 3)
        out = np.empty_like(d)
        check(lib().vr_environment_sample(self.handle, ptr(d), len(d), ptr(out)))
        return out

    def stats(self) -> N.vr_render_stats:
        st = N.vr_render_stats()
        check(lib().vr_render_stats_get(self.handle, C.byref(st)))
        return st

    def synchronize(self) -> None:
        check(lib().vr_scene_synchronize(self.handle))

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().vr_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


# ---------------------------------------------------------------- render ----
class CpuRenderTarget:
    """Host RGBA f32 accumulation buffer (render/target.rs:80-131 without Vulkan)."""

    def __init__(self, width: int, height: int):
        self.buffer = np.zeros((height, width, 4), dtype=np.float32)

    def dimensions(self) -> tuple[int, int]:
        return self.buffer.shape[1], self.buffer.shape[0]

    def clear(self) -> None:
        self.buffer[...] = 0.0


def iterative_render(target: CpuRenderTarget, scene: SceneAcceleration, settings: RenderSettings, samples: int,
                     seed: int = 0, first_sample: int = 0) -> None:
    """render/iterative.rs:11-55: target += sum of `samples` paths / total_samples per pixel."""
    w, h = target.dimensions()
    st = settings.to_c()
    buf = target.buffer
    check(lib().vr_render(scene.handle, C.byref(st), int(samples), ptr(buf), w, h, int(seed), int(first_sample)))


def render_device(scene: SceneAcceleration, settings: RenderSettings, samples: int, rgba_device: int, width: int,
                  height: int, seed: int = 0, first_sample: int = 0, stream: int = 0, albedo_device: int = 0,
                  normal_device: int = 0) -> None:
    """iterative_render into device buffers (raw CUDA pointers, RGBA f32), enqueued on `stream`.
    With albedo_device/normal_device set, also accumulates the first-hit feature buffers."""
    st = settings.to_c()
    s = C.c_void_p(stream or None)
    if albedo_device or normal_device:
        check(lib().vr_render_aov_device(scene.handle, C.byref(st), int(samples), C.c_void_p(rgba_device),
                                         C.c_void_p(albedo_device), C.c_void_p(normal_device), int(width),
                                         int(height), int(seed), int(first_sample), s))
    else:
        check(lib().vr_render_device(scene.handle, C.byref(st), int(samples), C.c_void_p(rgba_device), int(width),
                                     int(height), int(seed), int(first_sample), s))


def tonemap(rgba: np.ndarray, cm: ColorManagementSettings, scale: float) -> np.ndarray:
    """post_process.glsl:23-49 on the GPU."""
    rgba = np.ascontiguousarray(rgba, dtype=np.float32)
    out = np.empty_like(rgba)
    h, w = rgba.shape[0], rgba.shape[1]
    c = cm.to_c()
    check(lib().vr_tonemap(ptr(rgba), ptr(out), w, h, C.byref(c), float(scale)))
    return out


class LegacyTonemap(enum.IntEnum):
    """The legacy crate's Tonemap (voidray/src/pipeline.rs:59-68), numbered as
    its viewport shader numbers them (viewport_fragment.glsl:10-17)."""
    NONE = 0
    SimpleACES = 1
    SimpleReinhard = 2
    LumaReinhard = 3
    LumaWhitePreservingReinhard = 4
    RomBinDaHouse = 5
    Filmic = 6
    Uncharted2 = 7


def tonemap_legacy(rgba: np.ndarray, tonemap: LegacyTonemap, gamma: float, exposure: float, transparent: bool,
                   scale: float) -> np.ndarray:
    """viewport_fragment.glsl:27-67 on the GPU: exposure is a linear factor,
    Filmic ignores gamma, `transparent` keeps the scaled alpha."""
    rgba = np.ascontiguousarray(rgba, dtype=np.float32)
    out = np.empty_like(rgba)
    h, w = rgba.shape[0], rgba.shape[1]
    check(lib().vr_tonemap_legacy(ptr(rgba), ptr(out), w, h, int(tonemap), float(gamma), float(exposure),
                                  int(bool(transparent)), float(scale)))
    return out
