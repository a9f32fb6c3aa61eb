"""Seeded synthetic workloads (no external assets or datasets).

  cornell_box()        code-built Cornell box in [-1,1]^3: 5 walls (10
                       triangles), tall and short boxes (24 triangles, rotated
                       +15 / -18 degrees), ceiling emitter (17,12,4); pinhole
                       camera, fov 40 degrees.
  triangle_soup()      N triangles with centres U[0,1]^3 and vertex offsets
                       N(0, 0.01^2) (seed 1).
  soup_rays()          half coherent pinhole rays from z = -1, half incoherent
                       (origins U(cube), directions U(sphere)); tmax = inf.
  displaced_icosphere_scene()
                       geodesic icosphere (20 n^2 triangles; n = 316 gives
                       1,997,120) displaced radially by 4-octave value noise
                       (amplitude 0.1, seed 2) on a 2-triangle ground; materials
                       per 64-triangle patch uniformly among Lambertian (albedo
                       U(0.1,0.9)), metal (fuzz U(0,0.5)) and dielectric (1.5);
                       2048x1024 sky-gradient + sun (sigma 0.5 deg, peak 5e4) HDRI.
  mushroom_scene()     the reference's mushroom demo from its own asset folder
                       (OBJ meshes, JPEG textures), when that folder is given.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .scene import (Camera, Environments, Estimator, Materials, Mesh, RenderSettings, Scene, Surfaces,
                    degrees_to_radians)

f32 = np.float32


def _face_normals(p0, p1, p2):
    """Mesh::from_buffers face normal (p2-p1) x (p0-p1), normalised, in f32."""
    e1 = (p0 - p1).astype(f32)
    e2 = (p2 - p1).astype(f32)
    n = np.stack([e2[..., 1] * e1[..., 2] - e2[..., 2] * e1[..., 1],
                  e2[..., 2] * e1[..., 0] - e2[..., 0] * e1[..., 2],
                  e2[..., 0] * e1[..., 1] - e2[..., 1] * e1[..., 0]], -1).astype(f32)
    return (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(f32)


def _quad_mesh(q, with_normals=True) -> Mesh:
    q = np.asarray(q, dtype=f32)
    idx = np.array([0, 1, 2, 2, 0, 3], dtype=np.uint32)
    nrm = None
    if with_normals:
        n = _face_normals(q[0], q[1], q[2])
        nrm = np.repeat(n[None], 4, axis=0)
    return Mesh(q, idx, nrm)


def _box_mesh(center, size, angle_deg) -> Mesh:
    cx, cy, cz = center
    sx, sy, sz = size
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    corners = []
    for dx in (-0.5, 0.5):
        for dy in (-0.5, 0.5):
            for dz in (-0.5, 0.5):
                x, y, z = dx * sx, dy * sy, dz * sz
                corners.append((cx + ca * x + sa * z, cy + y, cz - sa * x + ca * z))
    c = np.array(corners, dtype=f32)  # index = 4*ix + 2*iy + iz
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    pos, nrm, idx = [], [], []
    ctr = np.array(center, dtype=f32)
    for f in faces:
        q = c[list(f)]
        n = _face_normals(q[0], q[1], q[2])
        if np.dot(n, q.mean(0) - ctr) < 0:  # outward winding
            q = q[::-1].copy()
            n = _face_normals(q[0], q[1], q[2])
        base = len(pos)
        pos.extend(q)
        nrm.extend([n] * 4)
        idx.extend([base, base + 1, base + 2, base + 2, base, base + 3])
    return Mesh(np.array(pos, f32), np.array(idx, np.uint32), np.array(nrm, f32))


def cornell_box(width=256, height=256, spp=16, max_depth=8, rr_depth=3, face_normals=True):
    """Returns (scene, settings) of the code-built Cornell box."""
    s = Scene()
    red = s.add_material(Materials.lambertian((0.63, 0.065, 0.05)))
    green = s.add_material(Materials.lambertian((0.14, 0.45, 0.091)))
    grey = s.add_material(Materials.lambertian((0.725, 0.725, 0.725)))
    light = s.add_material(Materials.colored_emissive((17.0, 12.0, 4.0), 1.0))
    walls = [
        ([(-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)], grey),   # floor
        ([(-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)], grey),       # ceiling
        ([(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)], grey),   # back
        ([(-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)], red),    # left
        ([(1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)], green),      # right
    ]
    for q, m in walls:
        s.add_object(m, s.add_mesh(_quad_mesh(q, face_normals)))
    s.add_object(grey, s.add_mesh(_box_mesh((-0.33, -0.4, -0.28), (0.58, 1.2, 0.58), 15.0)))
    s.add_object(grey, s.add_mesh(_box_mesh((0.34, -0.7, 0.3), (0.58, 0.6, 0.58), -18.0)))
    s.add_object(light, s.add_mesh(_quad_mesh([(-0.25, 0.99, -0.25), (0.25, 0.99, -0.25), (0.25, 0.99, 0.25),
                                              (-0.25, 0.99, 0.25)], face_normals)))
    s.camera = Camera.look_at((0.0, 0.0, 3.75), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), degrees_to_radians(40.0))
    st = RenderSettings(total_samples=spp, max_bounces=max_depth, rr_depth=rr_depth, estimator=Estimator.REFERENCE)
    return s, st


def triangle_soup(n: int, seed: int = 1) -> Mesh:
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3), dtype=np.float64).astype(f32)
    off = (rng.standard_normal((n, 3, 3)) * 0.01).astype(f32)
    pos = (c[:, None, :] + off).astype(f32).reshape(-1, 3)
    return Mesh(pos, np.arange(3 * n, dtype=np.uint32))


def soup_scene(n: int, seed: int = 1) -> Scene:
    s = Scene()
    m = s.add_material(Materials.lambertian((0.5, 0.5, 0.5)))
    s.add_object(m, s.add_mesh(triangle_soup(n, seed)))
    return s


def soup_rays(count: int, width: int = 4096, height: int = 2048, seed: int = 1, tmin: float = 1e-5) -> np.ndarray:
    """(count, 8) f32 rays: first half pinhole rays (row-major over width x
    height, subsampled evenly when count/2 < width*height), second half
    incoherent.  Columns: org xyz, tmin, dir xyz, tmax."""
    rng = np.random.default_rng(seed + 1000)
    n1 = count // 2
    n2 = count - n1
    rays = np.empty((count, 8), dtype=f32)
    # coherent: pinhole at (0.5, 0.5, -1) looking at +z, horizontal fov 60 deg
    idx = np.linspace(0, width * height - 1, n1).astype(np.int64) if n1 < width * height else np.arange(n1)
    px = (idx % width).astype(f32)
    py = (idx // width).astype(f32)
    tan_h = f32(math.tan(math.radians(30.0)))
    x = ((2.0 * (px + 0.5) / width) - 1.0).astype(f32) * tan_h
    y = (1.0 - (2.0 * (py + 0.5) / height)).astype(f32) * tan_h * f32(height / width)
    d = np.stack([x, y, np.ones_like(x)], -1).astype(f32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[:n1, 0:3] = (0.5, 0.5, -1.0)
    rays[:n1, 4:7] = d
    # incoherent
    rays[n1:, 0:3] = rng.random((n2, 3), dtype=np.float64).astype(f32)
    g = rng.standard_normal((n2, 3)).astype(f32)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    rays[n1:, 4:7] = g
    rays[:, 3] = tmin
    rays[:, 7] = np.inf
    return rays


# ------------------------------------------------------------ icosphere ---
def _icosahedron():
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], dtype=np.int64)
    return v, f


def geodesic_sphere(freq: int):
    """Unit-sphere vertices (shared) and triangles of a frequency-`freq`
    subdivided icosahedron: 20*freq^2 triangles."""
    v, faces = _icosahedron()
    ij = [(i, j) for i in range(freq + 1) for j in range(freq + 1 - i)]
    lid = {p: k for k, p in enumerate(ij)}
    I = np.array([p[0] for p in ij], np.float64)[:, None] / freq
    J = np.array([p[1] for p in ij], np.float64)[:, None] / freq
    loc = []
    for i in range(freq):
        for j in range(freq - i):
            loc.append((lid[(i, j)], lid[(i + 1, j)], lid[(i, j + 1)]))
            if i + j < freq - 1:
                loc.append((lid[(i + 1, j)], lid[(i + 1, j + 1)], lid[(i, j + 1)]))
    loc = np.array(loc, np.int64)
    npf = len(ij)
    pts = []
    tris = []
    for fi, (a, b, c) in enumerate(faces):
        p = v[a] + (v[b] - v[a]) * I + (v[c] - v[a]) * J
        pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
        tris.append(loc + fi * npf)
    pts = np.concatenate(pts)
    tris = np.concatenate(tris)
    # weld duplicated edge vertices
    key = np.round(pts * 1e6).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    return pts[first], inv.reshape(-1)[tris]


def value_noise(p: np.ndarray, seed: int = 2, octaves: int = 4, grid: int = 64) -> np.ndarray:
    """Sum of `octaves` octaves of trilinear value noise on a periodic lattice,
    normalised to [-1, 1]."""
    rng = np.random.default_rng(seed)
    lat = rng.uniform(-1.0, 1.0, size=(grid, grid, grid))
    out = np.zeros(len(p))
    amp, freq, norm = 1.0, 2.0, 0.0
    for _ in range(octaves):
        q = (p + 1.0) * freq
        i0 = np.floor(q).astype(np.int64)
        fr = q - i0
        fr = fr * fr * (3.0 - 2.0 * fr)
        acc = np.zeros(len(p))
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (fr[:, 0] if dx else 1 - fr[:, 0]) * (fr[:, 1] if dy else 1 - fr[:, 1]) * \
                        (fr[:, 2] if dz else 1 - fr[:, 2])
                    acc += w * lat[(i0[:, 0] + dx) % grid, (i0[:, 1] + dy) % grid, (i0[:, 2] + dz) % grid]
        out += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def sky_hdri(width: int = 2048, height: int = 1024, sun_elev_deg: float = 35.0, sun_azim_deg: float = 60.0,
             sigma_deg: float = 0.5, peak: float = 5e4) -> np.ndarray:
    """Lat-long RGB f32 image in the layout environments.rs:79-90 reads: row y
    looks along theta = (H-1-y) pi / H from straight down, column x along
    phi = 2 pi x / W, direction (-sin t cos p, -cos t, sin t sin p)."""
    y = np.arange(height, dtype=np.float64)[:, None]
    x = np.arange(width, dtype=np.float64)[None, :]
    th = (height - 1 - y + 0.5) * math.pi / height
    ph = (x + 0.5) * 2.0 * math.pi / width
    d = np.stack(np.broadcast_arrays(-np.sin(th) * np.cos(ph), -np.cos(th), np.sin(th) * np.sin(ph)), -1)
    elev = d[..., 1]
    zen = np.array([0.18, 0.36, 0.85])
    hor = np.array([0.85, 0.9, 1.0])
    gnd = np.array([0.25, 0.22, 0.18])
    tsky = np.clip(elev, 0.0, 1.0)[..., None] ** 0.5
    img = np.where(elev[..., None] >= 0, hor * (1 - tsky) + zen * tsky, gnd * (0.5 + 0.5 * np.clip(1 + elev, 0, 1))[..., None])
    se, sa = math.radians(sun_elev_deg), math.radians(sun_azim_deg)
    sun = np.array([math.cos(se) * math.cos(sa), math.sin(se), math.cos(se) * math.sin(sa)])
    ang = np.arccos(np.clip(d @ sun, -1.0, 1.0))
    sig = math.radians(sigma_deg)
    img = img + (peak * np.exp(-0.5 * (ang / sig) ** 2))[..., None] * np.array([1.0, 0.95, 0.88])
    return img.astype(f32)


def displaced_icosphere_scene(freq: int = 316, seed: int = 2, patch: int = 64, hdri_size=(2048, 1024),
                              width: int = 1920, height: int = 1080):
    """Returns (scene, settings) of the plain GPU render workload."""
    v, t = geodesic_sphere(freq)
    r = 1.0 + 0.1 * value_noise(v, seed=seed)
    pos = (v * r[:, None]).astype(np.float64)
    # smooth vertex normals (area weighted)
    p0, p1, p2 = pos[t[:, 0]], pos[t[:, 1]], pos[t[:, 2]]
    fn = np.cross(p1 - p0, p2 - p0)
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, t[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    nt = len(t)
    corner_p = pos[t].astype(f32)  # (nt, 3, 3)
    corner_n = vn[t].astype(f32)
    s = Scene()
    rng = np.random.default_rng(seed + 100)
    npatch = (nt + patch - 1) // patch
    kinds = rng.integers(0, 3, npatch)
    alb = rng.uniform(0.1, 0.9, (npatch, 3))
    fuzz = rng.uniform(0.0, 0.5, npatch)
    malb = rng.uniform(0.6, 0.95, (npatch, 3))
    flat_p = corner_p.reshape(-1, 3)
    flat_n = corner_n.reshape(-1, 3)
    for k in range(npatch):
        a, b = k * patch, min(nt, (k + 1) * patch)
        if kinds[k] == 0:
            m = s.add_material(Materials.lambertian(alb[k]))
        elif kinds[k] == 1:
            m = s.add_material(Materials.metal(malb[k], float(fuzz[k])))
        else:
            m = s.add_material(Materials.dielectric(1.5))
        mesh = Mesh(flat_p[3 * a:3 * b], np.arange(3 * (b - a), dtype=np.uint32), flat_n[3 * a:3 * b])
        s.add_object(m, s.add_mesh(mesh))
    ground = s.add_material(Materials.lambertian((0.5, 0.5, 0.5)))
    g = 40.0
    gy = -1.2
    q = np.array([(-g, gy, -g), (-g, gy, g), (g, gy, g), (g, gy, -g)], f32)
    s.add_object(ground, s.add_mesh(Mesh(q, np.array([0, 1, 2, 2, 0, 3], np.uint32),
                                         np.array([(0, 1, 0)] * 4, f32))))
    if hdri_size is not None:  # None: the caller sets a (shared) environment
        s.environment = Environments.hdri_image(sky_hdri(*hdri_size), importance_sample=True)
    s.camera = Camera.look_at((0.0, 0.35, 3.4), (0.0, -0.15, 0.0), (0.0, 1.0, 0.0), degrees_to_radians(50.0))
    st = RenderSettings(total_samples=256, max_bounces=12, rr_depth=3, estimator=Estimator.NEE,
                        firefly_clamp=float("inf"))
    return s, st


def spheres_scene(ground: bool = True, hdri: bool = False, seed: int = 3):
    """A few analytic spheres (Lambertian, metal, dielectric, emitter) over a
    ground plane and a small triangle box, the kind of scene the reference's
    Surfaces::sphere / ground_plane build (voidray_common/src/surfaces.rs)."""
    rng = np.random.default_rng(seed)
    s = Scene()
    grey = s.add_material(Materials.lambertian((0.6, 0.6, 0.6)))
    mats = [s.add_material(Materials.lambertian((0.8, 0.3, 0.2))),
            s.add_material(Materials.metal((0.9, 0.85, 0.7), 0.1)),
            s.add_material(Materials.dielectric(1.5)),
            s.add_material(Materials.colored_emissive((4.0, 3.0, 2.0), 1.0))]
    if ground:
        s.add_object(grey, s.add_analytic_surface(Surfaces.ground_plane(-1.0)))
    for k in range(6):
        c = (float(rng.uniform(-2, 2)), float(rng.uniform(-0.7, 0.5)), float(rng.uniform(-2.5, 0.5)))
        s.add_object(mats[k % 4], s.add_analytic_surface(Surfaces.sphere(c, float(rng.uniform(0.2, 0.5)))))
    s.add_object(grey, s.add_mesh(_box_mesh((0.9, -0.55, -1.0), (0.6, 0.8, 0.6), 20.0)))
    if hdri:
        s.environment = Environments.hdri_image(sky_hdri(128, 64, peak=200.0, sigma_deg=4.0))
    else:
        s.environment = Environments.uniform((0.5, 0.6, 0.8))
    s.camera = Camera.look_at((0.0, 0.6, 4.0), (0.0, -0.3, -0.8), (0.0, 1.0, 0.0), degrees_to_radians(55.0))
    st = RenderSettings(total_samples=16, max_bounces=8, rr_depth=0, estimator=Estimator.REFERENCE,
                        firefly_clamp=float("inf"))
    return s, st


def textured_scene(seed: int = 4):
    """Lambertian quads with image textures (nearest and bilinear, uvs running
    outside [0, 1] and negative to exercise the reference's wrapping), one
    with a normal map, a textured ground plane (uv = world x, z) and a
    sphere, under a uniform sky (texture.rs, simple.rs:83-133)."""
    from .scene import ImageTexture, SampleType

    rng = np.random.default_rng(seed)
    s = Scene()
    checker = ((np.indices((8, 8)).sum(0) % 2)[..., None] * np.array([0.7, 0.6, 0.2]) + 0.1).astype(f32)
    noise = rng.uniform(0.05, 0.95, (13, 17, 3)).astype(f32)
    nmap = np.zeros((4, 4, 3), f32)
    nmap[..., 1] = 1.0
    nmap[..., 0] = rng.uniform(-0.4, 0.4, (4, 4))
    t_check = s.add_texture(ImageTexture(checker, SampleType.Nearest))
    t_noise = s.add_texture(ImageTexture(noise, SampleType.Bilinear))
    t_nmap = s.add_texture(ImageTexture(nmap, SampleType.Nearest))
    m_check = s.add_material(Materials.lambertian_texture_no_normal(t_check))
    m_noise = s.add_material(Materials.lambertian_texture(t_noise, t_nmap))
    m_plain = s.add_material(Materials.lambertian((0.5, 0.5, 0.5)))
    quads = [([(-2.0, -1.0, -2.0), (2.0, -1.0, -2.0), (2.0, 1.5, -2.0), (-2.0, 1.5, -2.0)],
              [(-1.3, -0.7), (2.6, -0.7), (2.6, 1.9), (-1.3, 1.9)], m_noise),
             ([(-2.0, -1.0, -2.0), (-2.0, 1.5, -2.0), (-2.0, 1.5, 1.0), (-2.0, -1.0, 1.0)],
              [(0.0, 0.0), (0.0, 3.0), (3.0, 3.0), (3.0, 0.0)], m_check)]
    for q, uv, m in quads:
        pos = np.array(q, f32)
        nrm = _face_normals(pos[0], pos[1], pos[2])
        mesh = Mesh(pos, np.array([0, 1, 2, 2, 3, 0], np.uint32), np.repeat(nrm[None], 4, 0).astype(f32),
                    np.array(uv, f32))
        s.add_object(m, s.add_mesh(mesh))
    ground = s.add_material(Materials.lambertian_texture_no_normal(t_noise))
    s.add_object(ground, s.add_analytic_surface(Surfaces.ground_plane(-1.0)))
    s.add_object(m_plain, s.add_analytic_surface(Surfaces.sphere((0.4, -0.4, -0.8), 0.6)))
    s.environment = Environments.uniform((0.9, 0.95, 1.0))
    s.camera = Camera.look_at((0.8, 0.5, 3.5), (-0.4, -0.2, -1.0), (0.0, 1.0, 0.0), degrees_to_radians(60.0))
    st = RenderSettings(total_samples=8, max_bounces=6, rr_depth=0, estimator=Estimator.REFERENCE,
                        firefly_clamp=float("inf"))
    return s, st


def mushroom_scene(assets_dir: str, hdri_size=(512, 256)):
    """The reference's mushroom demo (voidray_app/src/examples/mushroom.rs:3-37)
    built from its asset folder: mushroom.obj and mossy_ground.obj with their
    albedo JPEGs and normal maps, the depth-of-field camera, ACES with gamma 1
    and exposure 1, 1000x1000.  Files the folder lacks are replaced: a missing
    normal-map JPEG by the same material without a normal map
    (simple.rs:29-34), a missing studio.exr by the synthetic sky.  Returns
    (scene, Settings, (width, height))."""
    from .scene import ColorManagementSettings, ImageTexture, SampleType, Settings, Tonemap

    def path(name):
        return os.path.join(assets_dir, name)

    s = Scene()
    for stem in ("mushroom", "mossy_ground"):
        albedo = s.add_image_texture(path(f"{stem}_albedo.jpg"), SampleType.Bilinear)
        if os.path.exists(path(f"{stem}_normal.jpg")):
            normal = s.add_texture(ImageTexture.from_file(path(f"{stem}_normal.jpg"), SampleType.Bilinear))
            mtl = s.add_material(Materials.lambertian_texture(albedo, normal))
        else:
            mtl = s.add_material(Materials.lambertian_texture_no_normal(albedo))
        s.add_object(mtl, s.add_mesh_from_file(path(f"{stem}.obj")))
    s.camera = Camera(eye=np.array([0.2, 2.8, -10.5], f32), direction=np.array([0.0, -0.2, 1.0], f32),
                      up=np.array([0.0, 1.0, 0.0], f32), fov=f32(0.17),
                      dof=(0.17, np.array([0.06, 2.14, 0.18], f32)))
    if os.path.exists(path("studio.exr")):
        s.environment = Environments.hdri(path("studio.exr"))
    else:
        s.environment = Environments.hdri_image(sky_hdri(*hdri_size))
    st = Settings()
    st.color_management = ColorManagementSettings(tonemap=Tonemap.ACES, gamma=1.0, exposure=1.0)
    return s, st, (1000, 1000)


def mix_scene(hdri: bool = False, seed: int = 5):
    """Spheres and a box with MixMaterials of the legacy crate
    (voidray/src/common/materials.rs:188-203): Lambertian/metal, nested
    dielectric/Lambertian/emitter mixes and a mix whose children are shared,
    over a ground plane."""
    rng = np.random.default_rng(seed)
    s = Scene()
    red = Materials.lambertian((0.8, 0.25, 0.2))
    gold = Materials.metal((0.9, 0.75, 0.4), 0.2)
    glass = Materials.dielectric(1.5)
    lamp = Materials.colored_emissive((3.0, 2.5, 2.0), 1.0)
    m0 = s.add_material(Materials.mix(red, gold, 0.3))
    m1 = s.add_material(Materials.mix(Materials.mix(glass, red, 0.5), lamp, 0.1))
    m2 = s.add_material(Materials.mix(gold, gold, 0.7))
    grey = s.add_material(Materials.lambertian((0.6, 0.6, 0.6)))
    s.add_object(grey, s.add_analytic_surface(Surfaces.ground_plane(-1.0)))
    for k in range(5):
        c = (float(rng.uniform(-2, 2)), float(rng.uniform(-0.6, 0.4)), float(rng.uniform(-2.5, 0.5)))
        s.add_object([m0, m1, m2][k % 3], s.add_analytic_surface(Surfaces.sphere(c, float(rng.uniform(0.25, 0.5)))))
    s.add_object(m0, s.add_mesh(_box_mesh((0.9, -0.55, -1.0), (0.6, 0.8, 0.6), 20.0)))
    if hdri:
        s.environment = Environments.hdri_image(sky_hdri(128, 64, peak=200.0, sigma_deg=4.0))
    else:
        s.environment = Environments.uniform((0.5, 0.6, 0.8))
    s.camera = Camera.look_at((0.0, 0.6, 4.0), (0.0, -0.3, -0.8), (0.0, 1.0, 0.0), degrees_to_radians(55.0))
    st = RenderSettings(total_samples=16, max_bounces=8, rr_depth=0, estimator=Estimator.REFERENCE,
                        firefly_clamp=float("inf"))
    return s, st


def mixed_job_set(count: int = 16, seed: int = 4, tri_range=(10_000, 200_000), scale: int = 10,
                  spp_range=(2, 32), depth_range=(8, 12)):
    """A many-scene job mix: `count` displaced-icosphere scenes with triangle
    counts log-uniform in `tri_range`, image sizes drawn from {256^2, 512^2,
    1280x720, 1920x1080} divided by `scale`, spp log-uniform in `spp_range`,
    depth uniform in `depth_range`, NEE or the reference estimator; every
    draw is seeded.  Returns [(scene, settings, spp, width, height, seed)]."""
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    out = []
    lo, hi = np.log(tri_range[0]), np.log(tri_range[1])
    for k in range(count):
        tris = float(np.exp(rng.uniform(lo, hi)))
        freq = max(2, int(round(math.sqrt(tris / 20.0))))
        s, st = displaced_icosphere_scene(freq=freq, seed=100 + k, patch=256, hdri_size=(64, 32))
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        w, h = max(8, w // scale), max(8, h // scale)
        spp = int(round(np.exp(rng.uniform(np.log(spp_range[0]), np.log(spp_range[1])))))
        st.max_bounces = int(rng.integers(depth_range[0], depth_range[1] + 1))
        st.total_samples = spp
        st.estimator = Estimator.NEE if rng.random() < 0.5 else Estimator.REFERENCE
        st.firefly_clamp = float(rng.choice([3.0, float("inf")]))
        out.append((s, st, spp, w, h, int(rng.integers(0, 1 << 30))))
    return out


def batched_job_set(count: int = 64, seed: int = 4, tri_range=(10_000, 2_000_000), spp_range=(4, 256),
                    depth_range=(8, 12), hdri_size=(2048, 1024)):
    """The batched workload at full size: `count` displaced-icosphere scenes
    (materials per 64-triangle patch, NEE estimator, clamp off) with triangle
    counts log-uniform in `tri_range`, resolution drawn from {256^2, 512^2,
    1280x720, 1920x1080}, spp log-uniform in `spp_range`, depth uniform in
    `depth_range`, all sharing one importance-sampled sky + sun HDRI.  Every
    draw is seeded.  Returns [(scene, settings, spp, width, height, seed)]."""
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    env = Environments.hdri_image(sky_hdri(*hdri_size), importance_sample=True)
    lo, hi = np.log(tri_range[0]), np.log(tri_range[1])
    out = []
    for k in range(count):
        tris = float(np.exp(rng.uniform(lo, hi)))
        freq = max(2, int(round(math.sqrt(tris / 20.0))))
        s, st = displaced_icosphere_scene(freq=freq, seed=200 + k, hdri_size=None)
        s.environment = env
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        spp = int(round(np.exp(rng.uniform(np.log(spp_range[0]), np.log(spp_range[1])))))
        st.max_bounces = int(rng.integers(depth_range[0], depth_range[1] + 1))
        st.total_samples = spp
        out.append((s, st, spp, w, h, int(rng.integers(0, 1 << 30))))
    return out
