"""Analytic surfaces (Surfaces::sphere, Surfaces::ground_plane,
voidray_common/src/surfaces.rs) in the oracle and the scene lowering; no GPU."""
import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W

MISS = 0xFFFFFFFF


def ray(o, d, tmin=1e-5, tmax=np.inf):
    return np.array([*o, tmin, *d, tmax], np.float32)


def one_sphere_scene():
    s = vr.Scene()
    m = s.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    s.add_object(m, s.add_analytic_surface(vr.Surfaces.sphere((0.0, 0.0, 0.0), 1.0)))
    s.add_object(m, s.add_analytic_surface(vr.Surfaces.ground_plane(-2.0)))
    return s


def test_sphere_and_plane_known_answers(oracle):
    osc = oracle.OracleScene(one_sphere_scene())
    rays = np.stack([ray((0, 0, -5), (0, 0, 1)),        # sphere front: t = 4
                     ray((0, 0, 0), (0, 0, 1)),         # from inside: far root t = 1
                     ray((0, 5, 0), (0, -1, 0)),        # sphere top at t = 4 before the plane (t = 7)
                     ray((3, 5, 0), (0, -1, 0)),        # misses the sphere: plane at t = 7
                     ray((3, 5, 0), (0, 1, 0)),         # away from everything
                     ray((0, 0, -5), (0, 0, 1), tmax=3.0)])  # the sphere is beyond tmax
    h = osc.intersect(rays)
    prims = h[:, 0].view(np.uint32)
    assert list(prims[:4]) == [0, 0, 0, 1] and prims[4] == MISS and prims[5] == MISS
    assert list(h[:4, 1]) == [4.0, 1.0, 4.0, 7.0]
    assert np.all(h[:4, 2:] == 0.0)


def test_lowering_and_validation(native):
    s, _ = W.spheres_scene()
    info = s.validate()
    assert info.num_triangles == 12
    bad = vr.Scene()
    m = bad.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    bad.add_object(5, bad.add_analytic_surface(vr.Surfaces.sphere((0, 0, 0), 1.0)))
    bad.materials.append(bad.materials[0])
    with pytest.raises(vr.VoidrayError):
        bad.validate()   # object's material index out of range
    with pytest.raises(vr.VoidrayError):
        vr.Scene().add_analytic_surface(object())


def test_surface_index_quirk_covers_analytic_surfaces(oracle):
    """Surface s renders with objects[s].material for analytic surfaces too."""
    s = vr.Scene()
    a = s.add_material(vr.Materials.lambertian((1.0, 0.0, 0.0)))
    b = s.add_material(vr.Materials.lambertian((0.0, 1.0, 0.0)))
    s0 = s.add_analytic_surface(vr.Surfaces.sphere((0, 0, 0), 1.0))
    s1 = s.add_analytic_surface(vr.Surfaces.sphere((3, 0, 0), 1.0))
    s.add_object(b, s1)   # object 0 (for surface 1) ...
    s.add_object(a, s0)   # ... but surface 0 renders with objects[0].material = b
    assert s.surface_materials() == [b, a]


def test_textured_scene_lowers_and_checks_indices(native, oracle):
    s, st = W.textured_scene()
    assert s.validate().num_triangles == 4
    o, _ = oracle.OracleScene(s).render(st, 2, 24, 16)
    assert np.all(np.isfinite(o))
    bad, _ = W.textured_scene()
    bad.materials[0].albedo_texture = 7
    with pytest.raises(vr.VoidrayError):
        bad.validate()
    metal, _ = W.textured_scene()
    metal.materials[0].kind = 1   # only Lambertian takes textures
    with pytest.raises(vr.VoidrayError):
        metal.validate()
