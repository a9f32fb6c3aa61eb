"""The C-ABI library loads, exports every symbol the headers under include/ declare,
and its host-side logic (scene lowering, SAH BVH build, flattening) holds its
invariants.  No GPU: nothing here launches a kernel."""
import re
from pathlib import Path

import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(vr_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol(native):
    lib = native.lib()
    names = declared()
    assert len(HEADERS) == 3 and len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(native.EXPORTED)
    assert lib.vr_abi_version() == 4


def test_no_device_is_an_error_not_a_fallback(native):
    if native.lib().vr_device_available():
        pytest.skip("a CUDA device is present")
    scene, _ = W.cornell_box()
    with pytest.raises(native.VoidrayError) as e:
        scene.build_acceleration()
    assert e.value.status == 7


@pytest.mark.parametrize("n,leaf,bins", [(1, 0, 0), (2, 0, 0), (5, 0, 0), (1000, 0, 0), (20000, 0, 0),
                                         (20000, 8, 32), (5000, 1, 4)])
def test_bvh_invariants_soup(native, n, leaf, bins):
    info = W.soup_scene(n, seed=n).validate(bvh_max_leaf=leaf, bvh_bins=bins)
    assert info.num_triangles == n
    assert info.max_depth < 64
    assert 1 <= info.num_nodes <= 2 * n


def test_bvh_invariants_degenerate(native):
    # every triangle identical: centroids coincide, the builder falls back to median splits
    pos = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (4096, 1))
    s = vr.Scene()
    m = s.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    s.add_object(m, s.add_mesh(vr.Mesh(pos, np.arange(len(pos)))))
    info = s.validate()
    assert info.num_triangles == 4096 and info.max_depth < 64


def test_bvh_invariants_cornell_and_icosphere(native):
    scene, _ = W.cornell_box()
    assert scene.validate().num_triangles == 36
    v, t = W.geodesic_sphere(40)
    s = vr.Scene()
    m = s.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    s.add_object(m, s.add_mesh(vr.Mesh(v, t)))
    info = s.validate()
    assert info.num_triangles == 20 * 40 * 40


def test_descriptor_errors(native):
    s = vr.Scene()
    m = s.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    with pytest.raises(vr.VoidrayError):
        vr.Mesh(np.zeros((3, 3), np.float32), [0, 1, 3])
    # surface without an object at the same index (the reference panics)
    s.add_mesh(vr.Mesh(np.eye(3, dtype=np.float32), [0, 1, 2]))
    with pytest.raises(vr.VoidrayError):
        s.validate()
    s.add_object(m + 5, 0)
    with pytest.raises(vr.VoidrayError):
        s.validate()
    with pytest.raises(vr.VoidrayError) as e:
        s.add_analytic_surface(None)
    assert e.value.status == 2


def test_surface_index_quirk(native):
    """scene.rs:377: the hit surface index selects the object, so surface s
    renders with objects[s].material even if that object names another surface."""
    s = vr.Scene()
    a = s.add_material(vr.Materials.lambertian((1, 0, 0)))
    b = s.add_material(vr.Materials.lambertian((0, 1, 0)))
    s0 = s.add_mesh(vr.Mesh(np.eye(3, dtype=np.float32), [0, 1, 2]))
    s1 = s.add_mesh(vr.Mesh(np.eye(3, dtype=np.float32) * 2, [0, 1, 2]))
    s.add_object(b, s1)
    s.add_object(a, s0)
    assert s.surface_materials() == [b, a]


def test_camera_look_at_f32(native):
    cam = vr.Camera.look_at((1.0, 0.0, 10.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 0.5)
    assert cam.direction.dtype == np.float32
    assert abs(float(np.dot(cam.direction, cam.up))) < 1e-6
    assert np.isclose(np.linalg.norm(cam.direction), 1.0, atol=1e-6)


def test_settings_defaults_match_reference(native):
    st = vr.RenderSettings()
    assert (st.total_samples, st.update_frequency, st.render_mode, st.firefly_clamp, st.max_bounces) == \
           (100, 0.1, vr.RenderMode.Full, 3.0, 10)
    cm = vr.ColorManagementSettings()
    assert (cm.tonemap, cm.gamma, cm.exposure, cm.transparent) == (vr.Tonemap.NONE, 2.2, 0.0, True)


def test_tuning_knobs_roundtrip_and_validation(native):
    from voidray_gb300 import autotune as T

    before = T.get_tuning()
    try:
        T.set_tuning({"shade_block": 128, "shade_blocks_per_sm": 16, "raygen_block": 64})
        assert T.get_tuning() == {"shade_block": 128, "shade_blocks_per_sm": 16, "raygen_block": 64}
        for bad in ({"shade_block": 96, "shade_blocks_per_sm": 8, "raygen_block": 256},
                    {"shade_block": 256, "shade_blocks_per_sm": 0, "raygen_block": 256},
                    {"shade_block": 256, "shade_blocks_per_sm": 8, "raygen_block": 512}):
            with pytest.raises(native.VoidrayError):
                T.set_tuning(bad)
        assert T.get_tuning()["shade_block"] == 128
    finally:
        T.set_tuning(before)


def test_tuning_cache_keys(tmp_path, monkeypatch):
    from voidray_gb300 import autotune as T

    monkeypatch.setenv("VOIDRAY_TUNING_CACHE", str(tmp_path / "t.json"))
    k1 = T.bucket_key("GB300", 2_000_000, 1920 * 1080, 256, 1)
    assert k1 == T.bucket_key("GB300", 1_500_000, 1900 * 1080, 300, 1)   # same buckets
    assert k1 != T.bucket_key("GB300", 2_000_000, 1920 * 1080, 256, 0)
    T.save_cache({k1: {"wavefront_paths": 1 << 25}})
    assert T.load_cache()[k1]["wavefront_paths"] == 1 << 25


def test_descriptor_limits_and_edge_cases(native):
    """Host validation of the edge cases the scene descriptor can carry: more
    analytic surfaces than VR_MAX_ANALYTICS, an unknown material kind, empty
    or ill-formed textures, and a scene whose only mesh has no triangles."""
    base = vr.Materials.lambertian((0.5, 0.5, 0.5))
    s = vr.Scene()
    m = s.add_material(base)
    for k in range(65):
        s.add_object(m, s.add_analytic_surface(vr.Surfaces.sphere((k, 0, 0), 0.4)))
    with pytest.raises(vr.VoidrayError) as e:
        s.validate()
    assert e.value.status == 2
    s = vr.Scene()
    bad = vr.Materials.lambertian((0.5, 0.5, 0.5))
    bad.kind = 9
    s.add_object(s.add_material(bad), s.add_mesh(vr.Mesh(np.eye(3, dtype=np.float32), [0, 1, 2])))
    with pytest.raises(vr.VoidrayError) as e:
        s.validate()
    assert e.value.status == 2
    for tex in (np.zeros((0, 4, 3), np.float32), np.zeros((4, 4), np.float32)):
        with pytest.raises(vr.VoidrayError):
            vr.ImageTexture(tex)
    s = vr.Scene()
    t = s.add_texture(vr.ImageTexture(np.ones((2, 2, 3), np.float32)))
    s.textures[t].sample_type = 7
    s.add_object(s.add_material(vr.Materials.lambertian_texture_no_normal(t)),
                 s.add_mesh(vr.Mesh(np.eye(3, dtype=np.float32), [0, 1, 2])))
    with pytest.raises(vr.VoidrayError):
        s.validate()   # unknown sampling
    s = vr.Scene()
    s.add_object(s.add_material(base), s.add_mesh(vr.Mesh(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32))))
    assert s.validate().num_triangles == 0


def test_non_finite_and_extreme_vertices(native):
    """A NaN or infinite vertex position is rejected by name (the reference's
    BVH sorts such boxes arbitrarily); finite coordinates up to 3e38, whose
    extents overflow to infinity inside the SAH binning, still build a BVH
    that passes the structural checks."""
    rng = np.random.default_rng(4)
    base = vr.Materials.lambertian((0.5, 0.5, 0.5))
    for bad in (np.nan, np.inf, -np.inf):
        s = vr.Scene()
        pos = rng.random((30, 3)).astype(np.float32)
        pos[7, 1] = bad
        s.add_object(s.add_material(base), s.add_mesh(vr.Mesh(pos, np.arange(30, dtype=np.uint32))))
        with pytest.raises(vr.VoidrayError, match="non-finite position") as e:
            s.validate()
        assert e.value.status == 1
    s = vr.Scene()
    pos = rng.uniform(-1, 1, (300, 3)).astype(np.float32)
    pos[::7] *= np.float32(3e38)
    pos[1::11] = np.float32(-3e38)
    pos[2::13] = 0.0
    s.add_object(s.add_material(base), s.add_mesh(vr.Mesh(pos, np.arange(300, dtype=np.uint32))))
    for leaf, bins in ((0, 0), (1, 2), (8, 64)):
        info = s.validate(bvh_max_leaf=leaf, bvh_bins=bins)
        assert info.num_triangles == 100


def test_bvh_build_independent_of_thread_count(tmp_path):
    """The SAH build runs on several host threads (subtrees, and the bounds /
    binning passes of large ranges); the tree is the serial depth-first one
    whatever the thread count.  The SAH cost, summed over every node in flat
    order, fingerprints the structure."""
    import json
    import os
    import subprocess
    import sys

    code = ("import json, sys; sys.path.insert(0, %r)\n"
            "from voidray_gb300 import workloads as W\n"
            "out = []\n"
            "for n in (70_000, 300_000):\n"
            "    s = W.soup_scene(n, seed=n)\n"
            "    for leaf, bins in ((0, 0), (8, 64)):\n"
            "        i = s.validate(bvh_max_leaf=leaf, bvh_bins=bins)\n"
            "        out.append([i.num_nodes, i.max_depth, i.max_leaf, i.sah_cost])\n"
            "print(json.dumps(out))\n") % str(Path(__file__).resolve().parents[1])
    runs = []
    for threads in ("1", "3", "8"):
        env = dict(os.environ, VR_BUILD_THREADS=threads)
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        runs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert runs[0] == runs[1] == runs[2]


def test_first_bad_triangle_is_reported_with_parallel_lowering():
    """Large meshes are lowered in pieces on several threads; with bad vertices
    in several pieces the error names the one of the lowest triangle, as a
    serial pass would."""
    n = 200_000
    pos = np.random.default_rng(5).random((3 * n, 3)).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32)
    pos[3 * 150_000 + 1, 2] = np.nan   # triangle 150000
    pos[3 * 90_000 + 2, 0] = np.inf    # triangle 90000: the first bad one
    pos[3 * 180_000, 1] = np.nan
    base = vr.Materials.lambertian((0.5, 0.5, 0.5))
    s = vr.Scene()
    s.add_object(s.add_material(base), s.add_mesh(vr.Mesh(pos, idx)))
    with pytest.raises(vr.VoidrayError, match=f"vertex {3 * 90_000 + 2} has a non-finite position"):
        s.validate()


def test_scene_acceleration_ref_accessors(native):
    """SceneAcceleration's surface_ref / material_ref / texture_ref / mesh_ref /
    object_ref (scene.rs:207-225) over the lists copied at build time; host only."""
    s = vr.Scene()
    m0 = s.add_material(vr.Materials.lambertian((0.5, 0.5, 0.5)))
    t0 = s.add_texture(vr.ImageTexture(np.ones((2, 2, 3), np.float32)))
    m1 = s.add_material(vr.Materials.lambertian_texture_no_normal(t0))
    mesh = vr.Mesh(np.eye(3, dtype=np.float32), [0, 1, 2])
    s0 = s.add_mesh(mesh)
    s1 = s.add_analytic_surface(vr.Surfaces.sphere((0, 0, 0), 1.0))
    o0 = s.add_object(m0, s0)
    o1 = s.add_object(m1, s1)
    acc = vr.SceneAcceleration.__new__(vr.SceneAcceleration)  # no vr_scene_create: the accessors need no device
    acc._h = None
    acc._keep_lists(s)
    s.add_material(vr.Materials.metal((1, 1, 1), 0.1))  # later edits of the scene do not reach the copies
    assert len(acc._materials) == 2
    assert acc.surface_ref(s0) is mesh and acc.mesh_ref(0) is mesh
    assert isinstance(acc.surface_ref(s1), vr.AnalyticSurface)
    assert acc.material_ref(m1) is s.materials[m1] and acc.texture_ref(t0) is s.textures[t0]
    assert acc.object_ref(o1).surface == s1 and acc.object_ref(o0).material == m0
