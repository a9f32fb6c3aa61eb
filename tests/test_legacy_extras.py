"""The legacy crate's extras: MixMaterial (voidray/src/common/materials.rs:
188-203) in the oracle and the library's material table, and the legacy
viewport's tonemaps (voidray/src/shaders/viewport_fragment.glsl:27-67)
against an FP64 golden.  GPU parity for both is in test_gpu_legacy_extras.py."""
from pathlib import Path

import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W

GOLDEN = Path(__file__).parent / "golden"


def furnace_scene(material):
    v, t = W.geodesic_sphere(5)
    corners = v[t].astype(np.float32)
    fn = np.cross(corners[:, 1] - corners[:, 0], corners[:, 2] - corners[:, 0])
    fn = (fn / np.linalg.norm(fn, axis=1, keepdims=True)).astype(np.float32)
    s = vr.Scene()
    m = s.add_material(material)
    s.add_object(m, s.add_mesh(vr.Mesh(corners.reshape(-1, 3), np.arange(corners.size // 3), np.repeat(fn, 3, 0))))
    s.environment = vr.Environments.uniform((1.0, 1.0, 1.0))
    s.camera = vr.Camera.look_at((0, 0, 3), (0, 0, 0), (0, 1, 0), vr.degrees_to_radians(30.0))
    return s, vr.RenderSettings(total_samples=1, max_bounces=5, firefly_clamp=float("inf"))


def test_mix_picks_children_with_the_factor(oracle):
    """Furnace: a flat-shaded convex sphere under a uniform environment of 1
    returns the albedo of the child that shaded the hit, so the share of each
    albedo among hit pixels estimates the mixing probabilities:
    u >= factor -> first."""
    a, b, c = (vr.Materials.lambertian((x, x, x)) for x in (0.2, 0.5, 0.8))
    s, st = furnace_scene(vr.Materials.mix(vr.Materials.mix(a, b, 0.5), c, 0.25))
    img, _ = oracle.OracleScene(s).render(st, 1, 96, 96)
    r = img[..., 0].ravel()
    vals = [np.float32(x) for x in (0.2, 0.5, 0.8)]
    # a rare grazing path that stays on the faceted sphere returns something else
    assert np.mean(~np.isin(r, vals + [np.float32(1.0)])) < 1e-3
    hit = np.isin(r, vals)
    n = hit.sum()
    assert n > 3000
    share = [float((r[hit] == x).mean()) for x in vals]
    for got, want in zip(share, [0.375, 0.375, 0.25]):
        assert abs(got - want) < 4 * np.sqrt(want * (1 - want) / n) + 1e-3, share


def test_mix_factor_extremes(oracle):
    """u is in [0, 1): factor 0 always takes the first child, factor 1 the second."""
    a, b = vr.Materials.lambertian((0.3, 0.3, 0.3)), vr.Materials.lambertian((0.7, 0.7, 0.7))
    for f, want in ((0.0, 0.3), (1.0, 0.7)):
        s, st = furnace_scene(vr.Materials.mix(a, b, f))
        r = oracle.OracleScene(s).render(st, 1, 32, 32)[0][..., 0]
        other = np.float32(0.7) if want == 0.3 else np.float32(0.3)
        assert not np.any(r == other) and np.mean(r == np.float32(want)) > 0.5


def test_material_table_flattens_mixes(native):
    s, _ = W.mix_scene()
    flat = s.flat_materials()
    # scene materials keep their handles; children follow, shared objects once
    assert [m.kind for m, _, _ in flat[:4]] == [6, 6, 6, 0]
    m0, m1, m2 = flat[0], flat[1], flat[2]
    assert flat[m0[1]][0].kind == 0 and flat[m0[2]][0].kind == 1
    inner = flat[m1[1]]
    assert inner[0].kind == 6 and flat[inner[1]][0].kind == 2 and inner[2] == m0[1]  # red is shared
    assert m2[1] == m2[2] == m0[2]   # gold is shared
    assert len(flat) == 4 + 5        # red, gold, inner mix, glass, lamp
    assert s.to_c()[0].num_materials == len(flat)
    s.validate()


def test_mix_depth_and_cycles_are_rejected(native):
    base = vr.Materials.lambertian((0.5, 0.5, 0.5))
    m = base
    for _ in range(8):
        m = vr.Materials.mix(m, base, 0.5)
    s, _ = furnace_scene(m)
    s.validate()                       # eight levels are allowed
    s, _ = furnace_scene(vr.Materials.mix(m, base, 0.5))
    with pytest.raises(vr.VoidrayError):
        s.validate()                   # nine are not
    a = vr.Materials.mix(base, base, 0.5)
    b = vr.Materials.mix(a, base, 0.5)
    a.first = b                        # a cycle, built by mutation
    s, _ = furnace_scene(b)
    with pytest.raises(vr.VoidrayError, match="cyclic"):
        s.validate()
    with pytest.raises(vr.VoidrayError):
        vr.Materials.mix(base, 3, 0.5)


def test_oracle_renders_mix_scene(oracle):
    s, st = W.mix_scene()
    img, _ = oracle.OracleScene(s).render(st, 2, 32, 24)
    assert np.all(np.isfinite(img)) and img[..., :3].mean() > 0.05


def test_legacy_tonemap_against_f64_golden(oracle):
    g = np.load(GOLDEN / "tonemap_legacy_f64.npz")
    x = g["input"]
    for tm in range(8):
        got = oracle.tonemap_legacy(x, tm, float(g["gamma"]), float(g["exposure"]), True, float(g["scale"]))
        ref = g[f"out_{tm}"]
        ok = np.isfinite(ref)
        big = ok & (np.abs(ref) > 1e-2)
        small = ok & ~big
        assert np.array_equal(np.isfinite(got), ok), tm
        assert np.allclose(got[big], ref[big], rtol=3e-5, atol=0), tm
        assert np.allclose(got[small], ref[small], rtol=0, atol=1e-3), tm
        opaque = oracle.tonemap_legacy(x, tm, float(g["gamma"]), float(g["exposure"]), False, float(g["scale"]))
        assert np.all(opaque[:, 3] == 1.0)


def test_legacy_enum_numbering():
    assert [t.value for t in vr.LegacyTonemap] == list(range(8))
    assert vr.LegacyTonemap.Filmic == 6 and vr.LegacyTonemap.RomBinDaHouse == 5
