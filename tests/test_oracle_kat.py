"""Known-answer tests pinning the CPU oracle (no GPU).

The reference ships no golden vectors for this path, so the oracle is pinned
on: the published PCG32 demo output, hand-computed Moller-Trumbore cases
(including the reference's absolute 1e-5 determinant epsilon and its
t > t_min rule), the slab test's edge cases, brute force vs the reference's
median BVH traversal, the sampler distributions, an FP64 numpy restatement of
tonemapping.glsl (tests/golden/tonemap_f64.npz, made by
tests/golden/make_golden.py), and an exact furnace identity.
"""
from pathlib import Path

import numpy as np
import pytest

from voidray_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_pcg32_published_vector(oracle):
    # pcg32-demo: pcg32_srandom_r(&rng, 42, 54) -> first six outputs
    out = oracle.pcg32(42, 0, 54, 6)
    assert list(out) == [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]


def test_sampler_distributions(oracle):
    n = 200000
    s = oracle.sampler(7, 3, 11, 0, n)
    assert np.allclose(np.linalg.norm(s, axis=1), 1.0, atol=1e-6)
    assert np.allclose(s.mean(0), 0.0, atol=0.01)
    assert np.allclose((s ** 2).mean(0), 1.0 / 3.0, atol=0.01)
    d = oracle.sampler(7, 3, 12, 1, n)[:, :2]
    assert (np.linalg.norm(d, axis=1) <= 1.0 + 1e-6).all()
    assert abs((np.linalg.norm(d, axis=1) < 0.5).mean() - 0.25) < 0.01
    c = oracle.sampler(7, 3, 13, 2, n)[:, :2]
    assert np.allclose(np.linalg.norm(c, axis=1), 1.0, atol=1e-5)
    u = oracle.sampler(7, 3, 14, 3, n)[:, 0]
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.005


def _one_triangle(p0, p1, p2):
    from voidray_gb300 import Materials, Mesh, Scene

    s = Scene()
    m = s.add_material(Materials.lambertian((0.5, 0.5, 0.5)))
    s.add_object(m, s.add_mesh(Mesh(np.array([p0, p1, p2], np.float32), [0, 1, 2])))
    return s


def _ray(o, d, tmin=1e-5, tmax=np.inf):
    return np.array([*o, tmin, *d, tmax], np.float32)


def test_triangle_known_answers(oracle):
    osc = oracle.OracleScene(_one_triangle((0, 0, 0), (1, 0, 0), (0, 1, 0)))
    # straight down the z axis onto (0.25, 0.5): t = 2, u weights v1, v weights v2
    t, u, v = osc.triangle_hit(0, _ray((0.25, 0.5, 2.0), (0, 0, -1)))
    assert (t, u, v) == (2.0, 0.25, 0.5)
    # edge and vertex hits are inside (u >= 0, v >= 0, u + v <= 1)
    assert osc.triangle_hit(0, _ray((0.5, 0.5, 1.0), (0, 0, -1)))[0] == 1.0
    assert osc.triangle_hit(0, _ray((0.0, 0.0, 1.0), (0, 0, -1))) is not None
    # outside
    assert osc.triangle_hit(0, _ray((0.6, 0.6, 1.0), (0, 0, -1))) is None
    assert osc.triangle_hit(0, _ray((-0.1, 0.5, 1.0), (0, 0, -1))) is None
    # behind the origin / at t <= tmin is rejected
    assert osc.triangle_hit(0, _ray((0.25, 0.25, -1.0), (0, 0, -1))) is None
    assert osc.triangle_hit(0, _ray((0.25, 0.25, 0.0), (0, 0, -1))) is None
    # parallel ray: |det| < tmin
    assert osc.triangle_hit(0, _ray((0.25, 0.25, 1.0), (1, 0, 0))) is None


def test_absolute_determinant_epsilon(oracle):
    """Triangle::hit rejects |det| < t_min (1e-5) however far the triangle is
    from the origin: a triangle with edges 1e-3 seen head-on has det = 1e-6."""
    osc = oracle.OracleScene(_one_triangle((0, 0, 0), (1e-3, 0, 0), (0, 1e-3, 0)))
    assert osc.triangle_hit(0, _ray((2e-4, 2e-4, 1.0), (0, 0, -1))) is None
    big = oracle.OracleScene(_one_triangle((0, 0, 0), (1e-2, 0, 0), (0, 1e-2, 0)))
    assert big.triangle_hit(0, _ray((2e-3, 2e-3, 1.0), (0, 0, -1))) is not None


def test_aabb_slab_edge_cases(oracle):
    box_min, box_max = np.zeros(3, np.float32), np.ones(3, np.float32)
    assert oracle.aabb_hit(box_min, box_max, _ray((0.5, 0.5, -1), (0, 0, 1)), 1e-5, np.inf)
    # axis-parallel ray outside the slab: 1/0 = inf gives (+-inf) bounds
    assert not oracle.aabb_hit(box_min, box_max, _ray((2.0, 0.5, -1), (0, 0, 1)), 1e-5, np.inf)
    # ray pointing away
    assert not oracle.aabb_hit(box_min, box_max, _ray((0.5, 0.5, -1), (0, 0, -1)), 1e-5, np.inf)
    # the default (empty) box always hits (aabb.rs:88-90)
    inf = np.float32(np.inf)
    assert oracle.aabb_hit(np.full(3, inf), np.full(3, -inf), _ray((5, 5, 5), (0, 0, 1)), 1e-5, np.inf)
    # zero-thickness box: t_max <= t_min rejects a ray hitting it head on
    flat_max = np.array([1, 1, 0], np.float32)
    assert not oracle.aabb_hit(box_min, flat_max, _ray((0.5, 0.5, 1), (0, 0, -1)), 1e-5, np.inf)


@pytest.mark.parametrize("n", [1, 4, 5, 37, 3000])
def test_median_bvh_equals_brute_force(oracle, n):
    scene = W.soup_scene(n, seed=n)
    rays = W.soup_rays(3000, 40, 40, seed=n)
    osc = oracle.OracleScene(scene)
    a, sa = osc.intersect(rays, mode=0, second=True)
    b, sb = osc.intersect(rays, mode=1, second=True)
    ia, ib = a[:, 0].view(np.uint32), b[:, 0].view(np.uint32)
    with np.errstate(invalid="ignore"):
        tie = np.isfinite(sb) & (sb - b[:, 1] <= 1e-6 * np.abs(b[:, 1]))
    assert np.all((ia == ib) | tie)
    same = ia == ib
    assert np.array_equal(a[same, 1:], b[same, 1:], equal_nan=True)


def test_tonemap_against_f64_golden(oracle):
    g = np.load(GOLDEN / "tonemap_f64.npz")
    x = g["input"]
    for tm in range(5):
        got = oracle.tonemap(x, tm, float(g["gamma"]), float(g["exposure"]), float(g["scale"]))
        ref = g[f"out_{tm}"]
        ok = np.isfinite(ref)
        big = ok & (np.abs(ref) > 1e-2)
        small = ok & ~big
        # f32 cancellation near zero (Uncharted2's f(0) - E/F) is amplified by pow(1/gamma)
        assert np.allclose(got[big], ref[big], rtol=3e-5, atol=0), tm
        assert np.allclose(got[small], ref[small], rtol=0, atol=1e-3), tm


def test_furnace_identity(oracle):
    """Convex flat-shaded sphere, uniform environment 1, albedo a: each path
    returns a (one bounce then escape) or 1 (miss)."""
    from voidray_gb300 import Camera, Environments, Materials, Mesh, RenderSettings, Scene, degrees_to_radians

    v, t = W.geodesic_sphere(5)
    corners = v[t].astype(np.float32)
    fn = np.cross(corners[:, 1] - corners[:, 0], corners[:, 2] - corners[:, 0])
    fn = (fn / np.linalg.norm(fn, axis=1, keepdims=True)).astype(np.float32)
    s = Scene()
    m = s.add_material(Materials.lambertian((0.6, 0.6, 0.6)))
    s.add_object(m, s.add_mesh(Mesh(corners.reshape(-1, 3), np.arange(corners.size // 3), np.repeat(fn, 3, 0))))
    s.environment = Environments.uniform((1.0, 1.0, 1.0))
    s.camera = Camera.look_at((0, 0, 3), (0, 0, 0), (0, 1, 0), degrees_to_radians(30.0))
    st = RenderSettings(total_samples=1, max_bounces=5, firefly_clamp=float("inf"))
    img, _ = oracle.OracleScene(s).render(st, 1, 32, 32)
    r = img[..., 0]
    assert np.all((r == np.float32(0.6)) | (r == np.float32(1.0))), np.unique(r)
    assert (r == np.float32(0.6)).mean() > 0.5


def test_cornell_energy_sanity(oracle):
    scene, st = W.cornell_box(rr_depth=0)
    img, rays = oracle.OracleScene(scene).render(st, 4, 32, 32)
    assert rays[0] > 32 * 32 * 4
    assert np.all(img[..., 3] == 1.0)
    assert 0.01 < img[..., :3].mean() < 3.0


# HDRIEnvironment::sample (voidray_common/src/environments.rs:57-90) with
# to_spherical_coords (voidray_renderer/src/util/math.rs:24-29) and lerp
# (math.rs:41-46), restated in numpy float32 in the reference's operation
# order; transcendental calls rounded from float64.
def _env_lookup_f32(img, d):
    f = np.float32
    h, w = img.shape[:2]
    flat = img.reshape(-1, 3)
    n_pix = len(flat)
    d = np.asarray(d, f)
    m2 = f(f(d[0] * d[0]) + f(d[1] * d[1])) + f(d[2] * d[2])
    inv = f(1.0) / f(np.sqrt(m2))
    n = d * inv
    sx = f(np.arccos(np.float64(-n[1])))
    sy = f(f(np.arctan2(np.float64(-n[2]), np.float64(n[0]))) + f(np.pi))
    u = sx / f(np.pi)
    v = sy / f(f(2.0) * f(np.pi))
    x = v * f(w)
    y = f(h - 1) - u * f(h)

    def usize(t):  # Rust `as usize`: NaN and negatives saturate to 0
        return 0 if not t > 0 else int(t)

    x0 = min(usize(x), w - 1)
    y0 = min(usize(y), h - 1)
    ax = x - f(x0)
    ay = y - f(y0)

    def lerp(a, b, t):
        return a * (f(1.0) - t) + b * t

    px = lambda i: flat[i % n_pix]
    top = lerp(px(y0 * w + x0), px(y0 * w + x0 + 1), ax)
    bot = lerp(px((y0 + 1) * w + x0), px((y0 + 1) * w + x0 + 1), ax)
    return lerp(top, bot, ay), (x0, y0, float(ax), float(ay))


ENV_DIRS = [
    (0.0, -1.0, 0.0),     # bottom pole: y0 = H-1, the next row wraps to row 0 (weight 0)
    (0.0, 1.0, 0.0),      # top pole: y = -1 saturates to row 0, ay = -1 extrapolates
    (-1.0, 0.0, 0.0),     # seam with -0.0 = -d.z: atan2(-0, -1) = -pi, x = 0
    (-1.0, 0.0, -0.0),    # seam with +0.0: atan2(+0, -1) = +pi, x = W, x0 = W-1, ax = 1
    (-1.0, 0.0, 1e-7), (-1.0, 0.0, -1e-7), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, -1.0),
    (1e-6, -1.0, 0.0), (1e-6, 1.0, -1e-6), (0.3, -0.9, 0.2), (-0.5, 0.5, -0.5),
]


def test_hdri_lookup_at_poles_and_seams(oracle):
    """The oracle's environment lookup against the float32 restatement, on
    the directions where the reference's quirks show (poles, the phi seam
    with either zero sign) and a few ordinary ones."""
    from voidray_gb300 import Camera, Environments, Scene

    rng = np.random.default_rng(8)
    img = rng.uniform(0.0, 4.0, (9, 16, 3)).astype(np.float32)
    s = Scene()
    s.environment = Environments.hdri_image(img)
    s.camera = Camera.look_at((0, 0, 1), (0, 0, 0), (0, 1, 0), 1.0)
    o = oracle.OracleScene(s)
    seen = set()
    for d in ENV_DIRS:
        want, (x0, y0, ax, ay) = _env_lookup_f32(img, d)
        got = o.env_eval(np.array(d, np.float32))
        assert np.allclose(got, want, rtol=1e-5, atol=1e-6), (d, got, want, x0, y0, ax, ay)
        seen.add((x0, y0, ax, ay))
    # the quirks are exercised: top-pole extrapolation and the x0 = W-1, ax = 1 seam
    assert any(ay < 0 for *_, ay in seen) and any(x0 == 15 and ax == 1.0 for x0, _, ax, _ in seen)


def test_zero_sample_call_adds_only_alpha(oracle):
    """iterative.rs:37-50 with samples = 0: rgb += 0, alpha += Color::a() = 1."""
    scene, st = W.cornell_box()
    start = np.random.default_rng(2).uniform(0, 1, (6, 5, 4)).astype(np.float32)
    o, rays = oracle.OracleScene(scene).render(st, 0, 5, 6, rgba=start.copy())
    assert np.array_equal(o[..., :3], start[..., :3]) and np.all(o[..., 3] == start[..., 3] + 1)
    assert rays[0] == 0
