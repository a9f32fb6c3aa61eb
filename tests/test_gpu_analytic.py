"""Analytic surfaces on the GPU against the oracle: closest and any hit on
ray batches, and renders with spheres and a ground plane (the arithmetic of
Sphere::hit / GroundPlane::hit is reproduced in the same operation order, so
hits and pixels match exactly up to the usual last-ulp transcendental cases)."""
import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W
from voidray_gb300.scene import Estimator, RenderSettings

from test_gpu_render import close_fraction, exact_fraction, gpu_render, relmse

pytestmark = pytest.mark.gpu
MISS = 0xFFFFFFFF


def scene_rays(n, seed=7):
    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-3, 3, (n, 3)) + np.array([0, 1.0, 2.0])
    d = rng.standard_normal((n, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 1e-5
    rays[:, 7] = np.inf
    return rays


@pytest.mark.parametrize("any_hit", [False, True])
def test_analytic_intersection_matches_oracle(gpu, oracle, any_hit):
    s, _ = W.spheres_scene()
    acc = s.build_acceleration()
    rays = scene_rays(200000)
    g = acc.hit(rays, any_hit=any_hit)
    o = oracle.OracleScene(s).intersect(rays, mode=2 if any_hit else 0)
    gp, op = g[:, 0].view(np.uint32), o[:, 0].view(np.uint32)
    if any_hit:
        assert np.array_equal(gp == MISS, op == MISS)
        return
    assert np.mean(gp == op) > 0.9999
    ana = (gp == op) & (gp != MISS) & (gp >= 12)
    assert ana.sum() > 1000                       # plenty of sphere / plane hits
    assert np.array_equal(g[ana, 1], o[ana, 1])   # t bit-identical


@pytest.mark.parametrize("rr", [0, 3])
def test_spheres_render_bit_parity(gpu, oracle, rr):
    s, st = W.spheres_scene()
    st = RenderSettings(**{**st.__dict__, "rr_depth": rr})
    g = gpu_render(s, st, 8, 64, 48)
    o, _ = oracle.OracleScene(s).render(st, 8, 64, 48)
    assert exact_fraction(g, o) >= 0.99
    assert relmse(g, o) < 1e-4


def test_spheres_nee_hdri(gpu, oracle):
    s, st = W.spheres_scene(hdri=True)
    st = RenderSettings(**{**st.__dict__, "estimator": Estimator.NEE, "rr_depth": 3})
    g = gpu_render(s, st, 8, 64, 48)
    o, _ = oracle.OracleScene(s).render(st, 8, 64, 48)
    assert close_fraction(g, o) >= 0.95
    assert relmse(g, o) < 1e-3


@pytest.mark.parametrize("rr", [0, 3])
def test_textured_render_bit_parity(gpu, oracle, rr):
    """Image textures (nearest and bilinear, uvs outside [0, 1]), a normal map
    and a textured ground plane, against the oracle's texture.rs restatement."""
    s, st = W.textured_scene()
    st = RenderSettings(**{**st.__dict__, "rr_depth": rr})
    g = gpu_render(s, st, 8, 64, 48)
    o, _ = oracle.OracleScene(s).render(st, 8, 64, 48)
    assert exact_fraction(g, o) >= 0.99
    assert relmse(g, o) < 1e-4


def test_textured_nee_matches_reference_estimator_in_expectation(gpu):
    """NEE skips the normal-mapped vertices (their scatter is not cosine
    distributed); both estimators converge to the same image."""
    s, st = W.textured_scene()
    ref = gpu_render(s, st, 512, 32, 24, seed=1)
    nee = gpu_render(s, RenderSettings(**{**st.__dict__, "estimator": Estimator.NEE, "rr_depth": 3}), 512, 32, 24,
                     seed=2)
    assert relmse(nee, ref) < 5e-3
