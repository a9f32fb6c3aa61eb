"""Queue conservation of the wavefront: every camera path is retired exactly
once (by a miss, an emitter, absorption, Russian roulette or the depth
limit), across wavefront splits, estimators and scenes."""
import ctypes as C

import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import _native as N
from voidray_gb300 import workloads as W
from voidray_gb300.scene import Estimator, RenderSettings

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("estimator,rr,wave", [(Estimator.REFERENCE, 0, 0), (Estimator.REFERENCE, 3, 777),
                                              (Estimator.NEE, 3, 0), (Estimator.NEE, 2, 5000)])
def test_every_path_retired_once(gpu, estimator, rr, wave):
    scene, st = W.cornell_box(rr_depth=rr)
    scene.environment = vr.Environments.hdri_image(W.sky_hdri(64, 32, peak=30.0, sigma_deg=5.0))
    st = RenderSettings(**{**st.__dict__, "estimator": estimator, "wavefront_paths": wave})
    acc = scene.build_acceleration()
    N.check(vr.lib().vr_scene_instrument(acc.handle, N.INSTR_WORK))
    before = acc.stats()
    w, h, spp = 48, 40, 6
    t = vr.CpuRenderTarget(w, h)
    vr.iterative_render(t, acc, st, spp, seed=3)
    ins = N.vr_instrument()
    N.check(vr.lib().vr_scene_instrument_get(acc.handle, C.byref(ins)))
    after = acc.stats()
    paths = after.paths - before.paths
    assert paths == w * h * spp
    assert ins.retired_paths == paths
    assert np.all(np.isfinite(t.buffer))


def test_metal_fallbacks_are_counted(gpu):
    """Metal::scatter resamples until the direction is above the surface
    (simple.rs:140-161).  On a Surfaces::quad, whose vertex normals are zero
    (the kept quirk), that never happens: the reference would loop forever,
    the GPU absorbs the path after 64 tries and counts it.  With real normals
    the loop always ends early and nothing is counted."""
    def run(zero_normals):
        s = vr.Scene()
        m = s.add_material(vr.Materials.metal((0.9, 0.9, 0.9), 0.3))
        q = [(-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)]
        if zero_normals:
            mesh = vr.Surfaces.quad(*q)
        else:
            mesh = vr.Mesh(np.array(q, np.float32), [0, 1, 2, 2, 0, 3], np.array([(0, 0, 1)] * 4, np.float32))
        s.add_object(m, s.add_mesh(mesh))
        s.environment = vr.Environments.uniform((0.5, 0.6, 0.7))
        s.camera = vr.Camera.look_at((0, 0, 3), (0, 0, -1), (0, 1, 0), vr.degrees_to_radians(30.0))
        acc = s.build_acceleration()
        N.check(vr.lib().vr_scene_instrument(acc.handle, N.INSTR_WORK))
        st = RenderSettings(total_samples=2, max_bounces=4, firefly_clamp=float("inf"))
        t = vr.CpuRenderTarget(16, 16)
        vr.iterative_render(t, acc, st, 2, seed=1)
        ins = N.vr_instrument()
        N.check(vr.lib().vr_scene_instrument_get(acc.handle, C.byref(ins)))
        return ins.metal_fallbacks, ins.retired_paths, t.buffer

    n0, paths0, img0 = run(True)
    n1, paths1, img1 = run(False)
    assert paths0 == paths1 == 16 * 16 * 2
    assert n0 == paths0           # every camera path hits the quad (fov 30, quad fills the view)
    assert np.all(img0[..., :3] == 0.0)
    assert n1 == 0 and img1[..., :3].mean() > 0.1
