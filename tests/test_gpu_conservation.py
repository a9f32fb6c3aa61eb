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
