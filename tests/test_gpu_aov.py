"""First-hit feature buffers (albedo, normal) rendered beside the radiance.

The AOV render must leave the radiance untouched (bit-identical to
vr_render_device) and the multi-scene batch must produce the same AOVs as a
render of the job alone.
"""
import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import workloads as W
from voidray_gb300.batch import Batch, RenderJob

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CORNELL_ALBEDOS = np.array([(0.63, 0.065, 0.05), (0.14, 0.45, 0.091), (0.725, 0.725, 0.725), (1.0, 1.0, 1.0)],
                           dtype=np.float32)


def zeros(w, h):
    return torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")


def render_aov(acc, st, spp, w, h, seed=0, first=0):
    rgba, alb, nrm = zeros(w, h), zeros(w, h), zeros(w, h)
    vr.render_device(acc, st, spp, rgba.data_ptr(), w, h, seed, first, 0, alb.data_ptr(), nrm.data_ptr())
    acc.synchronize()
    return rgba.cpu().numpy(), alb.cpu().numpy(), nrm.cpu().numpy()


def test_aov_radiance_unchanged_and_features_sane(gpu):
    scene, st = W.cornell_box(rr_depth=3)
    w, h, spp = 80, 64, 16
    acc = scene.build_acceleration()
    plain = zeros(w, h)
    vr.render_device(acc, st, spp, plain.data_ptr(), w, h, 3, 0)
    acc.synchronize()
    rgba, alb, nrm = render_aov(acc, st, spp, w, h, seed=3)
    assert np.array_equal(rgba, plain.cpu().numpy())
    assert np.all(alb[..., 3] == 1.0) and np.all(nrm[..., 3] == 1.0)
    assert np.all((alb[..., :3] >= 0.0) & (alb[..., :3] <= 1.0 + 1e-6))
    assert np.all(np.linalg.norm(nrm[..., :3], axis=-1) <= 1.0 + 1e-5)
    # pixels whose samples all hit one surface carry that surface's colour
    d = np.abs(alb[..., None, :3] - CORNELL_ALBEDOS[None, None]).max(-1).min(-1)
    assert np.mean(d < 1e-5) > 0.5
    # the top rows see the ceiling (or the light in it): normals face down, towards the camera rays
    top = nrm[1:4, w // 2 - 2:w // 2 + 2, :3].reshape(-1, 3)
    assert np.all(top[:, 1] < -0.5)


def test_aov_of_misses_is_clamped_environment(gpu):
    scene, st = W.cornell_box(rr_depth=0)
    scene.environment = vr.Environments.uniform((2.0, 0.5, 0.25))
    scene.camera = vr.Camera.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 60.0), (0.0, 1.0, 0.0), 0.3)
    acc = scene.build_acceleration()
    _, alb, nrm = render_aov(acc, st, 16, 32, 32)
    assert np.allclose(alb[..., :3], np.array([1.0, 0.5, 0.25], np.float32), rtol=1e-6)
    assert np.all(nrm[..., :3] == 0.0)


def test_aov_batch_matches_single(gpu):
    scene, st = W.cornell_box(rr_depth=3)
    acc = scene.build_acceleration()
    w, h, spp = 48, 40, 8
    ref = render_aov(acc, st, spp, w, h, seed=11, first=4)
    bufs = [zeros(w, h) for _ in range(6)]
    b = Batch(1 << 14)
    try:
        jobs = [RenderJob(acc, st, spp, bufs[0].data_ptr(), w, h, 11, 4, bufs[1].data_ptr(), bufs[2].data_ptr()),
                RenderJob(acc, st, spp, bufs[3].data_ptr(), w, h, 12, 0)]
        b.render(jobs)
        b.synchronize()
    finally:
        b.destroy()
    for got, want in zip(bufs[:3], ref):
        assert np.array_equal(got.cpu().numpy(), want)
    assert not bufs[4].any() and not bufs[5].any()


def test_aov_arguments_checked(gpu):
    scene, st = W.cornell_box()
    acc = scene.build_acceleration()
    a = zeros(8, 8)
    with pytest.raises(vr.VoidrayError):
        vr.render_device(acc, st, 1, a.data_ptr(), 8, 8, albedo_device=a.data_ptr())
    b = Batch(0)
    try:
        with pytest.raises(vr.VoidrayError):
            b.render([RenderJob(acc, st, 1, a.data_ptr(), 8, 8, 0, 0, a.data_ptr(), 0)])
    finally:
        b.destroy()
