"""What the trained denoiser gains over the plain progressive render, with
the shipped weights, on scenes of the training family that the training set
did not contain (other geometry, material and sun seeds, other cameras):

* at equal samples, the denoised frame's relMSE against a 1024-spp
  reference is well below the plain frame's at low sample counts;
* the acceptance rule: at equal time (the plain frame gets the samples that
  fit in the time of the AOV render plus the denoiser) the denoised frame
  still wins.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _relmse(x, r):
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


@pytest.fixture(scope="module")
def held_out(gpu):
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.denoise import Denoiser
    from voidray_gb300.scene import Estimator, RenderSettings

    s, _ = W.displaced_icosphere_scene(freq=60, seed=424242, hdri_size=None)
    s.environment = vr.Environments.hdri_image(W.sky_hdri(512, 256, 28.0, 130.0))
    s.camera = vr.Camera.look_at((2.6, 0.9, 2.2), (0.0, -0.1, 0.0), (0.0, 1.0, 0.0), vr.degrees_to_radians(45.0))
    acc = s.build_acceleration()
    st = RenderSettings(total_samples=1, max_bounces=8, rr_depth=3, estimator=Estimator.NEE, firefly_clamp=3.0)
    size = 128
    ref = torch.zeros((size, size, 4), device="cuda")
    vr.render_device(acc, st, 1024, ref.data_ptr(), size, size, seed=99)
    acc.synchronize()
    net = Denoiser.pretrained()
    yield acc, st, size, (ref[..., :3].double() / 1024).cpu().numpy(), net
    net.destroy()
    acc.destroy()


def _aov_render(vr, acc, st, spp, size, seed):
    bufs = [torch.zeros((size, size, 4), device="cuda") for _ in range(3)]
    vr.render_device(acc, st, spp, bufs[0].data_ptr(), size, size, seed=seed, albedo_device=bufs[1].data_ptr(),
                     normal_device=bufs[2].data_ptr())
    acc.synchronize()
    return bufs


@pytest.mark.parametrize("spp,factor", [(4, 0.35), (16, 0.5)])
def test_denoised_beats_plain_at_equal_samples(held_out, spp, factor):
    import voidray_gb300 as vr

    acc, st, size, ref, net = held_out
    rad, alb, nrm = _aov_render(vr, acc, st, spp, size, seed=3)
    out = torch.zeros_like(rad)
    net.denoise(rad, alb, nrm, 1.0 / spp, out, size, size)
    torch.cuda.synchronize()
    e_plain = _relmse((rad[..., :3].double() / spp).cpu().numpy(), ref)
    e_dn = _relmse(out[..., :3].double().cpu().numpy(), ref)
    assert e_dn < factor * e_plain, (e_dn, e_plain)


def test_denoised_beats_plain_at_equal_time(held_out):
    import voidray_gb300 as vr

    acc, st, size, ref, net = held_out
    spp = 8
    _aov_render(vr, acc, st, 1, size, seed=1)  # warm-up: scratch and workspace
    s = torch.cuda.Stream()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    bufs = [torch.zeros((size, size, 4), device="cuda") for _ in range(4)]
    net.denoise(bufs[0], bufs[1], bufs[2], 1.0, bufs[3], size, size, stream=s.cuda_stream)
    with torch.cuda.stream(s):
        for b in bufs:
            b.zero_()
        e0.record(s)
        vr.render_device(acc, st, spp, bufs[0].data_ptr(), size, size, seed=5, stream=s.cuda_stream,
                         albedo_device=bufs[1].data_ptr(), normal_device=bufs[2].data_ptr())
        net.denoise(bufs[0], bufs[1], bufs[2], 1.0 / spp, bufs[3], size, size, stream=s.cuda_stream)
        e1.record(s)
    e1.synchronize()
    t_dn = e0.elapsed_time(e1)
    plain = torch.zeros((size, size, 4), device="cuda")
    with torch.cuda.stream(s):
        e1.record(s)
        vr.render_device(acc, st, spp, plain.data_ptr(), size, size, seed=6, stream=s.cuda_stream)
        e2.record(s)
    e2.synchronize()
    t_plain = e1.elapsed_time(e2)
    spp_eq = max(spp, int(spp * t_dn / t_plain))
    plain.zero_()
    vr.render_device(acc, st, spp_eq, plain.data_ptr(), size, size, seed=6)
    acc.synchronize()
    e_dn = _relmse(bufs[3][..., :3].double().cpu().numpy(), ref)
    e_plain = _relmse((plain[..., :3].double() / spp_eq).cpu().numpy(), ref)
    assert e_dn < e_plain, (e_dn, e_plain, spp_eq, t_dn, t_plain)
