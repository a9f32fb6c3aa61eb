"""Served jobs on the GPU: a job's image and stopping point are the same alone
and in a mix (bit-identical), and the served image matches a plain render of
the same samples."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes(vr, W):
    from voidray_gb300.scene import Estimator, RenderSettings

    s1, st1 = W.cornell_box(rr_depth=3)
    s2 = vr.Scene()
    v, t = W.geodesic_sphere(10)
    m = s2.add_material(vr.Materials.lambertian((0.6, 0.5, 0.4)))
    s2.add_object(m, s2.add_mesh(vr.Mesh(v.astype(np.float32), t.astype(np.uint32), v.astype(np.float32))))
    s2.environment = vr.Environments.hdri_image(W.sky_hdri(64, 32, peak=40.0, sigma_deg=6.0))
    s2.camera = vr.Camera.look_at((0, 0.4, 3.0), (0, 0, 0), (0, 1, 0), vr.degrees_to_radians(40.0))
    st2 = RenderSettings(total_samples=1, max_bounces=6, rr_depth=2, estimator=Estimator.NEE,
                         firefly_clamp=float("inf"))
    return [(s1.build_acceleration(), st1), (s2.build_acceleration(), st2)]


def test_served_same_alone_and_in_mix(gpu):
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig

    scenes = _scenes(vr, W)
    cfg = ServerConfig(spp_per_pass=8, min_samples=16)

    def run(mix):
        srv = Server(GpuBackend(), cfg)
        acc, st = scenes[1]
        jid = srv.submit(JobRequest(acc, st, 40, 32, max_samples=256, target_relmse=2e-2, seed=5))
        for k in range(mix):
            a2, s2 = scenes[k % 2]
            srv.submit(JobRequest(a2, s2, 24 + 8 * k, 16, max_samples=64, target_relmse=1e-4, seed=10 + k))
        while not srv.idle():
            srv.step()
        j = srv.status(jid)
        return j.result, j.samples, j.n_a, j.n_b

    r0 = run(0)
    r1 = run(4)
    assert r0[1:] == r1[1:]
    assert np.array_equal(r0[0], r1[0])
    assert r0[1] < 256  # stopped on the error estimate


@pytest.mark.parametrize("adaptive,pipelined", [(False, False), (True, False), (True, True)])
def test_denoised_serving_same_alone_and_in_mix(gpu, adaptive, pipelined):
    """With the denoiser in the loop (AOV buffers, blended output) a job's
    stopping point, blend weight and image still depend only on the job."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.denoise import Denoiser
    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig

    scenes = _scenes(vr, W)
    cfg = ServerConfig(spp_per_pass=8, min_samples=16, adaptive=adaptive, pipelined=pipelined,
                       pass_paths=40 * 32 * 16, first_pass_spp=16)
    net = Denoiser.pretrained()

    def run(mix):
        backend = GpuBackend(denoiser=net)
        srv = Server(backend, cfg)
        acc, st = scenes[1]
        jid = srv.submit(JobRequest(acc, st, 40, 32, max_samples=128, target_relmse=2e-2, seed=5, denoise=True))
        for k in range(mix):
            a2, s2 = scenes[k % 2]
            srv.submit(JobRequest(a2, s2, 24 + 8 * k, 16, max_samples=64, target_relmse=1e-4, seed=10 + k,
                                  denoise=bool(k % 2)))
        while not srv.idle():
            srv.step()
        backend.finish()
        j = srv.status(jid)
        assert backend.denoise_calls > 0
        return j.result, j.samples, np.asarray(j.alpha).tolist(), j.estimate

    try:
        r0 = run(0)
        r1 = run(3)
        assert r0[1:] == r1[1:]
        assert np.array_equal(r0[0], r1[0])
    finally:
        net.destroy()
