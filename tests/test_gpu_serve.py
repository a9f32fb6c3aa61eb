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


@pytest.mark.parametrize("adaptive,pipelined,streams", [(False, False, 1), (True, False, 1), (True, True, 1),
                                                       (True, True, 2)])
def test_denoised_serving_same_alone_and_in_mix(gpu, adaptive, pipelined, streams):
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
        backend = GpuBackend(denoiser=net, render_streams=streams)
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
        backend.destroy()
        return j.result, j.samples, np.asarray(j.alpha).tolist(), j.estimate

    try:
        r0 = run(0)
        r1 = run(3)
        assert r0[1:] == r1[1:]
        assert np.array_equal(r0[0], r1[0])
    finally:
        net.destroy()


@pytest.mark.parametrize("denoised", [False, True])
def test_stats_kernel_matches_numpy(gpu, denoised):
    """vr_serve_stats_device against the numpy formulas the CPU scheduler uses
    (_estimate and blend_tile_moments): ragged tiles, several jobs of
    different sizes and sample counts in one launch."""
    import ctypes as C

    import torch

    from voidray_gb300 import _native as N
    from voidray_gb300.serve import BLEND_TILE, _estimate, blend_tile_moments

    rng = np.random.default_rng(3)
    shapes = [(40, 24, 8, 8), (17, 33, 5, 12), (64, 64, 32, 32)]
    bufs, table, offs, off = [], (N.vr_stats_job * len(shapes))(), [], 0
    for i, (h, w, na, nb) in enumerate(shapes):
        A = (rng.gamma(1.0, 0.4, (h, w, 4)) * na).astype(np.float32)
        B = (rng.gamma(1.0, 0.4, (h, w, 4)) * nb).astype(np.float32)
        DA = rng.gamma(1.0, 0.4, (h, w, 4)).astype(np.float32)
        DB = rng.gamma(1.0, 0.4, (h, w, 4)).astype(np.float32)
        t = [torch.from_numpy(x).cuda() for x in (A, B, DA, DB)]
        bufs.append((A, B, DA, DB, t))
        e = table[i]
        e.sum_a, e.sum_b = t[0].data_ptr(), t[1].data_ptr()
        e.den_a, e.den_b = (t[2].data_ptr(), t[3].data_ptr()) if denoised else (None, None)
        e.n_a, e.n_b, e.width, e.height, e.tile_offset = na, nb, w, h, off
        nt = -(-h // BLEND_TILE) * -(-w // BLEND_TILE)
        offs.append((off, nt))
        off += (6 if denoised else 1) * nt
    out = torch.full((off,), -1.0, dtype=torch.float64, device="cuda")
    N.check(N.lib().vr_serve_stats_device(table, len(shapes), C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    v = out.cpu().numpy()
    for (h, w, na, nb), (A, B, DA, DB, _), (o, nt) in zip(shapes, bufs, offs):
        a, b = A[..., :3].astype(np.float64) / na, B[..., :3].astype(np.float64) / nb
        plain = float(v[o:o + nt].sum()) / (3 * h * w)
        assert plain == pytest.approx(_estimate(a, b, na, nb), rel=1e-12)
        if denoised:
            m = (A[..., :3].astype(np.float64) + B[..., :3]) / (na + nb)
            ref = blend_tile_moments(a, b, m, DA[..., :3].astype(np.float64), DB[..., :3].astype(np.float64))
            got = v[o + nt:o + 6 * nt].reshape(ref.shape)
            assert np.allclose(got, ref, rtol=1e-12, atol=0)
    out2 = torch.full((off,), -1.0, dtype=torch.float64, device="cuda")
    N.check(N.lib().vr_serve_stats_device(table, len(shapes), C.c_void_p(out2.data_ptr()), None))
    torch.cuda.synchronize()
    assert np.array_equal(out2.cpu().numpy(), v)   # deterministic


@pytest.mark.parametrize("h,w", [(40, 24), (17, 33)])
def test_result_kernels_match_numpy(gpu, h, w):
    """vr_serve_sum_device and vr_serve_blend_device (a served job's final
    image) against the formulas they compute: sums of half-buffer pairs, the
    plain mean (A + B) / n, and alpha D + (1 - alpha) mean with alpha per
    16 x 16 tile (ragged tiles at the edges); the output is packed RGB."""
    import ctypes as C

    import torch

    from voidray_gb300 import _native as N
    from voidray_gb300.serve import BLEND_TILE

    rng = np.random.default_rng(7)
    n = 96
    A, B, D = (rng.gamma(1.0, 0.4, (h, w, 4)).astype(np.float32) * s for s in (48.0, 48.0, 1.0))
    ty, tx = -(-h // BLEND_TILE), -(-w // BLEND_TILE)
    alpha = rng.uniform(0.0, 1.0, (ty, tx)).astype(np.float32)
    alpha[0, 0] = 0.0
    tA, tB, tD, tal = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (A, B, D, alpha))
    p = lambda x: C.c_void_p(x.data_ptr())
    # sums of three pairs
    outs = [torch.full((h, w, 4), -1.0, dtype=torch.float32, device="cuda") for _ in range(3)]
    arr = C.c_void_p * 3
    N.check(N.lib().vr_serve_sum_device(arr(tA.data_ptr(), tB.data_ptr(), tD.data_ptr()),
                                        arr(tB.data_ptr(), tD.data_ptr(), tA.data_ptr()),
                                        arr(*[o.data_ptr() for o in outs]), 3, h * w, None))
    torch.cuda.synchronize()
    for o, (x, y) in zip(outs, [(A, B), (B, D), (D, A)]):
        assert np.array_equal(o.cpu().numpy(), x + y)
    # plain mean and blend
    mean = (A[..., :3] + B[..., :3]) * np.float32(1.0 / n)
    rgb = torch.full((h, w, 3), -1.0, dtype=torch.float32, device="cuda")
    N.check(N.lib().vr_serve_blend_device(p(tA), p(tB), n, None, None, w, h, p(rgb), None))
    torch.cuda.synchronize()
    assert np.allclose(rgb.cpu().numpy(), mean, rtol=1e-6, atol=0)
    N.check(N.lib().vr_serve_blend_device(p(tA), p(tB), n, p(tD), p(tal), w, h, p(rgb), None))
    torch.cuda.synchronize()
    am = np.repeat(np.repeat(alpha, BLEND_TILE, 0), BLEND_TILE, 1)[:h, :w, None]
    want = am * D[..., :3] + (1.0 - am) * mean
    assert np.allclose(rgb.cpu().numpy(), want, rtol=1e-5, atol=1e-7)
    assert N.lib().vr_serve_blend_device(p(tA), p(tB), n, p(tD), None, w, h, p(rgb), None) == 1


def test_backend_estimates_through_the_stats_kernel(gpu):
    """GpuBackend's per-pass estimate (one vr_serve_stats_device launch) equals
    the numpy half-buffer formula on the same buffers."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.serve import GpuBackend, JobRequest, JobState, _estimate

    scenes = _scenes(vr, W)
    be = GpuBackend()
    jobs = []
    for k, (w, h) in enumerate([(40, 24), (33, 17)]):
        acc, st = scenes[k]
        job = JobState(job_id=k, req=JobRequest(acc, st, w, h, max_samples=64, target_relmse=1e-3, seed=3 + k),
                       arrival=0.0)
        job.bufs = be.alloc(job)
        jobs.append(job)
    be.render([(j, 0, 0, 8) for j in jobs] + [(j, 1, 8, 6) for j in jobs])
    for j in jobs:
        j.n_a, j.n_b, j.samples = 8, 6, 14
    got = be.estimate_many(jobs)
    for j, e in zip(jobs, got):
        a = j.bufs[0][..., :3].double().cpu().numpy() / 8
        b = j.bufs[1][..., :3].double().cpu().numpy() / 6
        assert e == pytest.approx(_estimate(a, b, 8, 6), rel=1e-12)
    be.destroy()


def test_gpu_checkpoint_resume_is_bit_identical(gpu, tmp_path):
    """A denoised job checkpointed to disk after its first pass and resumed on
    a new server and backend (two render streams, other jobs in the mix)
    ends with the same samples, blend weights and image as without the
    interruption."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.denoise import Denoiser
    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig

    scenes = _scenes(vr, W)
    cfg = ServerConfig(min_samples=16, adaptive=True, pass_paths=40 * 32 * 64, first_pass_spp=16)
    net = Denoiser.pretrained()
    acc, st = scenes[1]
    req = lambda: JobRequest(acc, st, 40, 32, max_samples=256, target_relmse=5e-3, seed=21, denoise=True)
    try:
        be = GpuBackend(denoiser=net)
        s = Server(be, cfg)
        jid = s.submit(req())
        while not s.idle():
            s.step()
        ref = s.status(jid)
        ref = (ref.result, ref.samples, np.asarray(ref.alpha).tolist(), ref.passes)
        be.destroy()
        assert ref[3] >= 2

        be = GpuBackend(denoiser=net)
        s = Server(be, cfg)
        jid = s.submit(req())
        s.step()
        path = str(tmp_path / "job.npz")
        s.checkpoint(jid, path)
        be.destroy()

        be = GpuBackend(denoiser=net, render_streams=2)
        s = Server(be, cfg)
        a2, s2 = scenes[0]
        s.submit(JobRequest(a2, s2, 24, 16, max_samples=64, target_relmse=1e-4, seed=77))
        rid = s.submit(req(), resume=path)
        while not s.idle():
            s.step()
        j = s.status(rid)
        assert (j.samples, np.asarray(j.alpha).tolist(), j.passes) == ref[1:]
        assert np.array_equal(j.result, ref[0])
        be.destroy()
    finally:
        net.destroy()


def test_cancellations_in_flight_leave_other_jobs_unchanged(gpu):
    """Two render streams, pipelined passes, and jobs cancelled while their
    passes or estimates are in flight (their memory goes back to the
    allocator): the job that stays ends exactly as it does alone."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig

    scenes = _scenes(vr, W)
    cfg = ServerConfig(min_samples=16, adaptive=True, pipelined=True, pass_paths=40 * 32 * 24, first_pass_spp=16,
                       max_inflight=3)
    acc, st = scenes[1]
    keep = lambda: JobRequest(acc, st, 40, 32, max_samples=256, target_relmse=5e-3, seed=31)

    def run(with_others):
        be = GpuBackend(render_streams=2)
        s = Server(be, cfg)
        jid = s.submit(keep())
        others = []
        if with_others:
            for k in range(6):
                a2, s2 = scenes[k % 2]
                others.append(s.submit(JobRequest(a2, s2, 32 + 8 * k, 24, max_samples=512, target_relmse=1e-5,
                                                  seed=90 + k)))
        steps = 0
        while not s.idle():
            s.step()
            steps += 1
            if with_others and steps % 2 == 0:
                live = [o for o in others if s.status(o).state in ("waiting", "active")]
                if live:
                    s.cancel(live[0])
        be.finish()
        j = s.status(jid)
        out = (j.result, j.samples, j.n_a, j.n_b)
        be.destroy()
        return out, [s.status(o).state for o in others]

    (r0, _), (r1, states) = run(False), run(True)
    assert "cancelled" in states
    assert r0[1:] == r1[1:] and np.array_equal(r0[0], r1[0])
