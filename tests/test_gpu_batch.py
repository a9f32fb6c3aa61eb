"""Multi-scene batches: each job's image is bit-identical to rendering it
alone, whatever the mix, the job order and the wavefront split."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(vr, acc, st, spp, w, h, seed, first):
    import torch

    from voidray_gb300 import _native as N

    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    cst = st.to_c()
    stream = torch.cuda.Stream()
    N.check(vr.lib().vr_render_device(acc.handle, C.byref(cst), spp, out.data_ptr(), w, h, seed, first,
                                      C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    acc.synchronize()
    return out.cpu().numpy()


def _jobs(vr, W):
    from voidray_gb300.scene import Estimator, RenderSettings

    jobs = []
    s1, st1 = W.cornell_box(rr_depth=3)
    jobs.append((s1.build_acceleration(), st1, 12, 64, 48, 1, 0))
    s2 = vr.Scene()
    v, t = W.geodesic_sphere(12)
    m = s2.add_material(vr.Materials.lambertian((0.6, 0.5, 0.4)))
    s2.add_object(m, s2.add_mesh(vr.Mesh(v.astype(np.float32), t.astype(np.uint32), v.astype(np.float32))))
    s2.environment = vr.Environments.hdri_image(W.sky_hdri(64, 32, peak=80.0, sigma_deg=5.0))
    s2.camera = vr.Camera.look_at((0, 0.4, 3.0), (0, 0, 0), (0, 1, 0), vr.degrees_to_radians(40.0))
    st2 = RenderSettings(total_samples=20, max_bounces=6, rr_depth=2, estimator=Estimator.NEE,
                         firefly_clamp=float("inf"))
    jobs.append((s2.build_acceleration(), st2, 20, 40, 40, 7, 3))
    soup = W.soup_scene(5000, seed=3)
    soup.environment = vr.Environments.uniform((0.7, 0.8, 1.0))
    soup.camera = vr.Camera.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), (0, 1, 0), vr.degrees_to_radians(45.0))
    st3 = RenderSettings(total_samples=9, max_bounces=4, firefly_clamp=2.0)
    jobs.append((soup.build_acceleration(), st3, 9, 33, 17, 11, 0))
    return jobs


@pytest.mark.parametrize("max_wave", [0, 5000, 777])
def test_batch_equals_alone(gpu, max_wave):
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.batch import Batch, RenderJob

    jobs = _jobs(vr, W)
    alone = [_alone(vr, acc, st, spp, w, h, seed, first) for acc, st, spp, w, h, seed, first in jobs]
    batch = Batch(max_wave)
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, _, _, w, h, _, _ in jobs]
    stream = torch.cuda.Stream()
    # reversed order: the mix and the segment layout differ from the order above
    rj = [RenderJob(acc, st, spp, o.data_ptr(), w, h, seed, first)
          for (acc, st, spp, w, h, seed, first), o in zip(jobs, outs)][::-1]
    batch.render(rj, stream.cuda_stream)
    batch.synchronize(stream.cuda_stream)
    for a, o in zip(alone, outs):
        assert np.array_equal(o.cpu().numpy(), a)
    st = batch.stats()
    assert st.paths == sum(spp * w * h for _, _, spp, w, h, _, _ in jobs)


def test_batch_validation(gpu):
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.batch import Batch, RenderJob

    scene, st = W.cornell_box()
    acc = scene.build_acceleration()
    st.max_bounces = 40
    b = Batch()
    with pytest.raises(vr.VoidrayError):
        b.render([RenderJob(acc, st, 1, 0, 8, 8)])


@pytest.mark.parametrize("max_wave", [0, 5000])
def test_graph_replays_equal_direct_launches(gpu, max_wave):
    """Progressive passes of one job set: with graphs the first pass captures
    each distinct wave shape and later passes replay them; every pass's
    images equal the direct launches bit for bit (the jobs change their
    sample offsets and seeds between passes through the device job table)."""
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.batch import Batch, RenderJob

    jobs = _jobs(vr, W)
    stream = torch.cuda.Stream()
    results = {}
    for graphs in (False, True):
        batch = Batch(max_wave)
        batch.set_graphs(graphs)
        outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, _, _, w, h, _, _ in jobs]
        passes = 4
        for p in range(passes):
            rj = [RenderJob(acc, st, 2, o.data_ptr(), w, h, seed, first + 2 * p)
                  for (acc, st, spp, w, h, seed, first), o in zip(jobs, outs)]
            batch.render(rj, stream.cuda_stream)
            batch.synchronize(stream.cuda_stream)
        results[graphs] = [o.cpu().numpy() for o in outs]
        caps, reps = batch.graph_stats()
        if graphs:  # pass 1 runs directly, pass 2 captures, passes 3.. replay
            assert caps >= 1 and reps >= caps * (passes - 2)
        else:
            assert caps == 0 and reps == 0
        batch.destroy()
    for a, b in zip(results[False], results[True]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("max_wave", [0, 20000])
def test_mixed_job_set_equals_alone(gpu, max_wave):
    """The batched configuration at test size: 64 scenes of 10k-200k
    triangles, four image shapes (the 256^2 .. 1920x1080 set divided by 10),
    2-32 spp, depth 8-12, both estimators, clamp on and off, in one batch
    (one wave, or split into 20k-path waves): every job's image is
    bit-identical to rendering it alone."""
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.batch import Batch, RenderJob

    mix = W.mixed_job_set(64, seed=4)
    accs = [s.build_acceleration() for s, *_ in mix]
    alone = [_alone(vr, acc, st, spp, w, h, seed, 0) for acc, (s, st, spp, w, h, seed) in zip(accs, mix)]
    batch = Batch(max_wave)
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, _, _, w, h, _ in mix]
    stream = torch.cuda.Stream()
    batch.render([RenderJob(acc, st, spp, o.data_ptr(), w, h, seed, 0)
                  for acc, (s, st, spp, w, h, seed), o in zip(accs, mix, outs)], stream.cuda_stream)
    batch.synchronize(stream.cuda_stream)
    for k, (a, o) in enumerate(zip(alone, outs)):
        assert np.array_equal(o.cpu().numpy(), a), k
    assert batch.stats().paths == sum(spp * w * h for _, _, spp, w, h, _ in mix)
    batch.destroy()
    for acc in accs:
        acc.destroy()
