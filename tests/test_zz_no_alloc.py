"""vr_render_device_noalloc: the render entry point for callers that cannot
allocate device memory while they render.

A host application that has reserved the GPU's memory for its own pool (a
game engine, a compositor, a framework with a caching allocator) cannot let
the library cudaMalloc more scratch, and a real-time frame loop cannot take
the device-wide synchronisation of cudaFree or an allocation failure in the
middle of a frame.  This entry point takes its scratch from a fixed device
array inside the library instead.  The tests render through the C ABI with
both entry points and require the same pixels: on two no-alloc calls in a row
(different scenes, sizes and estimators, so the second call runs on scratch
the first one left behind), on a render cut into many small wavefronts, and
on an image close to the size limit; and they check that an image too large
for the fixed array is refused.

This file is named to be collected last: a failure here leaves every other
test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(vr, acc, st, spp, w, h, seed, noalloc):
    import torch

    from voidray_gb300 import _native as N

    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    cst = st.to_c()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    fn = vr.lib().vr_render_device_noalloc if noalloc else vr.lib().vr_render_device
    N.check(fn(acc.handle, C.byref(cst), spp, out.data_ptr(), w, h, seed, 0, stream))
    torch.cuda.synchronize()
    acc.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_render_device_twice(gpu):
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.scene import Estimator, RenderSettings

    # call 1: Cornell box, reference estimator with Russian roulette
    scene, st = W.cornell_box(rr_depth=3)
    acc = scene.build_acceleration()
    ref1 = _render(vr, acc, st, 16, 96, 96, 3, noalloc=False)
    got1 = _render(vr, acc, st, 16, 96, 96, 3, noalloc=True)

    # call 2, right after: another scene, size and estimator
    s2 = vr.Scene()
    v, t = W.geodesic_sphere(10)
    m = s2.add_material(vr.Materials.lambertian((0.6, 0.5, 0.4)))
    s2.add_object(m, s2.add_mesh(vr.Mesh(v.astype(np.float32), t.astype(np.uint32), v.astype(np.float32))))
    s2.environment = vr.Environments.hdri_image(W.sky_hdri(64, 32, peak=100.0, sigma_deg=5.0))
    s2.camera = vr.Camera.look_at((0, 0.5, 3.0), (0, 0, 0), (0, 1, 0), vr.degrees_to_radians(40.0))
    st2 = RenderSettings(total_samples=8, max_bounces=5, rr_depth=2, estimator=Estimator.NEE,
                         firefly_clamp=float("inf"))
    acc2 = s2.build_acceleration()
    ref2 = _render(vr, acc2, st2, 8, 80, 48, 9, noalloc=False)
    got2 = _render(vr, acc2, st2, 8, 80, 48, 9, noalloc=True)

    # same kernels and sample streams; only the wavefront size differs, which
    # does not change any pixel (per-pixel sums run in sample order)
    assert np.array_equal(got1, ref1)
    assert np.array_equal(got2, ref2)
    assert np.isfinite(got2).all() and got2[..., :3].mean() > 0.0


def test_noalloc_rejects_oversize_image(gpu):
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W

    scene, st = W.cornell_box()
    acc = scene.build_acceleration()
    cst = st.to_c()
    import torch

    w = h = 4096  # 16.7 Mpixels x 16 bytes exceeds the fixed scratch; refused before any launch
    # a full-size output buffer, so that even a regressed size check would write in bounds
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    status = vr.lib().vr_render_device_noalloc(acc.handle, C.byref(cst), 1, out.data_ptr(), w, h, 0, 0, None)
    torch.cuda.synchronize()
    assert status == 2, vr.lib().vr_last_error()
    assert b"no-alloc scratch" in vr.lib().vr_last_error()
    assert not bool(out.any()), "a refused call wrote to the output"
    del out


def test_noalloc_many_waves_and_near_limit(gpu):
    """Per-path arrays and queue counters reused across many wavefronts inside
    the fixed array, and the wavefront sized from what a 4-Mpixel image
    leaves of it: both bit-identical to vr_render_device."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W

    scene, st = W.cornell_box(rr_depth=3)
    acc = scene.build_acceleration()
    # 64x48 x 4 spp in wavefronts of 1024 paths: 12 waves
    st.wavefront_paths = 1024
    ref = _render(vr, acc, st, 4, 64, 48, 11, noalloc=False)
    got = _render(vr, acc, st, 4, 64, 48, 11, noalloc=True)
    assert np.array_equal(got, ref)
    # 2000x2000 at 1 spp: 64 MB of pixel sums leave room for a few thousand
    # paths per wavefront, so the frame runs as several hundred waves
    st.wavefront_paths = 0
    st.max_bounces = 4
    ref = _render(vr, acc, st, 1, 2000, 2000, 12, noalloc=False)
    got = _render(vr, acc, st, 1, 2000, 2000, 12, noalloc=True)
    assert np.array_equal(got, ref)
    assert np.isfinite(got).all() and got[..., :3].mean() > 0.0
