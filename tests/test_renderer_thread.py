"""The render-thread driver (renderer.rs one_shot): actions, statistics,
cancel, and the chunking kept from the reference."""
import time

import numpy as np
import pytest

import voidray_gb300 as vr
from voidray_gb300 import renderer as R
from voidray_gb300 import workloads as W


def test_chunk_size_follows_update_frequency():
    assert R.chunk_size(0.1, 0.01, 100) == 10
    assert R.chunk_size(0.0, 0.01, 100) == 1        # at least one sample per chunk
    assert R.chunk_size(10.0, 0.01, 37) == 37       # at most the remaining samples
    assert R.chunk_size(0.1, 0.01, 0) == 1


def test_invalid_actions_are_errors_not_panics(native):
    scene, st = W.cornell_box()
    r = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(8, 8))
    with pytest.raises(vr.VoidrayError):
        r.execute(vr.RenderAction.CANCEL)          # no render thread
    assert r.samples() == (0, 0) and r.elapsed_time() == 0.0 and r.remaining_time() is None


def test_render_without_device_reports_the_error(native):
    if native.lib().vr_device_available():
        pytest.skip("a CUDA device is present")
    scene, st = W.cornell_box()
    r = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(8, 8))
    r.execute(vr.RenderAction.RENDER)
    with pytest.raises(vr.VoidrayError):
        r.wait(60)
    assert not r.currently_rendering()


@pytest.mark.gpu
def test_one_shot_render_matches_single_call(gpu, monkeypatch):
    scene, st = W.cornell_box(rr_depth=3)
    st.total_samples = 10
    w, h = 40, 32
    monkeypatch.setattr(R, "chunk_size", lambda f, s, rem: 4)
    target = vr.CpuRenderTarget(w, h)
    r = vr.Renderer(scene, vr.Settings(render=st), target, seed=5)
    r.execute(vr.RenderAction.RENDER)
    r.wait(120)
    assert r.samples() == (10, 10) and not r.currently_rendering() and r.remaining_time() is None
    assert r.elapsed_time() > 0
    # chunks of 1, 4, 4, 4 samples: the last chunk renders 4 although 1 remains
    # (the reference's behaviour); samples 0..12, each weighted 1/10
    ref = vr.CpuRenderTarget(w, h)
    acc = scene.build_acceleration()
    vr.iterative_render(ref, acc, st, 13, seed=5)
    assert np.allclose(target.buffer[..., :3], ref.buffer[..., :3], rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_cancel_stops_the_render_early(gpu, monkeypatch):
    scene, st = W.cornell_box(rr_depth=3)
    st.total_samples = 100000
    monkeypatch.setattr(R, "chunk_size", lambda f, s, rem: 8)
    r = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(32, 32))
    r.execute(vr.RenderAction.RENDER)
    with pytest.raises(vr.VoidrayError):
        r.execute(vr.RenderAction.RENDER)       # already rendering
    time.sleep(0.2)
    r.execute(vr.RenderAction.CANCEL)
    r.wait(120)
    done, total = r.samples()
    assert 1 <= done < total and not r.currently_rendering()
