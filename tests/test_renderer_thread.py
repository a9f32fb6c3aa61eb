"""The render thread (renderer.rs one_shot): actions, statistics,
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


class _FakeAccel:
    def destroy(self):
        pass


def _fake_render(calls):
    """Stands in for the GPU call: adds a value that depends on the sample
    range only, in float32 like the accumulator, and records the chunks."""
    def render(target, accel, st, samples, seed=0, first_sample=0):
        calls.append((first_sample, samples))
        h, w = target.buffer.shape[:2]
        idx = np.arange(first_sample, first_sample + samples, dtype=np.float64)
        val = np.float32(np.sum(np.sin(idx * 0.37 + seed)) / st.total_samples)
        target.buffer[...] += val + np.arange(h * w * 4, dtype=np.float32).reshape(h, w, 4) * np.float32(1e-3)
    return render


def _fake_renderer(monkeypatch, tmp_path, total, seed=3):
    calls = []
    monkeypatch.setattr(R, "iterative_render", _fake_render(calls))
    monkeypatch.setattr(R, "chunk_size", lambda f, s, rem: 3)
    scene, st = W.cornell_box()
    monkeypatch.setattr(type(scene), "build_acceleration", lambda self: _FakeAccel())
    st.total_samples = total
    r = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(5, 4), seed=seed,
                    checkpoint_path=str(tmp_path / "ck.npz"))
    return r, calls


def test_checkpoint_resume_continues_the_chunk_sequence(monkeypatch, tmp_path):
    full, calls_full = _fake_renderer(monkeypatch, tmp_path, 11)
    full.execute(vr.RenderAction.RENDER)
    full.wait(60)
    assert calls_full == [(0, 1), (1, 3), (4, 3), (7, 3), (10, 3)]
    ck = vr.Checkpoint.load(str(tmp_path / "ck.npz"))
    assert (ck.samples, ck.total, ck.per_frame, ck.seed) == (11, 11, 3, 3)
    assert np.array_equal(ck.buffer, full.target.buffer)

    # stop after the chunk that ends at sample 7, then resume in a new renderer
    part, calls = _fake_renderer(monkeypatch, tmp_path, 11)
    orig = R.iterative_render

    def stop_at_7(target, accel, st, samples, seed=0, first_sample=0):
        orig(target, accel, st, samples, seed=seed, first_sample=first_sample)
        if first_sample + samples == 7:
            part.thread.execute(vr.RenderAction.CANCEL)
    monkeypatch.setattr(R, "iterative_render", stop_at_7)
    part.execute(vr.RenderAction.RENDER)
    part.wait(60)
    assert part.samples() == (7, 11)
    monkeypatch.setattr(R, "iterative_render", orig)
    resumed = vr.Renderer(part.scene, part.settings, vr.CpuRenderTarget(5, 4),
                          checkpoint_path=str(tmp_path / "ck2.npz"))
    resumed.resume(str(tmp_path / "ck.npz"))
    resumed.wait(60)
    assert calls == [(0, 1), (1, 3), (4, 3), (7, 3), (10, 3)]
    assert resumed.samples() == (11, 11) and resumed.seed == 3
    assert np.array_equal(resumed.target.buffer, full.target.buffer)


def test_resume_rejects_a_mismatched_checkpoint(monkeypatch, tmp_path):
    r, _ = _fake_renderer(monkeypatch, tmp_path, 5)
    r.execute(vr.RenderAction.RENDER)
    r.wait(60)
    scene, st = W.cornell_box()
    st.total_samples = 5
    with pytest.raises(vr.VoidrayError, match="shape"):
        vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(6, 4)).resume(str(tmp_path / "ck.npz"))
    st.total_samples = 6
    with pytest.raises(vr.VoidrayError, match="total samples"):
        vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(5, 4)).resume(str(tmp_path / "ck.npz"))


@pytest.mark.gpu
def test_resumed_render_is_bit_identical(gpu, monkeypatch, tmp_path):
    scene, st = W.cornell_box(rr_depth=3)
    st.total_samples = 14
    w, h = 40, 32
    monkeypatch.setattr(R, "chunk_size", lambda f, s, rem: 3)
    full = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(w, h), seed=9)
    full.execute(vr.RenderAction.RENDER)
    full.wait(120)

    ck_path = str(tmp_path / "ck.npz")
    part = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(w, h), seed=9, checkpoint_path=ck_path)
    orig = R.iterative_render

    def stop_at_7(target, accel, st_, samples, seed=0, first_sample=0):
        orig(target, accel, st_, samples, seed=seed, first_sample=first_sample)
        if first_sample + samples == 7:
            part.thread.execute(vr.RenderAction.CANCEL)
    monkeypatch.setattr(R, "iterative_render", stop_at_7)
    part.execute(vr.RenderAction.RENDER)
    part.wait(120)
    monkeypatch.setattr(R, "iterative_render", orig)
    assert part.samples() == (7, 14)
    resumed = vr.Renderer(scene, vr.Settings(render=st), vr.CpuRenderTarget(w, h))
    resumed.resume(ck_path)
    resumed.wait(120)
    assert resumed.samples() == (14, 14)
    assert np.array_equal(resumed.target.buffer, full.target.buffer)
