"""The render thread of voidray_renderer/src/render/renderer.rs on the GPU
backend.

`Renderer.execute(RenderAction.RENDER)` starts a one-shot progressive render
on a background thread (`RenderThread::one_shot`, renderer.rs:35-125): clear
the target, build the scene, render one sample and time it, size the
following chunks so that each takes about `update_frequency` seconds, render
chunk after chunk into the shared target (which a viewer may read between
chunks), update the statistics, and stop early on `RenderAction.CANCEL`.
`CONTINUOUS` clears the target and returns, like the reference's stub
(renderer.rs:127-148).  Each chunk is one `iterative_render` call (here
vr_render), continuing the sample streams where the last chunk stopped.

Kept from the reference on purpose: after the timed first sample every chunk
renders `samples_per_frame` samples, also the last one, while the counter
advances by at most the remaining samples (renderer.rs:86-93), so the last
chunk can add more samples than `total_samples` asks for, each weighted
1/total_samples.  Invalid actions (RENDER while rendering; CANCEL or REBUILD
with no render thread) raise VoidrayError instead of panicking.

Checkpoints (no reference counterpart): with `checkpoint_path` set, the
thread writes the accumulator, the samples done, the chunk size and the seed
after every chunk (atomically, by rename).  `Renderer.resume(path)` restores
the accumulator and continues with the same chunk sequence; the sample
streams are counter-based per (seed, sample index, pixel), so a resumed
render adds exactly the chunks the uninterrupted one would have added and
its image is bit-identical.
"""
from __future__ import annotations

import enum
import os
import queue
import threading
import time
from dataclasses import dataclass, replace
from typing import Optional

import numpy as np

from ._native import VoidrayError
from .scene import CpuRenderTarget, Scene, Settings, iterative_render


class RenderAction(enum.Enum):
    RENDER = 0      # single-shot render
    CONTINUOUS = 1  # begin continually rendering (a stub in the reference)
    REBUILD = 2     # rebuild the scene and clear the screen
    CANCEL = 3      # cancel a running render


@dataclass
class RendererStats:
    currently_rendering: bool = False
    samples: tuple[int, int] = (0, 0)
    time: Optional[tuple[float, Optional[float]]] = None  # (start, end) perf_counter seconds
    remaining: Optional[float] = None                     # seconds


@dataclass
class Checkpoint:
    buffer: np.ndarray   # the render target's RGBA f32 accumulator
    samples: int         # samples accumulated so far
    total: int           # RenderSettings.total_samples (the weight 1/total)
    per_frame: int       # samples per chunk after the first
    seed: int

    def save(self, path: str) -> None:
        tmp = path + ".tmp"
        with open(tmp, "wb") as f:
            np.savez(f, buffer=self.buffer, meta=np.array([self.samples, self.total, self.per_frame, self.seed],
                                                          np.int64))
        os.replace(tmp, path)

    @staticmethod
    def load(path: str) -> "Checkpoint":
        with np.load(path) as z:
            samples, total, per_frame, seed = (int(x) for x in z["meta"])
            return Checkpoint(np.array(z["buffer"], np.float32), samples, total, per_frame, seed)


def chunk_size(update_frequency: float, single_sample_s: float, remaining: int) -> int:
    """Samples per chunk after the timed first sample (renderer.rs:78-81)."""
    return min(max(int(update_frequency / single_sample_s), 1), max(remaining, 1))


class RenderThread:
    def __init__(self, target: CpuRenderTarget, stats: RendererStats, lock: threading.Lock, scene: Scene,
                 settings: Settings, one_shot: bool, seed: int = 0, checkpoint_path: Optional[str] = None,
                 resume: Optional[Checkpoint] = None):
        self.actions: queue.Queue = queue.Queue()
        self.error: Optional[BaseException] = None
        self.checkpoint_path = checkpoint_path
        self.resume = resume
        self._args = (target, stats, lock, scene, settings, seed)
        fn = self._one_shot if one_shot else self._continuous
        self.handle = threading.Thread(target=self._guard, args=(fn,), daemon=True)
        self.handle.start()

    def execute(self, action: RenderAction) -> None:
        self.actions.put(action)

    def _guard(self, fn) -> None:
        try:
            fn()
        except BaseException as e:  # reported by Renderer.wait(); the stats say the render stopped
            self.error = e
            _, stats, lock, *_ = self._args
            with lock:
                stats.currently_rendering = False

    def _continuous(self) -> None:
        target = self._args[0]
        target.clear()

    def _one_shot(self) -> None:
        target, stats, lock, scene, settings, seed = self._args
        with lock:
            stats.currently_rendering = True
            start = time.perf_counter()
            stats.time = (start, None)
        st = replace(settings.render)
        total = int(st.total_samples)
        ck = self.resume
        if ck is None:
            target.clear()
        accel = scene.build_acceleration()
        try:
            if ck is None:
                t1 = time.perf_counter()
                iterative_render(target, accel, st, 1, seed=seed, first_sample=0)
                single = max(time.perf_counter() - t1, 1e-9)
                samples = 1
                per_frame = chunk_size(st.update_frequency, single, total - samples)
                with lock:
                    stats.samples = (samples, total)
                    stats.remaining = single * (total - 1)
                self._save(target, samples, total, per_frame, seed)
            else:
                target.buffer[...] = ck.buffer
                samples, per_frame = ck.samples, ck.per_frame
                with lock:
                    stats.samples = (samples, total)
            while samples < total:
                delta = min(per_frame, total - samples)
                iterative_render(target, accel, st, per_frame, seed=seed, first_sample=samples)
                samples += delta
                elapsed = time.perf_counter() - start
                with lock:
                    stats.samples = (samples, total)
                    stats.remaining = elapsed / max(samples - (ck.samples if ck else 0), 1) * (total - samples)
                self._save(target, samples, total, per_frame, seed)
                try:
                    action = self.actions.get_nowait()
                except queue.Empty:
                    continue
                if action == RenderAction.CANCEL:
                    break
                raise VoidrayError(1, f"invalid action {action} during a render")
        finally:
            accel.destroy()
            with lock:
                stats.currently_rendering = False
                stats.time = (stats.time[0], time.perf_counter()) if stats.time else None
                stats.remaining = None

    def _save(self, target, samples, total, per_frame, seed) -> None:
        if self.checkpoint_path:
            Checkpoint(target.buffer.copy(), samples, total, per_frame, seed).save(self.checkpoint_path)


class Renderer:
    """renderer.rs:151-258 without the Vulkan queue: owns the statistics and
    the render thread; `target` is the CpuRenderTarget a viewer reads."""

    def __init__(self, scene: Scene, settings: Settings, target: CpuRenderTarget, seed: int = 0,
                 checkpoint_path: Optional[str] = None):
        self.scene = scene
        self.settings = settings
        self.target = target
        self.seed = seed
        self.checkpoint_path = checkpoint_path
        self.stats = RendererStats()
        self._lock = threading.Lock()
        self.thread: Optional[RenderThread] = None

    def execute(self, action: RenderAction) -> None:
        if action in (RenderAction.RENDER, RenderAction.CONTINUOUS):
            if self.currently_rendering():
                raise VoidrayError(1, f"invalid action {action}: already rendering")
            with self._lock:
                self.stats = RendererStats(currently_rendering=action == RenderAction.RENDER)
            self.thread = RenderThread(self.target, self.stats, self._lock, self.scene, self.settings,
                                       one_shot=action == RenderAction.RENDER, seed=self.seed,
                                       checkpoint_path=self.checkpoint_path)
        elif self.thread is not None:
            self.thread.execute(action)
        else:
            raise VoidrayError(1, f"invalid action {action}: no render thread")

    def resume(self, path: str) -> None:
        """Continues a one-shot render from a checkpoint written by a render of
        the same scene, settings and target size."""
        if self.currently_rendering():
            raise VoidrayError(1, "invalid action resume: already rendering")
        ck = Checkpoint.load(path)
        if ck.buffer.shape != self.target.buffer.shape:
            raise VoidrayError(1, f"checkpoint of shape {ck.buffer.shape} for a target of {self.target.buffer.shape}")
        if ck.total != int(self.settings.render.total_samples):
            raise VoidrayError(1, f"checkpoint for {ck.total} total samples, settings ask {self.settings.render.total_samples}")
        self.seed = ck.seed
        with self._lock:
            self.stats = RendererStats(currently_rendering=True)
        self.thread = RenderThread(self.target, self.stats, self._lock, self.scene, self.settings, one_shot=True,
                                   seed=ck.seed, checkpoint_path=self.checkpoint_path, resume=ck)

    def wait(self, timeout: Optional[float] = None) -> None:
        """Joins the render thread; re-raises its error."""
        if self.thread is not None:
            self.thread.handle.join(timeout)
            if self.thread.error is not None:
                raise self.thread.error

    def currently_rendering(self) -> bool:
        with self._lock:
            return self.stats.currently_rendering

    def samples(self) -> tuple[int, int]:
        with self._lock:
            return self.stats.samples

    def elapsed_time(self) -> float:
        with self._lock:
            if self.stats.time is None:
                return 0.0
            start, end = self.stats.time
            return (end if end is not None else time.perf_counter()) - start

    def remaining_time(self) -> Optional[float]:
        with self._lock:
            return self.stats.remaining
