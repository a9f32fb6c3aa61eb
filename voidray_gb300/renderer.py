"""The render-thread driver of voidray_renderer/src/render/renderer.rs on the
GPU backend.

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
"""
from __future__ import annotations

import enum
import queue
import threading
import time
from dataclasses import dataclass, replace
from typing import Optional

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


def chunk_size(update_frequency: float, single_sample_s: float, remaining: int) -> int:
    """Samples per chunk after the timed first sample (renderer.rs:78-81)."""
    return min(max(int(update_frequency / single_sample_s), 1), max(remaining, 1))


class RenderThread:
    def __init__(self, target: CpuRenderTarget, stats: RendererStats, lock: threading.Lock, scene: Scene,
                 settings: Settings, one_shot: bool, seed: int = 0):
        self.actions: queue.Queue = queue.Queue()
        self.error: Optional[BaseException] = None
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
        target.clear()
        accel = scene.build_acceleration()
        st = replace(settings.render)
        total = int(st.total_samples)
        try:
            t1 = time.perf_counter()
            iterative_render(target, accel, st, 1, seed=seed, first_sample=0)
            single = max(time.perf_counter() - t1, 1e-9)
            samples = 1
            with lock:
                stats.samples = (samples, total)
                stats.remaining = single * (total - 1)
            per_frame = chunk_size(st.update_frequency, single, total - samples)
            while samples < total:
                delta = min(per_frame, total - samples)
                iterative_render(target, accel, st, per_frame, seed=seed, first_sample=samples)
                samples += delta
                elapsed = time.perf_counter() - start
                with lock:
                    stats.samples = (samples, total)
                    stats.remaining = elapsed / samples * (total - samples)
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


class Renderer:
    """renderer.rs:151-258 without the Vulkan queue: owns the statistics and
    the render thread; `target` is the CpuRenderTarget a viewer reads."""

    def __init__(self, scene: Scene, settings: Settings, target: CpuRenderTarget, seed: int = 0):
        self.scene = scene
        self.settings = settings
        self.target = target
        self.seed = seed
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
                                       one_shot=action == RenderAction.RENDER, seed=self.seed)
        elif self.thread is not None:
            self.thread.execute(action)
        else:
            raise VoidrayError(1, f"invalid action {action}: no render thread")

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
