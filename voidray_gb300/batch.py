"""Multi-scene rendering: many render jobs in one wavefront launch per stage.

Each job is a built scene with its own settings, image, seed and sample
range.  Results are bit-identical to rendering every job alone.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _native as N
from ._native import check, lib
from .scene import RenderSettings, SceneAcceleration


@dataclass
class RenderJob:
    scene: SceneAcceleration
    settings: RenderSettings
    samples: int
    rgba_device: int          # device pointer to an RGBA f32 buffer of width x height
    width: int
    height: int
    seed: int = 0
    first_sample: int = 0
    albedo_device: int = 0    # optional first-hit AOV buffers (both or neither), same layout as rgba
    normal_device: int = 0

    def to_c(self) -> N.vr_render_job:
        return N.vr_render_job(self.scene.handle.value, self.settings.to_c(), int(self.samples), int(self.width),
                               int(self.height), int(self.first_sample), int(self.seed), int(self.rgba_device),
                               int(self.albedo_device) or None, int(self.normal_device) or None)


class Batch:
    """vr_batch handle: owns the shared wavefront scratch."""

    def __init__(self, max_wave_paths: int = 0):
        h = C.c_void_p()
        check(lib().vr_batch_create(int(max_wave_paths), C.byref(h)))
        self._h = h

    def render(self, jobs: list[RenderJob], stream: int = 0) -> None:
        arr = (N.vr_render_job * max(1, len(jobs)))(*[j.to_c() for j in jobs])
        check(lib().vr_batch_render(self._h, arr, len(jobs), C.c_void_p(stream or None)))

    def set_graphs(self, enable: bool = True) -> None:
        """Replay each wavefront's stage sequence as a cached CUDA graph."""
        check(lib().vr_batch_set_graphs(self._h, int(enable)))

    def graph_stats(self) -> tuple[int, int]:
        """(captures, replays)"""
        c, r = C.c_uint64(), C.c_uint64()
        check(lib().vr_batch_graph_stats(self._h, C.byref(c), C.byref(r)))
        return c.value, r.value

    def synchronize(self, stream: int = 0) -> None:
        check(lib().vr_batch_synchronize(self._h, C.c_void_p(stream or None)))

    def stats(self) -> N.vr_render_stats:
        st = N.vr_render_stats()
        check(lib().vr_batch_stats_get(self._h, C.byref(st)))
        return st

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().vr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
