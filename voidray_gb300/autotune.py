"""Autotuner of the wavefront renderer's launch shapes.

Knobs: paths per wavefront (the render settings' wavefront_paths), and the
block size / resident blocks per SM of the shade and raygen stages
(vr_tuning_set).  None of them changes a result; they trade occupancy, queue
coherence and scratch memory against each other, and the best choice
depends on the scene size, the image and the sample count.

The search is a coordinate descent (wavefront size first, then the shade
block, then its blocks per SM, then the raygen block), each configuration
timed with CUDA events on a short render of the caller's own workload after
a warm-up.  Results are cached per (GPU name, triangle-count bucket, pixel
bucket, spp bucket, estimator) in a JSON file (VOIDRAY_TUNING_CACHE, default
~/.cache/voidray_gb300/tuning.json), so a workload class is tuned once per
machine.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import time
from dataclasses import replace
from pathlib import Path

from . import _native as N
from ._native import check, lib

WAVEFRONTS = (1 << 22, 1 << 24, 1 << 26, 1 << 27, 1 << 28)
BLOCKS = (64, 128, 256)
PER_SM = (4, 8, 16)
DEFAULT = {"wavefront_paths": 1 << 28, "shade_block": 256, "shade_blocks_per_sm": 8, "raygen_block": 256}


def cache_path() -> Path:
    p = os.environ.get("VOIDRAY_TUNING_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "voidray_gb300" / "tuning.json"


def bucket_key(gpu: str, triangles: int, pixels: int, spp: int, estimator: int) -> str:
    lg = lambda x: int(math.log2(max(1, x)))
    return f"{gpu}|tri2^{lg(triangles)}|px2^{lg(pixels)}|spp2^{lg(spp)}|est{estimator}"


def get_tuning() -> dict:
    t = N.vr_tuning()
    check(lib().vr_tuning_get(C.byref(t)))
    return {"shade_block": t.shade_block, "shade_blocks_per_sm": t.shade_blocks_per_sm,
            "raygen_block": t.raygen_block}


def set_tuning(cfg: dict) -> None:
    t = N.vr_tuning(int(cfg["shade_block"]), int(cfg["shade_blocks_per_sm"]), int(cfg["raygen_block"]), 0)
    check(lib().vr_tuning_set(C.byref(t)))


def load_cache() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def save_cache(c: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(c, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only costs a re-tune


def apply(cfg: dict, settings):
    """Sets the launch shapes and returns the settings with the tuned wavefront size."""
    set_tuning(cfg)
    return replace(settings, wavefront_paths=int(cfg["wavefront_paths"]))


def tune(acc, settings, width: int, height: int, spp: int, *, use_cache: bool = True, repeats: int = 2,
         log=None) -> dict:
    """Best configuration for rendering `spp` samples of a width x height image
    of `acc` with `settings`; returns {knobs..., "ms": time, "trials": n,
    "cached": bool}.  Leaves the best launch shapes set."""
    import torch

    from .scene import render_device

    gpu = torch.cuda.get_device_name()
    info = acc.info()
    key = bucket_key(gpu, info.num_triangles, width * height, spp, int(settings.estimator))
    cache = load_cache() if use_cache else {}
    if key in cache:
        best = dict(cache[key], cached=True, key=key)
        set_tuning(best)
        return best

    out = torch.zeros((height, width, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    trials = 0

    def run(cfg) -> float:
        nonlocal trials
        st = apply(cfg, settings)
        render_device(acc, st, spp, out.data_ptr(), width, height, seed=1, stream=stream.cuda_stream)  # warm-up
        stream.synchronize()
        best_ms = float("inf")
        for r in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
                render_device(acc, st, spp, out.data_ptr(), width, height, seed=2 + r, stream=stream.cuda_stream)
                e1.record(stream)
            e1.synchronize()
            best_ms = min(best_ms, e0.elapsed_time(e1))
        trials += 1
        if log:
            log(f"[autotune] {cfg} {best_ms:.2f} ms")
        return best_ms

    total = spp * width * height
    cfg = dict(DEFAULT)
    best_ms = None
    t0 = time.perf_counter()
    for knob, values in (("wavefront_paths", [w for w in WAVEFRONTS if w <= max(total, WAVEFRONTS[0])]),
                         ("shade_block", BLOCKS), ("shade_blocks_per_sm", PER_SM), ("raygen_block", BLOCKS)):
        results = {}
        for v in values:
            c = dict(cfg, **{knob: v})
            results[v] = run(c)
        v_best = min(results, key=results.get)
        cfg[knob] = v_best
        best_ms = results[v_best]
    best = dict(cfg, ms=best_ms, trials=trials, seconds=time.perf_counter() - t0)
    if use_cache:
        cache[key] = best
        save_cache(cache)
    set_tuning(best)
    return dict(best, cached=False, key=key)


BATCH_WAVEFRONTS = (1 << 26, 1 << 27, 1 << 28)


def tune_batch(jobs, *, scale: int = 8, use_cache: bool = True, log=None) -> dict:
    """Best launch shapes for a many-job batch: the batch's wavefront size
    (vr_batch_create's max_wave_paths) and the shade / raygen launch shapes,
    by the same coordinate descent as tune(), each configuration timed with
    CUDA events on the caller's own jobs with their sample counts divided by
    `scale` (at least 1), graphs on, after two warm-up passes (direct, then
    capture).  `jobs`: [(acc, settings, spp, width, height, seed)].  Cached per
    (GPU, job count, triangle / pixel / sample buckets).  Returns {knobs...,
    "max_wave_paths", "ms", "trials", "cached"} and leaves the launch shapes set."""
    import torch

    from .batch import Batch, RenderJob

    gpu = torch.cuda.get_device_name()
    lg = lambda x: int(math.log2(max(1, x)))
    tris = sum(int(a.info().num_triangles) for a, *_ in jobs)
    pix = sum(w * h for _, _, _, w, h, _ in jobs)
    smp = sum(spp * w * h for _, _, spp, w, h, _ in jobs)
    key = f"{gpu}|batch{len(jobs)}|tri2^{lg(tris)}|px2^{lg(pix)}|smp2^{lg(smp)}"
    cache = load_cache() if use_cache else {}
    if key in cache:
        best = dict(cache[key], cached=True, key=key)
        set_tuning(best)
        return best
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, _, _, w, h, _ in jobs]
    stream = torch.cuda.Stream()
    trials = 0

    def run(cfg) -> float:
        nonlocal trials
        set_tuning(cfg)
        b = Batch(int(cfg["max_wave_paths"]))
        b.set_graphs(True)
        try:
            def one(p):
                b.render([RenderJob(acc, st, max(1, spp // scale), o.data_ptr(), w, h, seed, p * max(1, spp // scale))
                          for (acc, st, spp, w, h, seed), o in zip(jobs, outs)], stream.cuda_stream)
            one(0)
            one(1)
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one(2)
            one(3)
            e1.record(stream)
            e1.synchronize()
            b.synchronize(stream.cuda_stream)
            ms = e0.elapsed_time(e1) / 2
        finally:
            b.destroy()
        trials += 1
        if log:
            log(f"[autotune batch] {cfg} {ms:.2f} ms")
        return ms

    cfg = dict(DEFAULT)
    cfg.pop("wavefront_paths")
    cfg["max_wave_paths"] = 1 << 26
    best_ms = None
    t0 = time.perf_counter()
    for knob, values in (("max_wave_paths", BATCH_WAVEFRONTS), ("shade_block", BLOCKS),
                         ("shade_blocks_per_sm", PER_SM), ("raygen_block", BLOCKS)):
        results = {v: run(dict(cfg, **{knob: v})) for v in values}
        v_best = min(results, key=results.get)
        cfg[knob] = v_best
        best_ms = results[v_best]
    best = dict(cfg, ms=best_ms, trials=trials, seconds=time.perf_counter() - t0, sample_scale=scale)
    if use_cache:
        cache[key] = best
        save_cache(cache)
    set_tuning(best)
    return dict(best, cached=False, key=key)
