"""Throughput of the denoiser's kernels against the measured bf16 tensor peak.

    python -m voidray_gb300.denoise_bench [--width 1920 --height 1080] [--iters 20]

Times (CUDA events, after warm-up, on a dedicated stream) the forward pass
(inference: preprocess, 15 convolutions, pools, upsampling, postprocess) on
the mma.sync and the tcgen05 backends, and one training step (forward,
backward, Adam) with forward and backward-data on either backend.  FLOPs are
the network's algorithmic multiply-adds (2 * 9 * Cin * Cout per output pixel
of every 3x3 convolution, on the padded
channel counts the kernels compute) times the padded pixel count; a training
step counts three times the forward.
"""
from __future__ import annotations

import argparse
import json
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def _peak():
    try:
        p = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(p["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (of measured)"
    except (OSError, ValueError, KeyError):
        return 1900.0, "fallback 1.9 PFLOP/s"


def _inputs(h, w, n, seed=0):
    import torch

    g = torch.Generator(device="cuda").manual_seed(seed)
    rad = torch.rand((n, h, w, 4), generator=g, device="cuda") * 2.0
    alb = torch.rand((n, h, w, 4), generator=g, device="cuda")
    nrm = torch.nn.functional.normalize(torch.randn((n, h, w, 4), generator=g, device="cuda"), dim=-1)
    return rad, alb, nrm


def run(width=1920, height=1080, iters=20, batch=1, train_crop=128, train_batch=16):
    import torch

    from .denoise import Denoiser

    peak, src = _peak()
    net = Denoiser.pretrained()
    info = net.info()
    hp, wp = (height + 7) // 8 * 8, (width + 7) // 8 * 8
    flops = info.flops_per_pixel * hp * wp * batch
    stream = torch.cuda.Stream()
    rad, alb, nrm = _inputs(height, width, batch)
    out = torch.empty_like(rad)
    res = {"image": f"{width}x{height}", "batch": batch, "flops_per_frame": flops / batch,
           "peak_tflops": peak, "peak_source": src}

    def timed(fn, n):
        for _ in range(3):
            fn()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(n):
                fn()
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / n

    for name, backend in (("mma_sync", Denoiser.MMA_SYNC), ("tcgen05", Denoiser.TCGEN05)):
        net.set_backend(backend)
        if batch == 1:
            fn = lambda: net.denoise(rad[0], alb[0], nrm[0], 1.0, out[0], width, height, stream=stream.cuda_stream)
        else:
            sc = np.ones(batch, np.float32)
            fn = lambda: net.denoise_batch(rad, alb, nrm, sc, out, width, height, stream=stream.cuda_stream)
        ms = timed(fn, iters)
        net.status()
        tf = flops / (ms * 1e-3) / 1e12
        res[name] = {"ms": ms, "tflops": tf, "frac": tf / peak}
    # one training step (batch of crops), forward + backward + Adam, with forward
    # and backward-data on each backend (weight gradients on mma.sync in both)
    tr = _inputs(train_crop, train_crop, train_batch, seed=1)
    tgt = tr[0] * 0.9
    step = lambda: net.train_step(*tr, tgt, train_batch, train_crop, train_crop, 0.0, stream=stream.cuda_stream)
    for key, backend in (("train_step", Denoiser.TCGEN05), ("train_step_mma_sync", Denoiser.MMA_SYNC)):
        net.set_backend(backend)
        ms = timed(step, max(5, iters // 2))
        tflops = 3 * info.flops_per_pixel * train_crop * train_crop * train_batch / (ms * 1e-3) / 1e12
        res[key] = {"crop": train_crop, "batch": train_batch, "ms": ms, "tflops": tflops, "frac": tflops / peak}
    net.destroy()
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--iters", type=int, default=20)
    a = ap.parse_args(argv)
    print(json.dumps(run(a.width, a.height, a.iters, a.batch)))


if __name__ == "__main__":
    main()
