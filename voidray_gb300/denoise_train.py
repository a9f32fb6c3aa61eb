"""Training data and training loop of the learned denoiser.

    python -m voidray_gb300.denoise_train --views 2000 --out unet_bf16.npy

Data: seeded procedural scenes from the same family as the render workload
(displaced icospheres with per-patch Lambertian / metal / dielectric
materials over a ground plane, lit by a sky HDRI whose sun position is drawn
per scene), seen from random orbit cameras.  Each view gives one 256x256
pair: the input rendered at 4 spp (radiance, albedo, normal) and the target
at 1024 spp from an independent sample stream; a second input at a random
count of 16-512 spp teaches the network the noise levels a progressive
render passes through.  Everything is rendered by the library's tracer and
kept on the device.

Training: Adam on random crops (batch x crop x crop), cosine learning-rate
decay, L1 loss in log-demodulated space, all on the library's own BF16
forward/backward kernels.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import workloads as W
from .denoise import Denoiser
from .scene import Camera, Environments, Estimator, RenderSettings, degrees_to_radians, render_device

SIZE = 256
IN_SPP = 4
TARGET_SPP = 1024
EXTRA_SPP = (16, 32, 64, 128, 256, 512)
FIREFLY_CLAMP = 3.0


def relmse(x, r, eps=1e-2):
    """mean((x - r)^2 / (r^2 + eps)) over pixels and colour channels (torch tensors)."""
    return float(((x - r) ** 2 / (r * r + eps)).mean())


def scene_params(seed: int) -> dict:
    rng = np.random.default_rng(seed)
    return {"geo_seed": int(rng.integers(1000, 10**6)), "freq": int(rng.choice([20, 40, 80, 120])),
            "sun_elev": float(rng.uniform(8.0, 70.0)), "sun_azim": float(rng.uniform(0.0, 360.0)),
            "bounces": int(rng.integers(8, 13))}


def random_camera(rng) -> Camera:
    az = rng.uniform(0.0, 2.0 * math.pi)
    el = math.radians(rng.uniform(-4.0, 40.0))
    dist = rng.uniform(2.0, 5.0)
    eye = (dist * math.cos(el) * math.cos(az), 0.1 + dist * math.sin(el), dist * math.cos(el) * math.sin(az))
    at = tuple(rng.uniform(-0.4, 0.4, 3) * np.array([1.0, 0.5, 1.0]))
    return Camera.look_at(eye, at, (0.0, 1.0, 0.0), degrees_to_radians(float(rng.uniform(30.0, 60.0))))


def render_dataset(views: int, views_per_scene: int = 50, seed: int = 0, size: int = SIZE, log=print,
                   target_spp: int = TARGET_SPP):
    """Renders `views` training views; returns a dict of device tensors
    (views x size x size x 4, f32): rad4/alb4/nrm4 (4 spp means), radx/albx/nrmx
    (extra-spp means), target (target_spp mean), and the extra spp per view."""
    import torch

    n = views
    shape = (n, size, size, 4)
    keys = ("rad4", "alb4", "nrm4", "radx", "albx", "nrmx", "target")
    data = {k: torch.zeros(shape, dtype=torch.float32, device="cuda") for k in keys}
    extra = np.zeros(n, np.int64)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(seed + 7)
    t0 = time.perf_counter()
    v = 0
    scene_id = 0
    while v < n:
        sp = scene_params(seed * 100003 + scene_id)
        scene_id += 1
        s, _ = W.displaced_icosphere_scene(freq=sp["freq"], seed=sp["geo_seed"], hdri_size=None)
        s.environment = Environments.hdri_image(W.sky_hdri(1024, 512, sp["sun_elev"], sp["sun_azim"]))
        acc = s.build_acceleration()
        st = RenderSettings(total_samples=1, max_bounces=sp["bounces"], rr_depth=3, estimator=Estimator.NEE,
                            firefly_clamp=FIREFLY_CLAMP)
        for _ in range(min(views_per_scene, n - v)):
            acc.set_camera(random_camera(rng))
            xs = int(rng.choice(EXTRA_SPP))
            extra[v] = xs
            base = 1 + 4 * v
            with torch.cuda.stream(stream):
                h = stream.cuda_stream
                render_device(acc, st, IN_SPP, data["rad4"][v].data_ptr(), size, size, seed=base, stream=h,
                              albedo_device=data["alb4"][v].data_ptr(), normal_device=data["nrm4"][v].data_ptr())
                render_device(acc, st, xs, data["radx"][v].data_ptr(), size, size, seed=base + 1, stream=h,
                              albedo_device=data["albx"][v].data_ptr(), normal_device=data["nrmx"][v].data_ptr())
                render_device(acc, st, target_spp, data["target"][v].data_ptr(), size, size, seed=base + 2, stream=h)
                data["rad4"][v] /= IN_SPP
                data["alb4"][v] /= IN_SPP
                data["nrm4"][v] /= IN_SPP
                data["radx"][v] /= xs
                data["albx"][v] /= xs
                data["nrmx"][v] /= xs
                data["target"][v] /= target_spp
            v += 1
        stream.synchronize()
        acc.destroy()
        log(f"[data] {v}/{n} views, {time.perf_counter() - t0:.1f} s")
    for k in keys:
        bad = ~torch.isfinite(data[k])
        if bad.any():
            data[k][bad] = 0.0
    data["extra_spp"] = extra
    return data


def train(net: Denoiser, data: dict, train_idx: np.ndarray, steps: int, batch: int = 8, crop: int = 128,
          lr: float = 2e-3, seed: int = 0, log=print, log_every: int = 250, time_budget: float = 0.0,
          relmse_frac: float = 0.0, p4: float = 0.3):
    """Adam with linear warm-up and cosine decay.  With a time budget (s) the
    step count is cut after 50 timed steps so that the run fits in it.  The
    last relmse_frac of the steps use the relative-MSE loss; p4 is the share
    of crops whose input is the 4-spp render (the rest use the extra-spp one)."""
    import torch

    rng = np.random.default_rng(seed)
    size = data["rad4"].shape[1]
    bufs = {k: torch.empty((batch, crop, crop, 4), dtype=torch.float32, device="cuda")
            for k in ("rad", "alb", "nrm", "tgt")}
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    warm = max(1, min(500, steps // 10))
    hist = []
    t50 = t0
    it = 0
    while it < steps:
        if time_budget and it == 50:
            stream.synchronize()
            t50 = time.perf_counter()
        if time_budget and it == 250:
            stream.synchronize()
            per = (time.perf_counter() - t50) / 200
            steps = max(251, min(steps, int((time_budget - (time.perf_counter() - t0)) / per) + 250))
            log(f"[train] {per * 1e3:.2f} ms/step -> {steps} steps")
        if relmse_frac and it == int(steps * (1.0 - relmse_frac)):
            net.set_loss(Denoiser.LOSS_RELMSE)
            log(f"[train] step {it}: relative-MSE loss")
        lr_t = lr * min(1.0, (it + 1) / warm) * (0.01 + 0.99 * 0.5 * (1.0 + math.cos(math.pi * it / steps)))
        with torch.cuda.stream(stream):
            for b in range(batch):
                v = int(train_idx[rng.integers(0, len(train_idx))])
                y, x = (int(q) for q in rng.integers(0, size - crop + 1, 2))
                src = "4" if rng.random() < p4 else "x"
                bufs["rad"][b] = data["rad" + src][v, y:y + crop, x:x + crop]
                bufs["alb"][b] = data["alb" + src][v, y:y + crop, x:x + crop]
                bufs["nrm"][b] = data["nrm" + src][v, y:y + crop, x:x + crop]
                bufs["tgt"][b] = data["target"][v, y:y + crop, x:x + crop]
        want = (it % log_every == 0) or it == steps - 1
        loss = net.train_step(bufs["rad"], bufs["alb"], bufs["nrm"], bufs["tgt"], batch, crop, crop, lr_t,
                              want_loss=want, stream=stream.cuda_stream)
        if want:
            hist.append((it, loss))
            log(f"[train] step {it} loss {loss:.5f} lr {lr_t:.2e} {time.perf_counter() - t0:.1f} s")
        it += 1
    stream.synchronize()
    return {"steps": steps, "batch": batch, "crop": crop, "seconds": time.perf_counter() - t0, "loss": hist,
            "relmse_frac": relmse_frac, "p4": p4}


def evaluate(net: Denoiser, data: dict, idx: np.ndarray) -> dict:
    """relMSE against the high-spp target of the plain inputs and of their
    denoised versions, per input spp."""
    import torch

    size = data["rad4"].shape[1]
    out = torch.empty((size, size, 4), dtype=torch.float32, device="cuda")
    res = {}
    for src in ("4", "x"):
        for v in idx:
            v = int(v)
            spp = IN_SPP if src == "4" else int(data["extra_spp"][v])
            net.denoise(data["rad" + src][v], data["alb" + src][v], data["nrm" + src][v], 1.0, out, size, size)
            torch.cuda.synchronize()
            r = data["target"][v][..., :3]
            e_plain = relmse(data["rad" + src][v][..., :3], r)
            e_dn = relmse(out[..., :3], r)
            d = res.setdefault(spp, {"plain": [], "denoised": []})
            d["plain"].append(e_plain)
            d["denoised"].append(e_dn)
    return {int(k): {"views": len(v["plain"]), "plain_relmse": float(np.mean(v["plain"])),
                     "denoised_relmse": float(np.mean(v["denoised"]))} for k, v in sorted(res.items())}


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--views", type=int, default=2000)
    ap.add_argument("--views-per-scene", type=int, default=50)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--holdout", type=float, default=0.05)
    ap.add_argument("--out", default="unet_bf16.npy")
    ap.add_argument("--report", default=None)
    ap.add_argument("--init", default=None, help="start from these weights (bf16 .npy)")
    ap.add_argument("--time-budget", type=float, default=0.0, help="seconds of training (0: all steps)")
    ap.add_argument("--relmse-frac", type=float, default=0.5, help="share of steps with the relative-MSE loss")
    ap.add_argument("--p4", type=float, default=0.3, help="share of 4-spp inputs in the batches")
    ap.add_argument("--size", type=int, default=SIZE, help="view side in pixels")
    ap.add_argument("--target-spp", type=int, default=TARGET_SPP, help="samples per pixel of the targets")
    ap.add_argument("--compare", default=None, help="also evaluate these weights (bf16 .npy) on the held-out views")
    ap.add_argument("--backend", choices=("mma_sync", "tcgen05"), default="mma_sync",
                    help="forward and backward-data convolutions (the shipped weights: mma_sync)")
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    t0 = time.perf_counter()
    data = render_dataset(a.views, a.views_per_scene, a.seed, size=a.size, log=log, target_spp=a.target_spp)
    t_data = time.perf_counter() - t0
    rng = np.random.default_rng(a.seed + 1)
    perm = rng.permutation(a.views)
    nval = max(1, int(a.views * a.holdout))
    val, tr = perm[:nval], perm[nval:]
    net = Denoiser.pretrained(a.init) if a.init else Denoiser(seed=a.seed)
    net.set_backend(Denoiser.TCGEN05 if a.backend == "tcgen05" else Denoiser.MMA_SYNC)
    before = evaluate(net, data, val[:20])
    info = train(net, data, tr, a.steps, a.batch, a.crop, a.lr, a.seed, log=log, time_budget=a.time_budget,
                 relmse_frac=a.relmse_frac, p4=a.p4)
    after = evaluate(net, data, val)
    compared = None
    if a.compare:
        other = Denoiser.pretrained(a.compare)
        compared = evaluate(other, data, val)
        other.destroy()
    net.save(a.out)
    report = {"views": a.views, "train_views": int(len(tr)), "val_views": int(nval), "size": a.size,
              "input_spp": IN_SPP, "extra_spp": list(EXTRA_SPP), "target_spp": a.target_spp,
              "firefly_clamp": FIREFLY_CLAMP, "data_seconds": t_data, "train": info, "val_untrained": before,
              "val": after, "val_compare": compared, "compare_weights": a.compare}
    log(json.dumps({k: report[k] for k in ("val", "val_compare", "data_seconds")}))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(report, f, indent=1)
    torch.cuda.synchronize()
    net.destroy()


if __name__ == "__main__":
    main()
