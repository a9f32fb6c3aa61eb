#!/usr/bin/env python
"""Plain GPU render throughput of the voidray path on one or more GB300s.

Workload: the plain GPU render scene — a geodesic icosphere of 1,997,120
triangles displaced by 4-octave value noise (amplitude 0.1, seed 2) on a
2-triangle ground, materials per 64-triangle patch (Lambertian / metal /
dielectric 1.5), a synthetic 2048x1024 sky + sun HDRI importance-sampled;
1920x1080, 256 samples per pixel, max depth 12, Russian roulette from depth 3,
production (NEE) estimator.  A step renders one full 256-spp frame.
Metric: samples/s (camera paths per second), whole job over all GPUs.

  value  device-resident: the accumulation buffer lives in HBM, timed with
         CUDA events on the render stream (inputs are larger than L2).
  e2e    through the C ABI call with host buffers (vr_render): pinned host
         RGBA copied in and out every step, wall clock.

Multi-GPU: every rank renders its own sample range of the same frame (no
collective on the data path; weak scaling).  `--impl reference` times the CPU
restatement of the reference integrator (the oracle) on the host cores with
the same workload and metric.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
K_EXTEND_DRAM_BYTES_PER_LAUNCH = 2.374e9
sys.path.insert(0, str(ROOT))

CLOCK_FIELDS = ["uuid", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
                "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
                "clocks_event_reasons.sw_power_cap"]


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--spp", type=int, default=256)
    ap.add_argument("--freq", type=int, default=316, help="icosphere frequency (20*f^2 triangles)")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--wavefront", type=int, default=0, help="paths per wavefront (0 = library default)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-work-count", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-autotune", action="store_true", help="library default launch shapes")
    ap.add_argument("--serve-jobs", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=200.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-size", type=int, default=256, help="job image side")
    ap.add_argument("--serve-target", type=float, default=1e-3, help="target relMSE")
    ap.add_argument("--serve-streams", type=int, default=2, help="render streams of the served modes")
    return ap.parse_args()


def workload(args):
    from voidray_gb300 import workloads as W

    scene, st = W.displaced_icosphere_scene(freq=args.freq, width=args.width, height=args.height)
    st.total_samples = args.spp
    if args.wavefront:
        st.wavefront_paths = args.wavefront
    cfg = {
        "workload": "plain GPU render: displaced icosphere + ground, HDRI importance-sampled, 1920x1080 x 256 spp",
        "triangles": scene.num_triangles(),
        "resolution": f"{args.width}x{args.height}",
        "spp": args.spp,
        "max_depth": st.max_bounces,
        "estimator": "NEE + MIS, Russian roulette from depth 3",
        "firefly_clamp": "off",
        "hdri": "2048x1024 sky gradient + sun (sigma 0.5 deg, peak 5e4)",
    }
    return scene, st, cfg


class ClockSampler:
    """nvidia-smi sampled every 200 ms during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + ",".join(CLOCK_FIELDS), "--format=csv,noheader,nounits", "-lms",
                 "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self, uuid: str | None):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != len(CLOCK_FIELDS):
                continue
            if uuid and uuid not in parts[0] and parts[0] not in uuid:
                continue
            rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, val in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], r[4:]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(rows[0][2]),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()),
                "samples": len(rows), "reasons": sorted(reasons)}


def cpu_baseline(scene, st, args, budget_s):
    """The oracle (CPU restatement of the reference integrator, OpenMP over
    pixels like rayon) on a bounded sample of the same frame: 1 spp over a
    contiguous pixel range sized to about `budget_s` seconds."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np

    import pyoracle

    pyoracle.build()
    osc = pyoracle.OracleScene(scene)
    w, h = args.width, args.height
    rgba = np.zeros((h, w, 4), np.float32)
    cores = pyoracle.max_threads()
    start = (h // 2 - 8) * w  # rows through the middle of the frame (sphere and sky)
    probe = 4 * w
    t0 = time.perf_counter()
    osc.render(st, 1, w, h, seed=0, rgba=rgba, pixel_range=(start, start + probe))
    dt = time.perf_counter() - t0
    n = int(min(w * h - start, max(probe, probe * budget_s / max(dt, 1e-3))))
    n = max(w, (n // w) * w)
    start = max(0, (h * w - n) // 2 // w * w)
    t0 = time.perf_counter()
    _, rays = osc.render(st, 1, w, h, seed=0, rgba=rgba, pixel_range=(start, start + n))
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": f"1 spp over {n} pixels (rows {start // w}-{(start + n) // w - 1}) of the "
                      f"{w}x{h} frame, {dt:.1f} s; {int(rays[0])} extend + {int(rays[1])} shadow rays",
            "mrays_per_s": (int(rays[0]) + int(rays[1])) / dt / 1e6}


def serving_benchmark(args):
    """Poisson stream of render jobs drawn like the plain render scene (four
    resident displaced icospheres of 18k-800k triangles with the sky HDRI),
    each to a target relative MSE (estimated from the job's two half-buffers
    without a reference, checked against a 4096-spp reference after the run).
    plain: the requests rendered one at a time (one active job, the plain
    single-scene GPU path); served: continuous batching of every admitted job
    in one launch per pass; served_denoised: the same with AOVs and the
    learned denoiser, each job returning the plain mean or the denoised blend,
    whichever is predicted to be better."""
    import numpy as np
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.denoise import Denoiser
    from voidray_gb300.scene import Estimator, RenderSettings
    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig, poisson_arrivals

    size = args.serve_size
    hdri = vr.Environments.hdri_image(W.sky_hdri(1024, 512))
    pool = []
    for k, freq in enumerate((30, 60, 120, 200)):
        s, _ = W.displaced_icosphere_scene(freq=freq, seed=10 + k, hdri_size=None)
        s.environment = hdri
        acc = s.build_acceleration()
        # the reference's default firefly clamp (3.0): the sun seen through
        # metal / dielectric patches would otherwise keep every job far from
        # the target error
        st = RenderSettings(total_samples=1, max_bounces=8 + k, rr_depth=3, estimator=Estimator.NEE,
                            firefly_clamp=3.0)
        pool.append((acc, st, int(acc.info().device_bytes), s.num_triangles()))
    # 4096-spp references, one per scene (all jobs of a scene share its camera)
    refs = {}
    for acc, st, *_ in pool:
        t = vr.CpuRenderTarget(size, size)
        vr.iterative_render(t, acc, RenderSettings(**{**st.__dict__, "total_samples": 4096}), 4096, seed=99)
        refs[id(acc)] = t.buffer[..., :3].astype(np.float64)

    def relmse(x, r):
        return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))

    rng = np.random.default_rng(5)
    arrivals = poisson_arrivals(args.serve_rate, args.serve_jobs, seed=5)
    picks = [int(rng.integers(0, len(pool))) for _ in arrivals]
    net = Denoiser.pretrained()
    net.set_backend(Denoiser.TCGEN05)   # inference on the tcgen05 convolution
    out = {"jobs": args.serve_jobs, "rate_per_s": args.serve_rate, "image": f"{size}x{size}",
           "target_relmse": args.serve_target, "scenes_triangles": [p[3] for p in pool],
           "error_estimate": "half-buffer variance of the mean / (m^2 + 1e-2); denoised: reference-free "
                             "prediction of the blend's error from the halves",
           "reference": "4096 spp per scene", "denoiser": "U-Net 32/64/128/256, bf16, shipped weights",
           "warmup": "6 untimed jobs per mode on the same backend before the timed arrivals"}
    spp_pass = 32
    # plain: the progressive single-scene loop, one job at a time, 32 spp per
    # pass, stopping on the same half-buffer estimate.  served: continuous
    # batching with predictive per-job pass sizes (16M-path passes, jobs take
    # them in admission order).  served_denoised: the same plus AOVs and the
    # denoiser blend.
    plain_cfg = ServerConfig(memory_budget=150 * 10**9, max_active=1, spp_per_pass=spp_pass, min_samples=64)
    # the denoised path starts with a larger first pass: its blend estimate
    # needs a less noisy input, and its per-job sample counts are smaller
    served_cfg = ServerConfig(memory_budget=150 * 10**9, max_active=64, adaptive=True, pipelined=True,
                              pass_paths=1 << 24, first_pass_spp=64, min_samples=64, overshoot=1.15, max_inflight=3)
    served_dn_cfg = ServerConfig(memory_budget=150 * 10**9, max_active=64, adaptive=True, pipelined=True,
                                 pass_paths=1 << 24, first_pass_spp=128, min_samples=64, overshoot=1.2,
                                 max_inflight=3)
    out["served_config"] = {"adaptive": True, "pipelined": True, "pass_paths": 1 << 24, "max_active": 64,
                            "max_inflight": 3, "render_streams": args.serve_streams,
                            "first_pass_spp": {"served": 64, "served_denoised": 128},
                            "overshoot": {"served": 1.15, "served_denoised": 1.2}}
    modes = (("plain", plain_cfg, False), ("served", served_cfg, False), ("served_denoised", served_dn_cfg, True))
    for name, cfg, dn in modes:
        active = cfg.max_active
        backend = GpuBackend(denoiser=net if dn else None, render_streams=args.serve_streams if cfg.pipelined else 1)
        # untimed warm-up on the same backend: graph shapes, denoiser
        # workspaces and lazily loaded kernels, for every mode alike
        warm = Server(backend, cfg)
        warm.run([(0.0, JobRequest(pool[k % len(pool)][0], pool[k % len(pool)][1], size, size, max_samples=256,
                                   target_relmse=args.serve_target, seed=500 + k, scene_bytes=pool[k % len(pool)][2],
                                   denoise=dn)) for k in range(6)])
        backend.time = {k: 0.0 for k in backend.time}
        backend.denoise_calls = 0
        requests = []
        for i, t in enumerate(arrivals):
            acc, st, nbytes, _ = pool[picks[i]]
            requests.append((float(t), JobRequest(acc, st, size, size, max_samples=2048,
                                                  target_relmse=args.serve_target, seed=1000 + i,
                                                  scene_bytes=nbytes, denoise=dn)))
        srv = Server(backend, cfg)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        srv.run(requests)
        wall = time.perf_counter() - t0
        lat = srv.latencies()
        jobs = list(srv.jobs.values())
        samples = sum(j.samples * j.req.width * j.req.height for j in jobs)
        errs = [relmse(j.result.astype(np.float64), refs[id(j.req.scene)]) for j in jobs]
        out[name] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                     "jobs_per_s": len(lat) / wall, "samples_per_s": samples / wall, "wall_s": wall,
                     "passes": srv.passes, "max_active": active,
                     "mean_spp": float(np.mean([j.samples for j in jobs])),
                     "true_relmse_p50": float(np.median(errs)), "true_relmse_p99": float(np.percentile(errs, 99)),
                     "true_relmse_max": float(np.max(errs))}
        out[name]["host_phase_s"] = dict(backend.time)
        if dn:
            out[name]["denoised_jobs"] = int(sum(np.any(np.asarray(j.alpha) > 0) for j in jobs))
            out[name]["mean_alpha"] = float(np.mean([np.mean(j.alpha) for j in jobs]))
            out[name]["denoiser_calls"] = backend.denoise_calls
        backend.destroy()
    out["p50_speedup_served"] = out["plain"]["p50_s"] / out["served"]["p50_s"]
    out["p50_speedup_served_denoised"] = out["plain"]["p50_s"] / out["served_denoised"]["p50_s"]
    out["throughput_ratio_served"] = out["served"]["jobs_per_s"] / out["plain"]["jobs_per_s"]
    out["throughput_ratio_served_denoised"] = out["served_denoised"]["jobs_per_s"] / out["plain"]["jobs_per_s"]
    out["equal_time"] = denoiser_equal_time(pool, refs, net, size)
    net.destroy()
    for acc, *_ in pool:
        acc.destroy()
    return out


def denoiser_equal_time(pool, refs, net, size):
    """Acceptance rule of the denoiser: a denoised frame must beat the plain
    frame rendered in the same time.  For each scene and input spp: time the
    AOV render plus the denoiser (CUDA events), render the plain frame with
    as many samples as fit in that time, and compare both with the 4096-spp
    reference."""
    import numpy as np
    import torch

    from voidray_gb300.scene import render_device

    stream = torch.cuda.Stream()
    h = stream.cuda_stream
    rows = []
    bufs = [torch.zeros((size, size, 4), dtype=torch.float32, device="cuda") for _ in range(4)]

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            fn()
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for k, (acc, st, *_) in enumerate(pool):
        # warm-up: scratch allocation of the AOV render and the denoiser workspace
        render_device(acc, st, 1, bufs[0].data_ptr(), size, size, seed=6, stream=h,
                      albedo_device=bufs[1].data_ptr(), normal_device=bufs[2].data_ptr())
        net.denoise(bufs[0], bufs[1], bufs[2], 1.0, bufs[3], size, size, stream=h)
        render_device(acc, st, 1, bufs[0].data_ptr(), size, size, seed=6, stream=h)
        for spp in (4, 16, 64, 256):
            with torch.cuda.stream(stream):  # ordered after everything rendered on this stream
                for b in bufs:
                    b.zero_()
            stream.synchronize()
            t_r = timed(lambda: render_device(acc, st, spp, bufs[0].data_ptr(), size, size, seed=7, stream=h,
                                              albedo_device=bufs[1].data_ptr(), normal_device=bufs[2].data_ptr()))
            t_d = timed(lambda: net.denoise(bufs[0], bufs[1], bufs[2], 1.0 / spp, bufs[3], size, size, stream=h))
            den = bufs[3][..., :3].double().cpu().numpy()
            # plain frame in the same time: samples scale with the time budget
            t_plain_1 = timed(lambda: render_device(acc, st, spp, bufs[0].data_ptr(), size, size, seed=8, stream=h))
            spp_eq = max(spp, int(spp * (t_r + t_d) / max(t_plain_1, 1e-3)))
            with torch.cuda.stream(stream):
                bufs[0].zero_()
            t_eq = timed(lambda: render_device(acc, st, spp_eq, bufs[0].data_ptr(), size, size, seed=8, stream=h))
            stream.synchronize()
            plain = (bufs[0][..., :3].double() / spp_eq).cpu().numpy()
            r = refs[id(acc)]
            e_d = float(np.mean((den - r) ** 2 / (r * r + 1e-2)))
            e_p = float(np.mean((plain - r) ** 2 / (r * r + 1e-2)))
            rows.append({"scene": k, "spp": spp, "render_ms": t_r, "denoise_ms": t_d, "plain_spp": spp_eq,
                         "plain_ms": t_eq, "denoised_relmse": e_d, "plain_relmse": e_p,
                         "denoised_wins": e_d < e_p})
    return rows


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    scene, st, cfg = workload(args)
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np

    import pyoracle

    pyoracle.build()
    osc = pyoracle.OracleScene(scene)
    w, h = args.width, args.height
    rgba = np.zeros((h, w, 4), np.float32)
    # size a step to about 8 s of CPU work
    start = (h // 2) * w
    t0 = time.perf_counter()
    osc.render(st, 1, w, h, rgba=rgba, pixel_range=(start, start + 2 * w))
    dt = time.perf_counter() - t0
    n = int(min(w * h, max(w, 2 * w * 8.0 / max(dt, 1e-3))))
    n = max(w, (n // w) * w)
    start = (h * w - n) // 2 // w * w
    for _ in range(args.warmup):
        osc.render(st, 1, w, h, rgba=rgba, pixel_range=(start, start + n))
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        osc.render(st, 1, w, h, first_sample=k + 1, rgba=rgba, pixel_range=(start, start + n))
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    cores = pyoracle.max_threads()
    line = {
        "impl": "reference", "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port",
                         "sample": f"each step 1 spp over {n} pixels of the {w}x{h} frame"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import _native as N

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = vr.lib()
    scene, st, cfg = workload(args)
    t0 = time.perf_counter()
    acc = scene.build_acceleration()
    build_s = time.perf_counter() - t0
    info = acc.info()
    w, h, spp = args.width, args.height, args.spp
    npx = w * h
    tuning = None
    if not args.no_autotune and not args.wavefront:
        # launch shapes for this workload class (cached per GPU / scene / image / spp bucket)
        from voidray_gb300 import autotune

        tuning = autotune.tune(acc, st, w, h, spp)
        st = autotune.apply(tuning, st)
    cst = st.to_c()
    # a dedicated stream: its handle is non-zero, so the library launches on it
    # and the CUDA events below bracket the kernels (NULL would select the
    # scene's own stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = C.c_void_p(stream.cuda_stream)
    assert sh.value, "render stream handle must be non-zero"
    accum = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    # each rank and step renders its own sample range
    base = rank * (args.warmup + args.steps + 2) * spp

    def step(k):
        N.check(lib.vr_render_device(acc.handle, C.byref(cst), spp, accum.data_ptr(), w, h, 0, base + k * spp, sh))

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    N.check(lib.vr_scene_synchronize(acc.handle))
    N.check(lib.vr_scene_instrument(acc.handle, N.INSTR_STAGE_TIMES))
    st0 = acc.stats()
    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    clocks = ClockSampler()
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        step(args.warmup + k)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop(uuid)
    N.check(lib.vr_scene_synchronize(acc.handle))
    ins = N.vr_instrument()
    N.check(lib.vr_scene_instrument_get(acc.handle, C.byref(ins)))
    st1 = acc.stats()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    samples_per_rank = spp * npx * args.steps
    value = samples_per_rank * world / (ms / 1e3)
    ext_rays = st1.extend_rays - st0.extend_rays
    shd_rays = st1.shadow_rays - st0.shadow_rays
    launches = int(sum(ins.stage_launches[i] for i in range(5)))
    # wave_stats runs once per wavefront (with accumulate), finalize once per step
    gpu_launches = launches + int(ins.stage_launches[4]) + args.steps
    stage = {N.STAGES[i]: {"ms": round(ins.stage_ms[i], 3), "launches": int(ins.stage_launches[i])}
             for i in range(5)}

    # traversal work of the same frames (deterministic streams): counting run, untimed
    roofline = None
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    default_workload = (args.width, args.height, args.spp, args.freq) == (1920, 1080, 256, 316)
    if not args.no_work_count:
        N.check(lib.vr_scene_instrument(acc.handle, N.INSTR_WORK))
        c0 = acc.stats()
        step(args.warmup)  # same sample range as the first timed step
        N.check(lib.vr_scene_synchronize(acc.handle))
        wk = N.vr_instrument()
        N.check(lib.vr_scene_instrument_get(acc.handle, C.byref(wk)))
        c1 = acc.stats()
        rays1 = c1.extend_rays - c0.extend_rays
        # algorithmic bytes of the extend (closest-hit) stage for one frame:
        # 32 B ray in + 16 B hit out per ray, 64 B per inner-node visit, 48 B per triangle test
        alg_bytes = 48 * rays1 + 64 * wk.extend_node_visits + 48 * wk.extend_tri_tests
        ext_ms_per_frame = ins.stage_ms[1] / args.steps
        ext_launches_per_frame = ins.stage_launches[1] / args.steps
        achieved = alg_bytes / (ext_ms_per_frame / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": "k_extend (closest-hit BVH2 traversal)", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    # ncu dram__bytes_read.sum + dram__bytes_write.sum per k_extend launch, mean over the 12
                    # depths of one full-size wavefront of this workload (a constant from that capture:
                    # profiles/k_extend_k_shadow_1920x1080_256spp_dram_traffic.md); only valid at the
                    # default workload
                    "traffic": K_EXTEND_DRAM_BYTES_PER_LAUNCH if default_workload else None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback",
                    "algorithmic_bytes_per_launch": alg_bytes / max(ext_launches_per_frame, 1),
                    "avg_launch_ms": ext_ms_per_frame / max(ext_launches_per_frame, 1),
                    "per_ray": {"node_visits": wk.extend_node_visits / max(rays1, 1),
                                "tri_tests": wk.extend_tri_tests / max(rays1, 1)},
                    "extend_share_of_step": ins.stage_ms[1] / max(sum(ins.stage_ms[i] for i in range(5)), 1e-9)}

    # e2e through the C ABI with host buffers (pinned), wall clock
    host = torch.zeros((h, w, 4), dtype=torch.float32).pin_memory()
    hp = host.data_ptr()
    e2e_steps = max(1, args.steps)
    N.check(lib.vr_render(acc.handle, C.byref(cst), spp, hp, w, h, 1, base, ))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        N.check(lib.vr_render(acc.handle, C.byref(cst), spp, hp, w, h, 1, base + (k + 1) * spp))
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": spp * npx * e2e_steps * world / e2e_s, "unit": "samples/s",
           "h2d_bytes_per_step": npx * 16, "d2h_bytes_per_step": npx * 16,
           "call": "vr_render (host RGBA buffer, pinned)"}
    out_img = host.numpy()
    finite = bool(np.isfinite(out_img).all())

    acc.destroy()
    serve = None
    if rank == 0 and world == 1 and not args.no_serve:
        serve = serving_benchmark(args)
    dnb = None
    if rank == 0 and world == 1 and not args.no_serve:
        # the denoiser's kernels on a 1920x1080 frame (tensor-bound; see its roofline)
        from voidray_gb300 import denoise_bench

        dnb = denoise_bench.run(1920, 1080, iters=10)
        dnb["roofline"] = {"bound": "tensor", "kernel": "U-Net forward (15 3x3 convolutions), tcgen05",
                           "achieved": dnb["tcgen05"]["tflops"], "peak": dnb["peak_tflops"], "unit": "TFLOP/s",
                           "frac": dnb["tcgen05"]["frac"], "peak_source": dnb["peak_source"]}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(scene, st, args, args.cpu_seconds)
    if rank == 0:
        cfg.update({"l2": f"inputs larger than L2: scene {info.device_bytes / 1e6:.0f} MB on device, "
                          f"accumulation {npx * 16 / 1e6:.0f} MB",
                    "bvh": {"nodes": int(info.num_nodes), "max_depth": int(info.max_depth),
                            "sah_cost": round(info.sah_cost, 2), "build_s": round(build_s, 2)},
                    "wavefront_paths": st.wavefront_paths or (1 << 26),
                    "parallelism": f"replicas x{world}, disjoint sample ranges",
                    "tuning": tuning})
        line = {
            "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "mrays_per_s": (ext_rays + shd_rays) / (ms / 1e3) / 1e6,
            "rays": {"extend": int(ext_rays), "shadow": int(shd_rays)},
            "stages": stage, "gpu_launches": gpu_launches, "clocks": clk, "e2e": e2e, "roofline": roofline,
            "cpu_baseline": cpu, "image_finite": finite, "serving": serve, "denoiser": dnb,
        }
        print(json.dumps(line), flush=True)
    acc.destroy()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
