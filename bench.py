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
# bytes a 4-wide node visit reads: six float4 of child boxes and one of child codes
NODE_BYTES = 112
# DRAM and L2 bytes per closest-hit ray of k_extend on the default scene,
# from an ncu capture of all twelve k_extend launches of one 960x540 x 32 spp
# frame of it (the same 2M-triangle scene and HDRI, 34.4M extend rays); the
# bench scales them to its own launches by the extend rays per launch
K_EXTEND_DRAM_BYTES_PER_RAY = 149.9
K_EXTEND_L2_BYTES_PER_RAY = 1005.1
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
    ap.add_argument("--serve-large-jobs", type=int, default=16,
                    help="requests of the 1920x1080, 2M-triangle serving run (0 = skip)")
    ap.add_argument("--no-isect", action="store_true", help="skip the intersection microbenchmark")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched workload")
    ap.add_argument("--no-cornell", action="store_true", help="skip the Cornell box workload")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=2, help="timed steps of the batched workload")
    ap.add_argument("--isect-tris", type=int, default=1_000_000)
    ap.add_argument("--isect-rays", type=int, default=16_777_216)
    ap.add_argument("--isect-reps", type=int, default=5, help="timed launches per query kind")
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


def timed_on(stream, fn, reps):
    """Mean ms of `reps` calls of fn() enqueued on `stream`, CUDA events on that stream."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def intersection_benchmark(args, hbm_peak, peak_source):
    """The intersection microbenchmark: a soup of 1,000,000 triangles (centres
    uniform in [0,1]^3, vertex offsets N(0, 0.01^2), seed 1) in the SAH BVH and
    16,777,216 rays (half pinhole rays from z=-1 over 4096x2048, half with
    origins uniform in the cube and directions uniform on the sphere, tmax
    inf), closest hit and any hit through vr_intersect_device.  Rays (537 MB)
    and hits (268 MB) are larger than L2.  The CPU leg runs the oracle's
    restatement of SceneAcceleration::hit (median BVH, both children visited)
    on every 16th ray."""
    import numpy as np
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import _native as N
    from voidray_gb300 import workloads as W

    lib = vr.lib()
    n_tri, n_rays = args.isect_tris, args.isect_rays
    scene = W.soup_scene(n_tri, seed=1)
    rays = W.soup_rays(n_rays, seed=1)
    t0 = time.perf_counter()
    acc = scene.build_acceleration()
    build_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    dr = torch.from_numpy(rays).cuda()
    hits = torch.empty((n_rays, 4), dtype=torch.float32, device="cuda")
    out = {"workload": f"{n_tri} triangle soup (seed 1), {n_rays} rays (half pinhole 4096x2048, half incoherent)",
           "bvh_build_s": round(build_s, 2), "l2": "rays 537 MB + hits 268 MB per launch, larger than L2"}
    for name, any_hit in (("closest", 0), ("any", 1)):
        def launch():
            N.check(lib.vr_intersect_device(acc.handle, dr.data_ptr(), n_rays, hits.data_ptr(), any_hit, sh))
        for _ in range(3):
            launch()
        ms = timed_on(stream, launch, args.isect_reps)
        nv, nt = C.c_uint64(), C.c_uint64()
        N.check(lib.vr_intersect_count_device(acc.handle, dr.data_ptr(), n_rays, any_hit, C.byref(nv), C.byref(nt),
                                              sh))
        alg = 48 * n_rays + NODE_BYTES * nv.value + 48 * nt.value
        achieved = alg / (ms / 1e3) / 1e9
        out[name] = {"mrays_per_s": n_rays / (ms / 1e3) / 1e6, "ms_per_launch": ms, "launches": args.isect_reps,
                     "node_visits_per_ray": nv.value / n_rays, "tri_tests_per_ray": nt.value / n_rays,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                                  "frac": achieved / hbm_peak, "peak_source": peak_source,
                                  "algorithmic_bytes_per_launch": alg}}
    torch.cuda.synchronize()
    g = hits.cpu().numpy()  # any-hit result of the last launch
    N.check(lib.vr_intersect_device(acc.handle, dr.data_ptr(), n_rays, hits.data_ptr(), 0, sh))
    torch.cuda.synchronize()  # the launch ran on `stream`, not on torch's current stream
    closest = hits.cpu().numpy()
    ids_c, ids_a = closest[:, 0].view(np.uint32), g[:, 0].view(np.uint32)
    out["hit_fraction"] = float((ids_c != 0xFFFFFFFF).mean())
    out["any_agrees_with_closest_on_hit_miss"] = bool(np.array_equal(ids_c != 0xFFFFFFFF, ids_a != 0xFFFFFFFF))
    # end to end through the host-buffer call: rays in and hits out through pinned host memory
    hrays = torch.from_numpy(rays).pin_memory()
    hhits = torch.empty((n_rays, 4), dtype=torch.float32).pin_memory()
    N.check(lib.vr_intersect(acc.handle, hrays.data_ptr(), n_rays, hhits.data_ptr(), 0))
    t0 = time.perf_counter()
    for _ in range(args.isect_reps):
        N.check(lib.vr_intersect(acc.handle, hrays.data_ptr(), n_rays, hhits.data_ptr(), 0))
    e2e_s = (time.perf_counter() - t0) / args.isect_reps
    out["e2e_closest"] = {"mrays_per_s": n_rays / e2e_s / 1e6, "call": "vr_intersect (host rays and hits, pinned)",
                          "h2d_bytes_per_call": n_rays * 32, "d2h_bytes_per_call": n_rays * 16}
    if not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        pyoracle.build()
        osc = pyoracle.OracleScene(scene)
        sub = np.ascontiguousarray(rays[::16])
        t0 = time.perf_counter()
        oh, second = osc.intersect(sub, mode=0, second=True)
        dt = time.perf_counter() - t0
        mism = oh[:, 0].view(np.uint32) != ids_c[::16]
        t1 = oh[:, 1]
        with np.errstate(invalid="ignore"):
            tie = np.isfinite(second) & ((second - t1) <= 1e-6 * np.abs(t1))
        out["cpu_baseline"] = {"mrays_per_s": len(sub) / dt / 1e6, "cores": pyoracle.max_threads(), "kind": "port",
                               "sample": f"every 16th ray ({len(sub)} rays), closest hit, {dt:.1f} s"}
        out["parity_on_cpu_sample"] = {"rays": len(sub), "id_mismatches": int(mism.sum()),
                                       "near_ties": int(tie.sum()), "mismatches_outside_near_ties":
                                       int((mism & ~tie).sum())}
    acc.destroy()
    return out


def cornell_benchmark(args):
    """The Cornell box workload (code-built box, 34 triangles, 256x256, 16 spp,
    depth 8, Russian roulette from depth 3, the reference estimator, PCG32 seed
    0, ACES tonemap), whole frames: on the GPU through vr_render_device +
    vr_tonemap_device (device-timed) and vr_render + vr_tonemap (host buffers,
    wall clock), and by the oracle on all host cores. The first GPU frame and
    the oracle's frame are compared pixel for pixel, and after the tonemap."""
    import numpy as np
    import torch

    import voidray_gb300 as vr
    from voidray_gb300 import _native as N
    from voidray_gb300 import workloads as W
    from voidray_gb300.scene import ColorManagementSettings, Tonemap

    lib = vr.lib()
    w = h = 256
    spp = 16
    scene, st = W.cornell_box(width=w, height=h, spp=spp, max_depth=8, rr_depth=3)
    cm = ColorManagementSettings(tonemap=Tonemap.ACES, gamma=2.2, exposure=0.0).to_c()
    acc = scene.build_acceleration()
    cst = st.to_c()
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    accum = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ldr = torch.empty_like(accum)

    def frame(k):
        accum.zero_()
        N.check(lib.vr_render_device(acc.handle, C.byref(cst), spp, accum.data_ptr(), w, h, 0, k * spp, sh))
        N.check(lib.vr_tonemap_device(accum.data_ptr(), ldr.data_ptr(), w, h, C.byref(cm), 1.0, sh))

    with torch.cuda.stream(stream):
        frame(0)
        torch.cuda.synchronize()
        g_hdr, g_ldr = accum.cpu().numpy(), ldr.cpu().numpy()
        for k in range(3):
            frame(k + 1)
        frames = 200
        ms = timed_on(stream, lambda: [frame(k + 4) for k in range(frames)], 1) / frames
    out = {"workload": "Cornell box, 34 triangles, 256x256 x 16 spp, depth 8, RR from depth 3, reference "
                       "estimator, seed 0, ACES", "frames": frames,
           "ms_per_frame": ms, "samples_per_s": w * h * spp / (ms / 1e3)}
    # host buffers through the C ABI: the accumulation buffer in and out, the LDR frame out
    host = torch.zeros((h, w, 4), dtype=torch.float32).pin_memory()
    hl = torch.empty_like(host).pin_memory()
    reps = 50
    t0 = time.perf_counter()
    for k in range(reps):
        host.zero_()
        N.check(lib.vr_render(acc.handle, C.byref(cst), spp, host.data_ptr(), w, h, 0, k * spp))
        N.check(lib.vr_tonemap(host.data_ptr(), hl.data_ptr(), w, h, C.byref(cm), 1.0))
    e2e_s = (time.perf_counter() - t0) / reps
    out["e2e"] = {"samples_per_s": w * h * spp / e2e_s, "ms_per_frame": e2e_s * 1e3,
                  "call": "vr_render + vr_tonemap (host buffers, pinned)"}
    acc.destroy()
    if not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        pyoracle.build()
        osc = pyoracle.OracleScene(scene)
        t0 = time.perf_counter()
        o_hdr, rays = osc.render(st, spp, w, h, seed=0)
        dt = time.perf_counter() - t0
        o_ldr = pyoracle.tonemap(o_hdr, int(Tonemap.ACES), 2.2, 0.0, 1.0)
        out["cpu_baseline"] = {"samples_per_s": w * h * spp / dt, "ms_per_frame": dt * 1e3,
                               "cores": pyoracle.max_threads(), "kind": "port",
                               "sample": f"the whole frame, {int(rays[0])} rays"}
        d = o_hdr[..., :3].astype(np.float64) - g_hdr[..., :3]
        # the integrator's arithmetic is reproduced operation for operation
        # (bit-equal pixels); the tonemap's pow is the device's and the host's
        # own function, so the LDR frames agree to a few ulp.  The fitted ACES
        # curve maps black slightly below zero, and pow(negative, 1/gamma) is
        # NaN on both sides: those channels are compared as NaN positions.
        gl, ol = g_ldr[..., :3].astype(np.float64), o_ldr[..., :3].astype(np.float64)
        both = np.isfinite(gl) & np.isfinite(ol)
        out["parity"] = {"pixels_bit_equal": float(np.mean(np.all(g_hdr == o_hdr, axis=-1))),
                         "relmse": float(np.mean(d * d / (o_hdr[..., :3].astype(np.float64) ** 2 + 1e-2))),
                         "ldr_max_abs_diff": float(np.max(np.abs(gl - ol)[both])) if both.any() else 0.0,
                         "ldr_nan_channels": int(np.isnan(ol).sum()),
                         "ldr_nan_positions_equal": bool(np.array_equal(np.isnan(gl), np.isnan(ol)))}
    return out


def batch_benchmark(args):
    """The batched workload: 64 displaced-icosphere scenes (10k-2M triangles,
    log-uniform; materials per 64-triangle patch; one shared 2048x1024 sky +
    sun HDRI), each with its own resolution from {256^2, 512^2, 1280x720,
    1920x1080}, spp log-uniform in 4-256 and depth 8-12, rendered by one
    vr_batch per pass (all jobs share every wavefront launch), each wavefront's
    stage sequence replayed as a CUDA graph, launch shapes and wavefront size
    from the batch autotuner.  A step renders every job's full spp once.
    Beside it the same jobs rendered one at a time (one single-job render call
    each, library launch shapes), and every job's batched image compared bit
    for bit with its image rendered alone."""
    import numpy as np
    import torch

    from voidray_gb300 import autotune
    from voidray_gb300 import workloads as W
    from voidray_gb300.batch import Batch, RenderJob

    t0 = time.perf_counter()
    mix = W.batched_job_set(args.batch_jobs, seed=4)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    jobs = []
    for s, st, spp, w, h, seed in mix:
        jobs.append((s.build_acceleration(), st, spp, w, h, seed))
    build_s = time.perf_counter() - t0
    ntri = [int(a.info().num_triangles) for a, *_ in jobs]
    samples = sum(spp * w * h for _, _, spp, w, h, _ in jobs)
    out = {"jobs": len(jobs), "triangles_min_max_sum": [min(ntri), max(ntri), sum(ntri)],
           "pixels": sum(w * h for _, _, _, w, h, _ in jobs), "samples_per_step": samples,
           "spp_min_max": [min(j[2] for j in jobs), max(j[2] for j in jobs)],
           "scene_gen_s": round(gen_s, 1), "bvh_build_s": round(build_s, 1),
           "device_bytes": int(sum(a.info().device_bytes for a, *_ in jobs))}
    prev_tuning = autotune.get_tuning()
    tuning = autotune.tune_batch(jobs)
    out["tuning"] = tuning
    stream = torch.cuda.Stream()
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, _, _, w, h, _ in jobs]
    first = [torch.zeros_like(o) for o in outs]
    batch = Batch(int(tuning["max_wave_paths"]))
    batch.set_graphs(True)

    def step(k, bufs):
        batch.render([RenderJob(acc, st, spp, o.data_ptr(), w, h, seed, k * spp)
                      for (acc, st, spp, w, h, seed), o in zip(jobs, bufs)], stream.cuda_stream)

    step(0, first)  # direct launches; pass 0 is also the bit-identity sample
    for k in range(1, 3):  # graph capture, then replay
        step(k, outs)
    ms = timed_on(stream, lambda: [step(3 + k, outs) for k in range(args.batch_steps)], 1) / args.batch_steps
    batch.synchronize(stream.cuda_stream)
    caps, reps = batch.graph_stats()
    out.update({"ms_per_step": ms, "samples_per_s": samples / (ms / 1e3), "steps": args.batch_steps,
                "graph_captures": caps, "graph_replays": reps})
    batch.destroy()
    # the same jobs one at a time (one single-job render call each, library
    # launch shapes and wavefronts of up to 2^28 paths, one shared scratch); pass 0 again
    # for the comparison
    autotune.set_tuning({k: v for k, v in autotune.DEFAULT.items() if k != "wavefront_paths"})
    alone = [torch.zeros_like(o) for o in outs]
    single = Batch(1 << 28)

    def alone_pass():
        for (acc, st, spp, w, h, seed), o in zip(jobs, alone):
            single.render([RenderJob(acc, st, spp, o.data_ptr(), w, h, seed, 0)], stream.cuda_stream)

    ms_alone = timed_on(stream, alone_pass, 1)
    single.synchronize(stream.cuda_stream)
    single.destroy()
    autotune.set_tuning(prev_tuning)
    same = [bool(torch.equal(a, b)) for a, b in zip(alone, first)]
    out.update({"alone_ms_per_step": ms_alone, "alone_samples_per_s": samples / (ms_alone / 1e3),
                "speedup_vs_alone": ms_alone / ms, "jobs_bit_identical_to_alone": int(sum(same))})
    for acc, *_ in jobs:
        acc.destroy()
    return out


def serving_scenes(size_label, freqs, seeds, hdri, max_bounces_base=8):
    """Resident scenes of a serving run: displaced icospheres (materials per
    64-triangle patch) sharing one HDRI, with the reference's default firefly
    clamp (3.0): the sun seen through metal / dielectric patches would
    otherwise keep every job far from the target error."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.scene import Estimator, RenderSettings

    pool = []
    for k, (freq, seed) in enumerate(zip(freqs, seeds)):
        s, _ = W.displaced_icosphere_scene(freq=freq, seed=seed, hdri_size=None)
        s.environment = hdri
        acc = s.build_acceleration()
        st = RenderSettings(total_samples=1, max_bounces=max_bounces_base + k, rr_depth=3, estimator=Estimator.NEE,
                            firefly_clamp=3.0)
        pool.append((acc, st, int(acc.info().device_bytes), s.num_triangles()))
    return pool


def serving_references(pool, w, h, spp=4096):
    """Per scene: the `spp`-sample reference as the mean of two independent
    halves A, B (disjoint sample ranges), and the reference's own noise term
    mean(Var(ref) / (ref^2 + 1e-2)) with Var(ref) = (A - B)^2 / 4 per pixel
    and channel; a job's error against the true image is its measured error
    minus this term (the job and the reference are independent)."""
    import numpy as np

    import voidray_gb300 as vr
    from voidray_gb300.scene import RenderSettings

    refs = {}
    for acc, st, *_ in pool:
        halves = []
        for first in (0, spp // 2):
            t = vr.CpuRenderTarget(w, h)
            vr.iterative_render(t, acc, RenderSettings(**{**st.__dict__, "total_samples": spp // 2}), spp // 2,
                                seed=99, first_sample=first)
            halves.append(t.buffer[..., :3].astype(np.float64))
        ref = 0.5 * (halves[0] + halves[1])
        noise = float(np.mean((halves[0] - halves[1]) ** 2 / 4.0 / (ref * ref + 1e-2)))
        refs[id(acc)] = (ref, noise)
    return refs


def serving_run(pool, refs, net, w, h, n_jobs, rate, target, streams, plain_passes, warm_jobs, max_samples,
                dn_first_pass=96, only=None, dn_overshoot=1.2, max_inflight=3):
    """One Poisson request stream (seeded) served by every mode:
    plain_<n>: the plain single-scene GPU path, one job at a time, n spp per
    pass (plain_adaptive: one job at a time with predictive pass sizes, the
    job's predicted remaining samples in one pass); served: continuous
    batching of every admitted job in one launch per pass; served_denoised:
    the same with AOVs and the learned denoiser, each job returning the plain
    mean or the denoised blend, whichever is predicted to be better.  The
    best plain mode (lowest p50) is the denominator of the ratios."""
    import numpy as np
    import torch

    from voidray_gb300.serve import GpuBackend, JobRequest, Server, ServerConfig, poisson_arrivals

    rng = np.random.default_rng(5)
    arrivals = poisson_arrivals(rate, n_jobs, seed=5)
    picks = [int(rng.integers(0, len(pool))) for _ in arrivals]
    out = {"jobs": n_jobs, "rate_per_s": rate, "image": f"{w}x{h}", "target_relmse": target,
           "scenes_triangles": [p[3] for p in pool],
           "error_estimate": "half-buffer variance of the mean / (m^2 + 1e-2); denoised: reference-free "
                             "prediction of the blend's error from the halves",
           "reference": "4096 spp per scene (two independent 2048-spp halves); true_relmse = measured relMSE "
                        "against it minus its own noise term",
           "reference_noise_relmse": [refs[id(p[0])][1] for p in pool],
           "denoiser": "U-Net 32/64/128/256, bf16, shipped weights",
           "warmup": f"{warm_jobs} untimed jobs per mode on the same backend before the timed arrivals"}
    modes = []
    for n in plain_passes:
        if n == "adaptive":
            modes.append(("plain_adaptive", ServerConfig(memory_budget=150 * 10**9, max_active=1, adaptive=True,
                                                         pass_paths=1 << 26, first_pass_spp=64, min_samples=64,
                                                         overshoot=1.15), False))
        else:
            modes.append((f"plain_{n}", ServerConfig(memory_budget=150 * 10**9, max_active=1, spp_per_pass=n,
                                                     min_samples=64), False))
    modes.append(("served", ServerConfig(memory_budget=150 * 10**9, max_active=64, adaptive=True, pipelined=True,
                                         pass_paths=1 << 24, first_pass_spp=64, min_samples=64, overshoot=1.15,
                                         max_inflight=max_inflight), False))
    # the denoised path starts with a larger first pass: its blend estimate
    # needs a less noisy input (a smaller first pass makes the prediction
    # noisier and more conservative: 32 spp first passes ended at 134 spp per
    # 1080p job on average, 96 spp ones at 98)
    modes.append(("served_denoised", ServerConfig(memory_budget=150 * 10**9, max_active=64, adaptive=True,
                                                  pipelined=True, pass_paths=1 << 24, first_pass_spp=dn_first_pass,
                                                  min_samples=min(64, dn_first_pass), overshoot=dn_overshoot,
                                                  max_inflight=max_inflight), True))
    if only is not None:
        modes = [m for m in modes if m[0] in only]
    out["served_config"] = {"adaptive": True, "pipelined": True, "pass_paths": 1 << 24, "max_active": 64,
                            "max_inflight": max_inflight, "fill_paths": ServerConfig.fill_paths,
                            "render_streams": streams,
                            "first_pass_spp": {"served": 64, "served_denoised": dn_first_pass},
                            "overshoot": {"served": 1.15, "served_denoised": dn_overshoot}}
    for name, cfg, dn in modes:
        backend = GpuBackend(denoiser=net if dn else None, render_streams=streams if cfg.pipelined else 1)
        # untimed warm-up on the same backend: graph shapes, denoiser
        # workspaces and lazily loaded kernels, for every mode alike
        warm = Server(backend, cfg)
        warm.run([(0.0, JobRequest(pool[k % len(pool)][0], pool[k % len(pool)][1], w, h, max_samples=256,
                                   target_relmse=target, seed=500 + k, scene_bytes=pool[k % len(pool)][2],
                                   denoise=dn)) for k in range(warm_jobs)])
        backend.time = {k: 0.0 for k in backend.time}
        backend.denoise_calls = 0
        requests = []
        for i, t in enumerate(arrivals):
            acc, st, nbytes, _ = pool[picks[i]]
            requests.append((float(t), JobRequest(acc, st, w, h, max_samples=max_samples, target_relmse=target,
                                                  seed=1000 + i, scene_bytes=nbytes, denoise=dn)))
        srv = Server(backend, cfg)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        srv.run(requests)
        wall = time.perf_counter() - t0
        lat = srv.latencies()
        jobs = list(srv.jobs.values())
        samples = sum(j.samples * j.req.width * j.req.height for j in jobs)
        errs = []
        for j in jobs:
            ref, noise = refs[id(j.req.scene)]
            x = j.result.astype(np.float64)
            errs.append(float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2))) - noise)
        out[name] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                     "jobs_per_s": len(lat) / wall, "samples_per_s": samples / wall, "wall_s": wall,
                     "passes": srv.passes, "max_active": cfg.max_active,
                     "mean_spp": float(np.mean([j.samples for j in jobs])),
                     "true_relmse_p50": float(np.median(errs)), "true_relmse_p99": float(np.percentile(errs, 99)),
                     "true_relmse_max": float(np.max(errs)),
                     "jobs_meeting_target": int(sum(e <= target for e in errs))}
        out[name]["host_phase_s"] = dict(backend.time)
        if dn:
            out[name]["denoised_jobs"] = int(sum(np.any(np.asarray(j.alpha) > 0) for j in jobs))
            out[name]["mean_alpha"] = float(np.mean([np.mean(j.alpha) for j in jobs]))
            out[name]["denoiser_calls"] = backend.denoise_calls
        backend.destroy()
    plains = [m for m, _, _ in modes if m.startswith("plain")]
    if not plains:
        return out
    best = min(plains, key=lambda m: out[m]["p50_s"])
    out["plain_best"] = best
    for m in [x for x in ("served", "served_denoised") if x in out]:
        out[f"p50_speedup_{m}"] = out[best]["p50_s"] / out[m]["p50_s"]
        out[f"throughput_ratio_{m}"] = out[m]["jobs_per_s"] / out[best]["jobs_per_s"]
    return out


def serving_benchmark(args):
    """The serving workload at two job sizes.  `small`: 48 requests of 256x256
    on four resident displaced icospheres of 18k-800k triangles (a size at
    which one job alone leaves most of the GPU idle); `config5`: requests drawn
    like the plain-render scene -- 1920x1080 images of 2M-triangle displaced
    icospheres (four seeds) -- at the same 200 jobs/s Poisson rate.  Every job
    renders to a target relMSE of 1e-3 against its scene's 4096-spp reference,
    its own error estimated from its two half-buffers without a reference."""
    import voidray_gb300 as vr
    from voidray_gb300 import workloads as W
    from voidray_gb300.denoise import Denoiser

    net = Denoiser.pretrained()
    net.set_backend(Denoiser.TCGEN05)   # inference on the tcgen05 convolution
    out = {}
    hdri_small = vr.Environments.hdri_image(W.sky_hdri(1024, 512))
    pool = serving_scenes("small", (30, 60, 120, 200), (10, 11, 12, 13), hdri_small)
    size = args.serve_size
    refs = serving_references(pool, size, size)
    out["small"] = serving_run(pool, refs, net, size, size, args.serve_jobs, args.serve_rate, args.serve_target,
                               args.serve_streams, (32, 128, 512, "adaptive"), 6, 2048, dn_first_pass=96)
    out["small"]["equal_time"] = denoiser_equal_time(pool, {k: v[0] for k, v in refs.items()}, net, size)
    for acc, *_ in pool:
        acc.destroy()
    if args.serve_large_jobs:
        hdri = vr.Environments.hdri_image(W.sky_hdri(2048, 1024), importance_sample=True)
        pool = serving_scenes("config5", (316, 316, 316, 316), (2, 21, 22, 23), hdri)
        refs = serving_references(pool, 1920, 1080)
        out["config5"] = serving_run(pool, refs, net, 1920, 1080, args.serve_large_jobs, args.serve_rate,
                                     args.serve_target, args.serve_streams, (32, 128, "adaptive"), 2, 2048,
                                     dn_first_pass=96)
        for acc, *_ in pool:
            acc.destroy()
    net.destroy()
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
    default_scene = args.freq == 316
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
        # 32 B ray in + 16 B hit out per ray, 112 B per 4-wide node visit, 48 B per triangle test
        alg_bytes = 48 * rays1 + NODE_BYTES * wk.extend_node_visits + 48 * wk.extend_tri_tests
        ext_ms_per_frame = ins.stage_ms[1] / args.steps
        ext_launches_per_frame = ins.stage_launches[1] / args.steps
        achieved = alg_bytes / (ext_ms_per_frame / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": "k_extend (closest-hit 4-wide BVH traversal)", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    # dram__bytes_read.sum + dram__bytes_write.sum per k_extend launch: bytes per extend
                    # ray measured on a smaller frame of the same scene, times this run's extend rays per
                    # launch (the scene's figure; null for another scene)
                    "traffic": K_EXTEND_DRAM_BYTES_PER_RAY * rays1 / max(ext_launches_per_frame, 1)
                    if default_scene else None,
                    "traffic_source": "ncu dram bytes per extend ray (960x540 x 32 spp frame of the same scene) "
                                      "x extend rays per launch",
                    "l2_gbs": K_EXTEND_L2_BYTES_PER_RAY * rays1 / (ext_ms_per_frame / 1e3) / 1e9
                    if default_scene else None,
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
    isect = None
    if rank == 0 and world == 1 and not args.no_isect:
        isect = intersection_benchmark(args, hbm_peak, "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks
                                       else "fallback")
    cornell = None
    if rank == 0 and world == 1 and not args.no_cornell:
        cornell = cornell_benchmark(args)
    batched = None
    if rank == 0 and world == 1 and not args.no_batch:
        batched = batch_benchmark(args)
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
                    "wavefront_paths": st.wavefront_paths or (1 << 28),
                    "parallelism": f"replicas x{world}, disjoint sample ranges",
                    "tuning": tuning})
        line = {
            "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "mrays_per_s": (ext_rays + shd_rays) / (ms / 1e3) / 1e6,
            "rays": {"extend": int(ext_rays), "shadow": int(shd_rays)},
            "stages": stage, "gpu_launches": gpu_launches, "clocks": clk, "e2e": e2e, "roofline": roofline,
            "cpu_baseline": cpu, "image_finite": finite, "intersection": isect, "cornell": cornell, "batched": batched, "serving": serve, "denoiser": dnb,
        }
        print(json.dumps(line), flush=True)
    acc.destroy()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
