"""Serving layer: a continuous-batching request loop over the batched renderer.

No reference counterpart: the reference renders one scene at a time on its
render thread (voidray_renderer/src/render/renderer.rs:35-125), progressively
in chunks sized by `update_frequency`, with cancel and progress statistics.
Here many progressive renders run at once:

* A request names a resident scene (built once with vr_scene_create), its
  settings, image size, a sample cap and a target relative MSE.
* Admission: a waiting request is admitted when an active slot is free and its
  device footprint (two accumulation half-buffers, plus its scene if that scene
  is not resident yet) fits the memory budget; otherwise it waits (FIFO).
* Every pass renders `spp_per_pass` further samples of every active job in one
  batched launch (vr_batch_render); passes alternate between a job's two
  half-buffers A and B.  Requests that arrive meanwhile are admitted at the
  next pass, so their work overlaps on the device with the running jobs.
* After each pass a job's error is estimated from its half-buffers: with means
  a, b over nA, nB samples, the variance of the combined mean is about
  (a - b)^2 nA nB / (nA + nB)^2, and the estimate is its mean ratio to
  (m^2 + 1e-2) over pixels and channels (the relMSE definition).  A job
  finishes when the estimate reaches the target or its sample cap.
* Denoised serving (requests with denoise=True, a backend with a denoiser):
  the job also accumulates first-hit albedo / normal per half-buffer, and its
  output may be a blend Y = alpha D(P) + (1 - alpha) P of the denoised full
  mean D(P) and the plain mean P.  The error of Y is predicted from the
  halves without a reference: the denoiser's error at n_A samples is
  E|D(A) - B|^2 - Var(B) (B is independent of D(A)); its residual noise
  scales as 1/n (from E|D(A) - D(B)|^2), its bias is taken as constant
  between n_A and n (an over-estimate, the bias shrinks with n), and its
  covariance with the plain noise comes from E[(D(A) - D(B))(A - B)].
  Every term is normalised by (P^2 + 1e-2) like the plain estimate; since P
  shares B's noise this over-states the denoiser's error somewhat (jobs stop
  late rather than early), whereas normalising by the denoised image would
  under-state it (the denoiser's bias would lower its own weights).
  alpha minimises the predicted error, separately for every 16 x 16 pixel
  tile (smooth regions lean on the denoiser, detailed ones on the plain
  mean); the job finishes when the predicted image error (the mean over
  tiles) reaches the target, and returns that blend.  The plain progressive
  render stays the fallback (alpha = 0 everywhere).  The prediction also
  gives the samples a job still needs (noise terms ~ 1/n, bias constant),
  which sizes its next pass.
* A job's result depends only on its own sample streams and pass schedule,
  so it is the same alone and in any mix.

Backends: GpuBackend (torch device buffers + vr_batch) and FakeBackend (a
deterministic CPU stand-in used by the scheduler tests).
"""
from __future__ import annotations

import itertools
import math
import os
import time
from dataclasses import dataclass, field
from typing import Any, Callable, Optional

import numpy as np

EPS_REL = 1e-2  # relMSE denominator offset


@dataclass
class JobRequest:
    scene: Any                 # backend scene handle (SceneAcceleration for the GPU backend)
    settings: Any              # RenderSettings (total_samples is managed by the server)
    width: int
    height: int
    max_samples: int = 4096
    target_relmse: float = 1e-3
    seed: int = 0
    scene_bytes: int = 0       # device bytes of the scene (counted once while resident)
    denoise: bool = False      # render AOVs and allow a denoised / blended output


@dataclass
class JobState:
    job_id: int
    req: JobRequest
    arrival: float
    state: str = "waiting"     # waiting, active, done, cancelled, failed
    admitted: Optional[float] = None
    finished: Optional[float] = None
    samples: int = 0
    n_a: int = 0
    n_b: int = 0
    passes: int = 0
    estimate: float = float("inf")
    bufs: Any = None
    result: Optional[np.ndarray] = None
    error: str = ""
    alpha: float = 0.0         # weight of the denoised image in the output
    plain_estimate: float = float("inf")
    next_spp: int = 0          # adaptive: samples of the job's next pass (0: first pass)
    pending: bool = False      # pipelined: an estimate is in flight
    need_spp: int = 0          # samples the last estimate predicts the job needs (0: assume error ~ 1/n)
    ready: Any = None          # GPU backend: event after the buffers' fill or restore, until the first pass
    saved_bufs: Any = None     # submit(resume=...): accumulators restored at admission
    saved_meta: Optional[dict] = None  # and the pass state that goes with them

    @property
    def latency(self) -> Optional[float]:
        return None if self.finished is None else self.finished - self.arrival

    def footprint(self) -> int:
        # two RGBA f32 half-buffers, plus albedo/normal per half and the
        # denoiser's full-mean inputs and outputs when denoising
        return (9 if self.req.denoise else 2) * self.req.width * self.req.height * 16


@dataclass
class ServerConfig:
    memory_budget: int = 150 * 10**9
    max_active: int = 64
    spp_per_pass: int = 16
    min_samples: int = 32      # no error estimate before this many samples
    # predictive allocation (adaptive=True): a job's next pass renders the
    # samples its own estimate predicts it still needs (error ~ 1/n), split
    # evenly over its halves; jobs take their passes in admission order while
    # the pass has paths left (the first job of a pass always runs), so the
    # GPU gets large passes and jobs finish in order.  A job's sequence of
    # pass sizes depends only on its own estimates, never on the mix.
    adaptive: bool = False
    pass_paths: int = 1 << 24  # paths per pass the scheduler aims for
    first_pass_spp: int = 64
    min_pass_spp: int = 8
    overshoot: float = 1.1     # planned samples x this, against estimate noise
    # pipelined (adaptive only, backends with render_async / estimate_async /
    # poll): a job's error estimate runs on the device while the next pass
    # renders the jobs whose next pass size is already known
    pipelined: bool = False
    max_inflight: int = 2      # pipelined: passes whose estimates may be outstanding
    # pipelined: after a pass of at least this many paths (one that fills the
    # GPU by itself) the next pass waits for its estimates: issuing later
    # jobs' passes behind it would add their time to its jobs' latency and
    # gain no fill (0 = off)
    fill_paths: int = 1 << 26
    # adaptive: order in which jobs take a pass: "fifo" (admission order) or
    # "srpt" (shortest predicted remaining work first: paths the job still
    # needs by its last estimate; jobs before their first estimate count
    # their first pass).  Either way a job's pass sizes are its own.
    order: str = "fifo"


class FakeBackend:
    """CPU stand-in: a job's pixel value for sample s is a deterministic
    function of (seed, pixel, s), so results are reproducible and independent
    of the mix.  `fail_alloc` makes allocation fail for chosen job ids."""

    def __init__(self, fail_alloc: Callable[[int], bool] = lambda job_id: False, noise: float = 0.5):
        self.fail_alloc = fail_alloc
        self.noise = noise
        self.calls = []

    def alloc(self, job: JobState):
        if self.fail_alloc(job.job_id):
            raise MemoryError(f"allocation refused for job {job.job_id}")
        n = job.req.width * job.req.height
        return [np.zeros((n, 3)), np.zeros((n, 3))]

    def free(self, job: JobState) -> None:
        job.bufs = None

    def render(self, work: list[tuple[JobState, int, int, int]]) -> None:
        """work: (job, buffer index, first sample, samples)."""
        self.calls.append([(j.job_id, b, f, s) for j, b, f, s in work])
        for job, b, first, n in work:
            npx = job.req.width * job.req.height
            base = 0.2 + (np.arange(npx) % 17) / 20.0
            for k in range(first, first + n):
                rng = np.random.default_rng([job.req.seed, k])
                job.bufs[b] += (base + self.noise * rng.standard_normal(npx))[:, None]

    def save_bufs(self, job: JobState) -> list:
        return [np.array(b, copy=True) for b in job.bufs]

    def load_bufs(self, job: JobState, arrays: list) -> None:
        for dst, src in zip(job.bufs, arrays):
            dst[...] = src

    def means(self, job: JobState):
        a, b = job.bufs
        return a / max(job.n_a, 1), b / max(job.n_b, 1)

    def estimate(self, job: JobState) -> float:
        a, b = self.means(job)
        return _estimate(a, b, job.n_a, job.n_b)

    def result(self, job: JobState) -> np.ndarray:
        a, b = job.bufs
        return (a + b) / (job.n_a + job.n_b)

    # asynchronous interface (runs synchronously here; the scheduler logic is the same)
    def render_async(self, work):
        self.render(work)
        return None

    def estimate_async(self, jobs, after):
        return [self.estimate(j) for j in jobs]

    def poll(self, handle, block: bool = False):
        return handle


def _estimate(a, b, na: int, nb: int, xp=np) -> float:
    n = na + nb
    m = (a * na + b * nb) / n
    var = (a - b) ** 2 * (na * nb) / (n * n)
    return float(xp.mean(var / (m * m + EPS_REL)))


BLEND_TILE = 16  # blend weights are chosen per BLEND_TILE x BLEND_TILE pixel tile


def _tile_mean(x, tile: int, xp):
    """Per-tile means over the valid pixels and channels of an (H, W, C) array
    or tensor -> (ceil(H/tile), ceil(W/tile))."""
    h, w, c = x.shape
    th, tw = -(-h // tile), -(-w // tile)
    ph, pw = th * tile - h, tw * tile - w
    if xp is np:
        xs = np.pad(x, ((0, ph), (0, pw), (0, 0)))
        cnt = np.pad(np.ones((h, w)), ((0, ph), (0, pw)))
    else:
        import torch.nn.functional as F

        xs = F.pad(x.permute(2, 0, 1), (0, pw, 0, ph)).permute(1, 2, 0)
        cnt = F.pad(x.new_ones((1, h, w)), (0, pw, 0, ph))[0]
    s = xs.reshape(th, tile, tw, tile, c).sum((1, 3, 4))
    n = cnt.reshape(th, tile, tw, tile).sum((1, 3)) * c
    return s / n


def blend_tile_moments(a, b, p, da, db, tile: int = BLEND_TILE, xp=np):
    """blend_moments per tile: stacked (5, tiles_y, tiles_x)."""
    den = p * p + EPS_REL
    ab = a - b
    dd = da - db
    maps = [ab * ab / den, (da - b) ** 2 / den, (db - a) ** 2 / den, dd * dd / den, dd * ab / den]
    return xp.stack([_tile_mean(m, tile, xp) for m in maps])


def tile_blend(mt, na: int, nb: int, k: float = 1.0):
    """Per-tile best blend at k x (na + nb) samples from blend_tile_moments()
    values (numpy (5, ty, tx)); returns (plain image error, blend image error,
    alpha map).  Each tile takes its own optimal weight (alpha = 0 is the
    plain mean), so the blend is never predicted worse than plain."""
    s_ab, s_dab, s_dba, s_dd, s_ddab = (np.asarray(x, np.float64) for x in mt)
    n = na + nb
    v_p = s_ab * na * nb / (n * n)
    e_a = s_dab - s_ab * na / n
    e_b = s_dba - s_ab * nb / n
    tau2 = s_dd * na * nb / n
    kap = s_ddab * na * nb / n
    bias2 = np.maximum(0.0, 0.5 * ((e_a - tau2 / na) + (e_b - tau2 / nb)))
    v_p, v_eta, c = v_p / k, tau2 / n / k, kap / n / k
    e_d = bias2 + v_eta
    q = e_d + v_p - 2.0 * c
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = np.where(q > 0, np.clip((v_p - c) / q, 0.0, 1.0), 1.0)
    blend = np.maximum(alpha * alpha * e_d + (1 - alpha) ** 2 * v_p + 2 * alpha * (1 - alpha) * c, 0.0)
    return float(v_p.mean()), float(blend.mean()), alpha


def tile_samples_needed(mt, na: int, nb: int, target: float) -> int:
    """Fewest samples at which the per-tile blend's predicted image error reaches `target`."""
    n = na + nb
    err = lambda k: tile_blend(mt, na, nb, k)[1]
    if err(1.0) <= target:
        return n
    lo, hi = 1.0, 2.0
    while err(hi) > target and hi < 1e6:
        lo, hi = hi, hi * 2.0
    for _ in range(30):
        mid = 0.5 * (lo + hi)
        if err(mid) > target:
            lo = mid
        else:
            hi = mid
    return int(math.ceil(n * hi))


def blend_moments(a, b, p, da, db, xp=np) -> list:
    """The five pixel means the blend prediction needs (arrays or tensors,
    not yet converted to floats, so a caller can read many at once)."""
    den = p * p + EPS_REL
    ab = a - b
    dd = da - db
    return [xp.mean(ab * ab / den), xp.mean((da - b) ** 2 / den), xp.mean((db - a) ** 2 / den),
            xp.mean(dd * dd / den), xp.mean(dd * ab / den)]


def _blend_terms(m, na: int, nb: int):
    """(v_p, bias2, v_eta, c) at n = na + nb samples from blend_moments() values."""
    s_ab, s_dab, s_dba, s_dd, s_ddab = (float(x) for x in m)
    n = na + nb
    v_p = s_ab * na * nb / (n * n)
    var_a, var_b = s_ab * nb / n, s_ab * na / n
    e_a = s_dab - var_b
    e_b = s_dba - var_a
    tau2 = s_dd * na * nb / n
    kap = s_ddab * na * nb / n
    bias2 = max(0.0, 0.5 * ((e_a - tau2 / na) + (e_b - tau2 / nb)))
    return v_p, bias2, tau2 / n, kap / n


def _best_blend(v_p, bias2, v_eta, c):
    e_d = bias2 + v_eta
    q = e_d + v_p - 2.0 * c
    alpha = min(1.0, max(0.0, (v_p - c) / q)) if q > 0 else 1.0
    blend = alpha * alpha * e_d + (1.0 - alpha) ** 2 * v_p + 2.0 * alpha * (1.0 - alpha) * c
    return max(blend, 0.0), alpha


def blend_samples_needed(m, na: int, nb: int, target: float) -> int:
    """Fewest samples n' >= n at which the predicted error of the best of the
    plain mean and the blend reaches `target`: the noise terms (plain
    variance, residual denoiser noise, covariance) scale as n / n', the bias
    stays."""
    v_p, bias2, v_eta, c = _blend_terms(m, na, nb)
    n = na + nb

    def err(k):  # k = n' / n
        b, _ = _best_blend(v_p / k, bias2, v_eta / k, c / k)
        return min(b, v_p / k)

    if err(1.0) <= target:
        return n
    lo, hi = 1.0, 2.0
    while err(hi) > target and hi < 1e6:
        lo, hi = hi, hi * 2.0
    for _ in range(30):
        mid = 0.5 * (lo + hi)
        if err(mid) > target:
            lo = mid
        else:
            hi = mid
    return int(math.ceil(n * hi))


def blend_from_moments(m, na: int, nb: int):
    """(plain, blend, alpha) from blend_moments() values."""
    # Var(P) from the halves; D(A)'s error is E|D(A)-B|^2 - Var(B); the
    # residual denoiser noise x samples (tau2) from E|D(A)-D(B)|^2; its
    # covariance with the plain noise x samples from E[(D(A)-D(B))(A-B)]
    v_p, bias2, v_eta, c = _blend_terms(m, na, nb)
    blend, alpha = _best_blend(v_p, bias2, v_eta, c)
    return v_p, blend, alpha


def blend_prediction(a, b, p, da, db, na: int, nb: int, xp=np):
    """Predicted relMSE of the plain mean P and of the best blend
    alpha D(P) + (1 - alpha) P, from the half means a, b (na, nb samples),
    the full mean p and the denoised half means da, db.  Returns
    (plain, blend, alpha)."""
    return blend_from_moments(blend_moments(a, b, p, da, db, xp), na, nb)


class GpuBackend:
    """Device accumulation buffers (torch) and vr_batch objects that render
    the passes; with a denoiser, jobs that ask for it also get AOV buffers and
    blended outputs (the module docstring describes the prediction).

    With render_streams = 2, pipelined passes alternate between two batches
    (each with its own path-state scratch and graph cache) on two streams, so
    the deep bounces of one pass, which keep few rays alive, overlap the first
    bounces of the next.  A job is in at most one pass at a time, so this
    changes no job's samples."""

    def __init__(self, max_wave_paths: int = 0, denoiser=None, render_streams: int = 1):
        import torch

        from .batch import Batch

        self.torch = torch
        self.batches = [Batch(max_wave_paths) for _ in range(max(1, int(render_streams)))]
        for b in self.batches:
            b.set_graphs(True)   # passes of an unchanged job set replay one CUDA graph
        self.streams = [torch.cuda.Stream() for _ in self.batches]  # renders
        self.batch, self.stream = self.batches[0], self.streams[0]
        self._next = 0                         # batch / stream of the next asynchronous pass
        self.est_stream = torch.cuda.Stream()  # estimates (pipelined mode)
        self.res_stream = torch.cuda.Stream()  # final images: never queued behind later estimates
        self.dn = denoiser
        # final images run on their own stream, so they get their own handle
        # (a handle's workspace must not be shared by concurrent streams)
        self.dn_result = denoiser.clone() if denoiser is not None else None
        self.denoise_calls = 0
        self.time = {"render": 0.0, "estimate": 0.0, "result": 0.0}  # host wall seconds per phase

    def alloc(self, job: JobState):
        t = self.torch
        h, w = job.req.height, job.req.width
        k = 6 if (job.req.denoise and self.dn is not None) else 2
        # [A, B] radiance sums, then albedo A/B and normal A/B sums, zeroed on
        # the first render stream; a pass on another stream waits for the fill
        with t.cuda.stream(self.stream):
            bufs = [t.zeros((h, w, 4), dtype=t.float32, device="cuda") for _ in range(k)]
            job.ready = t.cuda.Event()
            job.ready.record(self.stream)
        return bufs

    def free(self, job: JobState) -> None:
        job.bufs = None

    def save_bufs(self, job: JobState) -> list:
        """Host copies of the job's accumulators (after its passes so far)."""
        for st in self.streams:
            st.synchronize()
        with self.torch.cuda.stream(self.stream):
            return [b.cpu().numpy() for b in job.bufs]

    def load_bufs(self, job: JobState, arrays: list) -> None:
        """Restores saved accumulators on the first render stream; passes on
        other streams wait for the copy like for the zero fill."""
        t = self.torch
        with t.cuda.stream(self.stream):
            for dst, src in zip(job.bufs, arrays):
                dst.copy_(t.from_numpy(np.ascontiguousarray(src, np.float32)))
            job.ready = t.cuda.Event()
            job.ready.record(self.stream)

    # -- rendering -------------------------------------------------------
    def _enqueue(self, work: list[tuple[JobState, int, int, int]], k: int = 0) -> None:
        from dataclasses import replace

        from .batch import RenderJob

        stream = self.streams[k]
        jobs = []
        for job, b, first, n in work:
            # the allocator must not hand these buffers to another job while this
            # stream still writes them (a job cancelled with its pass in flight)
            for t in job.bufs:
                t.record_stream(stream)
            if job.ready is not None:
                if k != 0:
                    stream.wait_event(job.ready)
                job.ready = None
            # buffers accumulate raw sums: total_samples = 1
            st = replace(job.req.settings, total_samples=1)
            aov = len(job.bufs) == 6
            jobs.append(RenderJob(job.req.scene, st, n, job.bufs[b].data_ptr(), job.req.width, job.req.height,
                                  job.req.seed, first, job.bufs[2 + b].data_ptr() if aov else 0,
                                  job.bufs[4 + b].data_ptr() if aov else 0))
        self.batches[k].render(jobs, stream.cuda_stream)

    def render(self, work: list[tuple[JobState, int, int, int]]) -> None:
        t0 = time.perf_counter()
        self._enqueue(work)
        self.batch.synchronize(self.stream.cuda_stream)
        self.time["render"] += time.perf_counter() - t0

    def render_async(self, work):
        """Enqueues the pass on the next render stream; returns an event
        recorded after it."""
        t0 = time.perf_counter()
        k = self._next
        self._next = (k + 1) % len(self.batches)
        self._enqueue(work, k)
        ev = self.torch.cuda.Event()
        ev.record(self.streams[k])
        self.time["render"] += time.perf_counter() - t0
        return ev

    # -- error estimates -------------------------------------------------
    def _stats(self, jobs: list[JobState], stream):
        """Enqueues on `stream`: the denoiser over both half-buffers of every
        denoising job (one batch per image size), then one statistics launch
        (vr_serve_stats_device) for all jobs: per 16 x 16 tile the plain
        variance term and, for denoising jobs, the five blend moments.
        Returns (one flat fp64 device tensor, per-job layout)."""
        import ctypes as C

        from . import _native as N

        t = self.torch
        for job in jobs:  # read on this stream: no reuse of the buffers before it is done
            for b in job.bufs:
                b.record_stream(stream)
        with t.cuda.stream(stream):
            den = {}
            groups = {}
            for job in jobs:
                if len(job.bufs) == 6:
                    groups.setdefault((job.req.height, job.req.width), []).append(job)
            for (h, w), items in groups.items():
                rad = t.stack([x for j in items for x in (j.bufs[0], j.bufs[1])])
                alb = t.stack([x for j in items for x in (j.bufs[2], j.bufs[3])])
                nrm = t.stack([x for j in items for x in (j.bufs[4], j.bufs[5])])
                scales = [s for j in items for s in (1.0 / j.n_a, 1.0 / j.n_b)]
                out = t.empty_like(rad)
                self.dn.denoise_batch(rad, alb, nrm, scales, out, w, h, stream=stream.cuda_stream)
                self.denoise_calls += 1
                for k, j in enumerate(items):
                    den[id(j)] = (out[2 * k], out[2 * k + 1])
            layout, off = [], 0
            table = (N.vr_stats_job * len(jobs))()
            for i, job in enumerate(jobs):
                h, w = job.req.height, job.req.width
                ty, tx = -(-h // BLEND_TILE), -(-w // BLEND_TILE)
                d = den.get(id(job))
                e = table[i]
                e.sum_a, e.sum_b = job.bufs[0].data_ptr(), job.bufs[1].data_ptr()
                e.den_a, e.den_b = (d[0].data_ptr(), d[1].data_ptr()) if d is not None else (None, None)
                e.n_a, e.n_b, e.width, e.height, e.tile_offset = job.n_a, job.n_b, w, h, off
                layout.append((job, off, ty, tx, d is not None))
                off += (6 if d is not None else 1) * ty * tx
            flat = t.empty(max(off, 1), dtype=t.float64, device="cuda")
            for c0 in range(0, len(jobs), N.STATS_MAX_JOBS):
                n = min(N.STATS_MAX_JOBS, len(jobs) - c0)
                N.check(N.lib().vr_serve_stats_device(C.byref(table, c0 * C.sizeof(N.vr_stats_job)), n,
                                                      C.c_void_p(flat.data_ptr()), C.c_void_p(stream.cuda_stream)))
            return flat, layout

    def _apply(self, jobs: list[JobState], v: np.ndarray, layout) -> list[float]:
        out = []
        for job, off, ty, tx, denoised in layout:
            h, w = job.req.height, job.req.width
            nt = ty * tx
            e = float(v[off:off + nt].sum()) / (3.0 * h * w)
            job.plain_estimate, job.alpha, job.need_spp = e, 0.0, 0
            if denoised:
                mt = v[off + nt:off + 6 * nt].reshape(5, ty, tx)
                _, blend, alpha = tile_blend(mt, job.n_a, job.n_b)
                job.need_spp = tile_samples_needed(mt, job.n_a, job.n_b, job.req.target_relmse)
                if blend < e:
                    job.alpha = alpha
                    e = blend
            out.append(e)
        return out

    def estimate(self, job: JobState) -> float:
        return self.estimate_many([job])[0]

    def estimate_many(self, jobs: list[JobState]) -> list[float]:
        """Estimates of all jobs of a pass, read back in one transfer."""
        t0 = time.perf_counter()
        flat, layout = self._stats(jobs, self.stream)
        with self.torch.cuda.stream(self.stream):
            v = flat.cpu().numpy()  # copied on the stream that computed it (then waited for)
        out = self._apply(jobs, v, layout)
        self.time["estimate"] += time.perf_counter() - t0
        return out

    def estimate_async(self, jobs: list[JobState], after):
        """Enqueues the estimates on the estimate stream after event `after`;
        the values land in pinned host memory.  poll() applies them."""
        t = self.torch
        t0 = time.perf_counter()
        es = self.est_stream
        with t.cuda.stream(es):
            if after is not None:
                es.wait_event(after)
            flat, layout = self._stats(jobs, es)
            host = t.empty(flat.shape, dtype=flat.dtype, pin_memory=True)
            host.copy_(flat, non_blocking=True)
            done = t.cuda.Event()
            done.record(es)
        self.time["estimate"] += time.perf_counter() - t0
        return (done, host, list(jobs), layout)

    def poll(self, handle, block: bool = False):
        done, host, jobs, layout = handle
        if not block and not done.query():
            return None
        t0 = time.perf_counter()
        done.synchronize()
        out = self._apply(jobs, host.numpy(), layout)
        self.time["estimate"] += time.perf_counter() - t0
        return out

    def finish(self) -> None:
        """Waits for all streams and reports kernel-side errors of the passes."""
        self.est_stream.synchronize()
        self.res_stream.synchronize()
        for b, st in zip(self.batches, self.streams):
            b.synchronize(st.cuda_stream)

    def destroy(self) -> None:
        for b in self.batches:
            b.destroy()

    # -- results ---------------------------------------------------------
    def result(self, job: JobState) -> np.ndarray:
        """The plain mean, or the blend alpha D(P) + (1 - alpha) P with alpha
        per BLEND_TILE tile (piecewise constant): the half-buffer sums, the
        denoiser's input and the blend are library kernels
        (vr_serve_sum_device, vr_serve_blend_device) on the result stream."""
        import ctypes as C

        from . import _native as N

        t = self.torch
        t0 = time.perf_counter()
        n = job.n_a + job.n_b
        h, w = job.req.height, job.req.width
        es = self.res_stream
        for b in job.bufs:
            b.record_stream(es)
        ptr = lambda x: C.c_void_p(x.data_ptr())
        with t.cuda.stream(es):
            rgb = t.empty((h, w, 3), dtype=t.float32, device="cuda")
            alpha = np.asarray(job.alpha, np.float32)
            if not alpha.any():
                N.check(N.lib().vr_serve_blend_device(ptr(job.bufs[0]), ptr(job.bufs[1]), n, None, None, w, h,
                                                       ptr(rgb), C.c_void_p(es.cuda_stream)))
            else:
                sums = [t.empty((h, w, 4), dtype=t.float32, device="cuda") for _ in range(3)]
                arr = C.c_void_p * 3
                N.check(N.lib().vr_serve_sum_device(arr(*[b.data_ptr() for b in job.bufs[0::2]]),
                                                     arr(*[b.data_ptr() for b in job.bufs[1::2]]),
                                                     arr(*[x.data_ptr() for x in sums]), 3, h * w,
                                                     C.c_void_p(es.cuda_stream)))
                d = t.empty((h, w, 4), dtype=t.float32, device="cuda")
                self.dn_result.denoise(sums[0], sums[1], sums[2], 1.0 / n, d, w, h, stream=es.cuda_stream)
                self.denoise_calls += 1
                ty, tx = -(-h // BLEND_TILE), -(-w // BLEND_TILE)
                tiles = np.broadcast_to(alpha, (ty, tx)) if alpha.ndim < 2 else alpha
                am = t.from_numpy(np.ascontiguousarray(tiles, np.float32)).to("cuda")
                N.check(N.lib().vr_serve_blend_device(ptr(job.bufs[0]), ptr(job.bufs[1]), n, ptr(d), ptr(am), w, h,
                                                       ptr(rgb), C.c_void_p(es.cuda_stream)))
        es.synchronize()
        out = rgb.cpu().numpy()
        self.time["result"] += time.perf_counter() - t0
        return out


class Server:
    def __init__(self, backend, config: ServerConfig = ServerConfig(), clock: Callable[[], float] = time.perf_counter):
        self.backend = backend
        self.cfg = config
        self.clock = clock
        self.jobs: dict[int, JobState] = {}
        self.waiting: list[int] = []
        self.active: list[int] = []
        self._ids = itertools.count()
        self.resident_scenes: dict[int, int] = {}  # id(scene) -> active users
        self.used = 0
        self.passes = 0
        self.pending: list = []   # pipelined: (estimate handle, jobs) in issue order
        self.last_pass_paths = 0

    # -- requests --------------------------------------------------------
    def submit(self, req: JobRequest, arrival: Optional[float] = None, resume: Optional[str] = None) -> int:
        """Queues a request; with `resume`, the job continues from a checkpoint
        written by checkpoint() for the same request (scene, settings, size,
        seed), so it renders exactly the passes it had left."""
        jid = next(self._ids)
        job = JobState(jid, req, self.clock() if arrival is None else arrival)
        if resume is not None:
            with np.load(resume, allow_pickle=False) as z:
                meta = {k: z[k].item() for k in z.files if k.startswith("m_")}
                job.saved_bufs = [np.array(z[f"buf{i}"]) for i in range(int(meta["m_nbufs"]))]
            if (meta["m_width"], meta["m_height"], meta["m_seed"]) != (req.width, req.height, req.seed):
                raise ValueError("checkpoint of a different request (size or seed)")
            job.saved_meta = meta
        self.jobs[jid] = job
        self.waiting.append(jid)
        return jid

    def checkpoint(self, job_id: int, path: str) -> None:
        """Writes an active job's accumulators and pass state to `path` (.npz,
        by rename).  The job must have no estimate in flight."""
        job = self.jobs[job_id]
        if job.state != "active" or job.pending:
            raise ValueError(f"job {job_id} is {job.state}{' with an estimate in flight' if job.pending else ''}")
        bufs = self.backend.save_bufs(job)
        meta = {"m_width": job.req.width, "m_height": job.req.height, "m_seed": job.req.seed,
                "m_nbufs": len(bufs), "m_samples": job.samples, "m_n_a": job.n_a, "m_n_b": job.n_b,
                "m_passes": job.passes, "m_next_spp": job.next_spp, "m_need_spp": job.need_spp,
                "m_estimate": job.estimate, "m_plain_estimate": job.plain_estimate}
        tmp = path + ".tmp"
        with open(tmp, "wb") as f:
            np.savez(f, **{f"buf{i}": b for i, b in enumerate(bufs)}, **{k: np.array(v) for k, v in meta.items()})
        os.replace(tmp, path)

    def cancel(self, job_id: int) -> None:
        job = self.jobs[job_id]
        if job.state == "waiting":
            self.waiting.remove(job_id)
        elif job.state == "active":
            self._release(job)
            self.active.remove(job_id)
        job.state = "cancelled"
        job.finished = self.clock()

    def status(self, job_id: int) -> JobState:
        return self.jobs[job_id]

    # -- admission ---------------------------------------------------------
    def _scene_cost(self, req: JobRequest) -> int:
        return 0 if id(req.scene) in self.resident_scenes else req.scene_bytes

    def _admit(self) -> None:
        still = []
        for jid in self.waiting:
            job = self.jobs[jid]
            need = job.footprint() + self._scene_cost(job.req)
            if len(self.active) < self.cfg.max_active and self.used + need <= self.cfg.memory_budget:
                try:
                    job.bufs = self.backend.alloc(job)
                    meta = job.saved_meta
                    if meta is not None:
                        if len(job.saved_bufs) != len(job.bufs):
                            raise ValueError("checkpoint buffers do not match the request (denoising on/off)")
                        self.backend.load_bufs(job, job.saved_bufs)
                        job.samples, job.n_a, job.n_b = meta["m_samples"], meta["m_n_a"], meta["m_n_b"]
                        job.passes, job.next_spp, job.need_spp = meta["m_passes"], meta["m_next_spp"], meta["m_need_spp"]
                        job.estimate, job.plain_estimate = meta["m_estimate"], meta["m_plain_estimate"]
                        job.saved_bufs = job.saved_meta = None
                except Exception as e:  # an allocation or restore failure fails this job only
                    job.bufs = None
                    job.state, job.error, job.finished = "failed", str(e), self.clock()
                    continue
                self.used += need
                key = id(job.req.scene)
                self.resident_scenes[key] = self.resident_scenes.get(key, 0) + 1
                job.state, job.admitted = "active", self.clock()
                self.active.append(jid)
            else:
                still.append(jid)
        self.waiting = still

    def _release(self, job: JobState) -> None:
        key = id(job.req.scene)
        n = self.resident_scenes.get(key, 1) - 1
        freed = job.footprint()
        if n <= 0:
            self.resident_scenes.pop(key, None)
            freed += job.req.scene_bytes
        else:
            self.resident_scenes[key] = n
        self.used -= freed
        self.backend.free(job)

    # -- passes ------------------------------------------------------------
    def _plan(self) -> list:
        """Work items (job, half, first sample, samples) of the next pass."""
        work = []
        if not self.cfg.adaptive:
            for jid in self.active:
                job = self.jobs[jid]
                n = min(self.cfg.spp_per_pass, job.req.max_samples - job.samples)
                work.append((job, job.passes % 2, job.samples, n))
            return work
        budget = self.cfg.pass_paths
        ids = self.active
        if self.cfg.order == "srpt":
            def remaining(jid):
                j = self.jobs[jid]
                return (j.next_spp or self.cfg.first_pass_spp) * j.req.width * j.req.height
            ids = sorted(self.active, key=lambda jid: (remaining(jid), jid))
        for jid in ids:
            job = self.jobs[jid]
            if job.pending:
                continue  # waits for its estimate
            want = job.next_spp or self.cfg.first_pass_spp
            want = max(1, min(want, job.req.max_samples - job.samples))
            paths = want * job.req.width * job.req.height
            if work and paths > budget:
                continue  # runs in a later pass, with the same size
            budget -= paths
            half = (want + 1) // 2
            work.append((job, 0, job.samples, half))
            if want - half:
                work.append((job, 1, job.samples + half, want - half))
        return work

    def _next_spp(self, job: JobState) -> int:
        if not math.isfinite(job.estimate):
            return self.cfg.first_pass_spp
        need = job.need_spp or job.samples * job.estimate / job.req.target_relmse
        more = int(math.ceil(self.cfg.overshoot * max(0.0, need - job.samples)))
        more = max(self.cfg.min_pass_spp, more + (more & 1))
        return min(more, job.req.max_samples - job.samples)

    def _finish_or_plan(self, job: JobState) -> bool:
        """After an estimate: retire the job (True) or plan its next pass."""
        if job.estimate <= job.req.target_relmse or job.samples >= job.req.max_samples:
            job.result = self.backend.result(job)
            job.state, job.finished = "done", self.clock()
            self._release(job)
            self.active.remove(job.job_id)
            return True
        if self.cfg.adaptive:
            job.next_spp = self._next_spp(job)
        return False

    def _harvest(self, block: bool) -> None:
        """Collects finished estimates in order (waits for the oldest if block)."""
        while self.pending:
            handle, jobs = self.pending[0]
            ests = self.backend.poll(handle, block=block)
            if ests is None:
                return
            self.pending.pop(0)
            block = False
            for job, e in zip(jobs, ests):
                if job.state != "active":
                    continue  # cancelled (or failed) while its estimate was in flight
                job.estimate, job.pending = e, False
                self._finish_or_plan(job)

    def _step_pipelined(self) -> int:
        self._admit()
        self._harvest(block=False)
        # a bounded number of passes in flight: a deeper queue would put later
        # jobs' passes ahead of the next pass of the jobs waiting for estimates
        limit = self.cfg.max_inflight
        if self.cfg.fill_paths and self.last_pass_paths >= self.cfg.fill_paths:
            limit = 1
        while len(self.pending) >= limit:
            self._harvest(block=True)
            self._admit()
        while True:
            work = self._plan()
            if work:
                break
            if not self.pending:
                return 0
            self._harvest(block=True)
            self._admit()
        try:
            ev = self.backend.render_async(work)
        except Exception as e:
            for job in {id(w[0]): w[0] for w in work}.values():
                job.state, job.error, job.finished = "failed", str(e), self.clock()
                self._release(job)
                self.active.remove(job.job_id)
            return 0
        self.passes += 1
        self.last_pass_paths = sum(n * job.req.width * job.req.height for job, _, _, n in work)
        rendered = {}
        for job, b, first, n in work:
            job.samples += n
            if b == 0:
                job.n_a += n
            else:
                job.n_b += n
            rendered[job.job_id] = job
        check = []
        for job in rendered.values():
            job.passes += 1
            if job.n_a and job.n_b and job.samples >= self.cfg.min_samples:
                job.pending = True
                check.append(job)
            else:
                job.next_spp = self._next_spp(job)
        if check:
            self.pending.append((self.backend.estimate_async(check, ev), check))
        return len(rendered)

    def step(self) -> int:
        """Admits what fits, renders one pass (every active job, or with
        adaptive allocation the jobs the pass has room for), estimates, retires
        finished jobs.  Returns the number of jobs rendered."""
        if self.cfg.pipelined and self.cfg.adaptive and hasattr(self.backend, "render_async"):
            return self._step_pipelined()
        self._admit()
        if not self.active:
            return 0
        work = self._plan()
        try:
            self.backend.render(work)
        except Exception as e:
            for job in {id(w[0]): w[0] for w in work}.values():
                job.state, job.error, job.finished = "failed", str(e), self.clock()
                self._release(job)
                self.active.remove(job.job_id)
            return 0
        self.passes += 1
        rendered = {}
        for job, b, first, n in work:
            job.samples += n
            if b == 0:
                job.n_a += n
            else:
                job.n_b += n
            rendered[job.job_id] = job
        check = []
        for job in rendered.values():
            job.passes += 1
            if job.n_a and job.n_b and job.samples >= self.cfg.min_samples:
                check.append(job)
        if check:
            if hasattr(self.backend, "estimate_many"):
                ests = self.backend.estimate_many(check)
            else:
                ests = [self.backend.estimate(j) for j in check]
            for job, e in zip(check, ests):
                job.estimate = e
        done = []
        for job in rendered.values():
            if job.estimate <= job.req.target_relmse or job.samples >= job.req.max_samples:
                job.result = self.backend.result(job)
                job.state, job.finished = "done", self.clock()
                done.append(job.job_id)
            elif self.cfg.adaptive:
                job.next_spp = self._next_spp(job)
        for jid in done:
            self._release(self.jobs[jid])
            self.active.remove(jid)
        return len(rendered)

    def idle(self) -> bool:
        return not self.waiting and not self.active

    def run(self, arrivals: list[tuple[float, JobRequest]] = (), until_idle: bool = True) -> None:
        """Replays `arrivals` (offset seconds, request) against the clock while
        stepping; returns when every request has finished."""
        start = self.clock()
        pending = sorted(arrivals, key=lambda x: x[0])
        i = 0
        while True:
            now = self.clock() - start
            while i < len(pending) and pending[i][0] <= now:
                self.submit(pending[i][1], arrival=start + pending[i][0])
                i += 1
            if self.idle():
                if i >= len(pending):
                    break
                time.sleep(max(0.0, min(pending[i][0] - now, 0.001)))
                continue
            self.step()
            if not until_idle and i >= len(pending):
                break
        if hasattr(self.backend, "finish"):
            self.backend.finish()

    def latencies(self, state: str = "done") -> np.ndarray:
        return np.array([j.latency for j in self.jobs.values() if j.state == state and j.latency is not None])


def poisson_arrivals(rate: float, count: int, seed: int = 0) -> np.ndarray:
    """Arrival offsets (seconds) of a Poisson stream."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, count))
