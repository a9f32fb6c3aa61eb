"""Serving-layer scheduler on a CPU fake device: admission by memory budget,
continuous batching, cancellation, failure isolation, determinism in a mix."""
import numpy as np
import pytest

from voidray_gb300.serve import FakeBackend, JobRequest, Server, ServerConfig, poisson_arrivals


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def req(seed=0, w=8, h=8, target=1e-3, max_samples=256, scene="s0", scene_bytes=0):
    return JobRequest(scene=scene, settings=None, width=w, height=h, max_samples=max_samples, target_relmse=target,
                      seed=seed, scene_bytes=scene_bytes)


def test_admission_waits_for_memory():
    cfg = ServerConfig(memory_budget=2 * (2 * 8 * 8 * 16), max_active=8, spp_per_pass=8, min_samples=16)
    s = Server(FakeBackend(), cfg, clock=Clock())
    ids = [s.submit(req(seed=i, target=0.0, max_samples=16)) for i in range(3)]
    s.step()
    assert [s.status(i).state for i in ids] == ["active", "active", "waiting"]
    assert s.used <= cfg.memory_budget
    s.step()  # first two finish (16 samples)
    assert s.status(ids[0]).state == "done" and s.status(ids[2]).state == "waiting"
    s.step()
    assert s.status(ids[2]).state == "active"
    while not s.idle():
        s.step()
    assert s.used == 0 and all(s.status(i).state == "done" for i in ids)


def test_continuous_batching_overlaps_late_arrivals():
    be = FakeBackend()
    s = Server(be, ServerConfig(spp_per_pass=4, min_samples=8), clock=Clock())
    a = s.submit(req(seed=1, target=0.0, max_samples=32))
    s.step()
    b = s.submit(req(seed=2, target=0.0, max_samples=32))
    s.step()
    assert {j for j, *_ in be.calls[-1]} == {a, b}  # the late request shares the pass
    while not s.idle():
        s.step()


def test_result_same_alone_and_in_mix():
    def run(mix):
        s = Server(FakeBackend(), ServerConfig(spp_per_pass=8, min_samples=16), clock=Clock())
        jid = s.submit(req(seed=7, target=2e-3, max_samples=512))
        for k in range(mix):
            s.submit(req(seed=100 + k, target=1e-4, max_samples=64))
        while not s.idle():
            s.step()
        j = s.status(jid)
        return j.result, j.samples

    r0, n0 = run(0)
    r1, n1 = run(5)
    assert n0 == n1 and np.array_equal(r0, r1)


def test_stops_at_target_error():
    s = Server(FakeBackend(noise=0.3), ServerConfig(spp_per_pass=16, min_samples=32), clock=Clock())
    jid = s.submit(req(seed=3, target=1e-3, max_samples=100000))
    while not s.idle():
        s.step()
    j = s.status(jid)
    assert j.state == "done" and j.estimate <= 1e-3 and j.samples < 100000


def test_cancel_and_failures_are_isolated():
    be = FakeBackend(fail_alloc=lambda jid: jid == 1)
    s = Server(be, ServerConfig(spp_per_pass=4, min_samples=8), clock=Clock())
    a = s.submit(req(seed=1, target=0.0, max_samples=64))
    b = s.submit(req(seed=2, target=0.0, max_samples=64))
    c = s.submit(req(seed=3, target=0.0, max_samples=64))
    s.step()
    assert s.status(b).state == "failed" and "allocation" in s.status(b).error
    s.cancel(c)
    assert s.status(c).state == "cancelled"
    s.step()
    assert {j for j, *_ in be.calls[-1]} == {a}
    while not s.idle():
        s.step()
    assert s.status(a).state == "done" and s.used == 0


def test_render_failure_fails_the_pass_only():
    class Flaky(FakeBackend):
        def __init__(self):
            super().__init__()
            self.fail_next = True

        def render(self, work):
            if self.fail_next:
                self.fail_next = False
                raise RuntimeError("device error")
            super().render(work)

    s = Server(Flaky(), ServerConfig(spp_per_pass=4, min_samples=8), clock=Clock())
    a = s.submit(req(seed=1, target=0.0, max_samples=16))
    s.step()
    assert s.status(a).state == "failed" and s.used == 0
    b = s.submit(req(seed=2, target=0.0, max_samples=16))
    while not s.idle():
        s.step()
    assert s.status(b).state == "done"


def test_resident_scene_counted_once():
    cfg = ServerConfig(memory_budget=10**9, spp_per_pass=4, min_samples=8)
    s = Server(FakeBackend(), cfg, clock=Clock())
    s.submit(req(seed=1, target=0.0, max_samples=8, scene="big", scene_bytes=1000))
    s.submit(req(seed=2, target=0.0, max_samples=8, scene="big", scene_bytes=1000))
    s._admit()
    assert s.used == 1000 + 2 * (2 * 8 * 8 * 16)
    while not s.idle():
        s.step()
    assert s.used == 0


def test_poisson_replay():
    arr = poisson_arrivals(2000.0, 12, seed=1)
    assert np.all(np.diff(arr) > 0)
    s = Server(FakeBackend(), ServerConfig(spp_per_pass=8, min_samples=16))
    s.run([(float(t), req(seed=i, target=5e-3, max_samples=128)) for i, t in enumerate(arr)])
    lat = s.latencies()
    assert len(lat) == 12 and np.all(lat > 0)


def _box(x, r=2):
    """(2r+1)^2 box filter with edge clamping (a linear stand-in denoiser)."""
    pad = np.pad(x, ((r, r), (r, r), (0, 0)), mode="edge")
    out = np.zeros_like(x)
    for dy in range(2 * r + 1):
        for dx in range(2 * r + 1):
            out += pad[dy:dy + x.shape[0], dx:dx + x.shape[1]]
    return out / (2 * r + 1) ** 2


def _halves(truth, sigma, na, nb, seed):
    rng = np.random.default_rng(seed)
    a = truth + sigma * rng.standard_normal(truth.shape) / np.sqrt(na)
    b = truth + sigma * rng.standard_normal(truth.shape) / np.sqrt(nb)
    return a, b, (a * na + b * nb) / (na + nb)


def _relmse(x, r):
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


@pytest.mark.parametrize("na,nb", [(64, 64), (96, 64)])
def test_blend_prediction_tracks_the_true_error(na, nb):
    """The reference-free prediction of the blended output's error (module
    docstring of serve.py) against the error measured with the known truth,
    for a linear smoothing 'denoiser' whose bias and noise are both sizeable."""
    from voidray_gb300.serve import blend_prediction

    yy, xx = np.mgrid[0:96, 0:96] / 96.0
    truth = np.stack([0.2 + 0.6 * (xx > 0.5) + 0.2 * yy, 0.5 + 0.3 * np.sin(6 * xx), 0.3 + 0.0 * yy], -1)
    sigma = 0.8 * (0.3 + truth)
    pred_p, pred_y, true_p, true_y = [], [], [], []
    for seed in range(6):
        a, b, p = _halves(truth, sigma, na, nb, seed)
        vp, blend, alpha = blend_prediction(a, b, p, _box(a), _box(b), na, nb)
        assert 0.0 < alpha < 1.0
        pred_p.append(vp)
        pred_y.append(blend)
        true_p.append(_relmse(p, truth))
        true_y.append(_relmse(alpha * _box(p) + (1 - alpha) * p, truth))
    assert np.mean(pred_p) == pytest.approx(np.mean(true_p), rel=0.15)
    assert np.mean(true_y) < 0.8 * np.mean(true_p)          # the blend helps here
    # normalising by the noisy plain mean makes the blend prediction err on
    # the safe side (jobs stop late, not early), by well under 2x
    assert 0.95 * np.mean(true_y) <= np.mean(pred_y) <= 1.6 * np.mean(true_y)


def test_blend_prediction_limits():
    from voidray_gb300.serve import blend_prediction

    truth = np.full((32, 32, 3), 0.5)
    a, b, p = _halves(truth, 0.5, 32, 32, 1)
    # a perfect denoiser takes the whole weight, a uselessly biased one none
    vp, blend, alpha = blend_prediction(a, b, p, truth, truth, 32, 32)
    assert alpha == pytest.approx(1.0, abs=0.05) and blend < 0.1 * vp
    vp, blend, alpha = blend_prediction(a, b, p, a + 0.5, b + 0.5, 32, 32)
    assert alpha < 0.05 and blend == pytest.approx(vp, rel=0.1)


ADAPTIVE = ServerConfig(adaptive=True, pass_paths=4 * 64 * 64, first_pass_spp=64, min_samples=64, max_active=64)


def test_adaptive_same_alone_and_in_mix():
    """Predictive allocation: a job's pass sizes follow its own estimates, so
    its samples, stopping point and image are the same in any mix."""
    def run(mix):
        s = Server(FakeBackend(noise=0.3), ADAPTIVE, clock=Clock())
        for k in range(mix):   # earlier arrivals take the pass budget first
            s.submit(req(seed=100 + k, target=5e-4, max_samples=4096))
        jid = s.submit(req(seed=7, target=1e-3, max_samples=4096))
        while not s.idle():
            s.step()
        j = s.status(jid)
        return j.result, j.samples, j.n_a, j.n_b

    r0, r1 = run(0), run(6)
    assert r0[1:] == r1[1:] and np.array_equal(r0[0], r1[0])


def test_adaptive_meets_target_in_few_passes():
    s = Server(FakeBackend(noise=0.3), ADAPTIVE, clock=Clock())
    jid = s.submit(req(seed=3, target=1e-3, max_samples=100000))
    while not s.idle():
        s.step()
    j = s.status(jid)
    assert j.estimate <= 1e-3
    assert j.passes <= 4                          # fixed 16-spp passes would need dozens
    assert abs(j.n_a - j.n_b) <= j.samples // 4   # halves stay balanced


def test_adaptive_finishes_jobs_in_admission_order():
    s = Server(FakeBackend(noise=0.3), ADAPTIVE, clock=Clock())
    ids = [s.submit(req(seed=20 + k, target=1e-3, max_samples=100000)) for k in range(6)]
    while not s.idle():
        s.step()
    finished = [s.status(i).finished for i in ids]
    assert finished == sorted(finished)


PIPELINED = ServerConfig(adaptive=True, pipelined=True, pass_paths=4 * 64 * 64, first_pass_spp=64, min_samples=64,
                         max_active=64)


class LaggingBackend(FakeBackend):
    """Estimates become visible only after `lag` polls, like device work still in flight."""

    def __init__(self, lag=2, **kw):
        super().__init__(**kw)
        self.lag = lag

    def estimate_async(self, jobs, after):
        return {"left": self.lag, "ests": [self.estimate(j) for j in jobs]}

    def poll(self, handle, block=False):
        if block:
            handle["left"] = 0
        if handle["left"] > 0:
            handle["left"] -= 1
            return None
        return handle["ests"]


@pytest.mark.parametrize("backend", [FakeBackend, LaggingBackend])
def test_pipelined_same_alone_and_in_mix(backend):
    """Pipelined passes: estimates arrive late, other jobs render meanwhile;
    each job's samples and image are still those of the job alone."""
    def run(mix):
        s = Server(backend(noise=0.3), PIPELINED, clock=Clock())
        for k in range(mix):
            s.submit(req(seed=100 + k, target=5e-4, max_samples=4096))
        jid = s.submit(req(seed=7, target=1e-3, max_samples=4096))
        while not s.idle():
            s.step()
        j = s.status(jid)
        assert j.estimate <= 1e-3 and not s.pending
        return j.result, j.samples, j.n_a, j.n_b

    r0, r1 = run(0), run(6)
    assert r0[1:] == r1[1:] and np.array_equal(r0[0], r1[0])


def test_pipelined_renders_while_estimates_are_in_flight():
    be = LaggingBackend(lag=3, noise=0.3)
    s = Server(be, PIPELINED, clock=Clock())
    ids = [s.submit(req(seed=40 + k, target=1e-3, max_samples=100000)) for k in range(8)]
    while not s.idle():
        s.step()
    # some pass rendered jobs while another job's estimate was still pending
    seen = [set(j for j, *_ in call) for call in be.calls]
    assert len(seen) >= 3 and any(len(a - b) > 0 for a, b in zip(seen, seen[1:]))
    assert all(s.status(i).state == "done" for i in ids)


class DepthBackend(LaggingBackend):
    """Records how many passes had estimates outstanding when each pass was issued."""

    def __init__(self, server_ref, **kw):
        super().__init__(**kw)
        self.server_ref = server_ref
        self.depths = []

    def render_async(self, work):
        self.depths.append(len(self.server_ref[0].pending))
        return super().render_async(work)


@pytest.mark.parametrize("fill_paths, deep", [(0, True), (1, False)])
def test_gpu_filling_passes_wait_for_their_estimates(fill_paths, deep):
    """A pass of at least fill_paths paths is not followed by another pass
    until its estimates are back; smaller passes still pipeline."""
    ref = [None]
    be = DepthBackend(ref, lag=3, noise=0.3)
    cfg = ServerConfig(adaptive=True, pipelined=True, pass_paths=4 * 64 * 64, first_pass_spp=64, min_samples=64,
                       max_active=64, max_inflight=3, fill_paths=fill_paths)
    s = Server(be, cfg, clock=Clock())
    ref[0] = s
    ids = [s.submit(req(seed=60 + k, target=1e-3, max_samples=100000)) for k in range(6)]
    while not s.idle():
        s.step()
    assert all(s.status(i).state == "done" for i in ids)
    # fill_paths=1: every pass fills the GPU, so none is issued behind another
    assert (max(be.depths) > 1) == deep
    if not deep:
        assert max(be.depths) == 0


def test_blend_samples_needed_is_consistent():
    """The planned sample count brings the predicted error to the target:
    scaling the noise moments by n / n' at the returned n' lands on it."""
    from voidray_gb300.serve import blend_from_moments, blend_samples_needed

    yy, xx = np.mgrid[0:64, 0:64] / 64.0
    truth = np.stack([0.2 + 0.6 * (xx > 0.5), 0.5 + 0.3 * np.sin(6 * xx), 0.3 + 0.0 * yy], -1)
    a, b, p = _halves(truth, 0.8 * (0.3 + truth), 32, 32, 0)
    from voidray_gb300.serve import blend_moments

    m = [float(x) for x in blend_moments(a, b, p, _box(a), _box(b))]
    plain, blend, _ = blend_from_moments(m, 32, 32)
    target = 0.5 * min(plain, blend)
    n2 = blend_samples_needed(m, 32, 32, target)
    assert n2 > 64
    # plain alone would need 64 * plain / target samples; the blend needs fewer
    assert n2 <= int(np.ceil(64 * plain / target)) + 1
    assert blend_samples_needed(m, 32, 32, 10.0) == 64


@pytest.mark.parametrize("pipelined", [False, True])
def test_srpt_order_keeps_results_mix_independent(pipelined):
    cfg = ServerConfig(adaptive=True, pipelined=pipelined, order="srpt", pass_paths=4 * 64 * 64, first_pass_spp=64,
                       min_samples=64, max_active=64)

    def run(mix):
        s = Server(LaggingBackend(noise=0.3), cfg, clock=Clock())
        for k in range(mix):
            s.submit(req(seed=100 + k, target=5e-4 if k % 2 else 2e-3, max_samples=4096))
        jid = s.submit(req(seed=7, target=1e-3, max_samples=4096))
        while not s.idle():
            s.step()
        j = s.status(jid)
        return j.result, j.samples

    r0, r1 = run(0), run(7)
    assert r0[1] == r1[1] and np.array_equal(r0[0], r1[0])


def test_srpt_finishes_short_jobs_first():
    cfg = ServerConfig(adaptive=True, order="srpt", pass_paths=64 * 64, first_pass_spp=64, min_samples=64)
    s = Server(FakeBackend(noise=0.3), cfg, clock=Clock())
    long_ = s.submit(req(seed=1, target=2e-4, max_samples=100000))
    short = s.submit(req(seed=2, target=2e-3, max_samples=100000))
    while not s.idle():
        s.step()
    assert s.status(short).finished < s.status(long_).finished


def test_tile_blend_beats_global_blend_where_regions_differ():
    """Half the image smooth (the box 'denoiser' is nearly unbiased there),
    half fine detail (it is badly biased): per-tile weights predict and
    achieve a lower error than one global weight, and the tile prediction
    stays on the safe side of the truth."""
    from voidray_gb300.serve import blend_prediction, blend_tile_moments, tile_blend

    yy, xx = np.mgrid[0:128, 0:128]
    detail = 0.5 + 0.4 * ((xx // 2 + yy // 2) % 2)
    truth = np.where((xx < 64)[..., None], 0.5, detail[..., None]) * np.ones((1, 1, 3))
    sigma = 0.9 * (0.3 + truth)
    na = nb = 32
    pred, true_t, true_g = [], [], []
    for seed in range(4):
        a, b, p = _halves(truth, sigma, na, nb, seed)
        mt = blend_tile_moments(a, b, p, _box(a), _box(b), 16)
        _, blend_t, alpha_map = tile_blend(mt, na, nb)
        _, blend_g, alpha_g = blend_prediction(a, b, p, _box(a), _box(b), na, nb)
        am = np.repeat(np.repeat(alpha_map, 16, 0), 16, 1)[..., None]
        true_t.append(_relmse(am * _box(p) + (1 - am) * p, truth))
        true_g.append(_relmse(alpha_g * _box(p) + (1 - alpha_g) * p, truth))
        pred.append(blend_t)
        assert alpha_map[:, :4].mean() > alpha_map[:, 4:].mean() + 0.2  # smooth half leans on the denoiser
    assert np.mean(true_t) < 0.9 * np.mean(true_g)
    assert 0.9 * np.mean(true_t) <= np.mean(pred) <= 1.8 * np.mean(true_t)


@pytest.mark.parametrize("adaptive", [False, True])
def test_checkpoint_resume_finishes_like_uninterrupted(tmp_path, adaptive):
    """A job checkpointed after a few passes and resumed on a new server (with
    other jobs in the mix) renders exactly the passes it had left: the same
    sample count, estimate and image as without the interruption."""
    cfg = ServerConfig(spp_per_pass=8, min_samples=16, adaptive=adaptive, first_pass_spp=16, pass_paths=8 * 8 * 64)
    target = 2e-3

    def full():
        s = Server(FakeBackend(), cfg, clock=Clock())
        jid = s.submit(req(seed=3, target=target, max_samples=512))
        while not s.idle():
            s.step()
        j = s.status(jid)
        return j.result, j.samples, j.estimate, j.passes

    ref = full()
    assert ref[3] >= 2   # at least two passes, so a checkpoint before the last one leaves work to do

    s = Server(FakeBackend(), cfg, clock=Clock())
    jid = s.submit(req(seed=3, target=target, max_samples=512))
    for _ in range(ref[3] - 1):
        s.step()
    assert s.status(jid).state == "active"
    path = str(tmp_path / "job.npz")
    s.checkpoint(jid, path)
    s2 = Server(FakeBackend(), cfg, clock=Clock())
    others = [s2.submit(req(seed=50 + k, target=5e-4, max_samples=128)) for k in range(2)]
    rid = s2.submit(req(seed=3, target=target, max_samples=512), resume=path)
    while not s2.idle():
        s2.step()
    j = s2.status(rid)
    assert (j.samples, j.estimate, j.passes) == ref[1:]
    assert np.array_equal(j.result, ref[0])
    assert all(s2.status(o).state == "done" for o in others)


def test_checkpoint_rejects_mismatch_and_in_flight(tmp_path):
    s = Server(FakeBackend(), ServerConfig(spp_per_pass=8, min_samples=16), clock=Clock())
    jid = s.submit(req(seed=3, max_samples=256))
    with pytest.raises(ValueError):
        s.checkpoint(jid, str(tmp_path / "w.npz"))   # still waiting
    s.step()
    s.checkpoint(jid, str(tmp_path / "a.npz"))
    with pytest.raises(ValueError):
        Server(FakeBackend()).submit(req(seed=4), resume=str(tmp_path / "a.npz"))


hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402


@settings(max_examples=40, deadline=None)
@given(seed=st.integers(0, 10_000), n_jobs=st.integers(1, 12), budget_jobs=st.integers(1, 6),
       mode=st.sampled_from(["plain", "adaptive", "pipelined"]), cancel_every=st.integers(0, 5))
def test_scheduler_invariants_under_random_load(seed, n_jobs, budget_jobs, mode, cancel_every):
    """Random arrivals, sizes, targets, memory budgets and cancellations:
    memory in use never exceeds the budget, every job ends done, cancelled
    or failed with its memory returned, and a chosen job's result equals
    its result alone (whatever else ran, unless it was cancelled)."""
    rng = np.random.default_rng(seed)
    sizes = [(int(rng.integers(4, 17)), int(rng.integers(4, 17))) for _ in range(n_jobs)]
    foot = max(2 * w * h * 16 for w, h in sizes)
    cfg = ServerConfig(memory_budget=budget_jobs * foot, max_active=int(rng.integers(1, 9)), spp_per_pass=8,
                       min_samples=16, adaptive=mode != "plain", pipelined=mode == "pipelined",
                       pass_paths=int(rng.integers(1, 5)) * 16 * 16 * 32, first_pass_spp=16)

    def make(k):
        w, h = sizes[k]
        return req(seed=1000 + k, w=w, h=h, target=float(rng.choice([5e-4, 1e-3, 3e-3])),
                   max_samples=int(rng.choice([64, 256, 1024])), scene=f"s{k % 3}")

    reqs = [make(k) for k in range(n_jobs)]
    s = Server(LaggingBackend(lag=int(rng.integers(0, 3)), noise=0.3), cfg, clock=Clock())
    ids = []
    step = 0
    pending = list(range(n_jobs))
    while pending or not s.idle():
        if pending and (step % 2 == 0 or s.idle()):
            ids.append(s.submit(reqs[pending.pop(0)]))
        s.step()
        step += 1
        assert 0 <= s.used <= cfg.memory_budget
        if cancel_every and step % (cancel_every + 3) == 0:
            live = [i for i in ids if s.status(i).state in ("waiting", "active") and i != ids[0]]
            if live:
                s.cancel(live[0])
        assert step < 100_000
    assert s.used == 0 and not s.resident_scenes
    assert all(s.status(i).state in ("done", "cancelled", "failed") for i in ids)
    # the first job (never cancelled) ends as it does alone
    j0 = s.status(ids[0])
    alone = Server(LaggingBackend(lag=0, noise=0.3), cfg, clock=Clock())
    a = alone.submit(reqs[0])
    while not alone.idle():
        alone.step()
    ja = alone.status(a)
    assert j0.state == ja.state == "done"
    assert (j0.samples, j0.n_a, j0.n_b) == (ja.samples, ja.n_a, ja.n_b)
    assert np.array_equal(j0.result, ja.result)
