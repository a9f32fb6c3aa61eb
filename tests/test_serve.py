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
