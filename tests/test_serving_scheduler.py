"""The continuous-batching scheduler's host logic (no GPU): the device work
of a request is replaced by a timer, so that admission by arrival, free
slots and the HBM budget, the two phases of a gradient request and the
statistics can be checked on the CPU."""
import threading
import time

import pytest

from geophyinv_gb300 import serving


class _FakeJob:
    """A request whose phases take a fixed host time; records the set of
    requests on the 'device' so that the test can check the budget."""
    live = {}
    peak_bytes = 0
    peak_count = 0
    lock = threading.Lock()
    phase_s = 0.02

    def __init__(self, req, graphs, stream):
        self.req = req
        self.res = serving.Result(req.rid, req.kind)
        self.phase = 0
        self.busy = None
        self.error = None
        self.pa = self
        self.t_end = time.perf_counter() + self.phase_s
        with self.lock:
            _FakeJob.live[req.rid] = serving.plan_bytes_estimate(req)
            _FakeJob.peak_bytes = max(_FakeJob.peak_bytes, sum(_FakeJob.live.values()))
            _FakeJob.peak_count = max(_FakeJob.peak_count, len(_FakeJob.live))

    def launch(self):
        pass

    def done(self):
        return time.perf_counter() >= self.t_end

    def finish_phase(self, pool=None):
        if self.req.kind == "acoustic_gradient" and self.phase == 0:
            self.phase = 1
            self.t_end = time.perf_counter() + self.phase_s
            return False
        self.res.records = ["phase %d" % self.phase]
        return True

    def close(self):
        with self.lock:
            _FakeJob.live.pop(self.req.rid, None)


class _FakeStream:
    cuda_stream = 0


@pytest.fixture
def fake(monkeypatch):
    _FakeJob.live = {}
    _FakeJob.peak_bytes = 0
    _FakeJob.peak_count = 0
    monkeypatch.setattr(serving, "_prepare", lambda req, graphs, stream: _FakeJob(req, graphs, stream))
    monkeypatch.setattr(serving, "_streams", lambda n: [_FakeStream() for _ in range(n)])
    return _FakeJob


def test_every_request_completes_and_gradients_take_two_phases(fake):
    reqs = serving.make_stream(20, rate=1000.0, seed=1, sides=(50, 100), steps=(10, 20), shots=(1, 3))
    res, st = serving.serve(reqs, max_inflight=4, realtime=False)
    assert sorted(res) == [r.rid for r in reqs]
    for r in reqs:
        assert res[r.rid].records == ["phase %d" % (1 if r.kind == "acoustic_gradient" else 0)]
        assert res[r.rid].t_done >= res[r.rid].t_admit
    assert st["requests"] == 20 and st["shots"] == sum(r.nshots for r in reqs)
    assert 0 < st["p50_s"] <= st["p99_s"]
    assert fake.peak_count <= 4


def test_admission_keeps_the_device_under_the_hbm_budget(fake):
    reqs = serving.make_stream(12, rate=1000.0, seed=2, sides=(50, 100), steps=(10, 20), shots=(1, 3))
    sizes = sorted(serving.plan_bytes_estimate(r) for r in reqs)
    budget = sizes[-1] + sizes[-2] - 1  # never room for the two largest together
    serving.serve(reqs, hbm_budget=budget, max_inflight=8, realtime=False)
    assert fake.peak_bytes <= budget
    assert fake.peak_count >= 2  # but smaller ones overlap


def test_requests_are_admitted_after_they_arrive(fake):
    reqs = serving.make_stream(6, rate=50.0, seed=3, sides=(50, 60), steps=(10, 12), shots=(1, 1))
    res, _ = serving.serve(reqs, max_inflight=8, realtime=True)
    for r in reqs:
        assert res[r.rid].t_admit >= r.arrival - 1e-3
