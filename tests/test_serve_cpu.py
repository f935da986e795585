"""Continuous-batching scheduler on the CPU with a fake executor: admission
against the memory budget, FIFO order, overlap of batches, and a failing
launch (failure injected on the host) that does not stop the service."""

import collections
import threading
import time

import numpy as np
import pytest

from fastlisaresponse_gb300.serve import BYTES_PER_SAMPLE, Request, ResponseServer, admit


class FakeExecutor:
    """Completes a batch `per_sample` seconds per sample after its launch;
    fails the launches whose index is in `fail_on`."""

    def __init__(self, lanes=2, per_sample=2e-7, fail_on=()):
        self.lanes = lanes
        self.per_sample = per_sample
        self.fail_on = set(fail_on)
        self.launches = []
        self.lock = threading.Lock()

    def launch(self, lane, batch):
        with self.lock:
            idx = len(self.launches)
            self.launches.append((lane, [r.n for r in batch], time.perf_counter()))
        if idx in self.fail_on:
            raise RuntimeError(f"injected failure on launch {idx}")
        end = time.perf_counter() + self.per_sample * sum(r.n for r in batch)
        return (end, [np.full(3, r.n) for r in batch])

    def finished(self, handle):
        return time.perf_counter() >= handle[0]

    def results(self, handle):
        return handle[1]


def _params(i):
    return (1e-22, 1e-3, 1e-15, 0.1 * i, 0.2, 0.3, 1.0, 0.5)


def test_admit_respects_budget_and_limits():
    q = collections.deque(Request(params=_params(i), n=n) for i, n in enumerate([100, 200, 300]))
    batch = admit(q, used=0, budget=350 * BYTES_PER_SAMPLE, max_batch_samples=10**9,
                  max_batch_sources=10)
    assert [r.n for r in batch] == [100, 200] and len(q) == 1
    q = collections.deque(Request(params=_params(i), n=100) for i in range(5))
    assert len(admit(q, 0, 10**12, max_batch_samples=250, max_batch_sources=10)) == 2
    assert len(admit(q, 0, 10**12, max_batch_samples=10**9, max_batch_sources=2)) == 2


def test_all_requests_complete_in_fifo_order():
    ex = FakeExecutor()
    with ResponseServer(0.1, executor=ex, memory_budget=1e12) as srv:
        reqs = [srv.submit(_params(i), 3000 + 10 * i) for i in range(40)]
        for r in reqs:
            assert r.result(timeout=10)[0] == r.n
    order = [n for _, ns, _ in ex.launches for n in ns]
    assert order == [r.n for r in reqs]
    st = srv.stats()
    assert st["requests"] == 40 and st["p99_ms"] >= st["p50_ms"] >= 0


def test_memory_budget_is_never_exceeded():
    ex = FakeExecutor(per_sample=1e-6)
    budget = 25000 * BYTES_PER_SAMPLE
    with ResponseServer(0.1, executor=ex, memory_budget=budget) as srv:
        reqs = [srv.submit(_params(i), 10000) for i in range(12)]
        for r in reqs:
            r.result(timeout=20)
    assert srv.peak_used <= budget
    assert max(len(ns) for _, ns, _ in ex.launches) <= 2
    with pytest.raises(ValueError, match="larger than the whole memory budget"):
        ResponseServer(0.1, executor=FakeExecutor(), memory_budget=1000).submit(_params(0), 5000)


def test_batches_overlap_on_two_lanes():
    """A request arriving while a long batch runs starts on the free lane
    before that batch finishes (continuous batching, not a queue)."""
    ex = FakeExecutor(per_sample=5e-6)  # 4e5 samples -> 2 s
    with ResponseServer(0.1, executor=ex, memory_budget=1e12) as srv:
        big = srv.submit(_params(0), 400000)
        time.sleep(0.05)
        small = srv.submit(_params(1), 3000)
        small.result(timeout=5)
        assert not big.done()
        assert small.t_launch < big.t_launch + 2.0
        big.result(timeout=20)
    assert {lane for lane, _, _ in ex.launches} == {0, 1}


def test_failed_launch_reports_and_service_continues():
    ex = FakeExecutor(fail_on={1})
    with ResponseServer(0.1, executor=ex, memory_budget=1e12, max_batch_sources=1) as srv:
        reqs = [srv.submit(_params(i), 3000) for i in range(4)]
        outcomes = []
        for r in reqs:
            try:
                r.result(timeout=10)
                outcomes.append("ok")
            except RuntimeError as e:
                outcomes.append(str(e))
    assert outcomes[1] == "injected failure on launch 1"
    assert outcomes.count("ok") == 3
    assert srv.used == 0


def test_invalid_requests_are_rejected():
    srv = ResponseServer(0.1, executor=FakeExecutor(), memory_budget=1e12)
    try:
        with pytest.raises(ValueError, match="params"):
            srv.submit((1.0, 2.0), 5000)
        with pytest.raises(ValueError, match="tdi_set"):
            srv.submit(_params(0), 5000, tdi_set=5)
        with pytest.raises(ValueError, match="garbage margin"):
            srv.submit(_params(0), 1500)
    finally:
        srv.close()


def test_dropped_results_keep_timings():
    """keep_results=False (load tests): results are released as requests
    complete, the timings and stats stay."""
    ex = FakeExecutor()
    with ResponseServer(0.1, executor=ex, memory_budget=1e12, keep_results=False) as srv:
        reqs = [srv.submit(_params(i), 3000 + i) for i in range(12)]
        for r in reqs:
            assert r.result(timeout=10) is None
    assert all(r.done() and r.latency >= 0 for r in reqs)
    assert srv.stats()["requests"] == 12
