"""The serving scheduler on the CPU with a fake executor: HBM-budget admission, continuous
batching into free slots while other batches run, rejection of oversized requests, isolation
of a failing request, latency percentiles.  Failures are made on the host (an executor that
raises), nothing touches a GPU."""

import time

import pytest
import torch

from fvdb.serving import ContinuousBatcher, Executor, Request, latency_stats


class FakeExecutor(Executor):
    def __init__(self, bytes_per_voxel=10, seconds_per_voxel=2e-6, bad=()):
        self.bpv = bytes_per_voxel
        self.spv = seconds_per_voxel
        self.bad = set(bad)
        self.concurrent = 0
        self.max_concurrent = 0
        self.launched: list[list[int]] = []

    def footprint(self, req):
        return req.n_voxels * self.bpv

    def launch(self, batch, slot):
        self.launched.append([r.rid for r in batch])
        self.concurrent += 1
        self.max_concurrent = max(self.max_concurrent, self.concurrent)
        return {"t_end": time.perf_counter() + self.spv * sum(r.n_voxels for r in batch), "batch": batch, "open": True}

    def poll(self, h):
        return time.perf_counter() >= h["t_end"]

    def finish(self, h):
        if h["open"]:
            self.concurrent -= 1
            h["open"] = False
        if any(r.rid in self.bad for r in h["batch"]):
            raise RuntimeError("injected failure")
        for r in h["batch"]:
            r.output = r.features * 2


def _req(rid, n, arrival=0.0):
    return Request(rid=rid, ijk=torch.zeros((n, 3), dtype=torch.int32), features=torch.full((n, 2), float(rid)), arrival=arrival)


def test_budget_admission_and_continuous_batching():
    ex = FakeExecutor()
    srv = ContinuousBatcher(ex, hbm_budget=10 * 3000, max_batch_voxels=2000, slots=2)
    reqs = [_req(i, 1000, arrival=0.004 * (i // 3)) for i in range(12)]  # arrivals in bursts of three
    out = srv.serve(reqs)
    assert all(r.error is None for r in out)
    assert all(torch.equal(r.output, r.features * 2) for r in out)
    assert srv.peak_used <= 10 * 3000  # never over budget
    assert ex.max_concurrent == 2  # a second batch ran while the first was in flight
    assert any(len(b) > 1 for b in ex.launched)  # requests were packed together
    assert all(len(b) <= 2 for b in ex.launched)  # max_batch_voxels respected
    # FIFO admission order
    flat = [rid for b in ex.launched for rid in b]
    assert flat == sorted(flat)


def test_oversized_request_is_rejected_and_others_served():
    ex = FakeExecutor()
    srv = ContinuousBatcher(ex, hbm_budget=10 * 5000, max_batch_voxels=100000, slots=2)
    reqs = [_req(0, 100), _req(1, 10000), _req(2, 100)]
    out = {r.rid: r for r in srv.serve(reqs)}
    assert out[1].error is not None and "budget" in out[1].error
    assert out[0].error is None and out[2].error is None


def test_failing_request_is_isolated():
    ex = FakeExecutor(bad={3})
    srv = ContinuousBatcher(ex, hbm_budget=10**9, max_batch_voxels=10**9, slots=1)
    reqs = [_req(i, 50) for i in range(6)]  # all arrive at once: one batch
    out = {r.rid: r for r in srv.serve(reqs)}
    assert "injected failure" in out[3].error
    for i in (0, 1, 2, 4, 5):
        assert out[i].error is None and torch.equal(out[i].output, out[i].features * 2)


def test_latency_stats():
    reqs = [_req(i, 10) for i in range(100)]
    for i, r in enumerate(reqs):
        r.arrival, r.done = 0.0, (i + 1) * 1e-3
    s = latency_stats(reqs)
    assert s["n"] == 100
    assert s["p50_ms"] == pytest.approx(50.0)
    assert s["p99_ms"] == pytest.approx(99.0)


def test_slots_must_be_positive():
    with pytest.raises(ValueError):
        ContinuousBatcher(FakeExecutor(), 1000, 1000, slots=0)
