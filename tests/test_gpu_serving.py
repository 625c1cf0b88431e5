"""Serving on the GPU: requests of very different sizes are packed into jagged batches on
several streams while others run; every result is bit-identical to the same request run
alone (stated tolerance: exact), and latency statistics are reported."""

import numpy as np
import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def _requests(n_req, seed):
    from fvdb.serving import Request

    rng = np.random.default_rng(seed)
    reqs = []
    t = 0.0
    for i in range(n_req):
        n = int(np.exp(rng.uniform(np.log(300), np.log(30000))))
        ijk = torch.from_numpy(random_sparse_ijk(n, 48, seed * 100 + i, lo=int(rng.integers(-64, 64))))
        # features given per input row, rows in a random order
        perm = torch.from_numpy(rng.permutation(ijk.shape[0]))
        feats = torch.randn(ijk.shape[0], 32, generator=torch.Generator().manual_seed(i)).bfloat16()
        t += rng.exponential(1.0 / 400.0)
        reqs.append(Request(rid=i, ijk=ijk[perm].contiguous(), features=feats, arrival=t))
    return reqs


def test_results_identical_alone_and_in_the_mix(cuda_device):
    from fvdb.serving import ContinuousBatcher, ConvStack, GPUExecutor, latency_stats, run_alone

    model = ConvStack([32, 64, 64, 32], cuda_device, seed=0)
    ex = GPUExecutor(model, cuda_device, slots=3)
    srv = ContinuousBatcher(ex, hbm_budget=1 << 30, max_batch_voxels=60000, slots=3)
    reqs = srv.serve(_requests(24, 1))
    assert all(r.error is None for r in reqs), [r.error for r in reqs if r.error]
    assert srv.batches < len(reqs)  # requests were packed
    sizes = {}
    for r in reqs:
        sizes.setdefault(r.batch_id, []).append(r.rid)
    assert max(len(v) for v in sizes.values()) > 1
    for r in reqs:
        y, ijk = run_alone(model, r, cuda_device)
        assert torch.equal(ijk, r.out_ijk)
        assert torch.equal(y, r.output), f"request {r.rid} differs between alone and batched"
    st = latency_stats(reqs)
    assert st["n"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0


def test_oversized_request_rejected_on_gpu(cuda_device):
    from fvdb.serving import ContinuousBatcher, ConvStack, GPUExecutor, Request

    model = ConvStack([32, 64], cuda_device)
    ex = GPUExecutor(model, cuda_device, slots=1)
    srv = ContinuousBatcher(ex, hbm_budget=1 << 22, max_batch_voxels=1 << 20, slots=1)
    big = Request(rid=0, ijk=torch.from_numpy(random_sparse_ijk(40000, 48, 0)), features=torch.zeros(40000, 32).bfloat16())
    small = Request(rid=1, ijk=torch.from_numpy(random_sparse_ijk(500, 16, 1)), features=torch.zeros(500, 32).bfloat16())
    out = {r.rid: r for r in srv.serve([big, small])}
    assert out[0].error is not None
    assert out[1].error is None and out[1].output.shape == (500, 64)


def test_footprint_bounds_measured_peak(cuda_device):
    """Admission's footprint() (the sum over a batch's requests) bounds the device memory the
    batch really takes: the growth of torch's peak allocation while the batch runs."""
    from fvdb.serving import ConvStack, GPUExecutor

    model = ConvStack([32, 64, 64, 32], cuda_device, seed=0)
    ex = GPUExecutor(model, cuda_device, slots=1)
    for seed, n_req in ((2, 1), (3, 6)):
        batch = _requests(n_req, seed)
        ex._run(batch, 0)  # first call: weight images and library state
        torch.cuda.synchronize(cuda_device)
        base = torch.cuda.memory_allocated(cuda_device)
        torch.cuda.reset_peak_memory_stats(cuda_device)
        ev, *_ = ex._run(batch, 0)
        ev.synchronize()
        peak = torch.cuda.max_memory_allocated(cuda_device) - base
        need = sum(ex.footprint(r) for r in batch)
        assert peak <= need, f"batch of {sum(r.n_voxels for r in batch)} voxels peaked at {peak} B > footprint {need} B"
