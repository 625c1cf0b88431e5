"""Continuous-batching serving loop for sparse-convolution stacks.

Requests (one voxel grid + per-voxel features each) arrive over time.  The scheduler keeps
a queue, admits requests into the next batch while their estimated device footprint fits an
HBM budget and a stream slot is free, packs each batch into one jagged GridBatch (every
kernel launch covers all grids of the batch), and launches it on its own CUDA stream.  While
earlier batches are still running, newly arrived requests are admitted as slots and memory
free up, so their work overlaps on the device.  Finished batches are detected by CUDA events
and their outputs are copied to pinned host memory asynchronously.  Latency is measured from
arrival to the moment the result is on the host.

Per-request results do not depend on the batch a request lands in: grids of a batch never
read each other's voxels, every output row is written once by one CTA, and a row's
accumulation order does not depend on the other rows of its tile (offsets a row lacks add
exact zeros).  The stack's outputs alone and in a mix are therefore bit-identical.

The reference has no serving loop; this is the build's continuous-batching layer over the
SparseConv3d path (fvdb/nn/modules.py:156-404 semantics).
"""

from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Sequence

import torch


@dataclasses.dataclass
class Request:
    """One grid to run through the stack.  ijk int32 [N, 3] and features [N, C] (host or
    device); ``arrival`` in seconds on the server clock."""

    rid: int
    ijk: torch.Tensor
    features: torch.Tensor
    arrival: float = 0.0
    # filled by the server
    output: torch.Tensor | None = None  # [N, C_out] rows in the grid's voxel order
    out_ijk: torch.Tensor | None = None  # voxel coordinates of the output rows
    done: float | None = None
    error: str | None = None
    batch_id: int | None = None

    @property
    def n_voxels(self) -> int:
        return int(self.ijk.shape[0])

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


class Executor:
    """Runs batches.  launch() returns a handle; poll() is non-blocking; finish() fills the
    requests' outputs (or raises)."""

    def footprint(self, req: Request) -> int:  # bytes of device memory the request needs
        raise NotImplementedError

    def launch(self, batch: list[Request], slot: int):
        raise NotImplementedError

    def poll(self, handle) -> bool:
        raise NotImplementedError

    def finish(self, handle) -> None:
        raise NotImplementedError


class ContinuousBatcher:
    """Scheduler of the serving loop (device-independent).

    hbm_budget: bytes the in-flight batches may use together (admission control);
    max_batch_voxels: cap on the voxels of one batch; slots: batches in flight at once
    (one CUDA stream each)."""

    def __init__(self, executor: Executor, hbm_budget: int, max_batch_voxels: int, slots: int = 2,
                 clock: Callable[[], float] = time.perf_counter, max_batch_requests: int | None = None):
        if slots < 1:
            raise ValueError("slots must be >= 1")
        self.ex = executor
        self.budget = int(hbm_budget)
        self.max_batch_voxels = int(max_batch_voxels)
        self.max_batch_requests = max_batch_requests
        self.slots = slots
        self.clock = clock
        self.queue: collections.deque[Request] = collections.deque()
        self.in_flight: dict[int, tuple[object, list[Request], int]] = {}  # slot -> (handle, batch, bytes)
        self.used = 0
        self.finished: list[Request] = []
        self.batches = 0
        self.peak_used = 0

    def submit(self, req: Request) -> None:
        need = self.ex.footprint(req)
        if need > self.budget or req.n_voxels > self.max_batch_voxels:
            req.error = f"request needs {need} bytes / {req.n_voxels} voxels: larger than the server's budget"
            req.done = self.clock()
            self.finished.append(req)
            return
        self.queue.append(req)

    def _reap(self) -> None:
        for slot in list(self.in_flight):
            handle, batch, nbytes = self.in_flight[slot]
            if not self.ex.poll(handle):
                continue
            try:
                self.ex.finish(handle)
            except Exception as e:  # the whole batch failed: retry its requests one by one
                self._isolate(batch, e)
            now = self.clock()
            for r in batch:
                if r.done is None:
                    r.done = now
                self.finished.append(r)
            self.used -= nbytes
            del self.in_flight[slot]

    def _isolate(self, batch: list[Request], err: Exception) -> None:
        if len(batch) == 1:
            batch[0].error = f"{type(err).__name__}: {err}"
            return
        for r in batch:
            try:
                h = self.ex.launch([r], slot=0)
                while not self.ex.poll(h):
                    time.sleep(1e-4)
                self.ex.finish(h)
            except Exception as e:
                r.error = f"{type(e).__name__}: {e}"

    def _admit(self) -> None:
        free = [s for s in range(self.slots) if s not in self.in_flight]
        while free and self.queue:
            batch, vox, nbytes = [], 0, 0
            while self.queue:
                if self.max_batch_requests is not None and len(batch) >= self.max_batch_requests:
                    break
                r = self.queue[0]
                need = self.ex.footprint(r)
                if self.used + nbytes + need > self.budget or vox + r.n_voxels > self.max_batch_voxels:
                    break
                batch.append(self.queue.popleft())
                vox += r.n_voxels
                nbytes += need
            if not batch:
                return  # wait for memory to free up
            slot = free.pop(0)
            for r in batch:
                r.batch_id = self.batches
            self.batches += 1
            try:
                handle = self.ex.launch(batch, slot)
            except Exception as e:
                self._isolate(batch, e)
                now = self.clock()
                for r in batch:
                    if r.done is None:
                        r.done = now
                    self.finished.append(r)
                continue
            self.in_flight[slot] = (handle, batch, nbytes)
            self.used += nbytes
            self.peak_used = max(self.peak_used, self.used)

    def step(self) -> None:
        self._reap()
        self._admit()

    def idle(self) -> bool:
        return not self.queue and not self.in_flight

    def serve(self, requests: Sequence[Request], poll_sleep: float = 5e-5) -> list[Request]:
        """Replays `requests` at their arrival times (seconds from now) and serves them all."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = self.clock()
        for r in pending:
            r.arrival += t0
        i = 0
        while i < len(pending) or not self.idle():
            now = self.clock()
            while i < len(pending) and pending[i].arrival <= now:
                self.submit(pending[i])
                i += 1
            self.step()
            if i < len(pending) and self.idle():
                time.sleep(max(0.0, min(pending[i].arrival - self.clock(), 1e-3)))
            elif poll_sleep:
                time.sleep(poll_sleep)
        for r in pending:
            r.arrival -= t0
            if r.done is not None:
                r.done -= t0
        return pending


def latency_stats(reqs: Sequence[Request]) -> dict:
    lat = sorted(r.latency for r in reqs if r.error is None and r.latency is not None)
    if not lat:
        return {"n": 0}

    def pct(p):
        return lat[min(len(lat) - 1, max(0, math.ceil(p / 100.0 * len(lat)) - 1))]

    span = max(r.done for r in reqs if r.done is not None) - min(r.arrival for r in reqs)
    vox = sum(r.n_voxels for r in reqs if r.error is None)
    return {"n": len(lat), "p50_ms": pct(50) * 1e3, "p99_ms": pct(99) * 1e3, "mean_ms": sum(lat) / len(lat) * 1e3,
            "voxels_per_s": vox / span if span > 0 else None, "span_s": span}


# ---------------------------------------------------------------------------- GPU executor
class ConvStack:
    """The served model: 3x3x3 stride-1 SparseConv3d layers with ReLU between them, one
    kernel map per batch grid reused by every layer."""

    def __init__(self, channels: Sequence[int], device, dtype=torch.bfloat16, seed: int = 0, kernel_size: int = 3):
        import fvdb

        g = torch.Generator().manual_seed(seed)
        self.fvdb = fvdb
        self.channels = list(channels)
        self.dtype = dtype
        self.kernel_size = kernel_size
        k3 = kernel_size**3
        self.weights = []
        for cin, cout in zip(self.channels[:-1], self.channels[1:]):
            w = torch.randn(cout, cin, kernel_size, kernel_size, kernel_size, generator=g) * math.sqrt(2.0 / (cin * k3))
            self.weights.append(w.to(device, dtype))

    def to_dtype(self, dtype) -> "ConvStack":
        other = object.__new__(ConvStack)
        other.__dict__.update(self.__dict__)
        other.dtype = dtype
        other.weights = [w.to(dtype) for w in self.weights]
        return other

    def bytes_per_voxel(self) -> int:
        es = torch.empty(0, dtype=self.dtype).element_size()
        act = sum(self.channels) * es + max(self.channels) * 4  # activations (+ transient)
        return act + self.kernel_size**3 * 4 + 4 + 160  # map, tile masks, grid build buffers

    def __call__(self, grid, x: torch.Tensor) -> torch.Tensor:
        pack, _ = grid.sparse_conv_kernel_map(self.kernel_size, 1)
        h = x.to(self.dtype)
        for i, w in enumerate(self.weights):
            # ReLU between layers, fused into the convolution's epilogue
            h = pack._conv_with_bias(h, w, None, False, None, relu=i + 1 < len(self.weights)).jdata
        return h


class GPUExecutor(Executor):
    """Packs a batch into one jagged GridBatch and runs the stack on the slot's CUDA stream.

    Each slot has a host worker thread of its own: launch() only hands the batch to it, so the
    scheduler never waits for a grid build's count read (the one host synchronisation of a
    build) and keeps admitting requests while batches are being built and run.  The native
    calls release the GIL while they wait.  Each slot's kernels report bounded-wait timeouts
    through the error flag of the slot's stream, so a failure is charged to its own batch."""

    def __init__(self, model: ConvStack, device, slots: int = 2):
        import concurrent.futures

        self.model = model
        self.device = torch.device(device)
        n = max(slots, 1)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(n)]
        self.workers = [concurrent.futures.ThreadPoolExecutor(max_workers=1, thread_name_prefix=f"fvdb-slot{i}")
                        for i in range(n)]

    def footprint(self, req: Request) -> int:
        return req.n_voxels * self.model.bytes_per_voxel() + (1 << 20)

    def _run(self, batch: list[Request], slot: int):
        fvdb = self.model.fvdb
        stream = self.streams[slot % len(self.streams)]
        with torch.cuda.device(self.device), torch.cuda.stream(stream):
            ijk = torch.cat([r.ijk for r in batch]).to(self.device, non_blocking=True)
            feats = torch.cat([r.features for r in batch]).to(self.device, non_blocking=True)
            offs = torch.tensor([0] + [r.n_voxels for r in batch], dtype=torch.int64).cumsum(0)
            jt = fvdb.JaggedTensor.from_data_and_offsets(ijk, offs.to(self.device, non_blocking=True))
            grid = fvdb.GridBatch.from_ijk(jt)
            # features arrive per input row: place them at their voxel's index
            idx = grid.ijk_to_index(jt, cumulative=True).jdata
            x = torch.zeros((grid.total_voxels, feats.shape[1]), dtype=feats.dtype, device=self.device)
            x[idx] = feats
            y = self.model(grid, x)
            out = torch.empty(y.shape, dtype=y.dtype, pin_memory=True)
            out.copy_(y, non_blocking=True)
            out_ijk = torch.empty(grid.ijk.jdata.shape, dtype=torch.int32, pin_memory=True)
            out_ijk.copy_(grid.ijk.jdata, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        # the grid's voxel offsets were read to the host by its build: no device read here
        return ev, out, out_ijk, grid._impl.joffsets_host.tolist()

    def launch(self, batch: list[Request], slot: int):
        return (self.workers[slot % len(self.workers)].submit(self._run, batch, slot), batch, slot)

    def poll(self, handle) -> bool:
        fut = handle[0]
        if not fut.done():
            return False
        return fut.exception() is not None or fut.result()[0].query()

    def finish(self, handle) -> None:
        fut, batch, slot = handle
        ev, out, out_ijk, o = fut.result()  # re-raises a failure of the build or the launch
        ev.synchronize()
        with torch.cuda.device(self.device), torch.cuda.stream(self.streams[slot % len(self.streams)]):
            self.model.fvdb._lib.load().check_device_errors(self.device)
        for b, r in enumerate(batch):
            r.output = out[o[b] : o[b + 1]]
            r.out_ijk = out_ijk[o[b] : o[b + 1]]

    def close(self) -> None:
        for w in self.workers:
            w.shutdown(wait=True)


def run_alone(model: ConvStack, req: Request, device) -> tuple[torch.Tensor, torch.Tensor]:
    """The stack on one request by itself (reference for the mix-invariance test and the
    per-request baseline)."""
    fvdb = model.fvdb
    ijk = req.ijk.to(device)
    grid = fvdb.GridBatch.from_ijk(ijk)
    idx = grid.ijk_to_index(ijk, cumulative=True).jdata
    x = torch.zeros((grid.total_voxels, req.features.shape[1]), dtype=req.features.dtype, device=device)
    x[idx] = req.features.to(device)
    y = model(grid, x)
    return y.cpu(), grid.ijk.jdata.cpu()
