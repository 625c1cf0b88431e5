"""Benchmark of the sparse-convolution hot path on one GB300 (or N replicas).

Workload (the headline configuration): a jagged batch of 4 surface-sparse grids, each from
2M points drawn uniformly on a random union of 3 sphere shells (radii U[0.2,0.45], centres
U[0.3,0.7]^3, clipped to [0,1)^3) voxelised at 256^3 (~150k-400k voxels per grid, seeds
100+b).  Layer 1: 3x3x3 stride-1 conv C 32->64; layer 2: 2x2x2 stride-2 conv C 64->64 onto
conv_grid(2,2).  Features N(0,1), Kaiming-normal weights, BF16 storage, FP32 accumulation.

One step = the forward of both layers as fvdb.nn.SparseConv3d runs it: kernel map of layer 1,
layer-1 contraction, conv_grid(2,2) + kernel map of layer 2, layer-2 contraction.
`value` = useful TFLOP/s of the step (2 * P * Cin * Cout summed over layers, P = valid
kernel-map entries), inputs resident in HBM.  `e2e` = the same metric through the public
API from pinned host buffers (ijk + features copied in, grid built, both layers, output read
back) per step.  The per-step working set (features, maps, outputs: several hundred MB) is
larger than the 129 MB L2, so no separate L2 flush is used.

--impl reference times the reference's CPU sparse-conv path (the oracle's restatement: kernel
map + gather -> torch.mm -> scatter, SparseConvolutionKernelMap.cu:417-509) on the host cores
with all threads, on a bounded sample of the same workload, and prints the same JSON line.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fvdb-core_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "SparseConv3d useful TFLOP/s & voxels/s, BF16/FP8 vs FP32 on 1 GB300; serve p99 ms"
WORKLOAD = "4 sphere-shell grids @256^3 (2M pts each), L1 3^3 s1 32->64 + L2 2^3 s2 64->64, bf16"


# ------------------------------------------------------------------ synthetic input -----
def sphere_shell_points(n_points: int, seed: int, device) -> torch.Tensor:
    g = torch.Generator(device="cpu").manual_seed(seed)
    centres = 0.3 + 0.4 * torch.rand(3, 3, generator=g)
    radii = 0.2 + 0.25 * torch.rand(3, generator=g)
    prob = radii**2 / (radii**2).sum()
    which = torch.multinomial(prob, n_points, replacement=True, generator=g)
    d = torch.randn(n_points, 3, generator=g)
    d = d / d.norm(dim=1, keepdim=True).clamp_min(1e-12)
    p = centres[which] + radii[which, None] * d
    p = p.clamp(0.0, 1.0 - 1e-6)
    return p.to(device)


def make_c2_inputs(device, rank: int = 0, n_points: int = 2_000_000):
    """ijk (jagged, int32, unsorted as voxelised) for the 4 grids."""
    ijk_parts = []
    for b in range(4):
        p = sphere_shell_points(n_points, 100 + b + 1000 * rank, device)
        ijk = torch.floor(p * 256 + 0.5).to(torch.int32)
        ijk_parts.append(torch.unique(ijk, dim=0))
    return ijk_parts


# ------------------------------------------------------------------ clocks sampler ------
class ClockSampler:
    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


# ------------------------------------------------------------------ model ---------------
class TwoLayer:
    def __init__(self, fvdb, device, dtype=torch.bfloat16, seed=0):
        g = torch.Generator().manual_seed(seed)
        self.fvdb = fvdb
        self.w1 = (torch.randn(64, 32, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * 32))).to(device, dtype)
        self.w2 = (torch.randn(64, 64, 2, 2, 2, generator=g) * math.sqrt(2.0 / (8 * 64))).to(device, dtype)

    def forward(self, grid, x, timers=None):
        # The coarse grid depends only on the fine grid.  Its build reads two counts back to the
        # host (one synchronisation); done first, everything after it (maps and contractions)
        # is queued while the GPU works, instead of the GPU idling behind a mid-step sync.
        p2, g2 = grid.sparse_conv_kernel_map(2, 2)
        p1, _ = grid.sparse_conv_kernel_map(3, 1)
        if timers:
            timers[0].record()
        h = p1.sparse_conv_3d(x, self.w1).jdata
        if timers:
            timers[1].record()
        y = p2.sparse_conv_3d(h, self.w2).jdata
        return y, p1, p2, g2


def useful_flops(p1, p2, cin1=32, cout1=64, cin2=64, cout2=64) -> tuple[float, int, int]:
    P1 = int((p1.out_in_map >= 0).sum())
    P2 = int((p2.out_in_map >= 0).sum())
    return 2.0 * (P1 * cin1 * cout1 + P2 * cin2 * cout2), P1, P2


# DRAM bytes (read + write) of one layer-1 contraction launch per voxel, from an ncu capture of
# one launch on the same workload generator at 1M points per grid (988,678 voxels): DRAM
# throughput 781.7 GB/s over the 335.26 us launch = 262.1 MB; traffic grows with the voxel count.
L1_DRAM_BYTES_PER_VOXEL = 781.685597e9 * 335.264e-6 / 988_678


def kernel_only_l1(lib, p1, x: torch.Tensor, w1: torch.Tensor, launches: int) -> dict:
    """Layer-1 tcgen05 contraction alone through the C ABI: over the index order (fvgb_conv_fwd_tc --
    the kernel the step runs) and, for comparison, over the map's row order (rows sorted by
    occupancy mask, fvgb_conv_fwd_tc_rows) and over a tile plan (fvgb_conv_fwd_tc_planned); plus
    the cost of building the row order and the plan.  Average launch durations from CUDA events
    around `launches` back-to-back launches on the current stream, and whether each output is
    bitwise identical to the same layer run through SparseConvPackInfo.sparse_conv_3d."""
    import ctypes

    n = x.shape[0]
    kmap = p1._impl.kmap()  # [rows padded to 128, K] int32, -1 = absent
    tm = p1._impl.tile_mask(False)
    K = kmap.shape[1]
    cout, cin = w1.shape[0], w1.shape[1]
    plan = p1._impl.tile_plan(False, cin * 2)
    wkio = w1.permute(4, 3, 2, 1, 0).reshape(K, cin, cout).contiguous()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nb = ctypes.c_size_t(0)
    assert lib.fvgb_tc_weight_bytes(2, ctypes.c_int64(K), cin, cout, ctypes.byref(nb)) == 0
    packed = torch.empty(nb.value, dtype=torch.uint8, device=x.device)
    assert lib.fvgb_tc_pack_weights(2, P(wkio), ctypes.c_int64(K), cin, cout, ctypes.c_int64(cin * cout),
                                    ctypes.c_int64(cout), ctypes.c_int64(1), P(packed), nb, stream) == 0
    err = torch.zeros(1, dtype=torch.int32, device=x.device)
    tiles = (n + 127) // 128
    rows = torch.empty(tiles * 128, dtype=torch.int32, device=x.device)
    rmask = torch.zeros(tiles, dtype=torch.int32, device=x.device)
    smap = torch.empty(tiles * 128, K, dtype=torch.int32, device=x.device)
    wsb = ctypes.c_size_t(0)
    assert lib.fvgb_kmap_row_order_workspace(ctypes.c_int64(n), K, ctypes.byref(wsb)) == 0
    ws = torch.empty(wsb.value, dtype=torch.uint8, device=x.device)
    ref = p1.sparse_conv_3d(x, w1).jdata

    def build_order(_y):
        rc = lib.fvgb_kmap_row_order(P(kmap), ctypes.c_int64(n), K, ctypes.c_int64(K), P(rows), P(rmask), P(smap),
                                     P(ws), ctypes.c_size_t(ws.numel()), stream)
        assert rc == 0, rc

    def ordered(y):
        rc = lib.fvgb_conv_fwd_tc_rows(2, P(x), ctypes.c_int64(n), cin, ctypes.c_int64(x.stride(0)), P(smap),
                                       ctypes.c_int64(n), K, P(rows), P(rmask), P(packed), cout, P(y),
                                       ctypes.c_int64(cout), None, None, 0, P(err), stream)
        assert rc == 0, rc

    def planned(y):
        rc = lib.fvgb_conv_fwd_tc_planned(2, P(x), ctypes.c_int64(n), cin, ctypes.c_int64(x.stride(0)), P(plan),
                                          ctypes.c_int64(n), K, P(packed), cout, P(y), ctypes.c_int64(cout), None,
                                          None, 0, P(err), stream)
        assert rc == 0, rc

    def unplanned(y):
        rc = lib.fvgb_conv_fwd_tc(2, P(x), ctypes.c_int64(n), cin, ctypes.c_int64(x.stride(0)), P(kmap),
                                  ctypes.c_int64(n), K, P(tm) if tm is not None else None, P(packed), cout, P(y),
                                  ctypes.c_int64(cout), None, P(err), stream)
        assert rc == 0, rc

    def build_plan(_y):
        rc = lib.fvgb_tc_plan_build(P(kmap), ctypes.c_int64(n), K, cin * 2, P(plan), ctypes.c_size_t(plan.numel()),
                                    stream)
        assert rc == 0, rc

    build_order(None)
    out = {}
    for name, fn in (("ordered", ordered), ("planned", planned), ("unplanned", unplanned), ("plan_build", build_plan),
                     ("order_build", build_order)):
        y = torch.empty(n, cout, device=x.device, dtype=torch.bfloat16)
        fn(y)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(launches):
            fn(y)
        b.record()
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        out[name] = {"ms": a.elapsed_time(b) / launches, "identical_to_step": bool(torch.equal(ref, y))}
    del out["plan_build"]["identical_to_step"], out["order_build"]["identical_to_step"]
    return out


def load_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "src": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


# ------------------------------------------------------------------ CPU baseline --------
def cpu_layer1_sample(ijk_np: np.ndarray, max_voxels: int, seed: int = 0) -> dict:
    """Reference CPU path on layer 1 of one grid (bounded sample): kernel map + GS conv."""
    from oracle import oracle as orc

    ijk = ijk_np[:max_voxels]
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    src, off = orc.grid_from_ijk(ijk, np.array([0, ijk.shape[0]]))
    kmap = orc.kernel_map(src, off, src, off, 3, 1)
    nbmap, nbsizes = orc.neighbour_map(kmap)
    x = torch.from_numpy(rng.standard_normal((src.shape[0], 32)).astype(np.float32))
    w = torch.from_numpy((rng.standard_normal((64, 32, 3, 3, 3)) * math.sqrt(2.0 / (27 * 32))).astype(np.float32))
    orc.gs_forward(x, w, nbmap, nbsizes, src.shape[0], middle=True)
    dt = time.perf_counter() - t0
    P = int(nbsizes.sum())
    return {"seconds": dt, "flops": 2.0 * P * 32 * 64, "voxels": int(src.shape[0]), "pairs": P}


def cpu_layer1_timed(ijk_np: np.ndarray, budget_s: float = 10.0) -> dict:
    """The reference CPU path on layer 1 of one whole grid, repeated until `budget_s` seconds of
    CPU work have been timed (after one untimed call); per-call mean."""
    cpu_layer1_sample(ijk_np, ijk_np.shape[0])
    calls, total, r = 0, 0.0, None
    while total < budget_s or calls == 0:
        r = cpu_layer1_sample(ijk_np, ijk_np.shape[0])
        total += r["seconds"]
        calls += 1
    return {"seconds": total / calls, "flops": r["flops"], "voxels": r["voxels"], "pairs": r["pairs"], "calls": calls,
            "total_s": total}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.set_num_threads(os.cpu_count() or 1)
    parts = make_c2_inputs("cpu")
    ijk0 = parts[0].numpy()
    sample = ijk0.shape[0]  # layer 1 of grid 0, whole
    for _ in range(args.warmup):
        cpu_layer1_sample(ijk0, sample)
    times, flops, vox = [], 0.0, 0
    for _ in range(args.steps):
        r = cpu_layer1_sample(ijk0, sample)
        times.append(r["seconds"])
        flops, vox = r["flops"], r["voxels"]
    t = sum(times) / len(times)
    value = flops / t / 1e12
    cores = torch.get_num_threads()
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "TFLOP/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": f"layer 1 of grid 0 ({sample} voxels) per step"},
        "voxels_per_s": vox / t,
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                          "sample": f"layer 1 (3^3 32->64) of grid 0 ({vox} voxels) per step: kernel map + gather/torch.mm/scatter, fp32"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ replicas ------------
def max_over_ranks(value: float, dist=None, device="cpu") -> float:
    """Max of a per-rank timing over all ranks (replicas: the job takes as long as the slowest)."""
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ GPU arm -------------
def run_gpu(args) -> None:
    import fvdb
    from fvdb import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    lib = _lib.cdll()
    import ctypes

    lib.fvgb_launch_count.restype = ctypes.c_uint64
    ijk_parts = make_c2_inputs(dev, rank, args.points)
    off = torch.tensor([0] + [p.shape[0] for p in ijk_parts], dtype=torch.int64).cumsum(0)
    ijk = torch.cat(ijk_parts, 0)
    grid = fvdb.GridBatch.from_ijk(fvdb.JaggedTensor.from_data_and_offsets(ijk, off.to(dev)))
    g = torch.Generator(device="cpu").manual_seed(7 + rank)
    x = torch.randn(grid.total_voxels, 32, generator=g).to(dev, torch.bfloat16)
    model = TwoLayer(fvdb, dev)

    # warm-up
    for _ in range(max(args.warmup, 1)):
        y, p1, p2, g2 = model.forward(grid, x)
    torch.cuda.synchronize()
    flops, P1, P2 = useful_flops(p1, p2)
    n_vox = grid.total_voxels

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.fvgb_launch_count()
    start.record()
    for i in range(args.steps):
        model.forward(grid, x, timers=ev[i])
    end.record()
    torch.cuda.synchronize()
    l1 = lib.fvgb_launch_count()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    conv_ms = statistics.median(a.elapsed_time(b) for a, b in ev)
    ms = max_over_ranks(ms, dist, dev)

    # end to end through the public API from pinned host buffers
    e2e_ms, h2d, d2h = float('nan'), 0, 0
    if not args.no_e2e:
        ijk_host = ijk.cpu().pin_memory()
        off_host = off.clone()
        x_host = x.cpu().pin_memory()
        e2e_steps = max(2, min(args.steps, 5))
        h2d = ijk_host.numel() * 4 + x_host.numel() * 2 + off_host.numel() * 8
        out_host = None  # pinned result buffer, allocated once like a serving loop would

        copy_stream = torch.cuda.Stream(device=dev)

        def e2e_step():
            nonlocal out_host
            ijk_d = ijk_host.to(dev, non_blocking=True)
            # the features travel on a copy stream while the grid is built from the coordinates
            copy_stream.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(copy_stream):
                x_d = x_host.to(dev, non_blocking=True)
            x_ready = torch.cuda.Event()
            x_ready.record(copy_stream)
            grid_e = fvdb.GridBatch.from_ijk(fvdb.JaggedTensor.from_data_and_offsets(ijk_d, off_host.to(dev, non_blocking=True)))
            # the voxel order of the built grid is the grid's own: features are given per input row,
            # so they are reordered through ijk_to_index as a user would
            idx = grid_e.ijk_to_index(fvdb.JaggedTensor.from_data_and_offsets(ijk_d, off_host.to(dev)), cumulative=True).jdata
            torch.cuda.current_stream().wait_event(x_ready)
            x_d.record_stream(torch.cuda.current_stream())
            x_sorted = torch.empty_like(x_d)
            x_sorted[idx] = x_d
            y_e, *_ = model.forward(grid_e, x_sorted)
            if out_host is None or out_host.shape != y_e.shape:
                out_host = torch.empty(y_e.shape, dtype=y_e.dtype).pin_memory()
            out_host.copy_(y_e, non_blocking=True)
            return out_host.numel() * out_host.element_size()

        # warm-up: first calls of the end-to-end-only operations (large index_put, ijk_to_index)
        for _ in range(max(args.warmup, 1)):
            e2e_step()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        d2h = 0
        for _ in range(e2e_steps):
            d2h = e2e_step()
        t1.record()
        torch.cuda.synchronize()  # the last result has reached host memory
        e2e_ms = t0.elapsed_time(t1) / e2e_steps

    kern = kernel_only_l1(lib, p1, x, model.w1, max(args.steps, 3))
    # the step builds its kernel maps every step, so it runs the index-order kernel (a row order or
    # a tile plan is built only for a map that is used again); the others are timed beside it
    kern_ms, kern_identical = kern["unplanned"]["ms"], kern["unplanned"]["identical_to_step"]
    peaks = load_peaks()
    conv1_flops = 2.0 * P1 * 32 * 64
    conv1_bytes = n_vox * 32 * 2 + n_vox * 64 * 2 + 27 * 32 * 64 * 2 + 4 * 27 * n_vox
    tf = flops * world / (ms * 1e-3) / 1e12
    line = {
        "metric": METRIC,
        "value": tf,
        "unit": "TFLOP/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "voxels": n_vox, "voxels_l2": g2.total_voxels, "pairs_l1": P1, "pairs_l2": P2,
                   "l2_policy": "inputs larger than L2 (per-step working set > 129 MB)", "parallelism": f"replicas{world}"},
        "voxels_per_s": n_vox * world / (ms * 1e-3),
        "e2e": {"value": flops / (e2e_ms * 1e-3) / 1e12 if e2e_ms == e2e_ms else None, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "gpu_launches": int(l1 - l0),
        "clocks": clk,
        "roofline": {
            "kernel": "conv_tc_fwd_kernel, layer-1 contraction (3^3 32->64)",
            "bound": "hbm",
            "achieved": conv1_bytes / (kern_ms * 1e-3) / 1e9,
            "peak": peaks["hbm_gbs"],
            "unit": "GB/s",
            "frac": conv1_bytes / (kern_ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
            "traffic": L1_DRAM_BYTES_PER_VOXEL * n_vox,
            "algorithmic_bytes": conv1_bytes,
            "peak_source": peaks["src"],
            "kernel_ms": kern_ms,
            "kernel_output_identical_to_step": kern_identical,
            "kernel_tflops": conv1_flops / (kern_ms * 1e-3) / 1e12,
            "tensor_frac": conv1_flops / (kern_ms * 1e-3) / 1e12 / peaks["bf16_tflops"],
            "layer1_window_ms": conv_ms,
            "row_order_build_ms": kern["order_build"]["ms"],
            "row_order_kernel_ms": kern["ordered"]["ms"],
            "row_order_output_identical_to_step": kern["ordered"]["identical_to_step"],
            "planned_kernel_ms": kern["planned"]["ms"],
            "planned_output_identical_to_step": kern["planned"]["identical_to_step"],
            "plan_build_ms": kern["plan_build"]["ms"],
        },
    }
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_layer1_timed(ijk_parts[0].cpu().numpy(), 10.0)
        line["cpu_baseline"] = {"value": r["flops"] / r["seconds"] / 1e12, "unit": "TFLOP/s", "cores": torch.get_num_threads(),
                                "kind": "port",
                                "sample": f"layer 1 (3^3 32->64) of grid 0 ({r['voxels']} voxels), fp32, kernel map + "
                                          f"gather/torch.mm/scatter, {r['calls']} calls in {r['total_s']:.1f} s"}
    legs = set() if args.no_extras else set(args.legs.split(","))
    if "fp32" in legs:
        line["fp32_plain"] = leg_fp32(fvdb, grid, x, model, flops, args)
        line["bf16_vs_fp32"] = tf / line["fp32_plain"]["value"] if line["fp32_plain"]["value"] else None
    if "c1" in legs:
        line["c1_fp32"] = leg_c1(fvdb, dev, args)
    if "halo" in legs:
        line["halo_l1"] = leg_halo(fvdb, grid, x, model, args)
    if "train" in legs:
        line["train_c3"] = leg_train(fvdb, dev, args)
    if "fp8" in legs:
        line["fp8_c4"] = leg_fp8(fvdb, dev, args)
    if "serve" in legs:
        line["serving_c5"] = leg_serve(fvdb, dev, args)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------------------------ extra legs ----------
def time_ms(fn, steps: int, warmup: int) -> float:
    for _ in range(max(warmup, 1)):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def rel_errors(got: torch.Tensor, ref: torch.Tensor) -> dict:
    d = (got.double() - ref.double())
    return {"rel_l2": float(d.norm() / ref.double().norm().clamp_min(1e-300)),
            "max_abs": float(d.abs().max()), "max_rel_to_scale": float(d.abs().max() / ref.double().abs().max().clamp_min(1e-300))}


def leg_fp32(fvdb, grid, x, model, flops, args) -> dict:
    """The same two-layer step in the plain FP32 form (CUDA-core FFMA, no TF32): the x1 of BF16."""
    w1, w2 = model.w1.float(), model.w2.float()
    xf = x.float()

    def step():
        p1, _ = grid.sparse_conv_kernel_map(3, 1)
        h = p1.sparse_conv_3d(xf, w1).jdata
        p2, _ = grid.sparse_conv_kernel_map(2, 2)
        p2.sparse_conv_3d(h, w2)

    ms = time_ms(step, max(2, args.steps // 2), 1)
    # errors of the BF16 step (the headline) and of this FP32 form against the same step in FP64
    y16, *_ = model.forward(grid, x)
    p1, _ = grid.sparse_conv_kernel_map(3, 1)
    p2, _ = grid.sparse_conv_kernel_map(2, 2)
    y64 = p2.sparse_conv_3d(p1.sparse_conv_3d(x.double(), model.w1.double()).jdata, model.w2.double()).jdata
    y32 = p2.sparse_conv_3d(p1.sparse_conv_3d(xf, w1).jdata, w2).jdata
    # the layer-1 FP32 contraction alone (map prebuilt) against the measured FFMA rate
    P1 = int((p1.out_in_map >= 0).sum())
    l1_ms = time_ms(lambda: p1.sparse_conv_3d(xf, w1), max(3, args.steps // 2), 2)
    l1_tflops = 2.0 * P1 * 32 * 64 / (l1_ms * 1e-3) / 1e12
    peak = ffma_peak_tflops()
    return {"value": flops / (ms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": ms, "dtype": "f32",
            "layer1_contraction_ms": l1_ms, "layer1_contraction_tflops": l1_tflops,
            "ffma_peak_tflops": peak, "layer1_frac_of_ffma_peak": l1_tflops / peak if peak else None,
            "errors_vs_fp64": {"bf16_step": rel_errors(y16, y64), "fp32_step": rel_errors(y32, y64)}}


def ffma_peak_tflops() -> float:
    """FP32 FMA rate of this GPU: the library's probe kernel (8 independent fma chains per
    thread, 8 CTAs of 256 threads per SM) timed with CUDA events, best of 3."""
    import ctypes

    from fvdb import _lib

    lib = _lib.cdll()
    out = torch.zeros(2, device="cuda")
    flops = ctypes.c_double(0.0)
    stream = torch.cuda.current_stream().cuda_stream
    best = 0.0
    for _ in range(4):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        rc = lib.fvgb_ffma_probe(ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(1 << 16), 8, ctypes.byref(flops),
                                 ctypes.c_void_p(stream))
        b.record()
        torch.cuda.synchronize()
        if rc != 0:
            return 0.0
        best = max(best, flops.value / (a.elapsed_time(b) * 1e-3) / 1e12)
    return best


def leg_c1(fvdb, dev, args) -> dict:
    """C1, the reference's CPU-sized case: 20,000 voxels drawn from 64^3 (seed 0), 16 -> 16
    channels, 3^3, FP32, no bias.  Forward time (kernel map included) and errors vs FP64."""
    g = torch.Generator().manual_seed(0)
    idx = torch.randperm(64 ** 3, generator=g)[:20000]
    ijk = torch.stack([idx // 4096, idx // 64 % 64, idx % 64], 1).to(dev, torch.int32)
    grid = fvdb.GridBatch.from_ijk(ijk)
    x = torch.randn(grid.total_voxels, 16, generator=g)
    w = torch.randn(16, 16, 3, 3, 3, generator=g) * math.sqrt(1.0 / (27 * 16))
    xf, wf = x.to(dev), w.to(dev)

    def step():
        p, _ = grid.sparse_conv_kernel_map(3, 1)
        return p.sparse_conv_3d(xf, wf).jdata

    ms = time_ms(step, max(3, args.steps), 2)
    y32 = step()
    p, _ = grid.sparse_conv_kernel_map(3, 1)
    y64 = p.sparse_conv_3d(x.double().to(dev), w.double().to(dev)).jdata
    P = int((p.out_in_map >= 0).sum())
    return {"voxels": grid.total_voxels, "pairs": P, "ms_per_step": ms, "us_per_step": ms * 1e3,
            "voxels_per_s": grid.total_voxels / (ms * 1e-3), "useful_tflops": 2.0 * P * 16 * 16 / (ms * 1e-3) / 1e12,
            "dtype": "f32", "errors_vs_fp64": rel_errors(y32, y64)}


def leg_halo(fvdb, grid, x, model, args) -> dict:
    """Layer 1 of the headline step (3^3, stride 1, 32 -> 64) through GridBatch.sparse_conv_halo
    (leaf-halo kernels, no kernel map) beside the kernel-map path (map build included), BF16 and
    FP32, forward and forward + backward; errors of each against FP64.  On the headline's
    sphere-shell grids and on a dense 96^3 block (every leaf full)."""
    dev = x.device
    r = torch.arange(96, dtype=torch.int32, device=dev)
    dense = fvdb.GridBatch.from_ijk(torch.stack(torch.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3))
    xd_dense = torch.randn(dense.total_voxels, 32, generator=torch.Generator().manual_seed(3)).to(dev, torch.bfloat16)
    out = {}
    for gname, gg, xx in (("shells", grid, x), ("dense96", dense, xd_dense)):
        w64 = model.w1.double()
        p1, _ = gg.sparse_conv_kernel_map(3, 1)
        y64 = p1.sparse_conv_3d(xx.double(), w64).jdata
        res = {"voxels": gg.total_voxels}
        for name, dt in (("bf16", torch.bfloat16), ("fp32", torch.float32)):
            xd, wd = xx.to(dt), model.w1.to(dt)
            jx = gg.jagged_like(xd)

            def halo_fwd():
                return gg.sparse_conv_halo(jx, wd).jdata

            def map_fwd():
                p, _ = gg.sparse_conv_kernel_map(3, 1)
                return p.sparse_conv_3d(xd, wd).jdata

            xg, wg = xd.clone().requires_grad_(True), wd.clone().requires_grad_(True)
            jg = gg.jagged_like(xg)
            dy = torch.ones(gg.total_voxels, wd.shape[0], device=dev, dtype=dt)

            def halo_train():
                gg.sparse_conv_halo(jg, wg).jdata.backward(dy)

            def map_train():
                p, _ = gg.sparse_conv_kernel_map(3, 1)
                p.sparse_conv_3d(xg, wg).jdata.backward(dy)

            steps = max(3, args.steps // 2)
            rr = {"halo_fwd_ms": time_ms(halo_fwd, steps, 2), "map_fwd_ms": time_ms(map_fwd, steps, 2),
                  "halo_fwd_bwd_ms": time_ms(halo_train, steps, 1), "map_fwd_bwd_ms": time_ms(map_train, steps, 1)}
            rr["halo_errors_vs_fp64"] = rel_errors(halo_fwd(), y64)
            rr["map_errors_vs_fp64"] = rel_errors(map_fwd(), y64)
            res[name] = rr
        out[gname] = res
    return out


def probe_row_gather(args) -> None:
    """Random 128-byte row gathers into the tensor-core A-operand layout (fvgb_row_gather_probe): a
    feature table of --probe-gather-rows rows x 128 bytes (default 2M = 256 MB, larger than L2),
    2^20 random row indices, one CTA per SM gathering 512 stages of 128 rows; best of 3 launches
    per method, timed with CUDA events.  Prints one JSON line."""
    import ctypes

    from fvdb import _lib

    lib = _lib.cdll()
    n = args.probe_gather_rows
    x = torch.randn(n, 64, device="cuda").bfloat16()
    rows = torch.randint(0, n, (1 << 20,), generator=torch.Generator().manual_seed(0), dtype=torch.int32).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nbytes = ctypes.c_int64(0)
    out = {}
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for mode, name in ((3, "cp_async_8_warps"), (1, "gather4_lane0_of_8_warps"), (2, "gather4_32_lanes_of_1_warp"),
                       (0, "gather4_1_thread"), (4, "half_gather4_half_cp_async")):
        best = None
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            rc = lib.fvgb_row_gather_probe(mode, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n),
                                           ctypes.c_void_p(rows.data_ptr()), rows.numel(), 512,
                                           ctypes.c_void_p(err.data_ptr()), ctypes.byref(nbytes), stream)
            b.record()
            torch.cuda.synchronize()
            assert rc == 0 and int(err.item()) == 0, (rc, int(err.item()))
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = {"ms": best, "GB_per_s": nbytes.value / (best * 1e-3) / 1e9,
                     "ns_per_16KB_stage_per_SM": best * 1e6 / (512.0)}
    print(json.dumps({"probe": "random 128-byte row gather into a 128B-swizzled shared-memory stage",
                      "table_rows": n, "table_mb": n * 128 / 1e6, "sms": sms, "stages_per_sm": 512, "results": out}))


def box_surface_ijk(n_boxes: int, resolution: int, seed: int, device) -> torch.Tensor:
    """Faces of n random axis-aligned boxes (sides U[0.1,0.5], min corner U[0,1-side]) at resolution^3."""
    g = torch.Generator().manual_seed(seed)
    out = []
    for _ in range(n_boxes):
        side = 0.1 + 0.4 * torch.rand(3, generator=g)
        lo = torch.rand(3, generator=g) * (1 - side)
        a = torch.floor(lo * resolution).long()
        b = torch.floor((lo + side) * resolution).long()
        for axis in range(3):
            u, v = [t for t in range(3) if t != axis]
            gu, gv = torch.meshgrid(torch.arange(a[u], b[u] + 1), torch.arange(a[v], b[v] + 1), indexing="ij")
            for face in (a[axis], b[axis]):
                pts = torch.empty(gu.numel(), 3, dtype=torch.long)
                pts[:, axis] = face
                pts[:, u] = gu.reshape(-1)
                pts[:, v] = gv.reshape(-1)
                out.append(pts)
    return torch.unique(torch.cat(out), dim=0).to(device, torch.int32)


def leg_train(fvdb, dev, args) -> dict:
    """conv3^3(64->64) -> ReLU -> conv3^3(64->64) on ~1M box-surface voxels at 512^3: forward +
    dgrad + wgrad, BF16 vs the plain FP32 form; errors vs the FP64 form on the same inputs."""
    grid = fvdb.GridBatch.from_ijk(box_surface_ijk(8, 512, 200, dev))
    g = torch.Generator().manual_seed(201)
    w1 = torch.randn(64, 64, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * 64))
    w2 = torch.randn(64, 64, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * 64))
    x0 = torch.randn(grid.total_voxels, 64, generator=g)
    dy = torch.randn(grid.total_voxels, 64, generator=g)
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    pack.build_implicit_gemm(training=True)
    P = int((pack.out_in_map >= 0).sum())
    flops = 2 * 3 * 2.0 * P * 64 * 64  # two layers x (fwd, dgrad, wgrad)

    def run(dtype):
        x = x0.to(dev, dtype).requires_grad_(True)
        a, b = w1.to(dev, dtype).requires_grad_(True), w2.to(dev, dtype).requires_grad_(True)
        d = dy.to(dev, dtype)

        def step():
            # conv -> ReLU (fused into the first convolution's epilogue) -> conv
            h = pack._conv_with_bias(x, a, None, False, None, relu=True).jdata
            y = pack.sparse_conv_3d(h, b).jdata
            x.grad = a.grad = b.grad = None
            y.backward(d)
            return y

        return step, x, a, b

    res = {"voxels": grid.total_voxels, "pairs": P, "useful_flops_per_step": flops}
    outs = {}
    for name, dtype in (("bf16", torch.bfloat16), ("fp32", torch.float32), ("fp64", torch.float64)):
        step, x, a, b = run(dtype)
        if name != "fp64":
            ms = time_ms(step, 3, 1)
            res[name] = {"ms_per_step": ms, "tflops": flops / (ms * 1e-3) / 1e12}
        y = step()
        outs[name] = (y.detach(), x.grad.detach(), a.grad.detach())
    res["bf16_vs_fp32"] = res["fp32"]["ms_per_step"] / res["bf16"]["ms_per_step"]
    for name in ("bf16", "fp32"):
        res[name]["errors_vs_fp64"] = {k: rel_errors(o, r) for k, o, r in zip(("y", "dx", "dw1"), outs[name], outs["fp64"])}
    # BF16 kernels against FP64 arithmetic on the same BF16-rounded operands and activations (same
    # ReLU masks): separates what the kernels add from BF16 storage (whose rounding of layer-1
    # outputs flips ReLU masks near zero and dominates the end-to-end gradient error above).
    bf = lambda t: t.bfloat16().double()
    xq = x0.to(dev).bfloat16().double().requires_grad_(True)
    w1q = w1.to(dev).bfloat16().double().requires_grad_(True)
    w2q = w2.to(dev).bfloat16().double()
    pre = pack.sparse_conv_3d(xq, w1q).jdata
    y1 = bf(pre.detach())
    h = torch.relu(y1).requires_grad_(True)
    y2 = pack.sparse_conv_3d(h, w2q).jdata
    dh = bf(torch.autograd.grad(y2, h, bf(dy.to(dev)))[0]) * (y1 > 0)
    dxq, dw1q = torch.autograd.grad(pre, (xq, w1q), dh)
    res["bf16"]["errors_vs_fp64_same_rounding"] = {
        "y": rel_errors(outs["bf16"][0], bf(y2.detach())), "dx": rel_errors(outs["bf16"][1], bf(dxq)),
        "dw1": rel_errors(outs["bf16"][2], bf(dw1q))}
    # FP64 arithmetic on BF16-rounded x, W1, W2 and dy with no other rounding, against FP64 on the
    # unrounded inputs: the input rounding alone moves pre-activations near zero across the ReLU
    # (round-to-nearest never changes the sign of a rounded output), so this shows how much of the
    # stack's gradient error the inputs' rounding accounts for.
    xr = x0.to(dev).bfloat16().double().requires_grad_(True)
    w1r = w1.to(dev).bfloat16().double().requires_grad_(True)
    yr = pack.sparse_conv_3d(torch.relu(pack.sparse_conv_3d(xr, w1r).jdata), w2.to(dev).bfloat16().double()).jdata
    dxr, dw1r = torch.autograd.grad(yr, (xr, w1r), dy.to(dev).bfloat16().double())
    res["fp64_on_bf16_rounded_inputs_vs_fp64"] = {
        "y": rel_errors(yr.detach(), outs["fp64"][0]), "dx": rel_errors(dxr, outs["fp64"][1]),
        "dw1": rel_errors(dw1r, outs["fp64"][2])}
    # One SparseConv3d (3^3, 64->64) forward + backward, BF16 vs FP64 on the unrounded inputs:
    # without a ReLU between layers no mask can flip, so this is the layer's own BF16 error.
    one = {}
    for name, dtype in (("bf16", torch.bfloat16), ("fp64", torch.float64)):
        xs = x0.to(dev, dtype).requires_grad_(True)
        ws = w1.to(dev, dtype).requires_grad_(True)
        ys = pack.sparse_conv_3d(xs, ws).jdata
        ys.backward(dy.to(dev, dtype))
        one[name] = (ys.detach(), xs.grad.detach(), ws.grad.detach())
    res["bf16"]["single_layer_errors_vs_fp64"] = {
        k: rel_errors(o, r) for k, o, r in zip(("y", "dx", "dw"), one["bf16"], one["fp64"])}
    return res


def shell_ijk(target: int, seed: int, device, res_cap: int = 4000) -> torch.Tensor:
    """One random sphere shell voxelised at a resolution chosen to give ~target voxels."""
    g = torch.Generator().manual_seed(seed)
    r = 0.2 + 0.25 * float(torch.rand(1, generator=g))
    c = 0.3 + 0.4 * torch.rand(3, generator=g)
    R = int(min(res_cap, max(16, math.sqrt(target / (1.55 * 4 * math.pi * r * r)))))
    d = torch.randn(int(target * 2.5), 3, generator=g).to(device)
    p = c.to(device) + r * d / d.norm(dim=1, keepdim=True)
    ijk = torch.floor(p.clamp(0, 1 - 1e-6) * R + 0.5).to(torch.int32)
    return torch.unique(ijk, dim=0)


def leg_fp8(fvdb, dev, args) -> dict:
    """~4M sphere-shell voxels at 1024^3 (shells added until the union reaches 4M): FP8-E4M3 3^3
    conv C128->256 (per-channel scales), then
    2^3 stride-2 transposed conv C256->128 from conv_grid(2,2) back onto the fine grid.  Timing
    FP8 and BF16; errors vs FP64 on 4096 sampled output rows."""
    # sphere shells (seeds 300, 301, ...) are added until their union holds ~4M voxels
    ijk = torch.zeros((0, 3), dtype=torch.int32, device=dev)
    target = args.c4_voxels
    for i in range(16):
        ijk = torch.unique(torch.cat([ijk, shell_ijk(min(1_000_000, target), 300 + i, dev, 1024)]), dim=0)
        if ijk.shape[0] >= target:
            break
    grid = fvdb.GridBatch.from_ijk(ijk)
    g = torch.Generator().manual_seed(301)
    x = torch.randn(grid.total_voxels, 128, generator=g).to(dev, torch.bfloat16)
    w1 = (torch.randn(256, 128, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * 128))).to(dev, torch.bfloat16)
    pack1, _ = grid.sparse_conv_kernel_map(3, 1)
    coarse = grid.conv_grid(2, 2)
    pack2, _ = grid.sparse_conv_kernel_map(2, 2, coarse)
    xc = torch.randn(coarse.total_voxels, 256, generator=g).to(dev, torch.bfloat16)
    w2 = (torch.randn(256, 128, 2, 2, 2, generator=g) * math.sqrt(2.0 / (8 * 256))).to(dev, torch.bfloat16)
    pack1.build_implicit_gemm()
    pack2.build_implicit_gemm(training=True)  # forward map + the transposed map the transposed conv reads
    P1 = int((pack1.out_in_map >= 0).sum())
    P2 = int((pack2.out_in_map >= 0).sum())
    f1, f2 = 2.0 * P1 * 128 * 256, 2.0 * P2 * 256 * 128
    res = {"voxels": grid.total_voxels, "coarse_voxels": coarse.total_voxels, "pairs_l1": P1, "pairs_l2": P2}
    with torch.no_grad():
        for prec in ("fp8", "bf16"):
            ms1 = time_ms(lambda: pack1.sparse_conv_3d(x, w1, precision=prec), 3, 1)
            ms2 = time_ms(lambda: pack2.sparse_transpose_conv_3d(xc, w2, precision=prec), 3, 1)
            res[prec] = {"l1_ms": ms1, "l1_tflops": f1 / (ms1 * 1e-3) / 1e12, "l2_ms": ms2, "l2_tflops": f2 / (ms2 * 1e-3) / 1e12}
        y1 = pack1.sparse_conv_3d(x, w1, precision="fp8").jdata
        y2 = pack2.sparse_transpose_conv_3d(xc, w2, precision="fp8").jdata
    # FP64 reference rows through the kernel maps
    sel = torch.randperm(grid.total_voxels, generator=g)[:4096].to(dev)
    m1 = pack1.out_in_map[sel].long()
    W1 = w1.double().permute(4, 3, 2, 1, 0).reshape(27, 128, 256)
    xd = torch.cat([x.double(), torch.zeros(1, 128, dtype=torch.float64, device=dev)])
    ref1 = torch.einsum("rkc,kco->ro", xd[torch.where(m1 >= 0, m1, grid.total_voxels)], W1)
    mt = pack2.out_in_map_bwd[sel].long()
    W2 = w2.double().permute(4, 3, 2, 0, 1).reshape(8, 256, 128)
    xcd = torch.cat([xc.double(), torch.zeros(1, 256, dtype=torch.float64, device=dev)])
    ref2 = torch.einsum("rkc,kco->ro", xcd[torch.where(mt >= 0, mt, coarse.total_voxels)], W2)
    res["errors_vs_fp64"] = {"l1": rel_errors(y1[sel], ref1), "l2_transposed": rel_errors(y2[sel], ref2)}
    return res


def leg_serve(fvdb, dev, args) -> dict:
    """Poisson arrivals swept over the requested rates, N log-uniform [1e4, 2e6] voxels per
    request (one sphere shell each), 4-layer 3^3 stack 32->64->64->32 with ReLU, BF16,
    continuous batching under an HBM budget; against the plain FP32 per-request form on the
    same arrival schedule.  The requests of every rate are drawn from one pool of distinct
    grids (sizes log-uniform) so their host buffers fit in pinned memory; features arrive as
    BF16 in both forms (the FP32 form computes in FP32).  Errors against the stack in FP64 are
    stated for a sample of served requests."""
    from fvdb.serving import ContinuousBatcher, ConvStack, GPUExecutor, Request, latency_stats, run_alone

    rates = [float(r) for r in args.serve_rates.split(",") if r]
    rng = np.random.default_rng(400)
    pool = []
    for i in range(args.serve_pool):
        n = int(math.exp(rng.uniform(math.log(1e4), math.log(2e6))))
        ijk = shell_ijk(n, 400 + i, dev).cpu().pin_memory()
        feats = torch.randn(ijk.shape[0], 32, generator=torch.Generator().manual_seed(i)).bfloat16().pin_memory()
        pool.append((ijk, feats))
    model = ConvStack([32, 64, 64, 32], dev, seed=0)
    model32 = model.to_dtype(torch.float32)
    out = {"requests_per_rate": args.serve_requests, "distinct_grids": len(pool),
           "pool_voxels_mean": float(np.mean([p[0].shape[0] for p in pool])), "rates": {}}
    forms = (("bf16_batched", model, 3, None), ("fp32_per_request", model32, 1, 1))
    servers = {}
    for name, mdl, slots, per_batch in forms:
        ex = GPUExecutor(mdl, dev, slots=slots)
        srv_args = dict(hbm_budget=48 << 30, max_batch_voxels=4_000_000, slots=slots, max_batch_requests=per_batch)
        servers[name] = (ex, srv_args)
        # warm-up: the smallest and the largest request of the pool alone, then every pool grid
        # once at a high rate (first-call costs and the allocator's growth to batch sizes stay out
        # of the measured latencies)
        for j in (min(range(len(pool)), key=lambda i: pool[i][0].shape[0]),
                  max(range(len(pool)), key=lambda i: pool[i][0].shape[0])):
            ContinuousBatcher(ex, **srv_args).serve([Request(rid=-1, ijk=pool[j][0], features=pool[j][1], arrival=0.0)])
        ContinuousBatcher(ex, **srv_args).serve([Request(rid=-2 - j, ijk=pool[j][0], features=pool[j][1],
                                                         arrival=0.001 * j) for j in range(len(pool))])
    sample_done = {}
    for ri, rate in enumerate(rates):
        r2 = np.random.default_rng(1000 + ri)
        picks = r2.integers(0, len(pool), size=args.serve_requests)
        arrivals = np.cumsum(r2.exponential(1.0 / rate, size=args.serve_requests))
        entry = {}
        for name, mdl, slots, per_batch in forms:
            ex, srv_args = servers[name]
            srv = ContinuousBatcher(ex, **srv_args)
            batch = [Request(rid=i, ijk=pool[int(k)][0], features=pool[int(k)][1], arrival=float(t))
                     for i, (k, t) in enumerate(zip(picks, arrivals))]
            done = srv.serve(batch)
            st = latency_stats(done)
            st["batches"] = srv.batches
            st["errors"] = sum(1 for r in done if r.error)
            entry[name] = st
            if name == "bf16_batched" and ri == len(rates) - 1:
                sample_done = {int(picks[r.rid]): r for r in done if r.error is None}
        out["rates"][str(int(rate) if rate == int(rate) else rate)] = entry
    # errors of served BF16 outputs (from the mix at the highest rate) against FP64 alone
    model64 = model.to_dtype(torch.float64)
    errs = []
    for k in sorted(sample_done)[: args.serve_error_sample]:
        r = sample_done[k]
        y64, ijk64 = run_alone(model64, r, dev)
        assert torch.equal(ijk64, r.out_ijk)
        errs.append(rel_errors(r.output, y64))
    if errs:
        out["errors_vs_fp64"] = {"requests": len(errs), "rel_l2_max": max(e["rel_l2"] for e in errs),
                                 "max_rel_to_scale_max": max(e["max_rel_to_scale"] for e in errs)}
    for ex, _ in servers.values():
        ex.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP32 / training / FP8 / serving legs")
    ap.add_argument("--legs", default="fp32,c1,halo,train,fp8,serve",
                    help="comma-separated extra legs to run after the headline step")
    ap.add_argument("--serve-rates", default="50,100,200,500,1000,2000",
                    help="Poisson request rates of the serving sweep (1/s)")
    ap.add_argument("--serve-requests", type=int, default=300, help="requests per rate in the serving leg")
    ap.add_argument("--serve-pool", type=int, default=40, help="distinct request grids the serving leg draws from")
    ap.add_argument("--serve-error-sample", type=int, default=4, help="served requests checked against FP64")
    ap.add_argument("--c4-voxels", type=int, default=4_000_000,
                    help="voxels of the FP8 leg's grid (4M is the stated size; smaller only for profiling captures)")
    ap.add_argument("--points", type=int, default=2_000_000,
                    help="points per grid (the headline workload uses 2M; smaller only for profiling captures)")
    ap.add_argument("--probe-gather", action="store_true",
                    help="only run the row-gather probe (cp.async vs TMA gather4) and print its JSON line")
    ap.add_argument("--probe-gather-rows", type=int, default=2 * 1024 * 1024,
                    help="rows of 128 bytes in the probe's table (2M = 256 MB, beyond L2; 256k = 32 MB fits L2)")
    args = ap.parse_args()
    if args.probe_gather:
        probe_row_gather(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
