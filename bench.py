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
        p1, _ = grid.sparse_conv_kernel_map(3, 1)
        if timers:
            timers[0].record()
        h = p1.sparse_conv_3d(x, self.w1).jdata
        if timers:
            timers[1].record()
        p2, g2 = grid.sparse_conv_kernel_map(2, 2)
        y = p2.sparse_conv_3d(h, self.w2).jdata
        return y, p1, p2, g2


def useful_flops(p1, p2, cin1=32, cout1=64, cin2=64, cout2=64) -> tuple[float, int, int]:
    P1 = int((p1.out_in_map >= 0).sum())
    P2 = int((p2.out_in_map >= 0).sum())
    return 2.0 * (P1 * cin1 * cout1 + P2 * cin2 * cout2), P1, P2


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


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.set_num_threads(os.cpu_count() or 1)
    parts = make_c2_inputs("cpu")
    ijk0 = parts[0].numpy()
    sample = 120_000
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
        "config": {"workload": WORKLOAD, "sample": f"layer 1 of grid 0, first {sample} voxels"},
        "voxels_per_s": vox / t,
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                          "sample": f"layer 1 (3^3 32->64) of grid 0 restricted to {vox} voxels: kernel map + gather/torch.mm/scatter, fp32"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


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
    t_all = torch.tensor([ms], device=dev)
    if dist:
        dist.all_reduce(t_all, op=dist.ReduceOp.MAX)
    ms = float(t_all.item())

    # end to end through the public API from pinned host buffers
    e2e_ms, h2d, d2h = float('nan'), 0, 0
    if not args.no_e2e:
        ijk_host = ijk.cpu().pin_memory()
        off_host = off.clone()
        x_host = x.cpu().pin_memory()
        e2e_steps = max(2, min(args.steps, 5))
        h2d = ijk_host.numel() * 4 + x_host.numel() * 2 + off_host.numel() * 8
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        d2h = 0
        for _ in range(e2e_steps):
            ijk_d = ijk_host.to(dev, non_blocking=True)
            x_d = x_host.to(dev, non_blocking=True)
            grid_e = fvdb.GridBatch.from_ijk(fvdb.JaggedTensor.from_data_and_offsets(ijk_d, off_host.to(dev, non_blocking=True)))
            # the voxel order of the built grid is the grid's own: features are given per input row,
            # so they are reordered through ijk_to_index as a user would
            idx = grid_e.ijk_to_index(fvdb.JaggedTensor.from_data_and_offsets(ijk_d, off_host.to(dev)), cumulative=True).jdata
            x_sorted = torch.empty_like(x_d)
            x_sorted[idx] = x_d
            y_e, *_ = model.forward(grid_e, x_sorted)
            out_host = y_e.to("cpu")
            d2h = out_host.numel() * out_host.element_size()
        t1.record()
        torch.cuda.synchronize()
        e2e_ms = t0.elapsed_time(t1) / e2e_steps

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
            "kernel": "layer-1 contraction (3^3 32->64)",
            "bound": "hbm",
            "achieved": conv1_bytes / (conv_ms * 1e-3) / 1e9,
            "peak": peaks["hbm_gbs"],
            "unit": "GB/s",
            "frac": conv1_bytes / (conv_ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
            "traffic": None,
            "peak_source": peaks["src"],
            "kernel_ms": conv_ms,
            "kernel_tflops": conv1_flops / (conv_ms * 1e-3) / 1e12,
        },
    }
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_layer1_sample(ijk_parts[0].cpu().numpy(), 120_000)
        line["cpu_baseline"] = {"value": r["flops"] / r["seconds"] / 1e12, "unit": "TFLOP/s", "cores": torch.get_num_threads(),
                                "kind": "port",
                                "sample": f"layer 1 (3^3 32->64) of grid 0 restricted to {r['voxels']} voxels, fp32, kernel map + gather/torch.mm/scatter ({r['seconds']:.2f} s)"}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--points", type=int, default=2_000_000,
                    help="points per grid (the headline workload uses 2M; smaller only for profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
