"""bench.py's N>1 path is replicas only (no data-path collective): each rank runs its own
synthetic grids and the job time is the max over ranks.  Checked with world_size 2 on CPU
(gloo), without a GPU."""

import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # per-rank replica inputs differ (seeded by rank) and need no exchange
    g = bench.sphere_shell_points(1000, 100 + 1000 * rank, "cpu")
    local_ms = 10.0 + 5.0 * rank
    dist.barrier()
    got = bench.max_over_ranks(local_ms, dist, "cpu")
    out[rank] = (got, float(g.sum()))
    dist.destroy_process_group()


def test_max_over_ranks_world_size_2():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0][0] == out[1][0] == 15.0
        assert out[0][1] != out[1][1]


def test_single_process_identity():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
