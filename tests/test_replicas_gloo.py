"""bench.py's multi-rank path (independent replicas, weak scaling) on CPU with the gloo backend,
world size 2: barrier semantics and the max-over-ranks job time."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    total_ms = 100.0 * (rank + 1)           # rank 1 is the slower replica
    out = bench.combine_ranks(total_ms, rays_per_step=1_000_000, steps=10, world=world, dist=dist)
    dist.barrier()
    q.put((rank, out))
    dist.destroy_process_group()


def test_two_replicas_take_max_time_and_sum_rays():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        ms, value = res[r]
        assert ms == pytest.approx(200.0)                 # slowest rank
        assert value == pytest.approx(2 * 10 * 1e6 / 0.2 / 1e6)  # all ranks' rays / max time


def test_single_rank_needs_no_process_group():
    import bench
    ms, v = bench.combine_ranks(50.0, 2_000_000, 5, 1)
    assert ms == 50.0 and v == pytest.approx(2e6 * 5 / 0.05 / 1e6)
