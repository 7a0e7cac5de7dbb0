"""Batch sharding across ranks (no data-path collective): each rank takes a
contiguous slice of the batch; gathering the slices reproduces the
single-process result.  Runs as two gloo ranks on CPU with the oracle
standing in for the per-rank transform."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from genfft_gb300.shard import shard_range


def test_shard_range_covers_batch():
    for batch in (1, 2, 7, 16384, 32):
        for world in (1, 2, 3, 4, 8):
            spans = [shard_range(batch, r, world) for r in range(world)]
            assert sum(c for _, c in spans) == batch
            pos = 0
            for s, c in spans:
                assert s == pos and c >= 0
                pos += c
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, batch = 256, 7
    rng = np.random.default_rng(0)  # same global batch on every rank
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    s, c = shard_range(batch, rank, world)
    mine = O.Impl("oracle").fft(x[s:s + c]) if c else np.zeros((0, n), np.complex64)
    parts = [None] * world
    dist.all_gather_object(parts, (s, mine))
    if rank == 0:
        full = np.concatenate([p for _, p in sorted(parts, key=lambda t: t[0])])
        q.put(bool(np.array_equal(full.view(np.uint8), O.Impl("oracle").fft(x).view(np.uint8))))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_two_rank_gloo_shards(world):
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert q.get(timeout=10) is True


def _timing_worker(rank, world, port, q):
    import sys
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    bench.barrier(world)
    # each rank's elapsed time differs; the reported time is the slowest
    got = bench.max_over_ranks(world, 1.0 + rank * 0.25)
    q.put((rank, got))
    dist.destroy_process_group()


def test_bench_time_is_max_over_ranks():
    """bench.py reports the slowest rank's time (its barrier and max-reduce
    run over gloo here, over NCCL under torchrun on GPUs)."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30500 + os.getpid() % 1000
    procs = [ctx.Process(target=_timing_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    assert res == [(0, 1.25), (1, 1.25)]
