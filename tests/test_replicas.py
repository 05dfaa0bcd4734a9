"""Replicas-only N>1 path on the CPU: two gloo ranks, each with its own
seed, combine their timing into the whole-job figure (slowest rank's time,
histories summed) -- the aggregation bench.py applies over NCCL on GPUs."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from branson_gb300.replicas import combine, replica_seed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = [0.25, 0.75][rank]
        hist = [1000.0, 3000.0][rank]
        t, h = combine(elapsed, hist, device="cpu")
        out.put((rank, t, h, replica_seed(777, rank)))
    finally:
        dist.destroy_process_group()


def test_replica_seeds_are_distinct():
    from branson_gb300.replicas import replica_seed
    seeds = {replica_seed(777, r) for r in range(64)}
    assert len(seeds) == 64 and replica_seed(777, 0) == 777


def test_two_gloo_ranks_combine_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, h, seed in res:
        assert t == 0.75 and h == 4000.0
    assert res[0][3] != res[1][3]


def test_single_process_combine_is_identity():
    from branson_gb300.replicas import combine
    assert combine(1.5, 42.0) == (1.5, 42.0)
