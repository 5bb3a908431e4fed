"""Host logic of the multi-GPU replica mode, on the CPU: the footprint-balanced
partition of systems over ranks, and the reductions over two gloo ranks
(world_size 2, 127.0.0.1).  No GPU: ranks exchange only host-side values."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from spc2_langevin_integration_gb300 import replicas


def _sizes(count=512, seed=2):
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(rng.uniform(np.log(256), np.log(32768))))) for _ in range(count)]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_every_system_once_and_balances(world):
    sizes = _sizes()
    parts = replicas.partition_by_footprint(sizes, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - sum(sizes) / world <= max(sizes)
    for p in parts:
        assert p == sorted(p)
    assert replicas.partition_by_footprint(sizes, world) == parts  # deterministic


def test_partition_edge_cases():
    assert replicas.partition_by_footprint([], 2) == [[], []]
    assert replicas.partition_by_footprint([5], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        replicas.partition_by_footprint([1], 0)
    with pytest.raises(ValueError):
        replicas.shard([1, 2], 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = _sizes(64, seed=7)
        mine = replicas.shard(sizes, world, rank)
        work = float(sum(sizes[i] for i in mine))
        fake_time = 1.0 + rank  # the slower rank sets the job time
        tmax = replicas.max_over_ranks(fake_time, dist)
        total = replicas.sum_over_ranks(work, dist)
        q.put((rank, mine, tmax, total))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sizes = _sizes(64, seed=7)
    got.sort()
    assert sorted(i for _, mine, _, _ in got for i in mine) == list(range(len(sizes)))
    for _, _, tmax, total in got:
        assert tmax == 2.0
        assert total == float(sum(sizes))
