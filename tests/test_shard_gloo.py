"""Multi-GPU batched runs split the instances across ranks (heatsim2_gb300.batch.shard) with no collective
on the data path.  Checked here with two gloo ranks on the CPU: every instance belongs to exactly one rank,
the loads are balanced, and the aggregation bench.py does at the end (sum of voxels, max of times) agrees."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from heatsim2_gb300 import workloads as W
from heatsim2_gb300.batch import shard


def _sizes():
    return [W.voxels(s) for s in W.uneven_batch(seed=2, n=64, nz_range=(2, 8), nxy_range=(4, 16))]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = _sizes()
    mine = shard(sizes, world, rank)
    owner = torch.zeros(len(sizes), dtype=torch.int64)
    owner[mine] = 1
    dist.all_reduce(owner)
    load = torch.tensor([sum(sizes[i] for i in mine)], dtype=torch.int64)
    total = load.clone()
    dist.all_reduce(total)
    longest = load.clone()
    dist.all_reduce(longest, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((owner.tolist(), int(total), int(longest), sum(sizes), max(sizes)))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_instances_shard_across_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    owner, total, longest, expect_total, biggest = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert owner == [1] * len(owner)
    assert total == expect_total
    assert longest <= expect_total / 2 + biggest


@pytest.mark.parametrize("world", [1, 3, 8])
def test_shard_is_a_partition(world):
    sizes = _sizes()
    parts = [shard(sizes, world, r) for r in range(world)]
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)
