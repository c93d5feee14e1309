"""Ensemble sharding across ranks: the partition covers every system once, balances the cost
model, is identical on every rank, and gathering works over a real 2-rank gloo group (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from particlesimulation_gb300 import sharding


def test_shard_covers_and_balances():
    costs = [sharding.system_cost(n, g ** 3) for n, g in
             [(4096, 32), (131072, 128), (20000, 64), (60000, 64), (9000, 32), (100000, 128), (5000, 32)]]
    for world in (1, 2, 3, 8):
        parts = sharding.shard(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        if world <= len(costs):
            assert max(loads) <= sum(costs) / world + max(costs)
    assert sharding.shard(costs, 4) == sharding.shard(list(costs), 4)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = sharding.shard(costs, world)
    # every rank computes the same partition without communicating
    check = [None] * world
    dist.all_gather_object(check, parts)
    assert all(c == parts for c in check)
    local = {i: ("rank", rank, i * i) for i in parts[rank]}
    merged = sharding.gather(local, world)
    out[rank] = sorted(merged.items())
    dist.barrier()
    dist.destroy_process_group()


def test_gather_over_two_gloo_ranks():
    costs = [float(c) for c in (5, 1, 8, 3, 3, 9, 2)]
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        ctx = mp.get_context("spawn")
        procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        a, b = out[0], out[1]
    assert a == b
    assert [k for k, _ in a] == list(range(len(costs)))
    owners = {k: v[1] for k, v in a}
    parts = sharding.shard(costs, 2)
    for r in range(2):
        assert all(owners[i] == r for i in parts[r])
