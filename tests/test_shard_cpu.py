"""Sharding of independent cloths across ranks, on CPU with two gloo ranks.

Each rank takes its share of a seeded batch (licenta_gb300.shard), steps it
with the FP32 oracle, and the shares are gathered: together they must cover
every cloth exactly once, stay balanced, and give bit for bit the states of
one process stepping the whole batch, because the step has no exchange
between cloths.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from licenta_gb300 import scenes, shard

STEPS = 3


def _specs():
    return scenes.batched_cloths(seed=21, count=10, n_min=6, n_max=20)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle.oracle_ffi import Oracle
        specs = _specs()
        mine = shard.my_share(specs, rank, world)
        o = Oracle([specs[i] for i in mine], fp64=False)
        o.step(STEPS, threads=1)
        states = {i: o.get_state(k)["x"] for k, i in enumerate(mine)}
        o.close()
        gathered = [None] * world
        dist.all_gather_object(gathered, states)
        if rank == 0:
            q.put(gathered)
    finally:
        dist.destroy_process_group()


def test_balance_is_deterministic_and_even():
    costs = [shard.cloth_cost(s) for s in scenes.batched_cloths(seed=0, count=256)]
    a, b = shard.balance(costs, 4), shard.balance(costs, 4)
    assert a == b
    loads = [sum(costs[i] for i in s) for s in a]
    assert sorted(i for s in a for i in s) == list(range(256))
    assert max(loads) / min(loads) < 1.02


def test_two_gloo_ranks_match_one_process():
    from oracle.oracle_ffi import Oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    merged = {}
    for part in gathered:
        assert not (set(part) & set(merged)), "a cloth was stepped by two ranks"
        merged.update(part)
    specs = _specs()
    assert sorted(merged) == list(range(len(specs)))
    o = Oracle(specs, fp64=False)
    o.step(STEPS, threads=1)
    for i in range(len(specs)):
        assert np.array_equal(merged[i], o.get_state(i)["x"]), f"cloth {i}"
    o.close()
