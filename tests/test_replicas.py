"""Replica bookkeeping: shard arithmetic, and the barrier/max/sum reductions
over two gloo ranks on the CPU (the multi-GPU job's host side; it has no
data-path collective to test)."""
import os
import socket

import pytest

from voxelpathtracer_gb300 import replicas


def test_shard_rows_cover_exactly():
    for H in (0, 1, 7, 1080, 2160):
        for world in (1, 2, 3, 4, 8):
            bands = [replicas.shard_rows(H, r, world) for r in range(world)]
            assert bands[0][0] == 0 and bands[-1][1] == H
            for (a0, a1), (b0, b1) in zip(bands, bands[1:]):
                assert a1 == b0
            sizes = [b - a for a, b in bands]
            assert max(sizes) - min(sizes) <= 1


def test_shard_rows_rejects_bad_rank():
    with pytest.raises(ValueError):
        replicas.shard_rows(10, 2, 2)
    with pytest.raises(ValueError):
        replicas.shard_rows(10, 0, 0)


def test_shard_worlds_partition_and_balance():
    import random
    rng = random.Random(3)
    costs = [rng.randint(256 * 256, 1024 * 576) for _ in range(64)]
    for world in (1, 2, 4, 8):
        parts = replicas.shard_worlds(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT bound: max load <= 4/3 of the ideal (plus the largest item's slack)
        assert max(loads) <= (4 / 3) * max(sum(costs) / world, max(costs)) + 1
    assert replicas.shard_worlds([], 3) == [[], [], []]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    info = replicas.rank_info()
    rep = replicas.Replicas(info.world)
    rep.barrier()
    mx = rep.max(10.0 * (rank + 1))
    sm = rep.sum(rank + 1)
    r0, r1 = replicas.shard_rows(1080, info.rank, info.world)
    rows = rep.sum(r1 - r0)
    rep.barrier()
    rep.close()
    q.put((rank, mx, sm, rows))


def test_two_rank_gloo_reductions():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, rows in got:
        assert mx == 20.0 and sm == 3.0 and rows == 1080.0
