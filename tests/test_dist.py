"""Multi-process paths on CPU (gloo, world size 2): instance sharding of the
batched solver and the max/sum reductions the benchmark uses."""
import os
import socket

import pytest

from ptdiff import dist as PD


def test_shard_instances_partition():
    for n in (0, 1, 7, 256):
        for world in (1, 2, 3, 8):
            got = [PD.shard_instances(n, r, world) for r in range(world)]
            flat = [i for g in got for i in g]
            assert flat == list(range(n))
            assert max(map(len, got)) - min(map(len, got)) <= 1
    with pytest.raises(ValueError):
        PD.shard_instances(4, 2, 2)


def test_shard_by_cells_balances():
    sizes = [1024 ** 2, 128 ** 2, 512 ** 2, 700 ** 2, 300 ** 2, 1000 ** 2]
    parts = PD.shard_by_cells(sizes, 2)
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.4


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = PD.shard_instances(10, rank, world)
        t = 1.0 + rank          # this rank's time
        q.put((rank, mine, PD.reduce_max(t), PD.reduce_sum(len(mine))))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] + res[1][1] == list(range(10))
    assert res[0][2] == res[1][2] == 2.0
    assert res[0][3] == res[1][3] == 10.0
