"""The N > 1 path of bench.py on the host: two gloo ranks on CPU (127.0.0.1).  Migrations are
independent units, sharded round-robin with no data-path exchange; the only collectives are
the timing reductions (max of the ranks' times, sum of their cell-updates)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = list(range(11))
        mine = bench.shard(units, rank, world)
        mx = bench.reduce_over_ranks(10.0 * (rank + 1), "max", world, "cpu")
        sm = bench.reduce_over_ranks(float(len(mine)), "sum", world, "cpu")
        out.put((rank, mine, mx, sm))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = [r[1] for r in res]
    assert sorted(shards[0] + shards[1]) == list(range(11))       # every unit exactly once
    assert not set(shards[0]) & set(shards[1])
    assert all(r[2] == 20.0 for r in res)                          # max over ranks
    assert all(r[3] == 11.0 for r in res)                          # sum over ranks


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert bench.reduce_over_ranks(3.5, "max", 1, "cpu") == 3.5
