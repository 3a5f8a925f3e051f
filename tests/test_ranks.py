"""Multi-process rank logic of bench.py on CPU (gloo, world_size 2): problem
sharding of an ensemble covers every problem exactly once, and the whole-job
figure is the units summed over ranks divided by the slowest rank's time."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist = bench.dist_init(world, backend="gloo")
    mine = bench.shard(10, rank, world)
    dist.barrier()
    # rank r pretends to take (r + 1) seconds for its own problems
    t_max, total, value = bench.aggregate(dist, float(rank + 1), float(len(mine)))
    out.put((rank, mine, t_max, total, value))
    dist.destroy_process_group()


def test_shard_covers_each_problem_once():
    import bench
    for n in (0, 1, 7, 512):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in bench.shard(n, r, world))
            assert got == list(range(n))
            sizes = [len(bench.shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def test_aggregate_single_process():
    import bench
    assert bench.aggregate(None, 2.0, 10.0) == (2.0, 10.0, 5.0)


@pytest.mark.timeout(120)
def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    (r0, m0, t0, n0, v0), (r1, m1, t1, n1, v1) = res
    assert sorted(m0 + m1) == list(range(10))
    assert t0 == t1 == 2.0          # slowest rank
    assert n0 == n1 == 10.0         # all problems
    assert v0 == v1 == 5.0
