"""Multi-GPU runs of bench.py are replicas (the path does not shard: every
rank holds whole graphs and answers its own roots).  The only cross-rank
step is the result reduction: edges summed, time = the slowest rank's.
Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    try:
        edges, secs = bench.reduce_results(1000.0 * (rank + 1), 0.5 + rank)
        roots = bench.rank_roots(list(range(1, 10001)), 8, rank)
        q.put((rank, edges, secs, roots))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    for rank, edges, secs, _ in got:
        assert edges == 3000.0  # sum over ranks
        assert secs == 1.5      # the slowest rank's time
    r0, r1 = got[0][3], got[1][3]
    assert len(r0) == len(r1) == 8 and r0 != r1  # each replica answers its own roots


def test_single_process_reduce_is_identity():
    import bench
    assert bench.reduce_results(5.0, 2.0) == (5.0, 2.0)
