"""Multi-GPU is replicas only (no exchange step in the forward model): the
bench's job time is the slowest rank's.  Checked with two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        t = bench.replica_time(10.0 + 5.0 * rank, dist, 'cpu')
        q.put((rank, t))
    finally:
        dist.destroy_process_group()


def test_replica_time_is_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 15.0, 1: 15.0}


def test_replica_time_single():
    import bench
    assert bench.replica_time(3.5) == 3.5
