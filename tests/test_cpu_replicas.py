"""Two gloo ranks on CPU: the replica aggregation used by multi-GPU bench
runs sums the work and takes the slowest rank's time."""
import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from globillum_gb300 import replicas
    paths, ms = replicas.aggregate(1000.0 * (rank + 1), 10.0 + rank, dist)
    q.put((rank, paths, ms, replicas.mpaths_per_s(paths, ms)))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, paths, ms, v in res:
        assert paths == 3000.0 and ms == 11.0
        assert v == pytest.approx(3000.0 / 0.011 / 1e6)


def test_single_process():
    from globillum_gb300 import replicas
    assert replicas.aggregate(5.0, 2.0) == (5.0, 2.0)
