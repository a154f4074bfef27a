"""bench.py's multi-rank path on CPU: world_size 2 over gloo.  The solve does
not shard (replicas only), so the only cross-rank step is the timing
reduction: the job time is the slowest rank's."""
import os
import socket
import sys

import pytest

from conftest import REPO


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        results[rank] = bench.max_over_ranks(1.0 + 2.5 * rank, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_world2():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    mgr = mp.Manager()
    results = mgr.dict()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert dict(results) == {0: 3.5, 1: 3.5}


def test_max_over_ranks_single():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(2.0, None) == 2.0
