"""The benchmark's multi-rank path on CPU: world_size 2 over gloo.

The path shards by pool (independent replicas, no collective on the data
path); the only collectives are the timing reductions.  The job's time is
the slowest rank's and its work the sum of the ranks' work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r ran 1000*(r+1) ops in (r+1) ms: the job took 2 ms for 3000 ops
    ms, value = bench.combine_ranks(float(rank + 1), 1000 * (rank + 1), world, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ms, value))


def test_combine_ranks_gloo_world2():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 2.0
        assert value == pytest.approx(3000 / 2e-3)


def test_combine_ranks_single():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.combine_ranks(4.0, 8000, 1) == (4.0, 8000 / 4e-3)
