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


def _pool_worker(rank, world, port, q):
    """One rank = one GPU's pool, stood in for on the CPU by the oracle's
    bitmap and walk: rank r owns pages [r*T, (r+1)*T) of the job, prefilled
    with its own seed, and serves its own requests."""
    import numpy as np
    import torch
    import torch.distributed as dist

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    T, n = 1 << 14, 2048
    words = oracle.bernoulli_bitmap(T, 0.5 + 0.2 * rank, 100 + rank)
    before = words.copy()
    ids, steps = oracle.replay_alloc(words, T, 2, n, 7 + rank, collab_width=32)
    # the job's view: every rank's pages in its own range, gathered over gloo
    local = torch.from_numpy(np.where(ids >= 0, ids.astype(np.int64) + rank * T, -1))
    parts = [torch.empty_like(local) for _ in range(world)]
    dist.all_gather(parts, local)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ids, before, words, [p.numpy() for p in parts]))


def test_one_pool_per_rank_gloo_world2():
    """Each rank's pool evolves only by its own requests: its results equal a
    run of the same pool alone, no rank's pages fall in another rank's range,
    and the gathered ids of the job are unique."""
    import numpy as np

    mp = pytest.importorskip("torch.multiprocessing")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.lib()   # build the oracle before the ranks load it
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world, T, n = 2, 1 << 14, 2048
    procs = [ctx.Process(target=_pool_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=120) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    gathered = out[0][4]
    for rank, ids, before, after, parts in out:
        # alone: the same pool, prefill and requests in this process
        w = oracle.bernoulli_bitmap(T, 0.5 + 0.2 * rank, 100 + rank)
        assert np.array_equal(w, before)
        ids_alone, _ = oracle.replay_alloc(w, T, 2, n, 7 + rank, collab_width=32)
        assert np.array_equal(ids, ids_alone) and np.array_equal(after, w)
        assert all(np.array_equal(a, b) for a, b in zip(parts, gathered))   # every rank gathered the same
        g = gathered[rank]
        ok = g >= 0
        assert ((g[ok] >= rank * T) & (g[ok] < (rank + 1) * T)).all()
    allg = np.concatenate(gathered)
    allg = allg[allg >= 0]
    assert np.unique(allg).size == allg.size
