"""Queue-based size classes (the per-class block queues backend).

* A one-warp replay equals the oracle's sequential replay: every block
  offset, the bitmap, and the queue contents after freeing everything.
* Parallel batches (persistent, plain, graph) give blocks that are aligned
  to their class, disjoint, inside the pool and on pages that were free;
  freed blocks are served again before new chunks are carved; after all
  frees every carved block is queued (pages held = queued bytes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
PAGE = 4096


def _sizes(n, seed):
    rng = np.random.default_rng(seed)
    return np.clip(np.exp(rng.uniform(np.log(16), np.log(65536), n)), 16, 65536).astype(np.uint32)


def _cls_bytes(sz):
    return np.maximum(16, 1 << np.ceil(np.log2(np.maximum(sz, 1))).astype(np.int64))


def _tab(groups):
    t = np.zeros(len(groups), dtype=DT)
    for i, (op, cnt, off) in enumerate(groups):
        t[i] = (op, cnt, off)
    return t


def _queued_pages(queued):
    return sum(n * (1 << (4 + c)) for c, n in enumerate(queued)) // PAGE


def test_serial_qmalloc_matches_oracle(cuda, pbm_mod, orc):
    torch = cuda
    pbm = pbm_mod
    T, occ, seed, S = 1 << 14, 0.05, 7, 23
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.prefill(occ, seed)
    pool.qmalloc_init(1 << 12)
    words = orc.bernoulli_bitmap(T, occ, seed)
    n = 320
    sizes = _sizes(n, 4)
    d_sizes = torch.from_numpy(sizes.astype(np.int32)).cuda()
    ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
    pool.qmalloc_batch(torch.from_numpy(_tab([(pbm.OP_MALLOC, n, 0)]).view(np.uint8).copy()).cuda(), None, 1,
                       d_sizes, ptrs, n, S, pbm.LAUNCH_SERIAL)
    got = ptrs.cpu().numpy()
    offs = np.where(got != 0, got - pool.base_ptr, -1)
    rep = orc.QMallocReplay(words, T, 12, cap=1 << 12)
    exp = np.zeros(n, dtype=np.int64)
    for q0 in range(0, n, 32):
        k = min(32, n - q0)
        own = np.array([orc.seed(S, q0 + l) for l in range(k)], dtype=np.int32)
        o, _ = rep.group(sizes[q0:q0 + k], own)
        exp[q0:q0 + k] = o
    assert np.array_equal(offs, exp)
    assert np.array_equal(pool.read_bitmap(), words)
    # free everything (serial): the queues hold exactly the oracle's blocks
    pool.qmalloc_batch(torch.from_numpy(_tab([(pbm.OP_MFREE, n, 0)]).view(np.uint8).copy()).cuda(), None, 1,
                       d_sizes, ptrs, n, S + 1, pbm.LAUNCH_SERIAL)
    for q0 in range(0, n, 32):
        rep.free(exp[q0:q0 + 32])
    queued, chunks, overflow, timeouts, bad = pool.qmalloc_counts()
    assert queued == rep.queued() and chunks == rep.q.chunks and overflow == 0 and timeouts == 0 and bad == 0
    assert (ptrs.cpu().numpy() == 0).all()
    rep.close()
    pool.close()


def _check_blocks(ptrs, sizes, base, T, before_words):
    ok = ptrs != 0
    off = ptrs[ok] - base
    cb = _cls_bytes(sizes[ok].astype(np.int64))
    assert (off % np.minimum(cb, PAGE) == 0).all()
    assert (off >= 0).all() and ((off + cb) <= T * PAGE).all()
    order = np.argsort(off)
    s, e = off[order], (off + cb)[order]
    assert (s[1:] >= e[:-1]).all()
    held = np.unpackbits(before_words.view(np.uint8), bitorder="little")[:T]
    pages = np.unique(np.concatenate([np.arange(a // PAGE, (b - 1) // PAGE + 1) for a, b in zip(s, e)]))
    assert held[pages].sum() == 0
    return ok.sum()


@pytest.mark.parametrize("mode", ["persistent", "plain", "graph"])
def test_parallel_qmalloc_rounds(cuda, pbm_mod, orc, mode):
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 18, 0.05, 8
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.prefill(occ, seed)
    pool.qmalloc_init(1 << 16)
    before = orc.bernoulli_bitmap(T, occ, seed)
    used0 = orc.used_pages(before, T)
    rng = np.random.default_rng(4)
    counts = np.clip(np.exp(rng.uniform(0, np.log(3001), 16)).astype(np.int64), 1, 3000)
    N = int(counts.sum())
    sizes = _sizes(N, 5)
    d_sizes = torch.from_numpy(sizes.astype(np.int32)).cuda()
    ptrs = torch.zeros(N, dtype=torch.int64, device="cuda")
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]])
    malloc_tab = _tab([(pbm.OP_MALLOC, int(c), int(o)) for c, o in zip(counts, offs)])
    free_tab = _tab([(pbm.OP_MFREE, int(c), int(o)) for c, o in zip(counts, offs)])

    def run(tab, sd):
        d = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
        if mode == "graph":
            g = pool.qmalloc_graph(d, len(tab), 1, d_sizes, ptrs, N, sd)
            g.replay()
            g.close()
        elif mode == "plain":
            hg = pbm.groups_array([(int(r["op"]), int(r["count"]), int(r["offset"])) for r in tab])
            pool.qmalloc_batch(d, hg, len(tab), d_sizes, ptrs, N, sd, pbm.LAUNCH_PLAIN)
        else:
            pool.qmalloc_batch(d, None, len(tab), d_sizes, ptrs, N, sd, pbm.LAUNCH_PERSISTENT)
        torch.cuda.synchronize()

    run(malloc_tab, 31)
    p = ptrs.cpu().numpy()
    assert _check_blocks(p, sizes, pool.base_ptr, T, before) == N
    _, chunks1, _, _, _ = pool.qmalloc_counts()
    used1 = pool.used()
    run(free_tab, 32)
    queued, _, overflow, timeouts, bad = pool.qmalloc_counts()
    assert overflow == 0 and timeouts == 0 and bad == 0
    assert _queued_pages(queued) == used1 - used0           # every carved block is queued again
    # the same requests again come from the queues: no new chunk, no new page
    run(malloc_tab, 33)
    p = ptrs.cpu().numpy()
    assert _check_blocks(p, sizes, pool.base_ptr, T, before) == N
    _, chunks2, _, _, _ = pool.qmalloc_counts()
    assert chunks2 == chunks1 and pool.used() == used1
    run(free_tab, 34)
    assert (ptrs.cpu().numpy() == 0).all()
    pool.close()
