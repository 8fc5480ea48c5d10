"""Size-classed malloc over the page pool (config 4 semantics).

* A one-warp replay equals the oracle's sequential replay: every block
  offset and the bitmap, bit for bit; freeing everything restores the prefill.
* Parallel batches (persistent, plain, graph) give blocks that are aligned to
  their size class, disjoint, inside the pool and on pages that were free;
  frees release every run exactly once."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
PAGE = 4096


def _sizes(n, seed):
    rng = np.random.default_rng(seed)
    return np.clip(np.exp(rng.uniform(np.log(16), np.log(65536), n)), 16, 65536).astype(np.uint32)


def _cls_bytes(sz):
    c = np.maximum(16, 1 << np.ceil(np.log2(np.maximum(sz, 1))).astype(np.int64))
    return c


def _tab(groups):
    t = np.zeros(len(groups), dtype=DT)
    for i, (op, cnt, off) in enumerate(groups):
        t[i] = (op, cnt, off)
    return t


def test_serial_malloc_matches_oracle(cuda, pbm_mod, orc):
    torch = cuda
    pbm = pbm_mod
    T, occ, seed, S = 1 << 14, 0.3, 7, 21
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.prefill(occ, seed)
    pool.malloc_init()
    words = orc.bernoulli_bitmap(T, occ, seed)
    before = words.copy()
    n = 300
    sizes = _sizes(n, 4)
    d_sizes = torch.from_numpy(sizes.astype(np.int32)).cuda()
    ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
    tab = _tab([(pbm.OP_MALLOC, n, 0)])
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    pool.malloc_batch(d_tab, None, 1, d_sizes, ptrs, n, S, pbm.LAUNCH_SERIAL)
    got = ptrs.cpu().numpy()
    offs = np.where(got != 0, got - pool.base_ptr, -1)
    rep = orc.MallocReplay(words, T, 12)
    exp = np.zeros(n, dtype=np.int64)
    for q0 in range(0, n, 32):
        k = min(32, n - q0)
        seed_small = orc.seed(S ^ 0x9E3779B9, q0)
        own = np.array([orc.seed(S, q0 + l) for l in range(k)], dtype=np.int32)
        o, _ = rep.group(sizes[q0:q0 + k], seed_small, own)
        exp[q0:q0 + k] = o
    assert np.array_equal(offs, exp)
    assert np.array_equal(pool.read_bitmap(), words)
    # free everything in one persistent batch: the prefill comes back exactly
    tab = _tab([(pbm.OP_MFREE, n, 0)])
    pool.malloc_batch(torch.from_numpy(tab.view(np.uint8).copy()).cuda(), None, 1, d_sizes, ptrs, n, S + 1,
                      pbm.LAUNCH_PERSISTENT)
    assert np.array_equal(pool.read_bitmap(), before)
    live, bad = pool.malloc_counts()
    assert live == 0 and bad == 0
    pool.close()


def _check_blocks(ptrs, sizes, base, T, before_words):
    ok = ptrs != 0
    off = ptrs[ok] - base
    cb = _cls_bytes(sizes[ok].astype(np.int64))
    assert (off % np.minimum(cb, PAGE) == 0).all()                # class-aligned below a page, else page-aligned
    assert (off >= 0).all() and ((off + cb) <= T * PAGE).all()    # inside the pool
    order = np.argsort(off)
    s, e = off[order], (off + cb)[order]
    assert (s[1:] >= e[:-1]).all()                                # disjoint
    held = np.unpackbits(before_words.view(np.uint8), bitorder="little")[:T]
    pages = np.unique(np.concatenate([np.arange(a // PAGE, (b - 1) // PAGE + 1) for a, b in zip(s, e)]))
    assert held[pages].sum() == 0                                 # only pages free before
    return ok.sum()


@pytest.mark.parametrize("mode", ["persistent", "plain", "graph"])
def test_parallel_malloc_free_rounds(cuda, pbm_mod, orc, mode):
    torch = cuda
    pbm = pbm_mod
    # 5% prefill: at 30% only ~2% of 32-page words still hold a free run of 16
    # pages, so most 64 KiB requests would find none (they fail, bounded)
    T, occ, seed = 1 << 18, 0.05, 8
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.prefill(occ, seed)
    pool.malloc_init()
    before = orc.bernoulli_bitmap(T, occ, seed)
    rng = np.random.default_rng(4)
    counts = np.clip(np.exp(rng.uniform(0, np.log(3001), 16)).astype(np.int64), 1, 3000)
    N = int(counts.sum())
    sizes = _sizes(N, 5)
    d_sizes = torch.from_numpy(sizes.astype(np.int32)).cuda()
    ptrs = torch.zeros(N, dtype=torch.int64, device="cuda")
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]])
    malloc_tab = _tab([(pbm.OP_MALLOC, int(c), int(o)) for c, o in zip(counts, offs)])
    # free every other group, then free the rest
    half_tab = _tab([(pbm.OP_MFREE if i % 2 == 0 else pbm.OP_MALLOC, int(c) if i % 2 == 0 else 0, int(o))
                     for i, (c, o) in enumerate(zip(counts, offs))])
    rest_tab = _tab([(pbm.OP_MFREE, int(c) if i % 2 else 0, int(o)) for i, (c, o) in enumerate(zip(counts, offs))])

    def run(tab, sd):
        d = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
        if mode == "graph":
            g = pool.malloc_graph(d, len(tab), 1, d_sizes, ptrs, N, sd)
            g.replay()
            g.close()
        elif mode == "plain":
            hg = pbm.groups_array([(int(r["op"]), int(r["count"]), int(r["offset"])) for r in tab])
            pool.malloc_batch(d, hg, len(tab), d_sizes, ptrs, N, sd, pbm.LAUNCH_PLAIN)
        else:
            pool.malloc_batch(d, None, len(tab), d_sizes, ptrs, N, sd, pbm.LAUNCH_PERSISTENT)
        torch.cuda.synchronize()

    run(malloc_tab, 31)
    p = ptrs.cpu().numpy()
    assert _check_blocks(p, sizes, pool.base_ptr, T, before) == N
    run(half_tab, 32)
    run(rest_tab, 34)
    assert np.array_equal(pool.read_bitmap(), before)
    live, bad = pool.malloc_counts()
    assert live == 0 and bad == 0
    assert (ptrs.cpu().numpy() == 0).all()
    pool.close()


@pytest.mark.parametrize("occ,seed", [(0.5, 8), (0.5, 9), (0.3, 3)])
def test_one_request_warp_walk_matches_oracle(cuda, pbm_mod, orc, occ, seed):
    """A batch of one 64 KiB request (a run of 16 pages): the request's lane
    takes its first jump and then the whole warp walks for it, 32 jumps per
    round.  With nothing else claiming, the run it gets is the one the
    oracle's one-lane span walk finds from the same seed, and the bitmap
    changes by exactly that run."""
    torch = cuda
    pbm = pbm_mod
    T, S = 1 << 16, 77
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.prefill(occ, seed)
    pool.malloc_init()
    before = pool.read_bitmap()
    exp_ids, _ = orc.replay_spans(before.copy(), T, np.array([16], dtype=np.int32), S, max_steps=4096)
    d_sizes = torch.tensor([65536], dtype=torch.int32, device="cuda")
    ptrs = torch.zeros(1, dtype=torch.int64, device="cuda")
    tab = _tab([(pbm.OP_MALLOC, 1, 0)])
    pool.malloc_batch(torch.from_numpy(tab.view(np.uint8).copy()).cuda(), None, 1, d_sizes, ptrs, 1, S,
                      pbm.LAUNCH_PERSISTENT, max_steps=4096)
    torch.cuda.synchronize()
    p = int(ptrs.cpu().numpy()[0])
    got = (p - pool.base_ptr) // PAGE if p else -1
    assert got == int(exp_ids[0])
    after = pool.read_bitmap()
    bits_b = np.unpackbits(before.view(np.uint8), bitorder="little")[:T]
    bits_a = np.unpackbits(after.view(np.uint8), bitorder="little")[:T]
    if got >= 0:
        assert (bits_a[got:got + 16] == 1).all() and (bits_b[got:got + 16] == 0).all()
        bits_a[got:got + 16] = 0
    assert np.array_equal(bits_a, bits_b)
    pool.close()
