"""CPU oracle self-checks (no GPU)."""
import ctypes

import numpy as np
import pytest


def py_lcg(x):
    v = 1103515245 * x + 12345
    r = abs(v) % (1 << 31)
    r = r if v >= 0 else -r
    return ((r + (1 << 31)) % (1 << 32)) - (1 << 31)


def test_lcg_matches_c_semantics(orc):
    rng = np.random.default_rng(0)
    xs = [0, 1, -1, 2**31 - 1, -2**31, 12345, -12345] + list(rng.integers(-2**31, 2**31, 500))
    for x in xs:
        assert orc.lcg(int(x)) == py_lcg(int(x))


def test_nonnegative_seeds_stay_nonnegative(orc):
    for r in range(1000):
        x = orc.seed(5, r)
        assert 0 <= x < 2**31
        for _ in range(5):
            x = orc.lcg(x)
            assert 0 <= x < 2**31


def test_bernoulli_prefill_fraction_and_padding(orc):
    T = 100_003
    for occ in (0.0, 0.5, 0.9, 1.0):
        w = orc.bernoulli_bitmap(T, occ, 7)
        used = orc.used_pages(w, T)
        assert abs(used / T - occ) < 0.01
        bits = np.unpackbits(w.view(np.uint8), bitorder="little")
        assert bits[T:].all()          # padding held


@pytest.mark.parametrize("strategy", [0, 1, 2, 3, 5, 6])
def test_replay_invariants(orc, strategy):
    T = 1 << 14
    w = orc.bernoulli_bitmap(T, 0.6, 3)
    before = w.copy()
    kw = {}
    if strategy == 3:
        kw["cursors"] = np.full(16, -1, dtype=np.int64)
    if strategy == 5:
        kw["arm"] = [0]
    if strategy == 6:
        kw["arms"] = np.array([orc.lib().orc_dist_clock_arm0(0, i, T) for i in range(16)], dtype=np.int64)
    ids, steps = orc.replay_alloc(w, T, strategy, 3000, 4, **kw)
    c = orc.check_alloc(w, before, T, ids)
    assert c.n_ok == 3000 and c.n_duplicates == 0 and c.n_not_marked == 0 and c.n_prefilled == 0
    assert c.used_after == orc.used_pages(before, T) + 3000
    assert (steps >= 1).all() if strategy != 3 else (steps >= 0).all()


@pytest.mark.parametrize("wb,W", [(32, 32), (64, 32), (32, 8), (32, 16), (64, 16)])
def test_collab_replay_claims_exactly_what_is_needed(orc, wb, W):
    T = 1 << 14
    w = orc.bernoulli_bitmap(T, 0.8, 9)
    before = w.copy()
    ids, steps = orc.replay_alloc(w, T, 2, 1000, 6, word_bits=wb, collab_width=W)
    c = orc.check_alloc(w, before, T, ids)
    assert c.n_ok == 1000 and c.n_duplicates == 0 and c.n_prefilled == 0
    assert c.used_after == orc.used_pages(before, T) + 1000   # nothing over-claimed


def test_checker_catches_planted_duplicate(orc):
    """A planted mistake (on the CPU, in the oracle's input): a duplicated id
    and an unmarked id are reported."""
    T = 4096
    w = orc.bernoulli_bitmap(T, 0.5, 1)
    before = w.copy()
    ids, _ = orc.replay_alloc(w, T, 1, 100, 2)
    bad = ids.copy()
    bad[5] = bad[4]
    free_page = int(np.nonzero(np.unpackbits(w.view(np.uint8), bitorder="little")[:T] == 0)[0][0])
    bad[7] = free_page
    c = orc.check_alloc(w, before, T, bad)
    assert c.n_duplicates == 1 and c.n_not_marked == 1


def test_span_walk_finds_runs_across_words(orc):
    """Known answers: the only free run of 40 pages starts at page 60 (bits
    28..31 of word 1, all of word 2, bits 0..3 of word 3) and is found only
    from a jump to word 1; a 6-page run is found from word 1 (page 60, across
    words 1/2), word 2 (page 64, inside it) or word 4 (page 157, across 4/5)."""
    T = 32 * 8
    w = np.full(8, 0xFFFFFFFF, dtype=np.uint32)
    w[1] = 0x0FFFFFFF          # pages 60..63 free
    w[2] = 0                   # pages 64..95 free
    w[3] = 0xFFFFFFF0          # pages 96..99 free
    w[4] = 0x1FFFFFFF          # pages 157..159 free
    w[5] = 0xFFFFFFF8          # pages 160..162 free
    before = w.copy()
    L = orc.lib()
    st = orc.c_int32()
    found = set()
    for seed in range(40):
        x = w.copy()
        found.add(L.orc_walk_span(orc.P(x), T, 40, seed, 256, orc.ctypes.byref(st)))
    assert found == {60}
    found6 = {L.orc_walk_span(orc.P(w.copy()), T, 6, seed, 256, orc.ctypes.byref(st)) for seed in range(40)}
    assert found6 <= {60, 64, 157} and len(found6) >= 2
    x = w.copy()
    assert L.orc_walk_span(orc.P(x), T, 40, 3, 64, orc.ctypes.byref(st)) == 60
    assert x[2] == 0xFFFFFFFF and x[1] == 0xFFFFFFFF and x[3] == 0xFFFFFFFF
    L.orc_free_run(orc.P(x), 60, 40)
    assert np.array_equal(x, before)
    # no run of 41 pages exists: bounded failure
    assert L.orc_walk_span(orc.P(w.copy()), T, 41, 1, 64, orc.ctypes.byref(st)) == -1 and st.value == 64


def test_span_replay_bitmap_accounting(orc):
    # an i.i.d. prefill leaves long free stretches only when it is sparse
    # (P(100 free in a row) = 0.995^100 = 0.6 here)
    T = 1 << 14
    w = orc.bernoulli_bitmap(T, 0.005, 5)
    before = w.copy()
    k = np.random.default_rng(2).integers(1, 100, size=60)
    ids, steps = orc.replay_spans(w, T, k, 7)
    ok = ids >= 0
    assert ok.mean() > 0.9 and (steps[ok] >= 1).all()
    cover = np.zeros(T, dtype=np.int32)
    for i, kk in zip(ids[ok], k[ok]):
        cover[i:i + kk] += 1
    assert cover.max() == 1
    held = np.unpackbits(before.view(np.uint8), bitorder="little")[:T]
    assert int((held.astype(np.int32) * cover).sum()) == 0
    assert orc.used_pages(w, T) == orc.used_pages(before, T) + int(k[ok].sum())
    assert ((ids[ok] // 32) != ((ids[ok] + k[ok] - 1) // 32)).any()     # some runs cross words
    for i, kk in zip(ids[ok], k[ok]):
        orc.lib().orc_free_run(orc.P(w), int(i), int(kk))
    assert np.array_equal(w, before)


def test_runs_and_fifo(orc):
    T = 1 << 12
    w = orc.bernoulli_bitmap(T, 0.2, 2)
    before = w.copy()
    k = np.random.default_rng(1).integers(1, 9, size=100)
    ids, _ = orc.replay_runs(w, T, k, 3)
    assert (ids >= 0).all() and (((ids & 31) + k) <= 32).all()
    assert orc.used_pages(w, T) == orc.used_pages(before, T) + int(k.sum())
    for i, kk in zip(ids, k):
        orc.lib().orc_free_run(orc.P(w), int(i), int(kk))
    assert np.array_equal(w, before)
    assert orc.fifo_replay([3, 5, 9], [("get", None), ("put", 3), ("get", None), ("get", None),
                                       ("get", None), ("get", None)]) == [3, 5, 9, 3, -1]


def test_cpu_churn_keeps_occupancy(orc):
    T = 1 << 16
    w = orc.bernoulli_bitmap(T, 0.9, 2)
    bits = np.unpackbits(w.view(np.uint8), bitorder="little")[:T]
    held = np.nonzero(bits)[0].astype(np.int32)
    used0 = orc.used_pages(w, T)
    secs, ok, fail, st, thr = orc.cpu_churn(w, T, held, 50000, 3, threads=4)
    assert ok == 50000 and fail == 0
    assert orc.used_pages(w, T) == used0
    assert np.unique(held).size == held.size


def test_cpu_claim_write_free_restores_bitmap(orc):
    T, N = 1 << 16, 1 << 12
    words = orc.bernoulli_bitmap(T, 0.5, 1)
    before = words.copy()
    secs, ok, steps, threads = orc.cpu_claim_write_free(words, T, 64, 64, N, 1, 3, threads=2)
    assert ok == 3 * N and steps >= ok and secs > 0 and threads == 2
    assert np.array_equal(words, before)


def test_malloc_replay_blocks_and_release(orc):
    """The malloc replay packs sub-page blocks aligned to their class, gives
    larger blocks their own runs, and the last free of a run releases it."""
    T = 1 << 12
    w = orc.bernoulli_bitmap(T, 0.2, 3)
    before = w.copy()
    rep = orc.MallocReplay(w, T, 12)
    rng = np.random.default_rng(2)
    sizes = np.clip(np.exp(rng.uniform(np.log(16), np.log(65536), 96)), 16, 65536).astype(np.uint64)
    offs = []
    for q0 in range(0, 96, 32):
        o, _ = rep.group(sizes[q0:q0 + 32], orc.seed(9, q0), [orc.seed(10, q0 + l) for l in range(32)])
        offs.append(o)
    offs = np.concatenate(offs)
    assert (offs >= 0).all()
    cb = np.maximum(16, 1 << np.ceil(np.log2(sizes.astype(np.float64))).astype(np.int64))
    assert (offs % np.minimum(cb, 4096) == 0).all()     # class-aligned below a page, page-aligned above
    order = np.argsort(offs)
    assert (offs[order][1:] >= (offs + cb)[order][:-1]).all()
    for o in offs:
        assert rep.free(o) == 1
    assert rep.free(offs[0]) == 0          # double free is rejected
    assert np.array_equal(w, before)


def test_qmalloc_replay_reuses_queued_blocks(orc):
    """Queue backend: blocks are aligned to their class (page-aligned above a
    page), disjoint and inside the pool; freed blocks come back first (FIFO)
    before any new chunk is carved; everything freed sits in the queues."""
    T, shift = 1 << 12, 12
    w = orc.empty_bitmap(T)
    q = orc.QMallocReplay(w, T, shift, cap=1 << 12)
    rng = np.random.default_rng(3)
    seeds = lambda g: np.array([orc.lib().orc_seed(11, g * 32 + l) for l in range(32)], dtype=np.int32)
    blocks = []
    for g in range(8):
        sizes = np.clip(np.exp(rng.uniform(np.log(16), np.log(65536), 32)), 16, 65536).astype(np.uint64)
        offs, _ = q.group(sizes, seeds(g))
        assert (offs >= 0).all()
        cls = np.maximum(16, 1 << np.ceil(np.log2(sizes.astype(np.float64))).astype(np.int64))
        assert (offs % np.minimum(cls, 1 << shift) == 0).all()
        blocks += list(zip(offs.tolist(), cls.tolist()))
    s = sorted(blocks)
    assert all(a + la <= b for (a, la), (b, _) in zip(s, s[1:]))
    assert s[-1][0] + s[-1][1] <= T << shift
    chunks = q.q.chunks
    used = orc.used_pages(w, T)
    offs = np.array([b for b, _ in blocks], dtype=np.int64)
    for i in range(0, len(offs), 32):
        assert q.free(offs[i:i + 32]).all()
    queued = q.queued()
    pages = sum(n * (1 << (4 + c)) for c, n in enumerate(queued)) >> shift
    assert pages == used and q.q.overflow == 0          # every carved block is queued again
    # the same requests again: served from the queues, no new chunk
    rng = np.random.default_rng(3)
    for g in range(8):
        sizes = np.clip(np.exp(rng.uniform(np.log(16), np.log(65536), 32)), 16, 65536).astype(np.uint64)
        offs2, _ = q.group(sizes, seeds(g))
        assert (offs2 >= 0).all()
    assert q.q.chunks == chunks and orc.used_pages(w, T) == used
    bad = q.free(np.array([8, (T << shift) + 16, -1], dtype=np.int64))
    assert list(bad) == [0, 0, 1] and q.q.bad_frees == 2
    q.close()
