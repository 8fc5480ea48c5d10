"""GPU runs at the workloads' own sizes, checked on the host by the oracle.

The allocation invariants here are judged by the oracle's own checker
(orc_check_alloc in oracle/oracle_core.c, a plain C loop over the ids and the
bitmaps copied to the host), not by the library's check kernel:

* every returned id is in range, returned once, marked held after the
  launch, and was free before it (so a page can never be handed to a second
  requester while another holds it, even if both free it later);
* the bits a launch set are exactly the ids it returned;
* the popcount follows prefill + granted - freed exactly, round by round.

Also here: the fail-fast launch budget (pbm_walk_config.fail_fast) in an
exhausted pool and its ordered hand-out of the free pages when a launch takes
most of them, and the collaborative walk's warp steps at 95-97% occupancy
against the oracle's sequential replay of the same requests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _new_bits(after, before, ids):
    """True iff the bits set by the launch are exactly the returned ids."""
    new = after & ~before
    got = ids[ids >= 0].astype(np.int64)
    mask = np.zeros_like(after)
    np.bitwise_or.at(mask, got >> 5, (np.uint32(1) << (got & 31).astype(np.uint32)))
    return np.array_equal(new, mask)


def _check_launch(orc, after, before, T, ids, used_before):
    c = orc.check_alloc(after, before, T, ids)
    assert c.n_out_of_range == 0 and c.n_duplicates == 0 and c.n_not_marked == 0, (
        c.n_out_of_range, c.n_duplicates, c.n_not_marked)
    assert c.n_prefilled == 0                      # every id was free when the launch started
    assert c.n_ok + c.n_failed == len(ids)
    assert c.used_after == used_before + c.n_ok
    assert _new_bits(after, before, ids)
    return c


@pytest.mark.parametrize("occ", [0.9, 0.95])
def test_config2_as_written_checked_by_the_oracle(cuda, pbm_mod, orc, occ):
    """2^24 pages, Bernoulli(occ) prefill with seed 2, 16 rounds of 2^22
    collaborative get-page requests (fail fast past the free pages, walks
    bounded at 1024 jumps), each round freeing a uniformly random 50% of what
    it got.  The pool runs out in the first round and stays exhausted."""
    torch = cuda
    pbm = pbm_mod
    T, N, rounds = 1 << 24, 1 << 22, 16
    pool = pbm.Pool(T, 4096)
    pool.prefill(occ, 2)
    words = orc.bernoulli_bitmap(T, occ, 2)
    assert np.array_equal(pool.read_bitmap(), words)
    used = orc.used_pages(words, T)
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=32, max_steps=1024, fail_fast=1)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(2)
    granted_total = 0
    for r in range(rounds):
        before = pool.read_bitmap()
        pool.alloc(cfg, N, 1000 + 31 * r, ids)
        after = pool.read_bitmap()
        h = ids.cpu().numpy()
        c = _check_launch(orc, after, before, T, h, used)
        assert c.n_ok <= T - used
        # the budget grants at most the free pages; nearly all of them are found.
        # The pool's free pages halve every round, and the last few hundred
        # can stay hidden from walks bounded at 1024 jumps (a jump covers 1024
        # of the 2^24 pages, while concurrent grabs hold words briefly)
        want = min(N, T - used)
        assert c.n_ok >= want - 512 - want // 100, (r, c.n_ok, T - used)
        used += c.n_ok
        granted_total += c.n_ok
        got = h[h >= 0]
        sel = rng.permutation(got)[: got.size // 2].astype(np.int32)
        pool.free(cfg, sel.size, torch.from_numpy(sel).cuda())
        w = pool.read_bitmap()
        assert orc.used_pages(w, T) == used - sel.size
        s64 = sel.astype(np.int64)
        assert not ((w[s64 >> 5] >> (s64 & 31).astype(np.uint32)) & 1).any()   # freed pages are clear
        used -= sel.size
    assert granted_total > 0
    pool.close()


@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_fail_fast_in_an_exhausted_pool(cuda, pbm_mod, orc, strategy):
    """More requests than free pages: with the launch budget the requests
    past the free pages fail with zero steps, the rest obey the invariants
    (oracle checker), and no more pages are granted than were free."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 20
    pool = pbm.Pool(T, 64)
    pool.prefill(0.95, 8)
    before = pool.read_bitmap()
    used = orc.used_pages(before, T)
    free = T - used
    n = free + (1 << 17)
    cfg = pbm.walk_config(strategy, max_steps=1024, fail_fast=1)
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    steps = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, n, 5, ids, steps)
    h, st = ids.cpu().numpy(), steps.cpu().numpy()
    c = _check_launch(orc, pool.read_bitmap(), before, T, h, used)
    assert c.n_ok <= free and c.n_failed >= n - free
    assert int(((h == -1) & (st == 0)).sum()) >= n - free    # refused by the budget, no walk
    assert (st[h >= 0] >= 1).all()
    pool.close()


@pytest.mark.parametrize("strategy", [0, 1, 2, 3, 5, 6])
def test_fail_fast_lists_the_free_pages_when_a_launch_takes_most_of_them(cuda, pbm_mod, orc, strategy):
    """A launch that asks for at least half of the free pages (but fewer than
    all of them) gets them from the budget pass's ordered list: every
    request succeeds with one step, and the pages handed out are exactly the
    lowest-numbered free pages."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 20
    pool = pbm.Pool(T, 64, max_slots=1 << 16)
    pool.prefill(0.9, 12)
    before = pool.read_bitmap()
    used = orc.used_pages(before, T)
    free = T - used
    n = (free * 3) // 5
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    steps = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc(pbm.walk_config(strategy, fail_fast=1), n, 3, ids, steps)
    h, st = ids.cpu().numpy(), steps.cpu().numpy()
    c = _check_launch(orc, pool.read_bitmap(), before, T, h, used)
    assert c.n_ok == n and (st == 1).all()
    bits = np.unpackbits(before.view(np.uint8), bitorder="little")[:T]
    lowest = np.nonzero(bits == 0)[0][:n]
    assert np.array_equal(np.sort(h), lowest)
    pool.close()


@pytest.mark.parametrize("strategy", [0, 1, 2, 3, 5, 6])
def test_fail_fast_changes_nothing_while_pages_remain(cuda, pbm_mod, orc, strategy):
    """Free pages well above the requests: every request succeeds with or
    without the budget, and the budget refuses nobody."""
    torch = cuda
    pbm = pbm_mod
    T, n = 1 << 20, 1 << 16
    for ff in (0, 1):
        pool = pbm.Pool(T, 64, max_slots=n)
        pool.prefill(0.5, 9)
        before = pool.read_bitmap()
        used = orc.used_pages(before, T)
        ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
        pool.alloc(pbm.walk_config(strategy, fail_fast=ff), n, 7, ids)
        c = _check_launch(orc, pool.read_bitmap(), before, T, ids.cpu().numpy(), used)
        assert c.n_ok == n and c.n_failed == 0
        pool.close()


@pytest.mark.parametrize("occ", [0.95, 0.97])
def test_collab_warp_steps_at_high_occupancy_match_the_oracle_replay(cuda, pbm_mod, orc, occ):
    """At 95-97% occupancy the closed-form CoRWBM_WAS undershoots, so the
    GPU's collaborative warp steps are compared with the oracle's sequential
    replay of the same requests instead.  Each warp walks the same jump
    sequence in both (same group seeds); only the claims of other warps
    differ (concurrent on the GPU, earlier in the replay), which changes a
    warp's outcome rarely while the requests are few against the free pages."""
    torch = cuda
    pbm = pbm_mod
    T, N, S = 1 << 20, 4096, 5
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, 2)
    words = orc.bernoulli_bitmap(T, occ, 2)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    pool.alloc(pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=32), N, S, ids, st)
    assert (ids.cpu().numpy() >= 0).all()
    g = st.cpu().numpy().reshape(-1, 32)[:, 0].astype(np.float64)
    r_ids, r_steps = orc.replay_alloc(words.copy(), T, pbm.COLLAB_RW_BM, N, S, collab_width=32)
    o = np.asarray(r_steps).reshape(-1, 32)[:, 0].astype(np.float64)
    assert (np.asarray(r_ids) >= 0).all()
    d = g - o
    se = d.std(ddof=1) / np.sqrt(d.size) if d.any() else 0.0
    assert abs(d.mean()) <= 3 * se + 0.02, (g.mean(), o.mean(), se)
    assert (d == 0).mean() >= 0.8                  # most warps take exactly the replay's jumps
    pool.close()


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 4096)])
def test_config3_buffer_manager_at_size_checked_on_the_host(cuda, pbm_mod, orc, policy, n_arms):
    """2^22 frames over 2^24 logical pages, Zipf(0.99) fetches through a
    seed-3 permutation in rounds of 2^18, pins held Geometric(0.25) rounds;
    run until the frames are full and evicting.  The maps are copied to the
    host and checked there: page -> frame and frame -> page are inverse,
    every page's pin count equals its fetches not yet released, reference
    bits sit only on resident pages, and every returned frame held its page
    when it was returned and still does while pinned."""
    import workloads

    torch = cuda
    pbm = pbm_mod
    # the first 4.2 M distinct pages arrive by about round 88 of 2^18 fetches;
    # the 40 rounds after that evict
    n_logical, n_frames, R, rounds = 1 << 24, 1 << 22, 1 << 18, 128
    pages = workloads.zipf_pages(n_logical, 0.99, R * rounds, 3)
    ptr, idx = workloads.release_lists(rounds, R, 0.25, 3)
    bm = pbm.BufferManager(n_logical, n_frames, policy=policy, n_arms=n_arms)
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.full((R * rounds,), -1, dtype=torch.int32, device="cuda")
    released = np.zeros(R * rounds, dtype=bool)
    evicting = False
    for r in range(rounds):
        a, b = int(ptr[r]), int(ptr[r + 1])
        bm.round(d_frames, d_idx[a:] if b > a else None, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:])
        released[idx[a:b]] = True
        c = bm.counters()
        evicting = evicting or c.evictions > 0
        if r % 32 == 31:
            frame, pins, ref, fpage = bm.read_tables()
            fr = d_frames[:(r + 1) * R].cpu().numpy()
            res = np.nonzero(frame >= 0)[0]
            assert (frame[res] < n_frames).all() and np.array_equal(fpage[frame[res]], res)   # page -> frame -> page
            mapped = np.nonzero(fpage >= 0)[0]
            assert np.array_equal(frame[fpage[mapped]], mapped)                          # frame -> page -> frame
            assert res.size == mapped.size and res.size <= n_frames
            assert not (frame < -1).any()                                              # nothing left loading
            held = (~released[:(r + 1) * R]) & (fr >= 0)
            want = np.bincount(pages[:(r + 1) * R][held], minlength=n_logical)
            assert np.array_equal(pins, want)                                           # exact pin accounting
            assert not ref[frame < 0].any()
            # a pinned fetch's frame still holds its page
            assert np.array_equal(fpage[fr[held]], pages[:(r + 1) * R][held])
            chk = bm.check()
            assert chk.mismatches == 0 and chk.loading == 0
    c = bm.counters()
    assert evicting and c.evictions > 0 and c.failures == 0 and c.timeouts == 0 and c.bad_unpins == 0
    assert c.hits + c.misses == R * rounds
    bm.close()


def test_config4_malloc_round_on_the_32gib_pool(cuda, pbm_mod, orc):
    """Config 4 at its own size: a 32 GiB pool of 4 KiB pages, 256 caller
    groups with LogU[1, 65536] requests (seed 4) and sizes LogU[16 B, 64 KiB]
    in one persistent launch; then a uniformly random 50% of the blocks
    freed and a second round of mallocs.  On the host: every live block
    (survivors and new ones together) is aligned to its class (or a page),
    inside the pool and disjoint from every other; freeing everything leaves
    an empty bitmap, no live run and no bad free."""
    import math

    torch = cuda
    pbm = pbm_mod
    T, PAGE = 1 << 23, 4096
    pool = pbm.Pool(T, PAGE, materialize=True)
    pool.malloc_init()
    rng = np.random.default_rng(4)
    DT = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])

    def logu_counts(n):
        return np.clip(np.floor(np.exp(rng.uniform(0.0, math.log(65537), n))), 1, 65536).astype(np.int64)

    def logu_sizes(n):
        return np.clip(np.exp(rng.uniform(math.log(16), math.log(65536), n)), 16, 65536).astype(np.uint32)

    c1, c2 = logu_counts(256), logu_counts(256)
    n1, n2 = int(c1.sum()), int(c2.sum())
    k = n1 // 2
    slots = n1 + k + n2
    sizes = np.zeros(slots, dtype=np.uint32)
    sizes[:n1] = logu_sizes(n1)
    sizes[n1 + k:] = logu_sizes(n2)
    d_sizes = torch.from_numpy(sizes.astype(np.int32)).cuda()
    ptrs = torch.zeros(slots, dtype=torch.int64, device="cuda")

    def launch(groups, seed):
        tab = np.zeros(len(groups), dtype=DT)
        for i, g in enumerate(groups):
            tab[i] = g
        pool.malloc_batch(torch.from_numpy(tab.view(np.uint8).copy()).cuda(), None, len(groups), d_sizes, ptrs,
                          slots, seed, pbm.LAUNCH_PERSISTENT, max_steps=512)
        torch.cuda.synchronize()

    def check(live_ptrs, live_sizes):
        ok = live_ptrs != 0
        off = live_ptrs[ok] - pool.base_ptr
        cb = np.maximum(16, 1 << np.ceil(np.log2(np.maximum(live_sizes[ok].astype(np.int64), 1))).astype(np.int64))
        assert (off % np.minimum(cb, PAGE) == 0).all()
        assert (off >= 0).all() and ((off + cb) <= T * PAGE).all()
        order = np.argsort(off)
        s, e = off[order], (off + cb)[order]
        assert (s[1:] >= e[:-1]).all()
        return int(ok.sum())

    offs1 = np.concatenate([[0], np.cumsum(c1)[:-1]])
    launch([(pbm.OP_MALLOC, int(c), int(o)) for c, o in zip(c1, offs1)], 41)
    p1 = ptrs.cpu().numpy()[:n1].copy()
    assert check(p1, sizes[:n1]) >= int(0.99 * n1)          # the first round fits the empty pool
    # free a uniform half: their pointers move to slots [n1, n1 + k)
    perm = rng.permutation(n1)
    gone, kept = perm[:k], perm[k:]
    ptrs[n1:n1 + k].copy_(torch.from_numpy(p1[gone]))
    launch([(pbm.OP_MFREE, k, n1)], 42)
    assert (ptrs[n1:n1 + k].cpu().numpy() == 0).all()
    offs2 = n1 + k + np.concatenate([[0], np.cumsum(c2)[:-1]])
    launch([(pbm.OP_MALLOC, int(c), int(o)) for c, o in zip(c2, offs2)], 43)
    p2 = ptrs.cpu().numpy()[n1 + k:].copy()
    live = np.concatenate([p1[kept], p2])
    live_sizes = np.concatenate([sizes[:n1][kept], sizes[n1 + k:]])
    check(live, live_sizes)
    live_runs, bad = pool.malloc_counts()
    assert bad == 0 and live_runs > 0
    # free everything that is live: the pool comes back empty
    nl = live.size
    ptrs[:nl].copy_(torch.from_numpy(live))
    launch([(pbm.OP_MFREE, nl, 0)], 44)
    live_runs, bad = pool.malloc_counts()
    assert live_runs == 0 and bad == 0
    assert pool.used() == 0
    pool.close()
