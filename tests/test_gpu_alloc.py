"""GPU parity of the page allocators against the CPU oracle.

* Serial replays (one thread, or one warp for the collaborative walk) must
  match the oracle's sequential replay bit for bit: ids, steps, bitmap.
* Parallel launches are checked on the allocation invariants: every id in
  range and held by exactly one requester, popcount == prefill + successes,
  no failures while free pages >= requests, and free-everything restores the
  prefill bitmap exactly.
* Mean steps agree with the reference's closed-form models within 3 SE.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SERIAL_CASES = [
    # strategy, word_bits, width, T, occ
    (0, 32, 32, 8192, 0.5),
    (0, 32, 32, 65536, 0.9),
    (1, 32, 32, 8192, 0.6),
    (1, 64, 32, 8192, 0.9),
    (1, 32, 32, 65536 + 17, 0.3),      # ragged pool: padding bits
    (2, 32, 32, 8192, 0.7),
    (2, 64, 32, 8192, 0.9),
    (2, 32, 16, 8192, 0.8),
    (2, 32, 8, 8192, 0.5),
    (2, 32, 32, 96, 0.2),             # tiny pool: duplicate words inside one warp
    (3, 32, 32, 8192, 0.6),
    (5, 32, 32, 8192, 0.5),
    (6, 32, 32, 8192, 0.5),
]


def _pool(pbm, T, occ, seed, page_size=64, max_slots=0):
    p = pbm.Pool(T, page_size, max_slots=max_slots)
    p.prefill(occ, seed)
    return p


@pytest.mark.parametrize("strategy,wb,W,T,occ", SERIAL_CASES)
def test_serial_replay_bit_exact(cuda, pbm_mod, orc, strategy, wb, W, T, occ):
    torch = cuda
    pbm = pbm_mod
    seed, S = 3, 11
    n = min(700, int(T * (1 - occ) * 0.6)) or 8
    pool = _pool(pbm, T, occ, seed, max_slots=64)
    words = orc.bernoulli_bitmap(T, occ, seed)
    assert np.array_equal(pool.read_bitmap(), words)
    cfg = pbm.walk_config(strategy, word_bits=wb, collab_width=W, max_steps=1 << 14)
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    steps = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, n, S, ids, steps, serial=True)
    torch.cuda.synchronize()
    kw = {}
    if strategy == 3:
        kw["cursors"] = np.full(64, -1, dtype=np.int64)
    if strategy == 5:
        kw["arm"] = [0]
    if strategy == 6:
        kw["arms"] = np.array([orc.lib().orc_dist_clock_arm0(0, i, T) for i in range(64)], dtype=np.int64)
    exp_ids, exp_steps = orc.replay_alloc(words, T, strategy, n, S, word_bits=wb, collab_width=W,
                                          max_steps=1 << 14, **kw)
    got_ids = ids.cpu().numpy()
    assert np.array_equal(got_ids, exp_ids), f"first mismatch at {np.nonzero(got_ids != exp_ids)[0][:5]}"
    assert np.array_equal(steps.cpu().numpy(), exp_steps)
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()


PARALLEL_CASES = [
    (0, 32, 32, 1 << 20, 0.5, 1 << 16),
    (1, 32, 32, 1 << 20, 0.9, 1 << 16),
    (1, 64, 32, 1 << 20, 0.9, 1 << 16),
    (2, 32, 32, 1 << 20, 0.9, 1 << 16),
    (2, 64, 32, 1 << 20, 0.95, 1 << 15),
    (2, 32, 8, 1 << 20, 0.75, 1 << 16),
    (2, 32, 16, 1 << 20, 0.0, 1 << 18),
    (3, 32, 32, 1 << 20, 0.5, 1 << 16),
    (5, 32, 32, 1 << 18, 0.5, 1 << 14),
    (6, 32, 32, 1 << 20, 0.5, 1 << 16),
    (4, 32, 32, 1 << 20, 0.5, 1 << 16),
]


@pytest.mark.parametrize("strategy,wb,W,T,occ,n", PARALLEL_CASES)
def test_parallel_invariants(cuda, pbm_mod, orc, strategy, wb, W, T, occ, n):
    torch = cuda
    pbm = pbm_mod
    seed = 5
    pool = _pool(pbm, T, occ, seed, max_slots=n)
    words = orc.bernoulli_bitmap(T, occ, seed)
    base = orc.used_pages(words, T)
    assert T - base >= n
    cfg = pbm.walk_config(strategy, word_bits=wb, collab_width=W)
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, n, 99, ids)
    chk = pool.check(ids, n)
    assert chk.n_out_of_range == 0 and chk.n_duplicates == 0 and chk.n_not_marked == 0
    assert chk.n_failed == 0 and chk.n_ok == n
    assert chk.used_pages == base + n
    h = ids.cpu().numpy()
    # none of the returned pages was held by the prefill
    held = (words[h >> 5] >> (h & 31).astype(np.uint32)) & 1
    assert int(held.sum()) == 0
    pool.free(cfg, n, ids)
    assert pool.used() == base
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()


def test_exhaustion_is_bounded(cuda, pbm_mod, orc):
    """More requests than free pages: the surplus fails within its step bound
    (no trap, no spin) and the rest obey the invariants."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 16
    pool = _pool(pbm, T, 0.97, 8)
    base = pool.used()
    free = T - base
    n = free + 3000
    for strategy in (0, 1, 2):
        pool.reset()
        pool.prefill(0.97, 8)
        cfg = pbm.walk_config(strategy, max_steps=512)
        ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
        pool.alloc(cfg, n, 5, ids)
        chk = pool.check(ids, n)
        assert chk.n_duplicates == 0 and chk.n_out_of_range == 0 and chk.n_not_marked == 0
        assert chk.n_ok + chk.n_failed == n
        assert chk.n_failed >= n - free
        assert chk.used_pages == base + chk.n_ok
    pool.close()


def _mean_se(x):
    x = np.asarray(x, dtype=np.float64)
    return x.mean(), x.std(ddof=1) / math.sqrt(len(x))


def test_page_probe_steps_match_rw_tas(cuda, pbm_mod, orc):
    """Config-1 pool (65,536 pages, Bernoulli(0.5), seed 1), hold phase with
    N = 16,384 requests: mean probes vs RW_TAS at the realised A."""
    import models

    torch = cuda
    pbm = pbm_mod
    T, N = 65536, 16384
    pool = _pool(pbm, T, 0.5, 1)
    A = T - pool.used()
    cfg = pbm.walk_config(pbm.RANDOM_WALK)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, N, 1, ids, st)
    m, se = _mean_se(st.cpu().numpy())
    pred = models.rw_tas(T, A, N)
    assert abs(m - pred) <= 3 * se, (m, se, pred)
    pool.close()


@pytest.mark.parametrize("occ", [0.9, 0.95, 0.97])
def test_word_probe_steps_match_rwbm_tas(cuda, pbm_mod, orc, occ):
    """Word probe in the regime the model assumes (few claims per word)."""
    import models

    torch = cuda
    pbm = pbm_mod
    T, N = 1 << 20, 4096
    pool = _pool(pbm, T, occ, 2)
    A = T - pool.used()
    cfg = pbm.walk_config(pbm.RANDOM_WALK_BM)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, N, 2, ids, st)
    m, se = _mean_se(st.cpu().numpy())
    pred = models.rwbm_tas(T, A, N)
    assert abs(m - pred) <= 3 * se, (m, se, pred)
    pool.close()


@pytest.mark.parametrize("strategy,T,occ", [(0, 1 << 20, 0.9), (1, 1 << 22, 0.9), (1, 1 << 22, 0.95),
                                            (1, 1 << 22, 0.97)])
def test_per_warp_max_steps_within_was_models(cuda, pbm_mod, orc, strategy, T, occ):
    """RW_WAS / RWBM_WAS: the mean over warps of the per-warp maximum of the
    steps (unitTests/metrics.h:23-31) lies between the model at the batch's
    starting occupancy (A free) and at its final one (A - N free), within 3 SE.
    N is small against the words (the word-probe model assumes independent
    bits, which claims piling into the same words break)."""
    import models

    torch = cuda
    pbm = pbm_mod
    N = 4096
    pool = _pool(pbm, T, occ, 2)
    A = T - pool.used()
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    pool.alloc(pbm.walk_config(strategy), N, 5, ids, st)
    assert (ids.cpu().numpy() >= 0).all()
    m, se = _mean_se(st.cpu().numpy().reshape(-1, 32).max(axis=1))
    model = models.rw_was if strategy == 0 else models.rwbm_was
    lo, hi = model(T, A, 0), model(T, A, N)
    assert lo - 3 * se <= m <= hi + 3 * se, (m, se, lo, hi)
    pool.close()


@pytest.mark.parametrize("occ", [0.8, 0.9])
def test_collab_warp_steps_match_corwbm_was(cuda, pbm_mod, orc, occ):
    """CoRWBM_WAS (warp steps of the collaborative walk, 32 lanes): where the
    window's expected free bits cover the warp (80-90% occupancy) the model
    gives one jump; measured within 3 SE (plus 0.01 for the rare warp that
    loses bits to a concurrent grab).  At 95% and above the model's normal
    approximation undershoots the walk (1.2 vs 1.66 jumps at 97% in the
    oracle's replay), so it is not checked there."""
    pytest.importorskip("mpmath")
    import models

    torch = cuda
    pbm = pbm_mod
    T, N = 1 << 20, 4096
    pool = _pool(pbm, T, occ, 2)
    A = T - pool.used()
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    pool.alloc(pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=32), N, 5, ids, st)
    assert (ids.cpu().numpy() >= 0).all()
    warp = st.cpu().numpy().reshape(-1, 32)
    assert (warp == warp[:, :1]).all()            # every lane reports its warp's jumps
    m, se = _mean_se(warp[:, 0])
    pred = models.corwbm_was(T, A, N)
    assert abs(m - pred) <= 3 * se + 0.01, (m, se, pred)
    pool.close()


def test_config1_claim_write_free(cuda, pbm_mod, orc):
    """Config 1 as written: 32,768 requests on a 65,536-page pool at 50%
    (seed 1) each claim one page, write their index into its 64-B payload,
    and free it; the bitmap must come back to the prefill exactly.  A held
    run checks the payloads through the pool's own page memory."""
    torch = cuda
    pbm = pbm_mod
    T, N = 65536, 32768
    pool = pbm.Pool(T, 64, materialize=True)
    pool.prefill(0.5, 1)
    words = orc.bernoulli_bitmap(T, 0.5, 1)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    # hold: claim + write, check, then free
    pool.claim_write_free(N, 1, ids, hold=True)
    chk = pool.check(ids, N)
    assert chk.n_ok == N and chk.n_duplicates == 0 and chk.n_not_marked == 0
    out = torch.empty(N * 16, dtype=torch.int32, device="cuda")
    pool.gather_pages(ids, N, 64, out)
    expect = torch.arange(N, dtype=torch.int32, device="cuda").repeat_interleave(16)
    assert torch.equal(out, expect)
    cfg = pbm.walk_config(pbm.RANDOM_WALK)
    pool.free(cfg, N, ids)
    assert np.array_equal(pool.read_bitmap(), words)
    # the literal config: claim, write, free inside one kernel
    pool.claim_write_free(N, 2, ids, hold=False)
    h = ids.cpu().numpy()
    assert (h >= 0).all()
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()


def test_runs_serial_and_parallel(cuda, pbm_mod, orc):
    torch = cuda
    pbm = pbm_mod
    T = 1 << 14
    pool = _pool(pbm, T, 0.3, 9)
    words = orc.bernoulli_bitmap(T, 0.3, 9)
    rng = np.random.default_rng(3)
    k = rng.integers(1, 9, size=300).astype(np.int32)
    dk = torch.from_numpy(k).cuda()
    ids = torch.full((300,), -9, dtype=torch.int32, device="cuda")
    st = torch.zeros(300, dtype=torch.int32, device="cuda")
    pool.alloc_runs(300, dk, 17, ids, st, serial=True)
    exp_ids, exp_st = orc.replay_runs(words, T, k, 17)
    assert np.array_equal(ids.cpu().numpy(), exp_ids)
    assert np.array_equal(st.cpu().numpy(), exp_st)
    assert np.array_equal(pool.read_bitmap(), words)
    pool.free_runs(300, ids, dk)
    assert np.array_equal(pool.read_bitmap(), orc.bernoulli_bitmap(T, 0.3, 9))
    pool.close()
    # parallel: runs are disjoint, inside one word each, and on free pages
    T = 1 << 18
    pool = _pool(pbm, T, 0.3, 9)
    before = orc.bernoulli_bitmap(T, 0.3, 9)
    # runs of 1..8 pages, ending near 33% occupancy, where every size still
    # finds a fitting word within a few jumps
    n = 2000
    k = rng.integers(1, 9, size=n).astype(np.int32)
    dk = torch.from_numpy(k).cuda()
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc_runs(n, dk, 18, ids, max_steps=1 << 14)
    h = ids.cpu().numpy()
    assert (h >= 0).all()
    assert (((h & 31) + k) <= 32).all()
    cover = np.zeros(T, dtype=np.int32)
    for i, kk in zip(h, k):
        cover[i:i + kk] += 1
    assert cover.max() == 1
    held_before = np.unpackbits(before.view(np.uint8), bitorder="little")[:T]
    assert int((held_before.astype(np.int32) * cover).sum()) == 0
    assert pool.used() == orc.used_pages(before, T) + int(k.sum())
    pool.free_runs(n, ids, dk)
    assert np.array_equal(pool.read_bitmap(), before)
    pool.close()


def test_spans_serial_and_parallel(cuda, pbm_mod, orc):
    """Runs that cross word boundaries: a one-thread replay equals the
    oracle (ids, steps, bitmap); in parallel, runs of 1..200 pages are
    disjoint, inside the pool and on free pages, and freeing restores the
    prefill."""
    torch = cuda
    pbm = pbm_mod
    T, occ = 1 << 15, 0.005
    pool = _pool(pbm, T, occ, 12)
    words = orc.bernoulli_bitmap(T, occ, 12)
    rng = np.random.default_rng(8)
    k = rng.integers(1, 100, size=120).astype(np.int32)
    dk = torch.from_numpy(k).cuda()
    ids = torch.full((120,), -9, dtype=torch.int32, device="cuda")
    st = torch.zeros(120, dtype=torch.int32, device="cuda")
    pool.alloc_spans(120, dk, 19, ids, st, serial=True)
    exp_ids, exp_st = orc.replay_spans(words, T, k, 19)
    assert np.array_equal(ids.cpu().numpy(), exp_ids)
    assert np.array_equal(st.cpu().numpy(), exp_st)
    assert np.array_equal(pool.read_bitmap(), words)
    assert ((exp_ids[exp_ids >= 0] // 32) != ((exp_ids[exp_ids >= 0] + k[exp_ids >= 0] - 1) // 32)).any()
    pool.free_runs(120, ids, dk)
    assert np.array_equal(pool.read_bitmap(), orc.bernoulli_bitmap(T, occ, 12))
    pool.close()
    # parallel, on an empty pool of 2^20 pages: 4000 runs of 1..200 pages
    T = 1 << 20
    pool = _pool(pbm, T, 0.0, 1)
    n = 4000
    k = rng.integers(1, 201, size=n).astype(np.int32)
    dk = torch.from_numpy(k).cuda()
    ids = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    pool.alloc_spans(n, dk, 20, ids, max_steps=1 << 12)
    h = ids.cpu().numpy()
    ok = h >= 0
    assert ok.mean() > 0.99
    cover = np.zeros(T, dtype=np.int32)
    for i, kk in zip(h[ok], k[ok]):
        cover[i:i + kk] += 1
    assert cover.max() == 1 and (h[ok] + k[ok] <= T).all()
    assert pool.used() == int(k[ok].sum())
    pool.free_runs(n, ids, dk)
    assert pool.used() == 0
    pool.close()


def test_fifo_serial_order(cuda, pbm_mod, orc):
    """Linked-list strategy: FIFO order over the free pages (getPageLinkedList
    pops the head, freePageLinkedList appends at the tail)."""
    torch = cuda
    pbm = pbm_mod
    T = 4096
    pool = _pool(pbm, T, 0.5, 4)
    words = orc.bernoulli_bitmap(T, 0.5, 4)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T]
    free_sorted = np.nonzero(bits == 0)[0]
    cfg = pbm.walk_config(pbm.LINKED_LIST)
    ids = torch.empty(100, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, 100, 0, ids, serial=True)
    a = ids.cpu().numpy()
    assert np.array_equal(a, free_sorted[:100])
    for x in a[[5, 1, 9]]:          # one put per call: parallel puts have no order
        pool.free(cfg, 1, torch.tensor([int(x)], dtype=torch.int32, device="cuda"))
    ids2 = torch.empty(int(len(free_sorted) - 100 + 3), dtype=torch.int32, device="cuda")
    pool.alloc(cfg, ids2.numel(), 0, ids2, serial=True)
    b = ids2.cpu().numpy()
    exp = orc.fifo_replay(free_sorted, [("get", None)] * 100 + [("put", x) for x in a[[5, 1, 9]]]
                          + [("get", None)] * ids2.numel())[100:]
    assert np.array_equal(b, np.array(exp))
    # pool exhausted: the next get fails cleanly
    one = torch.empty(1, dtype=torch.int32, device="cuda")
    pool.alloc(cfg, 1, 0, one)
    assert int(one.item()) == -1
    pool.close()
