"""Buffer manager with CLOCK replacement (config 3 semantics).

* One GPU thread replaying the rounds equals the oracle's single-thread
  replay bit for bit: every frame id, hit / miss / eviction / failure count.
* Many threads: the page table and frame words stay inverse maps, nothing
  is left half-loaded, pins equal the fetches still held, and with a backing
  store every fetched frame holds its page's bytes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trace(n_logical, rounds, round_size, seed):
    import workloads

    pages = workloads.zipf_pages(n_logical, 0.99, rounds * round_size, seed)
    ptr, idx = workloads.release_lists(rounds, round_size, 0.25, seed)
    return pages, ptr, idx


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 8)])
def test_serial_rounds_match_oracle(cuda, pbm_mod, orc, policy, n_arms):
    torch = cuda
    pbm = pbm_mod
    n_logical, n_frames, rounds, R = 4096, 512, 24, 64
    pages, ptr, idx = _trace(n_logical, rounds, R, 3)
    bm = pbm.BufferManager(n_logical, n_frames, policy=policy, n_arms=n_arms)
    ref = orc.BufMgrReplay(n_logical, n_frames, n_arms=n_arms, dist=policy)
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
    h_frames = np.full(rounds * R, -1, dtype=np.int32)
    for r in range(rounds):
        a, b = int(ptr[r]), int(ptr[r + 1])
        bm.round(d_frames, d_idx[a:] if b > a else None, b - a, d_pages[r * R:], R, r * R,
                 d_frames[r * R:], serial=True)
        h_frames[r * R:(r + 1) * R] = ref.round(h_frames, idx[a:b].copy(), pages[r * R:(r + 1) * R].copy(), r * R)
    torch.cuda.synchronize()
    assert np.array_equal(d_frames.cpu().numpy(), h_frames)
    c = bm.counters()
    e = ref.counters()
    assert (c.hits, c.misses, c.evictions, c.failures, c.unpins, c.bad_unpins) == \
        (e["hits"], e["misses"], e["evictions"], e["failures"], e["unpins"], e["bad_unpins"])
    assert c.hits > 0 and c.evictions > 0
    chk = bm.check()
    assert chk.mismatches == 0 and chk.loading == 0
    bm.close()
    ref.close()


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 4096)])
def test_parallel_rounds_invariants_and_copy(cuda, pbm_mod, policy, n_arms):
    torch = cuda
    pbm = pbm_mod
    n_logical, n_frames, rounds, R, fsz = 1 << 18, 1 << 14, 32, 2048, 64
    pages, ptr, idx = _trace(n_logical, rounds, R, 5)
    backing = torch.arange(n_logical, dtype=torch.int32, device="cuda").repeat_interleave(fsz // 4)
    bm = pbm.BufferManager(n_logical, n_frames, frame_size=fsz, policy=policy, n_arms=n_arms, backing=backing)
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
    released = np.zeros(rounds * R, dtype=bool)
    for r in range(rounds):
        a, b = int(ptr[r]), int(ptr[r + 1])
        bm.round(d_frames, d_idx[a:] if b > a else None, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:])
        released[idx[a:b]] = True
        if r % 8 == 7 or r == rounds - 1:
            chk = bm.check()
            assert chk.mismatches == 0 and chk.loading == 0 and chk.resident == chk.mapped_frames
            fr = d_frames[:(r + 1) * R].cpu().numpy()
            held = (~released[:(r + 1) * R]) & (fr >= 0)
            assert chk.pins == int(held.sum())
    c = bm.counters()
    assert c.bad_unpins == 0 and c.timeouts == 0
    assert c.hits + c.misses + c.failures == rounds * R
    assert c.misses - c.evictions <= n_frames
    # frames fetched in the last round are still pinned: their bytes are their page's
    fptr, fbytes = bm.frames()
    assert fbytes == n_frames * fsz
    last = d_frames[(rounds - 1) * R:]
    out = torch.empty(R * 4 // 4, dtype=torch.int32, device="cuda")
    bm.gather(last, R, 4, out)
    got = out.cpu().numpy()
    lp = pages[(rounds - 1) * R:]
    ok = last.cpu().numpy() >= 0
    assert ok.mean() > 0.99
    assert np.array_equal(got[ok], lp[ok])
    bm.close()


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 8)])
def test_parallel_rounds_fewer_frames_than_a_warp(cuda, pbm_mod, policy, n_arms):
    """16 frames, so one warp's sweep batch wraps the frames twice (two lanes
    examine each frame) and most fetches find every frame pinned: fetches
    fail after their bounded sweep (or give up a bounded wait on a page
    another request is loading), and the maps stay consistent."""
    torch = cuda
    pbm = pbm_mod
    n_logical, n_frames, rounds, R = 256, 16, 12, 256
    pages, ptr, idx = _trace(n_logical, rounds, R, 8)
    bm = pbm.BufferManager(n_logical, n_frames, policy=policy, n_arms=n_arms)
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
    released = np.zeros(rounds * R, dtype=bool)
    for r in range(rounds):
        a, b = int(ptr[r]), int(ptr[r + 1])
        bm.round(d_frames, d_idx[a:] if b > a else None, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:])
        released[idx[a:b]] = True
        chk = bm.check()
        assert chk.mismatches == 0 and chk.loading == 0 and chk.resident == chk.mapped_frames
        fr = d_frames[:(r + 1) * R].cpu().numpy()
        assert ((fr >= -1) & (fr < n_frames)).all()
        held = (~released[:(r + 1) * R]) & (fr >= 0)
        assert chk.pins == int(held.sum())
    c = bm.counters()
    assert c.bad_unpins == 0
    assert c.hits + c.misses + c.failures + c.timeouts == rounds * R
    assert c.failures > 0 and c.misses > 0
    bm.close()


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 8)])
def test_serial_rounds_by_page_equal_by_frame(cuda, pbm_mod, policy, n_arms):
    """Releasing each pin by its page (pbm_bufmgr_round_pages, release list
    naming the held-page array it writes) replays exactly as releasing it by
    its frame: the same frame ids, counters and page table, with failed
    fetches (16 frames) holding nothing and releasing nothing."""
    torch = cuda
    pbm = pbm_mod
    for n_logical, n_frames, rounds, R in ((4096, 512, 24, 64), (256, 16, 12, 256)):
        pages, ptr, idx = _trace(n_logical, rounds, R, 3)
        by_frame = pbm.BufferManager(n_logical, n_frames, policy=policy, n_arms=n_arms)
        by_page = pbm.BufferManager(n_logical, n_frames, policy=policy, n_arms=n_arms)
        d_pages = torch.from_numpy(pages).cuda()
        d_idx = torch.from_numpy(idx).cuda()
        fa = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
        fb = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
        held = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
        for r in range(rounds):
            a, b = int(ptr[r]), int(ptr[r + 1])
            rel = d_idx[a:] if b > a else None
            by_frame.round(fa, rel, b - a, d_pages[r * R:], R, r * R, fa[r * R:], serial=True)
            by_page.round_pages(held, rel, b - a, d_pages[r * R:], R, r * R, fb[r * R:], held[r * R:], serial=True)
        torch.cuda.synchronize()
        assert torch.equal(fa, fb)
        h = held.cpu().numpy()
        f = fb.cpu().numpy()
        assert np.array_equal(h, np.where(f >= 0, pages, -1))
        ca, cb = by_frame.counters(), by_page.counters()
        assert (ca.hits, ca.misses, ca.evictions, ca.failures, ca.unpins, ca.bad_unpins) == \
            (cb.hits, cb.misses, cb.evictions, cb.failures, cb.unpins, cb.bad_unpins)
        assert cb.bad_unpins == 0
        ta, tb = by_frame.read_tables(), by_page.read_tables()
        for x, y in zip(ta, tb):
            assert np.array_equal(x, y)
        by_frame.close()
        by_page.close()


@pytest.mark.parametrize("policy,n_arms", [(0, 1), (1, 4096)])
@pytest.mark.parametrize("frames", [1 << 14, 16])
def test_parallel_rounds_by_page_invariants(cuda, pbm_mod, policy, n_arms, frames):
    """Many threads, pins released by page: the maps stay inverse, pins equal
    the fetches still held, every held-page entry is its fetch's page exactly
    when the fetch got a frame, and no release is bad."""
    torch = cuda
    pbm = pbm_mod
    n_logical, rounds, R = (1 << 18, 32, 2048) if frames > 16 else (256, 12, 256)
    pages, ptr, idx = _trace(n_logical, rounds, R, 5)
    bm = pbm.BufferManager(n_logical, frames, policy=policy, n_arms=n_arms)
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
    held = torch.full((rounds * R,), -1, dtype=torch.int32, device="cuda")
    released = np.zeros(rounds * R, dtype=bool)
    for r in range(rounds):
        a, b = int(ptr[r]), int(ptr[r + 1])
        bm.round_pages(held, d_idx[a:] if b > a else None, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:],
                       held[r * R:])
        released[idx[a:b]] = True
        if r % 4 == 3 or r == rounds - 1:
            chk = bm.check()
            assert chk.mismatches == 0 and chk.loading == 0 and chk.resident == chk.mapped_frames
            fr = d_frames[:(r + 1) * R].cpu().numpy()
            hp = held[:(r + 1) * R].cpu().numpy()
            assert np.array_equal(hp, np.where(fr >= 0, pages[:(r + 1) * R], -1))
            assert chk.pins == int(((~released[:(r + 1) * R]) & (fr >= 0)).sum())
    c = bm.counters()
    assert c.bad_unpins == 0
    assert c.hits + c.misses + c.failures + c.timeouts == rounds * R
    bm.close()


@pytest.mark.parametrize("serial", [True, False])
def test_bad_releases_are_counted_and_undone(cuda, pbm_mod, serial):
    """Releases of pins nobody holds -- a page whose pins were all released, a
    page never fetched, an out-of-range page, by page and by frame -- are
    counted bad and leave the page table as it was."""
    torch = cuda
    pbm = pbm_mod
    bm = pbm.BufferManager(1024, 64, policy=0)
    pages = torch.tensor([5, 6, 7, 5], dtype=torch.int32, device="cuda")
    frames = torch.full((4,), -1, dtype=torch.int32, device="cuda")
    bm.round(None, None, 0, pages, 4, 0, frames, serial=True)
    before = bm.read_tables()
    f = frames.cpu().numpy()
    assert (f >= 0).all() and f[0] == f[3]
    # page 5 holds 2 pins, 6 and 7 one each; release 5 three times, 900 (never
    # fetched) once, 4096 (out of range) once, and frame f[1] twice
    names = torch.tensor([5, 5, 5, 900, 4096], dtype=torch.int32, device="cuda")
    order = torch.arange(5, dtype=torch.int32, device="cuda")
    bm.round_pages(names, order, 5, None, 0, 0, None, serial=serial)
    fnames = torch.tensor([int(f[1]), int(f[1])], dtype=torch.int32, device="cuda")
    bm.round(fnames, order, 2, None, 0, 0, None, serial=serial)
    torch.cuda.synchronize()
    c = bm.counters()
    frame, pins, ref, fpage = bm.read_tables()
    assert np.array_equal(frame, before[0]) and np.array_equal(fpage, before[3])
    expect = before[1].copy()
    if serial:
        # one at a time: the held pins go, every release beyond them is bad
        assert c.unpins == 3 and c.bad_unpins == 4
        expect[[5, 6]] = 0
    else:
        # the releases of a name in one warp (one block when the round also
        # fetches) merge into one atomic: a group asking for more pins than
        # the page holds is rejected whole
        assert c.unpins == 0 and c.bad_unpins == 7
    assert np.array_equal(pins, expect)
    chk = bm.check()
    assert chk.mismatches == 0 and chk.loading == 0 and chk.pins == int(expect.sum())
    bm.close()


@pytest.mark.parametrize("by_page", [False, True])
def test_release_only_round_leaves_the_clock_alone(cuda, pbm_mod, by_page):
    """A round with releases and no fetches unpins and does nothing else: no
    sweep runs, so the reference bits (and the frames) stay as they were."""
    torch = cuda
    pbm = pbm_mod
    n_logical, n_frames, R = 1 << 16, 1 << 12, 4096
    bm = pbm.BufferManager(n_logical, n_frames, policy=0)
    rng = np.random.default_rng(11)
    pages = torch.from_numpy(rng.integers(0, n_logical, R).astype(np.int32)).cuda()
    frames = torch.full((R,), -1, dtype=torch.int32, device="cuda")
    held = torch.full((R,), -1, dtype=torch.int32, device="cuda")
    bm.round_pages(None, None, 0, pages, R, 0, frames, held)
    torch.cuda.synchronize()
    before = bm.read_tables()
    assert before[2].sum() > 0                       # fetched pages carry their reference bit
    idx = torch.arange(R, dtype=torch.int32, device="cuda")
    if by_page:
        bm.round_pages(held, idx, R, None, 0, 0, None)
    else:
        bm.round(frames, idx, R, None, 0, 0, None)
    torch.cuda.synchronize()
    frame, pins, ref, fpage = bm.read_tables()
    assert np.array_equal(frame, before[0]) and np.array_equal(ref, before[2]) and np.array_equal(fpage, before[3])
    assert pins.sum() == 0
    c = bm.counters()
    assert c.unpins == R and c.bad_unpins == 0
    chk = bm.check()
    assert chk.mismatches == 0 and chk.pins == 0
    bm.close()
