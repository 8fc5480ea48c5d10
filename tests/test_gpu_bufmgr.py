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
