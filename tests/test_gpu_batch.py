"""Batched requests from many caller groups: plain (one launch per group),
persistent (one launch) and CUDA-graph replay run the same requests and must
all keep the allocation invariants; single-group persistent launches are
deterministic replays where the oracle can follow them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])


def _held_arena(orc, T, occ, seed):
    words = orc.bernoulli_bitmap(T, occ, seed)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(seed).shuffle(held)
    return words, held


def _descs(counts, op, start=0, arena_len=1 << 62):
    tab = np.zeros(len(counts), dtype=DT)
    cur = start
    for i, c in enumerate(counts):
        tab[i] = (op if isinstance(op, int) else op[i], c, cur % arena_len)
        cur += c
    return tab


@pytest.mark.parametrize("mode", ["plain", "persistent", "graph"])
@pytest.mark.parametrize("strategy,W,wb", [(2, 32, 32), (2, 16, 64), (2, 64, 32), (2, 64, 64), (1, 32, 32),
                                           (0, 32, 32)])
def test_swap_keeps_occupancy(cuda, pbm_mod, orc, mode, strategy, W, wb):
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    words, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    rng = np.random.default_rng(1)
    steps = 4
    counts = np.clip(np.exp(rng.uniform(0, np.log(4097), size=(steps, 64))).astype(np.int64), 1, 4096)
    tab = np.concatenate([_descs(counts[s], pbm.OP_SWAP, int(counts[:s].sum()), H) for s in range(steps)])
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    cfg = pbm.walk_config(strategy, word_bits=wb, collab_width=W)
    if mode == "graph":
        g = pool.graph(cfg, d_tab, 64, steps, arena, H, 500)
        for _ in range(steps):
            g.replay()
        g.close()
    else:
        for s in range(steps):
            rows = tab[s * 64:(s + 1) * 64]
            hg = pbm.groups_array([(int(r["op"]), int(r["count"]), int(r["offset"])) for r in rows])
            dg = d_tab[s * 64 * 16:(s + 1) * 64 * 16]
            pool.batch(cfg, dg, hg, 64, arena, H, 500 + s,
                       pbm.LAUNCH_PLAIN if mode == "plain" else pbm.LAUNCH_PERSISTENT)
    torch.cuda.synchronize()
    st = pool.stats()
    assert st.failures == 0
    assert st.successes == int(counts.sum()) == st.frees
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_out_of_range == 0 and chk.n_not_marked == 0
    assert chk.n_failed == 0
    assert chk.used_pages == H          # occupancy unchanged: every held page is in the arena
    a = arena.cpu().numpy()
    assert np.unique(a).size == H
    changed = int((a != held).sum())
    assert changed == min(H, int(counts.sum()))
    pool.close()


@pytest.mark.parametrize("fused", [True, False])
def test_graph_replays_past_its_steps_wrap(cuda, pbm_mod, orc, fused):
    """A graph of 2 descriptor tables replayed 5 times reads tables 0,1,0,1,0
    (never past the table), with a fresh seed each replay.  The unfused form
    (more groups than one block scans) runs its prefix kernel in the graph."""
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    n_groups = 64 if fused else 5000
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    words, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    rng = np.random.default_rng(3)
    counts = rng.integers(1, 40, size=(2, n_groups))
    tab = np.concatenate([_descs(counts[s], pbm.OP_SWAP, int(counts[:s].sum()), H) for s in range(2)])
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    g = pool.graph(pbm.walk_config(pbm.COLLAB_RW_BM), d_tab, n_groups, 2, arena, H, 900)
    for _ in range(5):
        g.replay()
    g.close()
    torch.cuda.synchronize()
    st = pool.stats()
    expect = 3 * int(counts[0].sum()) + 2 * int(counts[1].sum())
    assert st.failures == 0 and st.successes == expect == st.frees
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()


@pytest.mark.parametrize("fused", [True, False])
def test_graph_set_step_selects_the_table(cuda, pbm_mod, orc, fused):
    """The graph's step lives on the host and travels in the kernels'
    parameters: pbm_graph_set_step(k) makes the next replay read table
    k mod n_steps, and every request of that table is served exactly once --
    also the last tenth of the chunks, which the tail pools hand out (their
    counters start empty again after set_step)."""
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    n_groups = 64 if fused else 5000
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    words, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    rng = np.random.default_rng(5)
    hi = 4000 if fused else 60
    counts = rng.integers(1, hi, size=(3, n_groups))
    counts[1] //= 2   # three tables of different sizes
    tab = np.concatenate([_descs(counts[s], pbm.OP_SWAP, int(counts[:s].sum()), H) for s in range(3)])
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    g = pool.graph(pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=64, blocks_per_sm=5), d_tab, n_groups, 3,
                   arena, H, 700)
    done = 0
    for step in (1, 0, 4, 2, 2):   # replay reads table step mod 3
        g.set_step(step)
        g.replay()
        torch.cuda.synchronize()
        done += int(counts[step % 3].sum())
        st = pool.stats()
        assert st.failures == 0 and st.successes == done == st.frees
    # replays without set_step continue from the last step
    g.replay()
    torch.cuda.synchronize()
    done += int(counts[0].sum())   # step 3 -> table 0
    st = pool.stats()
    assert st.successes == done == st.frees
    g.close()
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()


def test_alloc_then_free_groups(cuda, pbm_mod, orc):
    """ALLOC groups fill an arena, FREE groups release it; mixed ops in one
    persistent batch keep the invariants and free restores the prefill."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 18
    pool = pbm.Pool(T, 64)
    pool.prefill(0.5, 6)
    words = orc.bernoulli_bitmap(T, 0.5, 6)
    base = orc.used_pages(words, T)
    counts = [1, 33, 1000, 7, 4096, 64, 1, 2048]
    N = sum(counts)
    arena = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    tab = _descs(counts, pbm.OP_ALLOC)
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM)
    pool.batch(cfg, d_tab, None, len(counts), arena, N, 9, pbm.LAUNCH_PERSISTENT)
    chk = pool.check(arena, N)
    assert chk.n_ok == N and chk.n_duplicates == 0 and chk.used_pages == base + N
    # free half the groups with FREE, swap the rest (mixed ops in one batch)
    ops = [pbm.OP_FREE if i % 2 == 0 else pbm.OP_SWAP for i in range(len(counts))]
    tab2 = _descs(counts, ops)
    d_tab2 = torch.from_numpy(tab2.view(np.uint8).copy()).cuda()
    pool.batch(cfg, d_tab2, None, len(counts), arena, N, 10, pbm.LAUNCH_PERSISTENT)
    n_freed = sum(c for c, o in zip(counts, ops) if o == pbm.OP_FREE)
    assert pool.used() == base + N - n_freed
    # free everything that is still held through FREE groups over the swapped slots
    keep = torch.cat([arena[int(tab2[i]["offset"]):int(tab2[i]["offset"]) + counts[i]]
                      for i in range(len(counts)) if ops[i] == pbm.OP_SWAP])
    pool.free(cfg, keep.numel(), keep)
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()


def test_single_group_persistent_matches_oracle(cuda, pbm_mod, orc):
    """One ALLOC group of 32*k requests through the persistent kernel with a
    pool so sparse that no two warps can race for a word: the result equals
    the oracle's group-by-group collaborative replay up to warp order, so ids
    match as a set per warp chunk and the bitmap matches exactly."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 22
    pool = pbm.Pool(T, 64)
    words = orc.empty_bitmap(T)
    n = 32 * 8
    arena = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    tab = _descs([n], pbm.OP_ALLOC)
    pool.batch(pbm.walk_config(pbm.COLLAB_RW_BM), torch.from_numpy(tab.view(np.uint8).copy()).cuda(),
               None, 1, arena, n, 33, pbm.LAUNCH_PERSISTENT)
    exp, _ = orc.replay_alloc(words, T, pbm.COLLAB_RW_BM, n, 33)
    got = arena.cpu().numpy()
    for c in range(0, n, 32):
        assert set(got[c:c + 32]) == set(exp[c:c + 32])
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()


@pytest.mark.parametrize("where", ["device", "pinned_host"])
def test_batch_results_buffer(cuda, pbm_mod, orc, where):
    """pbm_batch_launch_results writes request q's result to results[q]: the
    new page of an ALLOC or SWAP, the page a FREE released; into device memory
    or into pinned host memory the kernel writes directly."""
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    words, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    counts = [5000, 1, 64, 3000, 777]
    ops = [pbm.OP_SWAP, pbm.OP_SWAP, pbm.OP_FREE, pbm.OP_SWAP, pbm.OP_FREE]
    tab = _descs(counts, ops)
    N = sum(counts)
    if where == "device":
        res = torch.full((N,), -9, dtype=torch.int32, device="cuda")
    else:
        res = torch.full((N,), -9, dtype=torch.int32).pin_memory()
    before = arena.cpu().numpy().copy()
    for cfg in (pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=64), pbm.walk_config(pbm.COLLAB_RW_BM)):
        before = arena.cpu().numpy().copy()
        pool.batch(cfg, torch.from_numpy(tab.view(np.uint8).copy()).cuda(), None, len(counts), arena, H, 77,
                   pbm.LAUNCH_PERSISTENT, results=res)
        torch.cuda.synchronize()
        r = res.cpu().numpy() if where == "device" else res.numpy()
        after = arena.cpu().numpy()
        q = 0
        for c, op in zip(counts, ops):
            if op == pbm.OP_FREE:
                assert np.array_equal(r[q:q + c], before[q:q + c])       # the released pages
            else:
                assert np.array_equal(r[q:q + c], after[q:q + c])        # the new pages
            q += c
        # restore the released slots' pages so the next round starts from a full arena
        freed = np.concatenate([before[sum(counts[:i]):sum(counts[:i + 1])] for i, o in enumerate(ops)
                                if o == pbm.OP_FREE])
        ids = torch.from_numpy(freed.astype(np.int32)).cuda()
        st = torch.zeros(len(freed), dtype=torch.int32, device="cuda")
        n = len(freed)
        pool.alloc(pbm.walk_config(pbm.COLLAB_RW_BM), n, 5, ids)
        q = 0
        for c, op in zip(counts, ops):
            if op == pbm.OP_FREE:
                arena[q:q + c] = ids[:c]
                ids = ids[c:]
            q += c
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()


def test_graph_results_into_pinned_host(cuda, pbm_mod, orc):
    """pbm_batch_graph_create_results: each replay reads the staging table
    (refilled between replays) and writes its step's new pages into pinned
    host memory."""
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    words, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    stage = torch.zeros(16 * 8, dtype=torch.uint8, device="cuda")
    res = torch.full((40000,), -9, dtype=torch.int32).pin_memory()
    g = pool.graph(pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=64), stage, 8, 1, arena, H, 31, results=res)
    rng = np.random.default_rng(9)
    start = 0
    for step in range(3):
        counts = rng.integers(1, 5000, 8)
        tab = _descs(counts, pbm.OP_SWAP, start, H)
        stage.copy_(torch.from_numpy(tab.view(np.uint8).copy()))
        g.replay()
        torch.cuda.synchronize()
        n = int(counts.sum())
        a = arena.cpu().numpy()
        idx = (start + np.arange(n)) % H
        assert np.array_equal(res.numpy()[:n], a[idx])
        start = (start + n) % H
    g.close()
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()


def test_inline_table_launch(cuda, pbm_mod, orc):
    """Persistent launch with the host descriptor table carried in the kernel's
    parameters (d_groups NULL): the same oracle parity as a device table on a
    sparse pool, request-ordered results and invariants on a mixed batch, and
    tables that cannot be carried inline are rejected."""
    torch = cuda
    pbm = pbm_mod
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM)
    # parity: one ALLOC group on a pool where no two warps race for a word
    T = 1 << 22
    pool = pbm.Pool(T, 64)
    words = orc.empty_bitmap(T)
    n = 32 * 8
    arena = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    tab = _descs([n], pbm.OP_ALLOC)
    pool.batch(cfg, None, torch.from_numpy(tab.view(np.uint8).copy()), 1, arena, n, 33, pbm.LAUNCH_PERSISTENT)
    exp, _ = orc.replay_alloc(words, T, pbm.COLLAB_RW_BM, n, 33)
    got = arena.cpu().numpy()
    for c in range(0, n, 32):
        assert set(got[c:c + 32]) == set(exp[c:c + 32])
    assert np.array_equal(pool.read_bitmap(), words)
    pool.close()
    # mixed swap/free batch of 256 groups at 90%, results into pinned host memory
    T, occ, seed = 1 << 20, 0.9, 2
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    _, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    rng = np.random.default_rng(12)
    counts = rng.integers(1, 300, pbm.MAX_INLINE_GROUPS)
    ops = [pbm.OP_FREE if i % 7 == 3 else pbm.OP_SWAP for i in range(len(counts))]
    tab = _descs(counts, ops)
    h_tab = torch.from_numpy(tab.view(np.uint8).copy()).pin_memory()
    N = int(counts.sum())
    res = torch.full((N,), -9, dtype=torch.int32).pin_memory()
    before = arena.cpu().numpy().copy()
    bm0 = pool.read_bitmap()
    for c2 in (pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=64, blocks_per_sm=5), cfg):
        arena.copy_(torch.from_numpy(before))
        pool.write_bitmap(bm0)
        pool.batch(c2, None, h_tab, len(counts), arena, H, 78, pbm.LAUNCH_PERSISTENT, results=res)
        torch.cuda.synchronize()
        after = arena.cpu().numpy()
        r = res.numpy()
        q = 0
        for c, op in zip(counts, ops):
            c = int(c)
            want = before[q:q + c] if op == pbm.OP_FREE else after[q:q + c]
            assert np.array_equal(r[q:q + c], want)
            q += c
        swapped = np.concatenate([after[int(tab[i]["offset"]):int(tab[i]["offset"]) + int(counts[i])]
                                  for i in range(len(counts)) if ops[i] == pbm.OP_SWAP])
        untouched = after[N:]
        live = np.concatenate([swapped, untouched])
        assert len(np.unique(live)) == len(live)
        bits = np.unpackbits(pool.read_bitmap().view(np.uint8), bitorder="little")[:T]
        want_bits = np.zeros(T, dtype=np.uint8)
        want_bits[live] = 1
        assert np.array_equal(bits, want_bits)
    # too many groups, or a bad op, cannot be carried inline
    big = _descs([1] * (pbm.MAX_INLINE_GROUPS + 1), pbm.OP_SWAP)
    with pytest.raises(pbm.PbmError) as e:
        pool.batch(cfg, None, torch.from_numpy(big.view(np.uint8).copy()), len(big), arena, H, 1,
                   pbm.LAUNCH_PERSISTENT)
    assert e.value.rc == pbm.ERR_INVALID
    bad = _descs([4, 4], [pbm.OP_SWAP, 9])
    with pytest.raises(pbm.PbmError) as e:
        pool.batch(cfg, None, torch.from_numpy(bad.view(np.uint8).copy()), 2, arena, H, 1, pbm.LAUNCH_PERSISTENT)
    assert e.value.rc == pbm.ERR_INVALID
    pool.close()


def test_results_buffer_must_be_device_writable(cuda, pbm_mod, orc):
    """A pageable host buffer for results is refused before any launch (the
    kernel would otherwise write an address the device cannot reach)."""
    torch = cuda
    pbm = pbm_mod
    T = 1 << 16
    pool = pbm.Pool(T, 64)
    arena = torch.full((64,), -1, dtype=torch.int32, device="cuda")
    tab = _descs([64], pbm.OP_ALLOC)
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    pageable = np.full(64, -9, dtype=np.int32)
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM)
    with pytest.raises(pbm.PbmError) as e:
        pool.batch(cfg, d_tab, None, 1, arena, 64, 1, pbm.LAUNCH_PERSISTENT, results=pageable.ctypes.data)
    assert e.value.rc == pbm.ERR_INVALID
    with pytest.raises(pbm.PbmError) as e:
        pool.graph(cfg, d_tab, 1, 1, arena, 64, 1, results=pageable.ctypes.data)
    assert e.value.rc == pbm.ERR_INVALID
    torch.cuda.synchronize()
    assert pool.used() == 0 and (pageable == -9).all()
    pool.close()


@pytest.mark.parametrize("mode", ["plain", "persistent", "inline", "graph"])
def test_empty_groups_and_largest_group(cuda, pbm_mod, orc, mode):
    """Groups with no requests between others (first, middle, last), a group
    of the largest size (65,536 requests) and a batch of no groups: every
    request is served in request order, empty groups take no slot, and the
    invariants hold in every launch form."""
    torch = cuda
    pbm = pbm_mod
    T, occ, seed = 1 << 20, 0.9, 2
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, seed)
    _, held = _held_arena(orc, T, occ, seed)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    counts = [0, 65536, 0, 0, 17, 1, 0, 300, 0]
    tab = _descs(counts, pbm.OP_SWAP)
    N = sum(counts)
    res = torch.full((N,), -9, dtype=torch.int32, device="cuda")
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM, collab_width=64, blocks_per_sm=5)
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    hg = pbm.groups_array([(int(r["op"]), int(r["count"]), int(r["offset"])) for r in tab])
    # a batch of no groups is a no-op in every form
    pool.batch(cfg, d_tab, hg, 0, arena, H, 1, pbm.LAUNCH_PERSISTENT)
    pool.batch(cfg, d_tab, hg, 0, arena, H, 1, pbm.LAUNCH_PLAIN)
    torch.cuda.synchronize()
    assert pool.stats().successes == 0
    if mode == "graph":
        g = pool.graph(cfg, d_tab, len(counts), 1, arena, H, 41, results=res)
        g.replay()
        g.close()
    elif mode == "inline":
        pool.batch(cfg, None, torch.from_numpy(tab.view(np.uint8).copy()), len(counts), arena, H, 41,
                   pbm.LAUNCH_PERSISTENT, results=res)
    else:
        pool.batch(cfg, d_tab, hg, len(counts), arena, H, 41,
                   pbm.LAUNCH_PLAIN if mode == "plain" else pbm.LAUNCH_PERSISTENT, results=res)
    torch.cuda.synchronize()
    st = pool.stats()
    assert st.failures == 0 and st.successes == N == st.frees
    a = arena.cpu().numpy()
    assert np.array_equal(res.cpu().numpy(), a[:N])          # request q's page sits in slot q
    assert (a[:N] != held[:N]).all() and np.array_equal(a[N:], held[N:])
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()
