"""Serving loop: continuous batching of tenants' alloc / free / fetch streams.

* Invariants across tenants: every held page belongs to exactly one tenant
  and is marked in the bitmap; the pool holds the prefill plus every tenant's
  pages.
* Admission by a shared free-page budget: an ALLOC that does not fit waits
  for frees instead of being rejected; only an ALLOC larger than the whole
  budget is rejected.
* A tenant's results are the same alone and in the mix: status and page
  count of every request the mix admits (page ids may differ; the counts and
  the invariants are exact).  Under contention -- tenants whose combined
  demand exceeds the budget -- requests wait, and still get the same results.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream(rng, n, tenants, rate_pages, fetch=True):
    sizes = np.clip(np.exp(rng.uniform(0, np.log(4097), n)), 1, 4096).astype(np.int64)
    gaps = rng.exponential(sizes.mean() / rate_pages, n)
    arr = np.cumsum(gaps)
    ten = rng.integers(0, tenants, n)
    u = rng.uniform(size=n)
    ops = np.where(u < 0.45, 0, np.where(u < 0.90, 1, 2 if fetch else 1))
    return arr, ten, ops, sizes


def _run(pbm, torch, orc, T, arr, ten, ops, cnt, n_tenants, fetch_trace):
    pool = pbm.Pool(T, 64)
    pool.prefill(0.85, 5)
    bm = pbm.BufferManager(1 << 20, 1 << 14, policy=pbm.BM_DIST_CLOCK, n_arms=4096)
    srv = pbm.Server(pool, n_tenants, 1 << 18, n_streams=4, max_batch_requests=256, max_occupancy=0.95,
                     bufmgr=bm, fetch_pages=fetch_trace)
    res, rep, rc = srv.run(arr, ten, ops, cnt)
    return pool, bm, srv, res, rep, rc


def test_serving_invariants_and_alone_equals_mix(cuda, pbm_mod, orc):
    torch = cuda
    pbm = pbm_mod
    import workloads

    T = 1 << 20
    fetch_trace = torch.from_numpy(workloads.zipf_pages(1 << 20, 0.99, 1 << 20, 5)).cuda()
    rng = np.random.default_rng(5)
    arr, ten, ops, cnt = _stream(rng, 3000, 16, 5e7)
    pool, bm, srv, res, rep, rc = _run(pbm, torch, orc, T, arr, ten, ops, cnt, 16, fetch_trace)
    assert rc == pbm.OK
    status = np.array([r.status for r in res])
    assert set(np.unique(status)) <= {0, -1}                # done, or still waiting for memory at the end
    assert rep.stranded == int((status == -1).sum()) and rep.completed == int((status == 0).sum())
    assert rep.rejected == int((status != 0).sum())
    assert rep.batches >= 2 and rep.p99_s >= rep.p50_s > 0
    held = [srv.tenant_pages(t) for t in range(16)]
    allp = np.concatenate(held)
    assert (allp >= 0).all() and np.unique(allp).size == allp.size          # no page held twice
    base = orc.used_pages(orc.bernoulli_bitmap(T, 0.85, 5), T)
    assert pool.used() == base + allp.size                                   # popcount = prefill + tenants
    chk = pool.check(torch.from_numpy(allp).cuda(), allp.size)
    assert chk.n_not_marked == 0 and chk.n_duplicates == 0
    c = bm.counters()
    assert c.hits + c.misses == int(cnt[(ops == 2) & (status == 0)].sum()) and c.failures == 0
    mix_pages = np.array([r.pages for r in res])
    # tenant 3 alone: same requests, same arrival stamps
    sel = ten == 3
    pool2, bm2, srv2, res2, rep2, rc2 = _run(pbm, torch, orc, T, arr[sel], ten[sel], ops[sel], cnt[sel], 16,
                                            fetch_trace)
    assert rc2 == pbm.OK
    alone_pages = np.array([r.pages for r in res2])
    alone_status = np.array([r.status for r in res2])
    admitted = status[sel] == 0                              # the mix's admitted requests
    assert (alone_status == 0).all()                         # alone, nothing waits for other tenants
    assert np.array_equal(alone_pages[admitted], mix_pages[sel][admitted])
    if admitted.all():
        assert srv2.tenant_pages(3).size == held[3].size
    for o in (srv, srv2):
        o.close()
    for o in (bm, bm2):
        o.close()
    for o in (pool, pool2):
        o.close()


def _tenant_major(rng, tenants, cycles, max_pages):
    per = []
    for t in range(tenants):
        ops = []
        for c in range(cycles):
            x, y = (int(v) for v in rng.integers(1, max_pages + 1, 2))
            ops += [(0, x), (0, y), (1, x), (1, y)]
        per.append(ops)
    return per


def test_contended_budget_waits_and_results_match_alone(cuda, pbm_mod, orc):
    """8 tenants whose bursts together need about 3x the shared budget:
    ALLOCs wait for other tenants' frees (none is rejected or stranded), the
    invariants hold, and two tenants run alone get identical statuses and
    page counts, request by request."""
    torch = cuda
    pbm = pbm_mod
    T, tenants, cycles, max_pages = 1 << 20, 8, 24, 12000
    rng = np.random.default_rng(11)
    per = _tenant_major(rng, tenants, cycles, max_pages)
    # interleave the tenants' streams in a random order, each keeping its own order
    picks = np.concatenate([np.full(len(p), t) for t, p in enumerate(per)])
    rng.shuffle(picks)
    pos = [0] * tenants
    ten, ops, cnt = [], [], []
    for t in picks:
        o, k = per[t][pos[t]]
        pos[t] += 1
        ten.append(t)
        ops.append(o)
        cnt.append(k)
    ten, ops, cnt = np.array(ten), np.array(ops), np.array(cnt)
    arr = np.cumsum(rng.exponential(2e-6, len(ten)))       # all arrive within about a millisecond

    def run(sel):
        pool = pbm.Pool(T, 64)
        pool.prefill(0.9, 5)
        srv = pbm.Server(pool, tenants, 1 << 16, n_streams=4, max_batch_requests=64, max_occupancy=0.95)
        res, rep, rc = srv.run(arr[sel], ten[sel], ops[sel], cnt[sel])
        return pool, srv, res, rep, rc

    pool, srv, res, rep, rc = run(np.ones(len(ten), dtype=bool))
    budget = int(0.95 * T) - orc.used_pages(orc.bernoulli_bitmap(T, 0.9, 5), T)
    peak_demand = sum(max(a + b for (_, a), (_, b) in zip(p[0::4], p[1::4])) for p in per)
    assert peak_demand > 2 * budget                           # the tenants contend for the budget
    assert rc == pbm.OK
    status = np.array([r.status for r in res])
    pages = np.array([r.pages for r in res])
    assert (status == 0).all() and rep.stranded == 0 and rep.rejected == 0
    assert rep.waited > 0                                     # some ALLOCs waited for memory
    assert np.array_equal(pages[ops == 0], cnt[ops == 0])     # every ALLOC got all its pages
    held = [srv.tenant_pages(t) for t in range(tenants)]
    assert all(h.size == 0 for h in held)                     # every burst was freed
    assert pool.used() == orc.used_pages(orc.bernoulli_bitmap(T, 0.9, 5), T)
    assert rep.p99_s >= rep.p50_s > 0
    lat = np.array([r.done_s - a for r, a in zip(res, arr)])
    wait = np.array([r.admit_s - a for r, a in zip(res, arr)])
    assert wait.max() > 0 and (lat >= wait).all()             # latency includes the wait
    srv.close()
    pool.close()
    for t in (2, 5):
        sel = ten == t
        pool2, srv2, res2, rep2, rc2 = run(sel)
        assert rc2 == pbm.OK
        assert np.array_equal(np.array([r.status for r in res2]), status[sel])
        assert np.array_equal(np.array([r.pages for r in res2]), pages[sel])
        srv2.close()
        pool2.close()


def test_alloc_larger_than_the_budget_is_rejected(cuda, pbm_mod, orc):
    """Only an ALLOC that could never fit is rejected; the tenant's next
    requests go on."""
    pbm = pbm_mod
    T = 1 << 16
    pool = pbm.Pool(T, 64)
    pool.prefill(0.9, 3)
    srv = pbm.Server(pool, 2, 1 << 16, n_streams=2, max_batch_requests=16, max_occupancy=0.95)
    budget = int(0.95 * T) - pool.used()
    arr = np.array([0.0, 1e-6, 2e-6, 3e-6])
    ten = np.array([0, 0, 1, 0])
    ops = np.array([0, 0, 0, 1])
    cnt = np.array([budget + 1, 100, 50, 100])
    res, rep, rc = srv.run(arr, ten, ops, cnt)
    assert rc == pbm.OK
    assert [r.status for r in res] == [pbm.ERR_EXHAUSTED, 0, 0, 0]
    assert [r.pages for r in res] == [0, 100, 50, 100]
    assert rep.rejected == 1 and rep.stranded == 0
    srv.close()
    pool.close()
