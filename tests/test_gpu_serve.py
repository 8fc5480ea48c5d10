"""Serving loop: continuous batching of tenants' alloc / free / fetch streams.

* Invariants across tenants: every held page belongs to exactly one tenant
  and is marked in the bitmap; the pool holds the prefill plus every tenant's
  pages; no request is left unadmitted.
* A tenant's results are the same alone and in the mix: page counts per
  request and the pages held at the end (page ids may differ; the counts and
  the invariants are exact)."""
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
    assert rc == pbm.OK and rep.completed == len(arr)
    status = np.array([r.status for r in res])
    assert set(np.unique(status)) <= {0, pbm.ERR_EXHAUSTED}                 # done, or over the tenant's budget
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
    assert c.hits + c.misses == int(cnt[ops == 2].sum()) and c.failures == 0
    mix_pages = np.array([r.pages for r in res])
    # tenant 3 alone: same requests, same arrival stamps
    sel = ten == 3
    pool2, bm2, srv2, res2, rep2, rc2 = _run(pbm, torch, orc, T, arr[sel], ten[sel], ops[sel], cnt[sel], 16,
                                            fetch_trace)
    assert rc2 == pbm.OK
    alone_pages = np.array([r.pages for r in res2])
    assert np.array_equal(alone_pages, mix_pages[sel])
    assert np.array_equal(np.array([r.status for r in res2]), status[sel])
    assert srv2.tenant_pages(3).size == held[3].size
    for o in (srv, srv2):
        o.close()
    for o in (bm, bm2):
        o.close()
    for o in (pool, pool2):
        o.close()
