"""pbm_check_ids_noalloc, the invariant check for callers that cannot call
cudaMalloc (an engine that hands all device memory to its own pool at
start-up, or code running under a capture that forbids allocation).  It
keeps its scratch in a static device array, so it must give exactly the
counts of pbm_check_ids on the same inputs, call after call.  Collected
last on purpose: a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("n_ok", "n_failed", "n_out_of_range", "n_duplicates", "n_not_marked", "used_pages")


def _noalloc(pbm, pool, ids, n):
    r = pbm.CheckResult()
    rc = pbm.lib().pbm_check_ids_noalloc(pool.bitmap_ptr, pool.n_pages, ids.data_ptr(), n,
                                         ctypes.byref(r), None)
    return rc, r


def _pool_check(pbm, pool, ids, n):
    r = pbm.CheckResult()
    rc = pbm.lib().pbm_check_ids(pool.h, ids.data_ptr(), n, ctypes.byref(r), None)
    return rc, r


def test_noalloc_check_matches_pool_check_twice(cuda, pbm_mod):
    torch = cuda
    pbm = pbm_mod
    T, n = 1 << 20, 50000
    pool = pbm.Pool(T, 64)
    pool.prefill(0.5, 3)
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    pool.alloc(pbm.walk_config(pbm.COLLAB_RW_BM), n, 7, ids)
    torch.cuda.synchronize()

    # call 1: a clean allocation result
    rc_ref, ref = _pool_check(pbm, pool, ids, n)
    rc_na, na = _noalloc(pbm, pool, ids, n)
    assert rc_ref == rc_na == pbm.OK
    assert [getattr(na, f) for f in FIELDS] == [getattr(ref, f) for f in FIELDS]
    assert na.n_ok == n and na.n_duplicates == 0

    # call 2: planted faults; stale seen bits from call 1 would turn every id
    # into a duplicate, so this also shows the scratch is cleared per call
    bits = np.unpackbits(pool.read_bitmap().view(np.uint8), bitorder="little")[:T]
    free_page = int(np.nonzero(bits == 0)[0][0])
    bad = ids.clone()
    bad[10] = bad[3]
    bad[20] = T + 5
    bad[30] = -1
    bad[40] = free_page
    rc_ref2, ref2 = _pool_check(pbm, pool, bad, n)
    rc_na2, na2 = _noalloc(pbm, pool, bad, n)
    assert rc_ref2 == rc_na2 == pbm.ERR_CORRUPT
    assert [getattr(na2, f) for f in FIELDS] == [getattr(ref2, f) for f in FIELDS]
    assert (na2.n_duplicates, na2.n_out_of_range, na2.n_failed, na2.n_not_marked) == (1, 1, 1, 1)
    pool.close()


def test_noalloc_check_rejects_pools_over_its_limit(cuda, pbm_mod):
    torch = cuda
    pbm = pbm_mod
    ids = torch.zeros(4, dtype=torch.int32, device="cuda")
    bitmap = torch.zeros(8, dtype=torch.int32, device="cuda")
    r = pbm.CheckResult()
    rc = pbm.lib().pbm_check_ids_noalloc(bitmap.data_ptr(), (1 << 23) + 1, ids.data_ptr(), 4,
                                         ctypes.byref(r), None)
    assert rc == pbm.ERR_INVALID
