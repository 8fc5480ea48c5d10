"""The autotuner runs every candidate configuration on the caller's swap
batch, ranks them, and leaves the pool in its occupancy band."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])


def test_autotune_ranks_candidates_and_keeps_occupancy(cuda, pbm_mod, orc):
    torch = cuda
    pbm = pbm_mod
    T, occ = 1 << 20, 0.9
    pool = pbm.Pool(T, 64)
    pool.prefill(occ, 2)
    words = orc.bernoulli_bitmap(T, occ, 2)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(2).shuffle(held)
    H = len(held)
    arena = torch.from_numpy(held).cuda()
    counts = np.clip(np.exp(np.random.default_rng(4).uniform(0, np.log(4097), 64)).astype(np.int64), 1, 4096)
    tab = np.zeros(64, dtype=DT)
    tab["op"] = pbm.OP_SWAP
    tab["count"] = counts
    tab["offset"] = np.concatenate([[0], np.cumsum(counts)[:-1]])
    d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    res = pool.autotune(d_tab, 64, int(counts.sum()), arena, H, reps=2)
    assert len(res) == 2 * (1 + 2 + 16) + 2
    rates = [r.ops_per_s for r in res]
    assert all(r > 0 for r in rates) and rates == sorted(rates, reverse=True)
    kinds = {(r.cfg.strategy, r.cfg.word_bits, r.cfg.collab_width, r.cfg.stride, r.cfg.blocks_per_sm,
              r.cfg.free_merge) for r in res}
    assert len(kinds) == len(res)
    st = pool.stats()
    assert st.failures == 0
    chk = pool.check(arena, H)
    assert chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == H
    pool.close()
