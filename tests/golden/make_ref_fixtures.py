"""Generate golden fixtures from the reference's own device code.

Runs on a machine with a GPU.  Loads the cubins that oracle/Makefile
(`make ref`) compiles from the reference's sources (harness TUs under
oracle/ref_harness/ include those sources unchanged and pin clock()), calls
the reference's allocation routines one thread / one warp at a time through
the CUDA driver API, and writes their outputs as JSON next to this script
(or into the directory given as argv[1]).  The oracle's reference-mode
restatements are checked against these files by tests/test_oracle_pinning.py.

Every scenario keeps the pool far from exhaustion: the reference traps
(RandomWalkBasic.cuh:66-69) or spins (CollabRW_BM.cuh:123) when it runs out.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

from ref_driver import D, Driver  # noqa: E402


def int_map(n_pages, occ, seed):
    """int-per-page map: map[p] = bit p of the oracle's Bernoulli bitmap."""
    w = oracle.bernoulli_bitmap(n_pages, occ, seed)
    bits = np.unpackbits(w.view(np.uint8), bitorder="little")[:n_pages]
    return bits.astype(np.int32)


def clocks(rng, n):
    return rng.integers(-32768, 32768, size=n).astype(np.int32)


def grid_for(tid):
    return tid // 256 + 1, 256


def fx_lcg(drv):
    m = drv.module("ref_rwbm.cubin")
    rng = np.random.default_rng(101)
    vals = [0, 1, -1, 2, 12345, -12345, 2**31 - 1, -2**31, -2**31 + 1, 1103515245, -1103515245,
            32767, -32768, 65535 << 15]
    vals = [((v + 2**31) % 2**32) - 2**31 for v in vals]
    xin = np.array(vals + list(rng.integers(-2**31, 2**31, size=242)), dtype=np.int32)
    out = np.zeros_like(xin)
    di, do = drv.upload(xin), drv.alloc(out.nbytes)
    drv.launch(drv.fn(m, "fx_lcg"), 1, 256, len(xin), D(di), D(do))
    drv.d2h(out, do)
    return {"in": xin.tolist(), "out": out.tolist()}


def seq_scenario(drv, cubin, setup_args_fn, tid, ncalls, rng):
    m = drv.module(cubin)
    cl = clocks(rng, ncalls)
    dc = drv.upload(cl)
    ids = np.zeros(ncalls, np.int32)
    st = np.zeros(ncalls, np.int32)
    di, ds = drv.alloc(ids.nbytes), drv.alloc(st.nbytes)
    setup_args_fn(m)
    g, b = grid_for(tid)
    drv.launch(drv.fn(m, "fx_get_seq"), g, b, tid, ncalls, D(dc), D(di), D(ds))
    drv.d2h(ids, di)
    drv.d2h(st, ds)
    return cl, ids, st


def fx_rwbasic(drv):
    out = []
    rng = np.random.default_rng(102)
    for (tid, n, occ, seed) in [(3, 64, 0.5, 11), (70001, 32, 0.8, 21)]:
        T = 8192
        mp = int_map(T, occ, seed)
        dm = drv.upload(mp)
        cl, ids, st = seq_scenario(drv, "ref_rwbasic.cubin",
                                   lambda m: drv.launch(drv.fn(m, "fx_setup"), 1, 1, D(dm), T),
                                   tid, n, rng)
        fin = drv.d2h(np.zeros_like(mp), dm)
        out.append({"T": T, "occ": occ, "seed": seed, "tid": tid, "clocks": cl.tolist(),
                    "ids": ids.tolist(), "steps": st.tolist(), "final_map_sum": int(fin.sum()),
                    "final_changed": np.nonzero(fin != mp)[0].tolist()})
    return out


def fx_bitmap_seq(drv, cubin, scenarios, rng, with_crw=False):
    out = []
    for (tid, n, occ, seed) in scenarios:
        T = 8192
        L = T // 32
        w0 = oracle.bernoulli_bitmap(T, occ, seed)[:L].view(np.int32).copy()
        dw = drv.upload(w0)
        extra = {}
        if with_crw:
            lg = np.full(tid + 1, -1, np.int32)
            lb = np.zeros(tid + 1, np.int8)
            dlg, dlb = drv.upload(lg), drv.upload(lb)
            setup = lambda m: drv.launch(drv.fn(m, "fx_setup"), 1, 1, D(dw), L, T, D(dlg), D(dlb))
        else:
            setup = lambda m: drv.launch(drv.fn(m, "fx_setup"), 1, 1, D(dw), L, T)
        cl, ids, st = seq_scenario(drv, cubin, setup, tid, n, rng)
        fin = drv.d2h(np.zeros_like(w0), dw)
        if with_crw:
            extra["last_group"] = int(drv.d2h(np.zeros(tid + 1, np.int32), dlg)[tid])
            extra["last_bit"] = int(drv.d2h(np.zeros(tid + 1, np.int8), dlb)[tid])
        out.append(dict({"T": T, "L": L, "occ": occ, "seed": seed, "tid": tid, "clocks": cl.tolist(),
                         "ids": ids.tolist(), "steps": st.tolist(),
                         "final_words": fin.tolist()}, **extra))
    return out


def fx_warp_seq(drv, cubin, kernel, occ, seed, masks, npages, rng):
    T = 8192
    L = T // 32
    m = drv.module(cubin)
    w0 = oracle.bernoulli_bitmap(T, occ, seed)[:L].view(np.int32).copy()
    dw = drv.upload(w0)
    drv.launch(drv.fn(m, "fx_setup"), 1, 1, D(dw), L, T)
    n = len(masks)
    cl = clocks(rng, n)
    ms = np.array(masks, dtype=np.uint32)
    ids = np.full(n * 32, -7, np.int32)
    st = np.full(n * 32, -7, np.int32)
    dc, dm, di, ds = drv.upload(cl), drv.upload(ms), drv.upload(ids), drv.upload(st)
    if npages is None:
        drv.launch(drv.fn(m, kernel), 1, 32, n, D(dc), D(dm), D(di), D(ds))
    else:
        dn = drv.upload(np.array(npages, np.int32))
        drv.launch(drv.fn(m, kernel), 1, 32, n, D(dc), D(dm), D(dn), D(di), D(ds))
    drv.d2h(ids, di)
    drv.d2h(st, ds)
    fin = drv.d2h(np.zeros_like(w0), dw)
    r = {"T": T, "L": L, "occ": occ, "seed": seed, "clocks": cl.tolist(), "masks": ms.tolist(),
         "ids": ids.tolist(), "steps": st.tolist(), "final_words": fin.tolist()}
    if npages is not None:
        r["npages"] = list(npages)
    return r


def fx_find0range(drv):
    m = drv.module("ref_rwmalloc.cubin")
    rng = np.random.default_rng(105)
    vals = [0, -1, 1, 2, 3, 0x7fffffff, -2**31, 0x0000ffff, -65536, 0x00ff00ff, 0x0f0f0f0f, 6, 12, 0x80]
    xs = np.array(vals + list(rng.integers(-2**31, 2**31, size=200)) +
                  [int(v) for v in (rng.integers(0, 2**31, size=50) << 3)], dtype=np.int64)
    xs = (((xs + 2**31) % 2**32) - 2**31).astype(np.int32)
    n = len(xs)
    dx = drv.upload(xs)
    dl, dst, dxo = drv.alloc(4 * n), drv.alloc(4 * n), drv.alloc(4 * n)
    drv.launch(drv.fn(m, "fx_find0range"), (n + 255) // 256, 256, n, D(dx), D(dl), D(dst), D(dxo))
    return {"x": xs.tolist(), "len": drv.d2h(np.zeros(n, np.int32), dl).tolist(),
            "start": drv.d2h(np.zeros(n, np.int32), dst).tolist(),
            "x_out": drv.d2h(np.zeros(n, np.int32), dxo).tolist()}


def fx_pp(drv):
    m = drv.module("ref_pp.cubin")
    tp = drv.alloc(8)
    drv.launch(drv.fn(m, "fx_total_pages"), 1, 1, D(tp))
    T, BL = [int(v) for v in drv.d2h(np.zeros(2, np.int32), tp)]
    sc_map = int_map(T, 0.5, 16)
    d_sc = drv.upload(sc_map)
    d_dc = drv.upload(sc_map)
    d_arms = drv.alloc(4 * 1000000)
    words = oracle.bernoulli_bitmap(T, 0.4, 17)[:BL].view(np.int32).copy()
    d_words = drv.upload(words)
    d_nodes = drv.alloc(16 * T)
    drv.launch(drv.fn(m, "fx_setup"), 1, 1, D(d_sc), D(d_dc), D(d_arms), D(d_words), D(d_nodes))
    res = {"T": T, "bitmap_length": BL}
    # single clock
    n = 200
    di, ds = drv.alloc(4 * n), drv.alloc(4 * n)
    drv.launch(drv.fn(m, "fx_single_clock_seq"), 1, 1, n, D(di), D(ds))
    res["single_clock"] = {"occ": 0.5, "seed": 16, "ids": drv.d2h(np.zeros(n, np.int32), di).tolist(),
                           "steps": drv.d2h(np.zeros(n, np.int32), ds).tolist()}
    # distributed clock
    tid, clk, n = 7, 1234, 100
    da = drv.alloc(4)
    di, ds = drv.alloc(4 * n), drv.alloc(4 * n)
    drv.launch(drv.fn(m, "fx_dist_clock_seq"), 1, 32, tid, clk, n, D(da), D(di), D(ds))
    res["dist_clock"] = {"occ": 0.5, "seed": 16, "tid": tid, "clock": clk,
                         "arm0": int(drv.d2h(np.zeros(1, np.int32), da)[0]),
                         "ids": drv.d2h(np.zeros(n, np.int32), di).tolist(),
                         "steps": drv.d2h(np.zeros(n, np.int32), ds).tolist()}
    # getXPageRandomWalk_BM
    rng = np.random.default_rng(107)
    tid, X, n = 9, 3, 40
    cl = clocks(rng, n)
    dc = drv.upload(cl)
    di, ds = drv.alloc(4 * n), drv.alloc(4 * n)
    drv.launch(drv.fn(m, "fx_getxpage_seq"), 1, 32, tid, X, n, D(dc), D(di), D(ds))
    fin = drv.d2h(np.zeros_like(words), d_words)
    ch = np.nonzero(fin != words)[0]
    res["getxpage"] = {"occ": 0.4, "seed": 17, "tid": tid, "X": X, "clocks": cl.tolist(),
                       "ids": drv.d2h(np.zeros(n, np.int32), di).tolist(),
                       "steps": drv.d2h(np.zeros(n, np.int32), ds).tolist(),
                       "changed_idx": ch.tolist(), "changed_val": fin[ch].tolist()}
    # linked list (reference init kernel, then a get/free sequence)
    init = drv.fn(m, "_Z26initPagesLinkedList_kernelv")
    drv.launch(init, (T + 31) // 32, 32)
    ops = [-1] * 10 + [3, 7] + [-1] * 5 + [0] + [-1] * 3
    dops = drv.upload(np.array(ops, np.int32))
    do = drv.alloc(4 * len(ops))
    drv.launch(drv.fn(m, "fx_ll_seq"), 1, 1, len(ops), D(dops), D(do))
    res["linked_list"] = {"ops": ops, "out": drv.d2h(np.zeros(len(ops), np.int32), do).tolist()}
    return res


def main(out_dir=HERE):
    drv = Driver()
    rng = np.random.default_rng(2024)
    fixtures = {}
    fixtures["ref_lcg.json"] = fx_lcg(drv)
    fixtures["ref_rwbasic.json"] = fx_rwbasic(drv)
    drv.free_all()
    fixtures["ref_rwbm.json"] = fx_bitmap_seq(drv, "ref_rwbm.cubin", [(5, 64, 0.6, 12), (70003, 32, 0.9, 22)], rng)
    fixtures["ref_crw.json"] = fx_bitmap_seq(drv, "ref_crw.cubin", [(2, 64, 0.5, 14), (40000, 48, 0.85, 24)], rng,
                                             with_crw=True)
    drv.free_all()
    masks = [0xffffffff, 0xffffffff, 0x0000ffff, 0xaaaaaaaa, 0x1, 0x80000000, 0xffffffff, 0x00ff00ff,
             0xffffffff, 0x7fffffff, 0xffffffff, 0x3, 0xffffffff, 0xf0f0f0f0, 0xffffffff, 0xffffffff]
    fixtures["ref_collab.json"] = [fx_warp_seq(drv, "ref_collab.cubin", "fx_collab_seq", 0.7, 13, masks, None, rng),
                                   fx_warp_seq(drv, "ref_collab.cubin", "fx_collab_seq", 0.95, 23, masks[:8], None, rng)]
    drv.free_all()
    # getNPage retires every word it takes a run from (find0Range only reports
    # runs that start at bit 0 of a word), so a request with no such word left
    # would spin forever: keep requests (~40) far below the candidate words
    # (~230 words whose bit 0 is free at 10% occupancy).
    nmasks = [0xffffffff, 0x0000000f, 0x1, 0x3, 0x80000000]
    nrng = np.random.default_rng(106)
    npages = [int(v) for v in nrng.integers(1, 3, size=32 * len(nmasks))]
    fixtures["ref_getnpage.json"] = fx_warp_seq(drv, "ref_rwmalloc.cubin", "fx_getnpage_seq", 0.1, 15, nmasks,
                                                npages, rng)
    fixtures["ref_find0range.json"] = fx_find0range(drv)
    drv.free_all()
    fixtures["ref_parallelpage.json"] = fx_pp(drv)
    drv.free_all()
    os.makedirs(out_dir, exist_ok=True)
    for name, data in fixtures.items():
        with open(os.path.join(out_dir, name), "w") as f:
            json.dump(data, f, separators=(",", ":"))
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
