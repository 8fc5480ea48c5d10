"""Pins the oracle's restatements of the reference routines (orc_ref_*)
against outputs of the reference's own device code, run one thread / one
warp at a time with a fixed clock (fixtures from tests/golden/make_ref_fixtures.py)."""
import ctypes
import json
import os
from ctypes import byref, c_int32

import numpy as np
import pytest

from conftest import GOLDEN


def load(name):
    p = os.path.join(GOLDEN, name)
    if not os.path.exists(p):
        pytest.skip(f"{name} not generated yet")
    with open(p) as f:
        return json.load(f)


def int_map(orc, n_pages, occ, seed):
    w = orc.bernoulli_bitmap(n_pages, occ, seed)
    return np.unpackbits(w.view(np.uint8), bitorder="little")[:n_pages].astype(np.int32)


def bm_words(orc, T, occ, seed, L):
    return orc.bernoulli_bitmap(T, occ, seed)[:L].view(np.int32).copy()


def test_lcg(orc):
    fx = load("ref_lcg.json")
    for x, y in zip(fx["in"], fx["out"]):
        assert orc.lcg(x) == y, (x, y)


def test_random_walk_basic(orc):
    L = orc.lib()
    for sc in load("ref_rwbasic.json"):
        T = sc["T"]
        m = int_map(orc, T, sc["occ"], sc["seed"])
        m0 = m.copy()
        st = c_int32()
        for k, clk in enumerate(sc["clocks"]):
            pid = L.orc_ref_rwbasic_get(orc.P(m), T, sc["tid"], clk, byref(st))
            assert pid == sc["ids"][k] and st.value == sc["steps"][k], (k, pid, st.value)
        assert int(m.sum()) == sc["final_map_sum"]
        assert np.nonzero(m != m0)[0].tolist() == sc["final_changed"]


def test_random_walk_bm(orc):
    L = orc.lib()
    for sc in load("ref_rwbm.json"):
        w = bm_words(orc, sc["T"], sc["occ"], sc["seed"], sc["L"])
        st = c_int32()
        for k, clk in enumerate(sc["clocks"]):
            pid = L.orc_ref_rwbm_get(orc.P(w), sc["L"], sc["tid"], clk, byref(st))
            assert pid == sc["ids"][k] and st.value == sc["steps"][k], (k, pid, st.value)
        assert w.tolist() == sc["final_words"]


def test_clustered_walk_bm(orc):
    L = orc.lib()
    for sc in load("ref_crw.json"):
        w = bm_words(orc, sc["T"], sc["occ"], sc["seed"], sc["L"])
        tid = sc["tid"]
        lg = np.full(tid + 1, -1, np.int32)
        lb = np.zeros(tid + 1, np.int8)
        st = c_int32()
        for k, clk in enumerate(sc["clocks"]):
            pid = L.orc_ref_crw_get(orc.P(w), sc["L"], orc.P(lg), orc.P(lb), tid, clk, byref(st))
            assert pid == sc["ids"][k] and st.value == sc["steps"][k], (k, pid, st.value)
        assert w.tolist() == sc["final_words"]
        assert int(lg[tid]) == sc["last_group"] and int(lb[tid]) == sc["last_bit"]


def test_collab_rw_bm(orc):
    L = orc.lib()
    for sc in load("ref_collab.json"):
        w = bm_words(orc, sc["T"], sc["occ"], sc["seed"], sc["L"])
        ids = np.zeros(32, np.int32)
        st = np.zeros(32, np.int32)
        for k, (clk, mask) in enumerate(zip(sc["clocks"], sc["masks"])):
            ids[:] = -7
            st[:] = -7
            L.orc_ref_collab_get(orc.P(w), sc["L"], mask, 0, clk, orc.P(ids), orc.P(st))
            assert ids.tolist() == sc["ids"][32 * k:32 * k + 32], k
            assert st.tolist() == sc["steps"][32 * k:32 * k + 32], k
        assert w.tolist() == sc["final_words"]


def test_find0range(orc):
    fx = load("ref_find0range.json")
    L = orc.lib()
    for x, ln, stt, xo in zip(fx["x"], fx["len"], fx["start"], fx["x_out"]):
        xv, sv = c_int32(x), c_int32(-99)
        got = L.orc_ref_find0range(byref(xv), byref(sv))
        assert (got, sv.value, xv.value) == (ln, stt, xo), x


def test_getnpage(orc):
    sc = load("ref_getnpage.json")
    L = orc.lib()
    w = bm_words(orc, sc["T"], sc["occ"], sc["seed"], sc["L"])
    npg = np.array(sc["npages"], np.int32)
    ids = np.zeros(32, np.int32)
    st = np.zeros(32, np.int32)
    for k, (clk, mask) in enumerate(zip(sc["clocks"], sc["masks"])):
        ids[:] = -7
        st[:] = -7
        n = npg[32 * k:32 * k + 32].copy()
        L.orc_ref_getnpage(orc.P(w), sc["L"], sc["T"], mask, 0, 32, orc.P(n), clk, orc.P(ids), orc.P(st))
        assert ids.tolist() == sc["ids"][32 * k:32 * k + 32], k
        assert st.tolist() == sc["steps"][32 * k:32 * k + 32], k
    assert w.tolist() == sc["final_words"]


def test_parallel_page_clocks_xpage_and_list(orc):
    fx = load("ref_parallelpage.json")
    L = orc.lib()
    T, BL = fx["T"], fx["bitmap_length"]
    full = int_map(orc, T, 0.5, 16)
    # single clock: one shared arm from 0
    sc = fx["single_clock"]
    m = full.copy()
    arm = c_int32(0)
    st = c_int32()
    for k in range(len(sc["ids"])):
        pid = L.orc_ref_single_clock(orc.P(m), T, byref(arm), byref(st))
        assert (pid, st.value) == (sc["ids"][k], sc["steps"][k]), k
    # distributed clock: arm randomised from (tid, clock), then linear probe
    dc = fx["dist_clock"]
    assert L.orc_ref_dist_clock_arm(dc["tid"], dc["clock"], T) == dc["arm0"]
    m = full.copy()
    arms = np.zeros(dc["tid"] + 1, np.int32)
    arms[dc["tid"]] = dc["arm0"]
    for k in range(len(dc["ids"])):
        pid = L.orc_ref_dist_clock(orc.P(m), T, orc.P(arms), dc["tid"], byref(st))
        assert (pid, st.value) == (dc["ids"][k], dc["steps"][k]), k
    # getXPageRandomWalk_BM
    gx = fx["getxpage"]
    w = orc.bernoulli_bitmap(T, gx["occ"], gx["seed"])[:BL].view(np.int32).copy()
    w0 = w.copy()
    for k, clk in enumerate(gx["clocks"]):
        pid = L.orc_ref_getxpage_rwbm(orc.P(w), BL, gx["X"], gx["tid"], clk, byref(st))
        assert (pid, st.value) == (gx["ids"][k], gx["steps"][k]), k
    ch = np.nonzero(w != w0)[0]
    assert ch.tolist() == gx["changed_idx"] and w[ch].tolist() == gx["changed_val"]
    # linked list: head pops in node order, frees append at the tail
    ll = fx["linked_list"]
    nxt, tail, out = 0, [], []
    for op in ll["ops"]:
        if op < 0:
            if nxt < T:
                out.append(nxt)
                nxt += 1
            else:
                out.append(tail.pop(0))
        else:
            tail.append(op)
            out.append(-1)
    assert out == ll["out"]
