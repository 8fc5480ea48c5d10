"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, always as the checker or as the
timed CPU baseline -- never on the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, Structure, c_double, c_int, c_int8, c_int16, c_int32, c_int64, c_uint8, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class CheckT(Structure):
    _fields_ = [("n_ok", c_int64), ("n_failed", c_int64), ("n_out_of_range", c_int64),
                ("n_duplicates", c_int64), ("n_not_marked", c_int64), ("n_prefilled", c_int64),
                ("used_after", c_int64)]


_P = c_void_p
SIGS = [
    ("orc_lcg", c_int32, [c_int32]),
    ("orc_idx_mod", c_uint32, [c_int32, c_uint32]),
    ("orc_idx_hi", c_uint32, [c_int32, c_uint32]),
    ("orc_seed", c_int32, [c_uint32, c_uint32]),
    ("orc_hash64", c_uint64, [c_uint64, c_uint64]),
    ("orc_shl32", c_uint32, [c_uint32, c_uint32]),
    ("orc_words_for", ctypes.c_size_t, [c_uint64, c_int]),
    ("orc_thresh53", c_uint64, [c_double]),
    ("orc_prefill_bernoulli", None, [_P, c_uint64, c_uint64, c_uint64]),
    ("orc_set_padding", None, [_P, c_uint64]),
    ("orc_used_pages", c_uint64, [_P, c_uint64]),
    ("orc_check_alloc", None, [_P, _P, c_uint64, _P, c_int64, POINTER(CheckT)]),
    ("orc_walk_page", c_int32, [_P, c_uint32, c_int32, c_uint32, POINTER(c_int32)]),
    ("orc_walk_word", c_int32, [_P, c_uint32, c_int, c_int32, c_uint32, POINTER(c_int32)]),
    ("orc_walk_collab", None, [_P, c_uint32, c_int, c_int, _P, c_int32, c_uint32, c_uint32, _P, _P]),
    ("orc_walk_crw", c_int32, [_P, c_uint32, POINTER(c_int32), c_int32, c_uint32, POINTER(c_int32)]),
    ("orc_single_clock", c_int32, [_P, c_uint32, POINTER(c_uint64), c_uint32, POINTER(c_int32)]),
    ("orc_dist_clock", c_int32, [_P, c_uint32, POINTER(c_uint32), c_uint32, POINTER(c_int32)]),
    ("orc_dist_clock_arm0", c_uint32, [c_uint32, c_uint32, c_uint32]),
    ("orc_walk_run", c_int32, [_P, c_uint32, c_uint32, c_int32, c_uint32, POINTER(c_int32)]),
    ("orc_free_run", None, [_P, c_int32, c_uint32]),
    ("orc_free_page", None, [_P, c_int32]),
    ("orc_ref_rwbasic_get", c_int32, [_P, c_int32, c_int32, c_int16, POINTER(c_int32)]),
    ("orc_ref_rwbm_get", c_int32, [_P, c_int32, c_int32, c_int16, POINTER(c_int32)]),
    ("orc_ref_collab_get", None, [_P, c_int32, c_uint32, c_int32, c_int16, _P, _P]),
    ("orc_ref_crw_get", c_int32, [_P, c_int32, _P, _P, c_int32, c_int16, POINTER(c_int32)]),
    ("orc_ref_find0range", c_int32, [POINTER(c_int32), POINTER(c_int32)]),
    ("orc_ref_getnpage", None, [_P, c_int32, c_int32, c_uint32, c_int32, c_int32, _P, c_int16, _P, _P]),
    ("orc_ref_getxpage_rwbm", c_int32, [_P, c_int32, c_int32, c_int32, c_int16, POINTER(c_int32)]),
    ("orc_ref_single_clock", c_int32, [_P, c_int32, POINTER(c_int32), POINTER(c_int32)]),
    ("orc_ref_dist_clock", c_int32, [_P, c_int32, _P, c_int32, POINTER(c_int32)]),
    ("orc_ref_dist_clock_arm", c_int32, [c_int32, c_int16, c_int32]),
    ("orc_cpu_churn", c_double, [_P, c_uint64, _P, c_uint64, c_uint64, c_uint32, c_int, c_int, c_uint32,
                                 POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64)]),
    ("orc_hw_threads", c_int, []),
]


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGS:
            try:
                f = getattr(L, name)
            except AttributeError:
                continue
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def P(a: np.ndarray):
    return a.ctypes.data


# ---- convenience wrappers -------------------------------------------------------

def words_for(n_pages, word_bits=32):
    return int(lib().orc_words_for(n_pages, word_bits))


def bitmap_words(n_pages):
    """storage in 32-bit words (padded to a 64-bit boundary, like the device bitmap)"""
    return ((n_pages + 63) // 64) * 2


def empty_bitmap(n_pages):
    w = np.zeros(bitmap_words(n_pages), dtype=np.uint32)
    lib().orc_set_padding(P(w), n_pages)
    return w


def bernoulli_bitmap(n_pages, occ, seed):
    w = np.zeros(bitmap_words(n_pages), dtype=np.uint32)
    L = lib()
    L.orc_prefill_bernoulli(P(w), n_pages, L.orc_thresh53(occ), seed)
    return w


def used_pages(words, n_pages):
    return int(lib().orc_used_pages(P(words), n_pages))


def seed(S, r):
    return int(lib().orc_seed(S, r))


def lcg(x):
    return int(lib().orc_lcg(x))


def check_alloc(after, before, n_pages, ids):
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    out = CheckT()
    lib().orc_check_alloc(P(after), P(before) if before is not None else None, n_pages, P(ids),
                          len(ids), ctypes.byref(out))
    return out


def replay_alloc(words, n_pages, strategy, n, S, word_bits=32, collab_width=32, stride=1,
                 max_steps=4096, cursors=None, arms=None, arm=None):
    """Sequential replay of n single-page requests with the product's
    semantics (strategy ids as in include/pbm.h).  Mutates `words`."""
    L = lib()
    ids = np.full(n, -1, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    st = c_int32()
    if strategy == 2:  # collaborative walk: groups of collab_width consecutive requests
        W = collab_width
        need = np.ones(W, dtype=np.uint8)
        gid = np.full(W, -1, dtype=np.int32)
        gst = np.zeros(W, dtype=np.int32)
        for base in range(0, n, W):
            k = min(W, n - base)
            need[:] = 0
            need[:k] = 1
            gid[:] = -1
            L.orc_walk_collab(P(words), n_pages, word_bits, W, P(need), L.orc_seed(S, base), stride,
                              max_steps, P(gid), P(gst))
            ids[base:base + k] = gid[:k]
            steps[base:base + k] = gst[:k]
        return ids, steps
    for r in range(n):
        s0 = L.orc_seed(S, r)
        if strategy == 0:
            ids[r] = L.orc_walk_page(P(words), n_pages, s0, max_steps, ctypes.byref(st))
        elif strategy == 1:
            ids[r] = L.orc_walk_word(P(words), n_pages, word_bits, s0, max_steps, ctypes.byref(st))
        elif strategy == 3:
            c = c_int32(int(cursors[r % len(cursors)]))
            ids[r] = L.orc_walk_crw(P(words), n_pages, ctypes.byref(c), s0, max_steps, ctypes.byref(st))
            cursors[r % len(cursors)] = c.value
        elif strategy == 5:
            a = c_uint64(int(arm[0]))
            ids[r] = L.orc_single_clock(P(words), n_pages, ctypes.byref(a), max_steps, ctypes.byref(st))
            arm[0] = a.value
        elif strategy == 6:
            a = c_uint32(int(arms[r % len(arms)]))
            ids[r] = L.orc_dist_clock(P(words), n_pages, ctypes.byref(a), max_steps, ctypes.byref(st))
            arms[r % len(arms)] = a.value
        else:
            raise ValueError(strategy)
        steps[r] = st.value
    return ids, steps


def replay_runs(words, n_pages, npages, S, max_steps=4096):
    L = lib()
    n = len(npages)
    ids = np.full(n, -1, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    st = c_int32()
    for r in range(n):
        k = int(npages[r])
        if 1 <= k <= 32:
            ids[r] = L.orc_walk_run(P(words), n_pages, k, L.orc_seed(S, r), max_steps, ctypes.byref(st))
            steps[r] = st.value
    return ids, steps


def cpu_churn(words, n_pages, held, n_pairs, seed, threads=None, walk=1, max_steps=4096):
    """std::atomic host replay of alloc+free pairs; returns (seconds, ok, fail, steps)."""
    L = lib()
    if threads is None:
        threads = L.orc_hw_threads()
    ok, fail, st = c_uint64(), c_uint64(), c_uint64()
    secs = L.orc_cpu_churn(P(words), n_pages, P(held), len(held), n_pairs, seed, threads, walk, max_steps,
                           ctypes.byref(ok), ctypes.byref(fail), ctypes.byref(st))
    return secs, ok.value, fail.value, st.value, threads


def fifo_replay(free_pages_sorted, ops):
    """FIFO free list replay: ops = list of ('get', None) / ('put', id); returns gets' ids."""
    from collections import deque
    q = deque(int(x) for x in free_pages_sorted)
    out = []
    for op, arg in ops:
        if op == "get":
            out.append(q.popleft() if q else -1)
        else:
            q.append(int(arg))
    return out
