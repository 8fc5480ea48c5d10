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
    ("orc_walk_span", c_int32, [_P, c_uint32, c_uint32, c_int32, c_uint32, POINTER(c_int32)]),
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
    ("orc_cpu_claim_write_free", c_double, [_P, c_uint64, _P, c_uint32, c_uint32, c_uint64, c_uint32, c_int,
                                            c_uint32, c_uint32, POINTER(c_uint64), POINTER(c_uint64)]),
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


def replay_spans(words, n_pages, npages, S, max_steps=4096):
    """Serial replay of pbm_alloc_spans: request r claims npages[r] pages
    (runs may cross words) with seed orc_seed(S, r)."""
    L = lib()
    n = len(npages)
    ids = np.full(n, -1, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    st = c_int32()
    for r in range(n):
        k = int(npages[r])
        if 1 <= k <= 65536:
            ids[r] = L.orc_walk_span(P(words), n_pages, k, L.orc_seed(S, r), max_steps, ctypes.byref(st))
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


def cpu_claim_write_free(words, n_pages, page_size, payload_bytes, n, seed, reps, threads=None, max_steps=4096):
    """std::atomic host replay of claim/write/free; returns (seconds, ok, steps, threads)."""
    import numpy as np

    L = lib()
    if threads is None:
        threads = L.orc_hw_threads()
    pages = np.zeros(int(n_pages) * int(page_size), dtype=np.uint8)
    ok, st = c_uint64(), c_uint64()
    secs = L.orc_cpu_claim_write_free(P(words), n_pages, P(pages), page_size, payload_bytes, n, seed, threads,
                                      reps, max_steps, ctypes.byref(ok), ctypes.byref(st))
    return secs, ok.value, st.value, threads


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


class BmT(Structure):
    _fields_ = [("page_table", c_void_p), ("frame_state", c_void_p), ("ref", c_void_p), ("arms", c_void_p),
                ("hand", c_uint64), ("n_logical", c_uint32), ("n_frames", c_uint32), ("max_sweep", c_uint32),
                ("n_arms", c_uint32), ("dist", c_int), ("hits", c_uint64), ("misses", c_uint64),
                ("evictions", c_uint64), ("failures", c_uint64), ("unpins", c_uint64), ("bad_unpins", c_uint64)]


class BufMgrReplay:
    """Single-thread replay of the CLOCK buffer manager (oracle_bufmgr.c)."""

    def __init__(self, n_logical, n_frames, max_sweep=0, n_arms=1, dist=0):
        L = lib()
        L.orc_bm_init.argtypes = [ctypes.POINTER(BmT), c_uint32, c_uint32, c_uint32, c_uint32, c_int]
        L.orc_bm_free.argtypes = [ctypes.POINTER(BmT)]
        L.orc_bm_round.argtypes = [ctypes.POINTER(BmT), _P, _P, c_uint32, _P, c_uint32, c_uint32, _P]
        self.L = L
        self.b = BmT()
        L.orc_bm_init(ctypes.byref(self.b), n_logical, n_frames, max_sweep, n_arms, dist)

    def round(self, frames_of, release_idx, pages, slot0):
        frames_out = np.empty(len(pages), dtype=np.int32)
        self.L.orc_bm_round(ctypes.byref(self.b), P(frames_of), P(release_idx), len(release_idx),
                            P(pages), len(pages), slot0, P(frames_out))
        return frames_out

    def counters(self):
        b = self.b
        return dict(hits=b.hits, misses=b.misses, evictions=b.evictions, failures=b.failures,
                    unpins=b.unpins, bad_unpins=b.bad_unpins)

    def close(self):
        if self.b.page_table:
            self.L.orc_bm_free(ctypes.byref(self.b))


class MallocT(Structure):
    _fields_ = [("words", c_void_p), ("n_pages", c_uint32), ("page_shift", c_uint32), ("start_of", c_void_p),
                ("live", c_void_p), ("len_of", c_void_p)]


class MallocReplay:
    """Sequential replay of the size-classed malloc (oracle_malloc.c) on a
    bitmap the caller owns (mutated in place)."""

    def __init__(self, words, n_pages, page_shift):
        L = lib()
        L.orc_malloc_group.argtypes = [ctypes.POINTER(MallocT), _P, c_int, c_int32, _P, c_uint32, _P, _P]
        L.orc_malloc_free.argtypes = [ctypes.POINTER(MallocT), ctypes.c_int64]
        L.orc_malloc_free.restype = c_int
        self.L = L
        self.words = words
        self.start_of = np.full(n_pages, -1, dtype=np.int32)
        self.live = np.zeros(n_pages, dtype=np.int32)
        self.len_of = np.zeros(n_pages, dtype=np.uint8)
        self.m = MallocT(P(words), n_pages, page_shift, P(self.start_of), P(self.live), P(self.len_of))

    def group(self, sizes, seed_small, seed_own, max_steps=4096):
        sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        seed_own = np.ascontiguousarray(seed_own, dtype=np.int32)
        offs = np.zeros(len(sizes), dtype=np.int64)
        steps = np.zeros(len(sizes), dtype=np.int32)
        self.L.orc_malloc_group(ctypes.byref(self.m), P(sizes), len(sizes), seed_small, P(seed_own), max_steps,
                                P(offs), P(steps))
        return offs, steps

    def free(self, offset):
        return self.L.orc_malloc_free(ctypes.byref(self.m), int(offset))


class QMallocT(Structure):
    _fields_ = [("words", c_void_p), ("n_pages", c_uint32), ("page_shift", c_uint32), ("cap", c_uint32),
                ("class_of", c_void_p), ("ring", c_void_p), ("head", c_uint64 * 13), ("tail", c_uint64 * 13),
                ("avail", c_int64 * 13), ("space", c_int64 * 13), ("chunks", c_uint64), ("overflow", c_uint64),
                ("bad_frees", c_uint64)]


class QMallocReplay:
    """Sequential replay of the queue-based size classes (oracle_qmalloc.c)
    on a bitmap the caller owns (mutated in place)."""

    def __init__(self, words, n_pages, page_shift, cap=1 << 12):
        L = lib()
        L.orc_qmalloc_init.argtypes = [ctypes.POINTER(QMallocT), _P, c_uint32, c_uint32, c_uint32]
        L.orc_qmalloc_init.restype = c_int
        L.orc_qmalloc_destroy.argtypes = [ctypes.POINTER(QMallocT)]
        L.orc_qmalloc_group.argtypes = [ctypes.POINTER(QMallocT), _P, c_int, _P, c_uint32, _P, _P]
        L.orc_qmalloc_free_group.argtypes = [ctypes.POINTER(QMallocT), _P, c_int, _P]
        self.L = L
        self.words = words
        self.q = QMallocT()
        if L.orc_qmalloc_init(ctypes.byref(self.q), P(words), n_pages, page_shift, cap) != 0:
            raise MemoryError("orc_qmalloc_init")

    def group(self, sizes, seed_own, max_steps=4096):
        sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        seed_own = np.ascontiguousarray(seed_own, dtype=np.int32)
        offs = np.zeros(len(sizes), dtype=np.int64)
        steps = np.zeros(len(sizes), dtype=np.int32)
        self.L.orc_qmalloc_group(ctypes.byref(self.q), P(sizes), len(sizes), P(seed_own), max_steps, P(offs),
                                 P(steps))
        return offs, steps

    def free(self, offsets):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        ok = np.zeros(len(offsets), dtype=np.int32)
        self.L.orc_qmalloc_free_group(ctypes.byref(self.q), P(offsets), len(offsets), P(ok))
        return ok

    def queued(self):
        return [int(self.q.avail[c]) for c in range(13)]

    def close(self):
        if self.q.ring:
            self.L.orc_qmalloc_destroy(ctypes.byref(self.q))
