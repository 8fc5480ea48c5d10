"""ctypes binding of libpbm.so (the C ABI declared in include/pbm.h).

Mirrors the reference's host-side interface for the page allocator --
initMemoryManagement / resetMemoryManager / getFreePagePercentage /
prefillBuffer (source/RandomWalkBasic_BM.cuh:15-21) -- on an explicit pool
handle, plus the batch, graph and check entry points.  Device buffers are
passed as raw device pointers (ints) or as objects with ``data_ptr()``
(e.g. torch tensors); streams as raw cudaStream_t values (0 = default).

There is no CPU fallback: if libpbm.so is missing or fails to load, the
import raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, byref, c_char_p, c_double, c_int, c_int32,
                    c_int64, c_size_t, c_uint32, c_uint64, c_void_p)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpbm.so")

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_EXHAUSTED = -4
ERR_TIMEOUT = -5
ERR_UNSUPPORTED = -6
ERR_CORRUPT = -7

RANDOM_WALK = 0
RANDOM_WALK_BM = 1
COLLAB_RW_BM = 2
CLUSTERED_RW_BM = 3
LINKED_LIST = 4
SINGLE_CLOCK = 5
DIST_CLOCK = 6
STRATEGY_NAMES = {
    RANDOM_WALK: "RandomWalk", RANDOM_WALK_BM: "RandomWalk_BM", COLLAB_RW_BM: "CollabRW_BM",
    CLUSTERED_RW_BM: "ClusteredRandomWalk_BM", LINKED_LIST: "LinkedList",
    SINGLE_CLOCK: "SingleClock", DIST_CLOCK: "DistClock",
}

OP_ALLOC, OP_FREE, OP_SWAP, OP_MALLOC, OP_MFREE = 0, 1, 2, 3, 4
LAUNCH_PLAIN, LAUNCH_PERSISTENT, LAUNCH_SERIAL = 0, 1, 2
MAX_INLINE_GROUPS = 256           # PBM_MAX_INLINE_GROUPS
POOL_MATERIALIZE = 1


class PoolConfig(Structure):
    _fields_ = [("n_pages", c_uint64), ("page_size", c_uint32), ("flags", c_uint32),
                ("max_slots", c_uint32), ("reserved", c_uint32)]


class WalkConfig(Structure):
    _fields_ = [("strategy", c_int32), ("word_bits", c_int32), ("collab_width", c_int32),
                ("stride", c_uint32), ("max_steps", c_uint32), ("block_size", c_int32),
                ("blocks_per_sm", c_int32), ("free_merge", c_int32), ("fail_fast", c_int32),
                ("reserved", c_int32)]


class Group(Structure):
    _fields_ = [("op", c_int32), ("count", c_uint32), ("offset", c_uint64)]


class Stats(Structure):
    _fields_ = [("successes", c_uint64), ("failures", c_uint64), ("steps", c_uint64),
                ("frees", c_uint64)]


class CheckResult(Structure):
    _fields_ = [("n_ok", c_int64), ("n_failed", c_int64), ("n_out_of_range", c_int64),
                ("n_duplicates", c_int64), ("n_not_marked", c_int64), ("used_pages", c_int64)]


class DeviceState(Structure):
    _fields_ = [("words", c_void_p), ("base", c_void_p), ("n_pages", c_uint64), ("page_size", c_uint32),
                ("n_words32", c_uint32), ("n_words64", c_uint32), ("max_slots", c_uint32),
                ("cursors", c_void_p), ("arms", c_void_p), ("single_arm", c_void_p),
                ("fifo_state", c_void_p), ("fifo_ring", c_void_p), ("stats", c_void_p)]


BM_SINGLE_CLOCK, BM_DIST_CLOCK = 0, 1


class TuneResult(Structure):
    _fields_ = [("cfg", WalkConfig), ("ms_per_batch", ctypes.c_float), ("ms_mean", ctypes.c_float),
                ("ops_per_s", c_double)]


class BufMgrConfig(Structure):
    _fields_ = [("n_logical", c_uint64), ("n_frames", c_uint32), ("frame_size", c_uint32),
                ("policy", c_int32), ("n_arms", c_uint32), ("max_sweep", c_uint32), ("reserved", c_uint32)]


class BufMgrCounters(Structure):
    _fields_ = [("hits", c_uint64), ("misses", c_uint64), ("evictions", c_uint64), ("failures", c_uint64),
                ("unpins", c_uint64), ("bad_unpins", c_uint64), ("timeouts", c_uint64)]


class BufMgrCheck(Structure):
    _fields_ = [("resident", c_uint64), ("mapped_frames", c_uint64), ("mismatches", c_uint64),
                ("loading", c_uint64), ("pins", c_uint64)]


REQ_ALLOC, REQ_FREE, REQ_FETCH = 0, 1, 2


class Request(Structure):
    _fields_ = [("arrival_s", c_double), ("tenant", c_uint32), ("op", c_int32), ("count", c_uint32),
                ("reserved", c_uint32)]


class RequestResult(Structure):
    _fields_ = [("admit_s", c_double), ("launch_s", c_double), ("done_s", c_double), ("latency_s", c_double),
                ("pages", c_uint64), ("status", c_int32), ("reserved", c_uint32)]


class ServerConfig(Structure):
    _fields_ = [("n_tenants", c_uint32), ("ring_pages", c_uint32), ("n_streams", c_uint32),
                ("max_batch_requests", c_uint32), ("max_fetch_pages", c_uint32), ("tenant_quota_pages", c_uint32),
                ("max_occupancy", c_double), ("drain_timeout_s", c_double), ("walk", WalkConfig)]


class MonitorSample(Structure):
    _fields_ = [("t_s", c_double), ("used_pages", c_uint64), ("free_fraction", c_double), ("stats", Stats)]


class ServerReport(Structure):
    _fields_ = [("requests", c_uint64), ("completed", c_uint64), ("rejected", c_uint64), ("pages", c_uint64),
                ("batches", c_uint64), ("max_in_flight", c_uint64), ("wall_s", c_double), ("p50_s", c_double),
                ("p99_s", c_double), ("mean_batch_requests", c_double), ("waited", c_uint64),
                ("stranded", c_uint64)]


# (name, restype, argtypes) -- every entry point of include/pbm.h
SIGNATURES = [
    ("pbm_pool_create", c_int, [POINTER(PoolConfig), POINTER(c_void_p)]),
    ("pbm_pool_destroy", c_int, [c_void_p]),
    ("pbm_pool_info", c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint32), POINTER(c_void_p),
                              POINTER(c_size_t), POINTER(c_void_p)]),
    ("pbm_pool_reset", c_int, [c_void_p, c_void_p]),
    ("pbm_pool_prefill_bernoulli", c_int, [c_void_p, c_double, c_uint64, c_void_p]),
    ("pbm_pool_used", c_int, [c_void_p, POINTER(c_uint64), c_void_p]),
    ("pbm_pool_read_bitmap", c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    ("pbm_pool_write_bitmap", c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    ("pbm_pool_stats", c_int, [c_void_p, POINTER(Stats), c_void_p]),
    ("pbm_pool_device_state", c_int, [c_void_p, c_int, POINTER(DeviceState), c_void_p]),
    ("pbm_alloc", c_int, [c_void_p, POINTER(WalkConfig), c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]),
    ("pbm_alloc_serial", c_int, [c_void_p, POINTER(WalkConfig), c_uint32, c_uint32, c_void_p, c_void_p,
                                 c_void_p]),
    ("pbm_free", c_int, [c_void_p, POINTER(WalkConfig), c_uint32, c_void_p, c_void_p]),
    ("pbm_alloc_runs", c_int, [c_void_p, c_uint32, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p,
                               c_void_p]),
    ("pbm_alloc_runs_serial", c_int, [c_void_p, c_uint32, c_void_p, c_uint32, c_uint32, c_void_p,
                                      c_void_p, c_void_p]),
    ("pbm_alloc_spans", c_int, [c_void_p, c_uint32, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p,
                                c_void_p]),
    ("pbm_alloc_spans_serial", c_int, [c_void_p, c_uint32, c_void_p, c_uint32, c_uint32, c_void_p,
                                       c_void_p, c_void_p]),
    ("pbm_free_runs", c_int, [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]),
    ("pbm_claim_write_free", c_int, [c_void_p, c_uint32, c_uint32, c_uint32, c_int, c_uint32, c_void_p,
                                     c_void_p, c_void_p]),
    ("pbm_gather_pages", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]),
    ("pbm_batch_launch", c_int, [c_void_p, POINTER(WalkConfig), c_void_p, POINTER(Group), c_uint32,
                                 c_void_p, c_uint64, c_uint32, c_void_p, c_int, c_void_p]),
    ("pbm_batch_launch_results", c_int, [c_void_p, POINTER(WalkConfig), c_void_p, POINTER(Group), c_uint32,
                                         c_void_p, c_uint64, c_uint32, c_void_p, c_void_p, c_int, c_void_p]),
    ("pbm_batch_graph_create", c_int, [c_void_p, POINTER(WalkConfig), c_void_p, c_uint32, c_uint32,
                                       c_void_p, c_uint64, c_uint32, c_void_p, POINTER(c_void_p)]),
    ("pbm_batch_graph_create_results", c_int, [c_void_p, POINTER(WalkConfig), c_void_p, c_uint32, c_uint32,
                                               c_void_p, c_uint64, c_uint32, c_void_p, c_void_p, POINTER(c_void_p)]),
    ("pbm_graph_replay", c_int, [c_void_p, c_void_p]),
    ("pbm_graph_set_step", c_int, [c_void_p, c_uint32, c_void_p]),
    ("pbm_graph_destroy", c_int, [c_void_p]),
    ("pbm_check_ids", c_int, [c_void_p, c_void_p, c_uint32, POINTER(CheckResult), c_void_p]),
    ("pbm_check_ids_noalloc", c_int, [c_void_p, c_uint64, c_void_p, c_uint32, POINTER(CheckResult),
                                      c_void_p]),
    ("pbm_atomic_ceiling", c_int, [c_uint32, c_uint32, c_uint32, c_int, c_int, POINTER(c_double),
                                   POINTER(c_double)]),
    ("pbm_malloc_init", c_int, [c_void_p]),
    ("pbm_malloc_release", c_int, [c_void_p]),
    ("pbm_malloc_tables", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p)]),
    ("pbm_malloc_batch", c_int, [c_void_p, c_void_p, POINTER(Group), c_uint32, c_void_p, c_void_p, c_uint64,
                                 c_uint32, c_uint32, c_int, c_void_p]),
    ("pbm_malloc_graph_create", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_uint64,
                                        c_uint32, c_uint32, c_void_p, POINTER(c_void_p)]),
    ("pbm_malloc_counts", c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64), c_void_p]),
    ("pbm_qmalloc_init", c_int, [c_void_p, c_uint32]),
    ("pbm_qmalloc_release", c_int, [c_void_p]),
    ("pbm_qmalloc_batch", c_int, [c_void_p, c_void_p, POINTER(Group), c_uint32, c_void_p, c_void_p, c_uint64,
                                  c_uint32, c_uint32, c_int, c_void_p]),
    ("pbm_qmalloc_graph_create", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_uint64,
                                         c_uint32, c_uint32, c_void_p, POINTER(c_void_p)]),
    ("pbm_qmalloc_counts", c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64),
                                   POINTER(c_uint64), POINTER(c_uint64), c_void_p]),
    ("pbm_autotune", c_int, [c_void_p, c_void_p, c_uint32, c_uint64, c_void_p, c_uint64, c_uint32, c_int,
                             c_uint32, POINTER(TuneResult), c_uint32, POINTER(c_uint32), c_void_p]),
    ("pbm_bufmgr_create", c_int, [POINTER(BufMgrConfig), c_void_p, POINTER(c_void_p)]),
    ("pbm_bufmgr_destroy", c_int, [c_void_p]),
    ("pbm_bufmgr_reset", c_int, [c_void_p, c_void_p]),
    ("pbm_bufmgr_round", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_uint32,
                                 c_void_p, c_int, c_void_p]),
    ("pbm_bufmgr_round_pages", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_uint32,
                                       c_void_p, c_void_p, c_int, c_void_p]),
    ("pbm_bufmgr_stats", c_int, [c_void_p, POINTER(BufMgrCounters), c_void_p]),
    ("pbm_bufmgr_check", c_int, [c_void_p, POINTER(BufMgrCheck), c_void_p]),
    ("pbm_bufmgr_frames", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_size_t)]),
    ("pbm_bufmgr_gather", c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]),
    ("pbm_bufmgr_read_tables", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("pbm_server_create", c_int, [c_void_p, c_void_p, c_void_p, c_uint64, POINTER(ServerConfig),
                                  POINTER(c_void_p)]),
    ("pbm_server_run", c_int, [c_void_p, POINTER(Request), c_uint64, POINTER(RequestResult), POINTER(ServerReport)]),
    ("pbm_server_tenant_pages", c_int, [c_void_p, c_uint32, c_void_p, c_uint64, POINTER(c_uint64)]),
    ("pbm_server_destroy", c_int, [c_void_p]),
    ("pbm_monitor_start", c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_void_p)]),
    ("pbm_monitor_samples", c_int, [c_void_p, POINTER(MonitorSample), c_uint32, POINTER(c_uint32)]),
    ("pbm_monitor_stop", c_int, [c_void_p]),
    ("pbm_version", c_char_p, []),
    ("pbm_kernel_launches", c_uint64, []),
    ("pbm_device_sm_count", c_int, [POINTER(c_int)]),
]


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise RuntimeError(f"libpbm.so not built at {path}; run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


class PbmError(RuntimeError):
    def __init__(self, fn, rc):
        super().__init__(f"{fn} returned {rc}")
        self.rc = rc


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _check(fn, rc, allow=()):
    if rc != OK and rc not in allow:
        raise PbmError(fn, rc)
    return rc


def walk_config(strategy=COLLAB_RW_BM, word_bits=32, collab_width=32, stride=1, max_steps=4096,
                block_size=256, blocks_per_sm=0, free_merge=0, fail_fast=0) -> WalkConfig:
    return WalkConfig(strategy, word_bits, collab_width, stride, max_steps, block_size, blocks_per_sm,
                      free_merge, fail_fast, 0)


class Pool:
    """An explicit page pool (the reference's implicit per-TU pool as a handle)."""

    def __init__(self, n_pages: int, page_size: int = 4096, materialize: bool = False,
                 max_slots: int = 0):
        self.lib = lib()
        cfg = PoolConfig(n_pages, page_size, POOL_MATERIALIZE if materialize else 0, max_slots, 0)
        h = c_void_p()
        _check("pbm_pool_create", self.lib.pbm_pool_create(byref(cfg), byref(h)))
        self.h = h
        self.n_pages = n_pages
        self.page_size = page_size
        npg, psz, bm, nbytes, base = c_uint64(), c_uint32(), c_void_p(), c_size_t(), c_void_p()
        _check("pbm_pool_info", self.lib.pbm_pool_info(h, byref(npg), byref(psz), byref(bm),
                                                       byref(nbytes), byref(base)))
        self.bitmap_ptr = bm.value
        self.bitmap_bytes = nbytes.value
        self.base_ptr = base.value

    def close(self):
        if self.h:
            _check("pbm_pool_destroy", self.lib.pbm_pool_destroy(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference-named host helpers ------------------------------------------------
    def reset(self, stream=0):
        """resetMemoryManager()"""
        _check("pbm_pool_reset", self.lib.pbm_pool_reset(self.h, stream))

    def prefill(self, occupancy: float, seed: int, stream=0):
        """prefillBuffer(1 - occupancy), as i.i.d. Bernoulli bits"""
        _check("pbm_pool_prefill_bernoulli",
               self.lib.pbm_pool_prefill_bernoulli(self.h, occupancy, seed, stream))

    def used(self, stream=0) -> int:
        out = c_uint64()
        _check("pbm_pool_used", self.lib.pbm_pool_used(self.h, byref(out), stream))
        return out.value

    def free_fraction(self, stream=0) -> float:
        """getFreePagePercentage()"""
        return (self.n_pages - self.used(stream)) / self.n_pages

    def read_bitmap(self, stream=0):
        import numpy as np
        out = np.empty(self.bitmap_bytes // 4, dtype=np.uint32)
        _check("pbm_pool_read_bitmap",
               self.lib.pbm_pool_read_bitmap(self.h, out.ctypes.data, self.bitmap_bytes, stream))
        return out

    def write_bitmap(self, words, stream=0):
        import numpy as np
        w = np.ascontiguousarray(words, dtype=np.uint32)
        assert w.nbytes == self.bitmap_bytes
        _check("pbm_pool_write_bitmap",
               self.lib.pbm_pool_write_bitmap(self.h, w.ctypes.data, self.bitmap_bytes, stream))

    def stats(self, stream=0) -> Stats:
        s = Stats()
        _check("pbm_pool_stats", self.lib.pbm_pool_stats(self.h, byref(s), stream))
        return s

    # allocation -----------------------------------------------------------------
    def alloc(self, cfg: WalkConfig, n: int, seed: int, ids, steps=None, stream=0, serial=False):
        fn = self.lib.pbm_alloc_serial if serial else self.lib.pbm_alloc
        return _check("pbm_alloc", fn(self.h, byref(cfg), n, seed, _ptr(ids), _ptr(steps), stream))

    def free(self, cfg: WalkConfig, n: int, ids, stream=0):
        return _check("pbm_free", self.lib.pbm_free(self.h, byref(cfg), n, _ptr(ids), stream))

    def alloc_runs(self, n, npages, seed, ids, steps=None, max_steps=4096, stream=0, serial=False):
        fn = self.lib.pbm_alloc_runs_serial if serial else self.lib.pbm_alloc_runs
        return _check("pbm_alloc_runs", fn(self.h, n, _ptr(npages), seed, max_steps, _ptr(ids),
                                           _ptr(steps), stream))

    def alloc_spans(self, n, npages, seed, ids, steps=None, max_steps=4096, stream=0, serial=False):
        """Runs that may cross word boundaries (1 .. 65536 pages each)."""
        fn = self.lib.pbm_alloc_spans_serial if serial else self.lib.pbm_alloc_spans
        return _check("pbm_alloc_spans", fn(self.h, n, _ptr(npages), seed, max_steps, _ptr(ids),
                                            _ptr(steps), stream))

    def free_runs(self, n, ids, npages, stream=0):
        return _check("pbm_free_runs", self.lib.pbm_free_runs(self.h, n, _ptr(ids), _ptr(npages), stream))

    def claim_write_free(self, n, seed, ids, steps=None, payload_bytes=64, hold=False, max_steps=4096,
                         stream=0):
        return _check("pbm_claim_write_free",
                      self.lib.pbm_claim_write_free(self.h, n, seed, payload_bytes, int(hold), max_steps,
                                                    _ptr(ids), _ptr(steps), stream))

    def gather_pages(self, ids, n, bytes_per_page, out, stream=0):
        return _check("pbm_gather_pages", self.lib.pbm_gather_pages(self.h, _ptr(ids), n, bytes_per_page,
                                                                    _ptr(out), stream))

    def batch(self, cfg: WalkConfig, d_groups, h_groups, n_groups, arena, arena_len, seed, mode,
              steps=None, stream=0, results=None):
        """results: per-request output (device memory or pinned host memory).
        h_groups: a Group array, or a host tensor / address of packed descriptors.
        Persistent mode with d_groups None carries h_groups (at most
        MAX_INLINE_GROUPS) in the launch itself."""
        if h_groups is not None and not isinstance(h_groups, ctypes.Array):
            h_groups = ctypes.cast(ctypes.c_void_p(_ptr(h_groups)), POINTER(Group))
        if results is not None:
            return _check("pbm_batch_launch_results",
                          self.lib.pbm_batch_launch_results(self.h, byref(cfg), _ptr(d_groups), h_groups, n_groups,
                                                            _ptr(arena), arena_len, seed, _ptr(steps), _ptr(results),
                                                            mode, stream))
        return _check("pbm_batch_launch",
                      self.lib.pbm_batch_launch(self.h, byref(cfg), _ptr(d_groups), h_groups, n_groups,
                                                _ptr(arena), arena_len, seed, _ptr(steps), mode, stream))

    def graph(self, cfg: WalkConfig, d_groups, n_groups, n_steps, arena, arena_len, seed0, stream=0,
              results=None):
        g = c_void_p()
        _check("pbm_batch_graph_create_results",
               self.lib.pbm_batch_graph_create_results(self.h, byref(cfg), _ptr(d_groups), n_groups, n_steps,
                                                       _ptr(arena), arena_len, seed0, _ptr(results), stream,
                                                       byref(g)))
        return Graph(self.lib, g)

    # size-classed malloc -----------------------------------------------------------
    def malloc_init(self):
        _check("pbm_malloc_init", self.lib.pbm_malloc_init(self.h))

    def malloc_batch(self, d_groups, h_groups, n_groups, sizes, ptrs, arena_len, seed, mode, max_steps=4096,
                     stream=0):
        return _check("pbm_malloc_batch",
                      self.lib.pbm_malloc_batch(self.h, _ptr(d_groups), h_groups, n_groups, _ptr(sizes), _ptr(ptrs),
                                                arena_len, seed, max_steps, mode, stream))

    def malloc_graph(self, d_groups, n_groups, n_steps, sizes, ptrs, arena_len, seed0, max_steps=4096, stream=0):
        g = c_void_p()
        _check("pbm_malloc_graph_create",
               self.lib.pbm_malloc_graph_create(self.h, _ptr(d_groups), n_groups, n_steps, _ptr(sizes), _ptr(ptrs),
                                                arena_len, seed0, max_steps, stream, byref(g)))
        return Graph(self.lib, g)

    def malloc_counts(self, stream=0):
        live, bad = c_uint64(), c_uint64()
        _check("pbm_malloc_counts", self.lib.pbm_malloc_counts(self.h, byref(live), byref(bad), stream))
        return live.value, bad.value

    # queue-based size classes -------------------------------------------------------
    def qmalloc_init(self, ring_capacity=0):
        _check("pbm_qmalloc_init", self.lib.pbm_qmalloc_init(self.h, ring_capacity))

    def qmalloc_release(self):
        _check("pbm_qmalloc_release", self.lib.pbm_qmalloc_release(self.h))

    def qmalloc_batch(self, d_groups, h_groups, n_groups, sizes, ptrs, arena_len, seed, mode, max_steps=4096,
                      stream=0):
        return _check("pbm_qmalloc_batch",
                      self.lib.pbm_qmalloc_batch(self.h, _ptr(d_groups), h_groups, n_groups, _ptr(sizes), _ptr(ptrs),
                                                 arena_len, seed, max_steps, mode, stream))

    def qmalloc_graph(self, d_groups, n_groups, n_steps, sizes, ptrs, arena_len, seed0, max_steps=4096, stream=0):
        g = c_void_p()
        _check("pbm_qmalloc_graph_create",
               self.lib.pbm_qmalloc_graph_create(self.h, _ptr(d_groups), n_groups, n_steps, _ptr(sizes),
                                                 _ptr(ptrs), arena_len, seed0, max_steps, stream, byref(g)))
        return Graph(self.lib, g)

    def qmalloc_counts(self, stream=0):
        """(queued per class [13], chunks, overflow, timeouts, bad frees)"""
        q = (c_uint64 * 13)()
        ch, ov, to, bf = c_uint64(), c_uint64(), c_uint64(), c_uint64()
        _check("pbm_qmalloc_counts", self.lib.pbm_qmalloc_counts(self.h, q, byref(ch), byref(ov), byref(to),
                                                                 byref(bf), stream))
        return list(q), ch.value, ov.value, to.value, bf.value

    def autotune(self, d_groups, n_groups, requests, arena, arena_len, seed=77, reps=3, max_steps=4096,
                 max_out=64, stream=0):
        """Candidate configurations for this pool's occupancy, fastest first."""
        out = (TuneResult * max_out)()
        n = c_uint32()
        _check("pbm_autotune", self.lib.pbm_autotune(self.h, _ptr(d_groups), n_groups, requests, _ptr(arena),
                                                     arena_len, seed, reps, max_steps, out, max_out, byref(n),
                                                     stream))
        return [out[i] for i in range(n.value)]

    def check(self, ids, n, stream=0) -> CheckResult:
        r = CheckResult()
        rc = self.lib.pbm_check_ids(self.h, _ptr(ids), n, byref(r), stream)
        _check("pbm_check_ids", rc, allow=(ERR_CORRUPT,))
        return r


class Graph:
    def __init__(self, lib_, h):
        self.lib = lib_
        self.h = h

    def replay(self, stream=0):
        _check("pbm_graph_replay", self.lib.pbm_graph_replay(self.h, stream))

    def set_step(self, step, stream=0):
        _check("pbm_graph_set_step", self.lib.pbm_graph_set_step(self.h, step, stream))

    def close(self):
        if self.h:
            self.lib.pbm_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BufferManager:
    """Page table over n_logical pages cached in n_frames frames, CLOCK replacement."""

    def __init__(self, n_logical, n_frames, frame_size=0, policy=BM_SINGLE_CLOCK, n_arms=1, max_sweep=0,
                 backing=None):
        self.lib = lib()
        cfg = BufMgrConfig(n_logical, n_frames, frame_size, policy, n_arms, max_sweep, 0)
        self.n_logical, self.n_frames = n_logical, n_frames
        h = c_void_p()
        _check("pbm_bufmgr_create", self.lib.pbm_bufmgr_create(byref(cfg), _ptr(backing), byref(h)))
        self.h = h

    def round(self, frames_of, release_idx, n_release, pages, n, slot0, frames_out, serial=False, stream=0):
        return _check("pbm_bufmgr_round",
                      self.lib.pbm_bufmgr_round(self.h, _ptr(frames_of), _ptr(release_idx), n_release,
                                                _ptr(pages), n, slot0, _ptr(frames_out), int(serial), stream))

    def round_pages(self, pages_of, release_idx, n_release, pages, n, slot0, frames_out, held_out=None,
                    serial=False, stream=0):
        """The round with pins released by page (pages_of[release_idx[j]]);
        held_out, if given, receives each fetch's page (-1: no frame)."""
        return _check("pbm_bufmgr_round_pages",
                      self.lib.pbm_bufmgr_round_pages(self.h, _ptr(pages_of), _ptr(release_idx), n_release,
                                                      _ptr(pages), n, slot0, _ptr(frames_out), _ptr(held_out),
                                                      int(serial), stream))

    def reset(self, stream=0):
        _check("pbm_bufmgr_reset", self.lib.pbm_bufmgr_reset(self.h, stream))

    def counters(self, stream=0) -> BufMgrCounters:
        c = BufMgrCounters()
        _check("pbm_bufmgr_stats", self.lib.pbm_bufmgr_stats(self.h, byref(c), stream), allow=(ERR_CORRUPT,))
        return c

    def check(self, stream=0) -> BufMgrCheck:
        c = BufMgrCheck()
        _check("pbm_bufmgr_check", self.lib.pbm_bufmgr_check(self.h, byref(c), stream), allow=(ERR_CORRUPT,))
        return c

    def gather(self, frame_ids, n, bytes_per_frame, out, stream=0):
        return _check("pbm_bufmgr_gather", self.lib.pbm_bufmgr_gather(self.h, _ptr(frame_ids), n, bytes_per_frame,
                                                                      _ptr(out), stream))

    def read_tables(self, stream=0):
        """(frame of each page (-1 not resident), pins of each page, reference
        bit of each page, page of each frame (-1 empty)) as numpy arrays."""
        import numpy as np

        e = np.empty(self.n_logical, dtype=np.uint64)
        fp = np.empty(self.n_frames, dtype=np.uint32)
        _check("pbm_bufmgr_read_tables",
               self.lib.pbm_bufmgr_read_tables(self.h, e.ctypes.data, fp.ctypes.data, stream))
        frame = (e >> np.uint64(32)).astype(np.uint32).view(np.int32)
        pins = (e & np.uint64(0x3fffffff)).astype(np.int64)
        ref = ((e >> np.uint64(31)) & np.uint64(1)).astype(bool)
        return frame, pins, ref, fp.view(np.int32)

    def frames(self):
        p, n = c_void_p(), c_size_t()
        _check("pbm_bufmgr_frames", self.lib.pbm_bufmgr_frames(self.h, byref(p), byref(n)))
        return p.value, n.value

    def close(self):
        if self.h:
            self.lib.pbm_bufmgr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching serving loop over a pool (and optional buffer manager)."""

    def __init__(self, pool: Pool, n_tenants, ring_pages, n_streams=4, max_batch_requests=1024,
                 max_occupancy=0.95, drain_timeout_s=2.0, walk=None, bufmgr=None, fetch_pages=None,
                 max_fetch_pages=0, tenant_quota_pages=0):
        self.lib = lib()
        cfg = ServerConfig(n_tenants, ring_pages, n_streams, max_batch_requests, max_fetch_pages, tenant_quota_pages,
                           max_occupancy, drain_timeout_s, walk or walk_config())
        h = c_void_p()
        nf = 0 if fetch_pages is None else fetch_pages.numel()
        _check("pbm_server_create", self.lib.pbm_server_create(pool.h, bufmgr.h if bufmgr else None,
                                                               _ptr(fetch_pages), nf, byref(cfg), byref(h)))
        self.h = h
        self.n_tenants = n_tenants

    def run(self, arrivals, tenants, ops, counts):
        n = len(arrivals)
        reqs = (Request * n)()
        for i in range(n):
            reqs[i] = Request(float(arrivals[i]), int(tenants[i]), int(ops[i]), int(counts[i]), 0)
        res = (RequestResult * n)()
        rep = ServerReport()
        rc = self.lib.pbm_server_run(self.h, reqs, n, res, byref(rep))
        _check("pbm_server_run", rc, allow=(ERR_TIMEOUT,))
        return res, rep, rc

    def tenant_pages(self, tenant):
        import numpy as np

        k = c_uint64()
        _check("pbm_server_tenant_pages", self.lib.pbm_server_tenant_pages(self.h, tenant, None, 0, byref(k)))
        out = np.empty(k.value, dtype=np.int32)
        _check("pbm_server_tenant_pages",
               self.lib.pbm_server_tenant_pages(self.h, tenant, out.ctypes.data, k.value, byref(k)))
        return out

    def close(self):
        if self.h:
            self.lib.pbm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Monitor:
    """Occupancy and counters of a pool, sampled on a host thread while kernels run."""

    def __init__(self, pool: Pool, interval_us=100, max_samples=100000):
        self.lib = lib()
        h = c_void_p()
        _check("pbm_monitor_start", self.lib.pbm_monitor_start(pool.h, interval_us, max_samples, byref(h)))
        self.h = h
        self.max_samples = max_samples

    def samples(self):
        out = (MonitorSample * self.max_samples)()
        n = c_uint32()
        _check("pbm_monitor_samples", self.lib.pbm_monitor_samples(self.h, out, self.max_samples, byref(n)))
        return [out[i] for i in range(min(n.value, self.max_samples))]

    def stop(self):
        if self.h:
            rc = self.lib.pbm_monitor_stop(self.h)
            self.h = None
            _check("pbm_monitor_stop", rc)

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def groups_array(groups):
    """list of (op, count, offset) -> ctypes Group array"""
    arr = (Group * len(groups))()
    for i, (op, count, offset) in enumerate(groups):
        arr[i] = Group(op, count, offset)
    return arr


def atomic_ceiling(words=1 << 22, threads=152 * 2048, iters=64, returning=1, pattern=0):
    """RMW/s of uncontended atomicOr; pattern 1 = one line per warp, 2 = 32 lines, 0 = best."""
    ops, ms = c_double(), c_double()
    _check("pbm_atomic_ceiling", lib().pbm_atomic_ceiling(words, threads, iters, returning, pattern,
                                                         byref(ops), byref(ms)))
    return ops.value, ms.value


def kernel_launches() -> int:
    return lib().pbm_kernel_launches()


def version() -> str:
    return lib().pbm_version().decode()
