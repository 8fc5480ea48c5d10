"""Times the reference's own CUDA build on the alloc+free churn workload.

TEST INFRASTRUCTURE / REFERENCE TIMING ONLY.  Runs the reference's getPage and
freePage (CollabRW_BM.cuh:114-160 and :73-77, the warp-collaborative walk; or
RandomWalkBasic.cuh:52-83, the page-probe walk on an int-per-page map) from
the cubins that `make ref` builds from its unchanged sources, through the
CUDA driver API (ref_driver.py).  Each request is one thread of the harness
kernel fx_churn: release the page held in its arena slot, then take a new
one, as the reference's callers do one page per thread.  The reference has
no batched form; its most favourable launch form is used here: one launch
per at most `max_launch` requests (not one per caller group).

Safety: the reference's walks spin (CollabRW_BM.cuh:123) or trap
(RandomWalkBasic.cuh:64-67) when no page is free.  Releasing before taking
keeps the free pages at or above their start; in addition no launch carries
more than half of the free pages, and the bitmap is checked between steps
(the run stops if the free pages fall below 60% of their start, which would
mean the reference's write-back race -- CollabRW_BM.cuh:152-153 overwrites
frees that land in a word it holds -- had leaked that many).
"""
from __future__ import annotations

import time

import numpy as np

from ref_driver import D, Driver, have_cubin

POPC8 = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)


def _used_bits(words: np.ndarray) -> int:
    return int(POPC8[words.view(np.uint8)].sum())


def available(walk: str = "collab") -> bool:
    return have_cubin("ref_collab.cubin" if walk == "collab" else "ref_rwbasic.cubin")


def churn(words: np.ndarray, n_pages: int, held: np.ndarray, step_counts, warmup: int, walk: str = "collab",
          flush_bytes: int = 512 << 20, max_launch: int = 1 << 19, block: int = 256, clock_seed: int = 7):
    """Run len(step_counts) steps of churn; time the steps after `warmup`.

    words: the 32-bit bitmap (bit p of word p/32 set = page p held), n_pages
    pages; held: the held page ids (the arena, one slot per page).  Returns a
    dict with ops/s (2 per request), per-step times and the pages the run
    lost (held bits no slot refers to) or double-counted."""
    drv = Driver()
    H = int(held.size)
    used0 = _used_bits(words)
    free0 = n_pages - used0
    cap = int(min(max_launch, free0 // 2))
    if cap <= 0:
        raise ValueError("pool has no free pages")
    if walk == "collab":
        mod = drv.module("ref_collab.cubin")
        d_map = drv.upload(words.view(np.int32))
        drv.launch(drv.fn(mod, "fx_setup"), 1, 1, D(d_map), words.size, n_pages)
    elif walk == "rwbasic":
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:n_pages].astype(np.int32)
        mod = drv.module("ref_rwbasic.cubin")
        d_map = drv.upload(bits)
        drv.launch(drv.fn(mod, "fx_setup"), 1, 1, D(d_map), n_pages)
    else:
        raise ValueError(walk)
    f = drv.fn(mod, "fx_churn")
    clock_ptr = drv.global_ptr(mod, "fx_clock_val")
    d_arena = drv.upload(held.astype(np.int32))
    d_flush = drv.alloc(flush_bytes)
    rng = np.random.default_rng(clock_seed)
    ev = [(drv.event(), drv.event()) for _ in step_counts]
    off = 0
    done_steps = 0
    stopped = None
    wall0 = time.perf_counter()
    for s, n in enumerate(step_counts):
        n = int(n)
        drv.h2d(clock_ptr, rng.integers(-32768, 32768, size=1).astype(np.int32))
        drv.memset8(d_flush, s & 0xFF, flush_bytes)
        e0, e1 = ev[s]
        drv.record(e0)
        k0 = 0
        while k0 < n:
            k = min(cap, n - k0)
            drv.launch_async(f, (k + block - 1) // block, block, k, D(d_arena), H, off)
            off = (off + k) % H
            k0 += k
        drv.record(e1)
        drv.sync()
        done_steps = s + 1
        if s % 8 == 7 or s == len(step_counts) - 1:
            if walk == "collab":
                cur = drv.d2h(np.empty_like(words), d_map)
                free_now = n_pages - _used_bits(cur)
            else:
                cur = drv.d2h(np.empty(n_pages, np.int32), d_map)
                free_now = n_pages - int(np.count_nonzero(cur))
            if free_now < 0.6 * free0:
                stopped = f"free pages fell to {free_now} of {free0} after step {s}"
                break
    wall = time.perf_counter() - wall0
    ms = [drv.elapsed_ms(e0, e1) for e0, e1 in ev[warmup:done_steps]]
    reqs = [int(c) for c in list(step_counts)[warmup:done_steps]]
    arena = drv.d2h(np.empty(H, np.int32), d_arena)
    if walk == "collab":
        cur = drv.d2h(np.empty_like(words), d_map)
        bits = np.unpackbits(cur.view(np.uint8), bitorder="little")[:n_pages].astype(bool)
    else:
        bits = drv.d2h(np.empty(n_pages, np.int32), d_map) != 0
    ok_ids = (arena >= 0) & (arena < n_pages)
    u, c = np.unique(arena[ok_ids], return_counts=True)
    for e0, e1 in ev:
        drv.destroy_event(e0)
        drv.destroy_event(e1)
    drv.free_all()
    t = sum(ms)
    return {
        "value": 2.0 * sum(reqs) / (t * 1e-3) if t > 0 else None,
        "unit": "ops/s",
        "steps_timed": len(ms),
        "ms_per_step": t / max(1, len(ms)),
        "requests_timed": sum(reqs),
        "launch_cap": cap,
        "wall_s": wall,
        "stopped": stopped,
        "bad_ids": int((~ok_ids).sum()),
        "ids_held_twice": int((c > 1).sum()),
        "held_bits_without_owner": int(bits.sum()) - int(np.isin(np.nonzero(bits)[0], u).sum())
        if bits.sum() < (1 << 26) else None,
        "used_before": used0,
        "used_after": int(bits.sum()),
    }


def available_pp() -> bool:
    return have_cubin("ref_pp.cubin")


def churn_clock(walk: str, occupancy: float, step_counts, warmup: int, seed: int = 2,
                flush_bytes: int = 512 << 20, max_launch: int = 1 << 19, block: int = 256, arm_seed: int = 11):
    """Churn of the reference's SingleClock or DistClock (parallelPage.cu:491-509,
    571-592) on its own pool of TOTAL_N_PAGES pages (fixed at compile time,
    41,900,000), prefilled Bernoulli(occupancy) with `seed`; each request
    frees its arena slot's page and takes a new one (fx_churn_sc / _dc).

    Safety: releasing first keeps the free pages at or above their start and
    no launch asks for more than half of them; DistClock launches stay below
    its MAX_THREADS_DISTCLOCK arm slots (its arms are indexed by thread id);
    the single clock's int arm is read after every step and the run stops
    long before it could pass 2^31 (parallelPage.cu:498-499 would then index
    before the map).  DistClock's arms start at uniform random pages drawn on
    the host (the reference draws them from clock() in randomizeArmDistClock)."""
    import oracle

    assert walk in ("singleclock", "distclock")
    drv = Driver()
    mod = drv.module("ref_pp.cubin")
    info = drv.upload(np.zeros(2, np.int32))
    drv.launch(drv.fn(mod, "fx_total_pages"), 1, 1, D(info))
    T = int(drv.d2h(np.zeros(2, np.int32), info)[0])
    words = oracle.bernoulli_bitmap(T, occupancy, seed)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(seed).shuffle(held)
    H = int(held.size)
    free0 = T - H
    d_map = drv.upload(bits.astype(np.int32))
    del bits
    arm_info = drv.upload(np.zeros(2, np.int32))
    drv.launch(drv.fn(mod, "fx_sc_arm"), 1, 1, D(arm_info))
    max_dc = int(drv.d2h(np.zeros(2, np.int32), arm_info)[1])
    arms = np.random.default_rng(arm_seed).integers(0, T, size=max_dc).astype(np.int32)
    d_arms = drv.upload(arms)
    d_dummy = drv.alloc(1 << 20)
    drv.launch(drv.fn(mod, "fx_setup"), 1, 1, D(d_map), D(d_map), D(d_arms), D(d_dummy), D(d_dummy))
    cap = int(min(max_launch, free0 // 2, max_dc if walk == "distclock" else max_launch))
    f = drv.fn(mod, "fx_churn_sc" if walk == "singleclock" else "fx_churn_dc")
    f_arm = drv.fn(mod, "fx_sc_arm")
    d_arena = drv.upload(held)
    d_flush = drv.alloc(flush_bytes)
    ev = [(drv.event(), drv.event()) for _ in step_counts]
    off, done_steps, stopped, arm = 0, 0, None, 0
    for s, n in enumerate(step_counts):
        n = int(n)
        drv.memset8(d_flush, s & 0xFF, flush_bytes)
        e0, e1 = ev[s]
        drv.record(e0)
        k0 = 0
        while k0 < n:
            k = min(cap, n - k0)
            drv.launch_async(f, (k + block - 1) // block, block, k, D(d_arena), H, off)
            off = (off + k) % H
            k0 += k
        drv.record(e1)
        drv.sync()
        done_steps = s + 1
        if walk == "singleclock":
            drv.launch(f_arm, 1, 1, D(arm_info))
            arm = int(drv.d2h(np.zeros(2, np.int32), arm_info)[0])
            if arm < 0 or arm > 1_500_000_000:
                stopped = f"single-clock arm at {arm} after step {s}"
                break
    ms = [drv.elapsed_ms(e0, e1) for e0, e1 in ev[warmup:done_steps]]
    reqs = [int(c) for c in list(step_counts)[warmup:done_steps]]
    m = drv.d2h(np.empty(T, np.int32), d_map)
    arena = drv.d2h(np.empty(H, np.int32), d_arena)
    ok = (arena >= 0) & (arena < T)
    u, c = np.unique(arena[ok], return_counts=True)
    for e0, e1 in ev:
        drv.destroy_event(e0)
        drv.destroy_event(e1)
    drv.free_all()
    t = sum(ms)
    return {
        "value": 2.0 * sum(reqs) / (t * 1e-3) if t > 0 else None, "unit": "ops/s",
        "pool_pages": T, "occupancy": occupancy, "steps_timed": len(ms), "ms_per_step": t / max(1, len(ms)),
        "requests_timed": sum(reqs), "launch_cap": cap, "stopped": stopped, "final_arm": arm,
        "bad_ids": int((~ok).sum()), "ids_held_twice": int((c > 1).sum()),
        "used_before": H, "used_after": int(np.count_nonzero(m)),
    }
