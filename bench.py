#!/usr/bin/env python
"""Benchmark: alloc+free ops/s at 90% pool occupancy, batched vs plain launch.

Workload (one "step" = one batch): a pool of 2^24 pages x 4 KiB (64 GiB,
2 MiB bitmap) held at 90% occupancy (i.i.d. Bernoulli(0.9) prefill, seed 2).
Each step carries 256 caller groups whose request counts are log-uniform in
[1, 65536] (seed 4).  Every request is an alloc+free pair (PBM_OP_SWAP): it
claims a new page with the warp-collaborative walk and frees the page held in
its slot of a resident held-page arena (all prefilled pages, shuffled), so
occupancy stays at 90%.  Ops = 2 x requests (one alloc, one free).

Forms timed on the same requests:
  value    batched: one persistent kernel per step, replayed from a CUDA graph
  plain    one kernel launch per caller group (256 launches per step)
  e2e      through the C ABI with host buffers: the step's host descriptor
           table carried in the persistent launch's parameters, the step's new
           page ids written by the kernel into pinned host memory, all inside
           the timed region
The L2 is flushed (512 MiB write) between timed steps, outside the events.

Output: one JSON line per other workload ("detail" lines), then the headline
as the last line of stdout, a compact object of at most HEADLINE_MAX_BYTES.

`--impl reference` times the reference's algorithm on the host cores: the
std::atomic replay of its word-probe walk (RandomWalkBasic_BM) over the same
churn, all hardware threads (the reference ships no CPU implementation).  The
same line carries `reference_cuda_build`: the reference's own getPage/freePage
(CollabRW_BM and RandomWalkBasic), compiled from its sources for sm_103a, on
the same churn, one launch per <= 2^19 requests (its callers launch one
thread per request; it has no batched form).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "parallel-db-buffer-management_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

T_PAGES = 1 << 24
PAGE_SIZE = 4096
OCCUPANCY = 0.9
PREFILL_SEED = 2
GROUP_SEED = 4
N_GROUPS = 256
MAX_GROUP = 65536
SEED0 = 1000
METRIC = "alloc+free ops/s at 90% occupancy (batched persistent kernel, CUDA-graph replay)"
UNIT = "ops/s"
# DRAM bytes per alloc+free pair of the batch kernel: dram__bytes_read.sum +
# dram__bytes_write.sum of one captured launch (7.82 MB for the 1,420,753-pair
# step of `bench.py --profile --profile-walk pair32c`), summarised in
# profiles/batch_persistent_collab32_90pct.md.
NCU_DRAM_BYTES_PER_PAIR = 7.815424e6 / 1420753


HEADLINE_MAX_BYTES = 1400


def _sig(x, digits=5):
    """A float rounded to `digits` significant figures (keeps the headline short)."""
    if isinstance(x, float) and math.isfinite(x) and x != 0.0:
        return round(x, digits - 1 - int(math.floor(math.log10(abs(x)))))
    return x


def _short(d, digits=5):
    if isinstance(d, dict):
        return {k: _short(v, digits) for k, v in d.items()}
    if isinstance(d, (list, tuple)):
        return [_short(v, digits) for v in d]
    return _sig(d, digits)


# keys of the headline line, in print order; everything else is a detail line
HEADLINE_KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                 "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks",
                 "gpu_launches", "plain_value", "batched_over_plain", "invariants_ok", "reference_cuda_build")
SUB_KEYS = {
    "config": ("workload", "walk", "l2", "launch"),
    "e2e": ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"),
    "roofline": ("bound", "achieved", "peak", "unit", "frac", "traffic", "peak_source", "line_pattern_peak",
                 "hbm_frac"),
    "cpu_baseline": ("value", "unit", "cores", "kind", "sample"),
    "clocks": ("sm_mhz", "sm_max_mhz", "reasons"),
    "reference_cuda_build": ("collab_ops_s", "rwbasic_ops_s", "singleclock_ops_s", "distclock_ops_s"),
}


def headline(full):
    """The one JSON line printed last: the keys of HEADLINE_KEYS (nested
    objects cut to SUB_KEYS), floats to five significant figures.  A log
    reader that keeps only the end of stdout still sees the whole line; the
    rest of the run's results go out as detail lines before it."""
    out = {}
    for k in HEADLINE_KEYS:
        if k not in full:
            continue
        v = full[k]
        if isinstance(v, dict) and k in SUB_KEYS:
            v = {s: v[s] for s in SUB_KEYS[k] if s in v}
        out[k] = _short(v)
    s = json.dumps(out, separators=(",", ":"))
    if len(s) > HEADLINE_MAX_BYTES:           # long free-text fields go first, never the numbers
        for k, s2 in (("cpu_baseline", "sample"), ("config", "walk"), ("config", "workload")):
            if k in out and isinstance(out[k], dict) and s2 in out[k] and len(s) > HEADLINE_MAX_BYTES:
                out[k][s2] = str(out[k][s2])[:60]
                s = json.dumps(out, separators=(",", ":"))
    return s


def emit(full, details, path=None):
    """Detail lines first (one JSON object per workload, key "detail"), then
    the headline.  `path`: also write everything as one JSON file."""
    for name, obj in details.items():
        print(json.dumps({"detail": name, **(obj if isinstance(obj, dict) else {"value": obj})}), flush=True)
    if path:
        with open(path, "w") as f:
            json.dump({"headline": full, "details": details}, f, indent=1)
    print(headline(full), flush=True)


def env_rank():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


WALKS = ("collab32c", "pair32c", "pair32c6", "collab32", "collab64c", "word32", "word64", "page")


def named_walk(pbm, name):
    """Walk configurations by name (`--walk`); the `c` forms are the
    register-capped kernels at 5 blocks per SM, all with unmerged frees;
    `pair32c` serves two requests per lane (64 per warp, collab_width 64),
    `pair32c6` the same at 6 blocks per SM where the registers allow."""
    return {"collab32c": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32, blocks_per_sm=5),
            "pair32c": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=64, blocks_per_sm=5),
            "pair32c6": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=64, blocks_per_sm=6),
            "collab32": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32),
            "collab64c": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=64, collab_width=32, blocks_per_sm=5),
            "word32": pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32),
            "word64": pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=64),
            "page": pbm.walk_config(pbm.RANDOM_WALK)}[name]


def combine_ranks(ms, ops, world, dist=None, device="cpu"):
    """Whole-job throughput of N independent replicas: every rank ran `ops`
    operations in `ms` milliseconds of device time; the job's time is the
    slowest rank's (max over ranks), its work the sum.  Returns (max_ms, ops/s)."""
    if dist is not None and world > 1:
        import torch

        t = torch.tensor([float(ms), float(ops)], dtype=torch.float64, device=device)
        mx = t[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
        ms, total = float(mx.item()), float(t[1].item())
    else:
        total = float(ops) * world
    return ms, total / (ms * 1e-3)


def group_counts(n_steps, seed=GROUP_SEED):
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, math.log(MAX_GROUP + 1), size=(n_steps, N_GROUPS))
    return np.clip(np.floor(np.exp(u)), 1, MAX_GROUP).astype(np.int64)


def build_descriptors(counts, arena_len, op):
    """pbm_group table: (op int32, count uint32, offset uint64) per group, steps x groups."""
    dt = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
    tab = np.zeros(counts.shape, dtype=dt)
    flat = counts.reshape(-1).astype(np.uint64)
    starts = np.concatenate([[0], np.cumsum(flat)[:-1]]).astype(np.uint64) % np.uint64(arena_len)
    tab["op"] = op
    tab["count"] = counts.astype(np.uint32)
    tab["offset"] = starts.reshape(counts.shape)
    return tab


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_reference(args, rank):
    """CPU replay of the reference's word-probe walk (std::atomic, all threads)."""
    if rank != 0:
        return 0
    import oracle

    words = oracle.bernoulli_bitmap(T_PAGES, OCCUPANCY, PREFILL_SEED)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(PREFILL_SEED).shuffle(held)
    threads = oracle.lib().orc_hw_threads()
    pairs = 1 << 23
    # calibration: size every step so that warm-up + timed steps take ~90 s
    secs, ok, fail, st, _ = oracle.cpu_churn(words, T_PAGES, held, pairs, SEED0, threads)
    rate = 2 * ok / secs
    per_step_s = 90.0 / max(1, args.steps + args.warmup)
    pairs = int(max(1 << 18, min(1 << 30, rate * per_step_s / 2)))
    for w in range(args.warmup):
        oracle.cpu_churn(words, T_PAGES, held, pairs, SEED0 + 1 + w, threads)
    tot_ops, tot_s = 0, 0.0
    for k in range(args.steps):
        secs, ok, fail, st, _ = oracle.cpu_churn(words, T_PAGES, held, pairs, SEED0 + 100 + k, threads)
        tot_ops += 2 * ok
        tot_s += secs
    value = tot_ops / tot_s
    sample = (f"{pairs} alloc+free pairs per step on the 2^24-page pool at 90% occupancy "
              f"(word-probe walk, reference LCG, std::atomic fetch_or/fetch_and)")
    ref_gpu = reference_cuda_build(args)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda_build": {w + "_ops_s": (ref_gpu.get(w) or {}).get("value")
                                 for w in ("collab", "rwbasic", "singleclock", "distclock")},
    }
    emit(line, {"reference_cuda_build": ref_gpu}, args.details)
    return 0


def reference_cuda_build(args):
    """The reference's own device code on the same churn (fresh pool, same
    step request counts, L2 flushed between steps), when its cubins were built
    (they need the reference sources at build time) and a GPU is present."""
    try:
        import ref_timing
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"reference harness not importable: {e}"}
    if not ref_timing.available("collab"):
        return {"unavailable": "reference cubins not built (oracle/Makefile `ref` needs the reference sources)"}
    import oracle

    n = min(args.steps, 100) + args.warmup
    counts = group_counts(n).sum(axis=1)
    out = {"launch": "one launch per <= 2^19 requests, 256 threads per block", "steps": n - args.warmup,
           "warmup": args.warmup, "l2": "flushed between timed steps (512 MiB write)"}
    for walk in ("collab", "rwbasic"):
        words = oracle.bernoulli_bitmap(T_PAGES, OCCUPANCY, PREFILL_SEED)
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES]
        held = np.nonzero(bits)[0].astype(np.int32)
        np.random.default_rng(PREFILL_SEED).shuffle(held)
        try:
            out[walk] = ref_timing.churn(words, T_PAGES, held, counts, args.warmup, walk=walk)
        except Exception as e:  # noqa: BLE001
            out[walk] = {"unavailable": str(e)[:300]}
    out["walks"] = {"collab": "CollabRW_BM.cuh getPage/freePage (warp-collaborative, atomicExch of whole words)",
                    "rwbasic": "RandomWalkBasic.cuh getPage/freePage (page probe on an int-per-page map)",
                    "singleclock": "parallelPage.cu getPageSingleClock/freePageSingleClock on its own "
                                   "41,900,000-page pool",
                    "distclock": "parallelPage.cu getPageDistClock/freePageDistClock on its own 41,900,000-page "
                                 "pool (launches below its 10^6 arm slots)"}
    if ref_timing.available_pp():
        n_clk = min(args.steps, 20) + args.warmup
        clk_counts = group_counts(n_clk).sum(axis=1)
        for walk in ("singleclock", "distclock"):
            try:
                out[walk] = ref_timing.churn_clock(walk, OCCUPANCY, clk_counts, args.warmup, seed=PREFILL_SEED)
            except Exception as e:  # noqa: BLE001
                out[walk] = {"unavailable": str(e)[:300]}
    return out


def workload_config():
    return {
        "workload": "alloc+free churn at 90% occupancy: 2^24 x 4 KiB pages (64 GiB), 256 caller groups/step "
                    "with LogU[1,65536] requests (seed 4), swap op on a resident held-page arena",
        "pool_pages": T_PAGES, "page_size": PAGE_SIZE, "occupancy": OCCUPANCY, "prefill_seed": PREFILL_SEED,
        "groups_per_step": N_GROUPS, "walk": "autotuned for the 90% band (see tuned_config); reference arm: word-probe walk",
        "launch": "persistent kernel in a CUDA graph", "l2": "flushed between timed steps (512 MiB write)",
        "parallelism": "single GPU per rank (independent pools)",
    }


def cpu_baseline_sample(words, held):
    import oracle

    threads = oracle.lib().orc_hw_threads()
    pairs = 1 << 22
    secs, ok, _, _, _ = oracle.cpu_churn(words.copy(), T_PAGES, held.copy(), pairs, 7, threads)
    # size the sample to ~10 s of CPU work
    pairs = int(min(1 << 31, max(pairs, (2 * ok / secs) * 10.0 / 2)))
    w2, h2 = words.copy(), held.copy()
    secs, ok, fail, st, _ = oracle.cpu_churn(w2, T_PAGES, h2, pairs, 8, threads)
    return {"value": 2 * ok / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{pairs} alloc+free pairs on the same pool/occupancy, word-probe walk, "
                      f"std::atomic on {threads} host threads, {secs:.1f} s"}


def run_ours(args, rank, world, local_rank):
    import torch

    import pbm

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    pool = pbm.Pool(T_PAGES, PAGE_SIZE, materialize=True)
    pool.prefill(OCCUPANCY, PREFILL_SEED, sh)
    words = pool.read_bitmap(sh)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(PREFILL_SEED).shuffle(held)
    H = len(held)
    arena = torch.from_numpy(held).to(dev)
    n_steps = args.warmup + args.steps
    counts = group_counts(n_steps)
    tab = build_descriptors(counts, H, pbm.OP_SWAP)
    d_tab = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).to(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    # autotuner (untimed): candidates run on step 0's groups, swaps keep the
    # pool at 90%.  It tunes a scratch copy of the pool (same prefill, same
    # arena), so its few hundred passes of churn leave the measured pool as
    # the workload defines it: prefilled, then the warm-up and timed steps
    tuned = []
    if args.walk == "auto":
        scratch = pbm.Pool(T_PAGES, PAGE_SIZE, materialize=False)
        scratch.prefill(OCCUPANCY, PREFILL_SEED, sh)
        scratch_arena = arena.clone()
        tuned = scratch.autotune(d_tab[:N_GROUPS * 16], N_GROUPS, int(counts[0].sum()), scratch_arena, H,
                                 seed=SEED0 - 999, reps=7, stream=sh)
        torch.cuda.synchronize()
        scratch.close()
        del scratch_arena
    cfg = named_walk(pbm, "collab32c" if args.walk == "auto" else args.walk)
    if tuned:
        cfg = pbm.WalkConfig.from_buffer_copy(tuned[0].cfg)

    def cfg_dict(c):
        return {"walk": pbm.STRATEGY_NAMES[c.strategy], "word_bits": c.word_bits, "width": c.collab_width,
                "stride": c.stride, "blocks_per_sm": c.blocks_per_sm, "free_merge": c.free_merge}

    def h_groups(s):
        return pbm.groups_array([(pbm.OP_SWAP, int(tab[s, g]["count"]), int(tab[s, g]["offset"]))
                                 for g in range(N_GROUPS)])

    def timed(fn, steps_idx):
        ev = []
        for s in steps_idx:
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(s)
            e1.record(stream)
            ev.append((s, e0, e1))
        torch.cuda.synchronize()
        return [(s, e0.elapsed_time(e1)) for s, e0, e1 in ev]

    # ---- batched: graph replay ----
    graph = pool.graph(cfg, d_tab, N_GROUPS, n_steps, arena, H, SEED0, sh)
    for s in range(args.warmup):
        graph.replay(sh)
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = pbm.kernel_launches()
    t_wall0 = time.perf_counter()
    res_graph = timed(lambda s: graph.replay(sh), range(args.warmup, n_steps))
    t_wall1 = time.perf_counter()
    launches = pbm.kernel_launches() - l0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    pairs_per_step = counts.sum(axis=1)
    g_ms = sum(ms for _, ms in res_graph)
    g_ops = sum(2 * int(pairs_per_step[s]) for s, _ in res_graph)
    g_ms, value = combine_ranks(g_ms, g_ops, world, dist, dev)
    st = pool.stats(sh)

    # ---- plain: one launch per group (the ctypes group arrays are built
    # before the timed region, so the events see only the launches) ----
    plain_steps = range(args.warmup, min(n_steps, args.warmup + 100))
    plain_groups = {s: h_groups(s) for s in plain_steps}
    res_plain = timed(lambda s: pool.batch(cfg, None, plain_groups[s], N_GROUPS, arena, H, SEED0 + s,
                                           pbm.LAUNCH_PLAIN, stream=sh), plain_steps)
    p_ms = sum(ms for _, ms in res_plain)
    plain_value = sum(2 * int(pairs_per_step[s]) for s, _ in res_plain) / (p_ms * 1e-3)

    # ---- per-thread word-probe walk, batched (config-2 comparison) ----
    cfg_pt = pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32)
    g_pt = pool.graph(cfg_pt, d_tab, N_GROUPS, n_steps, arena, H, SEED0 + 7777, sh)
    for s in range(args.warmup):
        g_pt.replay(sh)
    res_pt = timed(lambda s: g_pt.replay(sh), range(args.warmup, min(n_steps, args.warmup + 100)))
    pt_ms = sum(ms for _, ms in res_pt)
    per_thread_value = sum(2 * int(pairs_per_step[s]) for s, _ in res_pt) / (pt_ms * 1e-3)

    # ---- e2e through the C ABI with host buffers ----
    h_tab = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).pin_memory()
    d_stage = torch.empty(N_GROUPS * 16, dtype=torch.uint8, device=dev)
    max_pairs = int(pairs_per_step.max())
    h_out = torch.empty(max_pairs, dtype=torch.int32).pin_memory()
    e2e_bytes_in, e2e_bytes_out = [], []

    # one launch per step with the step's host descriptor table carried in the
    # launch's parameters (no separate host-to-device copy); the kernel writes
    # every request's new page into the pinned host buffer h_out as it
    # finishes (device -> host over the chip-to-chip link, inside the step)
    h_tab_addr = h_tab.data_ptr()

    def e2e_step(s):
        pool.batch(cfg, None, h_tab_addr + s * N_GROUPS * 16, N_GROUPS, arena, H, SEED0 + 50000 + s,
                   pbm.LAUNCH_PERSISTENT, stream=sh, results=h_out)
        e2e_bytes_in.append(N_GROUPS * 16)
        e2e_bytes_out.append(4 * int(pairs_per_step[s]))

    for s in range(args.warmup):
        e2e_step(s)
    torch.cuda.synchronize()
    res_e2e = timed(e2e_step, range(args.warmup, min(n_steps, args.warmup + 100)))
    e_ms = sum(ms for _, ms in res_e2e)
    # the last step's results on the host are the arena's new pages
    s_last = res_e2e[-1][0]
    n_last, start = int(pairs_per_step[s_last]), int(tab[s_last, 0]["offset"])
    got = h_out[:n_last].numpy().copy()
    exp = np.concatenate([arena[start:min(H, start + n_last)].cpu().numpy(),
                          arena[:max(0, start + n_last - H)].cpu().numpy()])
    e2e_results_ok = bool(np.array_equal(got, exp))
    _, e2e_value = combine_ranks(e_ms, sum(2 * int(pairs_per_step[s]) for s, _ in res_e2e), world, dist, dev)

    # ---- invariants after all forms: occupancy unchanged, arena unique ----
    chk = pool.check(arena, H)
    ok_inv = (chk.n_duplicates == 0 and chk.n_out_of_range == 0 and chk.n_not_marked == 0
              and chk.n_failed == 0 and chk.used_pages == H)

    # ---- roofline: atomic ceiling and HBM ----
    ceil_line, _ = pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1, pattern=1)
    ceil_spread, _ = pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1,
                                        pattern=2)
    # the ceiling: uncontended atomicOr on distinct words spread over L2 slices
    # (32 lanes on 32 lines), the pattern of the frees and of per-page claims;
    # the one-line pattern (32 lanes on one 128-byte line) is reported beside it
    ceil_ops = ceil_spread
    pairs_s = value / 2 / world
    atomic_achieved = 2 * pairs_s          # algorithmic RMWs: one claim + one release per pair
    bytes_per_pair = 16                    # 4 B arena read + 4 B write + 2 x 4 B bitmap RMW
    hbm_achieved = bytes_per_pair * pairs_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    avg_pairs = float(np.mean([pairs_per_step[s] for s, _ in res_graph]))
    traffic = None if NCU_DRAM_BYTES_PER_PAIR is None else NCU_DRAM_BYTES_PER_PAIR * avg_pairs
    roofline = {
        "bound": "l2_atomic", "achieved": atomic_achieved / 1e9, "peak": ceil_ops / 1e9, "unit": "Gatomic/s",
        "frac": atomic_achieved / ceil_ops, "traffic": traffic,
        "peak_source": "spread-pattern atomicOr ceiling (32 lanes on 32 lines), same run",
        "line_pattern_peak": ceil_line / 1e9, "frac_of_line_pattern": atomic_achieved / ceil_line,
        "hbm_frac": hbm_achieved / hbm_peak,
        "kernel": "k_batch_persistent of the tuned walk (see tuned_config): one launch per graph replay",
        "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_achieved / hbm_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
    }

    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_base = cpu_baseline_sample(words, held)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": g_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": dict(workload_config(), walk="{walk}/{word_bits}b/w{width}/s{stride}/b{blocks_per_sm}".format(
            **cfg_dict(cfg))),
        "plain_value": plain_value, "batched_over_plain": value / world / plain_value,
        "per_thread_walk_value": per_thread_value,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(np.mean(e2e_bytes_in)),
                "d2h_bytes_per_step": int(np.mean(e2e_bytes_out)),
                "form": "one persistent launch per step carrying the step's pinned host descriptor table in its "
                        "parameters (pbm_batch_launch_results, d_groups NULL); each request's new page written by "
                        "the kernel into pinned host memory",
                "results_match_arena": e2e_results_ok},
        "roofline": roofline, "cpu_baseline": cpu_base, "clocks": clocks,
        "gpu_launches": int(launches),
        "wall_s_timed_region": t_wall1 - t_wall0,
        "mean_pairs_per_step": avg_pairs,
        "collab_mean_steps": (st.steps / max(1, st.successes + st.failures)),
        "failures": int(st.failures), "invariants_ok": bool(ok_inv),
        "atomic_ceiling_ops_s": {"line": ceil_line, "spread": ceil_spread},
        "tuned_config": cfg_dict(cfg),
        "autotune_top": [dict(cfg_dict(t.cfg), ops_per_s=t.ops_per_s) for t in tuned[:6]],
    }
    graph.close()
    g_pt.close()
    pool.close()
    del flush
    details = {"headline_full": {k: line[k] for k in ("roofline", "e2e", "cpu_baseline", "clocks", "tuned_config",
                                                      "autotune_top", "atomic_ceiling_ops_s", "per_thread_walk_value",
                                                      "collab_mean_steps", "failures", "mean_pairs_per_step",
                                                      "wall_s_timed_region")}}
    if rank == 0 and world == 1:
        details.update(run_configs(args, torch, pbm, stream))
    if rank == 0:
        emit(line, details, args.details)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------
# The other workloads of the path, measured in the same run (keys of "configs")
# ----------------------------------------------------------------------------

def _ev_ms(torch, stream, fn):
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def config_claim_write_free(torch, pbm, stream, reps=200, cpu=True):
    """65,536 pages x 64 B (2,048-word bitmap) at 50% occupancy (seed 1);
    32,768 threads (seed 1 + tid) each claim a page with the page-probe walk,
    write their tid into its 64-B payload and free it.  `cpu`: also time the
    std::atomic host replay of the same requests on the same bitmap."""
    sh = stream.cuda_stream
    T, N = 1 << 16, 1 << 15
    out = {}
    pool = pbm.Pool(T, 64, materialize=True)
    pool.prefill(0.5, 1, sh)
    before = pool.read_bitmap(sh)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    steps = torch.empty(N, dtype=torch.int32, device="cuda")
    for _ in range(5):
        pool.claim_write_free(N, 1, ids, steps, payload_bytes=64, stream=sh)
    ms = [_ev_ms(torch, stream, lambda: pool.claim_write_free(N, 1, ids, steps, payload_bytes=64, stream=sh))
          for _ in range(reps)]
    after = pool.read_bitmap(sh)
    st = steps.cpu().numpy()
    idv = ids.cpu().numpy()
    out = {"pairs_per_launch": N, "launches": reps, "ms_per_launch": float(np.median(ms)),
           "value": 2 * N / (np.median(ms) * 1e-3), "unit": "ops/s",
           "mean_steps": float(st[idv >= 0].mean()), "failures": int((idv < 0).sum()),
           "bitmap_restored": bool(np.array_equal(before, after)),
           "note": "L2-resident (8 KiB bitmap, 4 MiB pages); median launch time over the launches"}
    pool.close()
    if cpu:
        import oracle

        secs, ok, _, th = oracle.cpu_claim_write_free(before.copy(), T, 64, 64, N, 1, 20)
        passes = int(min(100000, max(20, 20 * 3.0 / max(secs, 1e-3))))
        w = before.copy()
        secs, ok, st, th = oracle.cpu_claim_write_free(w, T, 64, 64, N, 1, passes)
        out["cpu_replay"] = {"value": 2 * ok / secs, "unit": "ops/s", "cores": th, "kind": "port",
                             "mean_steps": st / max(1, ok), "bitmap_restored": bool(np.array_equal(w, before)),
                             "sample": f"{passes} passes over the {N} requests on the same bitmap, page-probe walk, "
                                       f"std::atomic on {th} host threads, {secs:.1f} s"}
    return out


def config_occupancy_sweep(torch, pbm, stream, flush, rounds=16, N=1 << 22, max_steps=1024):
    """2^24 x 4 KiB pages; occupancy {0,50,75,90,95}% (seed 2); per round one
    launch of 2^22 get-page requests, then one freeing a uniformly random 50%
    of that round's pages; 16 rounds.  Failures are bounded by max_steps."""
    sh = stream.cuda_stream
    pool = pbm.Pool(T_PAGES, PAGE_SIZE, materialize=True)
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    steps = torch.empty(N, dtype=torch.int32, device="cuda")
    # fail fast: a popcount pass before each launch sets its budget of free
    # pages, and the requests past it fail at once instead of walking
    # max_steps jumps (the pass is inside the timed launch)
    walks = {
        "collab32": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32, max_steps=max_steps,
                                    fail_fast=1),
        "word_probe32": pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32, max_steps=max_steps, fail_fast=1),
        "page_probe": pbm.walk_config(pbm.RANDOM_WALK, max_steps=max_steps, fail_fast=1),
    }
    gen = torch.Generator(device="cuda")
    res = {}
    for occ in (0.0, 0.5, 0.75, 0.9, 0.95):
        row = {}
        for wname, cfg in walks.items():
            pool.reset(sh)
            if occ > 0:
                pool.prefill(occ, PREFILL_SEED, sh)
            free0 = T_PAGES - pool.used(sh)          # the realised free pages of the prefill
            gen.manual_seed(PREFILL_SEED)
            t_ms, ops, fails, round0_steps, per_round = 0.0, 0, 0, None, []
            for r in range(rounds):
                flush.zero_()
                ta = _ev_ms(torch, stream, lambda: pool.alloc(cfg, N, SEED0 + 31 * r, ids, steps, stream=sh))
                ok = ids >= 0
                got = ids[ok]
                if r == 0:
                    round0_steps = float(steps[ok].double().mean().item()) if got.numel() else None
                fails += N - int(got.numel())
                sel = got[torch.randperm(got.numel(), generator=gen, device="cuda")[:got.numel() // 2]].contiguous()
                flush.zero_()
                tf = _ev_ms(torch, stream, lambda: pool.free(cfg, sel.numel(), sel, stream=sh))
                t_ms += ta + tf
                ops += N + sel.numel()
                per_round.append([round(ta, 4), round(tf, 4), int(got.numel())])
            # RW_TAS(T, A, N) = (T/N) ln(A / (A - N)), the mean probes of N page-probe
            # requests on A free pages (theoretical_models.py:20-21); reported where A >= 1.25 N
            # (near A = N the model diverges and failures at max_steps truncate the walk)
            model = (T_PAGES / N) * math.log(free0 / (free0 - N)) if wname == "page_probe" and free0 >= 1.25 * N else None
            row[wname] = {"value": ops / (t_ms * 1e-3), "ms_total": t_ms, "failures": fails,
                          "model_rw_tas_round0": model,
                          "round0_ops_s": (N + per_round[0][2] // 2) / ((per_round[0][0] + per_round[0][1]) * 1e-3),
                          "round0_granted": per_round[0][2], "mean_steps_round0": round0_steps,
                          "used_after": pool.used(sh), "per_round_ms_alloc_free_granted": per_round}
        res[f"{int(occ * 100)}%"] = row
    # the autotuner's pick per occupancy band (alloc+free swaps on held pages),
    # then that pick against the per-thread walks on the same swaps: batched
    # graph form, 20 steps of 256 LogU groups, L2 flushed before each step
    tuned, churn = {}, {}
    for occ in (0.5, 0.75, 0.9, 0.95):
        pool.reset(sh)
        pool.prefill(occ, PREFILL_SEED, sh)
        words = pool.read_bitmap(sh)
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES]
        held = np.nonzero(bits)[0].astype(np.int32)
        np.random.default_rng(PREFILL_SEED).shuffle(held)
        arena = torch.from_numpy(held).cuda()
        counts = group_counts(1)
        tab = build_descriptors(counts, len(held), pbm.OP_SWAP)
        d_tab = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        top = pool.autotune(d_tab, N_GROUPS, int(counts[0].sum()), arena, len(held), seed=5, reps=2, stream=sh)
        tuned[f"{int(occ * 100)}%"] = [{"walk": pbm.STRATEGY_NAMES[t.cfg.strategy], "word_bits": t.cfg.word_bits,
                                        "width": t.cfg.collab_width, "stride": t.cfg.stride,
                                        "blocks_per_sm": t.cfg.blocks_per_sm, "free_merge": t.cfg.free_merge,
                                        "ops_per_s": t.ops_per_s} for t in top[:3]]
        n_steps = 20
        counts = group_counts(n_steps, seed=GROUP_SEED + 1)
        tab = build_descriptors(counts, len(held), pbm.OP_SWAP)
        d_tab = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        row = {}
        cands = [("tuned", pbm.WalkConfig.from_buffer_copy(top[0].cfg) if top else pbm.walk_config()),
                 ("word_probe32", pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32)),
                 ("page_probe", pbm.walk_config(pbm.RANDOM_WALK))]
        for cname, cfg in cands:
            g = pool.graph(cfg, d_tab, N_GROUPS, n_steps, arena, len(held), 4242, sh)
            t_ms = 0.0
            for _ in range(n_steps):
                flush.zero_()
                t_ms += _ev_ms(torch, stream, lambda: g.replay(sh))
            g.close()
            row[cname] = 2 * int(counts.sum()) / (t_ms * 1e-3)
        chk = pool.check(arena, len(held), sh)
        row["invariants_ok"] = bool(chk.n_duplicates == 0 and chk.n_not_marked == 0 and chk.used_pages == len(held))
        churn[f"{int(occ * 100)}%"] = row
    pool.close()
    return {"rounds": rounds, "requests_per_launch": N, "max_steps": max_steps, "unit": "ops/s",
            "ops": "get-page requests issued + pages freed", "l2": "flushed before every launch",
            "fail_fast": "requests past the free pages counted before each launch fail at once",
            "by_occupancy": res, "autotune_by_band": tuned,
            "churn_by_occupancy_ops_s": churn,
            "churn_note": "alloc+free swaps on the held pages (occupancy constant), batched graph form"}


def config_strategies(torch, pbm, stream, flush, occs=(0.5, 0.9), n=1 << 20, reps=3):
    """Every allocation strategy of the reference's device API (parallelPage.cuh:7-75,
    the header-only walks) through pbm_alloc / pbm_free: a 2^24-page pool
    prefilled to each occupancy (seed 2), 2^20 claims in one launch, then their
    frees in one launch, L2 flushed before each; alloc+free ops/s (median of
    the repetitions) and mean steps per claim."""
    sh = stream.cuda_stream
    strategies = [("RandomWalk", pbm.RANDOM_WALK), ("RandomWalk_BM", pbm.RANDOM_WALK_BM),
                  ("CollabRW_BM", pbm.COLLAB_RW_BM), ("ClusteredRandomWalk_BM", pbm.CLUSTERED_RW_BM),
                  ("LinkedList", pbm.LINKED_LIST), ("SingleClock", pbm.SINGLE_CLOCK), ("DistClock", pbm.DIST_CLOCK)]
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    steps = torch.empty(n, dtype=torch.int32, device="cuda")
    out = {"pool_pages": T_PAGES, "requests_per_launch": n, "unit": "ops/s", "ops": "claims + frees",
           "l2": "flushed before every launch", "by_occupancy": {}}
    pool = pbm.Pool(T_PAGES, PAGE_SIZE)
    for occ in occs:
        res = {}
        for name, strat in strategies:
            cfg = pbm.walk_config(strat)
            pool.reset(sh)
            pool.prefill(occ, PREFILL_SEED, sh)
            used0 = pool.used(sh)
            pool.alloc(cfg, n, 11, ids, steps, stream=sh)       # untimed: builds the free list where one is used
            pool.free(cfg, n, ids, stream=sh)
            ms = []
            for r in range(reps):
                flush.zero_()
                ta = _ev_ms(torch, stream, lambda: pool.alloc(cfg, n, 12 + r, ids, steps, stream=sh))
                st = steps.cpu().numpy()
                ok = int((ids.cpu().numpy() >= 0).sum())
                flush.zero_()
                tf = _ev_ms(torch, stream, lambda: pool.free(cfg, n, ids, stream=sh))
                ms.append(ta + tf)
            res[name] = {"value": 2 * n / (float(np.median(ms)) * 1e-3), "claims_ok": ok,
                         "mean_steps": float(st[st > 0].mean()) if (st > 0).any() else 0.0,
                         "occupancy_restored": pool.used(sh) == used0}
        out["by_occupancy"][f"{int(occ * 100)}%"] = res
    pool.close()
    return out


def config_clock_churn(torch, pbm, stream, flush, n_steps=20, warmup=5):
    """This build's SingleClock and DistClock on the churn the reference's
    clocks are timed on: a pool of the reference's fixed 41,900,000 pages
    (parallelPage.cuh:3) at 90% occupancy (seed 2), steps of LogU group
    counts (seed 4), each request freeing its arena slot's page and taking a
    new one (one free launch and one claim launch per slice of the arena)."""
    sh = stream.cuda_stream
    T = 41_900_000
    pool = pbm.Pool(T, 4096)
    out = {"pool_pages": T, "occupancy": OCCUPANCY, "unit": "ops/s", "l2": "flushed before every step",
           "steps": n_steps}
    counts = group_counts(warmup + n_steps).sum(axis=1)
    for name, strat in (("singleclock", pbm.SINGLE_CLOCK), ("distclock", pbm.DIST_CLOCK)):
        pool.reset(sh)
        pool.prefill(OCCUPANCY, PREFILL_SEED, sh)
        words = pool.read_bitmap(sh)
        held = np.nonzero(np.unpackbits(words.view(np.uint8), bitorder="little")[:T])[0].astype(np.int32)
        np.random.default_rng(PREFILL_SEED).shuffle(held)
        H = len(held)
        arena = torch.from_numpy(held).cuda()
        # the reference's clocks search without a bound; 2^20 steps keeps this
        # build's bounded sweep from giving up where an arm crosses a long run
        # of held pages
        cfg = pbm.walk_config(strat, max_steps=1 << 20)
        st0 = pool.stats(sh)
        off, t_ms, ops = 0, 0.0, 0
        for s_i, n in enumerate(counts):
            n = int(n)
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            k0 = 0
            while k0 < n:
                k = min(n - k0, H - off)
                sl = arena[off:off + k]
                pool.free(cfg, k, sl, stream=sh)
                pool.alloc(cfg, k, 7000 + s_i * 131 + k0, sl, stream=sh)
                off = (off + k) % H
                k0 += k
            e1.record(stream)
            e1.synchronize()
            if s_i >= warmup:
                t_ms += e0.elapsed_time(e1)
                ops += 2 * n
        chk = pool.check(arena, H, sh)
        st1 = pool.stats(sh)
        out[name] = {"value": ops / (t_ms * 1e-3), "ms_per_step": t_ms / n_steps,
                     "failures": int(st1.failures - st0.failures),
                     "mean_steps": (st1.steps - st0.steps) / max(1, st1.successes + st1.failures - st0.successes
                                                                  - st0.failures),
                     "invariants_ok": bool(chk.n_duplicates == 0 and chk.n_not_marked == 0
                                           and chk.n_failed == 0 and chk.used_pages == H)}
        del arena
    pool.close()
    return out


def config_buffer_manager(torch, pbm, stream, flush, n_fetch=1 << 26, round_size=1 << 18):
    """2^22 frames x 4 KiB over 2^24 logical pages; 2^26 fetches Zipf(0.99)
    over a seed-3 permutation; each pin held Geometric(0.25) rounds."""
    import workloads

    sh = stream.cuda_stream
    n_logical, n_frames = 1 << 24, 1 << 22
    rounds = n_fetch // round_size
    t0 = time.perf_counter()
    pages = workloads.zipf_pages(n_logical, 0.99, n_fetch, 3)
    ptr, idx = workloads.release_lists(rounds, round_size, 0.25, 3)
    gen_s = time.perf_counter() - t0
    d_pages = torch.from_numpy(pages).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_frames = torch.empty(n_fetch, dtype=torch.int32, device="cuda")
    out = {"fetches": n_fetch, "round_size": round_size, "trace_gen_s": gen_s, "unit": "fetches/s",
           "l2": "flushed before every round"}
    # by_page: pins released by page (pbm_bufmgr_round_pages, release list
    # naming the held-page array the rounds write), else by frame.  The
    # distributed clock gets one arm per request of a round, as the
    # reference's arms are one per thread; 4096 arms shared by a round's
    # 2^18 requests shows what sharing arms costs
    runs = [("single_clock", pbm.BM_SINGLE_CLOCK, 1, 0, False),
            ("dist_clock", pbm.BM_DIST_CLOCK, round_size, 0, False),
            ("single_clock_by_page", pbm.BM_SINGLE_CLOCK, 1, 0, True),
            ("dist_clock_by_page", pbm.BM_DIST_CLOCK, round_size, 0, True),
            ("dist_clock_4096_arms", pbm.BM_DIST_CLOCK, 4096, 0, False),
            ("single_clock_copy4k", pbm.BM_SINGLE_CLOCK, 1, 4096, False)]
    backing = None
    d_held = torch.empty(n_fetch, dtype=torch.int32, device="cuda")
    for name, policy, arms, fsz, by_page in runs:
        if fsz and backing is None:
            backing = torch.empty(n_logical * fsz // 4, dtype=torch.int32, device="cuda")
        bm = pbm.BufferManager(n_logical, n_frames, frame_size=fsz, policy=policy, n_arms=arms,
                               backing=backing if fsz else None)
        d_frames.fill_(-1)
        d_held.fill_(-1)
        t_ms = 0.0
        for r in range(rounds):
            a, b = int(ptr[r]), int(ptr[r + 1])
            lo = r * round_size
            rel = d_idx[a:] if b > a else None
            if by_page:
                fn = lambda: bm.round_pages(d_held, rel, b - a, d_pages[lo:], round_size, lo, d_frames[lo:],
                                            d_held[lo:], stream=sh)
            else:
                fn = lambda: bm.round(d_frames, rel, b - a, d_pages[lo:], round_size, lo, d_frames[lo:], stream=sh)
            flush.zero_()
            t_ms += _ev_ms(torch, stream, fn)
        c = bm.counters(sh)
        chk = bm.check(sh)
        out[name] = {"value": n_fetch / (t_ms * 1e-3), "ms_total": t_ms, "hits": c.hits, "misses": c.misses,
                     "evictions": c.evictions, "failures": c.failures, "hit_rate": c.hits / max(1, n_fetch),
                     "table_mismatches": chk.mismatches, "half_loaded": chk.loading,
                     "frame_bytes": fsz, "arms": arms, "release": "by page" if by_page else "by frame",
                     "bad_unpins": c.bad_unpins, "timeouts": c.timeouts}
        bm.close()
    del backing, d_held
    return out


def config_malloc(torch, pbm, stream, flush, rounds=16, plain_rounds=4, max_steps=512):
    """32 GiB pool of 4 KiB pages; per round 256 malloc groups (LogU[1,65536]
    requests, sizes LogU[16 B, 64 KiB] in power-of-two classes, seed 4) and
    frees of a uniformly random 50% of the live blocks, in one launch."""
    sh = stream.cuda_stream
    T = 1 << 23
    rng = np.random.default_rng(4)
    counts = group_counts(rounds, seed=4)
    n_max = int(counts.sum(axis=1).max())
    live_cap = 3 * n_max
    gen = torch.Generator(device="cuda")
    out = {"pool_pages": T, "page_size": PAGE_SIZE, "rounds": rounds, "unit": "ops/s",
           "ops": "mallocs + frees", "l2": "flushed before every round", "max_steps": max_steps,
           "note": "the trace outgrows the pool (about 34 GB live before each round's frees on 32 GiB), "
                   "so part of every round fails after max_steps jumps"}
    for form in ("graph", "plain", "queue_graph"):
        queue = form == "queue_graph"
        pool = pbm.Pool(T, PAGE_SIZE, materialize=True)
        if queue:
            pool.qmalloc_init(1 << 22)
        else:
            pool.malloc_init()
        gen.manual_seed(4)
        slots = n_max + live_cap
        ptrs = torch.zeros(slots, dtype=torch.int64, device="cuda")
        sizes = torch.zeros(slots, dtype=torch.int32, device="cuda")
        n_groups = 2 * N_GROUPS
        dt = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
        d_tab = torch.zeros(n_groups * 16, dtype=torch.uint8, device="cuda")
        mk_graph = pool.qmalloc_graph if queue else pool.malloc_graph
        graph = (mk_graph(d_tab, n_groups, 1, sizes, ptrs, slots, 91, max_steps=max_steps, stream=sh)
                 if form != "plain" else None)
        live = torch.empty(0, dtype=torch.int64, device="cuda")
        t_ms, ops, fails = 0.0, 0, 0
        nr = plain_rounds if form == "plain" else rounds
        for r in range(nr):
            c = counts[r]
            n_new = int(c.sum())
            sz = np.clip(np.exp(rng.uniform(math.log(16), math.log(65536), n_new)), 16, 65536).astype(np.int32)
            sizes[:n_new].copy_(torch.from_numpy(sz))
            ptrs[:n_new].zero_()
            k = live.numel() // 2
            perm = torch.randperm(live.numel(), generator=gen, device="cuda")
            to_free, keep = live[perm[:k]], live[perm[k:]]
            ptrs[n_max:n_max + k].copy_(to_free)
            tab = np.zeros(n_groups, dtype=dt)
            offs = np.concatenate([[0], np.cumsum(c)[:-1]])
            tab["op"][:N_GROUPS] = pbm.OP_MALLOC
            tab["count"][:N_GROUPS] = c
            tab["offset"][:N_GROUPS] = offs
            fsplit = np.linspace(0, k, N_GROUPS + 1).astype(np.int64)
            tab["op"][N_GROUPS:] = pbm.OP_MFREE
            tab["count"][N_GROUPS:] = np.diff(fsplit)
            tab["offset"][N_GROUPS:] = n_max + fsplit[:-1]
            d_tab.copy_(torch.from_numpy(tab.view(np.uint8).copy()))
            flush.zero_()
            if graph is not None:
                t_ms += _ev_ms(torch, stream, lambda: graph.replay(sh))
            else:
                hg = pbm.groups_array([(int(t["op"]), int(t["count"]), int(t["offset"])) for t in tab])
                t_ms += _ev_ms(torch, stream, lambda: pool.malloc_batch(d_tab, hg, n_groups, sizes, ptrs, slots,
                                                                        1000 + r, pbm.LAUNCH_PLAIN,
                                                                        max_steps=max_steps, stream=sh))
            new = ptrs[:n_new]
            ok = new != 0
            fails += n_new - int(ok.sum().item())
            live = torch.cat([keep, new[ok]])
            if live.numel() > live_cap:
                live = live[:live_cap]
            ops += n_new + k
        out[form] = {"value": ops / (t_ms * 1e-3), "ms_total": t_ms, "rounds": nr, "failures": fails,
                     "used_pages": pool.used(sh)}
        if queue:
            queued, chunks, overflow, timeouts, bad = pool.qmalloc_counts(sh)
            out[form].update(queued_blocks=int(sum(queued)), chunks=int(chunks), overflow=int(overflow),
                             timeouts=int(timeouts), bad_frees=int(bad))
        else:
            lv, bad = pool.malloc_counts(sh)
            out[form].update(live_blocks=int(lv), bad_frees=int(bad))
        if graph is not None:
            graph.close()
        pool.close()
    out["graph_over_plain"] = out["graph"]["value"] / out["plain"]["value"]
    out["backends"] = {"graph, plain": "page runs with live counts per run (pbm_malloc_*)",
                       "queue_graph": "per-class block queues (pbm_qmalloc_*), CUDA-graph form"}
    return out


def config_serving(torch, pbm, stream, rates=(1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11), min_req=100, max_req=20000,
                   horizon_s=1.0):
    """64 tenants, Poisson arrivals at an aggregate page rate, batches
    LogU[1,65536] pages, mix 45% alloc / 45% free / 10% Zipf(0.99) fetch,
    seed 5; 2^24-page pool prefilled to 80%, shared budget up to 95%: an
    ALLOC that does not fit waits for frees (p50/p99 include the wait;
    `over_budget` counts only ALLOCs larger than the whole budget, `stranded`
    the requests still waiting when nothing more could run).  The rates past
    1e9 (the workload's range) look for the loop's capacity: where the wall
    time exceeds the arrival span, throughput is the saturation rate and the
    latencies include queueing."""
    import workloads

    T = T_PAGES
    tenants = 64
    fetch = torch.from_numpy(workloads.zipf_pages(T, 0.99, 1 << 24, 5)).cuda()
    mean_pages = (MAX_GROUP - 1) / math.log(MAX_GROUP)
    out = {"tenants": tenants, "pool_pages": T, "prefill": 0.8, "max_occupancy": 0.95,
           "unit": "pages/s", "rates": {}}
    for rate in rates:
        rng = np.random.default_rng(5)
        n = int(min(max_req, max(min_req, rate * horizon_s / mean_pages)))
        cnt = np.clip(np.floor(np.exp(rng.uniform(0, math.log(MAX_GROUP + 1), n))), 1, MAX_GROUP).astype(np.int64)
        arr = np.cumsum(rng.exponential(mean_pages / rate, n))
        ten = rng.integers(0, tenants, n)
        u = rng.uniform(size=n)
        ops = np.where(u < 0.45, 0, np.where(u < 0.90, 1, 2))
        pool = pbm.Pool(T, PAGE_SIZE)
        pool.prefill(0.8, PREFILL_SEED)
        bm = pbm.BufferManager(T, 1 << 22, policy=pbm.BM_DIST_CLOCK, n_arms=4096)
        srv = pbm.Server(pool, tenants, 1 << 16, n_streams=4, max_batch_requests=256, max_occupancy=0.95,
                         bufmgr=bm, fetch_pages=fetch, max_fetch_pages=1 << 20)
        res, rep, rc = srv.run(arr, ten, ops, cnt)
        st = np.array([r.status for r in res])
        out["rates"][f"{rate:.0e}"] = {
            "requests": n, "arrival_span_s": float(arr[-1]), "wall_s": rep.wall_s,
            "throughput": rep.pages / rep.wall_s, "p50_ms": rep.p50_s * 1e3, "p99_ms": rep.p99_s * 1e3,
            "batches": rep.batches, "mean_batch_requests": rep.mean_batch_requests,
            "max_in_flight": rep.max_in_flight, "over_budget": int((st == pbm.ERR_EXHAUSTED).sum()),
            "waited_for_memory": int(rep.waited), "stranded": int(rep.stranded), "rc": rc}
        srv.close()
        bm.close()
        pool.close()
    return out


def run_configs(args, torch, pbm, stream):
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    todo = [("claim_write_free_50pct", lambda: config_claim_write_free(torch, pbm, stream,
                                                                      cpu=not args.no_cpu_baseline)),
            ("occupancy_sweep", lambda: config_occupancy_sweep(torch, pbm, stream, flush)),
            ("strategies", lambda: config_strategies(torch, pbm, stream, flush)),
            ("clock_churn_reference_pool", lambda: config_clock_churn(torch, pbm, stream, flush)),
            ("buffer_manager", lambda: config_buffer_manager(torch, pbm, stream, flush)),
            ("malloc", lambda: config_malloc(torch, pbm, stream, flush)),
            ("serving", lambda: config_serving(torch, pbm, stream))]
    want = set(args.configs.split(",")) if args.configs not in ("all", "none") else None
    out = {}
    for name, fn in todo:
        if args.configs == "none" or (want is not None and name not in want):
            continue
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:  # noqa: BLE001 -- one workload's error must not hide the others
            out[name] = {"error": f"{type(e).__name__}: {e}"[:400]}
        out[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.synchronize()
    return out


def run_profile_kernel(args):
    """Small, bounded cases of the other kernels for ncu captures (a few GB
    on the device at most, inputs larger than L2 where the kernel reads
    any): `bufmgr` 16 rounds of 2^18 Zipf fetches on 2^20 frames, full and
    evicting from round 11 on (k_round; --bm-* options set the frames, rounds,
    hands, releases by page and 4 KiB copies),
    `malloc` 8 rounds of 32 malloc groups + frees on a 2 GiB pool
    (k_malloc_persistent), `alloc` 2^22 collaborative claims at 50%
    (k_alloc_collab) followed by `free` of half of them (k_free_pages)."""
    import torch

    import pbm
    import workloads

    torch.cuda.set_device(0)
    sh = torch.cuda.current_stream().cuda_stream
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    out = {"profile_kernel": args.profile_kernel}
    if args.profile_kernel == "bufmgr":
        R, rounds = 1 << 18, args.bm_rounds
        n_logical = 1 << args.bm_logical_log2
        pages = workloads.zipf_pages(n_logical, 0.99, R * rounds, 3)
        ptr, idx = workloads.release_lists(rounds, R, 0.25, 3)
        d_pages = torch.from_numpy(pages).cuda()
        d_idx = torch.from_numpy(idx).cuda()
        d_frames = torch.full((R * rounds,), -1, dtype=torch.int32, device="cuda")
        dist = args.bm_policy == "dist"
        fsz = args.bm_frame_size
        backing = torch.empty(n_logical * fsz // 4, dtype=torch.int32, device="cuda") if fsz else None
        bm = pbm.BufferManager(n_logical, 1 << args.bm_frames_log2, frame_size=fsz,
                               policy=pbm.BM_DIST_CLOCK if dist else pbm.BM_SINGLE_CLOCK, n_arms=R if dist else 1,
                               backing=backing)
        d_held = torch.full((R * rounds,), -1, dtype=torch.int32, device="cuda")
        per_round = []
        for r in range(rounds):
            a, b = int(ptr[r]), int(ptr[r + 1])
            flush.zero_()
            rel = d_idx[a:] if b > a else None
            if args.bm_by_page:
                bm.round_pages(d_held, rel, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:], d_held[r * R:],
                               stream=sh)
            else:
                bm.round(d_frames, rel, b - a, d_pages[r * R:], R, r * R, d_frames[r * R:], stream=sh)
            c = bm.counters(sh)
            per_round.append((c.hits, c.misses, c.evictions))
        torch.cuda.synchronize()
        c = bm.counters(sh)
        d = np.diff(np.array([(0, 0, 0)] + per_round), axis=0)
        out.update(hits=c.hits, misses=c.misses, mismatches=bm.check(sh).mismatches,
                   per_round_hits_misses_evictions=d.tolist())
        bm.close()
    elif args.profile_kernel == "malloc":
        T, groups, rounds = 1 << 19, 32, 8
        pool = pbm.Pool(T, PAGE_SIZE, materialize=True)
        queue = args.malloc_backend == "queue"
        if queue:
            pool.qmalloc_init(1 << 20)
        else:
            pool.malloc_init()
        batch = pool.qmalloc_batch if queue else pool.malloc_batch
        rng = np.random.default_rng(4)
        counts = np.clip(np.floor(np.exp(rng.uniform(0, math.log(MAX_GROUP + 1), (rounds, groups)))), 1,
                         MAX_GROUP).astype(np.int64)
        n_max = int(counts.sum(axis=1).max())
        sizes = torch.zeros(2 * n_max, dtype=torch.int32, device="cuda")
        ptrs = torch.zeros(2 * n_max, dtype=torch.int64, device="cuda")
        dt = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
        prev_c = np.zeros(groups, dtype=np.int64)
        for r in range(rounds):
            # this round's mallocs go to slots [0, n); the previous round's blocks,
            # moved to [n_max, n_max + n_prev), are freed in the same launch
            c = counts[r]
            n = int(c.sum())
            sizes[:n].copy_(torch.from_numpy(np.clip(np.exp(rng.uniform(math.log(16), math.log(65536), n)), 16,
                                                     65536).astype(np.int32)))
            tab = np.zeros(2 * groups, dtype=dt)
            tab["op"][:groups], tab["count"][:groups] = pbm.OP_MALLOC, c
            tab["offset"][:groups] = np.concatenate([[0], np.cumsum(c)[:-1]])
            tab["op"][groups:], tab["count"][groups:] = pbm.OP_MFREE, prev_c
            tab["offset"][groups:] = n_max + np.concatenate([[0], np.cumsum(prev_c)[:-1]])
            d_tab = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
            flush.zero_()
            batch(d_tab, None, 2 * groups, sizes, ptrs, 2 * n_max, 77 + r, pbm.LAUNCH_PERSISTENT, max_steps=512,
                  stream=sh)
            ptrs[n_max:].zero_()
            ptrs[n_max:n_max + n].copy_(ptrs[:n])
            ptrs[:n_max].zero_()
            prev_c = c
        torch.cuda.synchronize()
        st = pool.stats(sh)
        out.update(successes=st.successes, failures=st.failures, frees=st.frees)
        pool.close()
    elif args.profile_kernel == "catalog":
        # every kernel of the library once, for single-kernel captures (-k
        # NAME -c 1): a 2^24-page pool at 50% for the walks (2^22 requests),
        # frees, runs, the fail-fast budget pass, the checks, the free list,
        # the monitor's popcount and one plain batch launch
        import ctypes

        N = 1 << 22
        ids = torch.empty(N, dtype=torch.int32, device="cuda")
        pool = pbm.Pool(T_PAGES, PAGE_SIZE, max_slots=N)
        for strat in (pbm.RANDOM_WALK, pbm.RANDOM_WALK_BM, pbm.CLUSTERED_RW_BM, pbm.SINGLE_CLOCK, pbm.DIST_CLOCK,
                      pbm.COLLAB_RW_BM, pbm.LINKED_LIST):
            pool.reset(sh)
            pool.prefill(0.5, PREFILL_SEED, sh)
            cfg = pbm.walk_config(strat)
            flush.zero_()
            pool.alloc(cfg, N, 70 + strat, ids, stream=sh)
            flush.zero_()
            pool.free(cfg, N, ids, stream=sh)
        pool.used(sh)
        # fail-fast: a launch asking for more pages than are free (budget pass + free list)
        pool.reset(sh)
        pool.prefill(0.95, PREFILL_SEED, sh)
        flush.zero_()
        pool.alloc(pbm.walk_config(pbm.COLLAB_RW_BM, fail_fast=1), N, 80, ids, stream=sh)
        chk = pool.check(ids, N, sh)
        # runs across words, and their frees
        pool.reset(sh)
        pool.prefill(0.05, PREFILL_SEED, sh)
        R = 1 << 18
        k = torch.from_numpy(np.random.default_rng(1).integers(1, 65, R).astype(np.int32)).cuda()
        flush.zero_()
        pool.alloc_spans(R, k, 81, ids[:R], max_steps=256, stream=sh)
        flush.zero_()
        pool.free_runs(R, ids[:R], k, stream=sh)
        # the no-alloc check on a pool at its 2^23-page limit
        small = pbm.Pool(1 << 23, PAGE_SIZE)
        small.prefill(0.5, 3, sh)
        small.alloc(pbm.walk_config(pbm.COLLAB_RW_BM), 1 << 20, 82, ids[:1 << 20], stream=sh)
        res = pbm.CheckResult()
        pbm.lib().pbm_check_ids_noalloc(small.bitmap_ptr, small.n_pages, ids.data_ptr(), 1 << 20, ctypes.byref(res),
                                        sh)
        # the monitor's popcount beside nothing else
        mon = pbm.Monitor(small, interval_us=1000, max_samples=2)
        time.sleep(0.05)
        mon.stop()
        small.close()
        # one plain batch launch of the benchmark's walk (a 65,536-request swap group)
        pool.reset(sh)
        pool.prefill(OCCUPANCY, PREFILL_SEED, sh)
        words = pool.read_bitmap(sh)
        held = np.nonzero(np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES])[0].astype(np.int32)
        arena = torch.from_numpy(held).cuda()
        flush.zero_()
        pool.batch(named_walk(pbm, "pair32c"), None, pbm.groups_array([(pbm.OP_SWAP, 65536, 0)]), 1, arena,
                   len(held), 83, pbm.LAUNCH_PLAIN, stream=sh)
        torch.cuda.synchronize()
        out.update(used=pool.used(sh), fail_fast_ok=int(chk.n_ok), noalloc_ok=int(res.n_ok))
        pool.close()
        # the roofline's ceiling kernel, captured the same way
        pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1, pattern=2)
        torch.cuda.synchronize()
    elif args.profile_kernel == "misc":
        # one launch each: page-probe and word-probe walks (2^22 claims at 50%),
        # runs across words (2^18 runs of 1..64 pages at 5%), config 1's
        # claim/write/free, the queue malloc (2^18 requests), the atomicOr
        # ceiling, and one plain batch launch (a 65,536-request swap group)
        N = 1 << 22
        ids = torch.empty(N, dtype=torch.int32, device="cuda")
        pool = pbm.Pool(T_PAGES, PAGE_SIZE)
        for name, cfg in (("page", pbm.walk_config(pbm.RANDOM_WALK)), ("word", pbm.walk_config(pbm.RANDOM_WALK_BM))):
            pool.reset(sh)
            pool.prefill(0.5, PREFILL_SEED, sh)
            flush.zero_()
            pool.alloc(cfg, N, 60, ids, stream=sh)
        pool.reset(sh)
        pool.prefill(0.05, PREFILL_SEED, sh)
        R = 1 << 18
        k = torch.from_numpy(np.random.default_rng(1).integers(1, 65, R).astype(np.int32)).cuda()
        flush.zero_()
        pool.alloc_spans(R, k, 61, ids[:R], max_steps=256, stream=sh)
        pool.close()
        small = pbm.Pool(1 << 16, 64, materialize=True)
        small.prefill(0.5, 1, sh)
        small.claim_write_free(1 << 15, 1, ids[:1 << 15], stream=sh)
        small.close()
        qp = pbm.Pool(1 << 19, PAGE_SIZE, materialize=True)
        qp.qmalloc_init(1 << 18)
        sizes = torch.from_numpy(np.clip(np.exp(np.random.default_rng(2).uniform(math.log(16), math.log(65536), R)),
                                         16, 65536).astype(np.int32)).cuda()
        ptrs = torch.zeros(R, dtype=torch.int64, device="cuda")
        dt = np.dtype([("op", "<i4"), ("count", "<u4"), ("offset", "<u8")])
        tab = np.zeros(1, dtype=dt)
        tab[0] = (pbm.OP_MALLOC, R, 0)
        flush.zero_()
        qp.qmalloc_batch(torch.from_numpy(tab.view(np.uint8).copy()).cuda(), None, 1, sizes, ptrs, R, 62,
                         pbm.LAUNCH_PERSISTENT, stream=sh)
        qp.close()
        pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1, pattern=2)
        pool = pbm.Pool(T_PAGES, PAGE_SIZE)
        pool.prefill(OCCUPANCY, PREFILL_SEED, sh)
        words = pool.read_bitmap(sh)
        held = np.nonzero(np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES])[0].astype(np.int32)
        arena = torch.from_numpy(held).cuda()
        flush.zero_()
        pool.batch(named_walk(pbm, "collab32c"), None, pbm.groups_array([(pbm.OP_SWAP, 65536, 0)]), 1, arena,
                   len(held), 63, pbm.LAUNCH_PLAIN, stream=sh)
        torch.cuda.synchronize()
        out.update(used=pool.used(sh), held=len(held))
        pool.close()
    else:
        pool = pbm.Pool(T_PAGES, PAGE_SIZE)
        pool.prefill(0.5, PREFILL_SEED, sh)
        N = 1 << 22
        ids = torch.empty(N, dtype=torch.int32, device="cuda")
        cfg = pbm.walk_config(pbm.COLLAB_RW_BM)
        for r in range(3):
            flush.zero_()
            pool.alloc(cfg, N, 50 + r, ids, stream=sh)
            sel = ids[: N // 2].contiguous()
            flush.zero_()
            pool.free(cfg, sel.numel(), sel, stream=sh)
        torch.cuda.synchronize()
        st = pool.stats(sh)
        out.update(successes=st.successes, failures=st.failures, frees=st.frees, used=pool.used(sh))
        pool.close()
    print(json.dumps(out))
    return 0


def run_profile_case(args):
    """The batched form only, for ncu: the same pool, occupancy and groups as
    the benchmark, without page memory (the kernel never touches it), L2
    flushed before every replay."""
    import torch

    import pbm

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    sh = torch.cuda.current_stream().cuda_stream
    pool = pbm.Pool(T_PAGES, PAGE_SIZE, materialize=False)
    pool.prefill(OCCUPANCY, PREFILL_SEED, sh)
    words = pool.read_bitmap(sh)
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:T_PAGES]
    held = np.nonzero(bits)[0].astype(np.int32)
    np.random.default_rng(PREFILL_SEED).shuffle(held)
    arena = torch.from_numpy(held).to(dev)
    n_steps = args.warmup + args.steps
    counts = group_counts(n_steps)
    tab = build_descriptors(counts, len(held), pbm.OP_SWAP)
    d_tab = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).to(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    walk = {"collab32c": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32, blocks_per_sm=5,
                                         free_merge=0),
            "pair32c": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=64, blocks_per_sm=5),
            "pair32c6": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=64, blocks_per_sm=6),
            "collab32": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32),
            "collab64": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=64, collab_width=32),
            "word32": pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32)}[args.profile_walk]
    graph = pool.graph(walk, d_tab, N_GROUPS, n_steps, arena, len(held), SEED0, sh)
    for _ in range(n_steps):
        flush.zero_()
        graph.replay(sh)
    torch.cuda.synchronize()
    chk = pool.check(arena, len(held))
    print(json.dumps({"profile_case": args.profile_walk, "steps": n_steps,
                      "pairs": int(counts.sum()), "duplicates": chk.n_duplicates,
                      "used": chk.used_pages, "held": len(held)}))
    graph.close()
    pool.close()
    return 0


def pbm_sms():
    import ctypes

    import pbm

    n = ctypes.c_int()
    pbm.lib().pbm_device_sm_count(ctypes.byref(n))
    return n.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true", help="batched form only (for ncu)")
    ap.add_argument("--profile-walk", default="collab32c", choices=["collab32c", "pair32c", "collab32", "collab64",
                                                                     "word32"],
                    help="collab32c: collaborative walk, 32-bit words, register-capped 5 blocks/SM, "
                         "frees unmerged (the autotuner's pick at 90%%)")
    ap.add_argument("--walk", default="auto", choices=("auto",) + WALKS,
                    help="auto: the autotuner picks (untimed, before the timed steps); else a fixed walk")
    ap.add_argument("--profile-kernel", default=None, choices=["bufmgr", "malloc", "alloc", "misc", "catalog"],
                    help="a small case of another kernel, for ncu (alloc also runs the free kernel)")
    ap.add_argument("--bm-frames-log2", type=int, default=20,
                    help="--profile-kernel bufmgr: log2 of the frames (22 is the benchmark's buffer manager)")
    ap.add_argument("--bm-rounds", type=int, default=16,
                    help="--profile-kernel bufmgr: rounds of 2^18 fetches")
    ap.add_argument("--malloc-backend", default="runs", choices=["runs", "queue"],
                    help="--profile-kernel malloc: page runs (pbm_malloc_*) or per-class queues (pbm_qmalloc_*)")
    ap.add_argument("--bm-logical-log2", type=int, default=24,
                    help="--profile-kernel bufmgr: log2 of the logical pages (24 is the benchmark's)")
    ap.add_argument("--bm-policy", default="single", choices=["single", "dist"],
                    help="--profile-kernel bufmgr: one shared hand, or one private hand per request of a round")
    ap.add_argument("--bm-frame-size", type=int, default=0,
                    help="--profile-kernel bufmgr: bytes per frame copied from a backing store on a miss (0: none)")
    ap.add_argument("--bm-by-page", action="store_true",
                    help="--profile-kernel bufmgr: release pins by page (pbm_bufmgr_round_pages)")
    ap.add_argument("--configs", default="all",
                    help="other workloads measured after the headline: all, none, or a comma list of "
                         "claim_write_free_50pct,occupancy_sweep,strategies,clock_churn_reference_pool,"
                         "buffer_manager,malloc,serving")
    ap.add_argument("--details", default=None,
                    help="also write the headline and every workload's results as one JSON file here")
    args = ap.parse_args()
    rank, world, local_rank = env_rank()
    if args.profile:
        return run_profile_case(args)
    if args.profile_kernel:
        return run_profile_kernel(args)
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
