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
  e2e      through the C ABI with host buffers: step descriptors copied
           host->device from pinned memory, persistent launch, the step's new
           page ids copied device->host, all inside the timed region
The L2 is flushed (512 MiB write) between timed steps, outside the events.

`--impl reference` times the reference's algorithm on the host cores: the
std::atomic replay of its word-probe walk (RandomWalkBasic_BM) over the same
churn, all hardware threads (the reference ships no CPU implementation and its
CUDA path is timed separately).
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
# DRAM bytes per alloc+free pair of the batch kernel, from the ncu capture
# summarised in profiles/batch_persistent_collab32_90pct.md (None until captured).
NCU_DRAM_BYTES_PER_PAIR = None


def env_rank():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


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
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    # autotuner (untimed): candidates run on step 0's groups, swaps keep the pool at 90%
    tuned = pool.autotune(d_tab[:N_GROUPS * 16], N_GROUPS, int(counts[0].sum()), arena, H, seed=SEED0 - 999,
                          reps=4, stream=sh)
    torch.cuda.synchronize()
    cfg = pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32, free_merge=1)
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
    if dist:
        t = torch.tensor([g_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        g_ms = float(t.item())
    value = g_ops * world / (g_ms * 1e-3)
    st = pool.stats(sh)

    # ---- plain: one launch per group ----
    res_plain = timed(lambda s: pool.batch(cfg, None, h_groups(s), N_GROUPS, arena, H, SEED0 + s,
                                           pbm.LAUNCH_PLAIN, stream=sh), range(args.warmup, min(n_steps, args.warmup + 100)))
    p_ms = sum(ms for _, ms in res_plain)
    plain_value = sum(2 * int(pairs_per_step[s]) for s, _ in res_plain) / (p_ms * 1e-3)

    # ---- per-thread word-probe walk, batched (config-2 comparison) ----
    cfg_pt = pbm.walk_config(pbm.RANDOM_WALK_BM, word_bits=32, free_merge=1)
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

    def e2e_step(s):
        row = h_tab[s * N_GROUPS * 16:(s + 1) * N_GROUPS * 16]
        d_stage.copy_(row, non_blocking=True)
        pool.batch(cfg, d_stage, None, N_GROUPS, arena, H, SEED0 + 50000 + s, pbm.LAUNCH_PERSISTENT, stream=sh)
        start = int(tab[s, 0]["offset"])
        n = int(pairs_per_step[s])
        first = min(n, H - start)
        h_out[:first].copy_(arena[start:start + first], non_blocking=True)
        if n > first:
            h_out[first:n].copy_(arena[:n - first], non_blocking=True)
        e2e_bytes_in.append(N_GROUPS * 16)
        e2e_bytes_out.append(4 * n)

    for s in range(args.warmup):
        e2e_step(s)
    torch.cuda.synchronize()
    res_e2e = timed(e2e_step, range(args.warmup, min(n_steps, args.warmup + 100)))
    e_ms = sum(ms for _, ms in res_e2e)
    e2e_value = sum(2 * int(pairs_per_step[s]) for s, _ in res_e2e) / (e_ms * 1e-3) * world

    # ---- invariants after all forms: occupancy unchanged, arena unique ----
    chk = pool.check(arena, H)
    ok_inv = (chk.n_duplicates == 0 and chk.n_out_of_range == 0 and chk.n_not_marked == 0
              and chk.n_failed == 0 and chk.used_pages == H)

    # ---- roofline: atomic ceiling and HBM ----
    ceil_line, _ = pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1, pattern=1)
    ceil_spread, _ = pbm.atomic_ceiling(words=1 << 22, threads=pbm_sms() * 2048, iters=64, returning=1,
                                        pattern=2)
    ceil_ops = max(ceil_line, ceil_spread)
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
        "kernel": "k_batch_persistent<Collab,32,u32> (+ its 1-block prefix and step kernels in the graph)",
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
        "config": dict(workload_config(), walk=cfg_dict(cfg)),
        "plain_value": plain_value, "batched_over_plain": value / world / plain_value,
        "per_thread_walk_value": per_thread_value,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(np.mean(e2e_bytes_in)),
                "d2h_bytes_per_step": int(np.mean(e2e_bytes_out))},
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    graph.close()
    g_pt.close()
    pool.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
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
    walk = {"collab32": pbm.walk_config(pbm.COLLAB_RW_BM, word_bits=32, collab_width=32),
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
    ap.add_argument("--profile-walk", default="collab32", choices=["collab32", "collab64", "word32"])
    args = ap.parse_args()
    rank, world, local_rank = env_rank()
    if args.profile:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
