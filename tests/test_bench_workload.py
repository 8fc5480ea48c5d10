"""The benchmark's synthetic workload, checked on the host: the caller groups
of a step, their descriptor table (the pbm_group layout of include/pbm.h) and
the descriptor bytes the launch carries inline."""
import math
import os
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_group_counts_are_log_uniform_in_range():
    import bench

    c = bench.group_counts(64)
    assert c.shape == (64, bench.N_GROUPS)
    assert c.min() >= 1 and c.max() <= bench.MAX_GROUP
    # log-uniform on [1, 65536]: the mean of log(count) sits near half of log(65537)
    assert abs(np.log(c).mean() - math.log(bench.MAX_GROUP + 1) / 2) < 0.15
    assert np.array_equal(c, bench.group_counts(64))            # seeded


def test_descriptors_tile_the_arena_in_request_order():
    import bench

    H = 15_099_165
    c = bench.group_counts(5)
    tab = bench.build_descriptors(c, H, 2)
    assert tab.dtype.itemsize == 16 and tab.shape == c.shape
    assert (tab["op"] == 2).all() and np.array_equal(tab["count"], c)
    flat = tab.reshape(-1)
    starts = np.concatenate([[0], np.cumsum(c.reshape(-1))[:-1]]) % H
    assert np.array_equal(flat["offset"], starts)
    assert (flat["offset"] < H).all()
    # the bytes a launch carries inline: op, count, offset little-endian per group
    raw = flat.view(np.uint8).reshape(-1, 16)
    g = 7
    assert int.from_bytes(raw[g, 0:4].tobytes(), "little") == 2
    assert int.from_bytes(raw[g, 4:8].tobytes(), "little") == int(flat[g]["count"])
    assert int.from_bytes(raw[g, 8:16].tobytes(), "little") == int(flat[g]["offset"])


def test_a_step_fits_an_inline_table():
    import bench

    sys.path.insert(0, os.path.join(ROOT, "parallel-db-buffer-management_gb300"))
    import pbm

    assert bench.N_GROUPS <= pbm.MAX_INLINE_GROUPS
    with open(os.path.join(ROOT, "include", "pbm.h")) as f:
        hdr = f.read()
    assert f"#define PBM_MAX_INLINE_GROUPS {pbm.MAX_INLINE_GROUPS}" in hdr


def _full_line(bench, impl=None):
    """A headline object shaped like run_ours' (or run_reference's) with
    long free-text fields and every detail key a run carries."""
    full = {
        "metric": bench.METRIC, "value": 80567123456.789, "unit": bench.UNIT, "n_gpus": 1, "steps": 1000,
        "warmup": 5, "ms_per_step": 0.0375123456, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": dict(bench.workload_config(), walk="collab_rw_bm/32b/w64/s1/b5"),
        "plain_value": 1509876543.21, "batched_over_plain": 53.3612345,
        "e2e": {"value": 62912345678.9, "unit": bench.UNIT, "h2d_bytes_per_step": 4096,
                "d2h_bytes_per_step": 6012345, "form": "x" * 400, "results_match_arena": True},
        "roofline": {"bound": "l2_atomic", "achieved": 80.567, "peak": 127.51, "unit": "Gatomic/s",
                     "frac": 0.6318, "traffic": 8312345.6, "peak_source": "spread-pattern atomicOr ceiling",
                     "line_pattern_peak": 968.1, "frac_of_line_pattern": 0.083, "hbm_frac": 0.0949,
                     "kernel": "k" * 200, "hbm": {"achieved": 644.5, "peak": 6773.5}},
        "cpu_baseline": {"value": 333734840.97, "unit": bench.UNIT, "cores": 16, "kind": "port",
                         "sample": "y" * 300},
        "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 90},
        "gpu_launches": 1000, "invariants_ok": True, "autotune_top": [{"walk": "z" * 50}] * 6,
    }
    if impl:
        full["impl"] = impl
        full["reference_cuda_build"] = {"collab_ops_s": 11331234567.8, "rwbasic_ops_s": 18312345.6}
    return full


def test_headline_is_the_last_line_short_and_complete(capsys):
    import json

    import bench

    details = {"serving": {"rates": {f"1e+0{i}": {"p99_ms": 0.05} for i in range(5, 10)}, "blob": "w" * 30000}}
    bench.emit(_full_line(bench), details)
    lines = capsys.readouterr().out.strip().splitlines()
    last = lines[-1]
    assert len(last.encode()) <= bench.HEADLINE_MAX_BYTES
    h = json.loads(last)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "dtype",
              "config", "e2e", "roofline", "cpu_baseline", "clocks", "gpu_launches", "plain_value",
              "batched_over_plain", "invariants_ok"):
        assert k in h, k
    assert h["value"] > 0 and h["e2e"]["h2d_bytes_per_step"] == 4096 and h["e2e"]["d2h_bytes_per_step"] > 0
    assert set(h["roofline"]) >= {"bound", "achieved", "peak", "unit", "frac", "traffic"}
    # the fraction can be recomputed from the printed numbers
    assert abs(h["roofline"]["achieved"] / h["roofline"]["peak"] - h["roofline"]["frac"]) < 1e-3
    assert json.loads(lines[0])["detail"] == "serving"


def test_reference_headline_is_short(capsys):
    import json

    import bench

    bench.emit(_full_line(bench, impl="reference"), {"reference_cuda_build": {"collab": {"x": "v" * 5000}}})
    last = capsys.readouterr().out.strip().splitlines()[-1]
    assert len(last.encode()) <= bench.HEADLINE_MAX_BYTES
    h = json.loads(last)
    assert h["impl"] == "reference" and h["reference_cuda_build"]["collab_ops_s"] > 0
