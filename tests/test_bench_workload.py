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
