"""The monitor samples occupancy and counters while kernels run.

While a sequence of allocation launches grows the pool, samples taken by
the monitor's own stream show non-decreasing occupancy, at least one value
strictly between the start and the end (taken while the launches ran), and
the final sample equals the pool's occupancy and counters afterwards."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_monitor_samples_while_kernels_run(cuda, pbm_mod):
    torch = cuda
    pbm = pbm_mod
    T = 1 << 22
    pool = pbm.Pool(T, 64)
    pool.prefill(0.5, 3)
    used0 = pool.used()
    n = 1 << 15
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    # the page-probe walk from 50% towards a full pool: the later launches
    # walk long, so the whole sequence takes milliseconds of device time
    cfg = pbm.walk_config(pbm.RANDOM_WALK)
    mon = pbm.Monitor(pool, interval_us=50, max_samples=50000)
    time.sleep(0.01)
    for k in range(64):
        pool.alloc(cfg, n, 100 + k, ids)
    torch.cuda.synchronize()
    time.sleep(0.01)
    samples = mon.samples()
    mon.stop()
    used1 = pool.used()
    st = pool.stats()
    assert used1 == used0 + st.successes
    u = np.array([s.used_pages for s in samples])
    assert len(u) >= 3
    assert (np.diff(u) >= 0).all()
    assert u[0] >= used0 and u[-1] == used1
    assert ((u > used0) & (u < used1)).any()           # sampled while the launches ran
    last = samples[-1]
    assert last.stats.successes == st.successes and last.stats.failures == st.failures
    assert abs(last.free_fraction - (1 - used1 / T)) < 1e-12
    ts = np.array([s.t_s for s in samples])
    assert (np.diff(ts) > 0).all()
    pool.close()
