"""Generate model_predictions.json from the reference's theoretical_models.py.

Run in a checkout that has the reference project next to it: its root is
argv[1], else $PBM_REFERENCE_ROOT, else /root/reference.  The committed JSON pins
oracle/models.py, which restates those closed forms; the statistical tests
use the restatement, so the reference itself is not needed to run them.
"""
import json
import os
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PBM_REFERENCE_ROOT", "/root/reference")
sys.path.insert(0, ref)
import theoretical_models as tm  # noqa: E402

POINTS = [
    (2**24, 2**24, 2**22), (2**24, 2**23, 2**22), (2**24, int(0.3 * 2**24), 2**22),
    (65536, 32768, 16384), (65536, 32768, 1024), (2**20, 52429, 4096), (2**20, 31457, 4096),
    (2**24, 1677722, 2**16), (8192, 4096, 512),
]
out = []
for T, A, N in POINTS:
    row = {"T": T, "A": A, "N": N,
           "RW_TAS": tm.RW_TAS(T, A, N),
           "RWBM_TAS": tm.RWBM_TAS(T, A, N),
           "Queue_TAS": tm.Queue_TAS(T, A, N),
           "Queue_WAS": tm.Queue_WAS(T, A, N),
           "CoRWBM_WAS": float(tm.CoRWBM_WAS(T, A, N))}
    if T <= 2**20:   # the WAS sums run 10^7 Python iterations each
        row["RW_WAS"] = tm.RW_WAS(T, A, N)
        row["RWBM_WAS"] = tm.RWBM_WAS(T, A, N)
    out.append(row)
    print(row, flush=True)
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "model_predictions.json"), "w") as f:
    json.dump(out, f, indent=1)
