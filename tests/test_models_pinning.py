"""oracle/models.py restates the reference's theoretical_models.py; the
committed predictions (made by importing the reference) pin it."""
import json
import os

import pytest

from conftest import GOLDEN


def _rows():
    p = os.path.join(GOLDEN, "model_predictions.json")
    if not os.path.exists(p):
        pytest.skip("model_predictions.json not generated")
    with open(p) as f:
        return json.load(f)


def test_models_match_reference_outputs():
    import models

    for row in _rows():
        T, A, N = row["T"], row["A"], row["N"]
        assert models.rw_tas(T, A, N) == pytest.approx(row["RW_TAS"], rel=1e-12)
        assert models.rwbm_tas(T, A, N) == pytest.approx(row["RWBM_TAS"], rel=1e-9)
        assert models.queue_tas(T, A, N) == pytest.approx(row["Queue_TAS"])
        assert models.queue_was(T, A, N) == pytest.approx(row["Queue_WAS"])
        assert models.corwbm_was(T, A, N) == pytest.approx(row["CoRWBM_WAS"], rel=1e-9)
        if "RW_WAS" in row:
            assert models.rw_was(T, A, N) == pytest.approx(row["RW_WAS"], rel=1e-9)
            assert models.rwbm_was(T, A, N) == pytest.approx(row["RWBM_WAS"], rel=1e-9)
